"""Serving: results are the same alone and in the mix; admission respects the HBM budget."""
import time

import numpy as np
import pytest

from bvh_gb300 import meshgen, _capi as C
from bvh_gb300.serve import Server

pytestmark = pytest.mark.gpu


def _requests(k, rays=4096):
    out = []
    for t in range(k):
        n = int(np.exp(np.random.default_rng(t).uniform(np.log(1000), np.log(200_000))))
        m = meshgen.clustered(n, seed=100 + t) if t % 2 else meshgen.uniform_small(n, seed=100 + t)
        ro, rd = meshgen.sphere_rays(m, rays, seed=200 + t)
        out.append((m, [ro[:, 0].copy(), ro[:, 1].copy(), ro[:, 2].copy(), rd[:, 0].copy(), rd[:, 1].copy(),
                        rd[:, 2].copy()]))
    return out


def _hits(nr):
    return [np.zeros(nr, np.float32)] + [np.zeros(nr, np.int32) for _ in range(4)]


def _run(server, reqs, concurrent):
    hits = [_hits(len(r[1][0])) for r in reqs]
    done = {}
    if concurrent:
        for t, (m, rays) in enumerate(reqs):
            server.submit(t, m.arrays(), rays, hits[t])
    for t, (m, rays) in enumerate(reqs):
        if not concurrent:
            server.submit(t, m.arrays(), rays, hits[t])
        deadline = time.time() + 120
        while (t not in done if not concurrent else len(done) < len(reqs)) and time.time() < deadline:
            for r in server.poll(64, 50):
                done[r["tag"]] = r
        if concurrent:
            break
    assert len(done) == len(reqs)
    assert all(r["status"] == C.BVH_OK for r in done.values())
    return hits, done


def test_same_alone_and_in_the_mix(gpu, oracle_lib):
    reqs = _requests(16)
    alone = Server(slots=1)
    h_alone, _ = _run(alone, reqs, concurrent=False)
    alone.close()
    mix = Server(slots=8)
    h_mix, done = _run(mix, reqs, concurrent=True)
    st = mix.stats()
    mix.close()
    for a, b in zip(h_alone, h_mix):
        for x, y in zip(a, b):
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    # the served result is the oracle's traversal of the oracle's tree
    m, rays = reqs[3]
    nodes, _, _ = oracle_lib.lbvh(m.arrays(), 30)
    ro = np.stack(rays[:3], 1)
    rd = np.stack(rays[3:], 1)
    exp = oracle_lib.trace(nodes, m.arrays(), ro, rd)
    assert np.array_equal(h_alone[3][0].view(np.uint32), exp[0].view(np.uint32))
    assert np.array_equal(h_alone[3][1], exp[1])
    # work overlapped: more than one request was admitted before the first finished
    first_done = min(r["t_done_ns"] for r in done.values())
    assert sum(r["t_admit_ns"] < first_done for r in done.values()) > 1
    assert st["completed"] == 16


def test_budget_admission_and_rejection(gpu):
    reqs = _requests(6, rays=1024)
    per = max(36 * m.size() + m.size() * 161 + 44 * 1024 + (4 << 20) for m, _ in reqs)
    budget = int(per * 1.5)  # room for one request at a time
    sv = Server(budget_bytes=budget, slots=4)
    hits, done = _run(sv, reqs, concurrent=True)
    st = sv.stats()
    assert st["peak_in_flight_bytes"] <= budget
    assert st["budget_waits"] > 0
    big = meshgen.uniform_small(2_000_000, seed=9)
    ro, rd = meshgen.sphere_rays(big, 16, seed=1)
    h = _hits(16)
    sv.submit(99, big.arrays(), [ro[:, k].copy() for k in range(3)] + [rd[:, k].copy() for k in range(3)], h)
    res = []
    for _ in range(100):
        res += sv.poll(4, 50)
        if res:
            break
    assert res and res[0]["tag"] == 99 and res[0]["status"] == C.BVH_ERR_OUT_OF_MEMORY
    sv.close()
