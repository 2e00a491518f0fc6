"""Serving (per-request slots and batched ticks): results are the same alone and in the mix;
the HBM budget bounds the memory the server holds."""
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


def _equal_requests(k, n=100_000, rays=1024):
    out = []
    for t in range(k):
        m = meshgen.uniform_small(n, seed=300 + t)
        ro, rd = meshgen.sphere_rays(m, rays, seed=400 + t)
        out.append((m, [ro[:, 0].copy(), ro[:, 1].copy(), ro[:, 2].copy(), rd[:, 0].copy(), rd[:, 1].copy(),
                        rd[:, 2].copy()]))
    return out


def _one_at_a_time_budget(n=100_000, rays=1024):
    """Room for one request of n triangles (its mesh copy, workspace, rays and hits), not two."""
    return int(1.5 * (36 * n + 206 * n + 44 * rays))


def test_budget_admission_and_rejection(gpu):
    """The budget bounds what the slots hold together: with room for one request only, the
    requests run one after another (admissions wait), and one larger than the budget is rejected."""
    reqs = _equal_requests(6)
    budget = _one_at_a_time_budget()
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


def _pinned(arrays, torch):
    return [torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in arrays]


@pytest.mark.parametrize("pinned", [False, True])
def test_batched_ticks_same_alone_and_in_the_mix(gpu, pinned):
    """Batched ticks (one gather, batched build, traversal and scatter per batch) give every
    request the hits it gets alone on a per-request slot, bit for bit -- from pageable arrays
    (read directly where the GPU reads pageable memory, else copied) and from page-locked ones."""
    reqs = _requests(24)
    alone = Server(slots=1)
    h_alone, _ = _run(alone, reqs, concurrent=False)
    alone.close()
    if pinned:  # page-locked torch tensors (the device reads them through their mapped addresses)
        inputs = [(_pinned(m.arrays(), gpu), _pinned(rays, gpu)) for m, rays in reqs]
        hits = [[gpu.zeros(len(r[1][0]), dtype=gpu.float32).pin_memory()] +
                [gpu.zeros(len(r[1][0]), dtype=gpu.int32).pin_memory() for _ in range(4)] for r in reqs]
    else:
        inputs = [(m.arrays(), rays) for m, rays in reqs]
        hits = [_hits(len(r[1][0])) for r in reqs]
    sv = Server(slots=2, batched=True)
    for t, (arrays, rays) in enumerate(inputs):
        sv.submit(t, arrays, rays, hits[t])
    done = {}
    deadline = time.time() + 120
    while len(done) < len(reqs) and time.time() < deadline:
        for r in sv.poll(64, 50):
            done[r["tag"]] = r
    st = sv.stats()
    sv.close()
    assert len(done) == len(reqs) and all(r["status"] == C.BVH_OK for r in done.values())
    for a, b in zip(h_alone, hits):
        for x, y in zip(a, b):
            y = y.numpy() if hasattr(y, "numpy") else y
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    # requests were batched: fewer admissions (distinct admit times) than requests
    assert len({r["t_admit_ns"] for r in done.values()}) < len(reqs)
    assert st["completed"] == len(reqs)


def test_batched_ticks_respect_batch_limits(gpu):
    reqs = _requests(12, rays=512)
    sv = Server(slots=1, batched=True, batch_requests=3)
    hits, done = _run(sv, reqs, concurrent=True)
    sv.close()
    per_batch = {}
    for r in done.values():
        per_batch[r["t_admit_ns"]] = per_batch.get(r["t_admit_ns"], 0) + 1
    assert max(per_batch.values()) <= 3
    assert len(per_batch) >= 4


def test_batched_ticks_budget(gpu):
    reqs = _equal_requests(8)
    budget = _one_at_a_time_budget()
    sv = Server(budget_bytes=budget, slots=3, batched=True)
    hits, done = _run(sv, reqs, concurrent=True)
    st = sv.stats()
    sv.close()
    assert st["peak_in_flight_bytes"] <= budget  # what the slots held together, at most
    assert st["budget_waits"] > 0


def test_batched_ticks_need_30_bit_codes(gpu):
    with pytest.raises(C.BVHError) as e:
        Server(batched=True, morton_bits=63)
    assert e.value.status == C.BVH_ERR_UNSUPPORTED
