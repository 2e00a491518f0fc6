"""The device-side bounded waits give up and report it, and the GPU keeps working.

The library waits on the device in two places: the radix sort's look-back (in a build it waits
only on tiles that started earlier, so it always ends) and the grid barrier of the cooperative
PLOC kernel (its launch keeps every block resident, so every block arrives).
bvh_selftest_bounded_wait runs both against a partner that never comes -- a predecessor that never
publishes, a block that never arrives -- with a short poll limit.
"""
import time

import numpy as np
import pytest

from bvh_gb300 import Context, meshgen, _capi as C

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_device_still_answers(gpu, oracle_lib):
    lib = C.load_library()
    for polls in (1, 1000, 200_000):
        t0 = time.time()
        rc = lib.bvh_selftest_bounded_wait(0, polls)
        assert rc == C.BVH_ERR_TIMEOUT, C.BVHError(rc) if rc else rc
        assert time.time() - t0 < 10.0
    # the context is still usable: builds right afterwards are bit-exact (PLOC through the
    # cooperative kernel: 70,000 triangles reach it)
    ctx = Context(0)
    m = meshgen.uniform_small(5000, seed=3)
    nodes, idx = ctx.build_host(m, ctx.params(C.ALGO_LBVH))
    onodes, oidx, _ = oracle_lib.lbvh(m.arrays(), 30)
    assert np.array_equal(idx, oidx) and oracle_lib.node_fields_equal(nodes, onodes)
    m = meshgen.clustered(70_000, seed=5)
    nodes, idx = ctx.build_host(m, ctx.params(C.ALGO_PLOC, ploc_radius=25))
    onodes, oidx, _, _, rc = oracle_lib.ploc(m.arrays(), 25)
    assert rc == 0 and np.array_equal(idx, oidx) and oracle_lib.node_fields_equal(nodes, onodes)
    ctx.close()


def test_bounded_wait_rejects_bad_limits(gpu):
    lib = C.load_library()
    assert lib.bvh_selftest_bounded_wait(0, 0) == C.BVH_ERR_INVALID_ARG
    assert lib.bvh_selftest_bounded_wait(0, (1 << 24) + 1) == C.BVH_ERR_INVALID_ARG
    assert lib.bvh_selftest_bounded_wait(-1, 10) == C.BVH_ERR_INVALID_ARG
