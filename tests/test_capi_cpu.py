"""CPU tests of the C ABI library: it loads and exports every symbol include/bvh_gb300.h declares."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from bvh_gb300 import build, _capi
    build.build_library()
    return _capi.load_library()


def declared_functions():
    src = open(os.path.join(ROOT, "include", "bvh_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*[A-Za-z_][\w\s\*]*?\b(bvh_\w+)\s*\(", src, flags=re.M)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "bvh_build_device" in names and "bvh_trace" in names and len(names) >= 15


def test_library_exports_every_declared_symbol(lib):
    from bvh_gb300 import _capi
    for name in declared_functions():
        assert hasattr(lib, name), name
        assert name in _capi.SIGNATURES, f"{name} has no ctypes signature"


def test_status_strings(lib):
    for s in range(7):
        assert lib.bvh_status_string(s)
    assert lib.bvh_status_string(0) == b"ok"


def test_default_params(lib):
    from bvh_gb300 import _capi as C
    p = lib.bvh_default_params(C.ALGO_PLOC)
    assert p.algo == C.ALGO_PLOC and p.ploc_radius == 25 and p.morton_bits == 30
    p = lib.bvh_default_params(C.ALGO_LBVH_PLUS)
    assert p.morton_bits == 60 and p.treelet_rounds == 1


def test_context_without_gpu_is_an_error_not_a_crash(lib):
    from conftest import has_gpu
    if has_gpu():
        pytest.skip("GPU present")
    h = ctypes.c_void_p()
    assert lib.bvh_ctx_create(ctypes.byref(h), 0) == 1  # BVH_ERR_INVALID_ARG: no such device


def test_auto_camera_matches_reference_formula(lib):
    """autoCamera (src/render_engine.cu:601-637) on a unit box."""
    import numpy as np
    from bvh_gb300 import builders, _capi as C
    node = np.zeros(1, C.NODE_DTYPE)[0]
    node["min"] = (0, 0, 0)
    node["max"] = (1, 1, 1)
    cam = builders.auto_camera(node)
    diag = np.float32(np.sqrt(np.float32(3.0)))
    assert cam.fov_y_deg == 60.0 and tuple(cam.look_at) == (0.5, 0.5, 0.5)
    assert abs(cam.eye[0] - (0.5 + float(diag) * 0.5 / np.tan(np.pi / 6) * 1.2 * 0.6)) < 1e-5
