"""The oracle's heatmap and PPM-byte restatements against the reference's own host code:
applyHeatmapColormap / getTurboColor and savePPM from src/render_engine.cu, compiled from the
reference tree into oracle/_ref (skipped where the reference sources were absent)."""
import ctypes
import os

import numpy as np
import pytest

from oracle import oracle as O

LIB = os.path.join(os.path.dirname(os.path.abspath(O.__file__)), "_ref", "libref_render_host.so")


@pytest.fixture(scope="module")
def R():
    if not os.path.exists(LIB):
        pytest.skip("libref_render_host.so not built (reference sources absent)")
    lib = ctypes.CDLL(LIB)
    lib.ref_turbo_table.argtypes = [ctypes.c_void_p]
    lib.ref_apply_heatmap.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_float]
    lib.ref_save_ppm.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
    lib.ref_save_ppm.restype = ctypes.c_int
    return lib


def _turbo(R):
    out = np.zeros(256 * 3, np.float32)
    R.ref_turbo_table(out.ctypes.data)
    return out.reshape(256, 3)


def _counts(case, n, rng):
    if case == "all_zero":
        return np.zeros(n, np.int32)
    if case == "one_pixel":
        v = np.zeros(n, np.int32)
        v[n // 2] = 77
        return v
    if case == "large":
        v = rng.integers(0, 1 << 20, n, dtype=np.int32)
        v[rng.random(n) < 0.3] = 0
        return v
    if case == "negative":  # counted as no hit for the percentile, coloured at t = 0
        v = rng.integers(-5, 60, n, dtype=np.int32)
        return v
    v = rng.geometric(0.02, n).astype(np.int32)
    v[rng.random(n) < 0.25] = 0
    return v


@pytest.mark.parametrize("case,fixed", [("typical", 0.0), ("typical", 40.0), ("typical", 0.5), ("all_zero", 0.0),
                                        ("one_pixel", 0.0), ("large", 0.0), ("negative", 0.0)])
def test_heatmap_oracle_equals_reference(R, case, fixed):
    w, h = 96, 64
    vis = _counts(case, w * h, np.random.default_rng(sum(map(ord, case))))
    ref = np.zeros(w * h * 3, np.float32)
    R.ref_apply_heatmap(ref.ctypes.data, vis.ctypes.data, w, h, ctypes.c_float(fixed))
    got, _ = O.heatmap(vis, _turbo(R), fixed)
    assert np.array_equal(got.reshape(-1).view(np.uint32), ref.view(np.uint32))


def test_ppm_bytes_oracle_equals_reference(R, tmp_path):
    w, h = 97, 31
    rng = np.random.default_rng(3)
    v = (rng.random(w * h * 3, dtype=np.float32) * 1.4 - 0.2).astype(np.float32)
    v[:8] = [0.0, -0.0, 1.0, 0.5 / 255.0, 254.5 / 255.0, np.nan, np.inf, -np.inf]
    path = str(tmp_path / "img.ppm")
    assert R.ref_save_ppm(path.encode(), v.ctypes.data, w, h) == 1
    data = open(path, "rb").read()
    header = f"P6\n{w} {h}\n255\n".encode()
    assert data.startswith(header)
    ref = np.frombuffer(data[len(header):], np.uint8)
    assert np.array_equal(O.rgb8(v), ref)
