"""The parallel OBJ reader (bvh_load_obj) against the reference's own loadOBJ (src/loader.cpp),
compiled from the reference sources into oracle/_ref/libref_loader.so, on generated files."""
import os

import numpy as np
import pytest

import bvh_gb300
from bvh_gb300 import _capi as C


def _ref():
    from oracle import ref
    if not ref.loader_available():
        pytest.skip("reference loader (oracle/_ref/libref_loader.so) not built")
    return ref


def _write(tmp_path, name, text):
    p = tmp_path / name
    p.write_bytes(text.encode())
    return str(p)


def _same(path, threads=(1, 3, 8)):
    expect = _ref().ref_load_obj(path)
    assert expect is not None
    for t in threads:
        got = bvh_gb300.load_obj(path, threads=t).arrays()
        for a, b in zip(got, expect):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), t
    return expect[0].shape[0]


def _random_obj(rng, n_vertices, n_faces, crlf=False, extras=True):
    nl = "\r\n" if crlf else "\n"
    lines = ["# generated", "o thing", ""]
    v = rng.standard_normal((n_vertices, 3)).astype(np.float32) * 10
    emitted = 0
    faces = 0
    fmts = ["{a}", "{a}/{a}", "{a}//{a}", "{a}/{a}/{a}"]
    while emitted < n_vertices or faces < n_faces:
        if emitted < n_vertices and (faces >= n_faces or rng.random() < 0.5):
            x, y, z = v[emitted]
            lines.append(f"v {x!r} {y:.9g} {z:.6e}" if rng.random() < 0.5 else f"  v\t{x:.9g}  {y!r} {z!r}")
            emitted += 1
            if extras and rng.random() < 0.1:
                lines.append(f"vn 0 0 1{nl[:-1]}")
            continue
        k = int(rng.integers(3, 7))
        idx = []
        for _ in range(k):
            if emitted and rng.random() < 0.2:
                idx.append(-int(rng.integers(1, emitted + 1)))       # relative
            else:
                idx.append(int(rng.integers(1, n_vertices + 3)))     # absolute, sometimes ahead/out of range
        fmt = fmts[int(rng.integers(0, 4))]
        lines.append("f " + " ".join(fmt.format(a=i) for i in idx))
        faces += 1
        if extras and rng.random() < 0.05:
            lines.append("# comment")
            lines.append("")
            lines.append("s off")
    return nl.join(lines) + nl


@pytest.mark.parametrize("crlf", [False, True])
def test_small_cases(tmp_path, crlf):
    nl = "\r\n" if crlf else "\n"
    text = nl.join([
        "# triangle, quad, pentagon, and every index form",
        "v 0 0 0", "v 1 0 0", "v 0 1 0", "v 1 1 0", "v 2 2 2",
        "f 1 2 3",
        "f 1/1 2/2 3/3 4/4",
        "f 1//1 2//2 3//3 4//4 5//5",
        "f -1 -2 -3",
        "f 1 2 99",          # out of range: skipped
        "f 0 1 2",           # index 0 -> -1: skipped
        "f 6 1 2",           # vertex 6 not read yet: skipped
        "v 3 3 3",
        "f 6 1 2",           # now it is
        "vt 0.5 0.5", "vn 0 0 1", "g group", "usemtl m",
        "   v 4 5 6",         # leading spaces
        "v 7 8",              # missing z reads 0
        "f 1 2",              # a degenerate face adds nothing
        "",
    ]) + nl
    n = _same(_write(tmp_path, "small.obj", text))
    assert n == 1 + 2 + 3 + 1 + 1


def test_random_files_single_and_multi_threaded(tmp_path):
    rng = np.random.default_rng(0)
    for k in range(4):
        text = _random_obj(rng, 3000 + 977 * k, 4000 + 1313 * k, crlf=(k % 2 == 1))
        _same(_write(tmp_path, f"r{k}.obj", text))


def test_large_file_many_threads(tmp_path):
    rng = np.random.default_rng(1)
    text = _random_obj(rng, 60000, 90000, extras=False)
    assert len(text) > 256 * 4096  # large enough to be split across threads
    n = _same(_write(tmp_path, "big.obj", text), threads=(1, 16, 64))
    assert n > 100000


def test_bad_index_is_an_error_like_the_reference(tmp_path):
    path = _write(tmp_path, "bad.obj", "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 x\n")
    assert _ref().ref_load_obj(path) is None  # std::stoi throws
    with pytest.raises(C.BVHError):
        bvh_gb300.load_obj(path)


def test_missing_file_is_an_error(tmp_path):
    with pytest.raises(C.BVHError):
        bvh_gb300.load_obj(os.path.join(str(tmp_path), "nope.obj"))


def test_empty_file(tmp_path):
    assert bvh_gb300.load_obj(_write(tmp_path, "empty.obj", "")).size() == 0
