"""Generates the golden fixtures in this folder: seeded input meshes and the reference's own
outputs for them -- its .cu kernels compiled unmodified (oracle/ref_build.py) and replayed in its
host order with CUB/Thrust (oracle/_ref/libref_runner.so) on a GB300.  tests/test_oracle_cpu.py
checks the CPU oracle against them without a GPU.

Run on a GPU machine after the build:
    python -c "import __graft_entry__ as g; g.build()"
    python tests/golden/make_golden.py [out_dir]        # default: this folder

Each .npz holds v0..v8 (the SoA mesh, float32), kind ("lbvh30", "lbvh_plus60", "ploc<r>"),
nodes (the 48-byte BVHNode records as raw bytes), indices, radius (PLOC) and source.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from bvh_gb300 import meshgen  # noqa: E402
from oracle import ref  # noqa: E402

# (file stem, kind, generator, generator arguments, PLOC radius)
CASES = [
    ("lbvh30_uniform3000", "lbvh30", "uniform_small", {"n": 3000, "seed": 11}, 0),
    ("lbvh30_clustered8000", "lbvh30", "clustered", {"n": 8000, "seed": 12}, 0),
    ("lbvh30_identical257", "lbvh30", "uniform_small", {"n": 257, "seed": 13, "scale": 0.0}, 0),
    ("lbvh_plus60_clustered4000", "lbvh_plus60", "clustered", {"n": 4000, "seed": 14}, 0),
    ("lbvh_plus60_uniform2000", "lbvh_plus60", "uniform_small", {"n": 2000, "seed": 15}, 0),
    ("ploc10_clustered4000", "ploc10", "clustered", {"n": 4000, "seed": 16}, 10),
    ("ploc25_uniform3000", "ploc25", "uniform_small", {"n": 3000, "seed": 17}, 25),
]


def main(out_dir: str) -> None:
    if not ref.runner_available():
        raise SystemExit("oracle/_ref/libref_runner.so or the reference fatbins are missing: run the build first")
    R = ref.RefRunner()
    os.makedirs(out_dir, exist_ok=True)
    for stem, kind, gen, kw, radius in CASES:
        mesh = getattr(meshgen, gen)(**kw)
        arrays = [np.ascontiguousarray(a, np.float32) for a in mesh.arrays()]
        if kind == "lbvh30":
            nodes, idx, _ = R.lbvh(arrays)
        elif kind == "lbvh_plus60":
            nodes, idx, _ = R.lbvh_plus(arrays)
        else:
            nodes, idx, _, _, rc = R.ploc(arrays, radius)
            if rc != 0:
                raise SystemExit(f"{stem}: reference PLOC returned {rc}")
        out = {f"v{k}": arrays[k] for k in range(9)}
        out.update(kind=np.array(kind), nodes=np.ascontiguousarray(nodes).view(np.uint8).reshape(-1),
                   indices=np.ascontiguousarray(idx, np.uint32), radius=np.array(radius, np.int32),
                   source=np.array("reference kernels (unmodified .cu, default flags) via oracle/_ref on a GB300"))
        path = os.path.join(out_dir, stem + ".npz")
        np.savez_compressed(path, **out)
        print(f"{path}: {mesh.size()} triangles, {nodes.shape[0]} nodes")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.dirname(os.path.abspath(__file__)))
