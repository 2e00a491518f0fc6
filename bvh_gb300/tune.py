"""Build a tuning table for this GPU: bvh_autotune_build over a set of (algorithm, size) cases,
written as the JSON bvh_tuning_import reads.  Launch shapes never change a tree; the table only
makes builds faster.

    python -m bvh_gb300.tune --out table.json [--sizes 100000,1000000,10000000]

Load it into a context with Context.tuning_import(open(path).read()) (C: bvh_tuning_import).
"""
from __future__ import annotations

import argparse
import json

import numpy as np


def tune(sizes, device: int = 0) -> dict:
    import torch

    from . import _capi as C
    from . import meshgen
    from .builders import Context

    ctx = Context(device)
    stream = torch.cuda.current_stream(device).cuda_stream
    reports = []
    for n in sizes:
        mesh = meshgen.clustered(int(n), seed=1)
        dev = [torch.from_numpy(a).to(f"cuda:{device}") for a in mesh.arrays()]
        ptrs = [t.data_ptr() for t in dev]
        # one entry per (algorithm, size bucket): LBVH is tuned on 63-bit codes (the launch shapes
        # it picks serve every code width; a second LBVH case would overwrite the entry)
        for algo, kw in ((C.ALGO_LBVH, dict(morton_bits=63)),
                         (C.ALGO_LBVH_PLUS, dict(morton_bits=60, treelet_rounds=1)),
                         (C.ALGO_PLOC, dict(ploc_radius=25))):
            rep = ctx.autotune_build(ptrs, mesh.size(), ctx.params(algo, **kw), stream)
            reports.append({"n": int(n), "algo": algo, "params": kw, "chosen": rep["chosen"],
                            "best_ms": rep["best_ms"], "tree_changing": rep["tree_changing"]})
        del dev
    table = json.loads(ctx.tuning_export())
    table["reports"] = reports
    ctx.close()
    return table


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--sizes", default="100000,1000000,10000000")
    ap.add_argument("--device", type=int, default=0)
    args = ap.parse_args()
    sizes = [int(x) for x in args.sizes.split(",") if x]
    table = tune(sizes, args.device)
    with open(args.out, "w") as f:
        json.dump(table, f, indent=1)
    print(f"wrote {len(table['entries'])} entries to {args.out}")


if __name__ == "__main__":
    main()
