"""Generates treelet_dp_unrolled.cuh: the LBVH+ subset DP for N = 4..7 treelet leaves as
straight-line code, so that every subset cost lives in a register.

The DP is the one of optimizeTreeletSerial (src/cuda/lbvh_plus_builder.cu:119-165): subsets in
increasing numeric order (every proper subset comes first); cost[s] = min over splits of
cost[p] + cost[s ^ p], plus the area of s; single leaves cost 0.  The splits of s are the
nonempty subsets p of s without its lowest member, in increasing order, and the first minimum
is kept (a strict < from INF, so a subset whose splits all cost >= INF keeps INF and no split).
Subsets with four or more splits run two first-minimum chains over the two halves of their
splits, interleaved, and keep the second half's minimum only if it is strictly smaller: the same
result with half the dependency depth.

Run from this directory:  python gen_treelet_dp.py > treelet_dp_unrolled.cuh
"""
import sys


def subsets_of(mask):
    """Nonempty subsets of mask in increasing numeric order."""
    out = []
    p = mask & -mask
    while p:
        out.append(p)
        p = (p - mask) & mask
    return out


def emit(n, w):
    full = (1 << n) - 1
    w(f"// {n} leaves: {sum(len(subsets_of(s & (s - 1))) for s in range(1, full + 1) if bin(s).count('1') > 1)} "
      f"split evaluations.\n")
    w(f"__device__ __forceinline__ void dp_unrolled_{n}(const float* __restrict__ A, uint8_t* __restrict__ P) {{\n")
    for s in range(1, full + 1):
        if bin(s).count("1") == 1:
            w(f"  const float c{s} = 0.0f;\n")
            continue
        delta = s & (s - 1)
        last = s == full  # only its best split is needed
        splits = subsets_of(delta)
        w(("" if last else f"  float c{s};\n") + "  {\n")
        if len(splits) < 4:
            w("    float b = kTlInf, v;\n    uint32_t bp = 0xffu;\n")
            for p in splits:
                w(f"    v = __fadd_rn(c{p}, c{s ^ p});\n    if (v < b) {{ b = v; bp = {p}u; }}\n")
        else:
            # two independent first-minimum chains over the first and the second half of the
            # splits, interleaved; the second wins only if strictly smaller, so the first
            # minimum in split order is kept
            h = (len(splits) + 1) // 2
            a, z = splits[:h], splits[h:]
            w("    float b = kTlInf, b2 = kTlInf, v, v2;\n    uint32_t bp = 0xffu, bp2 = 0xffu;\n")
            for k in range(h):
                p = a[k]
                w(f"    v = __fadd_rn(c{p}, c{s ^ p});\n    if (v < b) {{ b = v; bp = {p}u; }}\n")
                if k < len(z):
                    q = z[k]
                    w(f"    v2 = __fadd_rn(c{q}, c{s ^ q});\n    if (v2 < b2) {{ b2 = v2; bp2 = {q}u; }}\n")
            w("    if (b2 < b) { b = b2; bp = bp2; }\n")
        if not last:
            w(f"    c{s} = __fadd_rn(b, A[{s} * 32]);\n")
        w(f"    P[{s} * 32] = (uint8_t)bp;\n  }}\n")
    w("}\n\n")


def main():
    w = sys.stdout.write
    w("// treelet_dp_unrolled.cuh -- generated by gen_treelet_dp.py; do not edit.\n")
    w("//\n// The LBVH+ subset DP (src/cuda/lbvh_plus_builder.cu:119-165) for N = 4..7 treelet leaves\n")
    w("// as straight-line code: subset costs in registers, areas A and best splits P in this\n")
    w("// lane's shared-memory columns (stride 32).  Leaves beyond a treelet's own count are\n")
    w("// never part of its subsets, so a smaller treelet can run a larger N.\n")
    w("#pragma once\n\nnamespace bvhgb {\n\n")
    for n in (4, 5, 6, 7):
        emit(n, w)
    w("}  // namespace bvhgb\n")


if __name__ == "__main__":
    main()
