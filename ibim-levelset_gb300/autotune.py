"""Launch-parameter autotuner: times candidate launch parameters (ibim_autotune) on representative
synthetic molecules per Chebyshev order and tube size and writes the table that ibim.py loads
(tuning_gb300.txt beside this file): rows "order min_points near_seg_pairs nearff_seg_pairs
tc_form", a row applying to plans of that order with at least min_points sources.

  python ibim-levelset_gb300/autotune.py [--out PATH] [--reps 5]

Run it on the GPU the library serves; its rows only repartition the same work, so results stay
within parity under any table (tests/test_tuning_gpu.py).
"""

from __future__ import annotations

import argparse
import math
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import ibim  # noqa: E402
import workloads  # noqa: E402

# (order, atoms, h): tube sizes from ~35 k to ~1.6 M points at the orders the configurations use
BUCKETS = [(5, 150, 0.5), (5, 600, 0.5), (5, 2000, 0.5), (5, 2000, 0.25), (4, 300, 0.5), (4, 2000, 0.5),
           (6, 1000, 0.5), (6, 2000, 0.25)]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "tuning_gb300.txt"))
    ap.add_argument("--reps", type=int, default=5)
    args = ap.parse_args()
    lib = ibim.lib()
    lib.ibim_tuning_clear()  # time every candidate against the built-in defaults
    ctx = ibim.Context(0)
    found = {}
    for order, atoms, h in BUCKETS:
        W = workloads.protein(atoms, 8_000_000 + atoms, h=h, order=order)
        r = ctx.autotune(W.mol.centers, W.mol.charges, W.mol.radii, W.config(ibim.PRECISION_MIXED), reps=args.reps)
        found.setdefault(order, []).append(r)
        print(f"order {order} atoms {atoms} h {h}: {r}", flush=True)
    ctx.close()
    lines = ["# order min_points near_seg_pairs nearff_seg_pairs tc_form   (measured cost ms: best / default)"]
    for order in sorted(found):
        rows = sorted(found[order], key=lambda r: r["points"])
        for k, r in enumerate(rows):
            # a row covers sizes from the geometric middle between its molecule and the previous one
            lo = 0 if k == 0 else int(math.sqrt(rows[k - 1]["points"] * r["points"]))
            lines.append(f"{order} {lo} {r['near_seg_pairs']} {r['nearff_seg_pairs']} {r['tc_form']}"
                         f"   # {r['points']} points: {r['best_ms']:.2f} / {r['default_ms']:.2f}")
    with open(args.out, "w") as f:
        f.write("\n".join(lines) + "\n")
    print("\n".join(lines))


if __name__ == "__main__":
    main()
