"""Generate the golden fixtures in tests/golden/ from the CPU oracle.

The reference (Julia) cannot run here and commits no data files, so the
fixtures are produced by the numpy/scipy restatement in oracle/sbp_oracle.py
and pin it against later drift.  Run from the repository root:
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import math
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import sbp_oracle as o  # noqa: E402

OUT = Path(__file__).resolve().parent


def main():
    rng = np.random.default_rng(20221116)
    data = {}
    for n in (3, 5, 9, 17, 33):
        u = rng.standard_normal(n * n)
        data[f"apply_u_{n}"] = u
        data[f"apply_negAu_{n}"] = o.neg_A_matrix_free(u, n)
        data[f"diagA_{n}"] = o.assemble(n).A.diagonal()
    for n in (5, 9, 17, 33):
        r = rng.standard_normal(n * n)
        data[f"restrict_in_{n}"] = r
        for kind in o.RESTRICT_KINDS:
            data[f"restrict_{kind}_{n}"] = o.restriction_2d(n, kind) @ r
        nc = (n + 1) // 2
        e = rng.standard_normal(nc * nc)
        data[f"prolong_in_{nc}"] = e
        data[f"prolong_{nc}"] = o.prolongation_2d(nc) @ e
    for n in (9, 17, 33):
        asm = o.assemble(n)
        f = rng.standard_normal(n * n)
        g = {k: rng.standard_normal(n) for k in "WESN"}
        data[f"rhs_f_{n}"] = f
        for k in "WESN":
            data[f"rhs_g{k}_{n}"] = g[k]
        data[f"rhs_b_{n}"] = asm.rhs(f, g)
    # solver histories
    n = 33
    asm = o.assemble(n)
    F, g, U = o.manufactured(n, "reference")
    b = asm.rhs(F, g)
    data["ref33_b"] = b
    hier = o.Hierarchy(n, o.MGOptions.reference_two_level(n))
    x, it, norms = o.mgcg(hier, b)
    data["ref33_mgcg2_norms"] = np.array(norms)
    data["ref33_mgcg2_x"] = x
    x, it, norms = o.cg(asm.A, b)
    data["ref33_cg_norms"] = np.array(norms)
    data["ref33_cg_x"] = x
    n = 65
    asm = o.assemble(n)
    F, g, U = o.manufactured(n, "baseline")
    b = asm.rhs(F, g)
    data["base65_b"] = b
    hier = o.Hierarchy(n, o.MGOptions(coarse_n=17))
    x, it, norms = o.mgcg(hier, b, reltol=1e-10)
    data["base65_vcycle17_norms"] = np.array(norms)
    data["base65_vcycle17_x"] = x
    data["base65_vcycle17_z"] = hier.vcycle(b)
    np.savez_compressed(OUT / "sbp_golden.npz", **data)
    print(f"wrote {OUT / 'sbp_golden.npz'} ({len(data)} arrays)")


if __name__ == "__main__":
    main()
