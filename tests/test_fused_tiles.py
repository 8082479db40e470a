"""CPU walk of the shared-memory indices of the fused V-cycle kernels.

PreFusedJob (pre-smoothing + residual + restriction) and PostFusedJob
(prolongation + post-smoothing) in ``sc_2022_gb300/csrc/sbp_kernels.cu``
stage one box per tile and sweep shrinking regions inside it.  This test
restates their tile and box arithmetic for both tile geometries (the
geometry constants are read from the CUDA source, so the two cannot drift)
and checks, for every tile of every level size and sweep count, that each
point a pass reads or writes lies inside its box, and that each point a
sweep reads was written by the pass before it.  Stencil reads reach one
point in each direction, two next to a side (the SBP boundary closure and
the Dirichlet SAT coupling)."""
import re
from pathlib import Path

import pytest

SRC = Path(__file__).resolve().parents[1] / "sc_2022_gb300" / "csrc" / "sbp_kernels.cu"


def _geometries():
    text = SRC.read_text()
    consts = {k: int(v) for k, v in re.findall(r"constexpr int (RTI|RTJ|TI|TJ) = (\d+);", text)}

    def args(name, kind):
        m = re.search(rf"using {name} = {kind}<([^>]*)>;", text)
        assert m, name
        vals = [a.strip() for a in m.group(1).split(",")]
        # the box dimensions; a trailing flag (interior path on/off) is not geometry
        return [consts[a] if a in consts else int(a) for a in vals if a not in ("true", "false")]

    return {"pre": {"large": args("PreLarge", "PreGeom"), "small": args("PreSmall", "PreGeom")},
            "post": {"large": args("PostLarge", "PostGeom"),
                     "small": args("PostSmall", "PostGeom")}}


GEOM = _geometries()
SIZES = [3, 5, 9, 17, 33, 65, 129, 257]


def ntiles(n, t):
    return 1 if n <= 1 else (n - 1 + t - 1) // t


def tile_range(t, size, n):
    """Tile t of a dimension covers [t*size + (t > 0), (t+1)*size + 1) clipped to n."""
    return (0 if t == 0 else t * size + 1), min(n, (t + 1) * size + 1)


def neighbours(i, j, n):
    out = []
    for d in (-2, -1, 1, 2):
        if abs(d) == 2 and not (i <= 2 or i >= n - 3):
            continue
        if 0 <= i + d < n:
            out.append((i + d, j))
    for d in (-2, -1, 1, 2):
        if abs(d) == 2 and not (j <= 2 or j >= n - 3):
            continue
        if 0 <= j + d < n:
            out.append((i, j + d))
    return out


def region(i0, i1, j0, j1):
    return {(i, j) for i in range(i0, i1 + 1) for j in range(j0, j1 + 1)}


def walk_pre(geom, nf, sweeps):
    RI, RJ, BI, BJ = geom
    nc = (nf + 1) // 2
    for ti in range(ntiles(nc, RI)):
        for tj in range(ntiles(nc, RJ)):
            ilo, ihi = tile_range(ti, RI, nc)
            jlo, jhi = tile_range(tj, RJ, nc)
            X0, Y0 = 2 * RI * ti - 4, 2 * RJ * tj - 4

            def inside(p):
                a, b = p[0] - X0, p[1] - Y0
                assert 0 <= a < BI and 0 <= b < BJ, (nf, ti, tj, p)

            ri0, ri1, rj0, rj1 = 2 * ilo - 1, 2 * ihi - 1, 2 * jlo - 1, 2 * jhi - 1
            lo = lambda v, h: max(v - h, 0)          # noqa: E731
            hi = lambda v, h: min(v + h, nf - 1)     # noqa: E731
            prev = region(lo(ri0, sweeps), hi(ri1, sweeps), lo(rj0, sweeps), hi(rj1, sweeps))
            for p in prev:
                inside(p)
            for sw in range(2, sweeps + 1):
                h = sweeps - sw + 1
                cur = region(lo(ri0, h), hi(ri1, h), lo(rj0, h), hi(rj1, h))
                for p in cur:
                    inside(p)
                    for q in neighbours(*p, nf):
                        inside(q)
                        assert q in prev, (nf, ti, tj, sw, p, q)
                prev = cur
            res = region(max(ri0, 0), min(ri1, nf - 1), max(rj0, 0), min(rj1, nf - 1))
            for p in res:
                inside(p)
                for q in neighbours(*p, nf):
                    inside(q)
                    assert q in prev, (nf, ti, tj, "residual", p, q)
            for I in range(ilo, ihi):
                for J in range(jlo, jhi):
                    for a in (-1, 0, 1):
                        for b in (-1, 0, 1):
                            p = (2 * I + a, 2 * J + b)
                            if 0 <= p[0] < nf and 0 <= p[1] < nf:
                                assert p in res, (nf, ti, tj, "restriction", I, J, p)


def walk_post(geom, n, sweeps):
    TI, TJ, BI, BJ, CI, CJ = geom
    nc = (n + 1) // 2
    for ti in range(ntiles(n, TI)):
        for tj in range(ntiles(n, TJ)):
            ilo, ihi = tile_range(ti, TI, n)
            jlo, jhi = tile_range(tj, TJ, n)
            X0, Y0 = TI * ti - 4, jlo - 4
            XC, YC = (TI // 2) * ti - 4, (jlo - 4) >> 1

            def inside(p):
                a, b = p[0] - X0, p[1] - Y0
                assert 0 <= a < BI and 0 <= b < BJ, (n, ti, tj, p)

            lo = lambda v, h: max(v - h, 0)          # noqa: E731
            hi = lambda v, h: min(v + h, n - 1)      # noqa: E731
            ti0, ti1, tj0, tj1 = ilo, ihi - 1, jlo, jhi - 1
            prev = region(lo(ti0, sweeps), hi(ti1, sweeps), lo(tj0, sweeps), hi(tj1, sweeps))
            for (i, j) in prev:
                inside((i, j))
                for da in ((0, 1) if i & 1 else (0,)):
                    for db in ((0, 1) if j & 1 else (0,)):
                        ci, cj = (i >> 1) + da, (j >> 1) + db
                        assert ci < nc and cj < nc
                        assert 0 <= ci - XC < CI and 0 <= cj - YC < CJ, (n, ti, tj, i, j)
            for sw in range(1, sweeps):
                h = sweeps - sw
                cur = region(lo(ti0, h), hi(ti1, h), lo(tj0, h), hi(tj1, h))
                for p in cur:
                    inside(p)
                    for q in neighbours(*p, n):
                        inside(q)
                        assert q in prev, (n, ti, tj, sw, p, q)
                prev = cur
            for p in region(ti0, ti1, tj0, tj1):
                inside(p)
                if sweeps > 0:
                    for q in neighbours(*p, n):
                        inside(q)
                        assert q in prev, (n, ti, tj, "last", p, q)


@pytest.mark.parametrize("name", ["large", "small"])
@pytest.mark.parametrize("sweeps", [1, 2, 3])
def test_pre_fused_tiles_stay_in_their_boxes(name, sweeps):
    for nf in SIZES:
        walk_pre(GEOM["pre"][name], nf, sweeps)


@pytest.mark.parametrize("name", ["large", "small"])
@pytest.mark.parametrize("sweeps", [0, 1, 2, 3])
def test_post_fused_tiles_stay_in_their_boxes(name, sweeps):
    for n in SIZES:
        walk_post(GEOM["post"][name], n, sweeps)


def test_walk_catches_a_short_box():
    # the walk itself must fail on a box one point too small
    RI, RJ, BI, BJ = GEOM["pre"]["small"]
    with pytest.raises(AssertionError):
        walk_pre((RI, RJ, BI, BJ - 1), 65, 3)
    TI, TJ, BI, BJ, CI, CJ = GEOM["post"]["small"]
    with pytest.raises(AssertionError):
        walk_post((TI, TJ, BI - 1, BJ, CI, CJ), 65, 3)
