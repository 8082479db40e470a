"""CPU walks of the register-wave kernels of the mixed-precision solve.

``sc_2022_gb300/csrc/sbp_kernels.cu`` runs three kernels as register waves,
a warp per strip marching along j with two rows per lane:

* ``k_dir_wave``: the CG direction p~ = z + beta p~_old and Ap over the whole
  grid (plain-stencil strips plus a flat walk of the SAT rows and columns);
* ``k_pre_wave``: three smoothing sweeps from zero, the residual and the
  restriction over the interior rectangle of a level's small-tile tiling,
  whose boundary ring of tiles runs as ``PreFusedJob`` beside it;
* ``k_post_wave``: the prolongation and three sweeps over the same kind of
  rectangle, with ``PostFusedJob`` on the ring.

The tests restate each kernel's strip arithmetic, with every constant and
strip-width candidate read from the CUDA source, and check the following for
every candidate width and the grid sizes the solver runs them on:

* the wave's points, together with the ring tiles or the SAT walk, cover
  the level exactly once;
* every load is inside the arrays;
* every stored value lies inside the rows and columns where each stage's
  inputs are real rows and columns. A stage at a warp's edge reads a clamped
  or zero neighbour, so its exact range shrinks by one row or column per
  stage."""
import re
from pathlib import Path

import numpy as np
import pytest

SRC = Path(__file__).resolve().parents[1] / "sc_2022_gb300" / "csrc" / "sbp_kernels.cu"
TEXT = SRC.read_text()


def const(name):
    return int(re.search(rf"constexpr int {name} = (\d+);", TEXT).group(1))


def cands_after(marker):
    body = TEXT[TEXT.index(marker):]
    m = re.search(r"static const int cands\[\] = \{([^}]*)\};", body)
    return [int(v) for v in m.group(1).split(",")]


def geom(name, kind):
    m = re.search(rf"using {name} = {kind}<([^>]*)>;", TEXT)
    return [int(v) for v in m.group(1).split(",")[:2]]


DIR_ROWS = const("kDirRows")
DIR_MIN_N = const("kDirWaveMinN")
WAVE_ROWS = const("kWaveRows")
POST_ROWS = const("kPostRows")
WAVE_MIN_FINE = const("kWaveMinFine")
DIR_CANDS = cands_after("cudaError_t launch_cg_dir_f32(")
PRE_CANDS = cands_after("static cudaError_t launch_pre_wave(")
POST_CANDS = cands_after("    PostWaveArgs a;")
PRE_RI, PRE_RJ = geom("PreSmall", "PreGeom")
POST_TI, POST_TJ = geom("PostSmall", "PostGeom")
LANES = np.arange(32)


def ntiles(n, t):
    return 1 if n <= 1 else (n - 1 + t - 1) // t


def tile_range(t, size, n):
    return (0 if t == 0 else t * size + 1), min(n, (t + 1) * size + 1)


def sat_walk(n):
    """The SAT CTAs' flat walk: rows 0 and n-1, then columns 0, 1, 2, n-3,
    n-2, n-1 of rows 1 .. n-2."""
    k = np.arange(2 * n + 6 * (n - 2))
    i = np.empty_like(k)
    j = np.empty_like(k)
    top = k < 2 * n
    i[top] = np.where(k[top] < n, 0, n - 1)
    j[top] = np.where(k[top] < n, k[top], k[top] - n)
    k2 = k[~top] - 2 * n
    c = k2 // (n - 2)
    i[~top] = 1 + k2 % (n - 2)
    j[~top] = np.where(c < 3, c, n - 6 + c)
    return i, j


# ---------------------------------------------------------------------------
# direction wave (odd n >= kDirWaveMinN; arrays padded, ld > n)
# ---------------------------------------------------------------------------
DIR_SIZES = [n for n in (1025, 1027, 1031, 1089, 1537, 2049, 2051, 4097) if n >= DIR_MIN_N]


@pytest.mark.parametrize("n", DIR_SIZES)
def test_direction_wave_covers_grid_once(n):
    nsi = (n - 2 + DIR_ROWS - 1) // DIR_ROWS
    rb_last = (n - 64 + 1) & ~1
    bi, bj = sat_walk(n)
    for cols in DIR_CANDS:
        nsj = (n - 6 + cols - 1) // cols
        count = np.zeros((n, n), dtype=np.int32)
        np.add.at(count, (bi, bj), 1)
        for si in range(nsi):
            rbn = DIR_ROWS * si
            rb0 = min(rbn, rb_last)
            r_lo, r_hi = rbn + 1, min(rbn + 1 + DIR_ROWS, n - 1)
            ra = rb0 + 2 * LANES
            own_x = (LANES > 0) & (ra >= r_lo) & (ra < r_hi)
            own_y = (LANES < 31) & (ra + 1 >= r_lo) & (ra + 1 < r_hi)
            owned = np.concatenate([ra[own_x], ra[own_y] + 1])
            assert len(np.unique(owned)) == len(owned)
            # loads rows rb0 .. rb0 + 63: the last may be the padding row n
            assert rb0 % 2 == 0 and rb0 >= 0 and rb0 + 63 <= n
            # the stencil of an owned row reads the rows above and below
            # from the warp (one shuffle each way): real rows, in the window
            assert owned.min() - 1 >= rb0 and owned.max() + 1 <= min(rb0 + 63, n - 1)
            for sj in range(nsj):
                c0 = 3 + cols * sj
                c1 = min(c0 + cols, n - 3)
                assert c1 > c0 and c0 - 1 >= 2 and c1 <= n - 3   # loaded columns
                count[owned[:, None], np.arange(c0, c1)[None, :]] += 1
        assert count.min() == 1 and count.max() == 1, (n, cols)


# ---------------------------------------------------------------------------
# pre-smoothing wave on a fine level nf (coarse nc = (nf + 1) / 2)
# ---------------------------------------------------------------------------
def pre_rect(nc):
    ntx, nty = ntiles(nc, PRE_RI), ntiles(nc, PRE_RJ)
    if ntx < 3 or nty < 3 or (nc - 1) % PRE_RI or (nc - 1) % PRE_RJ:
        return None
    Ia, Ib = PRE_RI + 1, PRE_RI * (ntx - 1) + 1
    Ja, Jb = PRE_RJ + 1, PRE_RJ * (nty - 1) + 1
    return (Ia, Ib, Ja, Jb) if Ib - Ia >= WAVE_ROWS and Ja < Jb else None


PRE_SIZES = [nf for nf in (1025, 1057, 1089, 2049, 4097) if nf >= WAVE_MIN_FINE]


@pytest.mark.parametrize("nf", PRE_SIZES)
def test_pre_wave_and_ring_cover_level_once(nf):
    nc = (nf + 1) // 2
    rect = pre_rect(nc)
    assert rect is not None
    Ia, Ib, Ja, Jb = rect
    nsi = (Ib - Ia + WAVE_ROWS - 1) // WAVE_ROWS
    # the ring: PreSmall tiles in the first or last tile row or column; a
    # tile writes f on its coarse range and v on fine rows 2 i_lo .. 2 i_hi - 1
    ntx, nty = ntiles(nc, PRE_RI), ntiles(nc, PRE_RJ)
    fring = np.zeros((nc, nc), dtype=np.int32)
    vring = np.zeros((nf, nf), dtype=np.int32)
    for ti in range(ntx):
        for tj in range(nty):
            if 0 < ti < ntx - 1 and 0 < tj < nty - 1:
                continue
            i0, i1 = tile_range(ti, PRE_RI, nc)
            j0, j1 = tile_range(tj, PRE_RJ, nc)
            fring[i0:i1, j0:j1] += 1
            vring[2 * i0:min(2 * i1 - 1, nf - 1) + 1, 2 * j0:min(2 * j1 - 1, nf - 1) + 1] += 1
    for cols in PRE_CANDS:
        nsj = (Jb - Ja + cols - 1) // cols
        fcount = fring.copy()
        vcount = vring.copy()
        for si in range(nsi):
            In = Ia + WAVE_ROWS * si
            I0 = min(In, Ib - WAVE_ROWS)
            I1 = min(In + WAVE_ROWS, Ib)
            ra = 2 * I0 - 4 + 2 * LANES                 # fine rows ra, ra + 1
            I = I0 + LANES - 2                           # coarse row centred on ra
            own = (LANES >= 2) & (I >= In) & (I < I1)
            # loads of b: fine rows ra, ra + 1 of every lane
            assert ra.min() >= 0 and ra.max() + 1 <= nf - 1
            # exact rows per stage (one fewer at each warp edge per stage):
            # b on the window, v2 one in, v3 two in, the residual three in
            lo, hi = ra.min(), ra.max() + 1
            v3_lo, v3_hi = lo + 2, hi - 2
            r_lo, r_hi = lo + 3, hi - 3
            Io = I[own]
            assert (2 * Io >= v3_lo).all() and (2 * Io + 1 <= v3_hi).all()
            # f at coarse row I reads the residual on fine rows 2I - 1 .. 2I + 1
            assert (2 * Io - 1 >= r_lo).all() and (2 * Io + 1 <= r_hi).all()
            for sj in range(nsj):
                J0 = Ja + cols * sj
                J1 = min(J0 + cols, Jb)
                c_first, c_last = 2 * J0 - 4, 2 * J1 + 2
                assert c_first >= 0 and c_last <= nf - 1         # columns of b loaded
                # stage exactness along j: v3 from c_first + 2, r from c_first + 3;
                # v3 at column x needs b up to x + 2 <= c_last
                vcols = np.arange(2 * J0, 2 * J1)               # v3 stores: c - 2
                assert vcols.min() >= c_first + 2 and vcols.max() + 2 <= c_last
                Js = np.arange(J0, J1)                          # f stores: c - 3 = 2J + 1
                assert (2 * Js - 1 >= c_first + 3).all() and (2 * Js + 1 + 3 <= c_last).all()
                fcount[Io[:, None], Js[None, :]] += 1
                rows = np.concatenate([2 * Io, 2 * Io + 1])
                vcount[rows[:, None], vcols[None, :]] += 1
        assert fcount.min() == 1 and fcount.max() == 1, (nf, cols)
        assert vcount.min() == 1 and vcount.max() == 1, (nf, cols)


# ---------------------------------------------------------------------------
# post-smoothing wave on a fine level n
# ---------------------------------------------------------------------------
def post_rect(n):
    ntx, nty = ntiles(n, POST_TI), ntiles(n, POST_TJ)
    if ntx < 3 or nty < 3 or (n - 1) % POST_TI or (n - 1) % POST_TJ:
        return None
    Ra, Rb = POST_TI + 1, POST_TI * (ntx - 1) + 1
    Ca, Cb = POST_TJ + 1, POST_TJ * (nty - 1) + 1
    return (Ra, Rb, Ca, Cb) if Ra < Rb and Ca < Cb and Rb - Ra >= 4 + POST_ROWS else None


POST_SIZES = [n for n in (1025, 1057, 1089, 2049, 4097) if n >= WAVE_MIN_FINE]


@pytest.mark.parametrize("n", POST_SIZES)
def test_post_wave_and_ring_cover_level_once(n):
    nc = (n + 1) // 2
    rect = post_rect(n)
    assert rect is not None
    Ra, Rb, Ca, Cb = rect
    nsi = (Rb - (Ra & ~1) + POST_ROWS - 1) // POST_ROWS
    ntx, nty = ntiles(n, POST_TI), ntiles(n, POST_TJ)
    ring = np.zeros((n, n), dtype=np.int32)
    for ti in range(ntx):
        for tj in range(nty):
            if 0 < ti < ntx - 1 and 0 < tj < nty - 1:
                continue
            i0, i1 = tile_range(ti, POST_TI, n)
            j0, j1 = tile_range(tj, POST_TJ, n)
            ring[i0:i1, j0:j1] += 1
    for cols in POST_CANDS:
        nsj = (Cb - Ca + cols - 1) // cols
        count = ring.copy()
        for si in range(nsi):
            rbn = (Ra & ~1) - 4 + POST_ROWS * si
            rb0 = min(rbn, (Rb - 4 - POST_ROWS + 1) & ~1)
            r_lo, r_hi = max(rbn + 4, Ra), min(rbn + 4 + POST_ROWS, Rb)
            ra = rb0 + 2 * LANES
            own_x = (ra >= r_lo) & (ra < r_hi)
            own_y = (ra + 1 >= r_lo) & (ra + 1 < r_hi)
            owned = np.concatenate([ra[own_x], ra[own_y] + 1])
            assert len(np.unique(owned)) == len(owned)
            # loads: v_in and b on fine rows rb0 .. rb0 + 63, e on coarse rows
            # rb0 / 2 + lane (the row below by shuffle)
            assert rb0 % 2 == 0 and rb0 >= 0 and rb0 + 63 <= n - 1
            assert rb0 // 2 + 31 <= nc - 1
            # F0 is exact on rows rb0 .. rb0 + 62 (lane 31's odd row lacks the
            # coarse row below), each sweep one row fewer at both edges
            assert owned.min() >= rb0 + 3 and owned.max() <= rb0 + 62 - 3
            for sj in range(nsj):
                c0 = Ca + cols * sj
                c1 = min(c0 + cols, Cb)
                c_first, c_last = c0 - 3, c1 + 2
                assert c_first >= 0 and c_last <= n - 1
                # coarse columns read: J = c >> 1 and J + 1, with J + 2 fetched
                # ahead at every even step
                assert (c_first >> 1) >= 0 and (c_last >> 1) + 2 <= nc - 1
                # sweep 3 at column c - 3 is exact from c_first + 3 and needs F0
                # up to three columns to the right
                assert c0 >= c_first + 3 and (c1 - 1) + 3 <= c_last
                count[owned[:, None], np.arange(c0, c1)[None, :]] += 1
        assert count.min() == 1 and count.max() == 1, (n, cols)
