"""CPU walk of the FP32 operator-apply wave's work split and register queue.

``k_apply_wave`` in ``sc_2022_gb300/csrc/sbp_kernels.cu`` splits the plain
5-point interior (rows 1 .. n-2, columns 3 .. n-4) into strips of
kApplyRows rows x `cols` columns, a warp per strip with two rows per lane,
and leaves the SAT rows and columns to extra CTAs that walk a flat index.
Each warp marches along j with its columns in a register queue kApplyAhead
deep.  This test restates that arithmetic (the constants and the strip-width
candidates are read from the CUDA source, so the two cannot drift) and
checks, for every candidate width and many grid sizes, that:

* every point of the grid is written exactly once, by a strip or by the
  boundary walk;
* every column a warp loads lies in 0 .. n-1, and each is loaded once, in
  order;
* every owned row's neighbours above and below are real rows of the loaded
  window, not clamped copies;
* the queue slot a step reads holds that step's column."""
import re
from pathlib import Path

import numpy as np
import pytest

SRC = Path(__file__).resolve().parents[1] / "sc_2022_gb300" / "csrc" / "sbp_kernels.cu"
TEXT = SRC.read_text()
ROWS = int(re.search(r"constexpr int kApplyRows = (\d+);", TEXT).group(1))
AHEAD = int(re.search(r"constexpr int kApplyAhead = (\d+);", TEXT).group(1))
_launch = TEXT[TEXT.index("static cudaError_t launch_apply_wave("):]
CANDS = [int(v) for v in
         re.search(r"static const int cands\[\] = \{([^}]*)\};", _launch).group(1).split(",")]

SIZES = [65, 66, 67, 100, 127, 128, 129, 130, 190, 191, 255, 256, 257, 500, 513, 1024, 1025,
         1031, 2049]


def march(S, D):
    """Replay the kernel's queue march for a strip of S output columns.

    Returns the loaded columns (relative to c0 - 1, in issue order) and, per
    step, the column the step's q0 holds."""
    loads = []

    def load():
        loads.append(len(loads))
        return loads[-1]

    load()                       # q2: column c0 - 1
    load()                       # q1: column c0
    qb = [load() if k < S else None for k in range(D)]
    used = []
    s = 0
    while s + 2 * D <= S:        # whole chunks, unguarded refills
        for k in range(D):
            used.append(qb[k])
            qb[k] = load()
        s += D
    while s < S:                 # the guarded tail
        for k in range(D):
            if s + k < S:
                used.append(qb[k])
                if s + k + D < S:
                    qb[k] = load()
        s += D
    return loads, used


@pytest.mark.parametrize("S", list(range(1, 3 * AHEAD + 3)) + [40, 64, 96, 128])
def test_queue_march_delivers_columns_in_order(S):
    loads, used = march(S, AHEAD)
    # columns c0 - 1 .. c0 + S (= c1) loaded once each, in order
    assert loads == list(range(S + 2))
    # step t reads column c0 + 1 + t (relative index t + 2)
    assert used == [t + 2 for t in range(S)]


def boundary_points(n):
    """The boundary CTAs' flat walk: rows 0 and n-1, then columns 0, 1, 2,
    n-3, n-2, n-1 of rows 1 .. n-2."""
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


@pytest.mark.parametrize("n", SIZES)
def test_strips_and_boundary_cover_the_grid_once(n):
    nsi = (n - 2 + ROWS - 1) // ROWS
    lanes = np.arange(32)
    bi, bj = boundary_points(n)
    for cols in CANDS:
        nsj = (n - 6 + cols - 1) // cols
        count = np.zeros((n, n), dtype=np.int32)
        np.add.at(count, (bi, bj), 1)
        for si in range(nsi):
            rb0 = ROWS * si
            r_hi = min(rb0 + 1 + ROWS, n - 1)
            rown = rb0 + 2 * lanes
            own_x = (lanes > 0) & (rown < r_hi)
            own_y = (lanes < 31) & (rown + 1 < r_hi)
            owned = np.concatenate([rown[own_x], rown[own_y] + 1])
            assert len(np.unique(owned)) == len(owned)
            # the loaded window: lane l holds rows min(rown, n-1), min(rown+1, n-1)
            window = np.stack([np.minimum(rown, n - 1), np.minimum(rown + 1, n - 1)], 1).ravel()
            assert window.min() >= 0 and window.max() <= n - 1
            exact = {r for r, w in zip(range(rb0, rb0 + 64), window) if r == w}
            for r in owned:
                assert r - 1 in exact and r + 1 in exact, (n, cols, si, r)
            for sj in range(nsj):
                c0 = 3 + cols * sj
                c1 = min(c0 + cols, n - 3)
                assert c1 > c0
                assert c0 - 1 >= 0 and c1 <= n - 1   # loaded columns c0 - 1 .. c1
                count[owned[:, None], np.arange(c0, c1)[None, :]] += 1
        assert count.min() == 1 and count.max() == 1, (n, cols)
