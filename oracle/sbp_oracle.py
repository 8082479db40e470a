"""CPU oracle for the matrix-free SBP-SAT Poisson solver path.

TEST INFRASTRUCTURE ONLY.  This module restates, in numpy/scipy, the
reference's algorithms for the hot path so that the CUDA library can be
checked against them.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import it,
and only as the checker.  The product library never calls into it.

Reference files restated here (paths inside AlexandreChern/SC_2022):

* ``diagonal_sbp.jl:56-147``   ``diagonal_sbp_D1`` (p=2 branch, H norm)
* ``diagonal_sbp.jl:189-197, 414-452`` ``diagonal_sbp_D2`` (p=2: D2, S0, SN)
* ``preconditioned_CG/level_2_multigrid_new.jl:48-123`` ``Operators_2d``
* ``preconditioned_CG/level_2_multigrid_new.jl:125-188`` ``Assembling_matrix``
* ``preconditioned_CG/level_2_multigrid_new.jl:190-246`` transfer matrices
* ``preconditioned_CG/level_2_multigrid_new.jl:258-291`` ``CG_CPU``
* ``preconditioned_CG/level_2_multigrid_new.jl:335-350`` Jacobi / Richardson
* ``preconditioned_CG/level_2_multigrid_new.jl:358-382`` ``Two_level_multigrid``
* ``preconditioned_CG/level_2_multigrid_new.jl:480-524`` ``mg_preconditioned_CG``
* ``split_matrix_free.jl:32-49, 324-486`` ``matrix_free_A_full_GPU`` (the -A apply)
* ``diagonal_sbp.jl:198-222`` p = 4 and p = 6 branches of ``diagonal_sbp_D2``
* ``diagonal_sbp.jl:462-495, 709-740`` ``variable_diagonal_sbp_D2`` (p = 2)
* ``preconditioned_CG/legacy_functions.jl:100-174`` ``get_operators`` (2D
  assembly from the variable-coefficient D2)
* ``preconditioned_CG/matrix_free_mg_cg.jl:17-38, 80-94`` matrix-free transfers

Parity pin: the reference is Julia and no Julia toolchain exists here, and
the reference commits no golden vectors.  The oracle is pinned by the
reference's own in-code cross checks, restated: the matrix-free -A apply
equals the kron-assembled operator (``split_matrix_free.jl:517``), the
matrix-free transfers equal the kron matrices
(``matrix_free_mg_cg.jl:636-646``), plus second-order convergence of the
discretisation error against the manufactured solution
(``matrix_free_mg_cg.jl:464``).  Parity against reference *outputs* is
therefore unpinned.

Grid convention (the reference's, Julia column-major): a grid function on
n x n points is a flat vector with element (i, j) at ``j*n + i``; i is the
fast index (x in the reference's ``u(x, y')``), j the slow index.  In numpy
a grid is held as ``U[j, i]`` (shape (n, n), C order), which has the same
flat order.  The reference's "W/E" sides (Dirichlet) are j = 0 / j = n-1,
its "S/N" sides (Neumann) are i = 0 / i = n-1.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

# Penalty parameters hard-coded by the reference
# (level_2_multigrid_new.jl:145-150; split_matrix_free.jl:453-455).
TAU_D_TIMES_H = -13.0   # tau_W = tau_E = -13/h
TAU_N = -1.0            # tau_S = tau_N
BETA = 1.0
# Dirichlet SAT coefficients on the three columns next to a Dirichlet side,
# after H-tilde scaling: (h*tau + 1.5*beta, -2*beta, 0.5*beta).
DIRICHLET_COEF = (TAU_D_TIMES_H + 1.5 * BETA, -2.0 * BETA, 0.5 * BETA)


# --------------------------------------------------------------------------
# 1D SBP operators, p = 2
# --------------------------------------------------------------------------
def sbp_1d(n: int):
    """1D second-order diagonal-norm SBP pieces on n points of [0, 1].

    Follows ``diagonal_sbp.jl:56-61,112-146`` (D1 norm H: bhinv = [2] so
    H = h*diag(1/2, 1, ..., 1, 1/2)) and ``diagonal_sbp.jl:191-197,414-452``
    (D2 with the one-sided boundary rows equal to the interior stencil,
    S0 = -BS/h on row 1, SN = BS/h on row n with BS = [3/2, -2, 1/2]).
    Returns (D2, H, HI, BS) as scipy CSR matrices (BS = SN - S0).
    """
    if n < 3:
        raise ValueError("SBP p=2 operator needs n >= 3")
    h = 1.0 / (n - 1)
    rows, cols, vals = [], [], []
    for r in range(n):
        if r == 0:
            c = (0, 1, 2)
        elif r == n - 1:
            c = (n - 1, n - 2, n - 3)
        else:
            c = (r - 1, r, r + 1)
        w = (1.0, -2.0, 1.0) if r in (0, n - 1) else (1.0, -2.0, 1.0)
        rows += [r, r, r]
        cols += list(c)
        vals += [v / h**2 for v in w]
    D2 = sp.csr_matrix((vals, (rows, cols)), shape=(n, n))
    hv = np.ones(n)
    hv[0] = hv[-1] = 0.5
    H = sp.diags(h * hv).tocsr()
    HI = sp.diags(1.0 / (h * hv)).tocsr()
    bs = np.array([1.5, -2.0, 0.5]) / h
    S0 = sp.csr_matrix((-bs, ([0, 0, 0], [0, 1, 2])), shape=(n, n))
    SN = sp.csr_matrix((bs, ([n - 1] * 3, [n - 1, n - 2, n - 3])), shape=(n, n))
    BS = (SN - S0).tocsr()
    return D2, H, HI, BS


# --------------------------------------------------------------------------
# 1D SBP operators, p = 4 and p = 6
# --------------------------------------------------------------------------
# diagonal_sbp.jl, the p == 4 and p == 6 branches of diagonal_sbp_D2
# (:198-222) and diagonal_sbp_D1 (:62-79): norm weights H = h / bhinv on the
# first and last bm points, the interior D2 stencil d, the bm x bn boundary
# closure bd (mirrored at the far end with the same values), and the boundary
# derivative BS.  Fractions are written as the reference writes them.
P4_BHINV = (48 / 17, 48 / 59, 48 / 43, 48 / 49)
P4_D = (-1 / 12, 4 / 3, -5 / 2, 4 / 3, -1 / 12)
P4_BD = ((2.0, -5.0, 4.0, -1.0, 0.0, 0.0),
         (1.0, -2.0, 1.0, 0.0, 0.0, 0.0),
         (-4 / 43, 59 / 43, -110 / 43, 59 / 43, -4 / 43, 0.0),
         (-1 / 49, 0.0, 59 / 49, -118 / 49, 64 / 49, -4 / 49))
P4_BS = (11 / 6, -3.0, 3 / 2, -1 / 3)

P6_BHINV = (43200 / 13649, 8640 / 12013, 4320 / 2711, 4320 / 5359, 8640 / 7877, 43200 / 43801)
P6_D = (1 / 90, -3 / 20, 3 / 2, -49 / 18, 3 / 2, -3 / 20, 1 / 90)
P6_BD = (
    (114170 / 40947, -438107 / 54596, 336409 / 40947, -276997 / 81894, 3747 / 13649,
     21035 / 163788, 0.0, 0.0, 0.0),
    (6173 / 5860, -2066 / 879, 3283 / 1758, -303 / 293, 2111 / 3516, -601 / 4395, 0.0, 0.0, 0.0),
    (-52391 / 81330, 134603 / 32532, -21982 / 2711, 112915 / 16266, -46969 / 16266,
     30409 / 54220, 0.0, 0.0, 0.0),
    (68603 / 321540, -12423 / 10718, 112915 / 32154, -75934 / 16077, 53369 / 21436,
     -54899 / 160770, 48 / 5359, 0.0, 0.0),
    (-7053 / 39385, 86551 / 94524, -46969 / 23631, 53369 / 15754, -87904 / 23631,
     820271 / 472620, -1296 / 7877, 96 / 7877, 0.0),
    (21035 / 525612, -24641 / 131403, 30409 / 87602, -54899 / 131403, 820271 / 525612,
     -117600 / 43801, 64800 / 43801, -6480 / 43801, 480 / 43801))
P6_BS = (25 / 12, -4.0, 3.0, -4 / 3, 1 / 4)

HIGH_ORDER = {4: (P4_BHINV, P4_D, P4_BD, P4_BS), 6: (P6_BHINV, P6_D, P6_BD, P6_BS)}


def high_order_min_n(p: int) -> int:
    """Smallest grid the reference accepts (diagonal_sbp.jl:417-420:
    N + 1 >= max(bn, 2 bm))."""
    bhinv, _, bd, _ = HIGH_ORDER[p]
    return max(len(bd[0]), 2 * len(bhinv))


def sbp_1d_high(n: int, p: int):
    """1D diagonal-norm SBP pieces of order p in {4, 6} on n points of
    [0, 1] (``diagonal_sbp.jl:198-222, 414-452`` for D2/S0/SN; ``:62-79,
    112-146`` for the norm H).  Returns (D2, H, HI, BS) as scipy CSR."""
    bhinv, d, bd, bsv = HIGH_ORDER[p]
    bm, bn, half = len(bhinv), len(bd[0]), len(d) // 2
    if n < high_order_min_n(p):
        raise ValueError(f"SBP p={p} operator needs n >= {high_order_min_n(p)}")
    h = 1.0 / (n - 1)
    rows, cols, vals = [], [], []
    for r in range(bm, n - bm):
        for k, c in enumerate(d):
            rows.append(r)
            cols.append(r - half + k)
            vals.append(c / h**2)
    for r in range(bm):
        for c in range(bn):
            if bd[r][c] != 0.0:
                rows += [r, n - 1 - r]
                cols += [c, n - 1 - c]
                vals += [bd[r][c] / h**2] * 2
    D2 = sp.csr_matrix((vals, (rows, cols)), shape=(n, n))
    hv = np.ones(n)
    for k in range(bm):
        hv[k] = hv[n - 1 - k] = 1.0 / bhinv[k]
    H = sp.diags(h * hv).tocsr()
    HI = sp.diags(1.0 / (h * hv)).tocsr()
    bs = np.array(bsv) / h
    nb = len(bsv)
    S0 = sp.csr_matrix((-bs, ([0] * nb, list(range(nb)))), shape=(n, n))
    SN = sp.csr_matrix((bs, ([n - 1] * nb, [n - 1 - k for k in range(nb)])), shape=(n, n))
    BS = (SN - S0).tocsr()
    return D2, H, HI, BS


def sbp_1d_p4(n: int):
    """The p = 4 pieces (:func:`sbp_1d_high` with p = 4)."""
    return sbp_1d_high(n, 4)


def _e(k: int, n: int):
    return sp.csr_matrix(([1.0], ([k], [0])), shape=(n, 1))


@dataclass
class Assembled:
    """Result of :func:`assemble` (``Assembling_matrix`` restated)."""
    n: int
    A: sp.csr_matrix            # SPD, = -H~ (D2 + SAT)
    H_tilde: sp.csr_matrix
    sat_r: dict                 # side -> n^2 x n sparse map of boundary data
    h: float = field(init=False)

    def __post_init__(self):
        self.h = 1.0 / (self.n - 1)

    def rhs(self, f_ref: np.ndarray, g: dict) -> np.ndarray:
        """b = -H~ (f_ref + sum_side SAT_side_r g_side)  (``:182-185``).

        ``f_ref`` is the D2-convention source (Delta u = f_ref), flat.
        ``g`` maps 'W','E','S','N' to length-n boundary vectors.
        """
        acc = np.asarray(f_ref, dtype=np.float64).ravel().copy()
        for side in ("W", "E", "S", "N"):
            acc += self.sat_r[side] @ np.asarray(g[side], dtype=np.float64)
        return -(self.H_tilde @ acc)


def assemble(n: int, p: int = 2) -> Assembled:
    """Restates ``Operators_2d`` + ``Assembling_matrix``
    (``level_2_multigrid_new.jl:48-188``) for N_x = N_y = n - 1 intervals and
    SBP order p (2, 4 or 6; the penalty parameters are the same for all, as
    in the reference).

    kron(X, I) acts on the slow index j, kron(I, X) on the fast index i.
    """
    if p == 2:
        D2x, H1x, HIx, BSx = sbp_1d(n)
    elif p in HIGH_ORDER:
        D2x, H1x, HIx, BSx = sbp_1d_high(n, p)
    else:
        raise ValueError("only p = 2, 4 and 6 are restated")
    D2y, H1y, HIy, BSy = D2x, H1x, HIx, BSx
    I = sp.identity(n, format="csr")
    e1 = _e(0, n)
    eN = _e(n - 1, n)
    E1 = sp.diags(e1.toarray().ravel()).tocsr()
    EN = sp.diags(eN.toarray().ravel()).tocsr()

    e_E = sp.kron(eN, I).tocsr()
    e_W = sp.kron(e1, I).tocsr()
    e_S = sp.kron(I, e1).tocsr()
    e_N = sp.kron(I, eN).tocsr()
    E_E = sp.kron(EN, I).tocsr()
    E_W = sp.kron(E1, I).tocsr()
    E_S = sp.kron(I, E1).tocsr()
    E_N = sp.kron(I, EN).tocsr()

    D2 = (sp.kron(D2x, I) + sp.kron(I, D2y)).tocsr()
    HI_x = sp.kron(HIx, I).tocsr()
    HI_y = sp.kron(I, HIy).tocsr()
    BS_x = sp.kron(BSx, I).tocsr()
    BS_y = sp.kron(I, BSy).tocsr()
    H_tilde = sp.kron(H1x, H1y).tocsr()

    h = 1.0 / (n - 1)
    tau_E = tau_W = TAU_D_TIMES_H / h
    tau_N = tau_S = TAU_N
    beta = BETA

    SAT_W = tau_W * HI_x @ E_W + beta * HI_x @ BS_x.T @ E_W
    SAT_E = tau_E * HI_x @ E_E + beta * HI_x @ BS_x.T @ E_E
    SAT_S = tau_S * HI_y @ E_S @ BS_y
    SAT_N = tau_N * HI_y @ E_N @ BS_y

    sat_r = {
        "W": (tau_W * HI_x @ E_W @ e_W + beta * HI_x @ BS_x.T @ E_W @ e_W).tocsr(),
        "E": (tau_E * HI_x @ E_E @ e_E + beta * HI_x @ BS_x.T @ E_E @ e_E).tocsr(),
        "S": (tau_S * HI_y @ E_S @ e_S).tocsr(),
        "N": (tau_N * HI_y @ E_N @ e_N).tocsr(),
    }
    A = D2 + SAT_W + SAT_E + SAT_S + SAT_N
    A = (-(H_tilde @ A)).tocsr()
    A.eliminate_zeros()
    A.sort_indices()
    return Assembled(n=n, A=A, H_tilde=H_tilde, sat_r=sat_r)


# --------------------------------------------------------------------------
# Variable-coefficient operator, p = 2
# --------------------------------------------------------------------------
def variable_sbp_1d(n: int, c) -> tuple:
    """``variable_diagonal_sbp_D2(2, N, B)`` (``diagonal_sbp.jl:470-495,
    709-740``) on n points of [0, 1] with nodal coefficients c (length n):
    M symmetric with face values (c_k + c_k+1)/2, S0 = -c_0 BS/h on the first
    row, SN = c_n-1 BS/h on the last (BS = (3/2, -2, 1/2)), and
    D = HI (-M + SN - S0).  Returns (D, S0, SN, HI, H, M), scipy CSR."""
    c = np.asarray(c, dtype=np.float64).ravel()
    assert c.size == n and n >= 3
    h = 1.0 / (n - 1)
    face = 0.5 * (c[:-1] + c[1:])                 # c_{k+1/2}
    diag = np.zeros(n)
    diag[:-1] += face
    diag[1:] += face
    M = sp.diags([-face, diag, -face], [-1, 0, 1], shape=(n, n)).tocsr() / h
    bs = np.array([1.5, -2.0, 0.5])
    S0 = sp.csr_matrix((-c[0] * bs / h, ([0, 0, 0], [0, 1, 2])), shape=(n, n))
    SN = sp.csr_matrix((c[-1] * bs / h, ([n - 1] * 3, [n - 1, n - 2, n - 3])), shape=(n, n))
    hv = np.ones(n)
    hv[0] = hv[-1] = 0.5
    H = sp.diags(h * hv).tocsr()
    HI = sp.diags(1.0 / (h * hv)).tocsr()
    D = (HI @ (-M + SN - S0)).tocsr()
    return D, S0, SN, HI, H, M


def assemble_variable(n: int, c) -> Assembled:
    """Second-order SBP-SAT operator for div(c grad u) = f_ref on the n x n
    grid, nodal coefficients c (flat, i fast), with the SATs of
    ``Assembling_matrix`` (``level_2_multigrid_new.jl:125-188``): Dirichlet
    on the slow-index sides W/E, Neumann on the fast-index sides S/N.  Each
    grid line carries the 1D operator of :func:`variable_sbp_1d` built from
    that line's coefficients (the 2D assembly of ``get_operators``,
    ``legacy_functions.jl:100-174``, which the reference runs with c = 1).
    The coefficient enters the SATs through the boundary derivative
    (SN - S0 carry c) and the Dirichlet penalty tau_D * c at the boundary
    point; with c = 1 the matrix is :func:`assemble`'s.  A = -H~ (D2 + SAT)
    is symmetric positive definite for c > 0."""
    c = np.asarray(c, dtype=np.float64).reshape(n, n)   # [j, i]
    h = 1.0 / (n - 1)
    tau_d = TAU_D_TIMES_H / h
    N = n * n
    # fast direction i (Neumann, tau_N = -1 on the boundary flux), per j
    rows_fast = []
    for j in range(n):
        D, S0, SN, HI, H, M = variable_sbp_1d(n, c[j, :])
        E = sp.diags(np.r_[1.0, np.zeros(n - 2), 1.0]).tocsr()
        rows_fast.append(D + TAU_N * HI @ E @ (SN - S0))
    L_fast = sp.block_diag(rows_fast).tocsr()
    # slow direction j (Dirichlet), per i, assembled on the transposed
    # ordering and permuted back
    rows_slow = []
    sat_w, sat_e = [], []
    for i in range(n):
        D, S0, SN, HI, H, M = variable_sbp_1d(n, c[:, i])
        BS = (SN - S0).tocsr()
        e1 = np.zeros(n)
        e1[0] = 1.0
        en = np.zeros(n)
        en[-1] = 1.0
        E1, En = sp.diags(e1).tocsr(), sp.diags(en).tocsr()
        pen = tau_d * (c[0, i] * HI @ E1 + c[-1, i] * HI @ En) + BETA * HI @ BS.T @ (E1 + En)
        rows_slow.append(D + pen)
        sat_w.append(tau_d * c[0, i] * HI @ e1 + BETA * HI @ BS.T @ e1)
        sat_e.append(tau_d * c[-1, i] * HI @ en + BETA * HI @ BS.T @ en)
    perm = np.arange(N).reshape(n, n).T.ravel()   # (i fast) <- (j fast)
    P = sp.csr_matrix((np.ones(N), (np.arange(N), perm)), shape=(N, N))
    L_slow = (P.T @ sp.block_diag(rows_slow) @ P).tocsr()
    _, _, _, HI1, H1, _ = variable_sbp_1d(n, np.ones(n))
    H_tilde = sp.kron(H1, H1).tocsr()
    A = (-(H_tilde @ (L_fast + L_slow))).tocsr()
    A.eliminate_zeros()
    A.sort_indices()
    # boundary-data maps (the data are u on W/E and the flux c du/dn on S/N)
    def side_map(vals_per_line, index_of):
        rr, cc, vv = [], [], []
        for line, vec in enumerate(vals_per_line):
            vec = np.asarray(vec).ravel()
            for k in np.nonzero(vec)[0]:
                rr.append(index_of(line, k))
                cc.append(line)
                vv.append(vec[k])
        return sp.csr_matrix((vv, (rr, cc)), shape=(N, n))
    hi0 = 1.0 / (h * 0.5)
    sat_r = {
        "W": side_map(sat_w, lambda i, k: k * n + i),
        "E": side_map(sat_e, lambda i, k: k * n + i),
        "S": sp.csr_matrix((np.full(n, TAU_N * hi0), (np.arange(n) * n, np.arange(n))),
                           shape=(N, n)),
        "N": sp.csr_matrix((np.full(n, TAU_N * hi0), (np.arange(n) * n + n - 1, np.arange(n))),
                           shape=(N, n)),
    }
    return Assembled(n=n, A=A, H_tilde=H_tilde, sat_r=sat_r)


def coarsen_coefficients(c: np.ndarray) -> np.ndarray:
    """Coarse nodal coefficients for the variable-coefficient multigrid: the
    full-weighting (1/4, 1/2, 1/4)^2 harmonic mean of the fine values around
    each coarse point, indices clamped at the edges.  It keeps the
    conductance of layers the injection would under-sample: at N = 513 on
    the layered field MGCG needs 11 iterations instead of 14.  c is (n, n),
    indexed [j, i]; returns ((n+1)/2, (n+1)/2)."""
    w = (0.25, 0.5, 0.25)
    inv = 1.0 / np.asarray(c, dtype=np.float64)
    p = np.pad(inv, 1, mode="edge")
    rows = w[0] * p[:-2, :] + w[1] * p[1:-1, :] + w[2] * p[2:, :]
    both = w[0] * rows[:, :-2] + w[1] * rows[:, 1:-1] + w[2] * rows[:, 2:]
    return (1.0 / both)[::2, ::2].copy()


def coefficient_field(n: int, kind: str = "smooth") -> np.ndarray:
    """Seeded coefficient fields (flat, i fast), all >= 0.5.
    'smooth': c = 1 + 0.5 sin(2 pi x + 1) cos(3 pi y);
    'layered': c jumps between 1 and 10 across y = 0.5 (smoothed over 2h)."""
    x = grid(n)
    X = x[None, :]
    Y = x[:, None]
    if kind == "smooth":
        C = 1.0 + 0.5 * np.sin(2 * math.pi * X + 1.0) * np.cos(3 * math.pi * Y)
    elif kind == "layered":
        C = 1.0 + 9.0 * 0.5 * (1.0 + np.tanh((Y - 0.5) * (n - 1) / 2.0)) + 0 * X
    else:
        raise ValueError(kind)
    return C.ravel()


def manufactured_variable(n: int):
    """u = sin(pi x) cos(pi y) with div(c grad u) = f_ref for the 'smooth'
    field; boundary data: u on W/E (y = 0, 1) and the outward flux
    c du/dn on S/N (x = 0, 1).  Returns (c, f_ref, g, u_exact), flat."""
    x = grid(n)
    X = x[None, :]
    Y = x[:, None]
    pi = math.pi
    U = np.sin(pi * X) * np.cos(pi * Y)
    Ux = pi * np.cos(pi * X) * np.cos(pi * Y)
    Uy = -pi * np.sin(pi * X) * np.sin(pi * Y)
    C = 1.0 + 0.5 * np.sin(2 * pi * X + 1.0) * np.cos(3 * pi * Y)
    Cx = 0.5 * 2 * pi * np.cos(2 * pi * X + 1.0) * np.cos(3 * pi * Y)
    Cy = -0.5 * 3 * pi * np.sin(2 * pi * X + 1.0) * np.sin(3 * pi * Y)
    F = C * (-2 * pi**2 * U) + Cx * Ux + Cy * Uy
    g = {"W": np.sin(pi * x), "E": -np.sin(pi * x),
         "S": -(C[:, 0] * Ux[:, 0]), "N": C[:, -1] * Ux[:, -1]}
    return C.ravel(), F.ravel(), g, U.ravel()


def neg_A_variable_matrix_free(u, c, n: int) -> np.ndarray:
    """(-A u) of :func:`assemble_variable` point by point: face-averaged
    coefficients in a 5-point stencil, the Dirichlet closure of the
    second-order operator scaled by the boundary coefficient."""
    U = np.asarray(u, dtype=np.float64).reshape(n, n)   # [j, i]
    C = np.asarray(c, dtype=np.float64).reshape(n, n)
    w = np.ones(n)
    w[0] = w[-1] = 0.5
    out = np.zeros_like(U)
    fx = 0.5 * (C[:, :-1] + C[:, 1:])     # faces along i
    fy = 0.5 * (C[:-1, :] + C[1:, :])     # faces along j
    X = np.zeros_like(U)
    X[:, :-1] += fx * (U[:, 1:] - U[:, :-1])
    X[:, 1:] += fx * (U[:, :-1] - U[:, 1:])
    Y = np.zeros_like(U)
    Y[:-1, :] += fy * (U[1:, :] - U[:-1, :])
    Y[1:, :] += fy * (U[:-1, :] - U[1:, :])
    bs = (1.5, -2.0, 0.5)
    for jb, s in ((0, 1), (n - 1, -1)):
        cb = C[jb, :]
        Y[jb, :] += cb * (bs[0] * U[jb, :] + bs[1] * U[jb + s, :] + bs[2] * U[jb + 2 * s, :])
        Y[jb, :] += TAU_D_TIMES_H * cb * U[jb, :]
        for k in range(3):
            Y[jb + k * s, :] += BETA * bs[k] * cb * U[jb, :]
    out = w[:, None] * X + w[None, :] * Y
    return out.ravel()


# --------------------------------------------------------------------------
# Manufactured problems
# --------------------------------------------------------------------------
def grid(n: int) -> np.ndarray:
    return np.linspace(0.0, 1.0, n)


def manufactured(n: int, kind: str = "reference"):
    """Return (f_ref, g, u_exact) on n x n points, all flat (i fast).

    ``kind='reference'``: u = sin(pi(x+y)), the reference's own problem
    (``level_2_multigrid_new.jl:36-38, 169-182``).
    ``kind='baseline'``: u = sin(pi x) cos(pi y) with -Delta u = f, mapped
    on the reference's sides (Dirichlet at y = 0, 1 = j sides, Neumann at
    x = 0, 1 = i sides; S/N data are the outward normal derivatives).
    f_ref is in the reference's D2 convention (Delta u = f_ref).
    """
    x = grid(n)
    X = x[None, :]   # varies along i (axis 1)
    Y = x[:, None]   # varies along j (axis 0)
    pi = math.pi
    if kind == "reference":
        U = np.sin(pi * X + pi * Y)
        F = -2 * pi**2 * U
        g = {"W": np.sin(pi * x), "E": -np.sin(pi * x),
             "S": -pi * np.cos(pi * x), "N": pi * np.cos(pi * x + pi)}
    elif kind == "baseline":
        U = np.sin(pi * X) * np.cos(pi * Y)
        F = -2 * pi**2 * U
        g = {"W": np.sin(pi * x),                 # u(x, 0)
             "E": -np.sin(pi * x),                # u(x, 1)
             "S": -pi * np.cos(pi * x),           # -u_x(0, y)
             "N": pi * math.cos(pi) * np.cos(pi * x)}  # u_x(1, y)
    else:
        raise ValueError(kind)
    return F.ravel(), g, U.ravel()


def h_error(asm: Assembled, x: np.ndarray, u: np.ndarray) -> float:
    """sqrt((x-u)' H~ (x-u))  (``matrix_free_mg_cg.jl:464``)."""
    d = np.asarray(x).ravel() - np.asarray(u).ravel()
    return float(math.sqrt(d @ (asm.H_tilde @ d)))


# --------------------------------------------------------------------------
# Matrix-free -A (split_matrix_free.jl:444-486 with the SBP_* kernels)
# --------------------------------------------------------------------------
def neg_A_matrix_free(u: np.ndarray, n: int | None = None) -> np.ndarray:
    """The reference's ``matrix_free_A_full_GPU`` output, odata = -A u.

    Written from the per-kernel formulas: interior 5-point stencil
    (``D2_split_naive_v2``, :32-49), Neumann rows with one-sided D2 and the
    alpha3 = -1 penalty halved (/2) or quartered at corners (/4)
    (``SBP_N!``/``SBP_S!``, :324-388), Dirichlet columns with one-sided D2,
    1.5*beta*u + h*alpha1*u at the boundary point and -2u, +0.5u spread into
    the next two columns, halved in the corner rows (``SBP_W!``/``SBP_E!``,
    :391-429), summed as in :478-483.
    """
    flat = np.asarray(u, dtype=np.float64)
    if n is None:
        n = int(round(math.sqrt(flat.size)))
    U = flat.reshape(n, n)          # U[j, i]
    out = np.zeros_like(U)
    # interior
    out[1:-1, 1:-1] = (U[1:-1, :-2] + U[1:-1, 2:] + U[:-2, 1:-1] + U[2:, 1:-1]
                       - 4 * U[1:-1, 1:-1])
    a1h = TAU_D_TIMES_H
    a3 = TAU_N
    b = BETA
    # --- W / E temporaries (SBP_W!, SBP_E!), interior rows i = 1..n-2 ---
    W = np.zeros((3, n))  # W[c, i] for columns j = c
    E = np.zeros((3, n))  # E[c, i] for columns j = n-3+c
    ii = slice(1, n - 1)
    W[0, ii] = (U[0, :-2] - 2 * U[0, 1:-1] + U[0, 2:]
                + U[0, 1:-1] - 2 * U[1, 1:-1] + U[2, 1:-1]
                + 2 * b * 1.5 * U[0, 1:-1] + 2 * a1h * U[0, 1:-1]) / 2
    W[1, ii] = 2 * b * (-1 * U[0, 1:-1])
    W[2, ii] = 0.5 * b * U[0, 1:-1]
    E[2, ii] = (U[-1, :-2] - 2 * U[-1, 1:-1] + U[-1, 2:]
                + U[-1, 1:-1] - 2 * U[-2, 1:-1] + U[-3, 1:-1]
                + 2 * b * 1.5 * U[-1, 1:-1] + 2 * a1h * U[-1, 1:-1]) / 2
    E[1, ii] = 2 * b * (-1 * U[-1, 1:-1])
    E[0, ii] = 0.5 * b * U[-1, 1:-1]
    for i in (0, n - 1):
        W[0, i] = (2 * b * 1.5 * U[0, i] + 2 * a1h * U[0, i]) / 4
        W[1, i] = (2 * b * (-1 * U[0, i])) / 2
        W[2, i] = (0.5 * b * U[0, i]) / 2
        E[2, i] = (2 * b * 1.5 * U[-1, i] + 2 * a1h * U[-1, i]) / 4
        E[1, i] = (2 * b * (-1 * U[-1, i])) / 2
        E[0, i] = (0.5 * b * U[-1, i]) / 2
    # --- N / S temporaries (SBP_N!, SBP_S!): rows i = 0 and i = n-1 ---
    Nrow = np.zeros(n)
    Srow = np.zeros(n)

    def nrow(j, edge):
        # i = 0 row; col j; one-sided in i, interior or one-sided in j
        li = U[j, 0] - 2 * U[j, 1] + U[j, 2]
        pen = 2 * a3 * (1.5 * U[j, 0] - 2 * U[j, 1] + 0.5 * U[j, 2])
        if j == 0:
            lj = U[0, 0] - 2 * U[1, 0] + U[2, 0]
        elif j == n - 1:
            lj = U[n - 1, 0] - 2 * U[n - 2, 0] + U[n - 3, 0]
        else:
            lj = U[j - 1, 0] - 2 * U[j, 0] + U[j + 1, 0]
        return (li + lj + pen) / (4 if edge else 2)

    def srow(j, edge):
        li = U[j, -1] - 2 * U[j, -2] + U[j, -3]
        pen = 2 * a3 * (1.5 * U[j, -1] - 2 * U[j, -2] + 0.5 * U[j, -3])
        if j == 0:
            lj = U[0, -1] - 2 * U[1, -1] + U[2, -1]
        elif j == n - 1:
            lj = U[n - 1, -1] - 2 * U[n - 2, -1] + U[n - 3, -1]
        else:
            lj = U[j - 1, -1] - 2 * U[j, -1] + U[j + 1, -1]
        return (li + lj + pen) / (4 if edge else 2)

    for j in range(n):
        edge = j in (0, n - 1)
        Nrow[j] = nrow(j, edge)
        Srow[j] = srow(j, edge)
    # merge (split_matrix_free.jl:478-483): boundary ring of `out` is zero
    out[0:3, :] += W
    out[n - 3:n, :] += E
    out[:, 0] += Nrow
    out[:, n - 1] += Srow
    return out.ravel()


def neg_A_coefficients(n: int):
    """Per-point description of -A used by the GPU kernels, restated from
    the assembled operator: -A u = wi*wj*(Li u + Lj u) + wj*Neumann(i)
    + wi*Dirichlet(j).  Returned for documentation/tests: diag(A)."""
    wi = np.ones(n)
    wi[0] = wi[-1] = 0.5
    ci = np.full(n, -2.0)
    ci[0] = ci[-1] = 1.0
    neu = np.zeros(n)
    neu[0] = neu[-1] = 1.5 * TAU_N
    dir_ = np.zeros(n)
    dir_[0] = dir_[-1] = DIRICHLET_COEF[0]
    WJ = wi[:, None]
    WI = wi[None, :]
    diag_negA = (WI * WJ * (ci[None, :] + ci[:, None]) + WJ * neu[None, :]
                 + WI * dir_[:, None])
    return -diag_negA.ravel()


# --------------------------------------------------------------------------
# Transfer operators (level_2_multigrid_new.jl:190-246,
# matrix_free_mg_cg.jl:17-38, 80-94)
# --------------------------------------------------------------------------
def prolongation_matrix(nc: int) -> sp.csr_matrix:
    """1D bilinear prolongation, nc -> 2nc-1 (``:190-203``)."""
    nf = 2 * nc - 1
    rows, cols, vals = [], [], []
    for r in range(nf):
        if r % 2 == 0:
            rows.append(r); cols.append(r // 2); vals.append(1.0)
        else:
            rows += [r, r]; cols += [r // 2, r // 2 + 1]; vals += [0.5, 0.5]
    return sp.csr_matrix((vals, (rows, cols)), shape=(nf, nc))


def restriction_matrix(nf: int) -> sp.csr_matrix:
    """1D SBP-preserving restriction (``restriction_matrix`` :205-218):
    boundary rows (1/2, 1/2), interior (1/4, 1/2, 1/4)."""
    nc = (nf + 1) // 2
    R = sp.lil_matrix((nc, nf))
    R[0, 0] = 0.5; R[0, 1] = 0.5
    R[nc - 1, nf - 2] = 0.5; R[nc - 1, nf - 1] = 0.5
    for c in range(1, nc - 1):
        R[c, 2 * c - 1] = 0.25; R[c, 2 * c] = 0.5; R[c, 2 * c + 1] = 0.25
    return R.tocsr()


def restriction_matrix_normal(nf: int) -> sp.csr_matrix:
    """1D full weighting with zero padding (``restriction_matrix_normal``
    :220-233): boundary rows (1/2, 1/4), interior (1/4, 1/2, 1/4)."""
    nc = (nf + 1) // 2
    R = sp.lil_matrix((nc, nf))
    R[0, 0] = 0.5; R[0, 1] = 0.25
    R[nc - 1, nf - 2] = 0.25; R[nc - 1, nf - 1] = 0.5
    for c in range(1, nc - 1):
        R[c, 2 * c - 1] = 0.25; R[c, 2 * c] = 0.5; R[c, 2 * c + 1] = 0.25
    return R.tocsr()


def prolongation_2d(nc: int) -> sp.csr_matrix:
    P = prolongation_matrix(nc)
    return sp.kron(P, P).tocsr()


RESTRICT_KINDS = ("normal", "sbp", "galerkin")


def restriction_2d(nf: int, kind: str = "normal") -> sp.csr_matrix:
    """2D restriction.  'normal' is the reference's ``restriction_2d``
    (:241-246, kron of ``restriction_matrix_normal``); 'sbp' is the kron of
    the SBP-preserving ``restriction_matrix``; 'galerkin' is P^T, which is
    the SBP-compatible restriction H~_2h^-1 P^T H~_h re-expressed for the
    H~-scaled residuals this operator produces (f_2h = H~_2h R_sbp H~_h^-1 r).
    """
    if kind == "normal":
        R = restriction_matrix_normal(nf)
        return sp.kron(R, R).tocsr()
    if kind == "sbp":
        R = restriction_matrix(nf)
        return sp.kron(R, R).tocsr()
    if kind == "galerkin":
        return prolongation_2d((nf + 1) // 2).T.tocsr()
    raise ValueError(kind)


def restriction_mf(r: np.ndarray, nf: int) -> np.ndarray:
    """Matrix-free full weighting on a zero-padded copy
    (``matrix_free_restriction_2d`` :80-94)."""
    R = np.asarray(r, dtype=np.float64).reshape(nf, nf)
    P = np.zeros((nf + 2, nf + 2))
    P[1:-1, 1:-1] = R
    nc = (nf + 1) // 2
    c = np.arange(nc)
    J, I = np.meshgrid(2 * c + 1, 2 * c + 1, indexing="ij")
    out = (4 * P[J, I] + 2 * (P[J, I - 1] + P[J, I + 1] + P[J - 1, I] + P[J + 1, I])
           + P[J - 1, I - 1] + P[J - 1, I + 1] + P[J + 1, I - 1] + P[J + 1, I + 1]) / 16
    return out.ravel()


def prolongation_mf(e: np.ndarray, nc: int) -> np.ndarray:
    """Matrix-free bilinear prolongation (``matrix_free_prolongation_2d``
    :17-38): injection at even points, 2- and 4-point averages elsewhere."""
    E = np.asarray(e, dtype=np.float64).reshape(nc, nc)
    nf = 2 * nc - 1
    out = np.zeros((nf, nf))
    out[::2, ::2] = E
    out[::2, 1::2] = (E[:, :-1] + E[:, 1:]) / 2
    out[1::2, ::2] = (E[:-1, :] + E[1:, :]) / 2
    out[1::2, 1::2] = (E[:-1, :-1] + E[1:, :-1] + E[:-1, 1:] + E[1:, 1:]) / 4
    return out.ravel()


# --------------------------------------------------------------------------
# Smoothers (level_2_multigrid_new.jl:335-350, matrix_free_mg_cg.jl:134-140)
# --------------------------------------------------------------------------
def richardson(x, A, b, maxiter=3, omega=0.15):
    """``modified_richardson!``: x <- x + omega (b - A x)."""
    x = np.array(x, dtype=np.float64, copy=True)
    for _ in range(maxiter):
        x = x + omega * (b - A @ x)
    return x


def jacobi(x, A, b, maxiter=3, omega=2.0 / 3.0, diag=None):
    """``jacobi_brittany!``: x <- omega D^-1 (b - (A - D) x) + (1-omega) x,
    i.e. x + omega D^-1 (b - A x)."""
    x = np.array(x, dtype=np.float64, copy=True)
    d = A.diagonal() if diag is None else diag
    for _ in range(maxiter):
        x = x + omega * (b - A @ x) / d
    return x


# --------------------------------------------------------------------------
# Multigrid hierarchy, V-cycle, MGCG, CG
# --------------------------------------------------------------------------
@dataclass
class MGOptions:
    """Options mirrored by the C-ABI ``sbp_options`` struct."""
    smoother: str = "jacobi"        # 'jacobi' (omega=2/3) or 'richardson' (0.15)
    omega: float | None = None
    nu_pre: int = 3
    nu_post: int = 3
    restriction: str = "galerkin"   # 'normal' | 'sbp' | 'galerkin'
    coarse_n: int = 65              # size at which the direct solve happens

    def w(self):
        if self.omega is not None:
            return self.omega
        return 2.0 / 3.0 if self.smoother == "jacobi" else 0.15

    @staticmethod
    def reference_two_level(n: int) -> "MGOptions":
        """The reference's GPU MGCG: two levels, Richardson 0.15, nu = 3,
        full-weighting 'normal' restriction, exact coarse solve at (n+1)/2
        (``matrix_free_mg_cg.jl:143-176, 281-324``)."""
        return MGOptions(smoother="richardson", omega=0.15, nu_pre=3, nu_post=3,
                         restriction="normal", coarse_n=(n + 1) // 2)


class Hierarchy:
    """Levels n, (n+1)/2, ... down to ``coarse_n``; each level re-discretised
    with :func:`assemble` like ``Assembling_matrix(level-1)``
    (``matrix_free_mg_cg.jl:455``), coarse level solved by a sparse LU
    (``:460``, ``A_2h \\ f`` at :166)."""

    def __init__(self, n: int, opts: MGOptions, p: int = 2, coef=None, galerkin: bool = False):
        """p: SBP order of every level.  coef (flat n x n, i fast): nodal
        coefficients of the variable-coefficient operator, carried to each
        coarse grid by :func:`coarsen_coefficients`.  galerkin: coarse
        operators P' A P instead of the re-discretised ones."""
        self.opts = opts
        self.p = p
        self.ns = [n]
        while self.ns[-1] > opts.coarse_n:
            nn = (self.ns[-1] + 1) // 2
            if nn < 3:
                break
            self.ns.append(nn)
        if self.ns[-1] != opts.coarse_n and len(self.ns) > 1:
            raise ValueError(f"n={n} does not coarsen to coarse_n={opts.coarse_n}")
        if coef is None:
            self.asm = [assemble(m, p) for m in self.ns]
        else:
            cs = [np.asarray(coef, dtype=np.float64).reshape(n, n)]
            for m in self.ns[1:]:
                cs.append(coarsen_coefficients(cs[-1]))
            self.coefs = [c.ravel() for c in cs]
            self.asm = [assemble_variable(m, c) for m, c in zip(self.ns, self.coefs)]
        self.A = [a.A for a in self.asm]
        self.R = [restriction_2d(m, opts.restriction) for m in self.ns[:-1]]
        self.P = [prolongation_2d(m) for m in self.ns[1:]]
        if galerkin:
            self.A = [self.A[0]]
            for P in self.P:
                self.A.append((P.T @ self.A[-1] @ P).tocsr())
        self.diag = [A.diagonal() for A in self.A]
        self.lu = spla.splu(self.A[-1].tocsc())

    def smooth(self, l, v, b, iters):
        o = self.opts
        if o.smoother == "jacobi":
            return jacobi(v, self.A[l], b, iters, o.w(), self.diag[l])
        return richardson(v, self.A[l], b, iters, o.w())

    def vcycle(self, b, l=0):
        """One V-cycle from v = 0 (``Two_level_multigrid`` :358-382 for two
        levels; recursive here)."""
        if l == len(self.ns) - 1:
            return self.lu.solve(np.asarray(b, dtype=np.float64))
        v = np.zeros_like(b)
        v = self.smooth(l, v, b, self.opts.nu_pre)
        r = b - self.A[l] @ v
        f = self.R[l] @ r
        e = self.vcycle(f, l + 1)
        v = v + self.P[l] @ e
        v = self.smooth(l, v, b, self.opts.nu_post)
        return v


def mgcg(hier: Hierarchy, b, x=None, abstol=None, reltol=None, maxiter=None):
    """``mg_preconditioned_CG`` (``level_2_multigrid_new.jl:480-524``),
    with the V-cycle of :class:`Hierarchy` as preconditioner.  Stops when
    ||r||_2 < abstol (abstol = reltol*||b - A x0|| if reltol given).
    Returns (x, iters, norms)."""
    A = hier.A[0]
    b = np.asarray(b, dtype=np.float64)
    x = np.zeros_like(b) if x is None else np.array(x, dtype=np.float64)
    r = b - A @ x
    if abstol is None:
        reltol = math.sqrt(np.finfo(float).eps) if reltol is None else reltol
        abstol = reltol * np.linalg.norm(r)
    maxiter = b.size if maxiter is None else maxiter
    z = hier.vcycle(r)
    p = z.copy()
    rz = r @ z
    norms = [float(np.linalg.norm(r))]
    it = 0
    for _ in range(maxiter):
        it += 1
        Ap = A @ p
        alpha = rz / (p @ Ap)
        x = x + alpha * p
        r = r - alpha * Ap
        rs = r @ r
        norms.append(float(math.sqrt(rs)))
        if math.sqrt(rs) < abstol:
            break
        z = hier.vcycle(r)
        rz_new = r @ z
        beta = rz_new / rz
        p = z + beta * p
        rz = rz_new
    return x, it, norms


def cg(A, b, x=None, abstol=None, reltol=None, maxiter=None):
    """``CG_CPU`` (``level_2_multigrid_new.jl:258-291``): textbook CG,
    stop when ||r|| < abstol.  Returns (x, iters, norms)."""
    b = np.asarray(b, dtype=np.float64)
    x = np.zeros_like(b) if x is None else np.array(x, dtype=np.float64)
    r = b - A @ x
    if abstol is None:
        reltol = math.sqrt(np.finfo(float).eps) if reltol is None else reltol
        abstol = reltol * np.linalg.norm(r)
    maxiter = b.size if maxiter is None else maxiter
    p = r.copy()
    rs = r @ r
    norms = [float(math.sqrt(rs))]
    it = 0
    for _ in range(maxiter):
        it += 1
        Ap = A @ p
        alpha = rs / (p @ Ap)
        x = x + alpha * p
        r = r - alpha * Ap
        rsn = r @ r
        norms.append(float(math.sqrt(rsn)))
        if math.sqrt(rsn) < abstol:
            break
        p = r + (rsn / rs) * p
        rs = rsn
    return x, it, norms


def misfit_loss_grad(asm: Assembled, f_ref, g: dict, ut):
    """Adjoint-path oracle (the reference has no adjoint code; this restates
    the calculus of its operator).  With b = asm.rhs(f_ref, g) and
    u = A^-1 b by a sparse direct solve (``matrix_free_mg_cg.jl:460`` uses
    ``lu`` the same way), L = 1/2 (u - ut)' H~ (u - ut),
    lam = A^-1 H~ (u - ut) (A is symmetric), dL/df = -H~ lam and
    dL/dg_side = -SAT_side' H~ lam (b = -H~ (f + sum SAT_side g_side)).
    Returns (L, df, dg, u, lam), all flat float64 arrays (dg: side -> n)."""
    lu = spla.splu(asm.A.tocsc())
    u = lu.solve(asm.rhs(f_ref, g))
    d = u - np.asarray(ut, dtype=np.float64).ravel()
    hd = asm.H_tilde @ d
    loss = 0.5 * float(d @ hd)
    lam = lu.solve(hd)
    hl = asm.H_tilde @ lam
    df = -hl
    dg = {s: -(asm.sat_r[s].T @ hl) for s in ("W", "E", "S", "N")}
    return loss, df, dg, u, lam


def cg_tolerance(A, b, x0, abstol):
    """IterativeSolvers.jl ``cg!`` stopping threshold used by the reference's
    nested iteration: max(reltol * |b - A x0|, abstol), reltol = sqrt(eps)."""
    r0 = float(np.linalg.norm(np.asarray(b) - A @ np.asarray(x0)))
    return max(math.sqrt(np.finfo(float).eps) * r0, abstol)


def nested_cg(n: int, b, b_2h, abstol: float):
    """``initial_guess_interpolation_CG`` (``matrix_free_mg_cg.jl:372-377``):
    exact solve of the coarse problem A_2h x_2h = b_2h (its own right-hand
    side), bilinear prolongation of x_2h as the initial guess, CG on A x = b.
    Returns (x, iters, norms)."""
    nc = (n + 1) // 2
    A = assemble(n).A
    x2h = spla.splu(assemble(nc).A.tocsc()).solve(np.asarray(b_2h, dtype=np.float64))
    x0 = prolongation_2d(nc) @ x2h
    return cg(A, b, x0, abstol=cg_tolerance(A, b, x0, abstol))


def nested_cg_three_level(n: int, b, b_2h, b_4h, abstol: float):
    """``initial_guess_interpolation_three_level_CG_GPU``
    (``matrix_free_mg_cg.jl:386-396``): exact solve on 4h, prolong, CG on 2h,
    prolong, CG on h.  Returns (x, iters_2h, iters_h, norms_2h, norms_h)."""
    n2 = (n + 1) // 2
    n4 = (n2 + 1) // 2
    A2 = assemble(n2).A
    A = assemble(n).A
    x4 = spla.splu(assemble(n4).A.tocsc()).solve(np.asarray(b_4h, dtype=np.float64))
    x2_0 = prolongation_2d(n4) @ x4
    x2, it2, nr2 = cg(A2, b_2h, x2_0, abstol=cg_tolerance(A2, b_2h, x2_0, abstol))
    x0 = prolongation_2d(n2) @ x2
    x, it, nr = cg(A, b, x0, abstol=cg_tolerance(A, b, x0, abstol))
    return x, it2, it, nr2, nr
