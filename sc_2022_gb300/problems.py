"""Right-hand sides of the benchmark configurations.

Inputs are generated on the host in FP64 and the SBP-SAT right-hand side
b = -H~ (f + SAT_r g) is assembled on the GPU (``sbp_rhs_f64``), replacing
the reference's sparse ``Assembling_matrix`` b (level_2_multigrid_new.jl:169-185).

Random draws use a counter-based splitmix64 generator so every language
binding reproduces the same problem from a seed: draw k of stream `seed` is
splitmix64(seed * 2^32 + k); uniforms take the top 53 bits, normals use
Box-Muller on two consecutive uniforms.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import _lib as L
from .solver import _stream_ptr, ptr

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = (x.astype(np.uint64) + _GOLDEN)
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


class Stream:
    """Sequential draws from the counter-based generator."""

    def __init__(self, seed: int):
        self.base = np.uint64((seed & 0xFFFFFFFF) << 32)
        self.k = 0

    def uniform(self, count: int = 1) -> np.ndarray:
        with np.errstate(over="ignore"):
            ctr = self.base + np.arange(self.k, self.k + count, dtype=np.uint64)
        self.k += count
        return (splitmix64(ctr) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)

    def normal(self, count: int = 1) -> np.ndarray:
        u = self.uniform(2 * count).reshape(count, 2)
        u1 = np.maximum(u[:, 0], 1e-300)
        return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * math.pi * u[:, 1])


def grid_coords(n: int) -> np.ndarray:
    return np.linspace(0.0, 1.0, n)


def manufactured(n: int, kind: str = "baseline"):
    """(f_lap, g, u_exact) for the manufactured solutions, host FP64.

    kind='baseline': u = sin(pi x) cos(pi y), -Delta u = f.
    kind='reference': u = sin(pi (x + y)) (level_2_multigrid_new.jl:36-38).
    f_lap is Delta u (the reference's D2 convention); grids are (n, n)
    indexed [j, i] with x along i.  Dirichlet data sit on the j = 0 / n-1
    sides (y = 0 / 1), Neumann data (outward normal derivatives) on the
    i = 0 / n-1 sides (x = 0 / 1), as in the reference.
    """
    x = grid_coords(n)
    X, Y = x[None, :], x[:, None]
    pi = math.pi
    if kind == "baseline":
        U = np.sin(pi * X) * np.cos(pi * Y)
        g = {"W": np.sin(pi * x), "E": -np.sin(pi * x),
             "S": -pi * np.cos(pi * x), "N": -pi * np.cos(pi * x)}
    elif kind == "reference":
        U = np.sin(pi * X + pi * Y)
        g = {"W": np.sin(pi * x), "E": -np.sin(pi * x),
             "S": -pi * np.cos(pi * x), "N": pi * np.cos(pi * x + pi)}
    else:
        raise ValueError(kind)
    return -2.0 * pi * pi * U, g, U


def bump_problem(n: int, seed: int):
    """Random Gaussian-bump source and trig boundary data.

    f(x, y) = sum_{k<8} a_k exp(-|(x,y) - c_k|^2 / (2 w_k^2)),
    c_k ~ U(0.1, 0.9)^2, w_k ~ U(0.02, 0.1), a_k ~ N(0, 1), with -Delta u = f;
    each side s in (W, E, S, N): g_s(t) = sum_{m=1..6} c_m / m^2 sin(m pi t + phi_m),
    c_m ~ N(0, 1), phi_m ~ U(0, 2 pi).
    Draw order: per bump (cx, cy, w, a), then per side and mode (c, phi).
    Returns (f_lap, g) with f_lap = -f in the D2 convention.
    """
    st = Stream(seed)
    x = grid_coords(n)
    F = np.zeros((n, n))
    for _ in range(8):
        cx, cy, w = st.uniform(3)
        cx = 0.1 + 0.8 * cx
        cy = 0.1 + 0.8 * cy
        w = 0.02 + 0.08 * w
        a = st.normal(1)[0]
        gx = np.exp(-(x - cx) ** 2 / (2 * w * w))
        gy = np.exp(-(x - cy) ** 2 / (2 * w * w))
        F += a * gy[:, None] * gx[None, :]
    g = {}
    for side in ("W", "E", "S", "N"):
        acc = np.zeros(n)
        for m in range(1, 7):
            c = st.normal(1)[0]
            phi = 2 * math.pi * st.uniform(1)[0]
            acc += c / (m * m) * np.sin(m * math.pi * x + phi)
        g[side] = acc
    return -F, g


def assemble_rhs(f_lap: np.ndarray | torch.Tensor, g: dict, device="cuda") -> torch.Tensor:
    """b = -H~ (f_lap + sum SAT_r g) on the GPU (sbp_rhs_f64)."""
    f = torch.as_tensor(f_lap, dtype=torch.float64, device=device).contiguous()
    n = int(round(math.sqrt(f.numel())))
    gs = [torch.as_tensor(g[k], dtype=torch.float64, device=device).contiguous()
          for k in ("W", "E", "S", "N")]
    b = torch.empty((n, n), dtype=torch.float64, device=device)
    L.check(L.load().sbp_rhs_f64(ptr(f), *[ptr(t) for t in gs], ptr(b), n, 1.0, _stream_ptr()),
            "sbp_rhs_f64")
    return b


def rhs_adjoint(lam: torch.Tensor):
    """(df, dg) with lam.b = df.f_lap + sum_side dg_side.g_side."""
    n = int(round(math.sqrt(lam.numel())))
    df = torch.empty((n, n), dtype=torch.float64, device=lam.device)
    dg = {k: torch.empty(n, dtype=torch.float64, device=lam.device) for k in "WESN"}
    L.check(L.load().sbp_rhs_adjoint_f64(ptr(lam), ptr(df), ptr(dg["W"]), ptr(dg["E"]),
                                         ptr(dg["S"]), ptr(dg["N"]), n, 1.0, _stream_ptr()),
            "sbp_rhs_adjoint_f64")
    return df, dg


def batch_sizes(count: int, seed: int, sizes=(65, 129, 257, 513, 1025)):
    """Grid sizes drawn log-uniformly from `sizes` (uniform over the list of
    powers of two plus one) by the project's counter-based stream."""
    st = Stream(seed)
    u = st.uniform(count)
    return [int(sizes[min(int(v * len(sizes)), len(sizes) - 1)]) for v in u]


def batch_problems(count: int, seed: int, device="cuda"):
    """The batched-solve configuration: `count` problems with sizes from
    :func:`batch_sizes` and bump/trig data of :func:`bump_problem` (seed
    seed * 1000 + k for problem k).  Returns (ns, bs) with bs the assembled
    right-hand sides on `device`."""
    ns = batch_sizes(count, seed)
    bs = []
    for k, n in enumerate(ns):
        f, g = bump_problem(n, seed * 1000 + k)
        bs.append(assemble_rhs(f, g, device=device).reshape(-1))
    return ns, bs
