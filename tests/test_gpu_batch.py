"""Batched MGCG: problems of mixed grid sizes solved together, against the
same problems solved one at a time (and the oracle for one of them)."""
import time

import numpy as np
import pytest
import torch

from oracle import sbp_oracle as o

pytestmark = pytest.mark.gpu


def host(t):
    torch.cuda.synchronize()
    return t.detach().cpu().numpy().ravel()


def relerr(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _sequential(sbp, ns, bs, opts, reltol):
    solvers = {n: sbp.Solver(n, opts) for n in sorted(set(ns))}
    xs, res = [], []
    for n, b in zip(ns, bs):
        x = torch.zeros_like(b)
        res.append(solvers[n].mgcg(b, x, reltol=reltol, maxiter=100))
        xs.append(x)
    return xs, res, solvers


def test_batch_matches_sequential(sbp):
    from sc_2022_gb300 import problems
    ns = [129, 65, 257, 129, 65, 257, 129, 513]
    bs = []
    for k, n in enumerate(ns):
        f, g = problems.bump_problem(n, 50 + k)
        bs.append(problems.assemble_rhs(f, g).reshape(-1))
    opts = sbp.default_options()
    B = sbp.BatchSolver(ns, opts)
    xs = [torch.zeros_like(b) for b in bs]
    rb = B.mgcg(bs, xs, reltol=1e-10, maxiter=100)
    xq, rq, _ = _sequential(sbp, ns, bs, opts, 1e-10)
    for k in range(len(ns)):
        assert rb[k].converged and rq[k].converged
        assert abs(rb[k].iters - rq[k].iters) <= 1
        assert relerr(host(xs[k]), host(xq[k])) < 1e-8
    # one problem against the oracle (V-cycle to 65^2, same stopping rule)
    n, b = ns[2], bs[2]
    hier = o.Hierarchy(n, o.MGOptions(coarse_n=65))
    xr, itr, nr = o.mgcg(hier, host(b), reltol=1e-10)
    assert rb[2].iters == itr
    assert relerr(host(xs[2]), xr) < 1e-9
    # a second solve reuses the captured graphs and starts from the caller's x
    xs2 = [torch.zeros_like(b) for b in bs]
    rb2 = B.mgcg(bs, xs2, reltol=1e-10, maxiter=100)
    for k in range(len(ns)):
        assert rb2[k].iters == rb[k].iters
        assert torch.equal(xs2[k], xs[k])


def test_batch_mixed_precision(sbp):
    from sc_2022_gb300 import _lib, problems
    ns, bs = problems.batch_problems(12, seed=9)
    opts = sbp.default_options(_lib.SBP_PREC_MIXED)
    B = sbp.BatchSolver(ns, opts)
    xs = [torch.zeros_like(b) for b in bs]
    rb = B.mgcg(bs, xs, reltol=1e-10, maxiter=100)
    xq, rq, _ = _sequential(sbp, ns, bs, sbp.default_options(), 1e-10)
    for k in range(len(ns)):
        assert rb[k].converged
        assert rb[k].iters <= rq[k].iters + 1
        assert relerr(host(xs[k]), host(xq[k])) < 1e-8


def test_batch_config_256_problems(sbp):
    # 256 problems, N log-uniform over {65, ..., 1025} by seed, bump/trig data,
    # FP64 MGCG to 1e-10: batched solve against 256 sequential solves
    from sc_2022_gb300 import problems
    ns, bs = problems.batch_problems(256, seed=4)
    assert len(set(ns)) == 5
    opts = sbp.default_options()
    B = sbp.BatchSolver(ns, opts)
    xs = [torch.zeros_like(b) for b in bs]
    budgets = B.autotune(bs, xs)                     # per-size launch shapes
    assert sorted(budgets) == sorted(set(ns))
    B.mgcg(bs, xs, reltol=1e-10, maxiter=100)          # warm-up
    for x in xs:
        x.zero_()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rb = B.mgcg(bs, xs, reltol=1e-10, maxiter=100)
    torch.cuda.synchronize()
    t_batch = time.perf_counter() - t0
    xq, rq, solvers = _sequential(sbp, ns, bs, opts, 1e-10)   # warm-up (captures)
    for x in xq:
        x.zero_()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for n, b, x in zip(ns, bs, xq):
        solvers[n].mgcg(b, x, reltol=1e-10, maxiter=100)
    torch.cuda.synchronize()
    t_seq = time.perf_counter() - t0
    worst = 0.0
    for k in range(len(ns)):
        assert rb[k].converged
        assert abs(rb[k].iters - rq[k].iters) <= 1
        worst = max(worst, relerr(host(xs[k]), host(xq[k])))
    print(f"256 problems: batched {1e3 * t_batch:.1f} ms, sequential {1e3 * t_seq:.1f} ms "
          f"({t_seq / t_batch:.2f}x), launches {B.last_launches}, worst rel. diff {worst:.2e}, "
          f"CTA budgets {budgets}")
    assert worst < 1e-8
    # every problem with N <= 257 against the C oracle's MGCG (same V-cycle,
    # same stopping rule): iterations within one, solutions to 1e-9
    import os
    from oracle import cpu_path
    cpu_path.set_threads(os.cpu_count() or 1)
    oracles = {n: cpu_path.CpuMG(n, smoother="jacobi", restriction="galerkin", coarse_n=65)
               for n in sorted(set(ns)) if n <= 257}
    checked, worst_o = 0, 0.0
    for k, n in enumerate(ns):
        if n not in oracles:
            continue
        bh = host(bs[k])
        xo, ito, _ = oracles[n].mgcg(bh, np.zeros_like(bh), 1e-10 * float(np.linalg.norm(bh)),
                                     maxiter=100)
        assert abs(rb[k].iters - ito) <= 1, (k, n, rb[k].iters, ito)
        err = relerr(host(xs[k]), xo)
        worst_o = max(worst_o, err)
        assert err < 1e-9, (k, n, err)
        checked += 1
    for m in oracles.values():
        m.close()
    print(f"{checked} problems with N <= 257 against the C oracle: worst rel. diff {worst_o:.2e}")
    assert checked == sum(1 for n in ns if n <= 257) and checked > 100


def test_batch_maxiter_then_larger_maxiter(sbp):
    # a first solve stopped by maxiter, then a solve with a larger maxiter
    # (the per-problem norm buffers grow; the batch recaptures its graphs)
    from sc_2022_gb300 import _lib, problems
    ns, bs = problems.batch_problems(6, seed=21)
    B = sbp.BatchSolver(ns, sbp.default_options())
    xs = [torch.zeros_like(b) for b in bs]
    r1 = B.mgcg(bs, xs, reltol=1e-10, maxiter=2)
    for n, r in zip(ns, r1):
        if n == 65:   # one level: the V-cycle is the exact coarse solve
            assert r.converged and r.iters == 1
        else:
            assert r.status == _lib.SBP_ERR_MAXITER and r.iters == 2
    xs = [torch.zeros_like(b) for b in bs]
    r2 = B.mgcg(bs, xs, reltol=1e-10, maxiter=500)
    xq, rq, _ = _sequential(sbp, ns, bs, sbp.default_options(), 1e-10)
    for k in range(len(ns)):
        assert r2[k].converged and abs(r2[k].iters - rq[k].iters) <= 1
        assert relerr(host(xs[k]), host(xq[k])) < 1e-8
