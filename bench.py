"""Benchmark of the fused forward + adjoint of one monotone component.

Workload (the metric's configuration): one MonotoneComponent with input
dimension 8, total-order-4 multi-index set (495 terms), ProbabilistHermite
basis (normalised), SoftPlus rectifier, AdaptiveClenshawCurtis quadrature
(quadPts 5, abs = rel tol 1e-6, maxSub 30); coefficients N(0, 0.05^2),
1,000,000 points N(0, I_8), sensitivities N(0, 1), all float64 from seeded
generators (synthetic data; the reference publishes no dataset for this path).

One step = Evaluate + LogDeterminant + CoeffGrad + LogDeterminantCoeffGrad of
every point, with the coefficient gradients contracted over the points
(sum_i sens_i dT_i/dc + sum_i dlogdet_i/dc), in one fused pass.

`value` is points/s with inputs resident in HBM (device time of the fused
call, CUDA events on its stream, L2 flushed between steps).  `e2e` is the
same through the C ABI with pinned host buffers (host->device copy of points
and sensitivities and device->host copy of T, logdet and the gradient inside
the timed region).  `--impl reference` times the reference algorithm (the
CPU restatement in oracle/, all host threads) on bounded samples.

The line also carries `kl_train`, the KL training workload: a 6-D
TriangularMap of total order 5 (HermiteFunctions basis, Exp rectifier, ACC tol
1e-7) trained from zero coefficients on 200,000 samples of a synthetic banana
target (x1 ~ N(0,1), x2 = x1^2 + 0.5 N(0,1), x_k = 0.8 x_{k-1} + 0.6 N(0,1)),
standard-normal reference density, 100 L-BFGS iterations.  It reports the
objective, the gradient norm and the device ms of one KL step (objective and
gradient of every component) as one CUDA-graph replay of the batched launch,
as direct batched launches, and as the per-component launch sequence, beside
the oracle's time for the same step on the host cores.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

DIM, ORDER, NPTS = 8, 4, 1_000_000
TOL, MAXSUB = 1e-6, 30
METRIC = "fused fwd+adjoint points/s (dim-8, order-4, FP64)"
KL_DIM, KL_ORDER, KL_N, KL_TOL = 6, 5, 200_000, 1e-7
# Training to convergence: L-BFGS with the diagonal preconditioner (the
# inverse mean squared per-point gradient of every coefficient at the start)
# until an iteration changes a component's objective by less than KL_FTOL_REL
# relative (NLopt's ftol_rel rule), at most KL_MAX_ITERS iterations.  The
# gradient norm is reported but is no stopping rule here: the problem is so
# ill-conditioned that a component's gradient norm falls below 0.05 while its
# objective is still 0.05 above the optimum.  Without the preconditioner
# L-BFGS needs thousands of iterations (3000 reach 0.290, the preconditioned
# run 0.2746 in 1000).  SLSQP from zero did not finish 100 iterations in 15
# minutes: its trial steps (the first is the full negative gradient) make the
# integrand so steep that the adaptive quadrature's cost per step grows by
# orders of magnitude.
KL_FTOL_REL, KL_MAX_ITERS = 1e-7, 3000
KL_ALG = "LD_LBFGS"
KL_TRAIN = dict(max_iters=KL_MAX_ITERS, max_evals=3 * KL_MAX_ITERS, ftol_rel=KL_FTOL_REL, algorithm=KL_ALG,
                precondition=True)
# CPU legs run in a child process on the oracle's timing build (the same
# source with the compiler's default floating-point contraction, -O3
# -fopenmp) with the threads bound one per core.
TIMING_ENV = {"OMP_PROC_BIND": "spread", "OMP_PLACES": "threads", "MPGB_ORACLE_BUILD": "timing"}
CPU_BUILD = ("oracle/ timing build (g++ -O3 -fopenmp, default FP contraction; no -march=native), "
             "OMP_PROC_BIND=spread OMP_PLACES=threads")
SIG_DIM, SIG_ORDER, SIG_NSIG, SIG_N = 8, 3, 5, 1_000_000


def synth(n, seed_pts=1, seed_sens=2):
    x = np.random.default_rng(seed_pts).standard_normal((DIM, n))
    s = np.random.default_rng(seed_sens).standard_normal((1, n))
    return x, s


def coeffs(nterms):
    return np.random.default_rng(0).normal(0.0, 0.05, nterms)


def banana(n, seed=11):
    """Synthetic banana target: x1 ~ N(0,1), x2 = x1^2 + 0.5 N(0,1),
    x_k = 0.8 x_{k-1} + 0.6 N(0,1) for k = 3..KL_DIM."""
    rng = np.random.default_rng(seed)
    x1 = rng.standard_normal(n)
    xs = [x1, x1 ** 2 + 0.5 * rng.standard_normal(n)]
    while len(xs) < KL_DIM:
        xs.append(0.8 * xs[-1] + 0.6 * rng.standard_normal(n))
    return np.stack(xs)


def kl_train(M, dev):
    """KL training workload on the device: preconditioned L-BFGS from zero
    coefficients to convergence (KL_TRAIN) with the CUDA-graph step; then, at
    the trained coefficients,
    the step time of the four launch modes (graph-batched, direct-batched, one
    fused launch set per component, and per component the reference
    objective's call sequence with dense outputs); then the same training with
    the per-component modes (objectives compared)."""
    import torch
    opts = M.MapOptions(basisType=M.BasisTypes.HermiteFunctions, posFuncType=M.PosFuncTypes.Exp,
                        quadType=M.QuadTypes.AdaptiveClenshawCurtis, quadAbsTol=KL_TOL, quadRelTol=KL_TOL)
    X = torch.as_tensor(banana(KL_N), device=dev)
    tm = M.CreateTriangular(KL_DIM, KL_DIM, KL_ORDER, opts)
    tm.SetCoeffs(np.zeros(tm.numCoeffs))
    l0 = M.launch_count()
    loss_g, r_g = M.TrainMap(tm, X, mode=0, **KL_TRAIN)
    launches = M.launch_count() - l0
    trained = np.array(tm.CoeffMap())
    steps = {m: M.KLStepTime(tm, X, mode=m, steps=10, return_values=True) for m in (0, 1, 2, 3)}
    ms = {m: v[0] for m, v in steps.items()}

    def rel(a, b):
        return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))

    gscale = np.abs(steps[0][2]).max()
    step_diff = {
        "loss_max_rel_diff_reference_calls": rel(steps[3][1], steps[0][1]),
        "grad_max_abs_diff_over_max_reference_calls": float(np.abs(steps[3][2] - steps[0][2]).max() / gscale),
        "loss_max_rel_diff_per_component_fused": rel(steps[2][1], steps[0][1]),
        "grad_max_abs_diff_over_max_per_component_fused": float(np.abs(steps[2][2] - steps[0][2]).max() / gscale),
    }

    # (one fused launch set per component trains bitwise as the batched step
    # does, checked by the tests; the reference call sequence sums in another
    # order)
    tm.SetCoeffs(np.zeros(tm.numCoeffs))
    loss_r, r_r = M.TrainMap(tm, X, mode=3, **KL_TRAIN)
    return {
        "workload": f"TriangularMap {KL_DIM}-D, total order {KL_ORDER} ({tm.numCoeffs} coefficients), "
                    f"HermiteFunctions + Exp, ACC tol {KL_TOL}, {KL_N} banana samples, standard-normal KL, "
                    f"L-BFGS with a diagonal preconditioner from zero coefficients until an iteration changes "
                    f"each component's objective by less than {KL_FTOL_REL} relative (at most {KL_MAX_ITERS} "
                    f"iterations)",
        "objective": float(r_g["total_loss"]), "objective_per_component": [float(v) for v in loss_g],
        "grad_norm": float(r_g["grad_norm"]), "iterations": int(r_g["iterations"]),
        "steps": int(r_g["steps"]), "train_ms_per_step": float(r_g["ms_per_step"]),
        "train_total_ms": float(r_g["total_ms"]), "gpu_launches": int(launches),
        "step_ms_at_trained_coeffs": {"graph_batched": ms[0], "direct_batched": ms[1],
                                      "per_component_fused": ms[2], "per_component_reference_calls": ms[3]},
        "batched_speedup_vs_reference_calls": ms[3] / ms[0],
        "batched_speedup_vs_per_component_fused": ms[2] / ms[0],
        "step_values_at_trained_coeffs": step_diff,
        "train_objective_reference_calls": float(r_r["total_loss"]),
        "train_objective_max_abs_diff_vs_reference_calls": float(np.max(np.abs(loss_g - loss_r))),
        "train_objective_per_component_reference_calls": [float(v) for v in loss_r],
        "reference_calls_train_iterations": int(r_r["iterations"]),
        "reference_calls_train_ms_per_step": float(r_r["ms_per_step"]),
    }, trained, (np.asarray(steps[0][1]), np.asarray(steps[0][2]))


def batch_specs(n_maps=64, seed=17):
    """Batched-maps workload: n_maps triangular maps (inputDim = outputDim),
    dims uniform in 2..16, total orders uniform in 2..6, point counts
    log-uniform in [1e3, 2e5]."""
    rng = np.random.default_rng(seed)
    dims = rng.integers(2, 17, n_maps)
    orders = rng.integers(2, 7, n_maps)
    npts = np.exp(rng.uniform(np.log(1e3), np.log(2e5), n_maps)).astype(int)
    return list(zip(dims.tolist(), orders.tolist(), npts.tolist()))


def batch_setup(M, dev):
    """The batched-maps workload (batch_specs) as one MapBatch call."""
    import torch
    opts = M.MapOptions(quadType=M.QuadTypes.AdaptiveClenshawCurtis, quadAbsTol=TOL, quadRelTol=TOL,
                        quadMaxSub=MAXSUB)
    rng = np.random.default_rng(18)
    maps, pts, sens = [], [], []
    for d, o, n in batch_specs():
        tm = M.CreateTriangular(d, d, o, opts)
        tm.SetCoeffs(rng.normal(0.0, 0.05, tm.numCoeffs))
        maps.append(tm)
        pts.append(torch.as_tensor(rng.standard_normal((d, n)), device=dev))
        sens.append(torch.as_tensor(rng.standard_normal((d, n)), device=dev))
    z = lambda *s: torch.zeros(*s, dtype=torch.float64, device=dev)
    ev = [z(m.outputDim, p.shape[1]) for m, p in zip(maps, pts)]
    ld = [z(p.shape[1]) for p in pts]
    cg = [z(m.numCoeffs) for m in maps]
    B = M.MapBatch(maps)
    return lambda: B.FusedForwardAdjoint(pts, sens, 1.0, ev, ld, cg)


def batch_maps(M, dev, autotune=True):
    """64 uneven maps: forward + log-determinant + coefficient adjoint of every
    map as one persistent launch (before and after autotuning) against one
    fused call per map; gradients compared."""
    import torch
    opts = M.MapOptions(quadType=M.QuadTypes.AdaptiveClenshawCurtis, quadAbsTol=TOL, quadRelTol=TOL,
                        quadMaxSub=MAXSUB)
    specs = batch_specs()
    rng = np.random.default_rng(18)
    maps, pts, sens = [], [], []
    for d, o, n in specs:
        tm = M.CreateTriangular(d, d, o, opts)
        tm.SetCoeffs(rng.normal(0.0, 0.05, tm.numCoeffs))
        maps.append(tm)
        pts.append(torch.as_tensor(rng.standard_normal((d, n)), device=dev))
        sens.append(torch.as_tensor(rng.standard_normal((d, n)), device=dev))
    z = lambda *s: torch.zeros(*s, dtype=torch.float64, device=dev)
    ev = [z(m.outputDim, p.shape[1]) for m, p in zip(maps, pts)]
    ld = [z(p.shape[1]) for p in pts]
    cg = [z(m.numCoeffs) for m in maps]
    cg1 = [z(m.numCoeffs) for m in maps]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def per_map():
        for m, p, s, e, l, g in zip(maps, pts, sens, ev, ld, cg1):
            m.FusedForwardAdjointImpl(p, sens=s, logdet_sens_scale=1.0, out_eval=e, out_logdet=l, coeff_grad=g)

    def timed(f, reps=3):
        f()
        torch.cuda.synchronize()
        best = 1e300
        for _ in range(reps):
            e0.record()
            f()
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        return best

    B = M.MapBatch(maps)
    batch = lambda: B.FusedForwardAdjoint(pts, sens, 1.0, ev, ld, cg)
    ms_single = timed(per_map)
    ms_default = timed(batch)
    out = {"workload": "64 TriangularMaps, dims uniform 2..16, total orders uniform 2..6, points log-uniform in "
                       "[1e3, 2e5], ProbHermite + SoftPlus, ACC tol 1e-6; forward + LogDeterminant + coefficient "
                       "adjoint of every map",
           "maps": len(maps), "points": int(sum(n for _, _, n in specs)),
           "coefficients": int(sum(m.numCoeffs for m in maps)),
           "per_map_fused_calls_ms": ms_single, "batch_ms_default_tuning": ms_default}
    if autotune:
        t0 = time.perf_counter()
        B.Autotune(pts, sens, 1.0, reps=1)
        out["autotune_s"] = time.perf_counter() - t0
        tpb, tiles = B.Tuning()
        out["tuning"] = {"block": tpb, "tiles_per_item": {f"d{d}_o{o}": t for (d, o), t in sorted(tiles.items())}}
    l0 = M.launch_count()
    ms_tuned = timed(batch)
    out["batch_ms"] = ms_tuned
    out["batch_gpu_launches_per_call"] = (M.launch_count() - l0) // 4
    out["points_per_s"] = out["points"] / (ms_tuned * 1e-3)
    out["speedup_vs_per_map_calls"] = ms_single / ms_tuned
    worst = 0.0
    for a, b in zip(cg, cg1):
        a, b = a.cpu().numpy(), b.cpu().numpy()
        worst = max(worst, float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)))
    out["grad_max_abs_diff_over_max_vs_per_map"] = worst
    return out


INV_DIM, INV_ORDER, INV_N, INV_TOL, INV_XTOL = 16, 3, 4_000_000, 1e-8, 1e-10
INV_PARITY_N = 20_000


def inverse_implicit(M, dev, cpu_seconds=8.0, parity=True):
    """Inverse at scale with implicit differentiation: a 16-D TriangularMap of
    total order 3 (969 terms in the last component), ProbHermite + SoftPlus,
    tol 1e-8, coefficients N(0, 0.03^2); 4,000,000 targets r ~ N(0, I_16);
    Inverse to xtol 1e-10, then the coefficient gradient (and dL/dr) of the
    random linear functional L = sum w * x by the implicit-function rule."""
    import torch
    opts = M.MapOptions(quadType=M.QuadTypes.AdaptiveClenshawCurtis, quadAbsTol=INV_TOL, quadRelTol=INV_TOL,
                        quadMaxSub=MAXSUB)
    tm = M.CreateTriangular(INV_DIM, INV_DIM, INV_ORDER, opts)
    coef = np.random.default_rng(31).normal(0.0, 0.03, tm.numCoeffs)
    tm.SetCoeffs(coef)
    g = torch.Generator(device=dev)
    g.manual_seed(32)
    r = torch.randn(INV_DIM, INV_N, dtype=torch.float64, device=dev, generator=g)
    w = torch.randn(INV_DIM, INV_N, dtype=torch.float64, device=dev, generator=g)
    x1 = torch.zeros(0, INV_N, dtype=torch.float64, device=dev)
    x = torch.zeros(INV_DIM, INV_N, dtype=torch.float64, device=dev)
    cg = torch.zeros(tm.numCoeffs, dtype=torch.float64, device=dev)
    pg = torch.zeros(INV_DIM, INV_N, dtype=torch.float64, device=dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(f, reps=2):
        f()
        torch.cuda.synchronize()
        best = 1e300
        for _ in range(reps):
            e0.record()
            f()
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        return best

    xn = torch.zeros_like(x)
    ms_newton = timed(lambda: tm.InverseImpl(x1, r, xn, xtol=INV_XTOL, ytol=INV_XTOL, method="Newton"))
    ms_inv = timed(lambda: tm.InverseImpl(x1, r, x, xtol=INV_XTOL, ytol=INV_XTOL))
    ok = ~torch.isnan(x).any(dim=0)
    newton_dx = float((xn[:, ok] - x[:, ok]).abs().max().item()) if bool(ok.any()) else 0.0
    del xn
    xs, ws = x[:, ok].contiguous(), w[:, ok].contiguous()
    ms_grad = timed(lambda: tm.InverseCoeffGradImpl(xs, ws, cg, pg[:, :xs.shape[1]]))
    out = {"workload": f"TriangularMap {INV_DIM}-D, total order {INV_ORDER} ({tm.numCoeffs} coefficients, 969 in the "
                       f"last component), ProbHermite + SoftPlus, ACC tol {INV_TOL}; {INV_N} targets r ~ N(0, I); "
                       f"Inverse to xtol {INV_XTOL}, then dL/dc and dL/dr of L = sum w * x (implicit rule)",
           "points": INV_N, "inverse_method": "Bracket (FindBracket + ITP, the reference's solver)",
           "inverse_ms": ms_inv, "inverse_points_per_s": INV_N / (ms_inv * 1e-3),
           "inverse_newton_ms": ms_newton, "inverse_newton_points_per_s": INV_N / (ms_newton * 1e-3),
           "newton_vs_itp_max_abs_dx": newton_dx,
           "no_root_fraction": float(1.0 - ok.double().mean().item()),
           "implicit_grad_ms": ms_grad, "implicit_grad_points_per_s": xs.shape[1] / (ms_grad * 1e-3),
           "coeff_grad_norm": float(cg.norm().item())}
    # the oracle's Inverse on a bounded sample of the same targets (host cores)
    out["cpu_inverse"] = cpu_leg("inverse", coef=coef, r=r[:, :20000].cpu().numpy(), seconds=cpu_seconds)
    out["inverse_speedup_vs_cpu"] = out["inverse_points_per_s"] / out["cpu_inverse"]["points_per_s"]
    if parity:
        # the timed ITP roots of the first INV_PARITY_N targets against the
        # oracle's ITP, component by component
        out["parity_sample"] = cpu_leg("inverse-parity", coef=coef, r=r[:, :INV_PARITY_N].cpu().numpy(),
                                       x=x[:, :INV_PARITY_N].cpu().numpy())
    return out


def sigmoid_centers(num_sig, bound=3.0):
    """Edge centers at +-bound and, for term k, k centers spread over the
    range (the Linear sum of the reference's sigmoid factory test)."""
    c = [-bound, bound]
    for k in range(1, num_sig + 1):
        c += [1.9 * bound * (j - (k - 1) / 2) / max(k - 1, 1) for j in range(k)]
    return np.array(c)


def sigmoid_setup(M, dev):
    """The sigmoid workload: an 8-D sigmoid TriangularMap (total order 3, 5
    Linear sigmoid terms, HermiteFunctions + SoftPlus), coefficients with
    non-negative diagonal terms, 1,000,000 points N(0, I) and sensitivities."""
    import torch
    opts = M.MapOptions(basisType=M.BasisTypes.HermiteFunctions, posFuncType=M.PosFuncTypes.SoftPlus)
    cen = np.column_stack([sigmoid_centers(SIG_NSIG)] * SIG_DIM)
    tm = M.CreateSigmoidTriangular(SIG_DIM, SIG_DIM, SIG_ORDER, cen, opts)
    lb, _ = tm.CoeffBounds()
    rng = np.random.default_rng(41)
    coef = rng.normal(0.0, 0.05, tm.numCoeffs)
    coef[lb == 0.0] = np.abs(coef[lb == 0.0]) + 0.01
    tm.SetCoeffs(coef)
    xh = rng.standard_normal((SIG_DIM, SIG_N))
    sh = rng.standard_normal((SIG_DIM, SIG_N))
    x = torch.as_tensor(xh, device=dev)
    s = torch.as_tensor(sh, device=dev)
    ev = torch.zeros(SIG_DIM, SIG_N, dtype=torch.float64, device=dev)
    ld = torch.zeros(SIG_N, dtype=torch.float64, device=dev)
    cg = torch.zeros(tm.numCoeffs, dtype=torch.float64, device=dev)
    step = lambda: tm.FusedForwardAdjointImpl(x, sens=s, logdet_sens_scale=1.0, out_eval=ev, out_logdet=ld,
                                              coeff_grad=cg)
    return tm, cen, coef, xh, sh, x, step


def sigmoid_maps(M, dev, steps=10, cpu_seconds=8.0):
    """Sigmoid expansions (CreateSigmoidTriangular, see sigmoid_setup): the
    fused forward + log-determinant + coefficient adjoint and the batched KL
    step on 1,000,000 points; the oracle's four reference calls on a sample
    of the same points on the host cores."""
    import torch
    tm, cen, coef, xh, sh, x, step = sigmoid_setup(M, dev)
    flush = torch.empty(256 * 1024 * 1024 // 8, dtype=torch.float64, device=dev)
    kl = lambda: tm.KLObjective(x)

    def timed(f):
        for _ in range(3):
            f()
        torch.cuda.synchronize()
        ms = []
        for k in range(steps):
            flush.fill_(float(k))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            f()
            e1.record()
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        return float(np.median(ms))

    ms_fused = timed(step)
    ms_kl = timed(kl)
    out = {"workload": f"sigmoid TriangularMap {SIG_DIM}-D (RectifiedMultivariateExpansion components), total order "
                       f"{SIG_ORDER}, {SIG_NSIG} sigmoid terms (Linear), HermiteFunctions + SoftPlus, "
                       f"{tm.numCoeffs} coefficients, {SIG_N} points N(0, I); fused Evaluate + LogDeterminant + "
                       f"CoeffGrad + LogDeterminantCoeffGrad (coefficient adjoint summed over points)",
           "points": SIG_N, "coefficients": tm.numCoeffs, "fused_ms": ms_fused,
           "fused_points_per_s": SIG_N / (ms_fused * 1e-3), "kl_step_ms": ms_kl,
           "l2": "flushed between steps (256 MB write)"}
    # the oracle on a bounded sample: the reference's four calls per component
    nmax = 400_000
    out["cpu_baseline"] = cpu_leg("sigmoid", cen=cen, coef=coef, x=xh[:, :nmax], s=sh[:, :nmax], seconds=cpu_seconds)
    out["speedup_vs_cpu"] = out["fused_points_per_s"] / out["cpu_baseline"]["points_per_s"]
    return out


def leg_inverse(a):
    """The oracle's Inverse of the inverse workload's map on a bounded sample
    of its targets (child process, timing build)."""
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    O.set_threads(cores)
    om = O.OracleTriangularMap(INV_DIM, INV_DIM, INV_ORDER, abs_tol=INV_TOL, rel_tol=INV_TOL, max_sub=MAXSUB)
    coef, rh, seconds = a["coef"], a["r"], float(a["seconds"])
    n = 200
    t0 = time.perf_counter()
    om.inverse(coef, np.zeros((0, n)), rh[:, :n], INV_XTOL, INV_XTOL)
    dt = time.perf_counter() - t0
    n2 = int(min(rh.shape[1], max(n, n * seconds / max(dt, 1e-6))))
    t0 = time.perf_counter()
    om.inverse(coef, np.zeros((0, n2)), rh[:, :n2], INV_XTOL, INV_XTOL)
    dt = time.perf_counter() - t0
    return {"points_per_s": n2 / dt, "cores": cores, "kind": "port",
            "sample": f"first {n2} targets, the oracle's Inverse (FindBracket + ITP); {CPU_BUILD}"}


def leg_inverse_parity(a):
    """The GPU's ITP roots against the oracle's (parity build), component by
    component: the oracle solves component c from the GPU's own earlier
    coordinates (child process).  The bar of the GPU tests: the same targets
    without a root (NaN); roots within 2 (xtol + ytol / slope), and, for at
    most 0.2 % of them (a last-bit change of T flipping an accept test of the
    adaptive quadrature), within 2 (xtol + (ytol + tol (1 + |r|)) / slope)."""
    from oracle import oracle as O
    O.build()
    O.set_threads(os.cpu_count() or 1)
    om = O.OracleTriangularMap(INV_DIM, INV_DIM, INV_ORDER, abs_tol=INV_TOL, rel_tol=INV_TOL, max_sub=MAXSUB)
    coef, r, xg = np.asarray(a["coef"]), np.asarray(a["r"]), np.asarray(a["x"])
    n = r.shape[1]
    cs = om.split(coef)
    t0 = time.perf_counter()
    nan_mismatch = strict_out = loose_out = roots = 0
    worst = 0.0
    for c, comp in enumerate(om.comps):
        guess = np.zeros((comp.input_dim, n))
        guess[:-1] = xg[:comp.input_dim - 1]
        ref = comp.inverse(cs[c], guess, r[c], INV_XTOL, INV_XTOL)
        got = xg[c]
        nan_mismatch += int((np.isnan(ref) != np.isnan(got)).sum())
        ok = ~np.isnan(ref) & ~np.isnan(got)
        pt = guess.copy()
        pt[-1] = np.where(ok, ref, 0.0)
        slope = np.maximum(comp.cont_derivative(cs[c], pt), 1e-300)
        diff = np.abs(got - ref)
        bound = 2.0 * (INV_XTOL + INV_XTOL / slope)
        loose = 2.0 * (INV_XTOL + (INV_XTOL + INV_TOL * (1.0 + np.abs(r[c]))) / slope)
        strict_out += int((ok & (diff > bound)).sum())
        loose_out += int((ok & (diff > loose)).sum())
        roots += int(ok.sum())
        if ok.any():
            worst = max(worst, float(np.max(diff[ok] / bound[ok])))
    return {"targets": n, "components": len(om.comps), "roots": roots, "oracle_s": time.perf_counter() - t0,
            "nan_pattern_mismatches": nan_mismatch, "outside_2(xtol+ytol/slope)": strict_out,
            "outside_loose_bound": loose_out, "max_diff_over_strict_bound": worst,
            "bar": "NaN at the same targets; roots within 2 (xtol + ytol / slope) of the oracle's ITP, at most "
                   "0.2 % within 2 (xtol + (ytol + tol (1 + |r|)) / slope) instead"}


def leg_sigmoid(a):
    """The oracle's four reference calls per component of the sigmoid map on a
    bounded sample of its points (child process, timing build)."""
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    O.set_threads(cores)
    om = O.sigmoid_triangular(SIG_DIM, SIG_DIM, SIG_ORDER, a["cen"], 1.5, O.SUM_LINEAR, O.POS_SOFTPLUS)
    coef, xh, sh, seconds = a["coef"], a["x"], a["s"], float(a["seconds"])

    def cpu(n):
        xs, ss = np.ascontiguousarray(xh[:, :n]), np.ascontiguousarray(sh[:, :n])
        t0 = time.perf_counter()
        om.evaluate(coef, xs)
        om.logdet(coef, xs)
        om.coeff_grad(coef, xs, ss).sum(axis=1)
        om.logdet_coeff_grad(coef, xs).sum(axis=1)
        return time.perf_counter() - t0

    n = 2000
    dt = cpu(n)
    n2 = int(min(xh.shape[1], max(n, n * seconds / max(dt, 1e-6))))
    dt = cpu(n2)
    return {"points_per_s": n2 / dt, "cores": cores, "kind": "port",
            "sample": f"first {n2} of the {SIG_N} points, the oracle's Evaluate + LogDeterminant + CoeffGrad + "
                      f"LogDeterminantCoeffGrad per component, gradients summed; {CPU_BUILD}"}


def cpu_leg(name, **arrays):
    """Runs a CPU leg of this benchmark in a child process (the oracle's
    timing build, threads bound one per core) and returns its JSON result.
    Arrays travel through a temporary .npz file."""
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        f = os.path.join(d, "in.npz")
        np.savez(f, **{k: np.asarray(v) for k, v in arrays.items()})
        env = dict(os.environ, **TIMING_ENV)
        if name in ("c2-parity", "kl-parity", "inverse-parity"):
            env.pop("MPGB_ORACLE_BUILD")  # parity: the strict build
        r = subprocess.run([sys.executable, os.path.abspath(__file__), "--cpu-leg", name, "--cpu-in", f],
                           env=env, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"CPU leg {name} failed: {r.stderr[-2000:]}")
        return json.loads(r.stdout.strip().splitlines()[-1])


def run_cpu_leg(args):
    a = dict(np.load(args.cpu_in)) if args.cpu_in else {}
    legs = {"c2": lambda: cpu_baseline(),
            "c2-parity": lambda: leg_c2_parity(a),
            "kl": lambda: kl_cpu_step_ms(a["coeffs"]),
            "kl-parity": lambda: leg_kl_parity(a),
            "inverse": lambda: leg_inverse(a),
            "inverse-parity": lambda: leg_inverse_parity(a),
            "sigmoid": lambda: leg_sigmoid(a)}
    print(json.dumps(legs[args.cpu_leg]()), flush=True)


def kl_cpu_step_ms(coeffs, target_seconds=8.0):
    """The oracle's KL step (every component's FastGaussianReverseKLObjective
    value and gradient, src/MapObjective.cpp:185-234, as TrainMap evaluates
    them one component at a time) at the given coefficients on a bounded
    sample, scaled to KL_N."""
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    O.set_threads(cores)
    tmo = O.OracleTriangularMap(KL_DIM, KL_DIM, KL_ORDER, basis=O.BASIS_HERMITE_FUNCTIONS, posfunc=O.POS_EXP,
                                abs_tol=KL_TOL, rel_tol=KL_TOL)
    c = np.asarray(coeffs, dtype=np.float64)
    X = banana(KL_N)

    def step(n):
        t0 = time.perf_counter()
        for comp, cc in zip(tmo.comps, tmo.split(c)):
            O.fast_gaussian_reverse_kl(comp, cc, np.ascontiguousarray(X[:comp.input_dim, :n]))
        return time.perf_counter() - t0

    n = 2000
    dt = step(n)
    n2 = int(min(KL_N, max(n, n * target_seconds / max(dt, 1e-6))))
    dt = step(n2)
    return {"ms_per_step": dt * 1e3 * KL_N / n2, "cores": cores, "kind": "port",
            "sample": f"first {n2} of the {KL_N} samples at the trained coefficients, scaled to {KL_N}; {CPU_BUILD}"}


def prefix_stats():
    """|M| (prefix nodes incl. root), T, nB and sum over term-carrying prefixes
    of max(depth-1, 0) for the total-order set -- inputs of the FLOP model."""
    from mpart_gb300 import FixedMultiIndexSet
    ms = FixedMultiIndexSet(DIM, ORDER)
    prefixes = {}
    for t in range(ms.Size()):
        m = ms.IndexToMulti(t)
        key = tuple(m[:-1])
        prefixes.setdefault(key, 0)
        prefixes[key] += 1
    nodes = len(prefixes)
    sc = sum(max(sum(1 for v in k if v > 0) - 1, 0) for k in prefixes)
    return nodes, ms.Size(), (DIM - 1) * ORDER, sc


def flops_per_point(evals_per_point):
    """Algorithmic FP64 flops of the fused algorithm per point (FMA = 2,
    exp/log/reciprocal = 1 each), with the mean integrand evaluations per
    point E and intervals I = (E - 2) / 3:
      A  prefix products + coefficient FMAs      (|M|-1) + 2T
      L  leading-coordinate recurrences          3 nB
      N  per node: basis 4P, df 2P, g/g' 8, h 2, adjoint parts P   -> 7P + 10
      Q  per interval: coarse/fine sums of h and of the P adjoint parts -> 18 + 10P
      X  endpoint x_D terms (log-det)            9P + 10
      W  per-point weights                       4(P+1)
      C  reduction over points: products + FMAs  S_C + 2T"""
    nodes, T, nB, sc = prefix_stats()
    P = ORDER
    E = evals_per_point
    I = (E - 2.0) / 3.0
    return ((nodes - 1) + 2 * T) + 3 * nB + E * (7 * P + 10) + I * (18 + 10 * P) + (9 * P + 10) + 4 * (P + 1) + \
        (sc + 2 * T)


def reference_flops_per_point(evals_per_point):
    """FP64 flops per point of the reference's own (unfactored) algorithm for
    the same fused step, counted from its term loops
    (MultivariateExpansionWorker.h, MonotoneIntegrand.h, MonotoneComponent.h):
    per integrand node with the coefficient gradient (the Parameters part)
      2 sum_{t with x_D} k_t   term products and coefficient FMAs of d_D f
      + 3 (p_D + 1)            last-coordinate recurrence and its derivative
      + 20                     g, g', weights, accumulation
      + 3 T_D                  scale and coarse/fine sums per gradient entry
    and per point once
      3 sum_{d < D} (p_d + 1)  leading-coordinate recurrences
      + 2 sum_t k_t + T        f(x_<D, 0) and its coefficient gradient,
    with k_t the nonzero factors of term t, T_D the terms that contain x_D,
    transcendentals at 1.  The fused kernel computes the same quantities
    with fewer operations (prefix products, a_k sums), so this count divided
    by the step time exceeds the FP64 peak; it says how much arithmetic the
    factoring removes, not how busy the pipe is."""
    from mpart_gb300 import FixedMultiIndexSet
    ms = FixedMultiIndexSet(DIM, ORDER)
    ks, kd, td = 0, 0, 0
    for t in range(ms.Size()):
        m = ms.IndexToMulti(t)
        k = sum(1 for v in m if v > 0)
        ks += k
        if m[-1] > 0:
            kd += k
            td += 1
    node = 2 * kd + 3 * (ORDER + 1) + 20 + 3 * td
    fixed = 3 * (DIM - 1) * (ORDER + 1) + 2 * ks + ms.Size()
    return evals_per_point * node + fixed


def mean_evals(sample=20000):
    """Mean integrand evaluations per point from the oracle's node counts (the
    GPU follows the same subdivision tree)."""
    from oracle import oracle as O
    O.build()
    s, d, o = O.total_order(DIM, ORDER)
    c = O.OracleComponent(DIM, s, d, o, abs_tol=TOL, rel_tol=TOL, max_sub=MAXSUB)
    x, _ = synth(sample)
    _, nev, _ = c.evaluate(coeffs(c.num_terms), x, return_evals=True)
    return float(nev.mean())


class Clocks:
    """nvidia-smi sampling during the timed region.  A reader thread stamps
    each sample with the host clock on arrival; only samples that arrive
    while the region is open (plus one interval after it closes) count, so a
    sample taken while nvidia-smi starts up or after the region is dropped."""

    INTERVAL_MS = 50

    def __init__(self, index):
        self.p = None
        self.index = index
        self.stamped = []
        self.t0 = self.t1 = None

    def _read(self):
        for line in self.p.stdout:
            if line.strip():
                self.stamped.append((time.monotonic(), line))

    def __enter__(self):
        import threading
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}",
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", str(self.INTERVAL_MS)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
            deadline = time.monotonic() + 5.0  # wait for the sampler to be running
            while not self.stamped and time.monotonic() < deadline:
                time.sleep(0.01)
        except Exception:
            self.p = None
        self.t0 = time.monotonic()
        return self

    def __exit__(self, *a):
        self.t1 = time.monotonic()
        self.lines = []
        if self.p is not None:
            time.sleep(self.INTERVAL_MS / 1000.0 * 1.5)
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()
            self.th.join(timeout=5)
            hi = self.t1 + self.INTERVAL_MS / 1000.0
            self.lines = [l for t, l in self.stamped if self.t0 < t <= hi]

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [v.strip() for v in l.split(",")]
            try:
                sm.append(float(f[0]))
                smax = float(f[1])
            except Exception:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower() in ("active", "1"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        return json.load(open(p))
    except Exception:
        return {}


# ----------------------------------------------------------------------------
# reference arm: the reference algorithm on the host cores
# ----------------------------------------------------------------------------
def cpu_reference_step(comp, coef, x, s):
    """Evaluate, LogDeterminant, CoeffGrad(sens) and LogDeterminantCoeffGrad
    (the reference's four calls, MonotoneComponent.h), reduced over points."""
    comp.evaluate(coef, x)
    comp.logdet(coef, x)
    g = comp.coeff_grad(coef, x, s[0])
    lg = comp.logdet_coeff_grad(coef, x)
    return g.sum(axis=1) + lg.sum(axis=1)


def cpu_baseline(target_seconds=12.0):
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    O.set_threads(cores)
    s_, d_, o_ = O.total_order(DIM, ORDER)
    comp = O.OracleComponent(DIM, s_, d_, o_, abs_tol=TOL, rel_tol=TOL, max_sub=MAXSUB)
    coef = coeffs(comp.num_terms)
    n = 2000
    x, s = synth(n)
    t0 = time.perf_counter()
    cpu_reference_step(comp, coef, x, s)
    dt = time.perf_counter() - t0
    n2 = int(min(NPTS, max(n, n * target_seconds / max(dt, 1e-6))))
    x, s = synth(n2)
    t0 = time.perf_counter()
    cpu_reference_step(comp, coef, x, s)
    dt = time.perf_counter() - t0
    return {"value": n2 / dt, "unit": "points/s", "cores": cores, "kind": "port",
            "sample": f"first {n2} of the {NPTS} points (same seeds), reference algorithm restated in "
                      f"oracle/ (C++17 + OpenMP, {cores} threads): Evaluate + LogDeterminant + CoeffGrad + "
                      f"LogDeterminantCoeffGrad, gradients summed over points; {CPU_BUILD}"}


def leg_kl_parity(a):
    """The batched KL step's per-component objectives and coefficient
    gradient at the trained coefficients against the oracle's parity build
    (FastGaussianReverseKLObjective per component, src/MapObjective.cpp:185-234)
    on all KL_N samples (child process): 1e-10 relative, the gradient (a mean
    over samples) floored at 1e-3 of its largest entry."""
    from oracle import oracle as O
    O.build()
    O.set_threads(os.cpu_count() or 1)
    tmo = O.OracleTriangularMap(KL_DIM, KL_DIM, KL_ORDER, basis=O.BASIS_HERMITE_FUNCTIONS, posfunc=O.POS_EXP,
                                abs_tol=KL_TOL, rel_tol=KL_TOL)
    X = banana(KL_N)
    t0 = time.perf_counter()
    loss, grad = [], []
    for comp, cc in zip(tmo.comps, tmo.split(np.asarray(a["coeffs"], dtype=np.float64))):
        l, g = O.fast_gaussian_reverse_kl(comp, cc, np.ascontiguousarray(X[:comp.input_dim]))
        loss.append(l)
        grad.append(np.asarray(g))
    dt = time.perf_counter() - t0
    loss, grad = np.array(loss), np.concatenate(grad)

    def check(g, r, floor):
        scale = np.nanmax(np.abs(r))
        tol = 1e-10 * np.maximum(np.abs(r), floor * scale)
        bad = ~((g == r) | (np.isnan(g) & np.isnan(r)) | (np.abs(g - r) <= tol))
        with np.errstate(invalid="ignore"):
            rel = np.abs(g - r) / np.maximum(np.abs(r), floor * scale)
        return {"entries": int(r.size), "outside_tol": int(bad.sum()),
                "max_rel_err": float(np.nanmax(rel)) if np.isfinite(rel).any() else None}

    return {"samples": KL_N, "oracle_s": dt,
            "tolerance": "1e-10 relative (the gradient floored at 1e-3 of its largest entry)",
            "objective_per_component": check(np.asarray(a["loss"]), loss, 0.0),
            "coeff_grad": check(np.asarray(a["grad"]), grad, 1e-3)}


def leg_c2_parity(a, chunk=50_000):
    """The timed run's outputs (T, log-det, reduced coefficient gradient)
    against the oracle's parity build on every one of the NPTS points (child
    process).  Per entry the bar of the GPU tests: |gpu - oracle| <=
    1e-10 max(|oracle|, 1e-6 max|oracle|), the gradient (a sum over points)
    floored at 1e-3 of its largest entry."""
    from oracle import oracle as O
    O.build()
    O.set_threads(os.cpu_count() or 1)
    s_, d_, o_ = O.total_order(DIM, ORDER)
    comp = O.OracleComponent(DIM, s_, d_, o_, abs_tol=TOL, rel_tol=TOL, max_sub=MAXSUB)
    coef = coeffs(comp.num_terms)
    x, sv = synth(NPTS)
    T = np.empty(NPTS)
    ld = np.empty(NPTS)
    cg = np.zeros(comp.num_terms)
    t0 = time.perf_counter()
    for k in range(0, NPTS, chunk):
        xs, ss = np.ascontiguousarray(x[:, k:k + chunk]), sv[:, k:k + chunk]
        T[k:k + chunk] = comp.evaluate(coef, xs)
        ld[k:k + chunk] = comp.logdet(coef, xs)
        cg += comp.coeff_grad(coef, xs, ss[0]).sum(axis=1) + comp.logdet_coeff_grad(coef, xs).sum(axis=1)
    dt = time.perf_counter() - t0

    def check(g, r, floor):
        scale = np.nanmax(np.abs(r))
        tol = 1e-10 * np.maximum(np.abs(r), floor * scale)
        bad = ~((g == r) | (np.isnan(g) & np.isnan(r)) | (np.abs(g - r) <= tol))
        with np.errstate(invalid="ignore"):
            rel = np.abs(g - r) / np.maximum(np.abs(r), floor * scale)
        return {"entries": int(r.size), "outside_tol": int(bad.sum()),
                "max_rel_err": float(np.nanmax(rel)) if np.isfinite(rel).any() else None}

    return {"points": NPTS, "oracle_s": dt, "tolerance": "1e-10 relative (floor 1e-6 of the largest entry; "
                                                         "1e-3 for the gradient summed over points)",
            "evaluate": check(a["T"], T, 1e-6), "logdet": check(a["ld"], ld, 1e-6),
            "coeff_grad": check(a["cg"], cg, 1e-3)}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    # the timing build with threads bound one per core (before the OpenMP
    # runtime is loaded with the oracle)
    os.environ.update(TIMING_ENV)
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    O.set_threads(cores)
    s_, d_, o_ = O.total_order(DIM, ORDER)
    comp = O.OracleComponent(DIM, s_, d_, o_, abs_tol=TOL, rel_tol=TOL, max_sub=MAXSUB)
    coef = coeffs(comp.num_terms)
    n = int(os.environ.get("MPGB_REF_SAMPLE", "20000"))
    x, s = synth(n)
    for _ in range(args.warmup):
        cpu_reference_step(comp, coef, x[:, :min(n, 2000)], s[:, :min(n, 2000)])
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cpu_reference_step(comp, coef, x, s)
    dt = (time.perf_counter() - t0) / args.steps
    v = n / dt
    sample = (f"{n} of the {NPTS} points per step (same seeds); reference algorithm restated in oracle/ "
              f"(C++17 + OpenMP, {cores} threads); {CPU_BUILD}; the reference itself does not build here")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "points/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"MonotoneComponent dim {DIM}, total order {ORDER} (495 terms), ProbHermite + "
                                   f"SoftPlus, ACC tol {TOL}, {NPTS} points", "points": NPTS, "sample_points": n},
            "cpu_baseline": {"value": v, "unit": "points/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------
# our arm
# ----------------------------------------------------------------------------
def run_gpu(args):
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    import mpart_gb300 as M
    M.load()
    opts = M.MapOptions(quadType=M.QuadTypes.AdaptiveClenshawCurtis, quadAbsTol=TOL, quadRelTol=TOL,
                        quadMaxSub=MAXSUB)
    comp = M.CreateComponent(M.FixedMultiIndexSet(DIM, ORDER), opts)
    coef = coeffs(comp.numCoeffs)
    comp.SetCoeffs(coef)
    N = args.points
    xh, sh = synth(N)
    x = torch.as_tensor(xh, device=dev)
    s = torch.as_tensor(sh, device=dev)
    out_T = torch.zeros(1, N, dtype=torch.float64, device=dev)
    out_ld = torch.zeros(N, dtype=torch.float64, device=dev)
    cg = torch.zeros(comp.numCoeffs, dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 8, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step():
        comp.FusedForwardAdjointImpl(x, sens=s, logdet_sens_scale=1.0, out_eval=out_T, out_logdet=out_ld,
                                     coeff_grad=cg)

    if args.profile and args.variant != "full":
        # Phase isolation for profiling: evaluate only (A + value quadrature),
        # log-det only (A), or the reduced adjoint without quadrature (A + C).
        variants = {
            "eval": lambda: comp.EvaluateImpl(x, out_T),
            "logdet": lambda: comp.LogDeterminantImpl(x, out_ld),
            "reduce": lambda: comp.FusedForwardAdjointImpl(x, logdet_sens_scale=1.0, coeff_grad=cg),
        }
        if args.variant == "sigmoid":
            # The sigmoid workload's fused step (see sigmoid_setup).
            step = sigmoid_setup(M, dev)[-1]
        elif args.variant in ("inverse", "inverse-newton"):
            # The inverse workload's map on 100,000 of its targets (ITP, or the Newton option).
            iopts = M.MapOptions(quadType=M.QuadTypes.AdaptiveClenshawCurtis, quadAbsTol=INV_TOL,
                                 quadRelTol=INV_TOL, quadMaxSub=MAXSUB)
            tmi = M.CreateTriangular(INV_DIM, INV_DIM, INV_ORDER, iopts)
            tmi.SetCoeffs(np.random.default_rng(31).normal(0.0, 0.03, tmi.numCoeffs))
            g = torch.Generator(device=dev)
            g.manual_seed(32)
            ri = torch.randn(INV_DIM, 100_000, dtype=torch.float64, device=dev, generator=g)
            x1i = torch.zeros(0, 100_000, dtype=torch.float64, device=dev)
            xi = torch.zeros(INV_DIM, 100_000, dtype=torch.float64, device=dev)
            meth = "Newton" if args.variant == "inverse-newton" else "Bracket"
            step = lambda: tmi.InverseImpl(x1i, ri, xi, xtol=INV_XTOL, ytol=INV_XTOL, method=meth)
        elif args.variant == "implicit":
            # The inverse workload's map: Inverse of 500,000 of its targets,
            # then the implicit gradient (InverseCoeffGradImpl) at the finite
            # roots; a step is one implicit-gradient call (16 fused launches,
            # the last component's first).
            iopts = M.MapOptions(quadType=M.QuadTypes.AdaptiveClenshawCurtis, quadAbsTol=INV_TOL,
                                 quadRelTol=INV_TOL, quadMaxSub=MAXSUB)
            tmi = M.CreateTriangular(INV_DIM, INV_DIM, INV_ORDER, iopts)
            tmi.SetCoeffs(np.random.default_rng(31).normal(0.0, 0.03, tmi.numCoeffs))
            g = torch.Generator(device=dev)
            g.manual_seed(32)
            ri = torch.randn(INV_DIM, 500_000, dtype=torch.float64, device=dev, generator=g)
            wi = torch.randn(INV_DIM, 500_000, dtype=torch.float64, device=dev, generator=g)
            x1i = torch.zeros(0, 500_000, dtype=torch.float64, device=dev)
            xi = torch.zeros(INV_DIM, 500_000, dtype=torch.float64, device=dev)
            tmi.InverseImpl(x1i, ri, xi, xtol=INV_XTOL, ytol=INV_XTOL)
            fin = ~torch.isnan(xi).any(dim=0)
            xs, ws = xi[:, fin].contiguous(), wi[:, fin].contiguous()
            cgi = torch.zeros(tmi.numCoeffs, dtype=torch.float64, device=dev)
            pgi = torch.zeros(INV_DIM, xs.shape[1], dtype=torch.float64, device=dev)
            step = lambda: tmi.InverseCoeffGradImpl(xs, ws, cgi, pgi)
        elif args.variant == "batch":
            # The batched-maps workload's batch call (default tuning).
            step = batch_setup(M, dev)
        elif args.variant == "kl":
            # The KL training workload's step at trained coefficients (the
            # workload's training with direct launches first); the profiled
            # calls sit in the NVTX range "kl_step".
            opts = M.MapOptions(basisType=M.BasisTypes.HermiteFunctions, posFuncType=M.PosFuncTypes.Exp,
                                quadType=M.QuadTypes.AdaptiveClenshawCurtis, quadAbsTol=KL_TOL, quadRelTol=KL_TOL)
            X = torch.as_tensor(banana(KL_N), device=dev)
            tm = M.CreateTriangular(KL_DIM, KL_DIM, KL_ORDER, opts)
            tm.SetCoeffs(np.zeros(tm.numCoeffs))
            M.TrainMap(tm, X, mode=1, **KL_TRAIN)

            def step():
                torch.cuda.nvtx.range_push("kl_step")
                tm.KLObjective(X)
                torch.cuda.nvtx.range_pop()
        else:
            step = variants[args.variant]

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    if args.profile:
        # Profiling mode (for ncu): the fused step only, no e2e / baselines.
        for _ in range(args.steps):
            step()
        torch.cuda.synchronize()
        return
    if world > 1:
        dist.barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    launches0 = M.launch_count()
    with Clocks(local) as clk:
        torch.cuda.synchronize()
        for k in range(args.steps):
            flush.fill_(float(k))  # L2 flush (256 MB > 129 MB L2) between steps, outside the events
            ev[k][0].record(stream)
            step()
            ev[k][1].record(stream)
        torch.cuda.synchronize()
    launches = M.launch_count() - launches0
    if world > 1:
        dist.barrier()
    times = [a.elapsed_time(b) for a, b in ev]
    t_step = float(np.mean(times)) * 1e-3
    from mpart_gb300.distributed import max_over_ranks
    t_step_max = max_over_ranks(t_step * args.steps, device=dev) / args.steps
    value = world * N / t_step_max

    # e2e: C ABI with pinned host buffers (copies inside the timed region).
    xp = torch.as_tensor(xh).pin_memory()
    sp = torch.as_tensor(sh).pin_memory()
    Tp = torch.zeros(1, N, dtype=torch.float64).pin_memory()
    ldp = torch.zeros(N, dtype=torch.float64).pin_memory()
    cgp = torch.zeros(comp.numCoeffs, dtype=torch.float64).pin_memory()

    def step_e2e():
        comp.FusedForwardAdjointImpl(xp, sens=sp, logdet_sens_scale=1.0, out_eval=Tp, out_logdet=ldp,
                                     coeff_grad=cgp)

    for _ in range(2):
        step_e2e()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step_e2e()
    torch.cuda.synchronize()
    t_e2e = (time.perf_counter() - t0) / args.steps
    t_e2e = max_over_ranks(t_e2e, device=dev)
    h2d = xh.nbytes + sh.nbytes
    d2h = Tp.numel() * 8 + ldp.numel() * 8 + cgp.numel() * 8

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return
    # roofline: FP64 pipe; peak from the DFMA probe (MEASURED_PEAKS.json has no FP64 entry).
    peak_tf, _ = M.fp64_probe()
    E = mean_evals()
    fpp = flops_per_point(E)
    achieved = fpp * N / t_step / 1e12
    traffic = None
    # DRAM bytes of one fused launch from the committed ncu capture (same
    # workload), scaled to this run's point count.
    prof = os.path.join(ROOT, "profiles", "fusedKernel_dim8_order4_1M.json")
    if os.path.exists(prof):
        try:
            pr = json.load(open(prof))
            traffic = (pr["dram_bytes_read"] + pr["dram_bytes_write"]) * N / pr["points"]
        except Exception:
            traffic = None
    line = {
        "metric": METRIC, "value": value, "unit": "points/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": t_step_max * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"MonotoneComponent dim {DIM}, total order {ORDER} (495 terms), ProbHermite + "
                               f"SoftPlus, ACC tol {TOL}/maxSub {MAXSUB}, {N} points, fused Evaluate + LogDeterminant "
                               f"+ CoeffGrad + LogDeterminantCoeffGrad", "points": N, "dim": DIM, "order": ORDER,
                   "l2": "flushed between steps (256 MB write)", "parallelism": f"replicas x{world}"},
        "e2e": {"value": world * N / t_e2e, "unit": "points/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak_tf, "unit": "TFLOP/s",
                     "frac": achieved / peak_tf, "traffic": traffic,
                     "peak_source": "DFMA probe in this run (MEASURED_PEAKS.json has no FP64 figure)",
                     "flops_per_point": fpp, "evals_per_point": E,
                     "reference_algorithm": {
                         "flops_per_point": reference_flops_per_point(E),
                         "equivalent_tflops": reference_flops_per_point(E) * N / t_step / 1e12,
                         "note": "flops of the reference's unfactored term loops for the same outputs; "
                                 "above the FP64 peak because the fused kernel needs fewer"}},
        "clocks": clk.summary(),
    }
    # Against the FP64 issue rate itself: 2 DFMA lanes per SM and clock (2
    # FLOP each) at the SM clock sampled during the timed steps.
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    mhz = line["clocks"].get("sm_mhz") or line["clocks"].get("sm_max_mhz")
    if mhz:
        issue = sms * 2 * 2 * mhz * 1e6 / 1e12
        line["roofline"]["issue_rate_peak"] = issue
        line["roofline"]["frac_of_issue_rate"] = achieved / issue
    line["dense_coeff_grad"] = dense_coeff_grad(comp, x, s, N, dev)
    line["plain_path"] = plain_path(M, coef, x, s, N, dev)
    line["plain_path"]["fused_speedup"] = line["plain_path"]["ms_per_step"] / (t_step * 1e3)
    line["cpu_baseline"] = cpu_leg("c2")
    if not args.no_parity and N == NPTS:
        # the timed step's outputs (last timed step) against the oracle on every point
        line["parity_full"] = cpu_leg("c2-parity", T=out_T.cpu().numpy().reshape(-1), ld=out_ld.cpu().numpy(),
                                      cg=cg.cpu().numpy())
    if not args.no_kl:
        kl, trained, (kl_loss, kl_grad) = kl_train(M, dev)
        if not args.no_parity:
            # the batched step's values at the trained coefficients against the
            # oracle on all KL_N samples
            kl["parity_full"] = cpu_leg("kl-parity", coeffs=trained, loss=kl_loss, grad=kl_grad)
        kl["cpu_step"] = cpu_leg("kl", coeffs=trained)
        kl["cpu_step"]["speedup_graph"] = (kl["cpu_step"]["ms_per_step"] /
                                           kl["step_ms_at_trained_coeffs"]["graph_batched"])
        line["kl_train"] = kl
    if not args.no_batch:
        line["batch_maps"] = batch_maps(M, dev)
    if not args.no_inverse:
        line["inverse_implicit"] = inverse_implicit(M, dev, parity=not args.no_parity)
    if not args.no_sigmoid:
        line["sigmoid_maps"] = sigmoid_maps(M, dev)
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def dense_coeff_grad(comp, x, s, N, dev, reps=3):
    """CoeffGradImpl with its dense numCoeffs x N output (the reference's
    per-point layout): 495 x 1,000,000 doubles = 3.96 GB written per call."""
    import torch
    out = torch.empty(comp.numCoeffs, N, dtype=torch.float64, device=dev)
    comp.CoeffGradImpl(x, s, out)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = 1e300
    for _ in range(reps):
        e0.record()
        comp.CoeffGradImpl(x, s, out)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    nbytes = out.numel() * 8
    del out
    return {"ms": best, "points_per_s": N / (best * 1e-3), "output_bytes": nbytes,
            "output_gb_per_s": nbytes / (best * 1e-3) / 1e9}


def plain_path(M, coef, x, s, N, dev):
    """The reference-structured GPU path (separate Evaluate, LogDeterminant,
    CoeffGrad and LogDeterminantCoeffGrad launches with full-width quadrature
    and dense outputs, then column sums) on the same inputs."""
    import torch
    opts = M.MapOptions(quadType=M.QuadTypes.AdaptiveClenshawCurtis, quadAbsTol=TOL, quadRelTol=TOL,
                        quadMaxSub=MAXSUB)
    p = M.PlainComponent(DIM, ORDER, opts)
    c = torch.as_tensor(coef, device=dev)
    sv = s[0].contiguous()
    ev = torch.zeros(N, dtype=torch.float64, device=dev)
    ld = torch.zeros(N, dtype=torch.float64, device=dev)
    cg = torch.zeros(p.numCoeffs, dtype=torch.float64, device=dev)
    p.FwdAdj(c, x, sv, ev, ld, cg)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    p.FwdAdj(c, x, sv, ev, ld, cg)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    del p
    return {"points_per_s": N / (ms * 1e-3), "ms_per_step": ms}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="mine", choices=["mine", "reference"])
    ap.add_argument("--points", type=int, default=NPTS)
    ap.add_argument("--profile", action="store_true", help="fused step only (for profilers)")
    ap.add_argument("--no-kl", action="store_true", help="skip the KL training workload")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-maps workload")
    ap.add_argument("--no-inverse", action="store_true", help="skip the inverse / implicit-gradient workload")
    ap.add_argument("--no-sigmoid", action="store_true", help="skip the sigmoid-expansion workload")
    ap.add_argument("--no-parity", action="store_true", help="skip the full-size parity check against the oracle")
    ap.add_argument("--cpu-leg", default=None, help=argparse.SUPPRESS)
    ap.add_argument("--cpu-in", default=None, help=argparse.SUPPRESS)
    ap.add_argument("--variant", default="full",
                    choices=["full", "eval", "logdet", "reduce", "kl", "sigmoid", "inverse", "inverse-newton", "implicit",
                             "batch"],
                    help="with --profile: which part of the step to run")
    args = ap.parse_args()
    if args.cpu_leg:
        run_cpu_leg(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
