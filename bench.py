"""Benchmark: transient 3D convection-diffusion, the OpenCMP hot path on one GB300.

Workload (one "step" = one implicit-Euler time step, what OpenCMP's transient loop does per step:
reassemble the bilinear and linear forms, refresh the preconditioner, Krylov-solve to a 1e-8 FP64
relative residual from the step's initial guess):
  unit cube, 64^3 cubes x 6 tetrahedra (1,572,864 tets), H1 order 2 (2,146,689 dofs), Dirichlet 0 on
  all faces, eps = 1e-2, w = (1, 0.5, 0.25), dt = 1e-3, u0 = Gaussian (sigma 0.1 at (0.25,0.25,0.25)).
Metric: DOF/s = dofs x steps / time. `value` is the optimised path: double-float assembly, FP32-inner
GMRES with FP64 refinement, and the learned initial guess (cubic extrapolation in time plus a network
trained on the solver's own trajectories, kept only while its convergence judge sees it save
iterations). `plain_fp64` is the plain FP64 GPU path (previous-step guess, OpenCMP's) on the same
steps; `mixed_previous_step_guess` and `mixed_extrapolated_guess` separate the two gains.
Inputs are resident in HBM and larger than L2 (the matrix alone is ~730 MB), so no L2 flush.

--impl reference: the CPU restatement of the same step (the oracle: C + OpenMP, all host
threads; NGSolve cannot run here) on the same mesh, the same steps after the same warm-up, from the
previous-step guess OpenCMP uses.
--config batched: 512 steady 2D convection-diffusion instances of mixed mesh sizes and orders.
--config ins: the Navier-Stokes lid-driven cavity (Taylor-Hood, Euler IMEX, flexible GMRES with the
Cahouet-Chabard pressure preconditioner).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

EPS, WIND, DT = 1e-2, (1.0, 0.5, 0.25), 1e-3
GAUSS = dict(c=(0.25, 0.25, 0.25), s=0.1)
METRIC = 'DOF/s to 1e-8 FP64 rel. residual: mixed+batched+learned vs plain FP64, 1 GB300'
WORKLOAD = ('transient 3D convection-diffusion, unit cube {}^3 x 6 tets, H1 p=2, eps=1e-2, w=(1,0.5,0.25), implicit '
            'Euler dt=1e-3, full reassembly every step, GMRES({}) + Jacobi to 1e-8 FP64 relative residual')
# DRAM bytes per matrix entry (dram__bytes_read.sum + dram__bytes_write.sum per launch / nnz) of the
# dominant kernel from ncu captures on the 48^3 x 6 case (nnz 25,755,265): gm_spmv<float> on the CSR
# copy (two launches: 221.7 and 222.0 MB), gm_spmv_sell on the SELL-32 copy (251.7 and 251.4 MB; the
# slices' padding is the difference); the traffic of a launch is this figure times the launch's nnz
TRAFFIC_PER_NNZ = {'gm_spmv_float': 8.615, 'gm_spmv_sell': 9.768}
# DRAM bytes moved by one reassembly of the optimised path (element kernel, diagonal pass, gather;
# ncu on the 48^3 x 6 case: 645 + 95 + 1,428 MB) per algorithmic byte of that case
ASSEMBLY_TRAFFIC_RATIO = 2168.0 / 227.0


def workload_config(n, restart, ndof, nnz, world=1):
    """The bench line's `config`: the problem both arms solve (the path each takes is in `path`)."""
    return {'workload': WORKLOAD.format(n, restart), 'ndof': ndof, 'nnz': nnz,
            'parallelism': 'replicas' if world > 1 else 'single GPU', 'l2': 'inputs larger than L2 (no flush)'}


def gaussian(X):
    c = np.asarray(GAUSS['c'])
    return np.exp(-((X - c) ** 2).sum(-1) / (2 * GAUSS['s'] ** 2))


def peaks():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as fh:
            d = json.load(fh)
        return float(d['hbm_gbs']), 'measured'
    except Exception:
        return 6800.0, 'fallback'


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self):
        self.samples, self.proc = [], None
        try:
            import torch
            self.dev = 'GPU-' + str(torch.cuda.get_device_properties(torch.cuda.current_device()).uuid)
        except Exception:
            self.dev = '0'

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,'
                 'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,'
                 'clocks_event_reasons.sw_power_cap', '--format=csv,noheader,nounits', '-i', self.dev, '-lms', '200'],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.samples.append([t.strip() for t in ln.split(',')])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        sm = [float(s[0]) for s in self.samples if s and s[0].replace('.', '').isdigit()]
        mx = [float(s[1]) for s in self.samples if len(s) > 1 and s[1].replace('.', '').isdigit()]
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        reasons = sorted({names[k] for s in self.samples for k in range(4) if len(s) > 2 + k and 'Active' in s[2 + k]
                          and 'Not' not in s[2 + k]})
        return {'sm_mhz': float(np.median(sm)) if sm else None, 'sm_max_mhz': max(mx) if mx else None,
                'reasons': reasons, 'samples': len(sm)}


def max_over_ranks(x: float, device: str = 'cuda') -> float:
    """The largest of the ranks' values (the slowest replica's time); x itself on a single process."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: int, steps: int, world: int, ms: float) -> float:
    """Units per second of the whole job: every replica processes `units_per_rank` per step; the
    time is the slowest replica's (weak scaling, no collective on the data path)."""
    return units_per_rank * steps * world / (ms * 1e-3)


def run_ours(args):
    import torch
    import torch.distributed as dist
    from opencmp_gb300 import fem, mesh as M, _lib

    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group('nccl')
    from opencmp_gb300 import build
    if rank == 0 or not os.path.exists(_lib.LIB_PATH):
        build.build()
    if world > 1:
        dist.barrier()

    n = args.n
    t0 = time.perf_counter()
    mesh = M.unit_cube(n)
    space = fem.Space(mesh, 'H1', 2, mesh.bc_names)
    setup_s = time.perf_counter() - t0
    ndof, nnz = space.ndof, space.nnz
    # each path assembles the Krylov matrix it iterates with (A D^-1 in FP64, or in FP32) in the same
    # pass as the FP64 values used for the residuals
    mats = {'fp64': fem.Matrix(space, jacobi64=True),
            'mixed': fem.Matrix(space, jacobi32=True, dfloat=True, sell=not args.csr32)}
    form = fem.make_form(mass=1.0, diff=EPS, dt=DT, wind=WIND)
    u0 = torch.as_tensor(fem.interpolate_p2(space, gaussian), device='cuda')
    b = torch.zeros(ndof, dtype=torch.float64, device='cuda')
    for M_ in mats.values():
        M_.assemble(form)
    A = mats['fp64']
    tuned = A.autotune()
    solvers = {
        'fp64': fem.KrylovSolver(mats['fp64'], method='GMRES', restart=args.restart, precond='jacobi',
                                 precision='fp64', tol=1e-8, maxit=2000, check_every=args.check_every),
        'mixed': fem.KrylovSolver(mats['mixed'], method='GMRES', restart=args.restart, precond='jacobi',
                                  precision='mixed', tol=1e-8, maxit=2000, inner_tol=args.inner_tol,
                                  check_every=args.check_every_mixed),
    }

    from opencmp_gb300.guess import LearnedGuess
    # history of k solutions: degree-p extrapolation in time (the fallback) + the network's correction
    guess = LearnedGuess(space, k=args.guess_k, base_order=args.guess_base, seed=0)

    launches = {}

    def step(kind, u_in, u_out, stats):
        sv = solvers['fp64' if kind == 'fp64' else 'mixed']
        sv.mat.assemble(form)
        sv.update()
        fem.assemble_rhs(space, form, fem.make_rhs(dt=DT, mass=1.0, uprev=u_in, dfloat=kind != 'fp64'), b)
        used = 'previous'
        if kind == 'learned':
            used = guess.predict(u_out)
        elif kind == 'extrap':
            guess.extrapolate(u_out)
        else:
            u_out.copy_(u_in)
        info = sv.solve(b, u_out)
        if kind in ('learned', 'extrap'):
            guess.push(u_out)
        if kind == 'learned':
            guess.judge(info, used)
        stats.append((info.iterations, info.outer_iterations, info.relres0, info.relres, used))

    def timed(kind, steps, warmup, e2e=False):
        u = [u0.clone(), torch.empty_like(u0)]
        h_in = torch.empty(ndof, dtype=torch.float64, pin_memory=True)
        h_out = torch.empty(ndof, dtype=torch.float64, pin_memory=True)
        h_in.copy_(u0.cpu())
        guess.reset()
        guess.reset_judge()
        guess.push(u0)
        if kind == 'learned' and not guess.trained:
            raise RuntimeError('the guess network is not trained')
        stats = []
        for k in range(warmup):
            step(kind, u[k % 2], u[(k + 1) % 2], stats)
        stats.clear()
        uc = u[warmup % 2]
        h_in.copy_(uc.cpu())
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        cur = warmup % 2
        torch.cuda.nvtx.range_push('timed_' + kind + ('_e2e' if e2e else ''))
        l0 = _lib.load().ocmp_launch_count()
        for k in range(steps):
            if e2e:
                u[cur].copy_(h_in, non_blocking=True)
                step(kind, u[cur], u[1 - cur], stats)
                h_out.copy_(u[1 - cur], non_blocking=True)
                torch.cuda.current_stream().synchronize()
                h_in, h_out = h_out, h_in
            else:
                step(kind, u[cur], u[1 - cur], stats)
            cur = 1 - cur
        launches[kind + ('_e2e' if e2e else '')] = int(_lib.load().ocmp_launch_count() - l0)
        torch.cuda.nvtx.range_pop()
        ev1.record()
        torch.cuda.synchronize()
        ms = max_over_ranks(ev0.elapsed_time(ev1))
        return ms, stats

    # training of the guess network on trajectories the solver produces (not timed): eps drawn
    # log-uniform in [1e-3, 1e-1] with numpy seed 0, first steps of each run from the extrapolated
    # guess; eps = 1e-2 is held out. Each run keeps its own FP64 matrix for the residual loss.
    t_train = time.perf_counter()
    rng = np.random.default_rng(0)
    eps_train = [float(10 ** rng.uniform(-3, -1)) for _ in range(args.train_runs)]
    train_mats = []
    for eps in eps_train:
        f_tr = fem.make_form(mass=1.0, diff=eps, dt=DT, wind=WIND)
        mats['mixed'].assemble(f_tr)
        solvers['mixed'].update()
        A_tr = fem.Matrix(space)
        A_tr.assemble(f_tr)
        train_mats.append(A_tr)
        uu = u0.clone()
        guess.reset()
        guess.push(uu)
        for _ in range(args.train_steps):
            fem.assemble_rhs(space, f_tr, fem.make_rhs(dt=DT, mass=1.0, uprev=uu), b)
            xx = torch.empty_like(uu)
            guess.extrapolate(xx)
            solvers['mixed'].solve(b, xx)
            guess.collect(xx, A_tr, b)
            guess.push(xx)
            uu = xx
    loss_before = guess.eval_loss()
    losses = guess.train(steps=args.train_iters, lr=3e-3)
    loss_after = guess.eval_loss()
    guess.drop_samples()
    del train_mats
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t_train

    clocks = Clocks()
    clocks.start()
    ms_plain, st_plain = timed('fp64', args.steps, args.warmup)
    plain_relres0 = [float(np.mean([s[2] for s in st_plain]))]
    ms_mixed, st_mixed = timed('mixed', args.steps, args.warmup)
    ms_extrap, st_extrap = timed('extrap', args.steps, args.warmup)
    # the dominant kernel of the optimised path, timed live: every FP32 GMRES SpMV launch of the timed
    # steps between CUDA events on its stream
    solvers['mixed'].spmv_timing(True)
    ms_opt, st_opt = timed('learned', args.steps, args.warmup)
    spmv_live = solvers['mixed'].spmv_stats()
    solvers['mixed'].spmv_timing(False)
    cl = clocks.stop()
    ms_e2e, _ = timed('learned', args.steps, args.warmup, e2e=True)

    # assembly of the optimised path alone (matrix with its Jacobi-scaled FP32 copy, and the
    # double-float mass right-hand side), timed with CUDA events over as many repetitions as steps
    A_mix = mats['mixed']
    u_a = u0.clone()
    for _ in range(3):
        A_mix.assemble(form)
        fem.assemble_rhs(space, form, fem.make_rhs(dt=DT, mass=1.0, uprev=u_a, dfloat=True), b)
    ea0, ea1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ea0.record()
    for _ in range(args.steps):
        A_mix.assemble(form)
        fem.assemble_rhs(space, form, fem.make_rhs(dt=DT, mass=1.0, uprev=u_a, dfloat=True), b)
    ea1.record()
    torch.cuda.synchronize()
    asm_ms = ea0.elapsed_time(ea1) / args.steps
    ne, nv = mesh.ne, mesh.nv
    # algorithmic bytes of one reassembly: values written once (FP64 and the FP32 scaled copy), the
    # right-hand side, the connectivity and the coordinates read once
    asm_bytes = 12 * nnz + 8 * ndof + 4 * 4 * ne + 8 * 3 * nv

    # SpMV roofline: FP64 CSR SpMV launches timed with CUDA events on the launching stream
    x = torch.randn(ndof, dtype=torch.float64, device='cuda')
    y = torch.empty_like(x)
    for _ in range(3):
        A.mult(x, y)
    reps = 50
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        A.mult(x, y)
    e1.record()
    torch.cuda.synchronize()
    spmv_ms = e0.elapsed_time(e1) / reps
    spmv_bytes = 12 * nnz + 4 * (ndof + 1) + 16 * ndof
    peak, peak_kind = peaks()
    achieved = spmv_bytes / (spmv_ms * 1e-3) / 1e9
    # gm_spmv<float>: FP32 values + int32 columns (8 B per entry), row pointers, the input vector and
    # the new basis vector (4 B per row each), the free mask (1 B per row)
    g_bytes = 8 * nnz + 4 * (ndof + 1) + 9 * ndof
    kname = 'gm_spmv_float' if args.csr32 else 'gm_spmv_sell'
    g_launches, g_ms = spmv_live
    g_avg = g_ms / max(g_launches, 1)
    g_achieved = g_bytes / (g_avg * 1e-3) / 1e9 if g_launches else None

    value = whole_job_rate(ndof, args.steps, world, ms_opt)
    plain = whole_job_rate(ndof, args.steps, world, ms_plain)
    e2e_val = whole_job_rate(ndof, args.steps, world, ms_e2e)
    line = {
        'metric': METRIC, 'value': value, 'unit': 'DOF/s', 'n_gpus': world, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': ms_opt / args.steps, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'f64+f32', 'data': 'synthetic (generated structured mesh, Gaussian initial condition)',
        'config': workload_config(n, args.restart, ndof, nnz, world),
        'path': 'optimised: double-float assembly, learned initial guess under its judge, FP32 inner GMRES + FP64 '
                'refinement',
        'plain_fp64': {'value': plain, 'unit': 'DOF/s', 'ms_per_step': ms_plain / args.steps,
                       'relres0_per_step': plain_relres0[0],
                       'iters_per_step': float(np.mean([s[0] for s in st_plain]))},
        'optimised': {'kind': 'double-float (FP32-pair) assembly, learned initial guess (degree-{} extrapolation '
                              'in time over {} solutions + per-dof MLP correction trained on the solver\'s own '
                              'trajectories), FP32 inner GMRES + FP64 iterative refinement'.format(args.guess_base,
                                                                                                  args.guess_k),
                      'relres0_per_step': float(np.mean([s[2] for s in st_opt])),
                      'relres0_network_steps': float(np.mean([s[2] for s in st_opt if s[4] == 'network']))
                      if any(s[4] == 'network' for s in st_opt) else None,
                      'iters_per_step': float(np.mean([s[0] for s in st_opt])),
                      'iters_network_steps': float(np.mean([s[0] for s in st_opt if s[4] == 'network']))
                      if any(s[4] == 'network' for s in st_opt) else None,
                      'outer_per_step': float(np.mean([s[1] for s in st_opt])),
                      'guess_kinds': {k: sum(1 for s in st_opt if s[4] == k) for k in ('network', 'probe', 'fallback')},
                      'max_relres': float(max(s[3] for s in st_opt)), 'speedup_vs_plain_fp64': value / plain,
                      'guess_enabled_at_end': bool(guess.enabled), 'guess_fallback': guess.fallback_reason},
        'mixed_extrapolated_guess': {'value': ndof * args.steps * world / (ms_extrap * 1e-3), 'unit': 'DOF/s',
                                     'ms_per_step': ms_extrap / args.steps,
                                     'relres0_per_step': float(np.mean([s[2] for s in st_extrap[4:]])),
                                     'iters_per_step': float(np.mean([s[0] for s in st_extrap])),
                                     'iters_full_history_steps': float(np.mean([s[0] for s in st_extrap[2:]]))},
        'mixed_previous_step_guess': {'value': ndof * args.steps * world / (ms_mixed * 1e-3), 'unit': 'DOF/s',
                                      'ms_per_step': ms_mixed / args.steps,
                                      'relres0_per_step': float(np.mean([s[2] for s in st_mixed])),
                                      'iters_per_step': float(np.mean([s[0] for s in st_mixed]))},
        'guess_training': {'eps': eps_train, 'steps_per_run': args.train_steps, 'adam_steps': args.train_iters,
                           'loss': 'residual |A e|^2 / |b|^2 relative to the extrapolation (1 = no gain)',
                           'loss_before': loss_before, 'loss_after': loss_after,
                           'loss_last_iters': float(np.mean(losses[-10:])), 'seconds': train_s},
        'e2e': {'value': e2e_val, 'unit': 'DOF/s', 'h2d_bytes_per_step': 8 * ndof, 'd2h_bytes_per_step': 8 * ndof},
        'roofline': {'bound': 'hbm', 'kernel': 'gm_spmv<float> (FP32 Krylov SpMV of the optimised path, CSR)' if args.csr32
                     else 'gm_spmv_sell (FP32 Krylov SpMV of the optimised path, SELL-32, 16-byte loads)',
                     'achieved': g_achieved, 'peak': peak, 'peak_kind': peak_kind, 'unit': 'GB/s',
                     'frac': g_achieved / peak if g_achieved else None,
                     'traffic': TRAFFIC_PER_NNZ[kname] * nnz if kname in TRAFFIC_PER_NNZ else None,
                     'traffic_source': 'ncu dram bytes on the 48^3 x 6 case, scaled by nnz',
                     'algorithmic_bytes': g_bytes, 'avg_launch_ms': g_avg, 'launches_timed': g_launches,
                     'timing': 'CUDA events around every launch in the timed steps, on the launching stream'},
        'roofline_fp64_spmv': {'bound': 'hbm', 'kernel': 'spmv64 (CSR FP64, ocmp_spmv) timed alone, 50 launches',
                               'achieved': achieved, 'peak': peak, 'unit': 'GB/s', 'frac': achieved / peak,
                               'algorithmic_bytes': spmv_bytes, 'avg_launch_ms': spmv_ms},
        'autotune': tuned,
        'assembly': {'kind': 'double-float element matrices + sorted segmented gather (FP64 values, FP32 Jacobi-scaled '
                             'SELL-32 copy, diagonal) + double-float mass right-hand side',
                     'ms_per_step': asm_ms, 'algorithmic_bytes': asm_bytes,
                     'achieved_gbs': asm_bytes / (asm_ms * 1e-3) / 1e9,
                     'frac': asm_bytes / (asm_ms * 1e-3) / 1e9 / peak,
                     'dram_per_algorithmic_byte': ASSEMBLY_TRAFFIC_RATIO},
        'gpu_launches': launches['learned'],
        'gpu_launches_by_path': launches,
        'clocks': cl,
        'setup_s': setup_s,
    }
    if rank == 0 and world == 1 and not args.no_cpu:
        line['cpu_baseline'] = cpu_baseline(args.cpu_n if args.cpu_n > 0 else n)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def run_ins(args):
    """Lid-driven cavity (OpenCMP INS model): unit square 256 x 256 x 2, Taylor-Hood P2/P1, nu = 1e-3
    (Re = 1000 with lid speed 1; the lid's corners at rest, so that the discrete lid does not leak),
    Euler IMEX steps dt = 1e-3 from rest (explicit convection, reassembly every step), the library's
    GMRES(50) with the Cahouet-Chabard block-diagonal preconditioner (velocity Jacobi; pressure: the
    strip direct solve of L_p + max(delta, 1) M_p plus the pressure-mass diagonal) to 1e-8. Every
    path runs the same first `ins_train` steps untimed (the learned path collects its training
    samples there: the run's own first steps), then times `steps` steps: plain FP64 GMRES
    (previous-step guess), FP32 inner GMRES + FP64 refinement with the previous-step guess, with the
    extrapolated guess, and with the learned guess under its judge."""
    import torch
    from opencmp_gb300 import fem, mesh as M, build, _lib
    from opencmp_gb300.guess import LearnedGuess
    from opencmp_gb300.saddle import SaddleSolver
    build.build()
    torch.cuda.set_device(0)
    n = args.n_ins
    m = M.unit_square(n)
    th = fem.TaylorHood(m, 2, m.bc_names)
    lab = {k: m.bc_names.index(k) for k in m.bc_names}
    nd = th.ndof
    dt, nu = 1e-3, 1e-3
    A = th.matrix()
    b = torch.zeros(nd, dtype=torch.float64, device='cuda')
    solvers = {p: SaddleSolver(th, A, restart=50, tol=1e-8, maxit=args.ins_maxit, inner_tol=0.1, precision=p)
               for p in ('fp64', 'mixed')}
    guess = LearnedGuess(th.C, k=args.guess_k, base_order=args.guess_base, seed=0)

    def bcs(u):
        # the lid first, the walls last: both top corners at rest
        for c, val in ((0, 1.0), (1, 0.0)):
            th.V.set_boundary({lab['top']: val}, th.component(u, c))
            th.V.set_boundary({lab['bottom']: 0.0, lab['left']: 0.0, lab['right']: 0.0}, th.component(u, c))

    def step(kind, u, stats, collect=False):
        sv = solvers['fp64' if kind == 'fp64' else 'mixed']
        uprev = u.clone()
        th.assemble(A, mass=1.0, nu=nu, dt=dt)
        th.assemble_rhs(b, dt=dt, mass=1.0, uprev=uprev, imex=uprev)
        sv.update(mass=1.0, dt=dt, nu=nu)
        used = 'previous'
        if kind == 'learned':
            used = guess.predict(u)
        elif kind == 'extrap':
            guess.extrapolate(u)
        if kind in ('learned', 'extrap'):
            # the undetermined constant pressure stays where the previous step left it
            sv.match_pressure_mean(u, uprev)
        bcs(u)
        info = sv.solve(b, u, raise_on_fail=False)
        if collect:
            guess.collect(u, A, b)
        if kind in ('learned', 'extrap'):
            guess.push(u)
            if kind == 'learned':
                guess.judge(info, used)
        stats.append((info.iterations, info.relres, info.status, info.relres0, used, info.inner_iterations))

    res = {}
    train_info = {}
    spmv_live, e2e_ms = (0, 0.0), float('nan')
    for p in ('fp64', 'mixed', 'extrap', 'learned'):
        u = torch.zeros(nd, dtype=torch.float64, device='cuda')
        bcs(u)
        st = []
        guess.reset()
        guess.reset_judge()
        guess.push(u)
        t_tr = time.perf_counter()
        for _ in range(args.ins_train):
            # the same untimed start for every path; the learned path collects its training samples
            # here (the run's own first steps, solved from the extrapolated guess; the IMEX matrix is
            # the same every step, so the live matrix serves the residual loss)
            step('extrap' if p in ('extrap', 'learned') else p, u, st, collect=p == 'learned')
        if p == 'learned' and guess.samples:
            l_before = guess.eval_loss()
            guess.train(steps=args.train_iters, lr=3e-3)
            train_info = dict(samples=len(guess.samples), adam_steps=args.train_iters, loss_before=l_before,
                              loss_after=guess.eval_loss(), seconds=time.perf_counter() - t_tr)
            guess.drop_samples()
            guess.reset_judge()
        elif p == 'learned':
            # samples start once the history holds guess_k steps: with fewer untimed steps the
            # network keeps its zero output and the learned path is the extrapolation
            train_info = dict(samples=0, adam_steps=0)
            guess.reset_judge()
        st.clear()
        lib_sv = solvers['fp64' if p == 'fp64' else 'mixed'].lib
        if p == 'learned' and lib_sv is not None:
            lib_sv.spmv_timing(True)
        torch.cuda.synchronize()
        l0 = _lib.load().ocmp_launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            step(p, u, st)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        if p == 'learned' and lib_sv is not None:
            spmv_live = lib_sv.spmv_stats()
            lib_sv.spmv_timing(False)
            # end to end: the solution back to pinned host memory after every step (the step's
            # inputs are the device-resident state; the boundary data is constant)
            u_host = torch.empty(nd, dtype=torch.float64, pin_memory=True)
            ue = u.clone()
            ste = []
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(args.steps):
                step(p, ue, ste)
                u_host.copy_(ue, non_blocking=True)
                torch.cuda.current_stream().synchronize()
            e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
        l2, dv = th.errors(u)
        res[p] = dict(ms_per_step=ms / args.steps, value=nd * args.steps / (ms * 1e-3), unit='DOF/s',
                      launches=int(_lib.load().ocmp_launch_count() - l0),
                      iters=float(np.mean([s[0] for s in st])), max_relres=float(max(s[1] for s in st)),
                      inner_cg_iters=float(np.mean([s[5] for s in st])),
                      relres0=float(np.mean([s[3] for s in st])),
                      converged=int(sum(1 for s in st if s[2] == 0)), u_l2=l2, div_l2=dv)
        if p == 'learned':
            res[p].update(guess_kinds={k: sum(1 for s in st if s[4] == k) for k in ('network', 'probe', 'fallback')},
                          guess_enabled_at_end=bool(guess.enabled), guess_fallback=guess.fallback_reason)
        print('ins {}: {:.2f} ms/step, {:.1f} iterations/step'.format(p, res[p]['ms_per_step'], res[p]['iters']),
              file=sys.stderr, flush=True)
    val = res['learned']['value']
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as fh:
            peak, peak_kind = float(json.load(fh)['hbm_gbs']), 'measured HBM copy'
    except Exception:
        peak, peak_kind = 6800.0, 'fallback HBM'
    nnz_ins = th.nnz
    g_bytes = 8 * nnz_ins + 4 * (nd + 1) + 9 * nd
    g_launches, g_ms = spmv_live
    g_avg = g_ms / max(g_launches, 1)
    g_achieved = g_bytes / (g_avg * 1e-3) / 1e9 if g_launches else None
    line = {'metric': METRIC + ' (INS lid-driven cavity)', 'value': val, 'unit': 'DOF/s', 'n_gpus': 1,
            'steps': args.steps, 'warmup': args.ins_train, 'ms_per_step': res['learned']['ms_per_step'],
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64+f32',
            'data': 'synthetic (generated structured mesh, cavity at rest)',
            'config': {'workload': 'INS lid-driven cavity {0}x{0}x2 tri, Taylor-Hood P2/P1, Re=1000, Euler IMEX '
                                   'dt=1e-3, lid corners at rest, GMRES(50) + Cahouet-Chabard (velocity '
                                   'Jacobi, pressure: strip direct solve of the pressure Laplacian + mass '
                                   'diagonal) to 1e-8; steps {1}..{2} from rest timed'.format(
                                       n, args.ins_train + 1, args.ins_train + args.steps),
                       'ndof': nd, 'nnz': th.nnz, 'l2': 'inputs larger than L2 (no flush)'},
            'plain_fp64': res['fp64'], 'mixed_previous_step_guess': res['mixed'],
            'mixed_extrapolated_guess': res['extrap'],
            'optimised': dict(res['learned'], kind='FP32 inner GMRES + FP64 refinement, learned guess (degree-{} '
                                                   'extrapolation + network trained on the run\'s first {} steps)'
                              .format(args.guess_base, args.ins_train)),
            'speedup_vs_plain_fp64': res['fp64']['ms_per_step'] / res['learned']['ms_per_step'],
            'e2e': {'value': nd / (e2e_ms * 1e-3), 'unit': 'DOF/s', 'h2d_bytes_per_step': 0,
                    'd2h_bytes_per_step': 8 * nd},
            'roofline': {'bound': 'hbm', 'kernel': 'gm_spmv<float> (FP32 Krylov SpMV of the saddle-point system, CSR)',
                         'achieved': g_achieved, 'peak': peak, 'peak_kind': peak_kind, 'unit': 'GB/s',
                         'frac': g_achieved / peak if g_achieved else None, 'traffic': None,
                         'algorithmic_bytes': g_bytes, 'avg_launch_ms': g_avg, 'launches_timed': g_launches,
                         'timing': 'CUDA events around every launch in the timed steps of the optimised path'},
            'guess_training': train_info, 'gpu_launches': res['learned']['launches']}
    print(json.dumps(line), flush=True)


def run_batched(args):
    """Config 4: 512 independent steady 2D convection-diffusion problems of 12 (mesh, order) classes
    (n in {16, 32, 64, 128}, H1 p in {1, 2, 3}). One step = assemble every instance (one batched
    assembly per class) and solve all of them with one solver group: every GMRES kernel launched once
    over all 512 uneven instances (ocmp_group_solve), FP32 inner GMRES + FP64 refinement, one restart
    cycle replayed from a CUDA graph. Recorded beside it: the same classes as 12 batched solves on 12
    host threads and streams, and the plain FP64 loop over instances."""
    import concurrent.futures as cf
    import torch
    from opencmp_gb300 import fem, mesh as M, build, _lib
    build.build()
    torch.cuda.set_device(0)
    rng = np.random.default_rng(0)
    N = args.instances
    ns = rng.choice([16, 32, 64, 128], N)
    ps = rng.choice([1, 2, 3], N)
    eps = 10 ** rng.uniform(-3, 0, N)
    ang = rng.uniform(0, 2 * np.pi, N)
    classes = {}
    for q in range(N):
        classes.setdefault((int(ns[q]), int(ps[q])), []).append(q)
    tol = 1e-8
    C = []
    for (n, p), idx in sorted(classes.items()):
        m = M.unit_square(n)
        sp = fem.Space(m, 'H1', p, m.bc_names)
        forms = [fem.make_form(diff=float(eps[q]), dt=1.0, wind=(float(np.cos(ang[q])), float(np.sin(ang[q]))))
                 for q in idx]
        A = fem.Matrix(sp, batch=len(idx), jacobi32=True)
        A1t = fem.Matrix(sp)
        A1t.assemble(forms[0])
        A1t.autotune()
        b1 = torch.zeros(sp.ndof, dtype=torch.float64, device='cuda')
        fem.assemble_rhs(sp, forms[0], fem.make_rhs(src_const=1.0), b1)
        sv = fem.KrylovSolver(A, method='GMRES', restart=args.restart_batch, precision='mixed', tol=tol,
                              maxit=20000, inner_tol=1e-4)
        C.append(dict(n=n, p=p, idx=idx, space=sp, forms=forms, A=A, b=b1.repeat(len(idx)),
                      x=torch.zeros(len(idx) * sp.ndof, dtype=torch.float64, device='cuda'), sv=sv))
    total_dofs = sum(c['space'].ndof * len(c['idx']) for c in C)
    group = fem.KrylovGroup([c['sv'] for c in C])
    bs = [c['b'] for c in C]
    xs = [c['x'] for c in C]

    def group_step():
        for c in C:
            c['A'].assemble_batch(c['forms'])
            c['sv'].update()
            c['x'].zero_()
        return group.solve(bs, xs, raise_on_fail=False)

    for _ in range(args.warmup):
        group_step()
    torch.cuda.synchronize()
    if args.group_only:
        # a profiling run: the group solve only
        for _ in range(args.steps):
            group_step()
        torch.cuda.synchronize()
        return
    l0 = _lib.load().ocmp_launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        infos = group_step()
    e1.record()
    torch.cuda.synchronize()
    t_b = e0.elapsed_time(e1) * 1e-3 / args.steps
    launches = int(_lib.load().ocmp_launch_count() - l0)
    # end to end: right-hand sides from pinned host memory, solutions back to it, every step
    b_host = [b.cpu().pin_memory() for b in bs]
    x_host = [torch.empty(x.numel(), dtype=torch.float64, pin_memory=True) for x in xs]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for b, bh in zip(bs, b_host):
            b.copy_(bh, non_blocking=True)
        group_step()
        for x, xh in zip(xs, x_host):
            xh.copy_(x, non_blocking=True)
        torch.cuda.synchronize()
    t_e2e = (time.perf_counter() - t0) / args.steps
    # algorithmic HBM bytes of the Krylov iterations each instance ran (FP32 SpMV: 4-byte value and
    # column per entry, x read, y written; classical Gram-Schmidt step j of a GMRES(m) cycle: about
    # 2 j + 4 vector passes, j averaging m / 2) and of its FP64 residuals (one per cycle: 12 bytes
    # per entry and 24 per row)
    mm = args.restart_batch
    alg = 0.0
    k = 0
    for c in C:
        nd, nz = c['space'].ndof, c['space'].nnz
        for _ in c['idx']:
            it = infos[k].iterations
            cyc = max(1, -(-it // mm))
            alg += it * (8.0 * nz + 8.0 * nd + 4.0 * (mm + 4) * nd) + cyc * (12.0 * nz + 24.0 * nd)
            k += 1
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as fh:
            peak, peak_kind = float(json.load(fh)['hbm_gbs']), 'measured'
    except Exception:
        peak, peak_kind = 6800.0, 'fallback'
    achieved = alg / t_b / 1e9

    # the same classes as 12 batched solves on 12 host threads (one stream each), for the record
    for c in C:
        c['stream'] = torch.cuda.Stream()

    def run_class(c):
        with torch.cuda.stream(c['stream']):
            c['A'].assemble_batch(c['forms'], stream=c['stream'])
            c['sv'].update(stream=c['stream'])
            c['x'].zero_()
            return c['sv'].solve_batch(c['b'], c['x'], stream=c['stream'], raise_on_fail=False)

    pool = cf.ThreadPoolExecutor(max_workers=len(C))

    def class_step():
        res = list(pool.map(run_class, C))
        torch.cuda.synchronize()
        return res

    class_step()
    t0 = time.perf_counter()
    for _ in range(max(1, min(args.steps, 3))):
        cres = class_step()
    t_c = (time.perf_counter() - t0) / max(1, min(args.steps, 3))
    cinf = [i for r in cres for i in r]

    # plain FP64 loop over instances: one matrix, one GMRES solve at a time
    plain = []
    for c in C:
        A1 = fem.Matrix(c['space'], jacobi64=True)
        sv1 = fem.KrylovSolver(A1, method='GMRES', restart=args.restart_batch, precision='fp64', tol=tol,
                               maxit=20000)
        plain.append((c, A1, sv1, torch.zeros(c['space'].ndof, dtype=torch.float64, device='cuda')))

    def plain_step():
        out = []
        for c, A1, sv1, x1 in plain:
            b1 = c['b'][:c['space'].ndof]
            for f in c['forms']:
                A1.assemble(f)
                sv1.update()
                x1.zero_()
                out.append(sv1.solve(b1, x1, raise_on_fail=False))
        torch.cuda.synchronize()
        return out

    plain_step()
    t0 = time.perf_counter()
    psteps = max(1, min(args.steps, 3))
    for _ in range(psteps):
        pinf = plain_step()
    t_p = (time.perf_counter() - t0) / psteps
    line = {'metric': METRIC + ' (batched instances)', 'value': total_dofs / t_b, 'unit': 'DOF/s', 'n_gpus': 1,
            'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': t_b * 1e3, 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64+f32', 'data': 'synthetic',
            'config': {'workload': '{} steady 2D convection-diffusion instances, n in {{16,32,64,128}}, H1 p in {{1,2,3}}, '
                                   'eps log-uniform [1e-3,1], |w|=1, f=1, Dirichlet 0, seed 0; GMRES({}) + Jacobi to '
                                   '1e-8; assembly + solve per step'.format(N, args.restart_batch),
                       'classes': len(C), 'total_dofs': total_dofs,
                       'l2': 'instances and bases exceed L2 together (no flush)'},
            'optimised': {'kind': 'one solver group over all instances: every GMRES kernel launched once for all {} '
                                  'uneven instances, FP32 inner GMRES + FP64 refinement, restart cycle from a CUDA '
                                  'graph'.format(N),
                          'max_relres': float(max(i.relres for i in infos)),
                          'converged': int(sum(1 for i in infos if i.status == 0)),
                          'iters_mean': float(np.mean([i.iterations for i in infos])),
                          'iters_max': int(max(i.iterations for i in infos))},
            'per_class_threads': {'value': total_dofs / t_c, 'unit': 'DOF/s', 'ms_per_step': t_c * 1e3,
                                  'kind': '12 batched solves (one per class) on 12 host threads and streams',
                                  'converged': int(sum(1 for i in cinf if i.status == 0))},
            'plain_fp64': {'value': total_dofs / t_p, 'unit': 'DOF/s', 'ms_per_step': t_p * 1e3,
                           'kind': 'loop over instances, FP64 GMRES',
                           'converged': int(sum(1 for i in pinf if i.status == 0)),
                           'iters_mean': float(np.mean([i.iterations for i in pinf]))},
            'speedup_vs_plain_fp64': t_p / t_b,
            'e2e': {'value': total_dofs / t_e2e, 'unit': 'DOF/s',
                    'h2d_bytes_per_step': int(sum(8 * b.numel() for b in bs)),
                    'd2h_bytes_per_step': int(sum(8 * x.numel() for x in xs))},
            'roofline': {'bound': 'hbm', 'kernel': 'whole group solve (gx_spmv, gx_dots, gx_orth, gx_combine, gx_resid)',
                         'achieved': achieved, 'peak': peak, 'unit': 'GB/s', 'frac': achieved / peak,
                         'peak_kind': peak_kind + ' HBM copy',
                         'bytes': 'algorithmic bytes of the iterations each instance ran, over the step time '
                                  '(assembly included in the time)',
                         'traffic': None},
            'gpu_launches': launches}
    print(json.dumps(line), flush=True)


def run_dg2d(args):
    """Config 2: steady 2D convection-diffusion, unit square 256 x 256 x 2 triangles, DG order 2
    (786,432 dofs), eps = 1e-3, rotating wind w = (-(y-0.5), x-0.5), Gaussian source (sigma 0.05 at
    (0.3, 0.5)), DG Dirichlet 0, interior penalty 10. One step = assemble the matrix and the
    right-hand side, factorise the strip direct preconditioner, GMRES to a 1e-8 FP64 relative
    residual from zero (OpenCMP's direct solve of this system, base_model.py:906-922, refactorises
    on every call too). `value`: FP64 GMRES, strip inverses built with the tensor-core products;
    `plain_fp64`: the same with FP32 SIMT products; `mixed`: FP32 inner GMRES + FP64 refinement with
    the tensor-core preconditioner. The configuration's own GMRES(50) + block Jacobi is run once for
    the record: it stagnates on this closed-streamline problem."""
    import torch
    from opencmp_gb300 import fem, mesh as M, build, _lib
    build.build()
    torch.cuda.set_device(0)
    n = args.n_dg
    m = M.unit_square(n)
    sp = fem.Space(m, 'L2', 2)
    X = m.coords
    W = torch.as_tensor(np.ascontiguousarray(np.stack([-(X[:, 1] - 0.5), X[:, 0] - 0.5], 1)), device='cuda')
    allb = m.label_mask(m.bc_names)
    form = fem.make_form(diff=1e-3, dt=1.0, wind_vtx=W, dg=True, ipc=10.0, nitsche_mask=allb)
    Xq = sp.quad_points()
    fq = torch.as_tensor(np.exp(-((Xq[..., 0] - 0.3) ** 2 + (Xq[..., 1] - 0.5) ** 2) / (2 * 0.05 ** 2)), device='cuda')
    rhs = fem.make_rhs(src_qp=fq, gval={k: 0.0 for k in range(len(m.bc_names))})
    nd, nnz = sp.ndof, sp.nnz
    A = fem.Matrix(sp)
    b = torch.zeros(nd, dtype=torch.float64, device='cuda')
    A.assemble(form)
    fem.assemble_rhs(sp, form, rhs, b)
    paths = {'tensor_fp64': ('fp64', 'tensor'), 'simt_fp64': ('fp64', 'simt'), 'tensor_mixed': ('mixed', 'tensor')}
    if args.dg_paths != 'all':
        # a profiling run: only the listed paths, no comparison record
        keep = args.dg_paths.split(',')
        paths = {k: v for k, v in paths.items() if k in keep}
    solvers = {}
    for k, (prec, kind) in paths.items():
        sv = fem.KrylovSolver(A, method='GMRES', restart=50, precond='strip', precision=prec, tol=1e-8, maxit=200)
        sv.strip_gemm(kind)
        solvers[k] = sv
    peak = None
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as fh:
            pk = json.load(fh)
        peak, peak_kind = float(pk['bf16_tflops']), 'measured'
    except Exception:
        peak, peak_kind = 1900.0, 'fallback'
    hbm_peak, hbm_kind = peaks()

    def step(sv, x, e2e=None):
        if e2e is not None:
            b_host, x_host = e2e
        A.assemble(form)
        fem.assemble_rhs(sp, form, rhs, b)
        sv.update()
        x.zero_()
        info = sv.solve(b, x, raise_on_fail=False)
        if e2e is not None:
            x_host.copy_(x, non_blocking=True)
        return info

    res = {}
    x = torch.zeros_like(b)
    for k, sv in solvers.items():
        for _ in range(args.warmup):
            step(sv, x)
        torch.cuda.synchronize()
        l0 = _lib.load().ocmp_launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        infos = []
        e0.record()
        for _ in range(args.steps):
            infos.append(step(sv, x))
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        res[k] = dict(value=nd / (ms * 1e-3), unit='DOF/s', ms_per_step=ms, launches=int(_lib.load().ocmp_launch_count() - l0),
                      iters=float(np.mean([i.iterations for i in infos])),
                      max_relres=float(max(i.relres for i in infos)),
                      converged=int(sum(1 for i in infos if i.status == 0)))
        print('dg2d {}: {:.1f} ms/step, {:.1f} iterations'.format(k, ms, res[k]['iters']), file=sys.stderr, flush=True)
    if args.dg_paths != 'all':
        return
    # the optimised path end to end: the right-hand side's source data from pinned host memory, the
    # solution back to it, every step
    sv = solvers['tensor_fp64']
    fq_host = fq.cpu().pin_memory()
    x_host = torch.empty(nd, dtype=torch.float64, pin_memory=True)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        fq.copy_(fq_host, non_blocking=True)
        step(sv, x, e2e=(None, x_host))
        torch.cuda.current_stream().synchronize()
    e1.record()
    torch.cuda.synchronize()
    ms_e2e = e0.elapsed_time(e1) / args.steps
    # dense products of one factorisation, timed per launch with CUDA events (the tile inversions,
    # panels and sweeps are the rest of the factorisation time)
    gem = {}
    for k, sv in solvers.items():
        sv.strip_timing(True)
        sv.update()
        st = sv.strip_stats()
        sv.strip_timing(False)
        gem[k] = dict(st, tflops=st['gemm_flops'] / (st['gemm_ms'] * 1e-3) / 1e12 if st['gemm_ms'] else None,
                      gbs=st['gemm_bytes'] / (st['gemm_ms'] * 1e-3) / 1e9 if st['gemm_ms'] else None)
    # the configuration's own preconditioner, once, for the record
    bj = fem.KrylovSolver(A, method='GMRES', restart=50, precond='block_jacobi', precision='fp64', tol=1e-8,
                          maxit=args.bj_iters)
    xb = torch.zeros_like(b)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ib = bj.solve(b, xb, raise_on_fail=False)
    torch.cuda.synchronize()
    t_bj = time.perf_counter() - t0
    tc = gem['tensor_fp64']
    # FLOP/s of the tensor-core products against the measured dense BF16 rate (TF32 runs at half of
    # it on this part, and the 3xTF32 split issues three products per FP32 product counted here)
    line = {'metric': METRIC + ' (steady DG convection-diffusion)', 'value': res['tensor_fp64']['value'],
            'unit': 'DOF/s', 'n_gpus': 1, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': res['tensor_fp64']['ms_per_step'], 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f64+f32+tf32', 'data': 'synthetic (generated structured mesh)',
            'config': {'workload': 'steady 2D convection-diffusion, unit square {0}x{0}x2 tri, DG p=2, eps=1e-3, '
                                   'rotating wind, Gaussian source, DG Dirichlet 0; assembly + strip direct '
                                   'preconditioner factorisation + GMRES(50) to 1e-8 FP64 relative residual '
                                   'per step'.format(n),
                       'ndof': nd, 'nnz': nnz, 'l2': 'strip inverses ({:.1f} GB) larger than L2 (no flush)'.format(
                           tc['bytes'] / 1e9)},
            'optimised': dict(res['tensor_fp64'], kind='FP64 GMRES, strip inverses in FP32 built with tcgen05 3xTF32 '
                                                       'products'),
            'mixed': dict(res['tensor_mixed'], kind='FP32 inner GMRES + FP64 refinement, same preconditioner (the '
                                                    'preconditioner dominates, so the FP32 inner iteration does not '
                                                    'pay here)'),
            'plain_fp64': dict(res['simt_fp64'], kind='FP64 GMRES, strip inverses in FP32 built with FP32 SIMT '
                                                      'products'),
            'block_jacobi_fp64': {'kind': 'FP64 GMRES(50) + block Jacobi (the configuration\'s own preconditioner)',
                                  'iterations': ib.iterations, 'relres_reached': ib.relres, 'status': ib.status,
                                  'seconds': t_bj},
            'factorisation': gem,
            'e2e': {'value': nd / (ms_e2e * 1e-3), 'unit': 'DOF/s', 'h2d_bytes_per_step': 8 * fq.numel(),
                    'd2h_bytes_per_step': 8 * nd},
            # the 3xTF32 split issues three TF32 products per FP32-equivalent product and TF32 runs at
            # 1.1 / 2.25 of the BF16 rate (nominal dense figures), so the products' own peak is the
            # measured BF16 rate x (1.1 / 2.25) / 3; their intensity (FP32-equivalent flops per
            # algorithmic byte) is above that peak's ridge against HBM, so they are tensor-bound
            'roofline': {'bound': 'tensor', 'kernel': 'tc_gemm_nt_kernel (tcgen05 kind::tf32, 3xTF32, TMA-staged)',
                         'achieved': tc['tflops'], 'peak': peak * (1.1 / 2.25) / 3.0,
                         'peak_kind': peak_kind + ' bf16 dense (burst) x nominal TF32/BF16 rate (1.1/2.25) / 3 '
                                                  '(three TF32 products per FP32-equivalent product)',
                         'unit': 'TFLOP/s', 'frac': tc['tflops'] / (peak * (1.1 / 2.25) / 3.0) if tc['tflops'] else None,
                         'flops': 'FP32-equivalent 2 M N K per product',
                         'intensity_flop_per_byte': tc['gemm_flops'] / tc['gemm_bytes'] if tc['gemm_bytes'] else None,
                         'ridge_flop_per_byte': peak * (1.1 / 2.25) / 3.0 * 1e12 / (hbm_peak * 1e9),
                         'achieved_gbs': tc['gbs'], 'traffic': None},
            'roofline_bf16': {'achieved': tc['tflops'], 'peak': peak, 'peak_kind': peak_kind + ' bf16 dense (burst)',
                              'unit': 'TFLOP/s', 'frac': tc['tflops'] / peak if tc['tflops'] else None},
            'gpu_launches': res['tensor_fp64']['launches']}
    if not args.no_cpu:
        line['cpu_baseline'] = dg2d_cpu_baseline(args.dg_cpu_n)
    print(json.dumps(line), flush=True)


def dg2d_cpu_baseline(n_cpu):
    """The reference's default for this call, a sparse direct solve (scipy spsolve, SuperLU), after
    the oracle's assembly, on the n_cpu x n_cpu x 2 mesh."""
    import scipy.sparse.linalg as spla
    from oracle import oracle as O
    from opencmp_gb300 import mesh as M
    O.build()
    O.lib().or_set_threads(os.cpu_count() or 1)
    m = M.unit_square(n_cpu)
    X = m.coords
    W = np.ascontiguousarray(np.stack([-(X[:, 1] - 0.5), X[:, 0] - 0.5], 1))
    o = O.Space(m, O.L2, 2, 0)
    allb = m.label_mask(m.bc_names)
    of = O.make_form(diff=1e-3, dt=1.0, wind_vtx=W, dg=True, ipc=10.0, nitsche_mask=allb)
    t0 = time.perf_counter()
    A = o.assemble(of)
    bo = o.rhs(of, O.make_rhs(src_kind=O.SRC_GAUSS, src=(1.0, 0.3, 0.5, 0.0, 0.05)))
    x = spla.spsolve(o.csr(A).tocsc(), bo)
    dt = time.perf_counter() - t0
    return {'value': o.ndof / dt, 'unit': 'DOF/s', 'cores': 1, 'kind': 'port',
            'sample': 'oracle assembly (OpenMP) + scipy spsolve (SuperLU, one thread) on the {0}x{0}x2 mesh ({1} '
                      'dofs), relres {2:.1e}'.format(n_cpu, o.ndof, o.relres(A, bo, x))}


def cpu_steps(n_cpu, warmup, steps, restart=30):
    """The oracle's implicit-Euler step (full reassembly + GMRES(restart)/Jacobi to 1e-8 from the
    previous-step guess, OpenCMP's start) on the n_cpu^3 x 6 mesh, all host threads: `warmup`
    untimed steps from the Gaussian start, then `steps` timed ones."""
    from oracle import oracle as O
    from opencmp_gb300 import mesh as M
    O.build()
    threads = os.cpu_count() or 1
    O.lib().or_set_threads(threads)
    m = M.unit_cube(n_cpu)
    s = O.Space(m, O.H1, 2, m.label_mask(m.bc_names))
    f = O.make_form(mass=1.0, diff=EPS, dt=DT, wind=WIND)
    u = _interp_p2_oracle(s, m)
    iters = []

    def one(u):
        A = s.assemble(f)
        b = s.rhs(f, O.make_rhs(dt=DT, mass=1.0, uprev=u))
        x = u.copy()
        it, _ = s.gmres(A, b, x, restart=restart, precond=1, tol=1e-8, maxit=2000)
        iters.append(it)
        return x

    for _ in range(warmup):
        u = one(u)
    iters.clear()
    t0 = time.perf_counter()
    for _ in range(steps):
        u = one(u)
    dt = time.perf_counter() - t0
    return s.ndof, dt, threads, float(np.mean(iters)) if iters else 0.0, s.nnz


def _interp_p2_oracle(s, m):
    from opencmp_gb300.fem import interpolate_p2_arrays
    return interpolate_p2_arrays(m.coords, s.sorted_conn(), s.dofs(), s.ndof, gaussian)


def cpu_baseline(n_cpu, warmup=1, steps=2):
    ndof, dt, threads, its, _ = cpu_steps(n_cpu, warmup, steps)
    return {'value': ndof * steps / dt, 'unit': 'DOF/s', 'cores': threads, 'kind': 'port',
            'sample': 'implicit-Euler steps {}..{} from the Gaussian start (full reassembly + GMRES(30)/Jacobi to '
                      '1e-8 from the previous-step guess, {:.1f} iterations per step) on the {}^3 x 6 tet mesh ({} '
                      'dofs), C oracle with OpenMP'.format(warmup + 1, warmup + steps, its, n_cpu, ndof)}


def run_reference(args):
    """The reference arm: OpenCMP's own algorithm for this step (NGSolve cannot be installed here, so
    its CPU restatement, the oracle) on the same mesh, the same steps after the same warm-up, from
    the previous-step guess OpenCMP uses, on all host cores."""
    rank = int(os.environ.get('RANK', '0'))
    if rank != 0:
        return
    steps = max(1, args.steps)
    ndof, dt, threads, its, nnz = cpu_steps(args.n, args.warmup, steps, args.restart)
    v = ndof * steps / dt
    line = {'metric': METRIC, 'value': v, 'unit': 'DOF/s', 'n_gpus': 0, 'steps': steps, 'warmup': args.warmup,
            'ms_per_step': dt / steps * 1e3, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
            'dtype': 'f64', 'data': 'synthetic (generated structured mesh, Gaussian initial condition)',
            'impl': 'reference',
            'config': workload_config(args.n, args.restart, ndof, nnz),
            'path': "OpenCMP's algorithm for the step (FP64 assembly, GMRES({}) + Jacobi from the previous-step "
                    "guess) restated by the oracle in C with OpenMP".format(args.restart),
            'cpu_baseline': {'value': v, 'unit': 'DOF/s', 'cores': threads, 'kind': 'port',
                             'sample': 'steps {}..{} from the Gaussian start on {} dofs, {:.1f} GMRES iterations per '
                                       'step, C oracle with OpenMP'.format(args.warmup + 1, args.warmup + steps,
                                                                          ndof, its)},
            'e2e': {'value': v, 'unit': 'DOF/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=20)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--n', type=int, default=64)
    ap.add_argument('--cpu-n', type=int, default=0, help='mesh of the cpu_baseline sample (0: the workload\'s)')
    ap.add_argument('--restart', type=int, default=30)
    ap.add_argument('--inner-tol', type=float, default=1e-4)
    # GMRES iterations between the host's convergence checks, per path at its measured best: the plain
    # FP64 path takes ~17 iterations per step, the mixed paths ~6 from the extrapolated guess
    ap.add_argument('--check-every', type=int, default=8, help='plain FP64 path')
    ap.add_argument('--check-every-mixed', type=int, default=6, help='mixed-precision paths')
    ap.add_argument('--no-cpu', action='store_true')
    ap.add_argument('--csr32', action='store_true', help='FP32 Krylov matrix in CSR order instead of SELL-32')
    ap.add_argument('--config', default='transient3d', choices=['transient3d', 'batched', 'ins', 'dg2d'])
    ap.add_argument('--n-dg', type=int, default=256)
    ap.add_argument('--dg-cpu-n', type=int, default=128, help='mesh of the dg2d cpu_baseline sample')
    ap.add_argument('--bj-iters', type=int, default=2000, help='block-Jacobi GMRES budget of the dg2d record')
    ap.add_argument('--dg-paths', default='all',
                    help='dg2d: comma-separated subset of tensor_fp64,simt_fp64,tensor_mixed to run alone (profiling)')
    ap.add_argument('--group-only', action='store_true', help='batched: run the group solve only (profiling)')
    ap.add_argument('--n-ins', type=int, default=256)
    ap.add_argument('--ins-train', type=int, default=100,
                    help='untimed first INS steps (training samples from step guess_k + 1 on)')
    ap.add_argument('--ins-maxit', type=int, default=1000, help='FGMRES iteration cap per INS step')
    ap.add_argument('--instances', type=int, default=512)
    ap.add_argument('--restart-batch', type=int, default=50)
    ap.add_argument('--train-runs', type=int, default=4)
    ap.add_argument('--train-steps', type=int, default=50)
    ap.add_argument('--train-iters', type=int, default=300)
    ap.add_argument('--guess-k', type=int, default=5, help='history length of the learned guess (2..6)')
    ap.add_argument('--guess-base', type=int, default=3, help='degree of the extrapolation it corrects')
    args = ap.parse_args()
    if args.impl == 'reference':
        run_reference(args)
    elif args.config == 'ins':
        run_ins(args)
    elif args.config == 'batched':
        run_batched(args)
    elif args.config == 'dg2d':
        run_dg2d(args)
    else:
        run_ours(args)


if __name__ == '__main__':
    main()
