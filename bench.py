"""Benchmark of the EMPEROR sampling hot path on GB300.

Workload (default): the 3-Keplerian, 2-instrument, N=1024, per-instrument
MA(1) system of the benchmark suite, parallel tempering with 10
temperatures x 256 walkers, stretch moves + swaps + ladder adaptation,
seeded synthetic data with that configuration's shapes and distributions.

A step is one PT sweep (nsteps=1: one stretch move of all T x W walkers,
then swaps and adaptation) on data resident in HBM.  The metric is
log-posterior evaluations x epochs per second of the whole job; the same
run reports PT sweeps/s, the FP64-plain form of the same sweep, the
roofline of the dominant kernel, an end-to-end number through the public
API with host buffers, and the reference-faithful CPU path on the host
cores.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = 'Kepler logL evals*epochs/s & PT steps/s: mixed vs FP64 plain @ |dlogL|<=1e-6'
CONFIG = 'c2'          # the configuration the metric is quoted on; others via --config
WORKLOADS = {
    'c1': 'RV PT sweep: 1 Keplerian, 1 instrument, N=256 (51 Peg shape)',
    'c2': 'RV PT sweep: 3 Keplerians, 2 instruments, N=1024, per-instrument MA(1)',
    'c4': 'RV PT sweep: 5 Keplerians, 3 instruments, N=4096, per-instrument MA(1)',
    'c5': 'RV PT sweep: 7 Keplerians, 4 instruments, N=16384, per-instrument MA(2)',
    'c3': 'RV PT sweep of a ragged batch: 4096 independent systems, N log-uniform in [50, 2000], '
          '1-4 Keplerians, 1-3 instruments',
    'gp': 'RV PT sweep with a celerite GP likelihood: 3 Keplerians, 2 instruments, N=1024, '
          'GonzRotationTerm GP (4 hyperparameters)',
    'c4grad': 'log-posterior gradients (adjoint kernel) of 65536 multistart points: 5 Keplerians, '
              '3 instruments, N=4096, per-instrument MA(1)',
}
SEED = 1234

# dram__bytes_read.sum + dram__bytes_write.sum of one launch of each workload's dominant
# kernel, from the ncu captures summarised under profiles/ (k_logpost_mixed_c2_halfstep.md,
# k_logpost_mixed_c3_ragged_stretch.md, k_gp_celerite_gp_sweep.md, k_grad_c4_gradient_batch.md);
# None where no capture was taken
NCU_TRAFFIC = {'c2': 623360, 'c3': 581037824, 'gp': 21445376, 'c4grad': 1083646568}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument('--gpus', type=int, default=1)
    p.add_argument('--steps', type=int, default=2000)
    p.add_argument('--warmup', type=int, default=10)
    p.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    p.add_argument('--fp64-steps', type=int, default=None)
    p.add_argument('--no-cpu-baseline', action='store_true')
    p.add_argument('--cpu-seconds', type=float, default=15.0)
    p.add_argument('--config', default=CONFIG, choices=sorted(WORKLOADS))
    p.add_argument('--map-iters', type=int, default=300,
                   help='iteration cap of the multistart MAP search (--config c4grad)')
    p.add_argument('--launch', default=None,
                   help='lanes,tile for the mixed kernel instead of the autotuner (e.g. 64,1024)')
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get('RANK', '0'))
    world = int(os.environ.get('WORLD_SIZE', '1'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return rank, world, local


def workload_config(setup, n, ndim, kp, nins, q, name=CONFIG):
    return {'workload': WORKLOADS[name],
            'ntemps': setup[0], 'nwalkers': setup[1], 'nsteps_per_sweep': setup[3],
            'epochs': n, 'ndim': ndim, 'planets': kp, 'instruments': nins, 'ma_order': q,
            'parameterisation': 1, 'seed': SEED, 'precision': 'mixed',
            'l2': 'flushed between timed steps (256 MiB write, outside the timed events)'}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
         'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
         'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', f'--id={self.index}', f'--query-gpu={self.Q}',
                 '--format=csv,noheader,nounits', '-lms', '200'],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for l in self.lines:
            f = [x.strip() for x in l.split(',')]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() in ('active', '1', 'yes'):
                    reasons.add(nm)
        return {'sm_mhz': float(np.median(sm)) if sm else None, 'sm_max_mhz': smax,
                'reasons': sorted(reasons), 'samples': len(sm)}


def ma_order(model):
    return max([b.moav for b in model.blocks if b.type_ == 'MOAV'] or [0])


def mixed_error(ctx, theta, logl_mixed):
    """|dlogL| / |logL| of the mixed-precision log-likelihoods the timed
    sweeps left in the walker state, against the FP64 kernel at the same
    theta (every walker slot with a finite FP64 value)."""
    import torch
    from astroemperor_gb300 import _native as N
    torch.cuda.synchronize()
    ll64 = ctx.logpost(theta.contiguous(), precision=N.EMP_PREC_FP64)[0]
    torch.cuda.synchronize()
    a, b = logl_mixed.reshape(-1).cpu().numpy(), ll64.reshape(-1).cpu().numpy()
    fin = np.isfinite(a) & np.isfinite(b)
    rel = np.abs(a[fin] - b[fin]) / np.abs(b[fin])
    return {'max_rel': float(rel.max()) if rel.size else None,
            'median_rel': float(np.median(rel)) if rel.size else None,
            'walkers': int(fin.sum()), 'bound': 1e-6,
            'what': 'stored mixed logL of the final walker states of the timed sweeps against the '
                    'FP64 kernel at the same theta'}


def cpu_baseline(model, data, truth, seconds, ncores=None):
    from oracle import cpu_baseline as cb
    lim = model.limits_free()
    rng = np.random.default_rng(7)
    th = np.clip(truth + 1e-3 * (lim[:, 1] - lim[:, 0]) * rng.normal(size=(64, len(truth))),
                 lim[:, 0], lim[:, 1])
    ncores = ncores or os.cpu_count() or 1
    eps, n, el, nc = cb.time_pool(model.spec(), data.as_dict(), th, ncores=ncores,
                                  min_seconds=seconds, max_seconds=2 * seconds)
    return eps * data.ndata, n, el, nc


def run_reference(args):
    """The reference's own CPU path (its algorithm restated in the oracle,
    since the reference cannot run here), with every host core.  One pool
    stays open; each step evaluates a bounded batch of walkers sized so that
    the whole warm-up + timed run takes about 90 s."""
    from astroemperor_gb300 import synth
    from oracle import cpu_baseline as cb
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    if args.config == 'c3':
        return run_reference_ragged(args)
    grad = args.config == 'c4grad'
    model, data, setup, truth = synth.build_model('c4' if grad else args.config, seed=SEED)
    # a gradient by forward differences costs ndim + 1 log-posterior evaluations
    per_unit = (model.ndim__ + 1) if grad else 1
    lim = model.limits_free()
    rng = np.random.default_rng(7)
    nc = os.cpu_count() or 1
    th = np.clip(truth + 1e-3 * (lim[:, 1] - lim[:, 0]) * rng.normal(size=(4096, len(truth))),
                 lim[:, 0], lim[:, 1])
    timer = cb.PoolTimer(model.spec(), data.as_dict(), nc)
    timer.warm(th)
    t1 = timer.step(th[:nc])                        # one evaluation per core
    budget = 90.0 / max(args.steps + args.warmup, 1)
    batch = int(min(len(th), max(nc, round(budget / max(t1, 1e-6)) * nc)))
    vals = []
    for i in range(args.warmup + args.steps):
        sel = th[(i * batch) % len(th):][:batch]
        if len(sel) < batch:
            sel = th[:batch]
        el = timer.step(sel)
        if i >= args.warmup:
            vals.append(len(sel) * data.ndata / el / per_unit)
    timer.close()
    v = float(np.median(vals)) if vals else float('nan')
    line = {'metric': METRIC, 'impl': 'reference', 'value': v, 'unit': 'evals*epochs/s',
            'n_gpus': 0, 'steps': args.steps, 'warmup': args.warmup,
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
            'data': 'synthetic',
            'config': workload_config(setup, data.ndata, model.ndim__, model.kplan__, data.nins,
                                      ma_order(model), args.config),
            'cpu_baseline': {'value': v, 'unit': 'evals*epochs/s', 'cores': nc, 'kind': 'port',
                             'sample': f'per step {batch} reference-faithful walker evaluations '
                                       f'(my_prior+my_likelihood, numpy over epochs) mapped over '
                                       f'multiprocessing.Pool({nc}); median over steps'
                                       + (f'; a gradient by forward differences counted as {per_unit} '
                                          f'evaluations' if grad else '')},
            'e2e': {'value': v, 'unit': 'evals*epochs/s', 'h2d_bytes_per_step': 0,
                    'd2h_bytes_per_step': 0}}
    print(json.dumps(line))
    return 0


def ragged_p0(models, truths, T, W, rng):
    out = []
    for m, th in zip(models, truths):
        lim = m.limits_free()
        c = np.clip(th, lim[:, 0], lim[:, 1])
        out.append(np.clip(c + 1e-3 * (lim[:, 1] - lim[:, 0]) * rng.normal(size=(T, W, len(c))),
                           lim[:, 0], lim[:, 1]))
    return out


def ragged_cpu_sample(sy, seconds, n_sys=64, per_sys=4, ncores=None):
    """Reference-faithful CPU rate on a sample of the batch's systems."""
    from oracle import cpu_baseline as cb
    rng = np.random.default_rng(7)
    pick = rng.choice(len(sy), size=min(n_sys, len(sy)), replace=False)
    specs = [sy[i][0].spec() for i in pick]
    datas = [sy[i][1].as_dict() for i in pick]
    n_ep = [sy[i][1].ndata for i in pick]
    p0 = ragged_p0([sy[i][0] for i in pick], [sy[i][2] for i in pick], 1, per_sys, rng)
    tasks = [(k, p0[k][0, j]) for k in range(len(pick)) for j in range(per_sys)]
    ncores = ncores or os.cpu_count() or 1
    v, ne, el, nc = cb.time_pool_many(specs, datas, tasks, n_ep, ncores=ncores,
                                      min_seconds=seconds, max_seconds=2 * seconds)
    return v, ne, el, nc, len(pick), per_sys


def main_ragged(args):
    """C3: every system of the ragged batch advances one PT sweep per step."""
    import ctypes as C
    import torch
    from astroemperor_gb300 import _native as N
    from astroemperor_gb300 import synth
    from astroemperor_gb300.batch import BatchContext, BatchPTSampler

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group('nccl')
    dev = torch.device('cuda', local if world > 1 else 0)
    torch.cuda.set_device(dev)
    # one survey of RAGGED['n_systems'] systems split across the ranks (each
    # system regenerates from its own (seed, index) key): strong scaling
    from astroemperor_gb300.replicas import shard
    n_all = synth.RAGGED['n_systems']
    mine = range(n_all)[shard(n_all, rank, world)]
    sy = [synth.ragged_model(SEED, s) for s in mine]
    models = [m for m, _, _ in sy]
    T, W, _, nsteps = synth.RAGGED['setup']
    n_ep = np.array([m.data.ndata for m in models], dtype=np.int64)
    kps = np.array([m.kplan__ for m in models], dtype=np.int64)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        v, ne, el, nc, npick, per = ragged_cpu_sample(sy, args.cpu_seconds)
        cpu = {'value': v, 'unit': 'evals*epochs/s', 'cores': nc, 'kind': 'port',
               'sample': f'{ne} reference-faithful evaluations over {npick} systems of the batch '
                         f'({per} walkers each; my_prior+my_likelihood per walker, numpy over '
                         f'epochs, Pool({nc})) in {el:.1f} s'}
    lib = N.load()
    ctx = BatchContext(models, str(dev))
    rng = np.random.default_rng(SEED + rank)
    p0 = ctx.pad(ragged_p0(models, [th for _, _, th in sy], T, W, rng))
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    fixed = tuple(int(x) for x in args.launch.split(',')) if args.launch else None

    def timed(precision, steps, warmup):
        bt = BatchPTSampler(ctx, ntemps=T, nwalkers=W, precision=precision, seed=SEED + rank,
                            record=False, autotune=not (fixed and precision == 'mixed'))
        if fixed and precision == 'mixed':
            ctx.set_launch(N.EMP_PREC_MIXED, *fixed)
            bt.launch = ctx.get_launch(N.EMP_PREC_MIXED) + (None,)
        bt.run(p0, nsweeps=max(warmup, 1))               # autotunes, then warms up
        st = bt._state_struct(nsteps)
        stream = bt.stream
        N.call('emp_pt_run', ctx.h, C.byref(st), None, 1, 1, stream.cuda_stream)
        stream.synchronize()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(steps)]
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        l0 = lib.emp_launch_count()
        for i in range(steps):
            with torch.cuda.stream(stream):
                flush.fill_(float(i))
                evs[i][0].record(stream)
            N.call('emp_pt_run', ctx.h, C.byref(st), None, 1, 1, stream.cuda_stream)
            with torch.cuda.stream(stream):
                evs[i][1].record(stream)
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in evs), lib.emp_launch_count() - l0, bt

    steps = args.steps
    clocks = ClockSampler(dev.index or 0)
    clocks.start()
    ms_mixed, launches, bt = timed('mixed', steps, args.warmup)
    clk = clocks.stop()
    err = mixed_error(ctx, bt.theta.reshape(ctx.S, -1, ctx.ndim), bt.logl)
    fp64_steps = args.fp64_steps or max(5, steps // 20)
    ms_fp64, _, bt64 = timed('fp64', fp64_steps, 3)
    from astroemperor_gb300.replicas import job_rate
    units_per_sweep = T * W * nsteps * int(n_ep.sum())
    _, t_mixed, value = job_rate(units_per_sweep * steps, ms_mixed / 1e3, device=dev)
    fp64_value = units_per_sweep * fp64_steps / (ms_fp64 / 1e3)

    # roofline: the stretch half-step shape (T*W/2 walkers of every system),
    # one launch of the same kernel and launch shape, timed alone
    half = torch.as_tensor(p0.reshape(ctx.S, T * W, ctx.ndim)[:, : T * W // 2].copy(), device=dev)
    rs = torch.cuda.Stream(device=dev)
    from astroemperor_gb300.autotune import graph_time
    hll = torch.empty(ctx.S, T * W // 2, dtype=torch.float64, device=dev)
    hlp = torch.empty_like(hll)
    k_ms = graph_time((ctx.h, half.data_ptr(), T * W // 2, None, None, hll.data_ptr(), hlp.data_ptr(),
                       None, N.EMP_PREC_MIXED, rs.cuda_stream), 10, rs)
    F = 58 * kps + 10
    flops_launch = float(np.sum(F * n_ep)) * (T * W // 2)
    f32, f64p = C.c_double(), C.c_double()
    N.call('emp_probe_peaks', C.byref(f32), C.byref(f64p), rs.cuda_stream)
    achieved = flops_launch / (k_ms * 1e-3) / 1e12
    peak32 = f32.value / 1e12
    roof = {'bound': 'fp32', 'achieved': achieved, 'peak': peak32, 'unit': 'TFLOP/s',
            'frac': achieved / peak32, 'traffic': NCU_TRAFFIC.get('c3'),
            'traffic_source': 'ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch',
            'algorithmic_bytes': int(n_ep.sum()) * 25 + ctx.S * (T * W // 2) * (8 * ctx.ndim + 16),
            'kernel': 'k_logpost<MIXED,Q=0> over all systems (stretch half-step shape)',
            'kernel_ms': k_ms, 'flop_per_eval_epoch': '58*planets + 10 per system',
            'launch': {'lanes': bt.launch[0], 'tile': bt.launch[1]},
            'peak_source': 'measured on this GPU by the library FMA probe (MEASURED_PEAKS.json '
                           'has no CUDA-core figure); compute-issue bound, not HBM or tensor',
            'fp64_peak_tflops': f64p.value / 1e12}

    # end to end: the whole slot-ordered state through pinned host memory
    SW = ctx.S * T * W
    h_theta = torch.empty(SW, ctx.ndim, dtype=torch.float64).pin_memory()
    h_ll = torch.empty(SW, dtype=torch.float64).pin_memory()
    h_lp = torch.empty(SW, dtype=torch.float64).pin_memory()
    h_theta.copy_(bt.theta.cpu())
    h_ll.copy_(bt.logl.cpu())
    h_lp.copy_(bt.logprior.cpu())
    e2e_steps = min(steps, 20)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        bt.sweep_host(h_theta, h_ll, h_lp)
    e2e_t = time.perf_counter() - t0
    bytes_io = SW * (ctx.ndim + 2) * 8
    e2e = {'value': units_per_sweep * e2e_steps / e2e_t, 'unit': 'evals*epochs/s',
           'h2d_bytes_per_step': bytes_io, 'd2h_bytes_per_step': bytes_io,
           'api': 'BatchPTSampler.sweep_host (pinned host state in, one sweep, state out)'}
    if rank == 0:
        cfg = {'workload': WORKLOADS['c3'], 'systems': n_all, 'systems_per_rank': int(ctx.S),
               'ntemps': T, 'nwalkers': W,
               'nsteps_per_sweep': nsteps, 'epochs_total': int(n_ep.sum()),
               'epochs_min_median_max': [int(n_ep.min()), int(np.median(n_ep)), int(n_ep.max())],
               'planets_hist': [int((kps == k).sum()) for k in range(1, 5)], 'ndim_max': int(ctx.ndim),
               'parameterisation': 1, 'seed': SEED, 'precision': 'mixed', 'recording': 'off',
               'l2': 'flushed between timed steps (256 MiB write, outside the timed events)'}
        line = {'metric': METRIC, 'value': value, 'unit': 'evals*epochs/s', 'n_gpus': world,
                'steps': steps, 'warmup': args.warmup, 'ms_per_step': ms_mixed / steps,
                'higher_is_better': True, 'scaling': 'strong', 'vs_baseline': None,
                'dtype': 'f32+f64 (mixed)',
                'data': 'synthetic (seeded generator with the configuration shapes)', 'config': cfg,
                'pt_sweeps_per_s': steps * world / t_mixed,
                'fp64_plain': {'value': fp64_value, 'unit': 'evals*epochs/s', 'steps': fp64_steps,
                               'ms_per_step': ms_fp64 / fp64_steps,
                               'launch': {'lanes': bt64.launch[0], 'tile': bt64.launch[1]}},
                'mixed_over_fp64': value / world / fp64_value,
                'roofline': roof, 'cpu_baseline': cpu, 'e2e': e2e, 'clocks': clk,
                'gpu_launches': int(launches), 'logl_error': err}
        if cpu:
            line['gpu_over_cpu'] = value / cpu['value']
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_reference_ragged(args):
    """Reference CPU path on the ragged batch: each step evaluates a bounded
    sample of walkers spread over 64 of the batch's systems."""
    from astroemperor_gb300 import synth
    from oracle import cpu_baseline as cb
    sy = synth.make_ragged(seed=SEED)
    rng = np.random.default_rng(7)
    pick = rng.choice(len(sy), size=64, replace=False)
    n_ep = [sy[i][1].ndata for i in pick]
    p0 = ragged_p0([sy[i][0] for i in pick], [sy[i][2] for i in pick], 1, 16, rng)
    tasks = [(k, p0[k][0, j]) for j in range(16) for k in range(len(pick))]
    nc = os.cpu_count() or 1
    timer = cb.PoolTimerMany([sy[i][0].spec() for i in pick], [sy[i][1].as_dict() for i in pick], nc)
    timer.step(tasks[:nc])
    t1 = timer.step(tasks[:4 * nc]) / (4 * nc)
    budget = 90.0 / max(args.steps + args.warmup, 1)
    batch = int(min(len(tasks), max(nc, round(budget / max(t1, 1e-6)))))
    vals = []
    for i in range(args.warmup + args.steps):
        sel = [tasks[(i * batch + j) % len(tasks)] for j in range(batch)]
        el = timer.step(sel)
        if i >= args.warmup:
            vals.append(sum(n_ep[k] for k, _ in sel) / el)
    timer.close()
    v = float(np.median(vals)) if vals else float('nan')
    T, W, _, nsteps = synth.RAGGED['setup']
    line = {'metric': METRIC, 'impl': 'reference', 'value': v, 'unit': 'evals*epochs/s',
            'n_gpus': 0, 'steps': args.steps, 'warmup': args.warmup,
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
            'data': 'synthetic',
            'config': {'workload': WORKLOADS['c3'], 'systems': len(sy), 'ntemps': T, 'nwalkers': W,
                       'nsteps_per_sweep': nsteps, 'parameterisation': 1, 'seed': SEED},
            'cpu_baseline': {'value': v, 'unit': 'evals*epochs/s', 'cores': nc, 'kind': 'port',
                             'sample': f'per step {batch} reference-faithful walker evaluations over '
                                       f'64 systems of the batch, multiprocessing.Pool({nc}); '
                                       f'median over steps'},
            'e2e': {'value': v, 'unit': 'evals*epochs/s', 'h2d_bytes_per_step': 0,
                    'd2h_bytes_per_step': 0}}
    print(json.dumps(line))
    return 0


def main_grad(args):
    """C4: one step = the log-posterior and its gradient at 65536 points (the
    multistart MAP's batch) through the adjoint kernel; units = points x epochs."""
    import ctypes as C
    import torch
    from astroemperor_gb300 import _native as N
    from astroemperor_gb300 import synth
    from astroemperor_gb300.engine import Context
    from astroemperor_gb300.replicas import job_rate

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group('nccl')
    dev = torch.device('cuda', local if world > 1 else 0)
    torch.cuda.set_device(dev)
    model, data, setup, truth = synth.build_model('c4', seed=SEED + rank)
    n, D = data.ndata, model.ndim__
    B = 65536
    lim = model.limits_free()
    rng = np.random.default_rng(SEED + rank)
    th = np.clip(truth + 0.02 * (lim[:, 1] - lim[:, 0]) * rng.normal(size=(B, D)), lim[:, 0], lim[:, 1])
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        # the reference has no gradient: its CPU path would take D+1 log-posterior
        # evaluations per point (forward differences)
        v, ne, el, nc = cpu_baseline(model, data, truth, args.cpu_seconds)
        cpu = {'value': v / (D + 1), 'unit': 'evals*epochs/s', 'cores': nc, 'kind': 'port',
               'sample': f'{ne} reference-faithful log-posterior evaluations (my_prior+my_likelihood '
                         f'per point, numpy over epochs, Pool({nc})) in {el:.1f} s; a gradient by forward '
                         f'differences costs {D + 1} of them'}
    lib = N.load()
    ctx = Context(model, str(dev))
    t = torch.as_tensor(th, dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    steps = min(args.steps, 100)
    with torch.cuda.stream(stream):
        for _ in range(max(args.warmup, 3)):
            out = ctx.logpost_grad(t, stream=stream)
    stream.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    clocks = ClockSampler(dev.index or 0)
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    l0 = lib.emp_launch_count()
    with torch.cuda.stream(stream):
        for i in range(steps):
            flush.fill_(float(i))
            evs[i][0].record(stream)
            out = ctx.logpost_grad(t, stream=stream)
            evs[i][1].record(stream)
    torch.cuda.synchronize()
    launches = lib.emp_launch_count() - l0
    clk = clocks.stop()
    ms = sum(a.elapsed_time(b) for a, b in evs)
    units = B * n
    _, t_all, value = job_rate(units * steps, ms / 1e3, device=dev)
    F = 58 * model.kplan__ + 10 + 7 * ma_order(model)
    Fg = 3 * F                                                  # forward + adjoint
    import ctypes as Cc
    f32, f64p = Cc.c_double(), Cc.c_double()
    N.call('emp_probe_peaks', Cc.byref(f32), Cc.byref(f64p), stream.cuda_stream)
    k_ms = ms / steps
    achieved = Fg * units / (k_ms * 1e-3) / 1e12
    peak32 = f32.value / 1e12
    roof = {'bound': 'fp32', 'achieved': achieved, 'peak': peak32, 'unit': 'TFLOP/s', 'frac': achieved / peak32,
            'traffic': NCU_TRAFFIC.get('c4grad'),
            'traffic_source': 'ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch (the MA '
                              'residual buffer written back from L2)',
            'algorithmic_bytes': n * 25 + B * (8 * D * 3 + 16),
            'kernel': 'k_grad<Q=1> (log-posterior and its adjoint gradient)', 'kernel_ms': k_ms,
            'flop_per_eval_epoch': Fg,
            'peak_source': 'measured on this GPU by the library FMA probe (MEASURED_PEAKS.json has no '
                           'CUDA-core figure); F counts forward + adjoint as 3 x the forward FLOP'}
    # end to end: points in from pinned host memory, gradients out
    h_th = torch.as_tensor(th, dtype=torch.float64).pin_memory()
    h_g = torch.empty(B, D, dtype=torch.float64).pin_memory()
    h_l = torch.empty(B, dtype=torch.float64).pin_memory()
    e2e_steps = min(steps, 20)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        with torch.cuda.stream(stream):
            t.copy_(h_th, non_blocking=True)
            ll, lp, gl, gp = ctx.logpost_grad(t, stream=stream)
            h_g.copy_(gl, non_blocking=True)
            h_l.copy_(ll, non_blocking=True)
        stream.synchronize()
    e2e_t = time.perf_counter() - t0
    e2e = {'value': units * e2e_steps / e2e_t, 'unit': 'evals*epochs/s', 'h2d_bytes_per_step': B * D * 8,
           'd2h_bytes_per_step': B * (D + 1) * 8,
           'api': 'Context.logpost_grad (points from pinned host memory in, gradient of logL and logL out)'}
    # time to MAP: multistart L-BFGS (the walker initialisation) from the same
    # 65536 points, every start to its own convergence or the iteration cap
    from astroemperor_gb300.mapfit import multistart_map
    ll0, lp0 = ctx.logpost(t, precision=N.EMP_PREC_FP64)
    keep = torch.isfinite(lp0)
    starts = t[keep].contiguous()
    tl, tp = ctx.logpost(torch.as_tensor(truth[None, :], dtype=torch.float64, device=dev),
                         precision=N.EMP_PREC_FP64)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = multistart_map(ctx, model, starts, iters=args.map_iters)
    torch.cuda.synchronize()
    t_map = time.perf_counter() - t0
    best = float(res['logp'].max().item())
    time_to_map = {'starts': int(starts.shape[0]), 'seconds': t_map, 'iterations': res['iterations'],
                   'gradient_evaluations': res['evaluations'],
                   'converged': int(res['converged'].sum().item()),
                   'best_logp': best, 'logp_at_generating_values': float((tl + tp).item()),
                   'what': 'multistart L-BFGS (mapfit.multistart_map) from the benchmark points with a '
                           'finite prior; every start stops at its own convergence or the iteration cap; '
                           'seconds include the eager torch bookkeeping'}
    if rank == 0:
        line = {'metric': METRIC, 'value': value, 'unit': 'evals*epochs/s', 'n_gpus': world,
                'steps': steps, 'warmup': max(args.warmup, 3), 'ms_per_step': k_ms,
                'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
                'dtype': 'f32+f64 (mixed)', 'data': 'synthetic (seeded generator with the configuration shapes)',
                'config': {'workload': WORKLOADS['c4grad'], 'points': B, 'epochs': n, 'ndim': D,
                           'planets': model.kplan__, 'instruments': data.nins, 'ma_order': ma_order(model),
                           'parameterisation': 1, 'seed': SEED,
                           'l2': 'flushed between timed steps (256 MiB write, outside the timed events)'},
                'fp64_plain': None, 'roofline': roof, 'cpu_baseline': cpu, 'e2e': e2e, 'clocks': clk,
                'gpu_launches': int(launches), 'time_to_map': time_to_map}
        if cpu:
            line['gpu_over_cpu'] = value / cpu['value']
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == 'reference':
        return run_reference(args)
    if args.config == 'c3':
        return main_ragged(args)
    if args.config == 'c4grad':
        return main_grad(args)

    import torch
    from astroemperor_gb300 import _native as N
    from astroemperor_gb300 import synth
    from astroemperor_gb300.engine import Context, PTSampler

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group('nccl')
    dev = torch.device('cuda', local if world > 1 else 0)
    torch.cuda.set_device(dev)

    # the CPU baseline pool is spawned (safe after CUDA init); run it first
    # so that the GPU timing is not disturbed by busy host cores
    model, data, setup, truth = synth.build_model(args.config, seed=SEED + rank)
    T, W, S, nsteps = setup
    n, D = data.ndata, model.ndim__
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        v, ne, el, nc = cpu_baseline(model, data, truth, args.cpu_seconds)
        cpu = {'value': v, 'unit': 'evals*epochs/s', 'cores': nc, 'kind': 'port',
               'sample': f'{ne} reference-faithful evaluations (my_prior+my_likelihood per walker, '
                         f'numpy over epochs, Pool({nc})) in {el:.1f} s'}

    lib = N.load()
    ctx = Context(model, str(dev))
    lim = model.limits_free()
    rng = np.random.default_rng(SEED + rank)
    p0 = np.clip(truth + 1e-3 * (lim[:, 1] - lim[:, 0]) * rng.normal(size=(T, W, D)),
                 lim[:, 0], lim[:, 1])
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    fixed = tuple(int(x) for x in args.launch.split(',')) if args.launch else None

    def timed_sweeps(precision, steps, warmup):
        s = PTSampler(W, D, model, ntemps=T, precision=precision, seed=SEED + rank, context=ctx,
                      autotune=not (fixed and precision == 'mixed'))
        if fixed and precision == 'mixed':
            ctx.set_launch(N.EMP_PREC_MIXED, *fixed)
            s.launch = ctx.get_launch(N.EMP_PREC_MIXED) + (None,)
        s.run_mcmc(p0, nsweeps=max(warmup, 1))          # warms up
        s._grow(steps + 2)
        st = s._state_struct(nsteps)
        rec = s._record_struct()
        import ctypes as C
        # capture the graph for these exact buffers outside the timed region
        N.call('emp_pt_run', ctx.h, C.byref(st), C.byref(rec), 1, 1, s.stream.cuda_stream)
        s.stream.synchronize()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(steps)]
        stream = s.stream
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        l0 = lib.emp_launch_count()
        for i in range(steps):
            with torch.cuda.stream(stream):
                flush.fill_(float(i))
                evs[i][0].record(stream)
            N.call('emp_pt_run', ctx.h, C.byref(st), C.byref(rec), 1, 1, stream.cuda_stream)
            with torch.cuda.stream(stream):
                evs[i][1].record(stream)
        torch.cuda.synchronize()
        launches = lib.emp_launch_count() - l0
        ms = sum(a.elapsed_time(b) for a, b in evs)
        return ms, launches, s

    clocks = ClockSampler(dev.index or 0)
    clocks.start()
    ms_mixed, launches, s_mixed = timed_sweeps('mixed', args.steps, args.warmup)
    clk = clocks.stop()
    err = mixed_error(ctx, s_mixed.theta, s_mixed.logl)
    fp64_steps = args.fp64_steps or max(20, args.steps // 20)
    ms_fp64, _, _ = timed_sweeps('fp64', fp64_steps, 3)

    from astroemperor_gb300.replicas import job_rate
    units_per_sweep = T * W * nsteps * n
    # replicas: summed work over the slowest rank's time
    _, t_mixed, value = job_rate(units_per_sweep * args.steps, ms_mixed / 1e3, device=dev)
    sweeps_s = args.steps * world / t_mixed
    fp64_value = units_per_sweep * fp64_steps / (ms_fp64 / 1e3)

    # ---- roofline of the dominant kernel: one half-step of the stretch move
    # (T*W/2 walkers x N epochs), launches captured in a CUDA graph and timed
    # with events on their stream
    th_half = torch.as_tensor(p0.reshape(-1, D)[: T * W // 2], dtype=torch.float64, device=dev)
    B = th_half.shape[0]
    ll = torch.empty(B, dtype=torch.float64, device=dev)
    lp = torch.empty_like(ll)
    rs = torch.cuda.Stream(device=dev)
    from astroemperor_gb300.autotune import graph_time
    k_ms = graph_time((ctx.h, th_half.data_ptr(), B, None, None, ll.data_ptr(),
                       lp.data_ptr(), None, N.EMP_PREC_MIXED, rs.cuda_stream), 50, rs)
    kp, q = model.kplan__, ma_order(model)
    F = 58 * kp + 10 + 7 * q                                   # FLOP per eval*epoch
    flops_launch = F * B * n
    import ctypes as C
    f32, f64p = C.c_double(), C.c_double()
    N.call('emp_probe_peaks', C.byref(f32), C.byref(f64p), rs.cuda_stream)
    achieved = flops_launch / (k_ms * 1e-3) / 1e12
    peak32 = f32.value / 1e12
    roof = {'bound': 'fp32', 'achieved': achieved, 'peak': peak32, 'unit': 'TFLOP/s',
            'frac': achieved / peak32, 'traffic': NCU_TRAFFIC.get(args.config),
            'traffic_source': 'ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch',
            'algorithmic_bytes': n * 25 + B * (8 * D + 16),
            'kernel': f'k_logpost<MIXED,Q={q}> (stretch half-step shape)',
            'kernel_ms': k_ms, 'flop_per_eval_epoch': F,
            'launch': {'lanes': s_mixed.launch[0], 'tile': s_mixed.launch[1]} if s_mixed.launch else None,
            'peak_source': 'measured on this GPU by the library FMA probe (MEASURED_PEAKS.json '
                           'has no CUDA-core figure); compute-issue bound, not HBM or tensor',
            'fp64_peak_tflops': f64p.value / 1e12}
    if any(b.type_ == 'Celerite2' for b in model.blocks):
        # the GP sweep's dominant kernel is k_gp_fused (the mixed celerite
        # preparation and recursion, M lanes per walker row): timed alone through
        # emp_gp_logl on the half-step's rows and their residuals (with the
        # conversion of those rows to float-float pairs); the mixed k_logpost
        # that writes the residuals in a sweep is reported beside it
        mod, e2 = ctx.model_eval(th_half)
        y = torch.as_tensor(data.RV, dtype=torch.float64, device=dev)
        rr = (y[None, :] - mod).t().contiguous()
        ee = e2.t().contiguous()
        gl = torch.empty(B, dtype=torch.float64, device=dev)
        g_ms = graph_time((ctx.h, th_half.data_ptr(), B, rr.data_ptr(), ee.data_ptr(), gl.data_ptr(),
                           N.EMP_PREC_MIXED, rs.cuda_stream), 50, rs, entry='emp_gp_logl')
        Mg = 4                                                  # state dimensions of the kernel
        Fg = 4.5 * Mg * Mg + 16.5 * Mg + 8                      # FLOP per row*epoch
        ach = Fg * B * n / (g_ms * 1e-3) / 1e12
        p64 = f64p.value / 1e12
        roof = {'bound': 'fp64', 'achieved': ach, 'peak': p64, 'unit': 'TFLOP/s', 'frac': ach / p64,
                'traffic': NCU_TRAFFIC.get(args.config),
                'traffic_source': 'ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch',
                'algorithmic_bytes': B * (16 * n + 8 * D + 8) + 8 * n,
                'kernel': 'k_gp_fused<4> (celerite preparation and float-float recursion, half-step rows)',
                'kernel_ms': g_ms,
                'flop_per_row_epoch': Fg,
                'peak_source': 'FP64 peak measured on this GPU by the library FMA probe (the '
                               "algorithm's arithmetic is FP64-equivalent)",
                # the float-float recursion issues FP32 instructions (about 10 per
                # FP64-equivalent operation): the same work against the FP32 pipe
                'fp32_pipe': {'peak': peak32, 'frac': ach / peak32},
                'rv_kernel': {'kernel': 'k_logpost<MIXED,Q=0> (residual rows for k_gp_fused)',
                              'kernel_ms_with_gp_kernels': k_ms, 'launch': roof['launch']}}

    # ---- end to end through the public sampler with host buffers
    s = s_mixed
    TWn = T * W
    h_state = s.host_state()                       # pinned: theta rows, logl, logprior
    e2e_steps = min(args.steps, 500)
    s.sweep_host_packed(h_state)                   # warm (graph for the packed call)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        s.sweep_host_packed(h_state)
    torch.cuda.synchronize()
    e2e_t = time.perf_counter() - t0
    bytes_io = TWn * (D + 2) * 8
    assert h_state.numel() * 8 == bytes_io
    e2e = {'value': units_per_sweep * e2e_steps / e2e_t, 'unit': 'evals*epochs/s',
           'h2d_bytes_per_step': bytes_io, 'd2h_bytes_per_step': bytes_io,
           'api': 'PTSampler.sweep_host_packed (pinned host state in, one sweep, state out, '
                  'synchronised every step)'}

    if rank == 0:
        line = {'metric': METRIC, 'value': value, 'unit': 'evals*epochs/s', 'n_gpus': world,
                'steps': args.steps, 'warmup': args.warmup,
                'ms_per_step': ms_mixed / args.steps, 'higher_is_better': True,
                'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32+f64 (mixed)',
                'data': 'synthetic (seeded generator with the configuration shapes)',
                'config': workload_config(setup, n, D, kp, data.nins, q, args.config),
                'pt_sweeps_per_s': sweeps_s,
                'fp64_plain': {'value': fp64_value, 'unit': 'evals*epochs/s', 'steps': fp64_steps,
                               'ms_per_step': ms_fp64 / fp64_steps},
                'mixed_over_fp64': value / world / fp64_value,
                'roofline': roof, 'cpu_baseline': cpu, 'e2e': e2e,
                'clocks': clk, 'gpu_launches': int(launches), 'logl_error': err}
        if cpu:
            line['gpu_over_cpu'] = value / cpu['value']
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == '__main__':
    sys.exit(main())
