"""Launch-shape autotuner for the log-posterior kernel.

The kernel's shape has two knobs (``emp_set_launch``): lanes per walker L
(a warp holds 32/L walkers for L < 32; a walker spans L/32 warps above) and
the epoch tile staged in shared memory.  The best pair depends on the batch
(walkers per launch), the number of epochs and the model (planets, MA
order): few walkers want many lanes each, long series want the largest
tile that still leaves room for several CTAs per SM.  ``autotune`` times
every candidate on a representative batch (launches captured in a CUDA
graph, timed with events on its own stream), keeps the fastest, sets it on the handle and caches the choice per
(model shape, batch, precision).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import _native as N

LANES = (8, 16, 32, 64, 128, 256)
TILES = (512, 1024, 2048, 4096)

_CACHE = {}


def shape_key(ctx, batch, precision):
    md = ctx.md
    return (int(md.n_planets), int(md.n_ins), int(md.ma_order), int(md.ma_global), int(md.ma_quirk),
            int(md.acc_order), int(md.n_free), len(ctx._t), int(batch), int(precision))


def candidates(n_epochs, batch):
    """(L, tile) pairs worth timing: at least ~2 epochs per lane."""
    out = []
    for L in LANES:
        if L > 8 and n_epochs < 2 * L:
            continue
        for t in TILES:
            if t > 2 * max(n_epochs, 512):
                continue
            out.append((L, t))
    return out


def graph_time(args, reps, stream, entry='emp_logpost'):
    """Device milliseconds per ``entry(*args)`` call (default
    ``emp_logpost``): ``reps`` calls (fewer for calls above ~5 ms) captured
    in one CUDA graph and replayed between two events, so that host-side call
    overhead does not enter the measurement."""
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        e0.record(stream)
        N.call(entry, *args)                                       # warm, sets attributes
        e1.record(stream)
    e1.synchronize()
    reps = int(max(1, min(reps, round(20.0 / max(e0.elapsed_time(e1), 1e-3)))))
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        for _ in range(reps):
            N.call(entry, *args)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # replay() launches on the current stream: keep the warm-up and the
    # timed replay on the same stream so that they cannot overlap
    with torch.cuda.stream(stream):
        g.replay()
        e0.record(stream)
        g.replay()
        e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def time_launch(ctx, theta, precision, reps, stream):
    B = theta.shape[0]
    ll = torch.empty(B, dtype=torch.float64, device=theta.device)
    lp = torch.empty_like(ll)
    args = (ctx.h, theta.data_ptr(), B, None, None, ll.data_ptr(), lp.data_ptr(), None,
            int(precision), stream.cuda_stream)
    return graph_time(args, reps, stream)


def autotune(ctx, theta, precision=N.EMP_PREC_MIXED, reps=None, use_cache=True, verbose=False):
    """Pick and set the fastest (L, tile) for a batch like ``theta`` [B, ndim].

    Returns (L, tile, ms_per_launch).
    """
    theta = theta.contiguous()
    B = theta.shape[0]
    key = shape_key(ctx, B, precision)
    if use_cache and key in _CACHE:
        L, tile, ms = _CACHE[key]
        ctx.set_launch(precision, L, tile)
        return L, tile, ms
    stream = torch.cuda.Stream(device=theta.device)
    n = len(ctx._t)
    if reps is None:
        reps = 8
    best = None
    results = []
    seen = set()
    for L, tile in candidates(n, B):
        ctx.set_launch(precision, L, tile)
        eff = ctx.get_launch(precision)                # tile as clamped by the library
        if eff in seen:
            continue
        seen.add(eff)
        ms = time_launch(ctx, theta, precision, reps, stream)
        results.append((ms, eff[0], eff[1]))
        if verbose:
            print(f'autotune L={eff[0]:4d} tile={eff[1]:5d} {ms * 1e3:9.2f} us')
        if best is None or ms < best[0]:
            best = (ms, eff[0], eff[1])
    ms, L, tile = best
    ctx.set_launch(precision, L, tile)
    _CACHE[key] = (L, tile, ms)
    return L, tile, ms


def representative_batch(model, batch, device, rng=None):
    """Draws inside the free parameters' limits (e, S, C kept moderate)."""
    rng = rng or np.random.default_rng(0)
    lim = model.limits_free()
    th = rng.uniform(lim[:, 0], lim[:, 1], size=(batch, len(lim)))
    for j, p in enumerate(model.free_parameters()):
        if p.name.startswith(('Ecc_sin', 'Ecc_cos')):
            th[:, j] *= 0.5
        elif p.name.startswith('Eccentricity'):
            th[:, j] = np.minimum(th[:, j], 0.5)
    return torch.as_tensor(th, dtype=torch.float64, device=device)


def autotune_batch(ctx, theta, precision=N.EMP_PREC_MIXED, reps=3, verbose=False):
    """(L, tile, ms) for a batch handle: every candidate timed on theta
    [S, B, ndim] (all systems in one launch), the fastest kept."""
    theta = theta.contiguous()
    S, B, _ = theta.shape
    stream = torch.cuda.Stream(device=theta.device)
    n_typ = int(np.median(ctx.n_epochs))
    ll = torch.empty(S, B, dtype=torch.float64, device=theta.device)
    lp = torch.empty_like(ll)
    best, seen = None, set()
    for L, tile in candidates(n_typ, B):
        ctx.set_launch(precision, L, tile)
        eff = ctx.get_launch(precision)
        if eff in seen:
            continue
        seen.add(eff)
        args = (ctx.h, theta.data_ptr(), B, None, None, ll.data_ptr(), lp.data_ptr(), None,
                int(precision), stream.cuda_stream)
        ms = graph_time(args, reps, stream)
        if verbose:
            print(f'autotune batch L={eff[0]:4d} tile={eff[1]:5d} {ms:9.3f} ms')
        if best is None or ms < best[0]:
            best = (ms, eff[0], eff[1])
    ms, L, tile = best
    ctx.set_launch(precision, L, tile)
    return L, tile, ms
