"""Many independent RV systems on one GPU: one handle, one sweep sequence.

EMPEROR fits one system per ``Simulation`` (``src/astroemperor/emp.py``);
a survey runs that script once per star.  :class:`BatchContext` loads S
systems of uneven epoch counts and models (planets, instruments) into one
native handle (``emp_create_batch``), and :class:`BatchPTSampler` advances
all of them together: every stretch half-step is one persistent launch
whose CTAs claim (system, walker-chunk) items costliest system first, swaps
run one CTA per system, and the whole sweep is one CUDA graph.

System s uses the Philox key ``seed + s * 0x9E3779B97F4A7C15`` (mod 2^64),
so its chain equals a one-system :class:`~astroemperor_gb300.engine.PTSampler`
run with that seed and the same launch shape.  Arrays hold the systems
back to back; parameter rows are padded to the largest free dimension.
Systems may carry celerite GP blocks (with or without: the batch runs the
largest GP state dimension) or, all of them, joint RV + astrometry data
(one astrometry descriptor per system).
"""
from __future__ import annotations

import ctypes as C
import math
from typing import Optional, Sequence

import numpy as np
import torch

from . import _native as N
from .engine import PRECISIONS, am_descriptor, default_betas, perm_units
from .model import ReddModel

GOLDEN = 0x9E3779B97F4A7C15


def system_seed(seed: int, s: int) -> int:
    """Philox key of system ``s`` of a batch keyed by ``seed``."""
    return (int(seed) + int(s) * GOLDEN) & ((1 << 64) - 1)


def pad_rows(rows: Sequence[np.ndarray], ndim: int) -> np.ndarray:
    """Stack per-system arrays [..., D_s] into [S, ..., ndim] (zero padded)."""
    first = np.asarray(rows[0])
    out = np.zeros((len(rows),) + first.shape[:-1] + (int(ndim),), dtype=np.float64)
    for s, r in enumerate(rows):
        r = np.asarray(r, dtype=np.float64)
        out[s, ..., :r.shape[-1]] = r
    return out


class BatchContext:
    """Native handle over S systems, each with its own compiled model."""

    def __init__(self, models: Sequence[ReddModel], device='cuda:0'):
        if len(models) < 1:
            raise ValueError('at least one system')
        self.lib = N.load()
        self.device = torch.device(device)
        if self.device.type != 'cuda':
            raise ValueError('the EMPEROR GPU engine runs on a CUDA device')
        torch.cuda.set_device(self.device)
        torch.cuda.init()
        self.models = list(models)
        S = len(models)
        self.S = S
        self.free_dims = np.array([m.ndim__ for m in models], dtype=np.int64)
        self.ndim = int(self.free_dims.max())
        self.n_epochs = np.array([m.data.ndata for m in models], dtype=np.int64)
        descs = (N.EmpModelDesc * S)()
        for s, m in enumerate(models):
            descs[s] = m.descriptor()
        self._descs = descs
        self._t = np.ascontiguousarray(np.concatenate([m.data.BJD for m in models]), dtype=np.float64)
        self._y = np.ascontiguousarray(np.concatenate([m.data.RV for m in models]), dtype=np.float64)
        self._e = np.ascontiguousarray(np.concatenate([m.data.eRV for m in models]), dtype=np.float64)
        self._i = np.ascontiguousarray(np.concatenate([m.data.Flag for m in models]), dtype=np.int32)
        self._o = np.concatenate([[0], np.cumsum(self.n_epochs)]).astype(np.int64)
        ds = N.EmpDatasetDesc()
        ds.n_systems = S
        ds.offsets = self._o.ctypes.data_as(C.POINTER(C.c_int64))
        ds.t = self._t.ctypes.data_as(C.POINTER(C.c_double))
        ds.y = self._y.ctypes.data_as(C.POINTER(C.c_double))
        ds.yerr = self._e.ctypes.data_as(C.POINTER(C.c_double))
        ds.inst = self._i.ctypes.data_as(C.POINTER(C.c_int32))
        h = C.c_void_p()
        N.call('emp_create_batch', descs, C.byref(ds), C.byref(h))
        self.h = h
        if self.lib.emp_num_systems(self.h) != S:
            raise RuntimeError('native handle reports a different system count')
        if getattr(models[0], 'am_data', None) is not None:
            # joint RV + astrometry: one descriptor per system, in order
            ams = (N.EmpAmDesc * S)()
            keep = []
            for s, m in enumerate(models):
                if getattr(m, 'am_data', None) is None:
                    raise ValueError(f'system {s}: astrometric and RV-only systems in one batch')
                ams[s], arrs = am_descriptor(m.am_data)
                keep.append(arrs)
            N.call('emp_set_astrometry', self.h, ams)

    def close(self):
        if getattr(self, 'h', None):
            self.lib.emp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_launch(self, precision: int, lanes: int, tile: int):
        N.call('emp_set_launch', self.h, int(precision), int(lanes), int(tile))

    def get_launch(self, precision: int):
        L, T = C.c_int(), C.c_int()
        N.call('emp_get_launch', self.h, int(precision), C.byref(L), C.byref(T))
        return L.value, T.value

    def pad(self, rows: Sequence[np.ndarray]) -> np.ndarray:
        """Stack per-system arrays [..., D_s] into [S, ..., ndim] (zero padded)."""
        if len(rows) != self.S:
            raise ValueError(f'{len(rows)} arrays for {self.S} systems')
        return pad_rows(rows, self.ndim)

    def logpost(self, theta: torch.Tensor, precision: int = N.EMP_PREC_MIXED, stream=None):
        """(logL, logprior) [S, B] of theta [S, B, ndim] (device FP64)."""
        theta = theta.contiguous()
        if theta.dim() != 3 or theta.shape[0] != self.S or theta.shape[2] != self.ndim:
            raise ValueError(f'theta must be [S={self.S}, B, ndim={self.ndim}]')
        B = theta.shape[1]
        logl = torch.empty(self.S, B, dtype=torch.float64, device=theta.device)
        logprior = torch.empty_like(logl)
        s = stream if stream is not None else torch.cuda.current_stream(theta.device)
        N.call('emp_logpost', self.h, theta.data_ptr(), B, None, None, logl.data_ptr(),
               logprior.data_ptr(), None, int(precision), s.cuda_stream)
        return logl, logprior


class BatchPTSampler:
    """Parallel tempering over S independent systems, T x W walkers each.

    ``betas``: one ladder [T] shared by every system, or [S, T]; default
    7**-t.  ``record``: keep each system's cold chain every ``thin`` sweeps
    (chain [rows, S, W, ndim], log_like / log_prob [rows, S, W]) and the
    ladder / swap-rate histories [rows, S, T] / [rows, S, T-1].
    """

    def __init__(self, models_or_context, ntemps=8, nwalkers=64, betas=None, adapt=True,
                 adapt_tau=1000, adapt_nu=1, precision='mixed', seed=0, a=2.0, device='cuda:0',
                 use_graph=True, record=True, thin=1, autotune=True):
        ctx = models_or_context if isinstance(models_or_context, BatchContext) \
            else BatchContext(models_or_context, device)
        if nwalkers % 2:
            raise ValueError('nwalkers must be even (the stretch move splits the ensemble in two)')
        self.ctx = ctx
        self.S, self.ndim = ctx.S, ctx.ndim
        self.nwalkers = int(nwalkers)
        if betas is None:
            betas = default_betas(int(ntemps))
        betas = np.asarray(betas, dtype=np.float64)
        if betas.ndim == 1:
            betas = np.broadcast_to(betas, (self.S, len(betas)))
        if betas.shape[0] != self.S:
            raise ValueError('betas must be [T] or [S, T]')
        self.ntemps = int(betas.shape[1])
        self.adaptive = bool(adapt)
        self.adapt_tau, self.adapt_nu = float(adapt_tau), float(adapt_nu)
        self.precision = PRECISIONS[precision]
        self.seed = int(seed)
        self.a = float(a)
        self.use_graph = bool(use_graph)
        self.record, self.thin = bool(record), max(1, int(thin))
        self.autotune = bool(autotune)
        self.launch = None
        self.device = ctx.device
        self.stream = torch.cuda.Stream(device=self.device)
        S, T, W, D = self.S, self.ntemps, self.nwalkers, self.ndim
        dev = self.device
        f64 = dict(dtype=torch.float64, device=dev)
        i32 = dict(dtype=torch.int32, device=dev)
        self.theta = torch.zeros(S * T * W, D, **f64)
        self.logl = torch.full((S * T * W,), -math.inf, **f64)
        self.logprior = torch.full((S * T * W,), -math.inf, **f64)
        self.members = torch.arange(S * T * W, **i32)
        self.betas_d = torch.tensor(np.ascontiguousarray(betas), **f64).reshape(S * T)
        self.counters = torch.zeros(4, dtype=torch.int64, device=dev)
        self.accepted_d = torch.zeros(S * T * W, **i32)
        self.swaps_d = torch.zeros(S * T, **i32)
        self.units = torch.tensor(perm_units(W), **i32)
        self.n_rec = torch.zeros(2, dtype=torch.int64, device=dev)
        wb = int(ctx.lib.emp_pt_work_bytes(T, W, D))
        self.work = torch.zeros(wb, dtype=torch.uint8, device=dev)
        self.cap = 0
        self.chain = self.log_like_h = self.log_prob_h = self.beta_h = self.tsw_h = None
        self._initialised = False

    # ------------------------------------------------------------------
    def _state_struct(self, nsteps: int) -> N.EmpPtState:
        st = N.EmpPtState()
        st.ntemps, st.nwalkers, st.ndim, st.nsteps = self.ntemps, self.nwalkers, self.ndim, int(nsteps)
        st.theta, st.logl, st.logprior = self.theta.data_ptr(), self.logl.data_ptr(), self.logprior.data_ptr()
        st.members, st.betas = self.members.data_ptr(), self.betas_d.data_ptr()
        st.counters = self.counters.data_ptr()
        st.accepted, st.swaps_accepted = self.accepted_d.data_ptr(), self.swaps_d.data_ptr()
        st.perm_units, st.n_perm_units = self.units.data_ptr(), int(self.units.numel())
        st.adapt = 1 if self.adaptive else 0
        st.seed = self.seed & ((1 << 64) - 1)
        st.a = self.a
        st.adapt_tau, st.adapt_nu, st.adapt_mode = self.adapt_tau, self.adapt_nu, 0
        st.precision = self.precision
        st.work, st.work_bytes = self.work.data_ptr(), int(self.work.numel())
        st.n_systems = self.S
        return st

    def _record_struct(self) -> N.EmpPtRecord:
        r = N.EmpPtRecord()
        r.capacity = self.cap
        r.thin = self.thin
        if self.cap:
            r.chain, r.log_like = self.chain.data_ptr(), self.log_like_h.data_ptr()
            r.log_prob, r.beta_history = self.log_prob_h.data_ptr(), self.beta_h.data_ptr()
            r.tsw_history = self.tsw_h.data_ptr()
        r.n_recorded = self.n_rec.data_ptr()
        return r

    def _grow(self, rows: int):
        S, T, W, D = self.S, self.ntemps, self.nwalkers, self.ndim
        used = int(self.n_rec[0].item()) if self.cap else 0
        newcap = used + int(rows)
        f64 = dict(dtype=torch.float64, device=self.device)

        def grow(old, shape):
            new = torch.zeros((newcap,) + shape, **f64)
            if old is not None and used:
                new[:used] = old[:used]
            return new
        self.chain = grow(self.chain, (S, W, D))
        self.log_like_h = grow(self.log_like_h, (S, W))
        self.log_prob_h = grow(self.log_prob_h, (S, W))
        self.beta_h = grow(self.beta_h, (S, T))
        self.tsw_h = grow(self.tsw_h, (S, max(T - 1, 1)))
        self.cap = newcap

    def set_positions(self, p0):
        """Walker positions [S, T, W, ndim] (rows padded to ndim), evaluated."""
        p0 = np.asarray(p0, dtype=np.float64)
        want = (self.S, self.ntemps, self.nwalkers, self.ndim)
        if p0.shape != want:
            raise ValueError(f'p0 shape {p0.shape} != {want}')
        with torch.cuda.stream(self.stream):
            self.theta.copy_(torch.from_numpy(p0.reshape(-1, self.ndim)).pin_memory(), non_blocking=True)
            self.members.copy_(torch.arange(self.members.numel(), dtype=torch.int32, device=self.device))
        st = self._state_struct(1)
        N.call('emp_pt_evaluate', self.ctx.h, C.byref(st), self.stream.cuda_stream)
        self._initialised = True

    def tune(self):
        """Pick the launch shape with the autotuner on a stretch-half-sized batch."""
        from .autotune import autotune_batch
        self.stream.synchronize()
        half = self.theta.reshape(self.S, self.ntemps * self.nwalkers, self.ndim)[:, : self.ntemps * (self.nwalkers // 2)]
        self.launch = autotune_batch(self.ctx, half.contiguous(), self.precision)
        return self.launch

    def run(self, p0=None, nsweeps=1, nsteps=1):
        """``nsweeps`` sweeps of ``nsteps`` stretch steps + swaps (+ adaptation)."""
        if p0 is not None:
            self.set_positions(p0)
        if not self._initialised:
            raise RuntimeError('give p0 (or call set_positions) first')
        if self.autotune and self.launch is None:
            self.tune()
            # stored values from the shape the sweeps use
            st = self._state_struct(1)
            N.call('emp_pt_evaluate', self.ctx.h, C.byref(st), self.stream.cuda_stream)
        if self.record:
            self._grow((int(nsweeps) + self.thin - 1) // self.thin + 1)
        st = self._state_struct(nsteps)
        rec = self._record_struct() if self.record else None
        N.call('emp_pt_run', self.ctx.h, C.byref(st), C.byref(rec) if rec is not None else None,
               int(nsweeps), 1 if self.use_graph else 0, self.stream.cuda_stream)
        self.stream.synchronize()
        return self

    def sweep_host(self, h_theta, h_logl, h_logprior):
        """One sweep of every system with the slot-ordered walker state
        (theta [S*T*W, ndim], logl, logprior) in pinned host memory: copied
        in, swept, copied back, waited for.  Nothing is recorded."""
        if not self._initialised:
            raise RuntimeError('run or set_positions first')
        s = self.stream
        with torch.cuda.stream(s):
            self.theta.copy_(h_theta, non_blocking=True)
            self.logl.copy_(h_logl, non_blocking=True)
            self.logprior.copy_(h_logprior, non_blocking=True)
        st = self._state_struct(1)
        N.call('emp_pt_run', self.ctx.h, C.byref(st), None, 1, 1 if self.use_graph else 0, s.cuda_stream)
        with torch.cuda.stream(s):
            h_theta.copy_(self.theta, non_blocking=True)
            h_logl.copy_(self.logl, non_blocking=True)
            h_logprior.copy_(self.logprior, non_blocking=True)
        s.synchronize()

    # ------------------------------------------------------------------ accessors
    @property
    def iteration(self):
        return int(self.n_rec[0].item()) if self.cap else 0

    @property
    def betas(self):
        return self.betas_d.reshape(self.S, self.ntemps).cpu().numpy()

    def _by_position(self, v):
        return v[self.members.long()]

    def coords(self, s: Optional[int] = None):
        """[S, T, W, ndim] walker positions (or [T, W, D_s] of system s)."""
        c = self._by_position(self.theta).reshape(self.S, self.ntemps, self.nwalkers, self.ndim)
        if s is None:
            return c.cpu().numpy()
        return c[s, :, :, : int(self.ctx.free_dims[s])].cpu().numpy()

    def log_like(self):
        return self._by_position(self.logl).reshape(self.S, self.ntemps, self.nwalkers).cpu().numpy()

    def log_prior(self):
        return self._by_position(self.logprior).reshape(self.S, self.ntemps, self.nwalkers).cpu().numpy()

    @property
    def accepted(self):
        return self.accepted_d.reshape(self.S, self.ntemps, self.nwalkers).cpu().numpy()

    @property
    def swaps_accepted(self):
        return self.swaps_d.reshape(self.S, self.ntemps).cpu().numpy()

    def get_chain(self, s: int, discard=0, thin=1):
        """Cold chain of system s: [rows, W, D_s]."""
        n = self.iteration
        d = int(self.ctx.free_dims[s])
        return self.chain[:n, s, :, :d][int(discard)::int(thin)].cpu().numpy()

    def get_log_like(self, s: int, discard=0, thin=1):
        return self.log_like_h[: self.iteration, s][int(discard)::int(thin)].cpu().numpy()

    def get_log_prob(self, s: int, discard=0, thin=1):
        return self.log_prob_h[: self.iteration, s][int(discard)::int(thin)].cpu().numpy()

    def get_betas(self, s: int):
        return self.beta_h[: int(self.n_rec[1].item()), s].cpu().numpy()

    def get_tsw(self, s: int):
        return self.tsw_h[: int(self.n_rec[1].item()), s, : max(self.ntemps - 1, 0)].cpu().numpy()
