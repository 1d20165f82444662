"""GPU parallel-tempering engine with reddemcee's ``PTSampler`` surface.

EMPEROR constructs ``reddemcee.PTSampler(nwalkers, ndim, my_likelihood,
my_prior, ntemps=..., pool=..., backend=..., betas=..., tsw_history=...,
smd_history=..., adapt_tau=..., adapt_nu=..., adapt_mode=...)``
(``src/astroemperor/emp.py:576-593``), runs ``sampler.run_mcmc(p, nsweeps,
nsteps, progress)`` (``support/endit_reddemcee.scr:3``,
``endit_freeze1.scr:9-12``) and reads ``get_chain/get_log_like/
get_log_prob/get_betas/get_tsw/get_smd/get_autocorr_time/
get_evidence_ti``, ``betas`` and ``backend[t]`` (``emp.py:961-967,
1375-1447``).  This class keeps that surface, but the two callables are
replaced by a compiled :class:`~astroemperor_gb300.model.ReddModel`, and the
walker state, the sweep loop and every history live in device memory.

Per sweep the device runs ``nsteps`` affine-invariant stretch moves
(Goodman & Weare 2010; emcee 3 ``StretchMove``, a = 2) on every
temperature, adjacent-temperature swaps from the hottest pair down, and
(while adaptation is on) the Vousden et al. 2016 ladder update.  Random
numbers come from Philox4x32-10 keyed by ``seed``.
"""
from __future__ import annotations

import ctypes as C
import math
from typing import Optional

import numpy as np
import torch

from . import _native as N
from .model import ReddModel


def _ptr(t: torch.Tensor) -> int:
    return t.data_ptr()


def default_betas(ntemps: int) -> np.ndarray:
    """Geometric ladder beta_t = 7**-t.

    The reference's recorded runs with the default ladder end at
    beta_9 = 2.478e-08 = 7**-9 (10 temperatures, ``tests/01_51peg_basic.ipynb``)
    and beta_11 = 5.057e-10 = 7**-11 (12 temperatures,
    ``tests/00_mini_test.ipynb``).
    """
    return 7.0 ** -np.arange(ntemps, dtype=np.float64)


def perm_units(W: int) -> np.ndarray:
    """Multipliers m with gcd(m, W) = 1: j -> (m j + b) mod W is a bijection."""
    return np.array([m for m in range(1, max(W, 2)) if math.gcd(m, W) == 1] or [1], dtype=np.int32)


def am_descriptor(am):
    """(emp_am_desc, arrays it points into) of the astrometric data of a
    joint fit; the arrays must outlive the emp_set_astrometry call."""
    f64 = lambda x: np.ascontiguousarray(x, dtype=np.float64)
    ng = am.n_gost
    gsv = np.zeros((2, 5, ng))
    for c, cat in enumerate(('GDR2', 'GDR3')):
        gsv[c][:, am.masks[cat]] = am.gsv[cat]
    arrs = {
        'catalogs': f64(am.catalogs), 'inv_cov': f64(am.inv_cov), 'log_det_cov': f64(am.log_det_cov),
        'astro_gost': f64(am.astro_gost),
        'hipp': f64(np.stack([am.hipp[k] for k in ('BJD', 'EPOCH', 'PARF', 'CPSI', 'SPSI', 'RES', 'SRES')])),
        'gost': f64(np.stack([am.gost[k] for k in ('BJD', 'CPSI', 'SPSI', 'parf')])),
        'gsv': f64(gsv)}
    d = N.EmpAmDesc()
    d.n_hipp, d.n_gost = am.n_hipp, ng
    for k, v in arrs.items():
        setattr(d, k, v.ctypes.data)
    d.common_t = float(am.common_t)
    return d, arrs


class Context:
    """Native handle: compiled model + dataset resident on one GPU."""

    def __init__(self, model: ReddModel, device='cuda:0'):
        self.lib = N.load()
        self.device = torch.device(device)
        if self.device.type != 'cuda':
            raise ValueError('the EMPEROR GPU engine runs on a CUDA device')
        torch.cuda.set_device(self.device)
        torch.cuda.init()
        self.model = model
        self.md = model.descriptor()
        d = model.data
        self._t = np.ascontiguousarray(d.BJD, dtype=np.float64)
        self._y = np.ascontiguousarray(d.RV, dtype=np.float64)
        self._e = np.ascontiguousarray(d.eRV, dtype=np.float64)
        self._i = np.ascontiguousarray(d.Flag, dtype=np.int32)
        self._o = np.array([0, len(self._t)], dtype=np.int64)
        ds = N.EmpDatasetDesc()
        ds.n_systems = 1
        ds.offsets = self._o.ctypes.data_as(C.POINTER(C.c_int64))
        ds.t = self._t.ctypes.data_as(C.POINTER(C.c_double))
        ds.y = self._y.ctypes.data_as(C.POINTER(C.c_double))
        ds.yerr = self._e.ctypes.data_as(C.POINTER(C.c_double))
        ds.inst = self._i.ctypes.data_as(C.POINTER(C.c_int32))
        h = C.c_void_p()
        N.call('emp_create', C.byref(self.md), C.byref(ds), C.byref(h))
        self.h = h
        if getattr(model, 'am_data', None) is not None and self.md.am_on:
            self._set_astrometry(model.am_data)

    def _set_astrometry(self, am):
        """Upload the astrometric data of a joint fit (emp_set_astrometry)."""
        d, keep = am_descriptor(am)
        N.call('emp_set_astrometry', self.h, C.byref(d))

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

    def logpost(self, theta: torch.Tensor, precision: int = N.EMP_PREC_MIXED,
                beta: Optional[torch.Tensor] = None, stream=None):
        """(logL, logprior) of theta [B, ndim] (device FP64)."""
        theta = theta.contiguous()
        B = theta.shape[0]
        logl = torch.empty(B, dtype=torch.float64, device=theta.device)
        logprior = torch.empty_like(logl)
        logp = torch.empty_like(logl) if beta is not None else None
        s = stream if stream is not None else torch.cuda.current_stream(theta.device)
        N.call('emp_logpost', self.h, _ptr(theta), B, None,
               _ptr(beta) if beta is not None else None, _ptr(logl), _ptr(logprior),
               _ptr(logp) if logp is not None else None, int(precision), s.cuda_stream)
        if beta is not None:
            return logl, logprior, logp
        return logl, logprior


    def logpost_grad(self, theta: torch.Tensor, stream=None):
        """(logL, logprior, dlogL/dtheta, dlogprior/dtheta) of theta [B, ndim],
        from the adjoint kernel (FP32 per epoch, FP64 sums)."""
        theta = theta.contiguous()
        B, D = theta.shape
        f64 = dict(dtype=torch.float64, device=theta.device)
        logl, logprior = torch.empty(B, **f64), torch.empty(B, **f64)
        gl, gp = torch.empty(B, D, **f64), torch.empty(B, D, **f64)
        s = stream if stream is not None else torch.cuda.current_stream(theta.device)
        N.call('emp_logpost_grad', self.h, _ptr(theta), B, _ptr(logl), _ptr(logprior), _ptr(gl),
               _ptr(gp), s.cuda_stream)
        return logl, logprior, gl, gp

    def model_eval(self, theta: torch.Tensor, stream=None):
        """my_model(theta) on the device: (model0, err20), each [B, ndata], FP64."""
        theta = theta.contiguous()
        B = theta.shape[0]
        n = len(self._t)
        model = torch.empty(B, n, dtype=torch.float64, device=theta.device)
        err2 = torch.empty_like(model)
        s = stream if stream is not None else torch.cuda.current_stream(theta.device)
        N.call('emp_model_eval', self.h, _ptr(theta), B, _ptr(model), _ptr(err2), s.cuda_stream)
        return model, err2

    def gp_logl(self, theta: torch.Tensor, resid: torch.Tensor, err2: torch.Tensor,
                precision: int = N.EMP_PREC_FP64, stream=None):
        """Celerite GP log-likelihood [B] of residual rows resid [B, ndata] with
        diagonal err2 [B, ndata] (time order) under the GP hyperparameters of
        theta [B, ndim] -- ``gp_.log_likelihood(Y_)`` with ``gp_.mean = model``."""
        theta = theta.contiguous()
        B = theta.shape[0]
        r = resid.t().contiguous()                     # epoch-major [ndata, B]
        e = err2.t().contiguous()
        logl = torch.empty(B, dtype=torch.float64, device=theta.device)
        s = stream if stream is not None else torch.cuda.current_stream(theta.device)
        N.call('emp_gp_logl', self.h, _ptr(theta), B, _ptr(r), _ptr(e), _ptr(logl), int(precision),
               s.cuda_stream)
        return logl


PRECISIONS = {'fp64': N.EMP_PREC_FP64, 'mixed': N.EMP_PREC_MIXED,
              N.EMP_PREC_FP64: N.EMP_PREC_FP64, N.EMP_PREC_MIXED: N.EMP_PREC_MIXED}


class PTState:
    """What ``run_mcmc`` returns; pass it back to continue on the device."""

    def __init__(self, sampler):
        self.sampler = sampler

    @property
    def coords(self):
        return self.sampler._coords_host()

    @property
    def log_like(self):
        return self.sampler._logl_host()

    @property
    def log_prob(self):
        return self.sampler._logp_host()

    @property
    def betas(self):
        return self.sampler.betas


class _TempBackend:
    """``sampler.backend[t]`` view (emcee-style backend of one temperature)."""

    def __init__(self, sampler, t):
        self.s, self.t = sampler, t

    @property
    def iteration(self):
        return self.s.iteration

    def get_chain(self, **kw):
        return self.s.get_chain(**kw)[self.t]

    def get_log_like(self, **kw):
        return self.s.get_log_like(**kw)[self.t]

    def get_log_prob(self, **kw):
        return self.s.get_log_prob(**kw)[self.t]

    def get_betas(self, **kw):
        return self.s.get_betas(**kw)[:, self.t]

    @property
    def accepted(self):
        return self.s.accepted[self.t]


class _Backend:
    def __init__(self, sampler):
        self.s = sampler

    def __getitem__(self, t):
        return _TempBackend(self.s, t)

    def __len__(self):
        return self.s.ntemps

    @property
    def iteration(self):
        return self.s.iteration

    @property
    def tsw_history_bool(self):
        return self.s.tsw_history_bool

    @property
    def smd_history_bool(self):
        return self.s.smd_history_bool

    @property
    def tsw_history(self):
        return self.s.get_tsw()

    @property
    def smd_history(self):
        return self.s.get_smd()


class PTSampler:
    """reddemcee-compatible parallel-tempering sampler on one GPU.

    ``log_likelihood``/``log_prior`` positional arguments of reddemcee are
    replaced by ``model`` (a compiled :class:`ReddModel`).  Extra keywords:
    ``precision`` ('mixed' or 'fp64'), ``seed``, ``a`` (stretch scale),
    ``device``, ``use_graph``.
    """

    def __init__(self, nwalkers, ndim, model: ReddModel, ntemps=5, pool=None, backend=None,
                 betas=None, tsw_history=True, smd_history=True, adapt_tau=1000, adapt_nu=1,
                 adapt_mode=0, precision='mixed', seed=None, a=2.0, device='cuda:0',
                 use_graph=True, moves=None, context: Optional[Context] = None, autotune=True):
        if model.ndim__ != ndim:
            raise ValueError(f'ndim={ndim} but the model has {model.ndim__} free parameters')
        if nwalkers % 2:
            raise ValueError('nwalkers must be even (the stretch move splits the ensemble in two)')
        if adapt_mode != 0:
            raise NotImplementedError('adapt_mode 0 (swap-rate equalisation) is the built ladder rule')
        self.model = model
        self.nwalkers, self.ndim = int(nwalkers), int(ndim)
        if betas is not None:
            betas = np.asarray(betas, dtype=np.float64)
            ntemps = len(betas)
        else:
            betas = default_betas(int(ntemps))
        self.ntemps = int(ntemps)
        self.tsw_history_bool = bool(tsw_history)
        self.smd_history_bool = bool(smd_history)
        self.adapt_tau, self.adapt_nu, self.adapt_mode = float(adapt_tau), float(adapt_nu), int(adapt_mode)
        self.adaptive = True
        self.precision = PRECISIONS[precision]
        self.a = float(a)
        self.use_graph = bool(use_graph)
        self.autotune = bool(autotune)
        self.launch = None                 # (lanes per walker, tile, ms) chosen by the autotuner
        if seed is None:
            seed = int(np.random.randint(0, 2 ** 62))
        self.seed = int(seed)
        self.ctx = context if context is not None else Context(model, device)
        self.device = self.ctx.device
        self.stream = torch.cuda.Stream(device=self.device)
        self.D_ = None
        self.pool = pool
        T, W, D = self.ntemps, self.nwalkers, self.ndim
        dev = self.device
        f64 = dict(dtype=torch.float64, device=dev)
        i32 = dict(dtype=torch.int32, device=dev)
        # walker state by slot in one allocation (theta rows, then logl, then
        # logprior), so that a host round trip is one copy each way
        self._state = torch.empty(T * W * (D + 2), **f64)
        self.theta = self._state[: T * W * D].view(T * W, D)
        self.logl = self._state[T * W * D: T * W * (D + 1)]
        self.logprior = self._state[T * W * (D + 1):]
        self.theta.zero_()
        self.logl.fill_(-math.inf)
        self.logprior.fill_(-math.inf)
        self._st_key = None
        self._st = None
        self.members = torch.arange(T * W, **i32)
        self.betas_d = torch.tensor(betas, **f64)
        self.counters = torch.zeros(4, dtype=torch.int64, device=dev)
        self.accepted_d = torch.zeros(T * W, **i32)
        self.swaps_d = torch.zeros(T, **i32)
        self.units = torch.tensor(perm_units(W), **i32)
        self.n_rec = torch.zeros(2, dtype=torch.int64, device=dev)
        wb = int(self.ctx.lib.emp_pt_work_bytes(T, W, D))
        self.work = torch.zeros(wb, dtype=torch.uint8, device=dev)
        self.cap = 0
        self.chain = self.log_like_h = self.log_prob_h = None
        self.beta_h = self.tsw_h = self.smd_h = None
        self._initialised = False
        self.backend = _Backend(self)

    # ------------------------------------------------------------------
    def _state_struct(self, nsteps: int) -> N.EmpPtState:
        key = (int(nsteps), self.adaptive, self.seed, self.a, self.adapt_tau, self.adapt_nu,
               self.adapt_mode, self.precision, self.work.data_ptr())
        if key == self._st_key:
            return self._st
        st = N.EmpPtState()
        st.ntemps, st.nwalkers, st.ndim, st.nsteps = self.ntemps, self.nwalkers, self.ndim, int(nsteps)
        st.theta, st.logl, st.logprior = _ptr(self.theta), _ptr(self.logl), _ptr(self.logprior)
        st.members, st.betas, st.counters = _ptr(self.members), _ptr(self.betas_d), _ptr(self.counters)
        st.accepted, st.swaps_accepted = _ptr(self.accepted_d), _ptr(self.swaps_d)
        st.perm_units, st.n_perm_units = _ptr(self.units), int(self.units.numel())
        st.adapt = 1 if self.adaptive else 0
        st.seed = self.seed & ((1 << 64) - 1)
        st.a = self.a
        st.adapt_tau, st.adapt_nu, st.adapt_mode = self.adapt_tau, self.adapt_nu, self.adapt_mode
        st.precision = self.precision
        st.work, st.work_bytes = _ptr(self.work), int(self.work.numel())
        st.n_systems = 1
        self._st_key, self._st = key, st
        return st

    def _record_struct(self) -> N.EmpPtRecord:
        r = N.EmpPtRecord()
        r.capacity = self.cap
        r.thin = 1
        r.chain, r.log_like, r.log_prob = _ptr(self.chain), _ptr(self.log_like_h), _ptr(self.log_prob_h)
        r.beta_history = _ptr(self.beta_h)
        r.tsw_history = _ptr(self.tsw_h) if self.tsw_history_bool else None
        r.smd_history = _ptr(self.smd_h) if self.smd_history_bool else None
        r.n_recorded = _ptr(self.n_rec)
        return r

    def _grow(self, extra: int):
        T, W, D = self.ntemps, self.nwalkers, self.ndim
        used = int(self.n_rec[0].item()) if self.cap else 0
        newcap = used + int(extra)
        f64 = dict(dtype=torch.float64, device=self.device)

        def grow(old, shape):
            new = torch.zeros((newcap,) + shape, **f64)
            if old is not None and used:
                new[:used] = old[:used]
            return new
        self.chain = grow(self.chain, (T, W, D))
        self.log_like_h = grow(self.log_like_h, (T, W))
        self.log_prob_h = grow(self.log_prob_h, (T, W))
        self.beta_h = grow(self.beta_h, (T,))
        self.tsw_h = grow(self.tsw_h, (max(T - 1, 1),))
        self.smd_h = grow(self.smd_h, (max(T - 1, 1),))
        self.cap = newcap

    def set_positions(self, p0):
        """Load walker positions [ntemps, nwalkers, ndim] and evaluate them."""
        p0 = np.asarray(p0, dtype=np.float64)
        if p0.shape != (self.ntemps, self.nwalkers, self.ndim):
            raise ValueError(f'p0 shape {p0.shape} != {(self.ntemps, self.nwalkers, self.ndim)}')
        with torch.cuda.stream(self.stream):
            self.theta.copy_(torch.from_numpy(p0.reshape(-1, self.ndim)).pin_memory(), non_blocking=True)
            self.members.copy_(torch.arange(self.ntemps * self.nwalkers, dtype=torch.int32, device=self.device))
        st = self._state_struct(1)
        N.call('emp_pt_evaluate', self.ctx.h, C.byref(st), self.stream.cuda_stream)
        self._initialised = True

    def run_mcmc(self, initial_state, nsweeps, nsteps=1, progress=False, use_graph=None):
        """``nsweeps`` sweeps of ``nsteps`` stretch steps + swaps (+ adaptation)."""
        if isinstance(initial_state, PTState) and initial_state.sampler is self and self._initialised:
            pass
        else:
            p0 = initial_state.coords if isinstance(initial_state, PTState) else initial_state
            self.set_positions(p0)
        nsweeps = int(nsweeps)
        if self.autotune and self.launch is None:
            from .autotune import autotune
            self.stream.synchronize()
            half = self.theta[: self.ntemps * (self.nwalkers // 2)]
            self.launch = autotune(self.ctx, half, self.precision)
            # stored values from the shape the sweeps use
            st = self._state_struct(1)
            N.call('emp_pt_evaluate', self.ctx.h, C.byref(st), self.stream.cuda_stream)
        self._grow(nsweeps)
        st = self._state_struct(nsteps)
        rec = self._record_struct()
        ug = self.use_graph if use_graph is None else bool(use_graph)
        N.call('emp_pt_run', self.ctx.h, C.byref(st), C.byref(rec), nsweeps, 1 if ug else 0,
               self.stream.cuda_stream)
        self.stream.synchronize()
        return PTState(self)

    def sweep_host(self, h_theta, h_logl, h_logprior, use_graph=None):
        """One sweep with the walker state kept in (pinned) host memory.

        Copies the slot-ordered state (theta [T*W, ndim], logl, logprior)
        to the device, runs one sweep, copies it back, and waits; the
        temperature membership table stays on the device.
        """
        if not self._initialised:
            raise RuntimeError('run_mcmc or set_positions first')
        s = self.stream
        with torch.cuda.stream(s):
            self.theta.copy_(h_theta, non_blocking=True)
            self.logl.copy_(h_logl, non_blocking=True)
            self.logprior.copy_(h_logprior, non_blocking=True)
        if self.cap == 0:
            self._grow(1)
        st = self._state_struct(1)
        rec = self._record_struct()
        ug = self.use_graph if use_graph is None else bool(use_graph)
        N.call('emp_pt_run', self.ctx.h, C.byref(st), C.byref(rec), 1, 1 if ug else 0, s.cuda_stream)
        with torch.cuda.stream(s):
            h_theta.copy_(self.theta, non_blocking=True)
            h_logl.copy_(self.logl, non_blocking=True)
            h_logprior.copy_(self.logprior, non_blocking=True)
        s.synchronize()

    def host_state(self):
        """A pinned host buffer laid out like the device state (theta rows by
        slot, then logl, then logprior), holding the current state."""
        h = torch.empty(self._state.numel(), dtype=torch.float64).pin_memory()
        self.stream.synchronize()
        h.copy_(self._state)
        return h

    def sweep_host_packed(self, h_state):
        """``sweep_host`` with the state in one pinned buffer from
        ``host_state()``: the copy in, the sweep and the copy back run as one
        CUDA graph (``emp_pt_run_host``); returns after the copy back."""
        if not self._initialised:
            raise RuntimeError('run_mcmc or set_positions first')
        if h_state.numel() != self._state.numel() or h_state.dtype != torch.float64:
            raise ValueError('h_state must be the pinned float64 buffer of host_state()')
        # the pinned-memory query once per buffer (it costs a driver call)
        if getattr(self, '_pinned_ptr', None) != h_state.data_ptr():
            if not h_state.is_pinned():
                raise ValueError('h_state must be the pinned float64 buffer of host_state()')
            self._pinned_ptr = h_state.data_ptr()
        if self.cap == 0:
            self._grow(1)
        st = self._state_struct(1)
        rec = self._rec_cached()
        N.call('emp_pt_run_host', self.ctx.h, C.byref(st), C.byref(rec), h_state.data_ptr(),
               self.stream.cuda_stream)
        self.stream.synchronize()

    def _rec_cached(self):
        key = (self.cap, self.chain.data_ptr() if self.chain is not None else 0,
               self.tsw_history_bool, self.smd_history_bool)
        if getattr(self, '_rec_key', None) != key:
            self._rec_key, self._rec = key, self._record_struct()
        return self._rec

    def select_adjustment(self, name='00'):
        """Freeze the ladder (endit_freeze1.scr:11 calls ``select_adjustment('00')``)."""
        if str(name) in ('00', '0', 'none', 'None'):
            self.adaptive = False
        else:
            raise ValueError(f'adjustment {name!r} not built')

    @property
    def config_adaptation_halflife(self):
        return self.adapt_tau if self.adaptive else 0

    @config_adaptation_halflife.setter
    def config_adaptation_halflife(self, v):
        # endit_freeze.scr:37 sets 0 to stop adapting
        if not v:
            self.adaptive = False
        else:
            self.adaptive = True
            self.adapt_tau = float(v)

    # ------------------------------------------------------------------ accessors
    @property
    def betas(self):
        return self.betas_d.detach().cpu().numpy().copy()

    @property
    def iteration(self):
        return int(self.n_rec[0].item()) if self.cap else 0

    def _coords_host(self):
        T, W = self.ntemps, self.nwalkers
        return self.theta[self.members.long()].reshape(T, W, self.ndim).cpu().numpy()

    def _logl_host(self):
        return self.logl[self.members.long()].reshape(self.ntemps, self.nwalkers).cpu().numpy()

    def _logp_host(self):
        b = self.betas_d.repeat_interleave(self.nwalkers)
        m = self.members.long()
        lp = self.logprior[m]
        out = torch.where(lp > -math.inf, b * self.logl[m] + lp, torch.full_like(lp, -math.inf))
        return out.reshape(self.ntemps, self.nwalkers).cpu().numpy()

    @property
    def accepted(self):
        return self.accepted_d.reshape(self.ntemps, self.nwalkers).cpu().numpy()

    @property
    def acceptance_fraction(self):
        it = max(self.iteration, 1)
        return self.accepted / float(it)

    def _hist(self, buf, discard=0, thin=1):
        n = self.iteration
        return buf[:n][int(discard)::int(thin)]

    def get_chain(self, flat=False, thin=1, discard=0):
        """Per temperature: [S, W, D] (or [S*W, D] with flat=True)."""
        c = self._hist(self.chain, discard, thin).cpu().numpy()      # [S, T, W, D]
        c = np.moveaxis(c, 1, 0)                                       # [T, S, W, D]
        if flat:
            return c.reshape(self.ntemps, -1, self.ndim)
        return c

    def get_log_like(self, flat=False, thin=1, discard=0):
        c = np.moveaxis(self._hist(self.log_like_h, discard, thin).cpu().numpy(), 1, 0)
        return c.reshape(self.ntemps, -1) if flat else c

    def get_log_prob(self, flat=False, thin=1, discard=0):
        c = np.moveaxis(self._hist(self.log_prob_h, discard, thin).cpu().numpy(), 1, 0)
        return c.reshape(self.ntemps, -1) if flat else c

    def get_betas(self, discard=0, thin=1):
        return self._hist(self.beta_h, discard, thin).cpu().numpy()

    def get_tsw(self, discard=0, thin=1):
        return self._hist(self.tsw_h, discard, thin).cpu().numpy()[:, :max(self.ntemps - 1, 0)]

    def get_smd(self, discard=0, thin=1):
        return self._hist(self.smd_h, discard, thin).cpu().numpy()[:, :max(self.ntemps - 1, 0)]

    def _kept(self, discard, thin):
        n = self.iteration
        discard, thin = int(discard), max(1, int(thin))
        return n, discard, thin, (max(0, n - discard) + thin - 1) // thin

    def get_autocorr_time(self, discard=0, thin=1, c=5, tol=50, quiet=False):
        """Integrated autocorrelation time per temperature and parameter
        (emcee's estimator: walker-averaged autocorrelation, automated window
        c).  The autocorrelation is computed on the device from the recorded
        chain (``emp_autocorr``, lags doubled until every window closes);
        the windows on the host."""
        from .stats import check_tau, tau_from_acf
        rows, discard, thin, n = self._kept(discard, thin)
        T, D = self.ntemps, self.ndim
        if n == 0:
            raise ValueError('no samples after discard')
        maxlag = min(n, 256)
        while True:
            f = torch.empty(T, D, maxlag, dtype=torch.float64, device=self.device)
            N.call('emp_autocorr', _ptr(self.chain), rows, T, self.nwalkers, D, discard, thin, maxlag,
                   _ptr(f), self.stream.cuda_stream)
            self.stream.synchronize()
            fh = f.cpu().numpy()
            res = [[tau_from_acf(fh[t, d], c) for d in range(D)] for t in range(T)]
            if all(ok for r in res for _, ok in r) or maxlag >= n:
                break
            maxlag = min(n, 4 * maxlag)
        tau = np.array([[v for v, _ in r] for r in res])
        for t in range(T):
            check_tau(tau[t], n, tol, quiet)
        return tau * thin

    def _ladder_sums(self, discard, stones=False):
        from .stats import stepping_stone_plan
        rows, discard, thin, n = self._kept(discard, 1)
        T = self.ntemps
        out_t = torch.zeros(T, 2, dtype=torch.float64, device=self.device)
        src = step = out_s = None
        ns = 0
        if stones:
            _, s_np, d_np = stepping_stone_plan(self.betas)
            ns = len(s_np)
            src = torch.as_tensor(s_np, dtype=torch.int32, device=self.device)
            step = torch.as_tensor(d_np, dtype=torch.float64, device=self.device)
            out_s = torch.zeros(max(ns, 1), 4, dtype=torch.float64, device=self.device)
        N.call('emp_ladder_sums', _ptr(self.log_like_h), rows, T, self.nwalkers, discard, 1,
               _ptr(src) if ns else None, _ptr(step) if ns else None, ns, _ptr(out_t),
               _ptr(out_s) if ns else None, self.stream.cuda_stream)
        self.stream.synchronize()
        return out_t.cpu().numpy(), (out_s[:ns].cpu().numpy() if ns else np.zeros((0, 4)))

    def get_evidence_ti(self, discard=0, pchip=True):
        """Thermodynamic integration of <log L>_beta over the ladder; the
        per-temperature means reduced on the device (``emp_ladder_sums``)."""
        from .stats import ti_from_means
        sums, _ = self._ladder_sums(discard)
        with np.errstate(invalid='ignore', divide='ignore'):
            mean = np.where(sums[:, 1] > 0, sums[:, 0] / np.maximum(sums[:, 1], 1), -np.inf)
        return ti_from_means(self.betas, mean, pchip=pchip)

    def get_evidence_ss(self, discard=0):
        """Stepping-stone log-evidence and its error (``stats.stepping_stone``),
        from the stones' sums reduced on the device (``emp_ladder_sums``)."""
        from .stats import ss_from_sums
        sums, stones = self._ladder_sums(discard, stones=True)
        return ss_from_sums(self.betas, sums, stones)

    def get_evidence_hybrid(self, discard=0):
        """reddemcee's 'hybrid' estimator (EMPEROR's default
        ``evidence_method``, ``emp.py:129``) is defined in reddemcee's own
        source, which the reference does not vendor; it is refused rather
        than replaced.  EMPEROR's postprocess catches the error and falls
        back to thermodynamic integration (``emp.py:1443-1445``); call
        ``get_evidence_ti`` or ``get_evidence_ss`` directly."""
        raise NotImplementedError("reddemcee's hybrid evidence estimator is not available on the GPU "
                                  "engine; use get_evidence_ti or get_evidence_ss")

    def run_adaptation_batches(self, p1, adaptation_batches, adaptation_nsweeps, nsweeps, nsteps=1,
                               tol0=10, tau_diff_to_converge=0.1):
        """The batched-adaptation driver of ``support/endit_freeze.scr``: run
        ``adaptation_nsweeps`` with the ladder adapting, up to
        ``adaptation_batches`` times, until the cold chain's integrated
        autocorrelation times are below 1/``tol0`` of the iterations and
        changed by less than ``tau_diff_to_converge`` since the last batch;
        then freeze the ladder (``config_adaptation_halflife = 0``) and run
        ``nsweeps`` more.  Returns (state, converged_during_adaptation, tau)."""
        state = p1
        old_tau = np.inf
        converged = False
        tau0 = None
        for _ in range(int(adaptation_batches)):
            state = self.run_mcmc(state, nsweeps=adaptation_nsweeps, nsteps=nsteps)
            tau0 = self.get_autocorr_time(quiet=True, tol=0)[0]
            niter = self.iteration
            converged = bool(np.all(tau0 * tol0 < niter))
            converged &= bool(np.all(np.abs(old_tau - tau0) / tau0 < tau_diff_to_converge))
            old_tau = tau0
            if converged:
                break
        self.config_adaptation_halflife = 0
        state = self.run_mcmc(state, nsweeps=nsweeps, nsteps=nsteps)
        return state, converged, tau0

    def save(self, path, discard=0, thin=1):
        """Write the run in the reference's post-run backend layout
        (``backend_io.save_run``); returns the path written."""
        from .backend_io import save_run
        return save_run(self, path, discard=discard, thin=thin)

    def get_func(self, name, kwargs=None):
        return getattr(self, name)(**(kwargs or {}))
