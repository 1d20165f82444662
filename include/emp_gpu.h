/*
 * emp_gpu.h -- C ABI of the GB300-native EMPEROR sampling hot path.
 *
 * The reference (EMPEROR / astroemperor 0.9.10) has no native FFI: its hot
 * path is Python text that it generates into a temporary run script and
 * hands to the third-party reddemcee PTSampler.  The entry points below are
 * the ones a binding of that path needs; each comment names the reference
 * interface it replaces (paths relative to the reference project root).
 *
 * Conventions
 *   - every call returns an int status: EMP_OK (0) or a negative EMP_E_* code;
 *     emp_last_error_string() gives a one-line message for the calling thread;
 *   - no exception, abort or device trap crosses this boundary; inputs that
 *     are outside the prior support or non-finite give logprior = -inf and
 *     are never evaluated further;
 *   - all array arguments of the hot calls are DEVICE pointers owned by the
 *     caller; the library allocates device memory only in emp_create (the
 *     dataset copy) and never inside emp_logpost / emp_pt_* calls;
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default);
 *   - a handle is not thread-safe: use one host thread per handle.
 */
#ifndef EMP_GPU_H
#define EMP_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EMP_ABI_VERSION 4

#define EMP_MAX_PARAMS   160   /* full theta length incl. fixed parameters */
#define EMP_MAX_PLANETS  16
#define EMP_MAX_INS      16
#define EMP_MAX_MA       3     /* moving-average order q */
#define EMP_MAX_GP_TERMS 8

/* GP terms of a celerite2 kernel (support/kernels/00.kernel, emp.py:341-412),
   as k(tau) = sum exp(-c tau) (a cos(d tau) + b sin(d tau)); gp_slot[k][i]
   is the full-theta index of the term's i-th parameter in the order below */
#define EMP_GP_REAL      1   /* RealTerm(a, c) */
#define EMP_GP_MATERN32  2   /* Matern32Term(sigma, rho), eps = 0.01 */
#define EMP_GP_ROTATION  3   /* RotationTerm(sigma, period, Q0, dQ, f) */
#define EMP_GP_GROT      4   /* the reference's GonzRotationTerm(rho, tau, A1, A2):
                                SHO(S0=A1, rho, tau) + SHO(S0=A2, rho/2, tau) */
#define EMP_GP_SHO      16   /* SHOTerm(amplitude, frequency, quality): + 1 if the
                                amplitude is sigma (else S0), + 2 if the frequency is
                                rho (else w0), + 4 if the quality is tau (else Q) */

/* status codes */
#define EMP_OK             0
#define EMP_E_INVALID     -1   /* bad argument / descriptor */
#define EMP_E_CUDA        -2   /* a CUDA runtime call failed */
#define EMP_E_UNSUPPORTED -3   /* model feature not built for this path */
#define EMP_E_SIZE        -4   /* a size is beyond a documented limit */
#define EMP_E_STATE       -5   /* call order / handle state */

/* Cosine terms carried in kep_param next to the Keplerian parameterisations
   0-4, 6, 7 (support/models/kep0*.model): sinusoid00.model (slots: period,
   amplitude, phase) and the two terms of magneticcycle00.model (slots:
   period, amplitude 1, amplitude 2, phase 1, phase 2; term 1 at half the
   frequency).  Both terms of a magnetic-cycle block use the block's first
   slot as kep_slot. */
#define EMP_TERM_SINUSOID 8
#define EMP_TERM_CYCLE_1 9
#define EMP_TERM_CYCLE_2 10

/* precision of the log-posterior */
#define EMP_PREC_FP64   0  /* plain FP64 everywhere */
#define EMP_PREC_MIXED  1  /* FP32 Kepler solve + RV sum; float-float phase;
                              compensated FP32 per-lane sums, FP64 across lanes */
/* emp_set_launch target of the adjoint kernel (emp_logpost_grad) */
#define EMP_LAUNCH_GRAD 2

/* prior kinds (support/priors/<Name>.prior) */
#define EMP_PRIOR_UNIFORM   0
#define EMP_PRIOR_NORMAL    1
#define EMP_PRIOR_JEFFREYS  2
#define EMP_PRIOR_BETA      3
#define EMP_PRIOR_NONE      4
#define EMP_PRIOR_ISOTROPIC 5   /* ln(sin(x)/2) - logZ, a0 = logZ (Isotropic.prior) */

typedef struct emp_prior {
    int32_t kind;
    int32_t _pad;
    double lo, hi;        /* support, inclusive (the reference's `limits`) */
    double a0, a1, a2;    /* Uniform/Jeffreys: a0 = ln(1/(hi-lo))
                             Normal: a0 = mu, a1 = 1/s, a2 = ln(s sqrt(2 pi)) + logZ
                             Beta:   a0 = a, a1 = b, a2 = ln B(a, b)
                             Isotropic: a0 = ln((cos lo - cos hi) / 2) */
} emp_prior;

/*
 * Compiled model: replaces the generated my_model / my_prior text
 * (emp_model.py:706-781, emp.py:182-254) and the theta index maps of
 * ReddModel.refresh__ (emp_model.py:223-305).
 */
typedef struct emp_model_desc {
    int32_t abi_version;          /* EMP_ABI_VERSION */
    int32_t n_full;               /* parameters incl. fixed ones */
    int32_t n_free;               /* ndim of the sampler */
    int32_t n_planets;
    int32_t n_ins;
    int32_t ma_order;             /* q; 0 = no MOAV block */
    int32_t ma_global;            /* 1: moav01 (global), 0: per instrument */
    int32_t ma_quirk;             /* 1: reproduce the reference's per-instrument
                                     no-op (moav00.model:18-19 writes to a copy) */
    int32_t acc_order;            /* acceleration polynomial order, 0 = none */
    int32_t offset_slot;          /* first full-theta index, -1 = none */
    int32_t jitter_slot;
    int32_t ma_slot;
    int32_t acc_slot;
    int32_t _pad0;
    int32_t kep_param[EMP_MAX_PLANETS];   /* parameterisation 0,1,2,3,4,6,7 or EMP_TERM_* */
    int32_t kep_slot[EMP_MAX_PLANETS];    /* first full-theta index of planet */
    int32_t full_src[EMP_MAX_PARAMS];     /* free index feeding slot, -1 = fixed */
    double  full_fixed[EMP_MAX_PARAMS];   /* value of fixed slots */
    /* prior of each free parameter, in the order my_prior sums them
       (block by block, emp.py:196-203); prior_block[i] = block number */
    emp_prior prior[EMP_MAX_PARAMS];
    int32_t prior_slot[EMP_MAX_PARAMS];   /* full-theta index of free param i */
    /* derived priors of Keplerian blocks, emp.py:205-226:
       [p][0]: Ecc (x = th[3]^2 + th[4]^2), [p][1]: Amp (x = th[1]^2 + th[2]^2) */
    emp_prior derived[EMP_MAX_PLANETS][2];
    double  loglike_const;        /* -0.5 ln(2 pi) ndat  (00.like:1) */
    /* sum, in my_prior's order, of the constant terms (Uniform, Jeffreys) of
       free and derived priors; the device adds the other terms to it */
    double  prior_const;
    int32_t n_prior_var;          /* terms that vary with theta (Normal, Beta) */
    int32_t _pad1;
    /* their indices: i < n_free -> free parameter i,
       n_free + 2p + k -> derived prior k of planet p */
    int32_t prior_var[EMP_MAX_PARAMS + 2 * EMP_MAX_PLANETS];
    /* Gaussian-process likelihood (support/likelihoods/02.like): with
       gp_nterms > 0 the log-likelihood is the celerite GP log-likelihood of the
       residuals with diagonal err2 instead of the independent Gaussian sum;
       with an MA that runs on the device (global, or per instrument without
       ma_quirk) the residuals are those after the MA recurrence, as 02.like's
       gp_.mean = model gives them; not combined with am_on */
    int32_t gp_nterms;
    int32_t _pad2;
    int32_t gp_kind[EMP_MAX_GP_TERMS];
    int32_t gp_slot[EMP_MAX_GP_TERMS][5];
    /* Hill stability priors (support/priors/Hill.prior, emp.py:222-227,
       block_repo.py:611-626): for every bit j (2 <= j <= EMP_MAX_PLANETS)
       set in hill_mask the prior is -inf unless each adjacent pair of the
       first j Keplerians, ordered by semi-major axis, passes the Hill
       criterion for a star of hill_starmass solar masses (the reference
       attaches one such prior to Keplerian block j for j = 2, 3, ...);
       periods, amplitudes and eccentricities are read as
       support/PAE/0<parameterisation>.pae reads them (0, 1, 2, 3, 4, 6) */
    int32_t hill_mask;
    int32_t _pad3;
    double  hill_starmass;
    /* joint RV + astrometry likelihood (support/likelihoods/a00.like): with
       am_on the log-likelihood adds the astrometric term of the data given to
       emp_set_astrometry; every Keplerian block then has seven slots (P, K,
       phase, e, w, inclination, node: akep00.model with parameterisation 0) */
    int32_t am_on;
    int32_t am_offset_slot;       /* offsets RA, DE, PLX, pm RA, pm DE (mas, mas/yr) */
    int32_t am_jitter_slot;       /* jitters of Hipparcos and Gaia */
    int32_t _pad4;
} emp_model_desc;

/*
 * Astrometric data of a joint fit (DataWrapper's AM mode,
 * qol_utils.py:103-455; the generated script's AM prologue,
 * emp_model.py:609-706), host FP64 arrays:
 */
typedef struct emp_am_desc {
    int32_t n_hipp;               /* Hipparcos abscissae */
    int32_t n_gost;               /* Gaia scan epochs (before the DR3 baseline) */
    const double* catalogs;       /* [3][7] Hipparcos, DR2, DR3: ref epoch, ra, dec
                                     (deg), parallax (mas), pmra, pmdec (mas/yr), rv */
    const double* inv_cov;        /* [3][5][5] inverse catalogue covariances */
    const double* log_det_cov;    /* [3] */
    const double* astro_gost;     /* [2][5] DR2, DR3 solutions relative to DR3 */
    const double* hipp;           /* [7][n_hipp]: BJD, EPOCH, PARF, CPSI, SPSI, RES, SRES */
    const double* gost;           /* [4][n_gost]: BJD, CPSI, SPSI, PARF */
    const double* gsv;            /* [2][5][n_gost]: DR2, DR3 solution vectors
                                     (pseudo-inverse of the release's design
                                     matrix) at its epochs, 0 at the others */
    double common_t;              /* the RV time origin (BJD) */
} emp_am_desc;

/*
 * One or more RV systems, ragged.  System s owns epochs
 * [offsets[s], offsets[s+1]).  Times must be sorted within each system and
 * already referenced to the system's first epoch (qol_utils.py:192-198).
 * inst holds 1-based instrument flags (the reference's `Flag` column).
 */
typedef struct emp_dataset_desc {
    int32_t n_systems;
    int32_t _pad;
    const int64_t* offsets;   /* host, n_systems+1 */
    const double* t;          /* host, days */
    const double* y;          /* host, m/s */
    const double* yerr;       /* host, m/s (sigma, not sigma^2) */
    const int32_t* inst;      /* host, 1..n_ins */
} emp_dataset_desc;

typedef struct emp_handle emp_handle;

/* Replaces: the generated temp script's data prologue + my_model/my_prior
   definitions (emp.py:137-175 write_script, emp_model.py:406-433).
   Copies the dataset to the device in the kernel layout. */
int emp_create(const emp_model_desc* model, const emp_dataset_desc* data,
               emp_handle** out);
int emp_destroy(emp_handle* h);

/* Many independent systems in one handle (ragged epoch counts, each with
   its own model): models[s] for s < data->n_systems, all with the same MA
   order.  Replaces mapping the reference's whole run over systems one
   script at a time.  The PT entry points then advance every system in the
   same launches: the stretch kernel is persistent (CTAs claim
   (system, walker-chunk) items, costliest systems first, from an atomic
   counter), swaps run one CTA per system, and the record keeps each
   system's cold chain (emp_pt_record.chain [rows][S][W][ndim], log_like /
   log_prob [rows][S][W], beta_history [rows][S][T], tsw_history
   [rows][S][T-1]; smd_history unused).  Systems may carry Celerite2 GP
   likelihoods (at most 65535 systems then): the GP kernels run every
   system with the largest state dimension of the batch, as a power of two
   (a system's unused dimensions stay zero; a system without GP terms then
   gets the Gaussian likelihood through the same recursion).  Joint RV +
   astrometry models: every system or none (EMP_E_UNSUPPORTED otherwise),
   with one emp_set_astrometry descriptor per system, at most 65535
   systems. */
int emp_create_batch(const emp_model_desc* models, const emp_dataset_desc* data,
                     emp_handle** out);
int emp_num_systems(emp_handle* h);

/* Replaces: my_likelihood(theta) (support/likelihoods/00.like:3-5) and
   my_prior(theta) (emp.py:190-251) evaluated for a batch of B walkers.
   theta [B][n_free] f64.  logl/logprior [B] f64 (device).
   If beta != NULL and logp != NULL, logp[b] = beta[b]*logl[b] + logprior[b]
   (logl is left at -inf when the prior is -inf).
   A batch handle (emp_create_batch) evaluates B rows per system: theta
   [S][B][ndim] with ndim the largest free dimension (shorter rows padded),
   beta and the outputs [S][B].  system_of is reserved and must be NULL.
   With a GP model (support/likelihoods/02.like) the likelihood is the
   celerite one; the handle keeps a row workspace for it, allocated by the
   first call with more rows than before (make that call outside any stream
   capture; growing it drops the handle's captured sweep graphs). */
int emp_logpost(emp_handle* h, const double* theta, int B,
                const int32_t* system_of, const double* beta,
                double* logl, double* logprior, double* logp,
                int precision, void* stream);

/* Gradient of my_likelihood and my_prior (the reference has none; it is the
   adjoint of support/likelihoods/00.like:3-5 through my_model,
   emp_model.py:706-781) for a batch of B walkers: logl/logprior [B] and
   grad_logl/grad_logprior [B][n_free] (device, FP64), with respect to the
   free parameters.  Planet constants in float-float from FP64, FP32
   per-epoch forward and adjoint terms, float-float sums finished in FP64.
   Every Keplerian parameterisation (kep00-kep07.model), sinusoid and
   magnetic-cycle terms, acceleration, up to 4 instruments, MA order <= 3,
   any number of epochs (streamed in tiles).  With MA and a series longer
   than one tile the handle keeps a residual buffer of B * epochs floats,
   allocated by the first call that needs more (make that call outside any
   stream capture).  Walkers outside the prior support get logl = -inf and
   a zero logl gradient.  GP models and batch handles: EMP_E_UNSUPPORTED. */
int emp_logpost_grad(emp_handle* h, const double* theta, int B, double* logl,
                     double* logprior, double* grad_logl, double* grad_logprior,
                     void* stream);

/* Replaces: the astrometric data prologue of the generated script
   (emp_model.py:609-706) for a handle whose model has am_on: copies the
   arrays to the device.  Call once after emp_create (or emp_create_batch),
   outside any stream capture.  For a batch handle `am` points to one
   descriptor per system, in system order; every descriptor is checked
   before anything is copied. */
int emp_set_astrometry(emp_handle* h, const emp_am_desc* am);

/* Replaces: my_model(theta) -> (model0, err20) (emp_model.py:706-781) for a
   batch of B walkers; model/err2 are device [B][n] in the dataset's input
   (time) order, model including the moving-average terms.  FP64.  Meant
   for fits and reporting (B small); the sampler never calls it. */
int emp_model_eval(emp_handle* h, const double* theta, int B, double* model,
                   double* err2, void* stream);

/* Replaces: gp_.compute(X_, diag=err2); gp_.log_likelihood(Y_) with
   gp_.mean = model (support/kernels/00.kernel, support/likelihoods/02.like)
   for a handle whose model has a Celerite2 GP: the celerite log-likelihood
   of B given residual rows under the GP hyperparameters of theta [B][n_free].
   resid and err2 are device FP64 [n][B] (epoch-major, the dataset's time
   order); logl [B].  Semiseparable recursion with M lanes per row, in FP64
   (EMP_PREC_FP64) or float-float (EMP_PREC_MIXED, the residuals converted
   first); logl = -inf where the covariance is not positive definite.
   EMP_E_UNSUPPORTED for a handle without a GP or a batch handle.  Uses (and on first need
   allocates) the handle's GP row workspace, as emp_logpost does.  The
   log-posterior entries compute the residuals themselves; this one serves
   callers with their own mean model. */
int emp_gp_logl(emp_handle* h, const double* theta, int B, const double* resid,
                const double* err2, double* logl, int precision, void* stream);

/* Parallel-tempering state, all device pointers owned by the caller.
   Walker slots are physical; `members[t*W + j]` names the slot that holds
   logical walker j of temperature t (swaps exchange slots, not positions).
   Replaces the walker state reddemcee keeps inside PTSampler
   (emp.py:576-593; reddemcee 0.8.5 / emcee 3.1.6). */
typedef struct emp_pt_state {
    int32_t ntemps, nwalkers, ndim;
    int32_t nsteps;               /* stretch steps per sweep */
    double* theta;                /* [T*W][ndim] by slot */
    double* logl;                 /* [T*W] by slot */
    double* logprior;             /* [T*W] by slot */
    int32_t* members;             /* [T][W] slot of (t, j) */
    double* betas;                /* [T] */
    int64_t* counters;            /* [4]: 0 = steps done, 1 = sweeps done */
    int32_t* accepted;            /* [T][W] cumulative stretch accepts */
    int32_t* swaps_accepted;      /* [T] cumulative swap accepts, pair (t-1,t) at t */
    int32_t* perm_units;          /* units modulo W (affine permutations) */
    int32_t n_perm_units;
    int32_t adapt;                /* 1: adapt the ladder after each sweep */
    uint64_t seed;
    double a;                     /* stretch scale, emcee default 2 */
    double adapt_tau;             /* engine_config['adapt_tau'] */
    double adapt_nu;              /* engine_config['adapt_nu'] */
    int32_t adapt_mode;           /* engine_config['adapt_mode'] (0 supported) */
    int32_t precision;            /* EMP_PREC_* used for every evaluation */
    void* work;                   /* device workspace of emp_pt_work_bytes() bytes */
    int64_t work_bytes;
    /* batched handles (emp_create_batch): every array above holds all
       systems back to back ([S][T][W] slots, [S][T] betas, theta rows of
       `ndim` = the largest free dimension, shorter rows padded); system s
       draws with key seed + s * 0x9E3779B97F4A7C15.  0 or 1 otherwise. */
    int32_t n_systems;
    int32_t _pad2;
} emp_pt_state;

/* Bytes of the workspace a PT state of this shape needs (swap log, per-sweep
   rows, the ladder of the running sweep). */
int64_t emp_pt_work_bytes(int ntemps, int nwalkers, int ndim);

/* Per-sweep history buffers (device, caller-owned; any may be NULL).
   Replaces the PTHDFBackend datasets written at emp.py:722-770. */
typedef struct emp_pt_record {
    int64_t capacity;             /* rows available */
    int32_t thin;                 /* record every `thin` steps */
    int32_t _pad;
    double* chain;                /* [capacity][T][W][ndim] */
    double* log_like;             /* [capacity][T][W] */
    double* log_prob;             /* [capacity][T][W] */
    double* beta_history;         /* [capacity_sweeps][T] */
    double* tsw_history;          /* [capacity_sweeps][T-1] */
    double* smd_history;          /* [capacity_sweeps][T-1] */
    int64_t* n_recorded;          /* [2]: rows in chain, rows in sweep hists */
} emp_pt_record;

/* Replaces: one PT sweep of reddemcee.PTSampler.run_mcmc
   (support/endit_reddemcee.scr:3): nsteps stretch moves of every
   temperature, adjacent swaps from the hottest pair down, ladder adaptation,
   history recording. Launches only; no host synchronisation. */
int emp_pt_sweep(emp_handle* h, const emp_pt_state* st,
                 const emp_pt_record* rec, void* stream);

/* No counterpart in the reference.  Same as emp_pt_sweep, for callers that
   cannot allocate device memory (all device memory owned by their own
   arena allocator, or no allocation allowed once the process runs): the
   workspace comes from a static device array of the library (st->work is
   ignored), so neither the caller nor the library allocates.  Limit:
   ntemps*nwalkers <= 32768 (EMP_E_SIZE beyond).  The first call on each
   device looks the array up and sets the kernels' attributes, and should
   come before any stream capture; calls share the array (each clears what
   must start at zero), so calls that overlap on the GPU race. */
int emp_pt_sweep_static(emp_handle* h, const emp_pt_state* st,
                        const emp_pt_record* rec, void* stream);

/* nsweeps sweeps; with use_graph != 0 one sweep is captured once into a
   CUDA graph (cached in the handle for this state) and replayed. */
int emp_pt_run(emp_handle* h, const emp_pt_state* st,
               const emp_pt_record* rec, int nsweeps, int use_graph,
               void* stream);

/* One sweep with the walker state in page-locked host memory, as a plugin
   whose caller keeps the state on the host would run it: host_state holds
   the state packed like the device buffers of `st` (theta rows by slot, then
   logl, then logprior; st->logl and st->logprior must follow st->theta that
   way), is copied in, swept and copied back, all inside one CUDA graph
   cached for (st, rec, host_state); the copy back starts after the stretch
   moves, on a second stream, while the swap and record kernels run.  Launches only: the caller synchronises
   `stream` before reading host_state.  One-system handles. */
int emp_pt_run_host(emp_handle* h, const emp_pt_state* st,
                    const emp_pt_record* rec, void* host_state, void* stream);

/* (Re)compute logl/logprior of every slot of `st` (initial state). */
int emp_pt_evaluate(emp_handle* h, const emp_pt_state* st, void* stream);

/* Lanes per walker (4, 8, 16, 32) and epoch tile used by emp_logpost /
   emp_pt_*; 0 = library default.  Set by the autotuner.  With precision =
   EMP_LAUNCH_GRAD: the adjoint kernel's epoch tile (lanes 0 or 32; tile 0
   = chosen per call, else a multiple of 32 up to 4096). */
int emp_set_launch(emp_handle* h, int precision, int lanes_per_walker,
                   int tile_epochs);
int emp_get_launch(emp_handle* h, int precision, int* lanes_per_walker,
                   int* tile_epochs);

/* Replaces: the per-temperature summaries behind reddemcee's
   get_evidence_ti / get_evidence_ss (read by postprocess, emp.py:1431-1447)
   from the log-likelihood history log_like [rows][ntemps][nwalkers] (device,
   the rows discard, discard+thin, ...): out_temp [ntemps][2] = sum and count
   of the finite values per temperature; for each of nstones stepping stones
   (samples of temperature stone_src[k], step stone_d[k] in beta; device
   arrays) out_stone [nstones][4] = max of d L, sum of exp(d L - max), sum
   of its square, count.  FP64, compensated sums. */
int emp_ladder_sums(const double* log_like, int rows, int ntemps, int nwalkers,
                    int discard, int thin, const int* stone_src,
                    const double* stone_d, int nstones, double* out_temp,
                    double* out_stone, void* stream);

/* Replaces: the autocorrelation function behind get_autocorr_time
   (emp.py:1372-1385; emcee's estimator): for the chain [rows][ntemps]
   [nwalkers][ndim] (device; rows discard, discard+thin, ...), f [ntemps]
   [ndim][maxlag] = the walkers' mean of each series' autocorrelation at lags
   0..maxlag-1 (mean removed, normalised by lag 0; a constant series counts
   as 1).  The integrated time and its window follow on the host.  At most
   51200 kept rows (EMP_E_SIZE). */
int emp_autocorr(const double* chain, int rows, int ntemps, int nwalkers, int ndim,
                 int discard, int thin, int maxlag, double* f, void* stream);

/* Measured CUDA-core throughput (FMA chains) for the roofline:
   fp32/fp64 FLOP/s of this device.  Launches a short probe kernel. */
int emp_probe_peaks(double* fp32_flops, double* fp64_flops, void* stream);

/* Number of this library's kernel launches issued so far (all handles). */
int64_t emp_launch_count(void);

const char* emp_last_error_string(void);
int emp_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* EMP_GPU_H */
