// emp_gp.cuh -- celerite Gaussian-process log-likelihood of a walker row.
//
// The reference's GP runs (support/kernels/00.kernel, support/likelihoods/
// 02.like, emp.py:341-412) build a celerite2 kernel from the row's
// hyperparameters, set the mean to the RV model, factorise K = k(|t_i - t_j|)
// + diag(err2) and return the Gaussian log-likelihood of the residuals.
// k(tau) = sum_j exp(-c_j tau) (a_j cos(d_j tau) + b_j sin(d_j tau)) is
// semiseparable, so the log-likelihood follows from the O(N J^2) recursion of
// Foreman-Mackey, Agol, Ambikasaran & Angus (2017, AJ 154, 220):
//
//   U_n = [a cos(d t_n) + b sin(d t_n), a sin(d t_n) - b cos(d t_n)],
//   V_n = [cos(d t_n), sin(d t_n)] per complex component, [a], [1] per real one,
//   phi_n = exp(-c (t_n - t_{n-1})),
//   S_n = phi_n (S_{n-1} + D_{n-1} W_{n-1} W_{n-1}^T) phi_n,
//   D_n = err2_n + sum(a) - U_n^T S_n U_n,   W_n = (V_n - S_n U_n) / D_n,
//   f_n = phi_n (f_{n-1} + W_{n-1} z_{n-1}), z_n = r_n - U_n^T f_n,
//   logL = -0.5 sum(z_n^2 / D_n + log D_n) - 0.5 N log(2 pi).
//
// k_logpost writes each valid row's residuals and err2 (epoch-major) and the
// prior.  The parts of the recursion that do not depend on its state (the
// sincos and exp) are evaluated for every (row, epoch) in parallel -- by
// k_gp_prep for the FP64 recursion k_gp, by the producer warps of k_gp_fused
// beside its float-float recursion for the mixed precision -- and the
// recursion runs with one lane per state dimension and finishes the mode:
// log-posterior rows, state slots, or the stretch move's Metropolis test.  FP64 on this GPU
// issues one warp instruction per ~64 cycles per SM sub-partition, so the
// transcendentals leave the sequential chain for parallel threads (and, in
// the mixed precision, run in float-float on the FP32 pipes), the lanes share
// a row's S, and log det needs no log per epoch.
#pragma once

#include "emp_kernels.cuh"

namespace emp {

// state dimensions of one term of the descriptor (a real component takes
// one, a complex component two; an SHO two in either regime)
__host__ __device__ inline int gp_term_dims(int kind) {
    if (kind == EMP_GP_REAL) return 1;
    if (kind == EMP_GP_MATERN32) return 2;
    if (kind == EMP_GP_ROTATION || kind == EMP_GP_GROT) return 4;
    if (kind >= EMP_GP_SHO && kind < EMP_GP_SHO + 8) return 2;
    return -1;
}

struct GPDim {
    double a, b, c, d;
    int sinpart;               // second dimension of a complex component
    int live;                  // 0: padding (U = V = 0)
};

__device__ inline void gp_real(GPDim* dm, int k, double a, double c) {
    dm[k] = GPDim{a, 0.0, c, 0.0, 0, 1};
}

__device__ inline void gp_complex(GPDim* dm, int k, double a, double b, double c, double d) {
    dm[k] = GPDim{a, b, c, d, 0, 1};
    dm[k + 1] = GPDim{a, b, c, d, 1, 1};
}

// celerite2 SHOTerm(S0, w0, Q) (eps = 1e-5) into dimensions k, k+1: two real
// components when Q < 1/2, one complex component otherwise
__device__ inline void gp_sho(GPDim* dm, int k, double S0, double w0, double Q) {
    if (Q < 0.5) {
        const double f = sqrt(fmax(1.0 - 4.0 * Q * Q, 1e-5));
        const double a = 0.5 * S0 * w0 * Q;
        gp_real(dm, k, a * (1.0 + 1.0 / f), 0.5 * w0 / Q * (1.0 - f));
        gp_real(dm, k + 1, a * (1.0 - 1.0 / f), 0.5 * w0 / Q * (1.0 + f));
    } else {
        const double f = sqrt(fmax(4.0 * Q * Q - 1.0, 1e-5));
        const double a = S0 * w0 * Q;
        gp_complex(dm, k, a, a / f, 0.5 * w0 / Q, 0.5 * w0 * f / Q);
    }
}

// coefficients of every term from the row's full parameter vector; returns
// the number of dimensions used
__device__ inline int gp_fill(const emp_model_desc* md, const double* th, GPDim* dm) {
    const double kTwoPi = 6.283185307179586;
    int k = 0;
    for (int j = 0; j < md->gp_nterms; ++j) {
        double p[5];
        for (int i = 0; i < 5; ++i) {
            const int s = md->gp_slot[j][i];
            if (s < 0) { p[i] = 0.0; continue; }
            const int src = md->full_src[s];
            p[i] = src >= 0 ? th[src] : md->full_fixed[s];
        }
        const int kind = md->gp_kind[j];
        if (kind == EMP_GP_REAL) {
            gp_real(dm, k, p[0], p[1]);
        } else if (kind == EMP_GP_MATERN32) {
            // celerite2 Matern32Term(sigma, rho), eps = 0.01
            const double w0 = 1.7320508075688772 / p[1], s2 = p[0] * p[0];
            gp_complex(dm, k, s2, s2 * w0 / 0.01, w0, 0.01);
        } else if (kind == EMP_GP_ROTATION) {
            // celerite2 RotationTerm(sigma, period, Q0, dQ, f)
            const double amp = p[0] * p[0] / (1.0 + p[4]);
            const double Q1 = 0.5 + p[2] + p[3];
            const double w1 = 4.0 * 3.141592653589793 * Q1 / (p[1] * sqrt(4.0 * Q1 * Q1 - 1.0));
            const double Q2 = 0.5 + p[2];
            const double w2 = 8.0 * 3.141592653589793 * Q2 / (p[1] * sqrt(4.0 * Q2 * Q2 - 1.0));
            gp_sho(dm, k, amp / (w1 * Q1), w1, Q1);
            gp_sho(dm, k + 2, p[4] * amp / (w2 * Q2), w2, Q2);
        } else if (kind == EMP_GP_GROT) {
            // two SHO terms at rho and rho/2 sharing tau (emp.py:404-405)
            const double rho = p[0], tau = p[1];
            const double w1 = kTwoPi / rho, w2 = kTwoPi / (0.5 * rho);
            gp_sho(dm, k, p[2], w1, 0.5 * w1 * tau);
            gp_sho(dm, k + 2, p[3], w2, 0.5 * w2 * tau);
        } else {
            // SHOTerm in any of (S0|sigma, w0|rho, Q|tau)
            const int bits = kind - EMP_GP_SHO;
            const double w0 = (bits & 2) ? kTwoPi / p[1] : p[1];
            const double Q = (bits & 4) ? 0.5 * w0 * p[2] : p[2];
            const double S0 = (bits & 1) ? p[0] * p[0] / (w0 * Q) : p[0];
            gp_sho(dm, k, S0, w0, Q);
        }
        k += gp_term_dims(kind);
    }
    return k;
}

// the prior and free parameters of row `row` in the launch's mode
__device__ inline double gp_row(const KArgs& A, int row, const double** th) {
    const int ds = A.dstride;
    if (A.mode == kModeGPOnly) { *th = A.theta + (size_t)row * ds; return 0.0; }
    if (A.mode == kModeLogpost) { *th = A.theta + (size_t)row * ds; return A.logprior[row]; }
    if (A.mode == kModeSlots) { *th = A.st_theta + (size_t)row * ds; return A.st_logprior[row]; }
    *th = A.gp_prop + (size_t)row * ds;
    return A.gp_meta[row].lp;
}

// System s of a batch handle seen as a one-system launch: its model, its
// series and every row array from that system's first element on (a
// one-system launch comes back unchanged).  Epoch-major arrays hold all
// systems' epochs ([epochs][rows]), row arrays [systems][rows].  In stretch
// mode the proposals carry the batch's own slot numbers, so the slot arrays
// stay whole and the temperatures and acceptance counts move instead.
__device__ __forceinline__ KArgs sys_rows(const KArgs& B, int s) {
    KArgs A = B;
    if (B.sys_off == nullptr) return A;
    const int64_t e0 = B.sys_off[s];
    const size_t rows = (size_t)B.nwalk, ds = (size_t)B.dstride;
    const size_t so = (size_t)s * rows;
    A.md = B.md + s;
    A.d.t = B.d.t + e0;
    A.d.n = (int)(B.sys_off[s + 1] - e0);
    if (B.gp_meta != nullptr) A.gp_meta = B.gp_meta + so;
    if (B.gp_prop != nullptr) A.gp_prop = B.gp_prop + so * ds;
    if (B.mode == kModeLogpost) {
        A.theta = B.theta + so * ds;
        A.logprior = B.logprior + so;
        A.logl = B.logl + so;
        if (B.logp != nullptr) A.logp = B.logp + so;
        if (B.beta != nullptr) A.beta = B.beta + so;
    } else if (B.mode == kModeSlots) {
        A.st_theta = B.st_theta + so * ds;
        A.st_logprior = B.st_logprior + so;
        A.st_logl = B.st_logl + so;
    } else if (B.mode == kModeStretch) {
        A.betas = B.betas + (size_t)s * B.T;
        A.accepted = B.accepted + (size_t)s * B.T * B.W;
    }
    return A;
}

// the GP kernels' view: the rows above and the GP row buffers
template <int M>
__device__ __forceinline__ KArgs gp_system(const KArgs& B, int s) {
    KArgs A = sys_rows(B, s);
    if (B.sys_off == nullptr) return A;
    const size_t ep = (size_t)B.sys_off[s] * (size_t)B.nwalk, so = (size_t)s * (size_t)B.nwalk;
    A.gp_r = B.gp_r + ep;
    A.gp_e = B.gp_e + ep;
    if (B.gp_u != nullptr) {
        A.gp_u = B.gp_u + ep * M;
        A.gp_v = B.gp_v + ep * M;
        A.gp_ph = B.gp_ph + ep * M;
    }
    A.gp_asum = B.gp_asum + so;
    return A;
}

// x as a float-float pair by bit manipulation (integer and FP32 instructions
// only; a double-to-float conversion would take the FP64 pipe): hi = x
// truncated to 24 significant bits, lo = the remaining 29 bits rounded to a
// float (|x - hi - lo| <= 2^-47 |x|).  |x| < 2^-125 flushes to zero; |x|
// must be below 2^128.
__device__ __forceinline__ float2 ff_split_bits(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7ffu) - 1023;
    if (e < -125) return make_float2(0.f, 0.f);
    const unsigned sign = (unsigned)(b >> 63) << 31;
    const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
    const float hi = __uint_as_float(sign | ((unsigned)(e + 127) << 23) | (unsigned)(m >> 29));
    const float lo = ldexpf(__uint2float_rn((unsigned)(m & 0x1FFFFFFFu)), e - 52);
    return make_float2(hi, sign ? -lo : lo);
}

// float-float helpers of the mixed recursion
__device__ __forceinline__ FF ff_of(float2 v) { return FF{v.x, v.y}; }
__device__ __forceinline__ FF ff_neg(FF a) { return FF{-a.hi, -a.lo}; }
__device__ __forceinline__ FF ff_shfl(FF a, int src, int width) {
    return FF{__shfl_sync(0xffffffffu, a.hi, src, width), __shfl_sync(0xffffffffu, a.lo, src, width)};
}
__device__ __forceinline__ FF ff_shfl_xor(FF a, int m, int width) {
    return FF{__shfl_xor_sync(0xffffffffu, a.hi, m, width), __shfl_xor_sync(0xffffffffu, a.lo, m, width)};
}
__device__ __forceinline__ FF ff_mulr(FF a, FF b) {                 // renormalised product
    const FF p = ff_mul(a, b);
    return ff_norm(p.hi, p.lo);
}

// ---------------------------------------------------------------------------
// float-float sin/cos and exp for the mixed prep.  FP64 transcendentals cost
// ~40-60 FP64 instructions each on a pipe that issues one warp instruction
// per ~64 cycles per sub-partition; here the FP64 part is only the
// Cody-Waite argument reduction (Cody & Waite 1980; the split constants are
// pi/2 and ln 2 cut into 33/33/53- and 32/53-bit doubles), and the series
// run in float-float on the FP32 pipes: Taylor coefficients 1/n! as
// float-float pairs, the terms that cannot reach 1e-16 of the result in
// plain FP32.  Relative error ~1e-15 (the recursion needs ~1e-12); for exp
// below e^-60 the low part falls into the FP32 subnormals (such factors only
// clear the recursion's memory).
// ---------------------------------------------------------------------------
#define EMP_FFC(h, l) FF{h, l}
__device__ __forceinline__ FF ff_horner(FF q, FF s, FF c) { return ff_add(ff_mul(q, s), c); }

// sin and cos of r, |r| <~ pi/4, r float-float
__device__ __forceinline__ void ff_sincos_red(FF r, FF& sn, FF& cs) {
    const FF s = ff_mulr(r, r);
    const float sh = s.hi;
    // sin r = r + r s (-1/3! + s (1/5! + s (-1/7! + s (1/9! + s T)))),
    // T = -1/11! + s/13! - s^2/15! in FP32
    const float T = fmaf(sh, fmaf(sh, -0x1.ae7f3ep-41f, 0x1.612462p-33f), -0x1.ae6456p-26f);
    FF q = ff_add(EMP_FFC(0x1.71de3ap-19f, 0x1.55b1ccp-45f), FF{sh * T, 0.f});
    q = ff_horner(q, s, EMP_FFC(-0x1.a01a02p-13f, 0x1.7f97fap-39f));
    q = ff_horner(q, s, EMP_FFC(0x1.111112p-7f, -0x1.dddddep-32f));
    q = ff_horner(q, s, EMP_FFC(-0x1.555556p-3f, 0x1.555556p-28f));
    sn = ff_add(r, ff_mul(r, ff_mulr(s, q)));
    // cos r = 1 + s (-1/2 + s (1/4! + s (-1/6! + s (1/8! + s (-1/10! + s U))))),
    // U = 1/12! - s/14! + s^2/16! in FP32
    const float U = fmaf(sh, fmaf(sh, 0x1.ae7f3ep-45f, -0x1.93974ap-37f), 0x1.1eed8ep-29f);
    FF c = ff_add(EMP_FFC(-0x1.27e4fcp-22f, 0x1.10ec14p-47f), FF{sh * U, 0.f});
    c = ff_horner(c, s, EMP_FFC(0x1.a01a02p-16f, -0x1.7f97fap-42f));
    c = ff_horner(c, s, EMP_FFC(-0x1.6c16c2p-10f, 0x1.27d27ep-35f));
    c = ff_horner(c, s, EMP_FFC(0x1.555556p-5f, -0x1.555556p-30f));
    c = ff_horner(c, s, EMP_FFC(-0.5f, 0.f));
    cs = ff_add(FF{1.f, 0.f}, ff_mul(s, c));
}

// (sin x, cos x) of a double x as float-float pairs
__device__ __forceinline__ void ff_sincos(double x, FF& sn, FF& cs) {
    if (!(fabs(x) < 1.6e6)) {                          // beyond the 3-part reduction
        double s, c;
        sincos(x, &s, &c);
        sn = ff_of(ff_split_bits(s));
        cs = ff_of(ff_split_bits(c));
        return;
    }
    const double kd = rint(x * 0.6366197723675814);
    double r = fma(-kd, 1.5707963267341256, x);
    r = fma(-kd, 6.077100506303966e-11, r);
    r = fma(-kd, 2.0222662487959506e-21, r);
    FF s, c;
    ff_sincos_red(ff_of(ff_split_bits(r)), s, c);
    switch (((int)kd) & 3) {
        case 0: sn = s; cs = c; break;
        case 1: sn = c; cs = ff_neg(s); break;
        case 2: sn = ff_neg(s); cs = ff_neg(c); break;
        default: sn = ff_neg(c); cs = s; break;
    }
}

// exp(-y), y >= 0, as a float-float pair (0 below 2^-126)
__device__ __forceinline__ FF ff_exp_neg(double y) {
    if (!(y < 87.0)) return FF{0.f, 0.f};
    const double kd = rint(-y * 1.4426950408889634);
    double r = fma(-kd, 0.6931471806019545, -y);
    r = fma(-kd, -4.2009150726810846e-11, r);
    const FF rf = ff_of(ff_split_bits(r));
    const float rh = rf.hi;
    // e^r = 1 + r (1 + r (1/2! + ... + r (1/8! + r T))), T = 1/9! + r/10! + r^2/11! in FP32
    const float T = fmaf(rh, fmaf(rh, 0x1.ae6456p-26f, 0x1.27e4fcp-22f), 0x1.71de3ap-19f);
    FF q = ff_add(EMP_FFC(0x1.a01a02p-16f, -0x1.7f97fap-42f), FF{rh * T, 0.f});
    q = ff_horner(q, rf, EMP_FFC(0x1.a01a02p-13f, -0x1.7f97fap-39f));
    q = ff_horner(q, rf, EMP_FFC(0x1.6c16c2p-10f, -0x1.27d27ep-35f));
    q = ff_horner(q, rf, EMP_FFC(0x1.111112p-7f, -0x1.dddddep-32f));
    q = ff_horner(q, rf, EMP_FFC(0x1.555556p-5f, -0x1.555556p-30f));
    q = ff_horner(q, rf, EMP_FFC(0x1.555556p-3f, -0x1.555556p-28f));
    q = ff_horner(q, rf, EMP_FFC(0.5f, 0.f));
    q = ff_horner(q, rf, EMP_FFC(1.f, 0.f));
    q = ff_horner(q, rf, EMP_FFC(1.f, 0.f));
    // times 2^k (k >= -126 since y < 87), exact
    const float sc = __int_as_float(((int)kd + 127) << 23);
    return FF{q.hi * sc, q.lo * sc};
}

// Everything of the FP64 recursion that does not depend on its state, for
// every (row, epoch) in parallel: U_n, V_n and phi_n (one sincos and one exp
// per component).  Thread (row, g): rows across the warp's lanes (coalesced
// [n][rows][M] writes), epochs g, g + E, ... with E = 8 * gridDim.y.
template <int M>
__global__ void __launch_bounds__(256) k_gp_prep(KArgs A0) {
    const KArgs A = gp_system<M>(A0, blockIdx.z);
    const int row = blockIdx.x * 32 + (threadIdx.x & 31);
    const int E = gridDim.y * 8;
    const int g = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (row >= A.nwalk) return;
    const double* th;
    const double lp = gp_row(A, row, &th);
    if (!(lp > -INFINITY)) return;
    double pa[M], pb[M], pc[M], pd[M], pv[M];
    bool ps[M];
    bool finite = true;
    double asum = 0.0;
    {
        GPDim dm[M];
#pragma unroll
        for (int k = 0; k < M; ++k) dm[k] = GPDim{0.0, 0.0, 0.0, 0.0, 0, 0};
        gp_fill(A.md, th, dm);
#pragma unroll
        for (int k = 0; k < M; ++k) {
            pa[k] = dm[k].a; pb[k] = dm[k].b; pc[k] = dm[k].c; pd[k] = dm[k].d;
            ps[k] = dm[k].sinpart != 0;
            pv[k] = dm[k].live ? 1.0 : 0.0;
            if (!ps[k]) asum += dm[k].a;
            finite = finite && isfinite(dm[k].a) && isfinite(dm[k].b) && isfinite(dm[k].c) &&
                     isfinite(dm[k].d);
        }
    }
    if (g == 0) A.gp_asum[row] = finite ? asum : NAN;
    if (!finite) return;
    const double* t = A.d.t;
    const int n = A.d.n;
    for (int i = g; i < n; i += E) {
        const double ti = t[i];
        const double dt = i > 0 ? ti - t[i - 1] : 0.0;
        double sn[M], cs[M], ph[M];
        const size_t o = ((size_t)i * A.nwalk + row) * M;
#pragma unroll
        for (int k = 0; k < M; ++k) {
            if (k > 0 && ps[k]) { sn[k] = sn[k - 1]; cs[k] = cs[k - 1]; ph[k] = ph[k - 1]; }
            else {
                if (pd[k] != 0.0) sincos(pd[k] * ti, &sn[k], &cs[k]);
                else { sn[k] = 0.0; cs[k] = 1.0; }
                ph[k] = pc[k] != 0.0 ? exp(-pc[k] * dt) : 1.0;
            }
            A.gp_u[o + k] = ps[k] ? pa[k] * sn[k] - pb[k] * cs[k] : pa[k] * cs[k] + pb[k] * sn[k];
            A.gp_v[o + k] = pv[k] * (ps[k] ? sn[k] : cs[k]);
            A.gp_ph[o + k] = ph[k];
        }
    }
}

// the mode's outputs of one row (all M lanes of the row call it)
template <int M>
__device__ __forceinline__ void gp_finish(const KArgs& A, int row, int k, bool live, bool valid, double lp,
                                          const double* th, double ll) {
    const emp_model_desc* md = A.md;
    // one value for the row: every lane takes lane 0's
    ll = __shfl_sync(0xffffffffu, ll, 0, M);
    if (A.mode == kModeGPOnly) {
        if (live && k == 0) A.logl[row] = ll;
    } else if (A.mode == kModeLogpost) {
        if (live && k == 0) {
            A.logl[row] = valid ? ll : -INFINITY;
            if (A.logp != nullptr && A.beta != nullptr)
                A.logp[row] = (valid && ll > -INFINITY) ? __dadd_rn(__dmul_rn(A.beta[row], ll), lp) : -INFINITY;
        }
    } else if (A.mode == kModeSlots) {
        if (live && k == 0) A.st_logl[row] = ll;
    } else {
        // stretch: every lane of the row takes the same decision; the
        // current walker's values are read before lane 0 replaces them
        bool acc = false;
        GPMeta m{};
        if (valid && ll > -INFINITY) {
            m = A.gp_meta[row];
            const double beta = A.betas[m.t];
            const double lpj = A.st_logprior[m.slot];
            const double llj = A.st_logl[m.slot];
            const double cur = lpj > -INFINITY ? __dadd_rn(__dmul_rn(beta, llj), lpj) : -INFINITY;
            const double nlp = __dadd_rn(__dmul_rn(beta, ll), lp);
            acc = metropolis(nlp, cur, m.z, md->n_free - 1, m.uword);
        }
        __syncwarp();
        if (acc) {
            if (k == 0) {
                A.st_logl[m.slot] = ll;
                A.st_logprior[m.slot] = lp;
                A.accepted[m.pos] += 1;
            }
            double* dst = A.st_theta + (size_t)m.slot * A.dstride;
            for (int d = k; d < md->n_free; d += M) dst[d] = th[d];
        }
    }
}

// The sequential recursion, M lanes per row (lane k owns state dimension k:
// row k of S, f_k, W_k), 32/M rows per warp.  Per epoch a lane does its S row
// update, (S U)_k and its W_k; U^T S U and U^T f are summed over the row's
// lanes by a butterfly (commutative, so every lane holds the same sum), and
// log det K is kept as a product renormalised to [1, 2) with its exponent
// counted, so no log is taken per epoch.  All lanes of a warp run every
// epoch (rows past the launch's rows repeat the last row; rows outside the
// prior compute on unwritten residuals and are discarded), which keeps the
// shuffles convergent.
template <int M>
__global__ void __launch_bounds__(128) k_gp(KArgs A0) {
    const KArgs A = gp_system<M>(A0, blockIdx.y);
    const unsigned FULL = 0xffffffffu;
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int rowr = gtid / M;
    const int k = gtid & (M - 1);
    const bool live = rowr < A.nwalk;
    const int row = live ? rowr : A.nwalk - 1;
    const emp_model_desc* md = A.md;
    const double* th;
    const double lp = gp_row(A, row, &th);
    const bool valid = live && (lp > -INFINITY);
    const double asum = valid ? A.gp_asum[row] : 0.0;
    const size_t ld = (size_t)A.nwalk;
    const int n = A.d.n;
    const double* Up = A.gp_u + (size_t)row * M + k;
    const double* Vp = A.gp_v + (size_t)row * M + k;
    const double* Pp = A.gp_ph + (size_t)row * M + k;
    const double* rp = A.gp_r + row;
    const double* ep = A.gp_e + row;
    double S[M];
#pragma unroll
    for (int j = 0; j < M; ++j) S[j] = 0.0;
    double f = 0.0, W = 0.0, Dp = 0.0, zp = 0.0, quad = 0.0, prod = 1.0;
    int pexp = 0;
    bool bad = !isfinite(asum);
    auto epoch = [&](int i, double Uk, double Vk, double Pk, double ri, double ei) {
        double Uj[M];
#pragma unroll
        for (int j = 0; j < M; ++j) Uj[j] = __shfl_sync(FULL, Uk, j, M);
        if (i > 0) {
            const double dw = Dp * W;
#pragma unroll
            for (int j = 0; j < M; ++j) {
                const double Wj = __shfl_sync(FULL, W, j, M);
                const double pj = __shfl_sync(FULL, Pk, j, M);
                S[j] = (Pk * pj) * fma(dw, Wj, S[j]);
            }
            f = Pk * fma(W, zp, f);
        }
        double su = 0.0;
#pragma unroll
        for (int j = 0; j < M; ++j) su = fma(S[j], Uj[j], su);
        double p1 = Uk * su, p2 = Uk * f;
#pragma unroll
        for (int off = M / 2; off >= 1; off >>= 1) {
            p1 += __shfl_xor_sync(FULL, p1, off, M);
            p2 += __shfl_xor_sync(FULL, p2, off, M);
        }
        const double D = ei + asum - p1;
        bad = bad || !(D > 0.0);
        const double iD = 1.0 / D;
        W = (Vk - su) * iD;
        const double z = ri - p2;
        quad = fma(z * z, iD, quad);
        // prod *= D, then its binary exponent moves into pexp
        prod *= D;
        {
            const int hi = __double2hiint(prod);
            const int ex = ((hi >> 20) & 0x7ff) - 1023;
            pexp += ex;
            prod = __hiloint2double(hi - (int)((unsigned)ex << 20), __double2loint(prod));
        }
        Dp = D; zp = z;
    };
    // the inputs of PF epochs are loaded one block ahead of their use
    constexpr int PF = 4;
    double cU[PF], cV[PF], cP[PF], cr[PF], ce[PF];
#pragma unroll
    for (int q = 0; q < PF; ++q) {
        const bool ok = valid && q < n;
        const size_t o = (size_t)q * ld;
        cU[q] = ok ? Up[o * M] : 0.0; cV[q] = ok ? Vp[o * M] : 0.0; cP[q] = ok ? Pp[o * M] : 1.0;
        cr[q] = ok ? rp[o] : 0.0; ce[q] = ok ? ep[o] : 1.0;
    }
    for (int i0 = 0; i0 < n; i0 += PF) {
        double nU[PF], nV[PF], nP[PF], nr[PF], ne[PF];
#pragma unroll
        for (int q = 0; q < PF; ++q) {
            const int i = i0 + PF + q;
            const bool ok = valid && i < n;
            const size_t o = (size_t)i * ld;
            nU[q] = ok ? Up[o * M] : 0.0; nV[q] = ok ? Vp[o * M] : 0.0; nP[q] = ok ? Pp[o * M] : 1.0;
            nr[q] = ok ? rp[o] : 0.0; ne[q] = ok ? ep[o] : 1.0;
        }
#pragma unroll
        for (int q = 0; q < PF; ++q)
            if (i0 + q < n)                                    // uniform across the warp
                epoch(i0 + q, cU[q], cV[q], cP[q], cr[q], ce[q]);
#pragma unroll
        for (int q = 0; q < PF; ++q) { cU[q] = nU[q]; cV[q] = nV[q]; cP[q] = nP[q]; cr[q] = nr[q]; ce[q] = ne[q]; }
    }
    double ll = -INFINITY;
    if (valid && !bad) {
        const double logdet = log(prod) + (double)pexp * 0.6931471805599453;
        ll = -0.5 * (quad + logdet) + md->loglike_const;
        if (!isfinite(ll)) ll = -INFINITY;
    }
    gp_finish<M>(A, row, k, live, valid, lp, th, ll);
}

// FP64 residual rows of a caller to the float-float pairs of k_gp_fused
static __global__ void __launch_bounds__(256) k_gp_cvt(const double* r, const double* e, float2* ro, float2* eo,
                                                 size_t count) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
        const FF a = ff_split(r[i]), b = ff_split(e[i]);
        ro[i] = make_float2(a.hi, a.lo);
        eo[i] = make_float2(b.hi, b.lo);
    }
}


// The mixed precision's preparation and recursion in one CTA: warps 1..3
// compute U, V and phi (sincos and exp in float-float after an FP64 argument
// reduction) and stage the residuals of the next chunk of kGPChunk epochs in
// shared memory while warp 0 runs the recursion in float-float arithmetic
// (~2^-46 relative per operation; FP32 instructions issue ~60 times as fast
// as FP64 ones on this GPU) on the current chunk, so the U, V, phi rows never
// go through device memory and the transcendentals stay off the recursion's
// dependent chain.
constexpr int kGPChunk = 16;
constexpr int kGPProducers = 3;                   // producer warps per CTA

template <int M>
__global__ void __launch_bounds__(32 * (1 + kGPProducers)) k_gp_fused(KArgs A0) {
    const KArgs A = gp_system<M>(A0, blockIdx.y);
    constexpr int R = 32 / M;                     // rows per CTA (one warp of the recursion)
    constexpr int E = kGPChunk;
    static_assert(M >= 2 && M <= 32, "the per-dimension bit masks hold 32 dimensions");
    static_assert((M & (M - 1)) == 0, "a row's lanes are lane & (M - 1)");
    __shared__ float2 sU[2][E][32], sV[2][E][32], sP[2][E][32];
    __shared__ float2 sr[2][E][R], se[2][E][R];
    __shared__ double s_c[R][M], s_d[R][M], s_asum[R];
    __shared__ float2 s_a[R][M], s_b[R][M];
    __shared__ unsigned s_ps[R], s_pv[R];         // bit k: dimension k is a sine part / is live
    __shared__ int s_on[R];                       // the row's inputs are computed (else neutral)
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ptid = threadIdx.x - 32;            // producer thread index (warps 1..)
    const int row0 = blockIdx.x * R;
    const int n = A.d.n;
    const size_t ld = (size_t)A.nwalk;
    const int nch = (n + E - 1) / E;

    // ---- producer: row constants, then the chunks ahead of the recursion
    auto fill = [&](int c, int b) {
        for (int task = ptid; task < E * R; task += 32 * kGPProducers) {
            const int e = task / R, rr = task - e * R;
            const int i = c * E + e;
            const int row = min(row0 + rr, A.nwalk - 1);
            const unsigned fps = s_ps[rr], fpv = s_pv[rr];
            const bool on = i < n && s_on[rr] != 0;
            if (on) {
                const double ti = A.d.t[i];
                const double dt = i > 0 ? ti - A.d.t[i - 1] : 0.0;
                FF sn[M], cs[M], ph[M];
#pragma unroll
                for (int k = 0; k < M; ++k) {
                    const bool ps = fps >> k & 1u, pv = fpv >> k & 1u;
                    const double pc = s_c[rr][k], pd = s_d[rr][k];
                    if (k > 0 && ps) { sn[k] = sn[k - 1]; cs[k] = cs[k - 1]; ph[k] = ph[k - 1]; }
                    else {
                        if (pd != 0.0) ff_sincos(pd * ti, sn[k], cs[k]);
                        else { sn[k] = FF{0.f, 0.f}; cs[k] = FF{1.f, 0.f}; }
                        ph[k] = pc != 0.0 ? ff_exp_neg(pc * dt) : FF{1.f, 0.f};
                    }
                    const FF fa = ff_of(s_a[rr][k]), fb = ff_of(s_b[rr][k]);
                    const FF u = ps ? ff_add(ff_mul(fa, sn[k]), ff_neg(ff_mul(fb, cs[k])))
                                    : ff_add(ff_mul(fa, cs[k]), ff_mul(fb, sn[k]));
                    const FF v = pv ? (ps ? sn[k] : cs[k]) : FF{0.f, 0.f};
                    sU[b][e][rr * M + k] = make_float2(u.hi, u.lo);
                    sV[b][e][rr * M + k] = make_float2(v.hi, v.lo);
                    sP[b][e][rr * M + k] = make_float2(ph[k].hi, ph[k].lo);
                }
                const size_t o = (size_t)i * ld + row;
                sr[b][e][rr] = reinterpret_cast<const float2*>(A.gp_r)[o];
                se[b][e][rr] = reinterpret_cast<const float2*>(A.gp_e)[o];
            } else {
#pragma unroll
                for (int k = 0; k < M; ++k) {
                    sU[b][e][rr * M + k] = make_float2(0.f, 0.f);
                    sV[b][e][rr * M + k] = make_float2(0.f, 0.f);
                    sP[b][e][rr * M + k] = make_float2(1.f, 0.f);
                }
                sr[b][e][rr] = make_float2(0.f, 0.f);
                se[b][e][rr] = make_float2(1.f, 0.f);
            }
        }
    };
    if (warp >= 1 && ptid < R) {
        {
            const int lane = ptid;
            const int rowr = row0 + lane;
            const bool live = rowr < A.nwalk;
            const int row = live ? rowr : A.nwalk - 1;
            const double* th;
            const double lp = gp_row(A, row, &th);
            GPDim dm[M];
#pragma unroll
            for (int k = 0; k < M; ++k) dm[k] = GPDim{0.0, 0.0, 0.0, 0.0, 0, 0};
            bool finite = true;
            double asum = 0.0;
            unsigned fps = 0u, fpv = 0u;
            if (lp > -INFINITY) {
                gp_fill(A.md, th, dm);
#pragma unroll
                for (int k = 0; k < M; ++k) {
                    if (!dm[k].sinpart) asum += dm[k].a;
                    finite = finite && isfinite(dm[k].a) && isfinite(dm[k].b) && isfinite(dm[k].c) &&
                             isfinite(dm[k].d);
                }
            }
#pragma unroll
            for (int k = 0; k < M; ++k) {
                s_c[lane][k] = dm[k].c;
                s_d[lane][k] = dm[k].d;
                s_a[lane][k] = ff_split_bits(dm[k].a);
                s_b[lane][k] = ff_split_bits(dm[k].b);
                fps |= (dm[k].sinpart ? 1u : 0u) << k;
                fpv |= (dm[k].live ? 1u : 0u) << k;
            }
            s_ps[lane] = fps;
            s_pv[lane] = fpv;
            s_on[lane] = (lp > -INFINITY && finite) ? 1 : 0;
            s_asum[lane] = finite ? asum : NAN;
        }
    }
    __syncthreads();
    if (warp >= 1) fill(0, 0);
    __syncthreads();

    // ---- consumer: the recursion on the staged chunks; the sums across a
    // row's lanes are broadcast from lane 0 so that every lane holds the same
    // D and z
    const int k = lane & (M - 1);
    const int rl = lane / M;
    const int rowr = row0 + rl;
    const bool live = rowr < A.nwalk;
    const int row = live ? rowr : A.nwalk - 1;
    const emp_model_desc* md = A.md;
    const double* th = nullptr;
    double lp = -INFINITY;
    bool valid = false;
    double asum_d = 0.0;
    FF asum{0.f, 0.f};
    FF S[M];
#pragma unroll
    for (int j = 0; j < M; ++j) S[j] = FF{0.f, 0.f};
    FF f{0.f, 0.f}, W{0.f, 0.f}, Dp{0.f, 0.f}, zp{0.f, 0.f}, quad{0.f, 0.f}, prod{1.f, 0.f};
    int pexp = 0;
    bool bad = false;
    if (warp == 0) {
        lp = gp_row(A, row, &th);
        valid = live && (lp > -INFINITY);
        asum_d = valid ? s_asum[rl] : 0.0;
        asum = ff_split(isfinite(asum_d) ? asum_d : 0.0);
        bad = !isfinite(asum_d);
    }
    auto epoch = [&](int i, FF Uk, FF Vk, FF Pk, FF ri, FF ei) {
        FF Uj[M];
#pragma unroll
        for (int j = 0; j < M; ++j) Uj[j] = ff_shfl(Uk, j, M);
        if (i > 0) {
            const FF dw = ff_mul(Dp, W);
#pragma unroll
            for (int j = 0; j < M; ++j) {
                const FF Wj = ff_shfl(W, j, M);
                const FF pj = ff_shfl(Pk, j, M);
                S[j] = ff_mul(ff_mul(Pk, pj), ff_add(ff_mul(dw, Wj), S[j]));
            }
            f = ff_mul(Pk, ff_add(ff_mul(W, zp), f));
        }
        FF t[M];
#pragma unroll
        for (int j = 0; j < M; ++j) t[j] = ff_mul(S[j], Uj[j]);
#pragma unroll
        for (int w = 1; w < M; w <<= 1)
#pragma unroll
            for (int j = 0; j + w < M; j += 2 * w) t[j] = ff_add(t[j], t[j + w]);
        const FF su = t[0];
        FF p1 = ff_mul(Uk, su), p2 = ff_mul(Uk, f);
#pragma unroll
        for (int off = M / 2; off >= 1; off >>= 1) {
            p1 = ff_add(p1, ff_shfl_xor(p1, off, M));
            p2 = ff_add(p2, ff_shfl_xor(p2, off, M));
        }
        p1 = ff_shfl(p1, 0, M);
        p2 = ff_shfl(p2, 0, M);
        const FF D = ff_add(ff_add(ei, asum), ff_neg(p1));
        bad = bad || !(D.hi > 0.f);
        const FF iD = ff_recip(D);
        W = ff_mul(ff_add(Vk, ff_neg(su)), iD);
        const FF z = ff_add(ri, ff_neg(p2));
        quad = ff_add(quad, ff_mul(ff_mul(z, z), iD));
        prod = ff_mul(prod, D);
        {
            const int ex = ((__float_as_int(prod.hi) >> 23) & 0xff) - 127;
            const float sc = __int_as_float((127 - ex) << 23);
            pexp += ex;
            prod.hi *= sc;
            prod.lo *= sc;
        }
        Dp = D; zp = z;
    };
    for (int c = 0; c < nch; ++c) {
        const int b = c & 1;
        if (warp >= 1) {
            if (c + 1 < nch) fill(c + 1, b ^ 1);
        } else {
            for (int e = 0; e < E; ++e) {
                const int i = c * E + e;
                if (i >= n) break;                            // uniform across the warp
                epoch(i, ff_of(sU[b][e][lane]), ff_of(sV[b][e][lane]), ff_of(sP[b][e][lane]),
                      ff_of(sr[b][e][rl]), ff_of(se[b][e][rl]));
            }
        }
        __syncthreads();
    }
    if (warp != 0) return;
    double ll = -INFINITY;
    if (valid && !bad) {
        const double q = (double)quad.hi + (double)quad.lo;
        const double logdet = log((double)prod.hi + (double)prod.lo) + (double)pexp * 0.6931471805599453;
        ll = -0.5 * (q + logdet) + md->loglike_const;
        if (!isfinite(ll)) ll = -INFINITY;
    }
    gp_finish<M>(A, row, k, live, valid, lp, th, ll);
}

}  // namespace emp
