// emp_kernels.cuh -- the log-posterior / stretch-move kernel template.
//
// Template parameters
//   PREC : EMP_PREC_FP64 or EMP_PREC_MIXED
//   Q    : moving-average order evaluated (0..3)
//   L    : lanes per walker (8..256, power of two)
//   NT   : threads per CTA (multiple of L and of 32)
//
// Per walker the kernel restates, in this order,
//   my_prior   (emp.py:190-251),
//   my_model   (emp_model.py:706-781: Keplerians kep0*.model, acc.model,
//               offset00.model, jitter00.model, moav01/moav00 recurrence),
//   my_likelihood (support/likelihoods/00.like:3-5),
// and in kModeStretch additionally the emcee stretch proposal and the
// Metropolis test of one half of a temperature's ensemble.
//
// FP64 is a scarce pipe on this GPU (a warp-wide FP64 instruction occupies
// the sub-partition's FP64 unit for tens of cycles), so the per-walker
// prologue of the mixed kernel keeps FP64 to the few operations whose
// rounding must match the reference: the stretch proposal, e = S^2 + C^2,
// exp of log-periods, the varying prior terms and the final sums.  Bounds
// of priors are compared exactly on the integer pipe.
#pragma once
#include <type_traits>
#include "emp_device.cuh"

namespace emp {

// ----------------------------------------------------------------------------
// exact double comparisons on the integer pipe
// ----------------------------------------------------------------------------
__device__ __forceinline__ long long dkey(double x) {
    long long b = __double_as_longlong(x);
    if (b == (long long)0x8000000000000000ULL) b = 0;          // -0.0 == +0.0
    return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ bool d_isnan(double x) {
    return (__double_as_longlong(x) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL;
}
// lo <= x <= hi as IEEE comparisons (false for NaN)
__device__ __forceinline__ bool in_support(double x, double lo, double hi) {
    if (d_isnan(x)) return false;
    const long long k = dkey(x);
    return k >= dkey(lo) && k <= dkey(hi);
}

// the prior terms with FP64 transcendentals, out of line (rare; keeps the
// kernels' code small)
static __device__ __noinline__ double prior_var_term_rare(const emp_prior& p, double x) {
    if (p.kind == EMP_PRIOR_BETA) return (p.a0 - 1.0) * log(x) + (p.a1 - 1.0) * log1p(-x) - p.a2;
    if (p.kind == EMP_PRIOR_ISOTROPIC) return log(0.5 * sin(x)) - p.a0;
    return 0.0;
}
// value of a prior term that varies with x (Normal, Beta); x in support
__device__ __forceinline__ double prior_var_term(const emp_prior& p, double x) {
    if (p.kind == EMP_PRIOR_NORMAL) {
        const double z = (x - p.a0) * p.a1;                // a1 = 1/s
        return -0.5 * z * z - p.a2;
    }
    return prior_var_term_rare(p, x);
}

// priors whose value varies with the parameter (the others are constants
// summed on the host)
__device__ __forceinline__ bool prior_varies(int kind) {
    return kind == EMP_PRIOR_NORMAL || kind == EMP_PRIOR_BETA || kind == EMP_PRIOR_ISOTROPIC;
}

__device__ __forceinline__ double derived_x(const double* th, int k) {
    return k == 0 ? th[3] * th[3] + th[4] * th[4] : th[1] * th[1] + th[2] * th[2];
}

// Hill stability priors (FP64, one thread).  The reference gives every
// Keplerian block after the first its own Hill prior over the planets up to
// and including it (block_repo.py:611-626 runs per block; the flag that would
// stop the repetition is only set in a local copy), so the prior is -inf
// unless, for every j in md->hill_mask, the first j Keplerians pass
// support/priors/Hill.prior: ordered by semi-major axis, each adjacent pair
// needs LHS > RHS.  Semi-major axes and minimum masses follow math_utils.py:31-61
// (cps); (P, K, e) are read per parameterisation as support/PAE/0*.pae reads
// them.  As in the reference, gamma = sqrt(1 - e) keeps the planets' own
// order while the masses and axes are sorted.  Not inlined: its dynamically
// indexed arrays would otherwise take the log-posterior kernels' registers.
static __device__ __noinline__ bool hill_stable(const emp_model_desc* md, const double* full) {
    const int mask = md->hill_mask;
    int K = 0;
    for (int j = 2; j <= EMP_MAX_PLANETS; ++j)
        if (mask & (1 << j)) K = j;
    const double Ms = md->hill_starmass;
    const double kPi = 3.141592653589793;
    double sma[EMP_MAX_PLANETS], mm[EMP_MAX_PLANETS], gam[EMP_MAX_PLANETS];
    for (int p = 0; p < K; ++p) {
        const double* v = full + md->kep_slot[p];
        const int par = md->kep_param[p];
        double P = v[0], Kp = v[1];
        if (par == 2 || par == 6) P = exp(v[0]);
        if (par == 2) Kp = v[1] * v[1] + v[2] * v[2];
        const double e = (par == 0 || par == 3 || par == 6) ? v[3] : v[3] * v[3] + v[4] * v[4];
        const double Ps = P * 86400.0;
        const double a = pow(6.6743e-11 * (Ms * 1.98847e30) * (Ps * Ps) / (4.0 * (kPi * kPi)), 1.0 / 3.0) /
                         1.495978707e11;
        sma[p] = a;
        mm[p] = (Kp / 28.4329) * sqrt(1.0 - e * e) * sqrt(Ms * a);
        gam[p] = sqrt(1.0 - e);
    }
    for (int j = 2; j <= K; ++j) {
        if (!(mask & (1 << j))) continue;
        int idx[EMP_MAX_PLANETS];
        for (int p = 0; p < j; ++p) idx[p] = p;
        for (int i = 1; i < j; ++i)                      // order by semi-major axis
            for (int q = i; q > 0 && sma[idx[q]] < sma[idx[q - 1]]; --q) {
                const int t = idx[q]; idx[q] = idx[q - 1]; idx[q - 1] = t;
            }
        double Mt = 0.0;
        for (int p = 0; p < j; ++p) Mt += mm[idx[p]];
        Mt = Ms * 1047.56 + Mt;
        for (int i = 0; i + 1 < j; ++i) {
            const double m0 = mm[idx[i]] / Mt, m1 = mm[idx[i + 1]] / Mt;
            const double alpha = m0 + m1;
            const double delta = sqrt(sma[idx[i + 1]] / sma[idx[i]]);
            const double s = m0 * gam[i] + m1 * gam[i + 1] * delta;
            const double lhs = pow(alpha, -3.0) * (m0 + m1 / (delta * delta)) * (s * s);
            const double rhs = 1.0 + pow(3.0 / alpha, 4.0 / 3.0) * (m0 * m1);
            if (!(lhs > rhs)) return false;
        }
    }
    return true;
}

// ----------------------------------------------------------------------------
// float-float helpers (mixed precision phase)
// ----------------------------------------------------------------------------
struct FF { float hi, lo; };

__device__ __forceinline__ FF ff_split(double x) {
    FF r;
    r.hi = (float)x;
    r.lo = (float)(x - (double)r.hi);
    return r;
}
// a * b with a, b float-float, |error| ~ 2^-46 |ab|
__device__ __forceinline__ FF ff_mul(FF a, FF b) {
    const float p = __fmul_rn(a.hi, b.hi);
    const float e = __fmaf_rn(a.hi, b.hi, -p);
    FF r;
    r.hi = p;
    r.lo = e + __fmaf_rn(a.hi, b.lo, __fmul_rn(a.lo, b.hi));
    return r;
}
// x - rint(x) of a float-float, normalised to |hi| <= 0.5
__device__ __forceinline__ FF ff_frac(FF a) {
    const float n = rintf(a.hi);
    const float h = __fsub_rn(a.hi, n);               // exact
    const float s = __fadd_rn(h, a.lo);
    const float n2 = rintf(s);
    const float s2 = __fsub_rn(s, n2);
    FF r;
    r.hi = s2;
    r.lo = __fsub_rn(a.lo, __fsub_rn(__fadd_rn(s2, n2), h));   // fast two-sum tail
    return r;
}
// 1/x in float-float (one reciprocal and a residual correction)
__device__ __forceinline__ FF ff_recip(FF x) {
    const float r = __frcp_rn(x.hi);
    float e = __fmaf_rn(-x.hi, r, 1.0f);
    e = __fmaf_rn(-x.lo, r, e);
    FF o;
    o.hi = r;
    o.lo = __fmul_rn(r, e);
    return o;
}

// fast two-sum: hi + lo renormalised (|hi| >= |lo| or hi == 0)
__device__ __forceinline__ FF ff_norm(float hi, float lo) {
    const float sum = __fadd_rn(hi, lo);
    FF r;
    r.hi = sum;
    r.lo = __fsub_rn(lo, __fsub_rn(sum, hi));
    return r;
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
    const float sum = __fadd_rn(a.hi, b.hi);
    const float bb = __fsub_rn(sum, a.hi);
    const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(sum, bb)), __fsub_rn(b.hi, bb));
    return ff_norm(sum, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}
// 1/sqrt(x), x > 0: hardware estimate and one Newton step on the exact
// residual 1 - x r0^2 (relative error ~1e-14)
__device__ __forceinline__ FF ff_rsqrt(FF x) {
    const float r0 = rsqrtf(x.hi);
    const float t = __fmul_rn(r0, r0);
    const float te = __fmaf_rn(r0, r0, -t);
    FF q = ff_mul(x, FF{t, te});
    const float h = __fsub_rn(__fsub_rn(1.f, q.hi), q.lo);
    return ff_norm(r0, __fmul_rn(__fmul_rn(0.5f, r0), h));
}
// sqrt(x), x >= 0, the same way
__device__ __forceinline__ FF ff_sqrt(FF x) {
    if (!(x.hi > 0.f)) return FF{0.f, 0.f};
    const float s0 = x.hi * rsqrtf(x.hi);
    const float t = __fmul_rn(s0, s0);
    const float te = __fmaf_rn(s0, s0, -t);
    const float d = __fadd_rn(__fsub_rn(__fsub_rn(x.hi, t), te), x.lo);
    return ff_norm(s0, __fmul_rn(d, __fdividef(0.5f, s0)));
}

// ----------------------------------------------------------------------------
// per-planet constants
// ----------------------------------------------------------------------------
// FP64: [0]=freq [1]=phase [2]=e [3]=K cw [4]=K sqrt(1-e^2) sw [5]=K e cw [6]=tp [7]=use_tp
__device__ __forceinline__ void planet_consts_fp64(int par, const double* v, double* pc) {
    Elements el = planet_elements(par, v);
    const double freq = 2. * kPi / el.per;                   // kep01.model:11
    pc[0] = freq;
    pc[1] = el.phase;
    pc[2] = el.e;
    pc[3] = el.K * el.cw;
    pc[4] = el.K * sqrt(1.0 - el.e * el.e) * el.sw;
    pc[5] = el.K * el.e * el.cw;
    pc[6] = el.tp;
    pc[7] = (double)el.use_tp;
}

// planet_consts_mixed for parameterisations 0, 1, 3 and 4 from float-float
// copies of the planet's slots (vh + vl = the FP64 values to ~2^-48): the
// same constants in FP32 float-float arithmetic, without FP64 operations
__device__ __forceinline__ void planet_consts_mixed_ff(int par, const float* vh, const float* vl, float* pc) {
    FF per{vh[0], vl[0]}, K{vh[1], vl[1]}, x2{vh[2], vl[2]};
    FF e{0.f, 0.f}, cw{1.f, 0.f}, sw{0.f, 0.f};
    if (par >= EMP_TERM_SINUSOID) {
        // cosine terms: e = 0 Keplerians (period doubled exactly for the
        // first magnetic-cycle term)
        if (par == EMP_TERM_CYCLE_1) { per.hi *= 2.f; per.lo *= 2.f; }
        if (par == EMP_TERM_CYCLE_2) K = FF{vh[2], vl[2]};
        if (par == EMP_TERM_CYCLE_1) x2 = FF{vh[3], vl[3]};
        if (par == EMP_TERM_CYCLE_2) x2 = FF{vh[4], vl[4]};
    } else if (par == 0 || par == 3) {
        e = FF{vh[3], vl[3]};
        float s32, c32;
        sincosf(vh[4], &s32, &c32);
        sw.hi = s32;
        cw.hi = c32;
    } else {
        const FF S{vh[3], vl[3]}, C{vh[4], vl[4]};
        e = ff_add(ff_mul(S, S), ff_mul(C, C));
        // e >= 1e-6 (1e-5 for parameterisation 4) against the float-float
        // split of the FP64 threshold
        const float th = par == 4 ? 9.999999747378752e-06f : 9.999999974752427e-07f;
        const float tl = par == 4 ? 2.526212474884132e-13f : 2.5247572468697606e-15f;
        if (e.hi > th || (e.hi == th && e.lo >= tl)) {
            const FF rs = ff_rsqrt(e);
            cw = ff_mul(C, rs);
            sw = ff_mul(S, rs);
        }
    }
    const FF sq = ff_sqrt(ff_add(FF{1.f, 0.f}, ff_mul(FF{-e.hi, -e.lo}, e)));
    const FF f = ff_recip(per);
    FF ph;
    if (par == 3 || par == 4) {
        FF q = ff_mul(x2, f);
        q.hi = -q.hi; q.lo = -q.lo;
        ph = ff_frac(q);
    } else {
        const FF inv2pi = {0.15915493667125702f, 6.4206382432985265e-09f};   // 1/(2 pi) as float-float
        ph = ff_frac(ff_mul(x2, inv2pi));
    }
    pc[0] = f.hi;
    pc[1] = f.lo;
    pc[2] = ph.hi;
    pc[3] = ph.lo;
    const FF en = ff_norm(e.hi, e.lo);
    const FF A = ff_mul(K, cw);
    const FF An = ff_norm(A.hi, A.lo);
    const FF Bn = [&] { const FF b = ff_mul(ff_mul(K, sq), sw); return ff_norm(b.hi, b.lo); }();
    const FF Cn = [&] { const FF c = ff_mul(A, en); return ff_norm(c.hi, c.lo); }();
    pc[4] = en.hi;  pc[8] = en.lo;
    pc[5] = An.hi;  pc[9] = An.lo;
    pc[6] = Bn.hi;  pc[10] = Bn.lo;
    pc[7] = Cn.hi;  pc[11] = Cn.lo;
    const float ef = pc[4];
    const float den = __fdividef(1.f, 4.f * ef + 0.5f);
    const float a = (1.f - ef) * den;
    pc[12] = a;
    pc[13] = a * a * a;
    pc[14] = 0.5f * den;
    pc[15] = __fdividef(0.078f, 1.f + ef);
}

// 1/sqrt(x) and sqrt(x) to ~1e-14: FP32 estimate, one FP64 Newton step
// (two or three FP64 operations instead of a full FP64 square root)
__device__ __forceinline__ double rsqrt_refined(double x) {
    const double r0 = (double)rsqrtf((float)x);
    return r0 * fma(-0.5 * x * r0, r0, 1.5);
}
__device__ __forceinline__ double sqrt_refined(double x) {
    const float s0 = sqrtf((float)x);
    if (!(s0 > 0.f)) return 0.0;
    return fma(fma(-(double)s0, (double)s0, x), (double)(0.5f / s0), (double)s0);
}

__device__ __forceinline__ void split_ff(double x, float& hi, float& lo) {
    hi = (float)x;
    lo = (float)(x - (double)hi);
}

// mixed: [0]=f_hi [1]=f_lo (cycles/day) [2]=ph_hi [3]=ph_lo (cycles)
//        [4]=e [5]=A=K cw [6]=B=K sqrt(1-e^2) sw [7]=C=K e cw, and [8..11]
//        the low parts of e, A, B, C: the constants are formed in FP64 and
//        kept as float-float pairs, so their rounding adds no systematic
//        error to the model (a rounded constant shifts every epoch alike)
static __device__ __noinline__ void planet_consts_mixed(int par, const double* v, float* pc) {
    double per, K, e = 0.0, cw = 1.0, sw = 0.0;
    bool use_tp = false;
    double phase = 0.0, tp = 0.0;
    if (par == 0 || par == 3 || par == 6) {
        per = par == 6 ? exp(v[0]) : v[0];
        K = v[1];
        e = v[3];
        float s32, c32;
        sincosf((float)v[4], &s32, &c32);
        sw = s32;
        cw = c32;
        if (par == 3) { use_tp = true; tp = v[2]; } else { phase = v[2]; }
    } else if (par == 2) {
        per = exp(v[0]);
        const float As = (float)v[1], Ac = (float)v[2];
        const float K32 = As * As + Ac * Ac;
        K = (double)K32;
        float ph = acosf(Ac * rsqrtf(K32));
        if (As < 0.f) ph = 6.28318530717958647692f - ph;
        phase = (double)ph;
    } else {
        per = par == 7 ? exp(v[0]) : v[0];
        K = v[1];
        if (par == 4) { use_tp = true; tp = v[2]; } else { phase = v[2]; }
    }
    if (par == 1 || par == 2 || par == 4 || par == 7) {
        e = v[3] * v[3] + v[4] * v[4];                      // FP64 as the reference
        const double thr = (par == 2 || par == 4) ? 1e-5 : 1e-6;
        if (e >= thr) {
            const double rs = rsqrt_refined(e);
            cw = v[4] * rs;
            sw = v[3] * rs;
        }
    }
    const double sq = sqrt_refined(fma(-e, e, 1.0));
    const FF f = ff_recip(ff_split(per));
    FF ph;
    if (use_tp) {
        FF p = ff_mul(ff_split(tp), f);
        p.hi = -p.hi; p.lo = -p.lo;
        ph = ff_frac(p);
    } else {
        const FF inv2pi = {0.15915493667125702f, 6.4206382432985265e-09f};   // 1/(2 pi) as float-float
        ph = ff_frac(ff_mul(ff_split(phase), inv2pi));
    }
    pc[0] = f.hi;
    pc[1] = f.lo;
    pc[2] = ph.hi;
    pc[3] = ph.lo;
    const double A = K * cw;
    split_ff(e, pc[4], pc[8]);
    split_ff(A, pc[5], pc[9]);
    split_ff(K * sq * sw, pc[6], pc[10]);
    split_ff(A * e, pc[7], pc[11]);
    // starter of the Kepler solve (Mikkola 1987, Celest. Mech. 40, 329)
    const float ef = pc[4];
    const float den = __fdividef(1.f, 4.f * ef + 0.5f);
    const float a = (1.f - ef) * den;
    pc[12] = a;
    pc[13] = a * a * a;
    pc[14] = 0.5f * den;
    pc[15] = __fdividef(0.078f, 1.f + ef);
}

// one Keplerian term at one epoch (FP64)
__device__ __forceinline__ double rv_term_f64(const double* pc, double t) {
    double M;
    if (pc[7] != 0.0) M = __dmul_rn(pc[0], __dsub_rn(t, pc[6]));   // kep03/04: freq*(X_-tp)
    else M = __dadd_rn(__dmul_rn(pc[0], t), pc[1]);                // kep01.model:12
    // np.remainder(M + pi, 2 pi) - pi
    double Mr = fmod(M + kPi, kTwoPi);
    if (Mr < 0.0) Mr += kTwoPi;
    Mr -= kPi;
    const double e = pc[2];
    double s, c;
    kepler_f64(Mr, e, s, c);
    // K (cos(f + w) + e cos w) with cos f = (cos E - e)/(1 - e cos E),
    // sin f = sqrt(1-e^2) sin E / (1 - e cos E)
    const double inv = 1.0 / (1.0 - e * c);
    return (pc[3] * (c - e) - pc[4] * s) * inv + pc[5];
}

// mean anomaly in [-pi, pi] from float-float time and planet constants;
// mlo receives the part of (cycles mod 1) * 2 pi that the FP32 result drops
__device__ __forceinline__ float mean_anomaly_mixed(const float* pc, float th, float tl, float& mlo) {
    // cycles = (th + tl) * (fh + fl) + (ph_hi + ph_lo), reduced mod 1; the
    // error-free transforms use _rn intrinsics so they are not contracted
    const float fh = pc[0], fl = pc[1];
    const float p = __fmul_rn(th, fh);
    const float pe = __fmaf_rn(th, fh, -p);
    const float x = __fadd_rn(p, pc[2]);                 // TwoSum(p, ph_hi)
    const float bv = __fsub_rn(x, p);
    const float xe = __fadd_rn(__fsub_rn(p, __fsub_rn(x, bv)), __fsub_rn(pc[2], bv));
    const float fr = __fsub_rn(x, rintf(x));             // exact
    const float lo = pe + xe + pc[3] + __fmaf_rn(th, fl, tl * fh);
    const float cyc0 = __fadd_rn(fr, lo);
    const float cb = __fsub_rn(cyc0, fr);                // TwoSum(fr, lo) error
    const float ce = __fadd_rn(__fsub_rn(fr, __fsub_rn(cyc0, cb)), __fsub_rn(lo, cb));
    const float cyc = __fsub_rn(cyc0, rintf(cyc0));      // exact
    const float M = __fmul_rn(cyc, 6.28318530717958647692f);
    // 2 pi = 6.2831855f - 1.7484555e-07
    mlo = __fadd_rn(__fmaf_rn(cyc, 6.28318530717958647692f, -M),
                    __fmaf_rn(cyc, -1.7484555e-07f, __fmul_rn(ce, 6.28318530717958647692f)));
    return M;
}
__device__ __forceinline__ float mean_anomaly_mixed(const float* pc, float th, float tl) {
    float mlo;
    return mean_anomaly_mixed(pc, th, tl, mlo);
}

// sin and cos of x (|x| <= ~8) to about 1 ulp without the special
// function unit: Cody-Waite reduction by pi/2 (the first part of pi/2 has
// 12 significant bits, so q * C1 and x - q * C1 are exact for |q| <= 4),
// Taylor polynomials of degree 9 (sin) and 10 (cos) on |r| <= pi/4
// (truncation below 2e-9), and the quadrant rotation.
__device__ __forceinline__ void sincos_acc(float x, float& s, float& c) {
    const float q = rintf(__fmul_rn(x, 0.636619772367581343f));
    float r = __fmaf_rn(-q, 1.5703125f, x);
    r = __fmaf_rn(-q, 4.83826794896619231e-04f, r);
    r = __fmaf_rn(-q, 2.56328273e-12f, r);
    const float r2 = __fmul_rn(r, r);
    float ps = __fmaf_rn(r2, 2.75573192e-06f, -1.98412698e-04f);
    ps = __fmaf_rn(r2, ps, 8.33333333e-03f);
    ps = __fmaf_rn(r2, ps, -1.66666667e-01f);
    const float sr = __fmaf_rn(__fmul_rn(r2, r), ps, r);
    float pc = __fmaf_rn(r2, -2.75573192e-07f, 2.48015873e-05f);
    pc = __fmaf_rn(r2, pc, -1.38888889e-03f);
    pc = __fmaf_rn(r2, pc, 4.16666667e-02f);
    pc = __fmaf_rn(r2, pc, -0.5f);
    const float cr = __fmaf_rn(r2, pc, 1.f);
    const int qi = (int)q;
    const float ss = (qi & 1) ? cr : sr;
    const float cc = (qi & 1) ? sr : cr;
    s = (qi & 2) ? -ss : ss;
    c = ((qi + 1) & 2) ? -cc : cc;
}

// NE independent FP32 Kepler solves of E - (e + elo) sin E = M + mlo:
// second-order series start, joint Halley iterations with the special
// function unit's sin/cos until every |dE| < 1e-3, then one Newton step
// whose residual uses sincos_acc, an error-free E - M and the low parts of
// M and e; (sin E, cos E) are rotated by that step.  The hardware sin/cos
// (absolute error ~4e-7) only steer the iterations: the converged E is off
// by at most ~2e-6, which the Newton step reduces below 1e-11.
template <int NE>
__device__ __forceinline__ void kepler_f32_n(const float (&M)[NE], const float (&mlo)[NE], float e,
                                             float elo, float (&s)[NE], float (&c)[NE]) {
    float E[NE];
#pragma unroll
    for (int k = 0; k < NE; ++k) {
        float sM, cM;
        __sincosf(M[k], &sM, &cM);
        E[k] = M[k] + e * sM * (1.f + e * cM);
    }
#pragma unroll 1
    for (int it = 0; it < 16; ++it) {
        bool more = false;
#pragma unroll
        for (int k = 0; k < NE; ++k) {
            float sk, ck;
            __sincosf(E[k], &sk, &ck);
            const float f = E[k] - e * sk - M[k];
            const float f1 = 1.f - e * ck;
            const float f2 = e * sk;
            const float d = __fdividef(f * f1, f1 * f1 - 0.5f * f * f2);
            E[k] -= d;
            more |= fabsf(d) >= 1e-3f;
        }
        if (!more) break;
    }
#pragma unroll
    for (int k = 0; k < NE; ++k) {
        float sa, ca;
        sincos_acc(E[k], sa, ca);
        // E - M as an exact float pair (TwoSum)
        const float dh = __fsub_rn(E[k], M[k]);
        const float bv = __fsub_rn(dh, E[k]);
        const float dl = __fadd_rn(__fsub_rn(E[k], __fsub_rn(dh, bv)), __fsub_rn(-M[k], bv));
        // F = E - M - mlo - (e + elo) sin E; e sin E nearly cancels dh
        float F = __fmaf_rn(-e, sa, dh);
        F = __fadd_rn(F, __fmaf_rn(-elo, sa, __fsub_rn(dl, mlo[k])));
        const float f1 = __fmaf_rn(-elo, ca, __fmaf_rn(-e, ca, 1.f));
        const float d = __fdividef(F, f1);
        const float d2 = d * d;
        const float cd = 1.f - 0.5f * d2;
        const float sd = d * (1.f - d2 * (1.f / 6.f));
        s[k] = __fmaf_rn(sa, cd, -ca * sd);
        c[k] = __fmaf_rn(ca, cd, sa * sd);
    }
}

// ----------------------------------------------------------------------------
// Two epochs per instruction: the same mixed-precision steps on float2 pairs
// with the packed FP32 instructions of sm_100+ (__ffma2_rn, __fadd2_rn,
// __fmul2_rn).  Each element is rounded exactly as the scalar operation
// would be; only the special-function and rounding-to-integer steps stay
// per element.
// ----------------------------------------------------------------------------
// special-function unit approximations (PTX .approx.ftz forms); used where
// the result only steers an iteration or is refined afterwards
__device__ __forceinline__ float rcp_fast(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float rsqrt_fast(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float lg2_fast(float x) {
    float r;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float ex2_fast(float x) {
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
// 1/x to about 1 ulp: the approximation and one Newton step
__device__ __forceinline__ float rcp_nr(float x) {
    const float r = rcp_fast(x);
    return __fmaf_rn(__fmaf_rn(-x, r, 1.f), r, r);
}

__device__ __forceinline__ float2 bc2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
// a - b with one rounding (the product b * -1 is exact)
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, bc2(-1.f), a); }
// nearest integer by adding and subtracting 1.5 * 2^23, two packed FP32 adds instead of two
// round-to-integer instructions (equal to rintf for |a| < 2^22; beyond, an integer within 1 of
// a, which keeps a - rint2_add(a) exact and the phase reduction correct)
__device__ __forceinline__ float2 rint2_add(float2 a) {
    const float2 m = make_float2(12582912.f, 12582912.f);
    return __fadd2_rn(__fadd2_rn(a, m), make_float2(-12582912.f, -12582912.f));
}
__device__ __forceinline__ float2 rcp_approx2(float2 a) { return make_float2(rcp_fast(a.x), rcp_fast(a.y)); }
// 1/a to about 1 ulp per element
__device__ __forceinline__ float2 rcp_nr2(float2 a) {
    const float2 r = rcp_approx2(a);
    return __ffma2_rn(__ffma2_rn(make_float2(-a.x, -a.y), r, make_float2(1.f, 1.f)), r, r);
}

// mean_anomaly_mixed on a pair of epochs
__device__ __forceinline__ float2 mean_anomaly_pair(const float* pc, float2 th, float2 tl, float2& mlo) {
    const float2 fh = bc2(pc[0]), ph = bc2(pc[2]);
    const float2 p = mul2(th, fh);
    const float2 pe = fma2(th, fh, make_float2(-p.x, -p.y));
    const float2 x = add2(p, ph);
    const float2 bv = sub2(x, p);
    const float2 xe = add2(sub2(p, sub2(x, bv)), sub2(ph, bv));
    const float2 fr = sub2(x, rint2_add(x));
    const float2 lo = add2(add2(add2(pe, xe), bc2(pc[3])), fma2(th, bc2(pc[1]), mul2(tl, fh)));
    const float2 cyc0 = add2(fr, lo);
    const float2 cb = sub2(cyc0, fr);
    const float2 ce = add2(sub2(fr, sub2(cyc0, cb)), sub2(lo, cb));
    const float2 cyc = sub2(cyc0, rint2_add(cyc0));
    const float2 tp = bc2(6.28318530717958647692f);
    const float2 M = mul2(cyc, tp);
    mlo = add2(fma2(cyc, tp, make_float2(-M.x, -M.y)), fma2(cyc, bc2(-1.7484555e-07f), mul2(ce, tp)));
    return M;
}

// sincos_acc on a pair
__device__ __forceinline__ void sincos_acc_pair(float2 x, float2& s, float2& c) {
    // q = rint(x 2/pi) (|x| is a few radians), and its integer from the bits of x 2/pi + 1.5 * 2^23
    const float2 qm = add2(mul2(x, bc2(0.636619772367581343f)), bc2(12582912.f));
    const float2 q = add2(qm, bc2(-12582912.f));
    float2 r = fma2(q, bc2(-1.5703125f), x);
    r = fma2(q, bc2(-4.83826794896619231e-04f), r);
    r = fma2(q, bc2(-2.56328273e-12f), r);
    const float2 r2 = mul2(r, r);
    float2 ps = fma2(r2, bc2(2.75573192e-06f), bc2(-1.98412698e-04f));
    ps = fma2(r2, ps, bc2(8.33333333e-03f));
    ps = fma2(r2, ps, bc2(-1.66666667e-01f));
    const float2 sr = fma2(mul2(r2, r), ps, r);
    float2 pc = fma2(r2, bc2(-2.75573192e-07f), bc2(2.48015873e-05f));
    pc = fma2(r2, pc, bc2(-1.38888889e-03f));
    pc = fma2(r2, pc, bc2(4.16666667e-02f));
    pc = fma2(r2, pc, bc2(-0.5f));
    const float2 cr = fma2(r2, pc, bc2(1.f));
    const int qx = __float_as_int(qm.x) - 0x4B400000, qy = __float_as_int(qm.y) - 0x4B400000;
    float ssx = (qx & 1) ? cr.x : sr.x, ccx = (qx & 1) ? sr.x : cr.x;
    float ssy = (qy & 1) ? cr.y : sr.y, ccy = (qy & 1) ? sr.y : cr.y;
    s = make_float2((qx & 2) ? -ssx : ssx, (qy & 2) ? -ssy : ssy);
    c = make_float2(((qx + 1) & 2) ? -ccx : ccx, ((qy + 1) & 2) ? -ccy : ccy);
}

// Kepler's equation E - (e + elo) sin E = M + mlo on NP pairs of epochs,
// without iteration.  Start: Mikkola's cubic approximation (Mikkola 1987,
// Celest. Mech. 40, 329: with a = (1 - e)/(4 e + 1/2), b = M/2/(4 e + 1/2),
// z = cbrt(b + sign(b) sqrt(b^2 + a^3)), s = z - a/z corrected by
// -0.078 s^5/(1 + e), E0 = M + e (3 s - 4 s^3)); its error is below 4e-3
// for e < 0.99.  One Halley step on a residual that uses sincos_acc, an
// error-free E0 - M and the low parts of M and e then leaves an error
// below 5e-9 (cubic convergence); (sin E, cos E) are the accurate values at
// E0 rotated by the step.  kc = the planet's [a, a^3, 1/2/(4e+1/2),
// 0.078/(1+e)].
template <int NP>
__device__ __forceinline__ void kepler_pairs(const float2 (&M)[NP], const float2 (&mlo)[NP], float e,
                                             float elo, const float* kc, float2 (&s)[NP],
                                             float2 (&c)[NP]) {
    const float2 ev = bc2(e), nev = bc2(-e), one = bc2(1.f), nelo = bc2(-elo);
    const float ka = kc[0];
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        const float2 b = mul2(M[k], bc2(kc[2]));
        const float2 x = fma2(b, b, bc2(kc[1]));                   // > 0: a > 0 for e < 1
        float2 t, z;
        t.x = b.x + copysignf(x.x * rsqrt_fast(x.x), b.x);
        t.y = b.y + copysignf(x.y * rsqrt_fast(x.y), b.y);
        z.x = copysignf(ex2_fast(lg2_fast(fabsf(t.x)) * (1.f / 3.f)), t.x);
        z.y = copysignf(ex2_fast(lg2_fast(fabsf(t.y)) * (1.f / 3.f)), t.y);
        float2 sm = sub2(z, mul2(bc2(ka), rcp_approx2(z)));
        float2 s2 = mul2(sm, sm);
        sm = fma2(mul2(mul2(bc2(-kc[3]), s2), s2), sm, sm);
        s2 = mul2(sm, sm);
        const float2 E0 = fma2(mul2(ev, sm), fma2(bc2(-4.f), s2, bc2(3.f)), M[k]);
        float2 sa, ca;
        sincos_acc_pair(E0, sa, ca);
        // residual E0 - M - mlo - (e + elo) sin E0 with E0 - M exact
        const float2 dh = sub2(E0, M[k]);
        const float2 bv = sub2(dh, E0);
        const float2 dl = sub2(sub2(E0, sub2(dh, bv)), add2(M[k], bv));
        float2 f = fma2(nev, sa, dh);
        f = add2(f, fma2(nelo, sa, sub2(dl, mlo[k])));
        const float2 f1 = fma2(nelo, ca, fma2(nev, ca, one));
        const float2 f2 = mul2(ev, sa);
        const float2 den = fma2(mul2(bc2(-0.5f), f), f2, mul2(f1, f1));
        const float2 d = mul2(mul2(f, f1), rcp_approx2(den));
        const float2 d2 = mul2(d, d);
        const float2 cd = fma2(bc2(-0.5f), d2, one);
        const float2 sd = d;      // |d| <= 4e-3: the d^3/6 term is below 1.1e-8
        s[k] = fma2(mul2(ca, sd), bc2(-1.f), mul2(sa, cd));
        c[k] = fma2(sa, sd, mul2(ca, cd));
    }
}

// reference arithmetic: ((ndim-1) ln z + nlp) - cur > ln u (out of line: rare)
static __device__ __noinline__ bool metropolis_fp64(double nlp, double cur, double z, int dm1, double u) {
    return __dsub_rn(__dadd_rn(__dmul_rn((double)dm1, log(z)), nlp), cur) > log(u);
}
// log u < x with FP32 logarithms; inside a guard band the FP64 values decide
__device__ __forceinline__ bool metropolis(double nlp, double cur, double z, int dm1, uint32_t uword) {
    const double u = u32u(uword);
    const float lz = __logf((float)z);
    const float lu = __logf((float)u);
    const float a = (float)(nlp - cur);
    const float m = a + (float)dm1 * lz - lu;
    const float guard = 1e-4f * (1.f + fabsf(a) + fabsf(lu) + (float)dm1 * fabsf(lz));
    if (m > guard) return true;
    if (m < -guard) return false;
    return metropolis_fp64(nlp, cur, z, dm1, u);
}

// ----------------------------------------------------------------------------
// affine maps out = G u + x of the MA state (x: NQ, G: NQ x NQ row-major)
// ----------------------------------------------------------------------------
template <typename R, int NQ>
__device__ __forceinline__ void map_identity(R* m) {
#pragma unroll
    for (int i = 0; i < NQ; ++i) {
        m[i] = R(0);
#pragma unroll
        for (int j = 0; j < NQ; ++j) m[NQ + i * NQ + j] = (i == j) ? R(1) : R(0);
    }
}
// a <- a o b  (b first, then a): (Ga Gb, Ga xb + xa)
template <typename R, int NQ>
__device__ __forceinline__ void map_compose(R* a, const R* b) {
    R o[NQ + NQ * NQ];
#pragma unroll
    for (int i = 0; i < NQ; ++i) {
        R v = a[i];
#pragma unroll
        for (int k = 0; k < NQ; ++k) v += a[NQ + i * NQ + k] * b[k];
        o[i] = v;
#pragma unroll
        for (int j = 0; j < NQ; ++j) {
            R g = R(0);
#pragma unroll
            for (int k = 0; k < NQ; ++k) g += a[NQ + i * NQ + k] * b[NQ + k * NQ + j];
            o[NQ + i * NQ + j] = g;
        }
    }
#pragma unroll
    for (int k = 0; k < NQ + NQ * NQ; ++k) a[k] = o[k];
}
// b <- a o b  (b first, then a)
template <typename R, int NQ>
__device__ __forceinline__ void map_compose_left(const R* a, R* b) {
    R o[NQ + NQ * NQ];
#pragma unroll
    for (int k = 0; k < NQ + NQ * NQ; ++k) o[k] = a[k];
    map_compose<R, NQ>(o, b);
#pragma unroll
    for (int k = 0; k < NQ + NQ * NQ; ++k) b[k] = o[k];
}
template <typename R, int NQ>
__device__ __forceinline__ void map_apply(const R* m, const R* u, R* out) {
#pragma unroll
    for (int i = 0; i < NQ; ++i) {
        R v = m[i];
#pragma unroll
        for (int k = 0; k < NQ; ++k) v += m[NQ + i * NQ + k] * u[k];
        out[i] = v;
    }
}

// ----------------------------------------------------------------------------
// lane accumulators and their group sums (FP64 plain; float-float mixed, so
// that the mixed kernel's sums need no FP64 instruction until the end)
// ----------------------------------------------------------------------------
template <int PREC> struct LaneAcc;

template <> struct LaneAcc<EMP_PREC_FP64> {
    double v;
    __device__ __forceinline__ void init() { v = 0.0; }
    __device__ __forceinline__ void add(double x) { v += x; }
    template <int L>
    __device__ __forceinline__ double group_sum(double* red, int r) const {
        constexpr int WL = L < 32 ? L : 32;
        double s = v;
#pragma unroll
        for (int o = WL / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, WL);
        if (L > 32) {
            __syncthreads();
            if ((r & 31) == 0) red[r >> 5] = s;
            __syncthreads();
            if (r == 0) {
                double t = 0.0;
                for (int w = 0; w < L / 32; ++w) t += red[w];
                s = t;
            }
        }
        return s;
    }
};

// TwoSum of floats: s + e == a + b exactly
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

template <> struct LaneAcc<EMP_PREC_MIXED> {
    float hi, lo;
    __device__ __forceinline__ void init() { hi = 0.f; lo = 0.f; }
    __device__ __forceinline__ void add(float x) {
        float s, e;
        two_sum(hi, x, s, e);
        hi = s;
        lo = __fadd_rn(lo, e);
    }
    template <int L>
    __device__ __forceinline__ double group_sum(double* red, int r) const {
        constexpr int WL = L < 32 ? L : 32;
        float h = hi, l = lo;
#pragma unroll
        for (int o = WL / 2; o > 0; o >>= 1) {
            const float oh = __shfl_xor_sync(0xffffffffu, h, o, WL);
            const float ol = __shfl_xor_sync(0xffffffffu, l, o, WL);
            float s, e;
            two_sum(h, oh, s, e);
            h = s;
            l = __fadd_rn(__fadd_rn(l, ol), e);
        }
        if (L > 32) {
            float* rf = reinterpret_cast<float*>(red);
            __syncthreads();
            if ((r & 31) == 0) { rf[2 * (r >> 5)] = h; rf[2 * (r >> 5) + 1] = l; }
            __syncthreads();
            if (r == 0) {
                for (int w = 1; w < L / 32; ++w) {
                    float s, e;
                    two_sum(h, rf[2 * w], s, e);
                    h = s;
                    l = __fadd_rn(__fadd_rn(l, rf[2 * w + 1]), e);
                }
            }
        }
        return (double)h + (double)l;
    }
    // the group total as a float-float pair (no FP64 instruction), for
    // groups of at most one warp; every lane holds it
    template <int L>
    __device__ __forceinline__ FF group_sum_ff() const {
        static_assert(L <= 32, "one warp");
        float h = hi, l = lo;
#pragma unroll
        for (int o = L / 2; o > 0; o >>= 1) {
            const float oh = __shfl_xor_sync(0xffffffffu, h, o, L);
            const float ol = __shfl_xor_sync(0xffffffffu, l, o, L);
            float s, e;
            two_sum(h, oh, s, e);
            h = s;
            l = __fadd_rn(__fadd_rn(l, ol), e);
        }
        return FF{h, l};
    }
};

// Mixed kernels of 128 threads are held to 5 resident CTAs per SM (at most
// 102 registers): a half-step of 10 x 256 walkers at 64 lanes is 640 CTAs,
// which then run in one wave on 152 SMs instead of 608 + 32.
template <int PREC, int Q, int L, int NT>
__global__ void __launch_bounds__(NT, (PREC == EMP_PREC_MIXED && NT == 128) ? 5 : 1) k_logpost(KArgs A) {
    using R = typename P<PREC>::R;
    constexpr int G = NT / L;
    constexpr int PC = P<PREC>::kPC;
    constexpr int NQ = Q > 0 ? Q : 1;
    constexpr int NE = (PREC == EMP_PREC_MIXED) ? 4 : 1;   // epochs in flight per lane
    extern __shared__ __align__(16) unsigned char smem[];

    Smem lay;
    lay.build(PREC, Q, L, G, A.tile, A.lay_full, A.lay_free, A.lay_planets, A.lay_ins, A.lay_acc,
              (A.gp_r != nullptr && Q > 0) ? 1 : 0);

    const int tid = threadIdx.x;
    const int g = tid / L;
    const int r = tid - g * L;

    unsigned char* gs = smem + lay.tile_bytes + g * lay.group_bytes;
    double* full = reinterpret_cast<double*>(gs + lay.off_full);
    float* fullh = reinterpret_cast<float*>(gs + lay.off_fullf);
    float* fulll = fullh + lay.n_fullf;
    double* thp = reinterpret_cast<double*>(gs + lay.off_thp);
    R* pcs = reinterpret_cast<R*>(gs + lay.off_pc);
    R* insc = reinterpret_cast<R*>(gs + lay.off_ins);
    double* accc = reinterpret_cast<double*>(gs + lay.off_acc);
    double* red = reinterpret_cast<double*>(gs + lay.off_red);
    R* scan = reinterpret_cast<R*>(gs + lay.off_scan);
    double* pterm = reinterpret_cast<double*>(gs + lay.off_pterm);
    double* misc = reinterpret_cast<double*>(gs + lay.off_misc);
    R* gmx = reinterpret_cast<R*>(gs + lay.off_gma);     // [tile]: zero-state residual (GP with MA)
    R* gmg = gmx + A.tile;                               // [q][tile]: its sensitivity
    int* flag = reinterpret_cast<int*>(misc + 4);
    constexpr int INSW = kInsW;

    // epoch tile (the dataset is only read here, never written by a sweep)
    const int tile = A.tile;
    unsigned char* ts = smem;
    R* s_t0;  R* s_t1;  R* s_y;  R* s_ylo;  R* s_s2;  int* s_in;  R* s_dt;
    if (PREC == EMP_PREC_FP64) {
        s_t0 = reinterpret_cast<R*>(ts);
        s_t1 = s_t0;                       // unused
        s_y = s_t0 + tile;
        s_ylo = s_y;                       // unused
        s_s2 = s_y + tile;
        s_in = reinterpret_cast<int*>(s_s2 + tile);
        s_dt = reinterpret_cast<R*>(ts + Smem::align16((3 * tile) * (int)sizeof(R) + 4 * tile));
    } else {
        s_t0 = reinterpret_cast<R*>(ts);
        s_t1 = s_t0 + tile;
        s_y = s_t1 + tile;
        s_ylo = s_y + tile;
        s_s2 = s_ylo + tile;
        s_in = reinterpret_cast<int*>(s_s2 + tile);
        s_dt = reinterpret_cast<R*>(s_in + tile);
    }
    // stage epochs [base, base + nt) of the series starting at e0 in the
    // lane-chunk layout (coalesced reads, conflict-free lane reads)
    auto stage = [&](int64_t e0s, int base, int nt) {
        const int C = (nt + L - 1) / L;
        for (int idx = tid; idx < nt; idx += NT) {
            const int rr = idx / C;
            const int kk = idx - rr * C;
            const int pos = kk * L + ((rr + kk) & (L - 1));
            const int64_t gi = e0s + base + idx;
            if (PREC == EMP_PREC_FP64) {
                s_t0[pos] = (R)A.d.t[gi];
                s_y[pos] = (R)A.d.y[gi];
                s_s2[pos] = (R)A.d.s2[gi];
            } else {
                s_t0[pos] = (R)A.d.t_hi[gi];
                s_t1[pos] = (R)A.d.t_lo[gi];
                s_y[pos] = (R)A.d.y32[gi];
                s_ylo[pos] = (R)A.d.y_lo[gi];
                s_s2[pos] = (R)A.d.s2_32[gi];
            }
            s_in[pos] = A.d.inst[gi];
#pragma unroll
            for (int c = 0; c < Q; ++c) {
                if (PREC == EMP_PREC_FP64) s_dt[c * tile + pos] = (R)A.d.dt[(size_t)c * A.d.n + gi];
                else s_dt[c * tile + pos] = (R)A.d.dt32[(size_t)c * A.d.n + gi];
            }
        }
    };
    // Programmatic dependent launch: the next kernel of a sweep may start its
    // independent part once every CTA of this one runs, and this one stages
    // the whole series of a one-system handle (one tile) before it waits for
    // the previous kernel's results (both instructions are no-ops for a
    // launch without the attribute).
    asm volatile("griddepcontrol.launch_dependents;");
    const bool prestaged = A.work_counter == nullptr && A.sys_off == nullptr && A.d.n <= tile;
    if (prestaged) stage(0, 0, A.d.n);
    asm volatile("griddepcontrol.wait;" ::: "memory");

    // items: one per CTA for a plain handle; (system, walker chunk) pairs
    // claimed from an atomic counter, costliest systems first, for a batch
    __shared__ int s_item;
    int item = blockIdx.x;
    for (;;) {
    if (A.work_counter != nullptr) {
        __syncthreads();
        if (tid == 0) s_item = atomicAdd(A.work_counter, 1);
        __syncthreads();
        item = s_item;
        if (item >= A.n_sys * A.cps) break;
    }
    const int sidx = A.sys_order != nullptr ? item / A.cps : 0;
    const int sys = A.sys_order != nullptr ? A.sys_order[sidx] : 0;
    const int chunk = item - sidx * A.cps;
    const emp_model_desc* md = A.md + sys;
    const int n_full = md->n_full;
    const int n_free = md->n_free;
    const int n_planets = md->n_planets;
    const int n_ins = md->n_ins;
    const int acc_order = md->acc_order;
    const int wk = chunk * G + g;
    const bool active = wk < A.nwalk;
    const int64_t e0 = A.sys_off != nullptr ? A.sys_off[sys] : 0;
    const double t0 = A.sys_t0 != nullptr ? A.sys_t0[sys] : A.d.t0;
    const int ds = A.dstride;
    const uint64_t seed = A.seed + (uint64_t)sys * 0x9E3779B97F4A7C15ULL;
    const int pbase = sys * A.T * A.W;       // positions / slots of this system
    const int bbase = sys * A.T;             // its inverse temperatures

    // ---------------- walker identity and theta -------------------------
    int t_idx = 0, j_idx = 0, slot_j = 0;
    double z = 1.0;
    uint32_t uword = 0u;
    if (active) {
        if (r == 0) flag[0] = 0;
        if (A.mode == kModeLogpost) {
            slot_j = sys * A.nwalk + wk;     // rows of a batch handle are [S][B]
            for (int d = r; d < n_free; d += L) thp[d] = A.theta[(size_t)slot_j * ds + d];
        } else if (A.mode == kModeSlots) {
            slot_j = pbase + wk;
            for (int d = r; d < n_free; d += L) thp[d] = A.st_theta[(size_t)slot_j * ds + d];
        } else {
            const int Wh = A.W >> 1;
            t_idx = wk / Wh;
            const int jj = wk - t_idx * Wh;
            j_idx = 2 * jj + A.half;
            slot_j = A.members[pbase + t_idx * A.W + j_idx];
            const uint64_t it = (uint64_t)A.counters[0] + (uint64_t)A.step_in_sweep;
            U4 rr = rng_draw(seed, (uint32_t)(t_idx * A.W + j_idx), it,
                             kRngStretch0 + (uint32_t)A.half);
            uword = rr.w;
            // one warp per group forms z and the proposal (FP64, the
            // reference's operation order); the others only wait
            if (r < 32) {
                const int kk = (int)mulhi32(rr.z, (uint32_t)Wh);
                const int k_idx = 2 * kk + (1 - A.half);
                const int slot_k = A.members[pbase + t_idx * A.W + k_idx];
                // emcee StretchMove.get_proposal: zz = ((a-1) u + 1)^2 / a
                const double zz = __dadd_rn(__dmul_rn(A.a - 1.0, u53(rr.x, rr.y)), 1.0);
                z = A.a_inv_exact != 0.0 ? __dmul_rn(__dmul_rn(zz, zz), A.a_inv_exact)
                                         : __dmul_rn(zz, zz) / A.a;
                if (r == 0) misc[2] = z;
                const double* sj = A.st_theta + (size_t)slot_j * ds;
                const double* ck = A.st_theta + (size_t)slot_k * ds;
                for (int d = r; d < n_free; d += (L < 32 ? L : 32))
                    thp[d] = __dsub_rn(ck[d], __dmul_rn(__dsub_rn(ck[d], sj[d]), z));
            }
        }
    }
    __syncthreads();
    if (A.mode == kModeStretch) z = misc[2];
    if (active) {
        for (int s = r; s < n_full; s += L) {
            const int src = md->full_src[s];
            const double v = src >= 0 ? thp[src] : md->full_fixed[s];
            full[s] = v;
            if (PREC == EMP_PREC_MIXED) {
                const float h = (float)v;
                fullh[s] = h;
                fulll[s] = (float)(v - (double)h);
            }
        }
    }
    __syncthreads();

    // ---------------- prior (lane-parallel) and per-walker constants -------
    if (active) {
        for (int d = r; d < n_free; d += L) {
            const emp_prior& p = md->prior[d];
            const double x = thp[d];
            if (!in_support(x, p.lo, p.hi)) flag[0] = 1;
            else if (prior_varies(p.kind)) pterm[d] = prior_var_term(p, x);
        }
        for (int q2 = r; q2 < 2 * n_planets; q2 += L) {
            const int p = q2 >> 1, k = q2 & 1;
            const emp_prior& dp = md->derived[p][k];
            if (dp.kind == EMP_PRIOR_NONE) continue;
            const double x = derived_x(full + md->kep_slot[p], k);
            if (!in_support(x, dp.lo, dp.hi)) flag[0] = 1;
            else if (prior_varies(dp.kind))
                pterm[n_free + q2] = prior_var_term(dp, x);
        }
        for (int p = r; p < n_planets; p += L) {
            if (PREC == EMP_PREC_FP64)
                planet_consts_fp64(md->kep_param[p], full + md->kep_slot[p], (double*)(pcs + p * PC));
            else {
                const int par = md->kep_param[p], ks = md->kep_slot[p];
                if (par == 0 || par == 1 || par == 3 || par == 4 || par >= EMP_TERM_SINUSOID)
                    planet_consts_mixed_ff(par, fullh + ks, fulll + ks, (float*)(pcs + p * PC));
                else
                    planet_consts_mixed(par, full + ks, (float*)(pcs + p * PC));
            }
        }
        for (int k = r; k < n_ins; k += L) {
            R* ic = insc + k * INSW;
            const double off = md->offset_slot >= 0 ? full[md->offset_slot + k] : 0.0;
            const double jit = md->jitter_slot >= 0 ? full[md->jitter_slot + k] : 0.0;
            ic[0] = (R)off;
            ic[2] = (R)(off - (double)(R)off);              // 0 in FP64
            if (PREC == EMP_PREC_FP64) ic[1] = (R)(jit * jit);
            else { const float jf = (float)jit; ic[1] = (R)(jf * jf); }
#pragma unroll
            for (int c = 0; c < Q; ++c) {
                const int base = md->ma_global ? md->ma_slot + 2 * c : md->ma_slot + 2 * Q * k + 2 * c;
                const double phi = full[base], tau = full[base + 1];
                ic[3 + 2 * c] = (R)phi;
                if (PREC == EMP_PREC_FP64) ic[4 + 2 * c] = (R)(-1.0 / tau);
                else ic[4 + 2 * c] = (R)(-1.44269504f / (float)tau);   // exp2 scale
            }
        }
        for (int j = r; j < acc_order; j += L) accc[j] = full[md->acc_slot + j];
    }
    __syncthreads();
    if (active && r == 0) {
        double lp = -INFINITY;
        if (flag[0] == 0 && (md->hill_mask == 0 || hill_stable(md, full))) {
            lp = md->prior_const;
            const int nv = md->n_prior_var;
            for (int i = 0; i < nv; ++i) lp += pterm[md->prior_var[i]];
        }
        misc[0] = lp;
    }
    __syncthreads();
    const double lp = active ? misc[0] : -INFINITY;
    const bool valid = active && (lp > -INFINITY);
    // GP likelihood: this kernel writes the residuals, k_gp does the rest
    const bool gp_on = A.gp_r != nullptr;

    // ---------------- likelihood over epoch tiles ------------------------
    const int n = A.sys_off != nullptr ? (int)(A.sys_off[sys + 1] - e0) : A.d.n;

    LaneAcc<PREC> acc;                     // lane total: FP64, or float-float
    acc.init();
    R carry[NQ];
#pragma unroll
    for (int m = 0; m < NQ; ++m) carry[m] = R(0);

    for (int base = 0; base < n; base += tile) {
        const int nt = min(tile, n - base);
        const int C = (nt + L - 1) / L;
        __syncthreads();
        if (!prestaged) stage(e0, base, nt);
        __syncthreads();

        // per-lane sequential pass over the lane's chunk, NE epochs at a time
        KSum<R> ks; ks.init();
        R xh[NQ];
        R gh[NQ][NQ];
        R S1[NQ];
        R S2[NQ][NQ];
#pragma unroll
        for (int m = 0; m < NQ; ++m) {
            xh[m] = R(0); S1[m] = R(0);
#pragma unroll
            for (int q2 = 0; q2 < NQ; ++q2) { gh[m][q2] = (m == q2) ? R(1) : R(0); S2[m][q2] = R(0); }
        }
        // the pass over the lane's epochs, compiled once with the GP residual
        // writes and once without, so that the Gaussian path carries none of them
        auto epoch_pass = [&](auto gpw) {
            constexpr bool GPW = decltype(gpw)::value;
            if (valid) {
                const int nr = max(0, min(C, nt - r * C));
    #pragma unroll 1
                for (int k0 = 0; k0 < nr; k0 += NE) {
                    int pos[NE];
                    bool ok[NE];
                    R model[NE];
    #pragma unroll
                    for (int e = 0; e < NE; ++e) {
                        const int kk = k0 + e < nr ? k0 + e : nr - 1;
                        ok[e] = k0 + e < nr;
                        pos[e] = kk * L + ((r + kk) & (L - 1));
                        model[e] = R(0);
                    }
                    if constexpr (PREC == EMP_PREC_FP64) {
    #pragma unroll
                        for (int e = 0; e < NE; ++e) {
                            const double t = (double)s_t0[pos[e]];
                            double m = 0.0;
                            for (int p = 0; p < n_planets; ++p)
                                m += rv_term_f64((const double*)(pcs + p * PC), t);
                            if (acc_order > 0) {
                                // np.polyval(concat(theta_acc, [0]), X_ - X_[0])
                                double x = t - t0, pv = 0.0;
                                for (int j = 0; j < acc_order; ++j) pv = pv * x + accc[j];
                                m += pv * x;
                            }
                            model[e] = (R)m;
                        }
                    } else {
                        constexpr int NP = NE / 2;
                        float th[NE], tl[NE];
    #pragma unroll
                        for (int e = 0; e < NE; ++e) { th[e] = (float)s_t0[pos[e]]; tl[e] = (float)s_t1[pos[e]]; }
                        float2 th2[NP], tl2[NP], mod2[NP];
    #pragma unroll
                        for (int j = 0; j < NP; ++j) {
                            th2[j] = make_float2(th[2 * j], th[2 * j + 1]);
                            tl2[j] = make_float2(tl[2 * j], tl[2 * j + 1]);
                            mod2[j] = bc2(0.f);
                        }
                        for (int p = 0; p < n_planets; ++p) {
                            const float* pc = (const float*)(pcs + p * PC);
                            float2 M[NP], ml[NP], sn[NP], cs[NP];
    #pragma unroll
                            for (int j = 0; j < NP; ++j) M[j] = mean_anomaly_pair(pc, th2[j], tl2[j], ml[j]);
                            const float ec = pc[4], el = pc[8];
                            kepler_pairs<NP>(M, ml, ec, el, pc + 12, sn, cs);
    #pragma unroll
                            for (int j = 0; j < NP; ++j) {
                                // (A (cos E - e) - B sin E) / (1 - e cos E) + C with
                                // float-float A, B, C, e
                                const float2 cme = sub2(sub2(cs[j], bc2(ec)), bc2(el));
                                const float2 inv = rcp_nr2(fma2(bc2(-el), cs[j], fma2(bc2(-ec), cs[j], bc2(1.f))));
                                const float2 hi = fma2(fma2(bc2(pc[5]), cme, mul2(bc2(-pc[6]), sn[j])), inv, bc2(pc[7]));
                                const float2 lo = fma2(fma2(bc2(pc[9]), cme, mul2(bc2(-pc[10]), sn[j])), inv, bc2(pc[11]));
                                mod2[j] = add2(mod2[j], add2(hi, lo));
                            }
                        }
    #pragma unroll
                        for (int j = 0; j < NP; ++j) {
                            model[2 * j] = (R)mod2[j].x;
                            model[2 * j + 1] = (R)mod2[j].y;
                        }
                        if (acc_order > 0) {
    #pragma unroll
                            for (int e = 0; e < NE; ++e) {
                                const float x = (th[e] - (float)t0) + tl[e];
                                float pv = 0.f;
                                for (int j = 0; j < acc_order; ++j) pv = pv * x + (float)accc[j];
                                model[e] += (R)(pv * x);
                            }
                        }
                    }
                    // mixed: the per-epoch quantities that do not depend on the MA
                    // state (residual, 1/err2, log err2, MA coefficients) two epochs
                    // per instruction; the recurrence below stays sequential
                    R bb[NE], ww[NE], lw[NE], aa[NE][NQ];
                    if constexpr (PREC == EMP_PREC_MIXED) {
    #pragma unroll
                        for (int j = 0; j < NE / 2; ++j) {
                            const int p0 = pos[2 * j], p1 = pos[2 * j + 1];
                            const float* i0 = (const float*)(insc + s_in[p0] * INSW);
                            const float* i1 = (const float*)(insc + s_in[p1] * INSW);
                            const float2 m2 = make_float2((float)model[2 * j], (float)model[2 * j + 1]);
                            const float2 b2 = add2(sub2(sub2(make_float2(s_y[p0], s_y[p1]), make_float2(i0[0], i1[0])), m2),
                                                   sub2(make_float2(s_ylo[p0], s_ylo[p1]), make_float2(i0[2], i1[2])));
                            const float2 e2 = add2(make_float2(s_s2[p0], s_s2[p1]), make_float2(i0[1], i1[1]));
                            const float2 w2 = rcp_nr2(e2);
                            const float2 l2 = mul2(make_float2(lg2_fast(e2.x), lg2_fast(e2.y)),
                                                   bc2(0.69314718055994531f));
                            bb[2 * j] = b2.x; bb[2 * j + 1] = b2.y;
                            ww[2 * j] = w2.x; ww[2 * j + 1] = w2.y;
                            lw[2 * j] = l2.x; lw[2 * j + 1] = l2.y;
    #pragma unroll
                            for (int c = 0; c < Q; ++c) {
                                const float2 x2 = mul2(make_float2(s_dt[c * tile + p0], s_dt[c * tile + p1]),
                                                       make_float2(i0[4 + 2 * c], i1[4 + 2 * c]));
                                const float2 a2 = mul2(make_float2(i0[3 + 2 * c], i1[3 + 2 * c]),
                                                       make_float2(ex2_fast(x2.x), ex2_fast(x2.y)));
                                aa[2 * j][c] = a2.x; aa[2 * j + 1][c] = a2.y;
                            }
                        }
                    }
    #pragma unroll
                    for (int e = 0; e < NE; ++e) {
                        if (!ok[e]) continue;
                        const int ps = pos[e];
                        R b, w, lt;
                        [[maybe_unused]] const R* ic = insc;
                        if constexpr (PREC == EMP_PREC_FP64) {
                            ic = insc + s_in[ps] * INSW;
                            const R err2 = s_s2[ps] + ic[1];
                            b = s_y[ps] - (model[e] + ic[0]);
                            w = R(1) / err2;
                            lt = (R)log((double)err2);
                        } else {
                            b = bb[e]; w = ww[e]; lt = lw[e];
                        }
                        if constexpr (GPW) {
                            // GP likelihood: hand the residual and err2 to k_gp
                            // (with MA the residual follows the recurrence, below)
                            const size_t gi = (size_t)(e0 + base + r * C + k0 + e) * A.nwalk + wk;
                            if constexpr (PREC == EMP_PREC_FP64) {
                                if (Q == 0) A.gp_r[gi] = (double)b;
                                A.gp_e[gi] = (double)(s_s2[ps] + insc[s_in[ps] * INSW + 1]);
                            } else {
                                // float-float pairs for k_gp_fused
                                if (Q == 0) reinterpret_cast<float2*>(A.gp_r)[gi] = make_float2((float)b, 0.f);
                                reinterpret_cast<float2*>(A.gp_e)[gi] =
                                    make_float2((float)(s_s2[ps] + insc[s_in[ps] * INSW + 1]), 0.f);
                            }
                            if (Q == 0) continue;
                        }
                        if (Q == 0) {
                            ks.add(b * b * w + lt);
                        } else {
                            R x = b;
                            R gn[NQ];
    #pragma unroll
                            for (int q2 = 0; q2 < NQ; ++q2) gn[q2] = R(0);
    #pragma unroll
                            for (int c = 0; c < Q; ++c) {
                                R a;
                                if constexpr (PREC == EMP_PREC_FP64)
                                    a = ic[3 + 2 * c] * (R)exp((double)(s_dt[c * tile + ps] * ic[4 + 2 * c]));
                                else
                                    a = aa[e][c];
                                x -= a * xh[c];
    #pragma unroll
                                for (int q2 = 0; q2 < NQ; ++q2) gn[q2] -= a * gh[c][q2];
                            }
    #pragma unroll
                            for (int m = NQ - 1; m > 0; --m) {
                                xh[m] = xh[m - 1];
    #pragma unroll
                                for (int q2 = 0; q2 < NQ; ++q2) gh[m][q2] = gh[m - 1][q2];
                            }
                            xh[0] = x;
    #pragma unroll
                            for (int q2 = 0; q2 < NQ; ++q2) gh[0][q2] = gn[q2];
                            if constexpr (GPW) {
                                // the residual is x + g . u once the scan gives
                                // this lane's incoming state u
                                gmx[ps] = x;
    #pragma unroll
                                for (int q2 = 0; q2 < NQ; ++q2) gmg[q2 * tile + ps] = gn[q2];
                                continue;
                            }
                            const R wx = w * x;
                            ks.add(wx * x + lt);
    #pragma unroll
                            for (int q2 = 0; q2 < NQ; ++q2) {
                                S1[q2] += wx * gn[q2];
                                const R wg = w * gn[q2];
    #pragma unroll
                                for (int q3 = 0; q3 < NQ; ++q3) S2[q2][q3] += wg * gn[q3];
                            }
                        }
                    }
                }
            }
        };
        if (gp_on) epoch_pass(std::true_type{});
        else epoch_pass(std::false_type{});
        if (valid) {
            acc.add((R)ks.s);
            acc.add((R)(-ks.c));
        }

        if (Q > 0) {
            // join the lane chunks: inclusive scan of the affine maps
            // out = G u + x of the group's lanes (warp shuffles; warp totals
            // through shared memory when a group spans several warps)
            constexpr int MS = NQ + NQ * NQ;   // map size
            constexpr int WL = L < 32 ? L : 32;
            const int lw = r & (WL - 1);
            R mv[MS];
#pragma unroll
            for (int m = 0; m < NQ; ++m) {
                mv[m] = xh[m];
#pragma unroll
                for (int q2 = 0; q2 < NQ; ++q2) mv[NQ + m * NQ + q2] = gh[m][q2];
            }
#pragma unroll
            for (int off = 1; off < WL; off <<= 1) {
                R pv[MS];
#pragma unroll
                for (int k = 0; k < MS; ++k) pv[k] = __shfl_up_sync(0xffffffffu, mv[k], off, WL);
                if (lw >= off) map_compose<R, NQ>(mv, pv);
            }
            R ex[MS];
#pragma unroll
            for (int k = 0; k < MS; ++k) ex[k] = __shfl_up_sync(0xffffffffu, mv[k], 1, WL);
            if (lw == 0) map_identity<R, NQ>(ex);
            R wpre[MS], all[MS];
            map_identity<R, NQ>(wpre);
            if (L > 32) {
                R* tot = scan;                                   // [L/32][MS]
                if (lw == WL - 1) {
#pragma unroll
                    for (int k = 0; k < MS; ++k) tot[(r >> 5) * MS + k] = mv[k];
                }
                __syncthreads();
                const int w = r >> 5;
                for (int k = 0; k < w; ++k) map_compose_left<R, NQ>(tot + k * MS, wpre);
#pragma unroll
                for (int k = 0; k < MS; ++k) all[k] = wpre[k];
                for (int k = w; k < L / 32; ++k) map_compose_left<R, NQ>(tot + k * MS, all);
            } else {
#pragma unroll
                for (int k = 0; k < MS; ++k) all[k] = __shfl_sync(0xffffffffu, mv[k], WL - 1, WL);
            }
            // incoming state of this lane: its exclusive prefix after the
            // earlier warps, applied to the tile's incoming state
            R cw[NQ], u[NQ];
            map_apply<R, NQ>(wpre, carry, cw);
            map_apply<R, NQ>(ex, cw, u);
            R extra = R(0);
#pragma unroll
            for (int q2 = 0; q2 < NQ; ++q2) {
                extra += R(2) * u[q2] * S1[q2];
#pragma unroll
                for (int q3 = 0; q3 < NQ; ++q3) extra += u[q2] * u[q3] * S2[q2][q3];
            }
            if (valid) acc.add(extra);
            if (gp_on && valid) {
                // GP with MA: this lane's residuals after the recurrence
                const int nr = max(0, min(C, nt - r * C));
                for (int k = 0; k < nr; ++k) {
                    const int ps = k * L + ((r + k) & (L - 1));
                    R rr = gmx[ps];
#pragma unroll
                    for (int q2 = 0; q2 < NQ; ++q2) rr += gmg[q2 * tile + ps] * u[q2];
                    const size_t gi = (size_t)(e0 + base + r * C + k) * A.nwalk + wk;
                    if constexpr (PREC == EMP_PREC_FP64) A.gp_r[gi] = (double)rr;
                    else reinterpret_cast<float2*>(A.gp_r)[gi] = make_float2((float)rr, 0.f);
                }
            }
            R nc[NQ];
            map_apply<R, NQ>(all, carry, nc);
#pragma unroll
            for (int m = 0; m < NQ; ++m) carry[m] = nc[m];
        }
    }

    // ---------------- group reduction ------------------------------------
    const double v = acc.template group_sum<L>(red, r);
    const double logl = (valid && r == 0) ? (-0.5 * v + md->loglike_const) : -INFINITY;

    // ---------------- epilogue --------------------------------------------
    if (gp_on) {
        // the prior (and in stretch mode the proposal) for k_gp
        if (active && r == 0) {
            if (A.mode == kModeLogpost) A.logprior[slot_j] = lp;
            else if (A.mode == kModeSlots) A.st_logprior[slot_j] = lp;
            else {
                GPMeta m;
                m.lp = lp; m.z = z; m.uword = uword; m.slot = slot_j;
                m.pos = t_idx * A.W + j_idx; m.t = t_idx;
                A.gp_meta[(size_t)sys * A.nwalk + wk] = m;     // rows [S][nwalk]
            }
        }
        if (active && A.mode == kModeStretch) {
            double* dst = A.gp_prop + ((size_t)sys * A.nwalk + wk) * ds;
            for (int d = r; d < n_free; d += L) dst[d] = thp[d];
        }
    } else if (A.am_rv != nullptr && A.mode == kModeStretch) {
        // joint astrometry: the proposal, its prior and its RV logL for k_am,
        // which adds the astrometric term and makes the Metropolis test
        if (active && r == 0) {
            GPMeta m;
            m.lp = lp; m.z = z; m.uword = uword; m.slot = slot_j;
            m.pos = t_idx * A.W + j_idx; m.t = t_idx;
            A.gp_meta[(size_t)sys * A.nwalk + wk] = m;       // rows [S][nwalk]
            A.am_rv[(size_t)sys * A.nwalk + wk] = logl;
        }
        if (active) {
            double* dst = A.gp_prop + ((size_t)sys * A.nwalk + wk) * ds;
            for (int d = r; d < n_free; d += L) dst[d] = thp[d];
        }
    } else if (A.mode == kModeLogpost) {
        if (active && r == 0) {
            A.logl[slot_j] = logl;
            A.logprior[slot_j] = lp;
            if (A.logp != nullptr && A.beta != nullptr)
                A.logp[slot_j] = valid ? __dadd_rn(__dmul_rn(A.beta[slot_j], logl), lp) : -INFINITY;
        }
    } else if (A.mode == kModeSlots) {
        if (active && r == 0) {
            A.st_logl[slot_j] = logl;
            A.st_logprior[slot_j] = lp;
        }
    } else {
        if (active && r == 0) {
            const double beta = A.betas[bbase + t_idx];
            const double lpj = A.st_logprior[slot_j];
            const double llj = A.st_logl[slot_j];
            const double cur = lpj > -INFINITY ? __dadd_rn(__dmul_rn(beta, llj), lpj) : -INFINITY;
            int acc = 0;
            if (valid) {
                const double nlp = __dadd_rn(__dmul_rn(beta, logl), lp);
                acc = metropolis(nlp, cur, z, n_free - 1, uword) ? 1 : 0;
            }
            misc[1] = acc ? 1.0 : 0.0;
            if (acc) {
                A.st_logl[slot_j] = logl;
                A.st_logprior[slot_j] = lp;
                A.accepted[pbase + t_idx * A.W + j_idx] += 1;
            }
        }
        __syncthreads();
        if (active && misc[1] != 0.0) {
            double* dst = A.st_theta + (size_t)slot_j * ds;
            for (int d = r; d < n_free; d += L) dst[d] = thp[d];
        }
    }
    if (A.work_counter == nullptr) break;
    }   // items
}

}  // namespace emp
