// emp_device.cuh -- device code of the EMPEROR RV log-posterior hot path.
//
// One kernel template evaluates the log-posterior of a batch of walkers:
//   * a CTA holds G walker groups of L lanes (G*L = NT threads);
//   * the CTA stages the dataset into shared memory one epoch tile at a
//     time (coalesced global reads, a lane-chunk layout in shared memory);
//   * each lane of a group walks a contiguous chunk of the tile's epochs
//     sequentially, so the moving-average recurrence of the reference
//     (support/models/moav01.model:7-15) is a per-lane loop; the chunks are
//     joined by an affine-map scan across the group's lanes;
//   * group sums are reduced with warp shuffles (+ shared memory across warps).
// The same kernel also runs one half-step of the affine-invariant stretch
// move (propose -> evaluate -> Metropolis accept) for parallel tempering.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>
#include "emp_gpu.h"

namespace emp {

constexpr double kTwoPi = 6.283185307179586476925286766559;
constexpr double kPi = 3.1415926535897932384626433832795;
constexpr int kMaxQ = EMP_MAX_MA;
// per-instrument constants of the log-posterior kernel: offset, jitter^2,
// offset low part (mixed), then (Phi, -1/tau) per MA term
constexpr int kInsW = 3 + 2 * kMaxQ;

// ----------------------------------------------------------------------------
// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror & Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11).
// ----------------------------------------------------------------------------
struct U4 { uint32_t x, y, z, w; };

__host__ __device__ __forceinline__ uint32_t mulhi32(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
    return __umulhi(a, b);
#else
    return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32);
#endif
}

__host__ __device__ __forceinline__ U4 philox(U4 c, uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = mulhi32(M0, c.x), lo0 = M0 * c.x;
        uint32_t hi1 = mulhi32(M1, c.z), lo1 = M1 * c.z;
        U4 n;
        n.x = hi1 ^ c.y ^ k0;
        n.y = lo1;
        n.z = hi0 ^ c.w ^ k1;
        n.w = lo0;
        c = n;
        k0 += W0;
        k1 += W1;
    }
    return c;
}

// purposes (third counter word)
constexpr uint32_t kRngStretch0 = 1u;   // + half
constexpr uint32_t kRngSwapPerm = 3u;
constexpr uint32_t kRngSwapAcc = 4u;

__host__ __device__ __forceinline__ U4 rng_draw(uint64_t seed, uint32_t index,
                                                 uint64_t iter, uint32_t purpose) {
    U4 c{index, (uint32_t)iter, purpose, (uint32_t)(iter >> 32)};
    return philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
}

// uniform in [0,1) with 53 random bits from two words (numpy's rand())
__host__ __device__ __forceinline__ double u53(uint32_t a, uint32_t b) {
    uint64_t k = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
    return (double)k * (1.0 / 9007199254740992.0);
}
// uniform in (0,1) from one word
__host__ __device__ __forceinline__ double u32u(uint32_t a) {
    return ((double)a + 0.5) * (1.0 / 4294967296.0);
}

// ----------------------------------------------------------------------------
// dataset as laid out in device memory (one system)
// ----------------------------------------------------------------------------
struct DevData {
    int n;                 // epochs
    int q;                 // MA order stored in dt arrays
    double t0;             // acceleration origin (first epoch in time order)
    const double* t;       // [n]
    const double* y;       // [n]
    const double* s2;      // [n] yerr^2
    const double* dt;      // [q][n] lag-(c+1) time gaps, +inf where no predecessor
    const float* t_hi;     // float-float split of t
    const float* t_lo;
    const float* y32;
    const float* y_lo;     // y - (double)y32
    const float* s2_32;
    const float* dt32;     // [q][n]
    const int* inst;       // [n] 0-based instrument
};

// kModeGPOnly: k_gp alone on caller residual rows (emp_gp_logl)
enum Mode : int { kModeLogpost = 0, kModeStretch = 1, kModeSlots = 2, kModeGPOnly = 3 };

// what the stretch kernel hands to the GP kernel per proposal
struct GPMeta {
    double lp;                 // log-prior of the proposal (-inf: outside the support)
    double z;                  // stretch factor
    uint32_t uword;            // Metropolis random word
    int slot;                  // physical slot of the walker
    int pos;                   // logical position t * W + j within its system
    int t;                     // temperature index
};

// threads of a k_am CTA: four walker rows, one warp each
constexpr int kAmThreads = 128;

// astrometric data on the device (emp_am_desc, emp_set_astrometry)
struct AmDev {
    int n_hipp, n_gost;
    const double* catalogs;    // [3][7]
    const double* inv_cov;     // [3][5][5]
    const double* log_det_cov; // [3]
    const double* astro_gost;  // [2][5]
    const double* hipp;        // [7][n_hipp]
    const double* gost;        // [4][n_gost]
    const double* gsv;         // [2][5][n_gost]
    double common_t;
};

struct KArgs {
    const emp_model_desc* md;
    DevData d;
    int mode;
    int nwalk;             // walkers handled by this launch
    int tile;              // epochs per shared-memory tile
    // kModeLogpost
    const double* theta;   // [nwalk][n_free]
    const double* beta;    // [nwalk] or null
    double* logl;
    double* logprior;
    double* logp;          // or null
    // PT (kModeStretch / kModeSlots)
    double* st_theta;      // [slots][n_free]
    double* st_logl;
    double* st_logprior;
    const int* members;    // [T][W]
    const double* betas;   // [T]
    const int64_t* counters;
    int* accepted;         // [T][W]
    int W;
    int half;
    int step_in_sweep;
    uint64_t seed;
    double a;
    double a_inv_exact;        // 1/a when a is a power of two (then zz^2/a == zz^2 * (1/a)), else 0
    // systems (one for a plain handle; many for a batch handle)
    int T;                     // temperatures per system (PT modes)
    int n_sys;                 // systems processed by this launch
    int cps;                   // CTA items per system
    const int64_t* sys_off;    // [S+1] epoch offsets, null = one system
    const double* sys_t0;      // [S] acceleration origins, null = d.t0
    const int* sys_order;      // [S] systems costliest first, null = one system
    int* work_counter;         // persistent scheduling counter, null = one item per CTA
    int dstride;               // theta row stride (largest free dimension)
    int lay_full, lay_free, lay_planets, lay_ins, lay_acc;   // layout maxima
    // GP likelihood (md->gp_nterms > 0): the kernel writes the residuals and
    // err2 of every walker row, epoch-major ([n][nwalk]), and in stretch mode
    // the proposal; k_gp then forms the log-likelihood (and the Metropolis test)
    double* gp_r;
    double* gp_e;
    double* gp_prop;           // [nwalk][dstride] proposals (stretch)
    GPMeta* gp_meta;           // [nwalk] (stretch)
    double* gp_u;              // [n][nwalk][M] U, V and phi of the recursion (k_gp_prep)
    double* gp_v;
    double* gp_ph;
    double* gp_asum;           // [nwalk] k(0) of each row's kernel (NaN: bad coefficients)
    // joint RV + astrometry (md->am_on): in stretch mode the kernel writes
    // the proposal, its meta (gp_prop, gp_meta) and its RV logL (am_rv); k_am
    // adds the astrometric term and finishes every mode
    double* am_rv;             // [nwalk] (stretch)
    AmDev am;
    const AmDev* am_sys;       // [S] one per system of a batch handle (null: am)
};


// ----------------------------------------------------------------------------
// shared memory layout (bytes), computed identically on host and device
// ----------------------------------------------------------------------------
struct Smem {
    int tile_bytes;        // staged epochs
    int group_bytes;       // per walker group
    int off_full, off_thp, off_pc, off_ins, off_acc, off_red, off_scan, off_pterm, off_misc;
    int off_gma;               // GP with a live MA: per epoch of the tile x and g[q] (0 bytes otherwise)
    int off_fullf, n_fullf;    // float-float copy of the full vector (mixed): hi [n], lo [n]
    int total;

    __host__ __device__ static int align16(int x) { return (x + 15) & ~15; }

    // gp_ma: a GP likelihood on the residuals of a live MA recurrence (the
    // lane-chunk pass keeps each epoch's zero-state residual and its
    // sensitivity to the incoming state until the scan gives that state)
    __host__ __device__ void build(int prec, int q, int L, int G, int tile, int n_full,
                                   int n_free, int n_planets, int n_ins, int acc_order, int gp_ma = 0) {
        int rs = prec == EMP_PREC_FP64 ? 8 : 4;          // real size
        int per_epoch = (prec == EMP_PREC_FP64) ? (8 * 3 + 4 + 8 * q)
                                                : (4 * 5 + 4 + 4 * q);
        tile_bytes = align16(per_epoch * tile + 64);
        int o = 0;
        off_full = o; o += align16(8 * n_full);
        n_fullf = prec == EMP_PREC_FP64 ? 0 : n_full;
        off_fullf = o; o += align16(8 * n_fullf);
        off_thp = o;  o += align16(8 * (n_free > 0 ? n_free : 1));
        off_pc = o;   o += align16(rs * (prec == EMP_PREC_FP64 ? 8 : 16) * (n_planets > 0 ? n_planets : 1));
        off_ins = o;  o += align16(rs * kInsW * (n_ins > 0 ? n_ins : 1));
        off_acc = o;  o += align16(8 * (acc_order > 0 ? acc_order : 1));
        off_red = o;  o += align16(8 * 4 * ((L + 31) / 32));
        // MA scan: warp totals [L/32][q + q^2] when a walker spans several warps
        off_scan = o; o += align16((L > 32 && q > 0) ? rs * (L / 32) * (q + q * q) : 0);
        off_pterm = o; o += align16(8 * (n_free + 2 * n_planets + 1));
        off_misc = o; o += 64;
        off_gma = o;  o += align16((gp_ma && q > 0) ? rs * tile * (1 + q) : 0);
        group_bytes = align16(o);
        total = tile_bytes + G * group_bytes;
    }
};

// ----------------------------------------------------------------------------
// per-planet elements (FP64): per, K, phase (rad, or NAN with tp), tp, e, w
// support/models/kep00..kep07.model prologues
// ----------------------------------------------------------------------------
struct Elements { double per, K, phase, tp, e, cw, sw; int use_tp; };

__device__ __forceinline__ void omega_from_sc(double S, double C, double ecc, double thr,
                                              double& cw, double& sw) {
    if (ecc < thr) { cw = 1.0; sw = 0.0; return; }
    double w = acos(C / sqrt(ecc));
    if (S < 0) w = kTwoPi - w;
    sincos(w, &sw, &cw);
}

static __device__ Elements planet_elements(int par, const double* v) {
    Elements el;
    el.use_tp = 0; el.tp = 0.0;
    switch (par) {
        case EMP_TERM_SINUSOID: case EMP_TERM_CYCLE_1: case EMP_TERM_CYCLE_2: {
            // A cos(2 pi t / per' + phase) as an e = 0 Keplerian; the first
            // magnetic-cycle term runs at pi / per, i.e. per' = 2 per (exact)
            el.per = par == EMP_TERM_CYCLE_1 ? 2.0 * v[0] : v[0];
            el.K = par == EMP_TERM_CYCLE_2 ? v[2] : v[1];
            el.phase = par == EMP_TERM_SINUSOID ? v[2] : (par == EMP_TERM_CYCLE_1 ? v[3] : v[4]);
            el.e = 0.0; el.cw = 1.0; el.sw = 0.0;
        } break;
        case 0: case 6: {
            el.per = par == 6 ? exp(v[0]) : v[0];
            el.K = v[1]; el.phase = v[2]; el.e = v[3];
            sincos(v[4], &el.sw, &el.cw);
        } break;
        case 1: case 7: {
            el.per = par == 7 ? exp(v[0]) : v[0];
            el.K = v[1]; el.phase = v[2];
            el.e = v[3] * v[3] + v[4] * v[4];
            omega_from_sc(v[3], v[4], el.e, 1e-6, el.cw, el.sw);
        } break;
        case 2: {
            el.per = exp(v[0]);
            double As = v[1], Ac = v[2];
            el.K = As * As + Ac * Ac;
            el.e = v[3] * v[3] + v[4] * v[4];
            omega_from_sc(v[3], v[4], el.e, 1e-5, el.cw, el.sw);
            double ph = acos(Ac / sqrt(el.K));
            if (As < 0) ph = kTwoPi - ph;
            el.phase = ph;
        } break;
        case 3: {
            el.per = v[0]; el.K = v[1]; el.tp = v[2]; el.use_tp = 1; el.phase = 0.0;
            el.e = v[3];
            sincos(v[4], &el.sw, &el.cw);
        } break;
        case 4: default: {
            el.per = v[0]; el.K = v[1]; el.tp = v[2]; el.use_tp = 1; el.phase = 0.0;
            el.e = v[3] * v[3] + v[4] * v[4];
            omega_from_sc(v[3], v[4], el.e, 1e-5, el.cw, el.sw);
        } break;
    }
    return el;
}

// ----------------------------------------------------------------------------
// Kepler solvers
// ----------------------------------------------------------------------------
// FP64: Danby start + Halley to |dE| <= 1e-15 (same iteration as the oracle)
__device__ __forceinline__ void kepler_f64(double Mr, double e, double& s, double& c) {
    double sM = sin(Mr);
    double E = Mr + 0.85 * e * (sM > 0.0 ? 1.0 : (sM < 0.0 ? -1.0 : 0.0));
#pragma unroll 1
    for (int it = 0; it < 60; ++it) {
        sincos(E, &s, &c);
        double f = E - e * s - Mr;
        double f1 = 1.0 - e * c;
        double f2 = e * s;
        double d1 = -f / f1;
        double d = -f / (f1 + 0.5 * d1 * f2);
        E = E + d;
        if (fabs(d) <= 1e-15) break;
    }
    sincos(E, &s, &c);
}


// ----------------------------------------------------------------------------
// precision traits
// ----------------------------------------------------------------------------
template <int PREC> struct P;

template <> struct P<EMP_PREC_FP64> {
    using R = double;
    // planet constants: [0]=freq [1]=phase [2]=e [3]=Kcw [4]=K sqrt(1-e^2) sw [5]=K e cw [6]=tp/use
    static constexpr int kPC = 8;
};
template <> struct P<EMP_PREC_MIXED> {
    using R = float;
    // [0]=f_hi [1]=f_lo (cycles/day) [2]=ph_hi [3]=ph_lo (cycles) [4]=e [5]=A [6]=B [7]=C,
    // [8..11] = the low parts of e, A, B, C (float-float constants),
    // [12..15] = Kepler starter constants of e (a, a^3, 0.5 / (4 e + 0.5), 0.078 / (1 + e))
    static constexpr int kPC = 16;
};

// ----------------------------------------------------------------------------
// compensated (Kahan) accumulator
// ----------------------------------------------------------------------------
template <typename R> struct KSum {
    R s, c;
    __device__ __forceinline__ void init() { s = R(0); c = R(0); }
    __device__ __forceinline__ void add(R x) {
        R y = x - c;
        R t = s + y;
        c = (t - s) - y;
        s = t;
    }
};

}  // namespace emp
