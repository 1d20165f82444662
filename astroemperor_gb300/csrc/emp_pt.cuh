// emp_pt.cuh -- temperature swaps, ladder adaptation and history recording.
//
// Semantics restated from the parallel-tempering sampler EMPEROR drives
// (reddemcee.PTSampler, emp.py:576-593; swap rule and ladder dynamics of
// Vousden, Farr & Mandel 2016, MNRAS 455, 1919, as in ptemcee):
//   * after the stretch steps of a sweep, temperature pairs (i, i-1) are
//     visited from the hottest pair down; walker j of temperature i is
//     paired with walker pi_i(j) of temperature i-1 (pi_i a random affine
//     permutation of 0..W-1) and the pair is exchanged with probability
//     min(1, exp((beta_{i-1} - beta_i) (logL_i - logL_{i-1})));
//   * with adaptation on, the interior inverse temperatures follow
//     T_{k+1} - T_k <- (T_{k+1} - T_k) exp(kappa (A_k - A_{k+1})),
//     kappa = adapt_tau / (t + adapt_tau) / adapt_nu, t = sweeps done,
//     A_k = this sweep's swap acceptance of pair (k, k+1); the coldest and
//     hottest temperatures stay fixed.
#pragma once
#include "emp_device.cuh"

namespace emp {

constexpr int kMaxTemps = 256;

struct SwapArgs {
    int T, W, D, nsteps;
    const double* theta;
    const double* logl;
    int* members;
    double* betas;
    int64_t* counters;
    int* swaps_accepted;
    const int* units;
    int nunits;
    int adapt;
    int adapt_mode;
    double adapt_tau, adapt_nu;
    uint64_t seed;
    double* betas_used;       // [T] scratch: ladder of this sweep
    int64_t* chain_row;       // scratch: row the record kernel writes, -1 none
    // histories
    double* beta_hist;
    double* tsw_hist;
    double* smd_hist;
    int64_t* n_rec;           // [2]
    int64_t cap;
    int thin;
    int record_chain;
};

__global__ void __launch_bounds__(1024) k_swap(SwapArgs S) {
    __shared__ int s_cnt[32];
    __shared__ double s_dst[32];
    __shared__ double s_ratio[kMaxTemps];
    __shared__ double s_smd[kMaxTemps];
    __shared__ double s_invb[kMaxTemps];

    const int tid = threadIdx.x;
    const int nth = blockDim.x;
    const uint64_t sweep = (uint64_t)S.counters[1];
    const int T = S.T, W = S.W, D = S.D;

    for (int t = tid; t < T; t += nth) S.betas_used[t] = S.betas[t];
    __syncthreads();

    for (int i = T - 1; i >= 1; --i) {
        U4 pr = rng_draw(S.seed, (uint32_t)i, sweep, kRngSwapPerm);
        const uint32_t m = (uint32_t)S.units[pr.x % (uint32_t)S.nunits];
        const uint32_t b = pr.y % (uint32_t)W;
        const double dbeta = S.betas[i - 1] - S.betas[i];
        int cnt = 0;
        double dist = 0.0;
        for (int j = tid; j < W; j += nth) {
            const int jp = (int)(((uint64_t)m * (uint64_t)j + b) % (uint64_t)W);
            const int ia = i * W + j, ib = (i - 1) * W + jp;
            const int sa = S.members[ia], sb = S.members[ib];
            U4 ra = rng_draw(S.seed, (uint32_t)ia, sweep, kRngSwapAcc);
            const double paccept = dbeta * (S.logl[sa] - S.logl[sb]);
            if (log(u32u(ra.x)) < paccept) {
                S.members[ia] = sb;
                S.members[ib] = sa;
                ++cnt;
                const double* xa = S.theta + (size_t)sa * D;
                const double* xb = S.theta + (size_t)sb * D;
                double ss = 0.0;
                for (int d = 0; d < D; ++d) { double v = xa[d] - xb[d]; ss += v * v; }
                dist += sqrt(ss);
            }
        }
        // block reduction
        for (int o = 16; o > 0; o >>= 1) {
            cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
            dist += __shfl_xor_sync(0xffffffffu, dist, o);
        }
        if ((tid & 31) == 0) { s_cnt[tid >> 5] = cnt; s_dst[tid >> 5] = dist; }
        __syncthreads();
        if (tid == 0) {
            int c = 0; double dd = 0.0;
            for (int w = 0; w < (nth + 31) / 32; ++w) { c += s_cnt[w]; dd += s_dst[w]; }
            s_ratio[i - 1] = (double)c / (double)W;
            s_smd[i - 1] = c > 0 ? dd / (double)c : 0.0;
            S.swaps_accepted[i] += c;
        }
        __syncthreads();
    }

    if (tid == 0) {
        // histories of this sweep (ladder used during the sweep)
        const int64_t row = S.n_rec[1];
        const bool rec_sweep = (S.thin <= 1) || ((int64_t)sweep % S.thin == (S.thin - 1));
        if (rec_sweep && row < S.cap) {
            if (S.beta_hist) for (int t = 0; t < T; ++t) S.beta_hist[row * T + t] = S.betas[t];
            if (S.tsw_hist) for (int k = 0; k < T - 1; ++k) S.tsw_hist[row * (T - 1) + k] = s_ratio[k];
            if (S.smd_hist) for (int k = 0; k < T - 1; ++k) S.smd_hist[row * (T - 1) + k] = s_smd[k];
            S.n_rec[1] = row + 1;
        }
        const int64_t crow = S.n_rec[0];
        if (S.record_chain && rec_sweep && crow < S.cap) {
            *S.chain_row = crow;
            S.n_rec[0] = crow + 1;
        } else {
            *S.chain_row = -1;
        }
        // ladder adaptation (mode 0: swap-acceptance equalisation)
        if (S.adapt && T > 2) {
            const double kappa = S.adapt_tau / ((double)sweep + S.adapt_tau) / S.adapt_nu;
            for (int t = 0; t < T - 1; ++t) s_invb[t] = 1.0 / S.betas[t];
            double cum = s_invb[0];
            for (int k = 0; k < T - 2; ++k) {
                const double dS = kappa * (s_ratio[k] - s_ratio[k + 1]);
                cum = __dadd_rn(cum, __dmul_rn(s_invb[k + 1] - s_invb[k], exp(dS)));
                S.betas[k + 1] = 1.0 / cum;
            }
        }
        S.counters[0] += S.nsteps;
        S.counters[1] += 1;
    }
}

struct RecArgs {
    int T, W, D;
    const double* theta;
    const double* logl;
    const double* logprior;
    const int* members;
    const double* betas_used;
    const int64_t* chain_row;
    double* chain;
    double* log_like;
    double* log_prob;
};

__global__ void __launch_bounds__(256) k_record(RecArgs R) {
    const int64_t row = *R.chain_row;
    if (row < 0) return;
    const int64_t TW = (int64_t)R.T * R.W;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t g0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (R.chain) {
        const int64_t tot = TW * R.D;
        double* dst = R.chain + row * tot;
        for (int64_t idx = g0; idx < tot; idx += stride) {
            const int64_t tj = idx / R.D;
            const int d = (int)(idx - tj * R.D);
            dst[idx] = R.theta[(int64_t)R.members[tj] * R.D + d];
        }
    }
    for (int64_t idx = g0; idx < TW; idx += stride) {
        const int slot = R.members[idx];
        const double ll = R.logl[slot], lp = R.logprior[slot];
        if (R.log_like) R.log_like[row * TW + idx] = ll;
        if (R.log_prob) {
            const int t = (int)(idx / R.W);
            R.log_prob[row * TW + idx] = lp > -INFINITY ? __dadd_rn(__dmul_rn(R.betas_used[t], ll), lp) : -INFINITY;
        }
    }
}

// CUDA-core throughput probe: independent FMA chains
template <typename T>
__global__ void __launch_bounds__(256) k_fma_probe(T* out, int iters, T seed) {
    T a0 = seed + (T)threadIdx.x, a1 = a0 + (T)1, a2 = a0 + (T)2, a3 = a0 + (T)3;
    T a4 = a0 + (T)4, a5 = a0 + (T)5, a6 = a0 + (T)6, a7 = a0 + (T)7;
    const T m = (T)0.999999, c = (T)1e-7;
#pragma unroll 1
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            a0 = a0 * m + c; a1 = a1 * m + c; a2 = a2 * m + c; a3 = a3 * m + c;
            a4 = a4 * m + c; a5 = a5 * m + c; a6 = a6 * m + c; a7 = a7 * m + c;
        }
    }
    T s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == (T)-1.2345) out[blockIdx.x] = s;   // keeps the chains live
}

}  // namespace emp
