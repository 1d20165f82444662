// emp_stats.cu -- post-run reductions of the sampler's histories on the device.
//
// The reference's postprocess reads, through reddemcee's PTSampler, the
// integrated autocorrelation time of the chains (emp.py:1372-1385) and the
// log-evidence by thermodynamic integration or stepping stones
// (emp.py:1431-1447).  Both need only small summaries of the histories,
// which stay in device memory; these kernels produce them, and the host
// finishes the estimators on arrays of a few hundred numbers:
//   * k_ladder_sums: per temperature the sum and count of the finite
//     log-likelihoods of the kept rows (thermodynamic integration); per
//     stepping stone (a rung of samples and an inverse-temperature step
//     d) the maximum of d L and the sums of exp(d L - max) and its square;
//   * k_autocov: the autocorrelation of every walker's series of every
//     parameter at lags 0..maxlag-1 (direct sums over the kept rows, each
//     series' mean removed, normalised by its lag-0 value; a series that
//     never moves counts as 1 at every lag), averaged over the walkers.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "emp_gpu.h"

namespace emp {
int stats_fail(int code, const char* msg);
void count_launch();
}

namespace {

constexpr int kStatThreads = 256;

// (sum, compensation) of doubles: Neumaier's variant of Kahan summation
struct KS {
    double s, c;
    __device__ void add(double x) {
        const double t = s + x;
        c += fabs(s) >= fabs(x) ? (s - t) + x : (x - t) + s;
        s = t;
    }
};

__device__ double block_sum(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sh[k];
    return t;      // valid in thread 0
}

__device__ double block_max(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double t = -INFINITY;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t = fmax(t, sh[k]);
    __syncthreads();
    return t;      // valid in every thread
}

struct LadderArgs {
    const double* log_like;   // [rows][T][W]
    int rows, T, W, discard, thin;
    const int* stone_src;     // [nstones] temperature whose samples each stone uses
    const double* stone_d;    // [nstones] inverse-temperature step
    int nstones;
    double* out_temp;         // [T][2]: sum, count
    double* out_stone;        // [nstones][4]: max, sum exp(a - max), sum exp(2(a - max)), count
};

// blockIdx.x < T: a temperature's sums; above: a stepping stone
__global__ void __launch_bounds__(kStatThreads) k_ladder_sums(LadderArgs A) {
    __shared__ double sh[kStatThreads / 32];
    const int b = blockIdx.x;
    const int nkept = A.rows > A.discard ? (A.rows - A.discard + A.thin - 1) / A.thin : 0;
    const int64_t n = (int64_t)nkept * A.W;
    const int t = b < A.T ? b : A.stone_src[b - A.T];
    auto sample = [&](int64_t k) -> double {
        const int64_t r = A.discard + (k / A.W) * A.thin, w = k % A.W;
        return A.log_like[(r * A.T + t) * A.W + w];
    };
    if (b < A.T) {
        KS acc{0.0, 0.0};
        double cnt = 0.0;
        for (int64_t k = threadIdx.x; k < n; k += blockDim.x) {
            const double x = sample(k);
            if (isfinite(x)) { acc.add(x); cnt += 1.0; }
        }
        const double s = block_sum(acc.s + acc.c, sh);
        const double c = block_sum(cnt, sh);
        if (threadIdx.x == 0) { A.out_temp[2 * t] = s; A.out_temp[2 * t + 1] = c; }
        return;
    }
    const int st = b - A.T;
    const double d = A.stone_d[st];
    double m = -INFINITY;
    for (int64_t k = threadIdx.x; k < n; k += blockDim.x) {
        const double x = sample(k);
        if (isfinite(x)) m = fmax(m, d * x);
    }
    m = block_max(m, sh);
    double s1 = 0.0, s2 = 0.0, cnt = 0.0;
    if (m > -INFINITY) {
        for (int64_t k = threadIdx.x; k < n; k += blockDim.x) {
            const double x = sample(k);
            if (!isfinite(x)) continue;
            const double e = exp(d * x - m);
            s1 += e;
            s2 += e * e;
            cnt += 1.0;
        }
    }
    s1 = block_sum(s1, sh);
    s2 = block_sum(s2, sh);
    cnt = block_sum(cnt, sh);
    if (threadIdx.x == 0) {
        double* o = A.out_stone + 4 * st;
        o[0] = m; o[1] = s1; o[2] = s2; o[3] = cnt;
    }
}

struct AcfArgs {
    const double* chain;      // [rows][T][W][D]
    int rows, T, W, D, discard, thin, maxlag;
    double* f;                // [T][D][maxlag], accumulated (zeroed by the caller)
};

// one block per (temperature, parameter, walker) series; the series, its
// mean removed, is staged in shared memory as floats, each thread owns lags
__global__ void __launch_bounds__(kStatThreads) k_autocov(AcfArgs A) {
    extern __shared__ float xs[];
    __shared__ double sh[kStatThreads / 32];
    __shared__ double s_c0;
    const int64_t sidx = blockIdx.x;
    const int w = (int)(sidx % A.W);
    const int d = (int)((sidx / A.W) % A.D);
    const int t = (int)(sidx / ((int64_t)A.W * A.D));
    const int n = A.rows > A.discard ? (A.rows - A.discard + A.thin - 1) / A.thin : 0;
    auto at = [&](int i) -> double {
        const int64_t r = A.discard + (int64_t)i * A.thin;
        return A.chain[((r * A.T + t) * A.W + w) * A.D + d];
    };
    KS acc{0.0, 0.0};
    for (int i = threadIdx.x; i < n; i += blockDim.x) acc.add(at(i));
    double mean = block_sum(acc.s + acc.c, sh);
    if (threadIdx.x == 0) sh[0] = mean / (double)(n > 0 ? n : 1);
    __syncthreads();
    mean = sh[0];
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) xs[i] = (float)(at(i) - mean);
    __syncthreads();
    // lag 0 first (the normaliser)
    double c0 = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) c0 += (double)xs[i] * (double)xs[i];
    c0 = block_sum(c0, sh);
    if (threadIdx.x == 0) s_c0 = c0;
    __syncthreads();
    c0 = s_c0;
    double* f = A.f + ((int64_t)t * A.D + d) * A.maxlag;
    const double inv = 1.0 / (double)A.W;
    for (int lag = threadIdx.x; lag < A.maxlag; lag += blockDim.x) {
        double v;
        if (c0 == 0.0) {
            v = 1.0;
        } else {
            float s = 0.f;
            double tot = 0.0;
            int i = 0;
            // float sums over blocks of 256 products, added in FP64
            while (i + lag < n) {
                const int end = min(n - lag, i + 256);
                s = 0.f;
                for (; i < end; ++i) s = fmaf(xs[i], xs[i + lag], s);
                tot += (double)s;
            }
            v = tot / c0;
        }
        atomicAdd(f + lag, v * inv);
    }
}

}  // namespace

extern "C" int emp_ladder_sums(const double* log_like, int rows, int ntemps, int nwalkers, int discard,
                               int thin, const int* stone_src, const double* stone_d, int nstones,
                               double* out_temp, double* out_stone, void* stream) {
    if (!log_like || !out_temp) return emp::stats_fail(EMP_E_INVALID, "a NULL argument");
    if (rows < 0 || ntemps < 1 || nwalkers < 1 || discard < 0 || thin < 1 || nstones < 0)
        return emp::stats_fail(EMP_E_INVALID, "bad sizes");
    if (nstones > 0 && (!stone_src || !stone_d || !out_stone))
        return emp::stats_fail(EMP_E_INVALID, "stepping stones need their arrays");
    LadderArgs a{log_like, rows, ntemps, nwalkers, discard, thin, stone_src, stone_d, nstones,
                 out_temp, out_stone};
    k_ladder_sums<<<ntemps + nstones, kStatThreads, 0, (cudaStream_t)stream>>>(a);
    emp::count_launch();
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return emp::stats_fail(EMP_E_CUDA, cudaGetErrorString(e));
    return EMP_OK;
}

extern "C" int emp_autocorr(const double* chain, int rows, int ntemps, int nwalkers, int ndim,
                            int discard, int thin, int maxlag, double* f, void* stream) {
    if (!chain || !f) return emp::stats_fail(EMP_E_INVALID, "a NULL argument");
    if (rows < 0 || ntemps < 1 || nwalkers < 1 || ndim < 1 || discard < 0 || thin < 1 || maxlag < 1)
        return emp::stats_fail(EMP_E_INVALID, "bad sizes");
    const int n = rows > discard ? (rows - discard + thin - 1) / thin : 0;
    const size_t smem = (size_t)(n > 0 ? n : 1) * sizeof(float);
    if (smem > 200 * 1024)
        return emp::stats_fail(EMP_E_SIZE, "more than 51200 kept rows per series");
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(f, 0, sizeof(double) * (size_t)ntemps * ndim * maxlag, s);
    if (e != cudaSuccess) return emp::stats_fail(EMP_E_CUDA, cudaGetErrorString(e));
    if (smem > 48 * 1024) {
        e = cudaFuncSetAttribute((const void*)k_autocov, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 200 * 1024);
        if (e != cudaSuccess) return emp::stats_fail(EMP_E_CUDA, cudaGetErrorString(e));
    }
    AcfArgs a{chain, rows, ntemps, nwalkers, ndim, discard, thin, maxlag, f};
    const int64_t blocks = (int64_t)ntemps * ndim * nwalkers;
    if (blocks > 0x7fffffff) return emp::stats_fail(EMP_E_SIZE, "too many series");
    k_autocov<<<(unsigned)blocks, kStatThreads, smem, s>>>(a);
    emp::count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return emp::stats_fail(EMP_E_CUDA, cudaGetErrorString(e));
    return EMP_OK;
}
