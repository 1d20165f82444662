// emp_model_eval.cuh -- my_model(theta) -> (model0, err20) on the device
// (emp_model.py:706-781), FP64, for fits and reporting.
#pragma once
#include "emp_kernels.cuh"

namespace emp {

// pass 1: mean model (Keplerians, acceleration, offsets) and err2 per epoch
__global__ void __launch_bounds__(256) k_model_mean(const emp_model_desc* md, DevData d,
                                                    const int* dev2orig, const double* theta,
                                                    double* model_out, double* err2_out) {
    extern __shared__ __align__(16) double sm[];
    const int b = blockIdx.y;
    const int n_full = md->n_full, n_free = md->n_free, np = md->n_planets, ni = md->n_ins;
    double* full = sm;
    double* pcs = full + n_full;
    double* ins = pcs + 8 * (np > 0 ? np : 1);
    double* acc = ins + 2 * ni;
    const double* th = theta + (size_t)b * n_free;
    for (int s = threadIdx.x; s < n_full; s += blockDim.x) {
        int src = md->full_src[s];
        full[s] = src >= 0 ? th[src] : md->full_fixed[s];
    }
    __syncthreads();
    for (int p = threadIdx.x; p < np; p += blockDim.x)
        planet_consts_fp64(md->kep_param[p], full + md->kep_slot[p], pcs + 8 * p);
    for (int k = threadIdx.x; k < ni; k += blockDim.x) {
        ins[2 * k] = md->offset_slot >= 0 ? full[md->offset_slot + k] : 0.0;
        double j = md->jitter_slot >= 0 ? full[md->jitter_slot + k] : 0.0;
        ins[2 * k + 1] = j * j;
    }
    for (int j = threadIdx.x; j < md->acc_order; j += blockDim.x) acc[j] = full[md->acc_slot + j];
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.n; i += gridDim.x * blockDim.x) {
        const double t = d.t[i];
        double m = 0.0;
        for (int p = 0; p < np; ++p) m += rv_term_f64(pcs + 8 * p, t);
        if (md->acc_order > 0) {
            double x = t - d.t0, pv = 0.0;
            for (int j = 0; j < md->acc_order; ++j) pv = pv * x + acc[j];
            m += pv * x;
        }
        const int k = d.inst[i];
        m += ins[2 * k];
        const int o = dev2orig[i];
        model_out[(size_t)b * d.n + o] = m;
        err2_out[(size_t)b * d.n + o] = d.s2[i] + ins[2 * k + 1];
    }
}

// pass 2: moving-average recurrence, one thread per walker, sequential in
// the device epoch order (per-instrument runs are contiguous there; a lag
// with no predecessor has dt = +inf and so a zero coefficient)
__global__ void k_model_ma(const emp_model_desc* md, DevData d, const int* dev2orig,
                           const double* theta, int B, double* model_out) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B || d.q == 0) return;
    const int q = d.q;
    const double* th = theta + (size_t)b * md->n_free;
    auto fullv = [&](int s) -> double {
        int src = md->full_src[s];
        return src >= 0 ? th[src] : md->full_fixed[s];
    };
    double hist[kMaxQ] = {0.0, 0.0, 0.0};   // final residuals at lags 1..q
    for (int i = 0; i < d.n; ++i) {
        const int k = d.inst[i];
        const int o = dev2orig[i];
        double* mp = model_out + (size_t)b * d.n + o;
        double res = d.y[i] - *mp;
        double ma = 0.0;
        for (int c = 0; c < q; ++c) {
            int base = md->ma_global ? md->ma_slot + 2 * c : md->ma_slot + 2 * q * k + 2 * c;
            double dt = d.dt[(size_t)c * d.n + i];
            double a = fullv(base) * exp(-dt / fullv(base + 1));
            ma += a * hist[c];
        }
        *mp += ma;
        res -= ma;
        for (int c = q - 1; c > 0; --c) hist[c] = hist[c - 1];
        hist[0] = res;
    }
}

}  // namespace emp
