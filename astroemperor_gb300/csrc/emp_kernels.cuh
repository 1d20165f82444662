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
#pragma once
#include "emp_device.cuh"

namespace emp {

template <int PREC>
__device__ __forceinline__ void planet_consts(const Elements& el,
                                              typename P<PREC>::R* pc);

template <>
__device__ __forceinline__ void planet_consts<EMP_PREC_FP64>(const Elements& el, double* pc) {
    double freq = 2. * kPi / el.per;                       // kep01.model:11
    pc[0] = freq;
    pc[1] = el.phase;
    pc[2] = el.e;
    pc[3] = el.K * el.cw;
    pc[4] = el.K * sqrt(1.0 - el.e * el.e) * el.sw;
    pc[5] = el.K * el.e * el.cw;
    pc[6] = el.tp;
    pc[7] = (double)el.use_tp;
}

template <>
__device__ __forceinline__ void planet_consts<EMP_PREC_MIXED>(const Elements& el, float* pc) {
    // cycles = t * (1/P) + ph, reduced to [-0.5, 0.5) in float-float
    double fc = 1.0 / el.per;
    double ph = el.use_tp ? -el.tp * fc : el.phase * (1.0 / kTwoPi);
    ph -= rint(ph);
    float fh = (float)fc;
    float phh = (float)ph;
    pc[0] = fh;
    pc[1] = (float)(fc - (double)fh);
    pc[2] = phh;
    pc[3] = (float)(ph - (double)phh);
    pc[4] = (float)el.e;
    pc[5] = (float)(el.K * el.cw);
    pc[6] = (float)(el.K * sqrt(1.0 - el.e * el.e) * el.sw);
    pc[7] = (float)(el.K * el.e * el.cw);
}

// one Keplerian term at one epoch
__device__ __forceinline__ double rv_term_f64(const double* pc, double t) {
    double M;
    if (pc[7] != 0.0) M = __dmul_rn(pc[0], __dsub_rn(t, pc[6]));   // kep03/04: freq*(X_-tp)
    else M = __dadd_rn(__dmul_rn(pc[0], t), pc[1]);                // kep01.model:12
    // np.remainder(M + pi, 2 pi) - pi
    double Mr = fmod(M + kPi, kTwoPi);
    if (Mr < 0.0) Mr += kTwoPi;
    Mr -= kPi;
    double e = pc[2];
    double s, c;
    kepler_f64(Mr, e, s, c);
    // K (cos(f + w) + e cos w) with cos f = (cos E - e)/(1 - e cos E),
    // sin f = sqrt(1-e^2) sin E / (1 - e cos E)
    double inv = 1.0 / (1.0 - e * c);
    return (pc[3] * (c - e) - pc[4] * s) * inv + pc[5];
}

__device__ __forceinline__ float rv_term_mixed(const float* pc, float th, float tl) {
    // float-float phase: u = th*fh exactly split, plus cross terms and phase
    // (explicit _rn intrinsics: the error-free transforms must not be
    // contracted into FMAs by the compiler)
    float fh = pc[0], fl = pc[1];
    float p = __fmul_rn(th, fh);
    float pe = __fmaf_rn(th, fh, -p);                 // exact low part of th*fh
    float x = __fadd_rn(p, pc[2]);                    // TwoSum(p, ph_hi)
    float bv = __fsub_rn(x, p);
    float xe = __fadd_rn(__fsub_rn(p, __fsub_rn(x, bv)), __fsub_rn(pc[2], bv));
    float nint = rintf(x);
    float fr = __fsub_rn(x, nint);                    // exact
    float lo = pe + xe + pc[3] + __fmaf_rn(th, fl, tl * fh);
    float cyc = __fadd_rn(fr, lo);
    cyc = __fsub_rn(cyc, rintf(cyc));
    float M = cyc * 6.28318530717958647692f;
    float e = pc[4];
    float s, c;
    kepler_f32(M, e, s, c);
    float inv = __frcp_rn(1.f - e * c);
    return __fmaf_rn(__fmaf_rn(pc[5], c - e, -pc[6] * s), inv, pc[7]);
}

template <int PREC, int Q, int L, int NT>
__global__ void __launch_bounds__(NT) k_logpost(KArgs A) {
    using R = typename P<PREC>::R;
    constexpr int G = NT / L;
    constexpr int PC = P<PREC>::kPC;
    constexpr int NQ = Q > 0 ? Q : 1;
    extern __shared__ __align__(16) unsigned char smem[];

    const emp_model_desc* md = A.md;
    const int n_full = md->n_full;
    const int n_free = md->n_free;
    const int n_planets = md->n_planets;
    const int n_ins = md->n_ins;
    const int acc_order = md->acc_order;

    Smem lay;
    lay.build(PREC, Q, L, G, A.tile, n_full, n_free, n_planets, n_ins, acc_order);

    const int tid = threadIdx.x;
    const int g = tid / L;
    const int r = tid - g * L;
    const int wk = blockIdx.x * G + g;
    const bool active = wk < A.nwalk;

    unsigned char* gs = smem + lay.tile_bytes + g * lay.group_bytes;
    double* full = reinterpret_cast<double*>(gs + lay.off_full);
    double* thp = reinterpret_cast<double*>(gs + lay.off_thp);
    R* pcs = reinterpret_cast<R*>(gs + lay.off_pc);
    R* insc = reinterpret_cast<R*>(gs + lay.off_ins);
    double* accc = reinterpret_cast<double*>(gs + lay.off_acc);
    double* red = reinterpret_cast<double*>(gs + lay.off_red);
    R* scan = reinterpret_cast<R*>(gs + lay.off_scan);
    double* misc = reinterpret_cast<double*>(gs + lay.off_misc);
    constexpr int INSW = 2 + 2 * kMaxQ;

    // ---------------- walker identity and theta -------------------------
    int t_idx = 0, j_idx = 0, slot_j = 0;
    double z = 1.0, logu = 0.0;
    if (active) {
        if (A.mode == kModeLogpost) {
            for (int d = r; d < n_free; d += L) thp[d] = A.theta[(size_t)wk * n_free + d];
        } else if (A.mode == kModeSlots) {
            slot_j = wk;
            for (int d = r; d < n_free; d += L) thp[d] = A.st_theta[(size_t)wk * n_free + d];
        } else {
            const int Wh = A.W >> 1;
            t_idx = wk / Wh;
            const int jj = wk - t_idx * Wh;
            j_idx = 2 * jj + A.half;
            slot_j = A.members[t_idx * A.W + j_idx];
            const uint64_t it = (uint64_t)A.counters[0] + (uint64_t)A.step_in_sweep;
            U4 rr = rng_draw(A.seed, (uint32_t)(t_idx * A.W + j_idx), it,
                             kRngStretch0 + (uint32_t)A.half);
            const int kk = (int)mulhi32(rr.z, (uint32_t)Wh);
            const int k_idx = 2 * kk + (1 - A.half);
            const int slot_k = A.members[t_idx * A.W + k_idx];
            // emcee StretchMove.get_proposal: zz = ((a-1) u + 1)^2 / a
            double zz = __dadd_rn(__dmul_rn(A.a - 1.0, u53(rr.x, rr.y)), 1.0);
            z = __dmul_rn(zz, zz) / A.a;
            logu = log(u32u(rr.w));
            const double* sj = A.st_theta + (size_t)slot_j * n_free;
            const double* ck = A.st_theta + (size_t)slot_k * n_free;
            for (int d = r; d < n_free; d += L)
                thp[d] = __dsub_rn(ck[d], __dmul_rn(__dsub_rn(ck[d], sj[d]), z));
        }
    }
    __syncthreads();
    if (active) {
        for (int s = r; s < n_full; s += L) {
            int src = md->full_src[s];
            full[s] = src >= 0 ? thp[src] : md->full_fixed[s];
        }
    }
    __syncthreads();

    // ---------------- prior and per-walker constants ---------------------
    if (active) {
        if (r == 0) misc[0] = log_prior(md, full);
        for (int p = r; p < n_planets; p += L) {
            Elements el = planet_elements(md->kep_param[p], full + md->kep_slot[p]);
            planet_consts<PREC>(el, pcs + p * PC);
        }
        for (int k = r; k < n_ins; k += L) {
            R* ic = insc + k * INSW;
            double off = md->offset_slot >= 0 ? full[md->offset_slot + k] : 0.0;
            double jit = md->jitter_slot >= 0 ? full[md->jitter_slot + k] : 0.0;
            ic[0] = (R)off;
            ic[1] = (R)(jit * jit);
#pragma unroll
            for (int c = 0; c < Q; ++c) {
                int base = md->ma_global ? md->ma_slot + 2 * c
                                         : md->ma_slot + 2 * Q * k + 2 * c;
                double phi = full[base], tau = full[base + 1];
                ic[2 + 2 * c] = (R)phi;
                if (PREC == EMP_PREC_FP64) ic[3 + 2 * c] = (R)(-1.0 / tau);
                else ic[3 + 2 * c] = (R)(-1.4426950408889634 / tau);   // exp2 scale
            }
        }
        for (int j = r; j < acc_order; j += L) accc[j] = full[md->acc_slot + j];
    }
    __syncthreads();
    const double lp = active ? misc[0] : -INFINITY;
    const bool valid = active && (lp > -INFINITY);

    // ---------------- likelihood over epoch tiles ------------------------
    const int n = A.d.n;
    const int tile = A.tile;
    unsigned char* ts = smem;
    // tile arrays
    R* s_t0;  R* s_t1;  R* s_y;  R* s_s2;  int* s_in;  R* s_dt;
    if (PREC == EMP_PREC_FP64) {
        s_t0 = reinterpret_cast<R*>(ts);
        s_t1 = s_t0;                       // unused
        s_y = s_t0 + tile;
        s_s2 = s_y + tile;
        s_in = reinterpret_cast<int*>(s_s2 + tile);
        s_dt = reinterpret_cast<R*>(ts + Smem::align16((3 * tile) * (int)sizeof(R) + 4 * tile));
    } else {
        s_t0 = reinterpret_cast<R*>(ts);
        s_t1 = s_t0 + tile;
        s_y = s_t1 + tile;
        s_s2 = s_y + tile;
        s_in = reinterpret_cast<int*>(s_s2 + tile);
        s_dt = reinterpret_cast<R*>(s_in + tile);
    }

    double dsum = 0.0;                     // lane total, FP64
    R carry[NQ];
#pragma unroll
    for (int m = 0; m < NQ; ++m) carry[m] = R(0);

    for (int base = 0; base < n; base += tile) {
        const int nt = min(tile, n - base);
        const int C = (nt + L - 1) / L;
        __syncthreads();
        for (int idx = tid; idx < nt; idx += NT) {
            const int rr = idx / C;
            const int kk = idx - rr * C;
            const int pos = kk * L + ((rr + kk) & (L - 1));
            const int gi = base + idx;
            if (PREC == EMP_PREC_FP64) {
                s_t0[pos] = (R)A.d.t[gi];
                s_y[pos] = (R)A.d.y[gi];
                s_s2[pos] = (R)A.d.s2[gi];
            } else {
                s_t0[pos] = (R)A.d.t_hi[gi];
                s_t1[pos] = (R)A.d.t_lo[gi];
                s_y[pos] = (R)A.d.y32[gi];
                s_s2[pos] = (R)A.d.s2_32[gi];
            }
            s_in[pos] = A.d.inst[gi];
#pragma unroll
            for (int c = 0; c < Q; ++c) {
                if (PREC == EMP_PREC_FP64) s_dt[c * tile + pos] = (R)A.d.dt[(size_t)c * n + gi];
                else s_dt[c * tile + pos] = (R)A.d.dt32[(size_t)c * n + gi];
            }
        }
        __syncthreads();

        // per-lane sequential pass over the lane's chunk
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
        if (valid) {
            const int nr = max(0, min(C, nt - r * C));
#pragma unroll 1
            for (int kk = 0; kk < nr; ++kk) {
                const int pos = kk * L + ((r + kk) & (L - 1));
                R model = R(0);
                if (PREC == EMP_PREC_FP64) {
                    const double t = (double)s_t0[pos];
                    if (acc_order > 0) {
                        // np.polyval(concat(theta_acc, [0]), X_ - X_[0])
                        double x = t - A.d.t0, pv = 0.0;
                        for (int j = 0; j < acc_order; ++j) pv = pv * x + accc[j];
                        pv = pv * x;
                        for (int p = 0; p < n_planets; ++p)
                            model = (R)((double)model + rv_term_f64((const double*)(pcs + p * PC), t));
                        model = (R)((double)model + pv);
                    } else {
                        for (int p = 0; p < n_planets; ++p)
                            model = (R)((double)model + rv_term_f64((const double*)(pcs + p * PC), t));
                    }
                } else {
                    const float th = (float)s_t0[pos], tl = (float)s_t1[pos];
                    for (int p = 0; p < n_planets; ++p)
                        model += (R)rv_term_mixed((const float*)(pcs + p * PC), th, tl);
                    if (acc_order > 0) {
                        float x = (th - (float)A.d.t0) + tl, pv = 0.f;
                        for (int j = 0; j < acc_order; ++j) pv = pv * x + (float)accc[j];
                        model += (R)(pv * x);
                    }
                }
                const int ki = s_in[pos];
                const R* ic = insc + ki * INSW;
                model += ic[0];
                const R err2 = s_s2[pos] + ic[1];
                R b = s_y[pos] - model;
                R w, lt;
                if (PREC == EMP_PREC_FP64) { w = R(1) / err2; lt = (R)log((double)err2); }
                else { w = (R)__frcp_rn((float)err2); lt = (R)(__log2f((float)err2) * 0.69314718055994531f); }
                if (Q == 0) {
                    ks.add(b * b * w + lt);
                } else {
                    R x = b;
                    R gn[NQ];
#pragma unroll
                    for (int q2 = 0; q2 < NQ; ++q2) gn[q2] = R(0);
#pragma unroll
                    for (int c = 0; c < Q; ++c) {
                        R dtc = s_dt[c * tile + pos];
                        R a;
                        if (PREC == EMP_PREC_FP64) a = ic[2 + 2 * c] * (R)exp((double)(dtc * ic[3 + 2 * c]));
                        else a = ic[2 + 2 * c] * (R)exp2f((float)(dtc * ic[3 + 2 * c]));
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
        double tile_part = (double)ks.s - (double)ks.c;

        if (Q > 0) {
            // join the lane chunks: inclusive scan of affine maps
            // out = Gm u + xm over the group's lanes (Hillis-Steele, smem)
            constexpr int MS = NQ + NQ * NQ;   // map size
            R* buf0 = scan;
            R* buf1 = scan + MS * L;
            {
                R* mp = buf0 + r * MS;
#pragma unroll
                for (int m = 0; m < NQ; ++m) {
                    mp[m] = xh[m];
#pragma unroll
                    for (int q2 = 0; q2 < NQ; ++q2) mp[NQ + m * NQ + q2] = gh[m][q2];
                }
            }
            __syncthreads();
            R* src = buf0;
            R* dst = buf1;
            for (int off = 1; off < L; off <<= 1) {
                R* o = dst + r * MS;
                const R* a = src + r * MS;
                if (r >= off) {
                    const R* bq = src + (r - off) * MS;   // earlier prefix
                    // (Ga, xa) o (Gb, xb) = (Ga Gb, Ga xb + xa)
#pragma unroll
                    for (int m = 0; m < NQ; ++m) {
                        R v = a[m];
#pragma unroll
                        for (int q2 = 0; q2 < NQ; ++q2) v += a[NQ + m * NQ + q2] * bq[q2];
                        o[m] = v;
#pragma unroll
                        for (int q3 = 0; q3 < NQ; ++q3) {
                            R gv = R(0);
#pragma unroll
                            for (int q2 = 0; q2 < NQ; ++q2) gv += a[NQ + m * NQ + q2] * bq[NQ + q2 * NQ + q3];
                            o[NQ + m * NQ + q3] = gv;
                        }
                    }
                } else {
#pragma unroll
                    for (int m = 0; m < MS; ++m) o[m] = a[m];
                }
                __syncthreads();
                R* tmp = src; src = dst; dst = tmp;
            }
            // incoming state of this lane = prefix(r-1) applied to carry
            R u[NQ];
            if (r == 0) {
#pragma unroll
                for (int m = 0; m < NQ; ++m) u[m] = carry[m];
            } else {
                const R* pm = src + (r - 1) * MS;
#pragma unroll
                for (int m = 0; m < NQ; ++m) {
                    R v = pm[m];
#pragma unroll
                    for (int q2 = 0; q2 < NQ; ++q2) v += pm[NQ + m * NQ + q2] * carry[q2];
                    u[m] = v;
                }
            }
            double extra = 0.0;
#pragma unroll
            for (int q2 = 0; q2 < NQ; ++q2) {
                extra += 2.0 * (double)u[q2] * (double)S1[q2];
#pragma unroll
                for (int q3 = 0; q3 < NQ; ++q3) extra += (double)u[q2] * (double)u[q3] * (double)S2[q2][q3];
            }
            tile_part += extra;
            // carry for the next tile = full prefix applied to carry
            {
                const R* pm = src + (L - 1) * MS;
                R nc[NQ];
#pragma unroll
                for (int m = 0; m < NQ; ++m) {
                    R v = pm[m];
#pragma unroll
                    for (int q2 = 0; q2 < NQ; ++q2) v += pm[NQ + m * NQ + q2] * carry[q2];
                    nc[m] = v;
                }
#pragma unroll
                for (int m = 0; m < NQ; ++m) carry[m] = nc[m];
            }
        }
        if (valid) dsum += tile_part;
    }

    // ---------------- group reduction ------------------------------------
    double v = dsum;
    constexpr int WL = L < 32 ? L : 32;
#pragma unroll
    for (int o = WL / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, WL);
    if (L > 32) {
        __syncthreads();
        if ((r & 31) == 0) red[r >> 5] = v;
        __syncthreads();
        if (r == 0) {
            double s = 0.0;
            for (int w = 0; w < L / 32; ++w) s += red[w];
            v = s;
        }
    }
    const double logl = valid ? (-0.5 * v + md->loglike_const) : -INFINITY;

    // ---------------- epilogue --------------------------------------------
    if (A.mode == kModeLogpost) {
        if (active && r == 0) {
            A.logl[wk] = logl;
            A.logprior[wk] = lp;
            if (A.logp != nullptr && A.beta != nullptr)
                A.logp[wk] = valid ? __dadd_rn(__dmul_rn(A.beta[wk], logl), lp) : -INFINITY;
        }
    } else if (A.mode == kModeSlots) {
        if (active && r == 0) {
            A.st_logl[wk] = logl;
            A.st_logprior[wk] = lp;
        }
    } else {
        if (active && r == 0) {
            const double beta = A.betas[t_idx];
            const double lpj = A.st_logprior[slot_j];
            const double llj = A.st_logl[slot_j];
            const double cur = lpj > -INFINITY ? __dadd_rn(__dmul_rn(beta, llj), lpj) : -INFINITY;
            const double nlp = valid ? __dadd_rn(__dmul_rn(beta, logl), lp) : -INFINITY;
            const double lnpdiff = __dadd_rn(__dmul_rn((double)(n_free - 1), log(z)), nlp) - cur;
            const int acc = (valid && lnpdiff > logu) ? 1 : 0;
            misc[1] = acc ? 1.0 : 0.0;
            if (acc) {
                A.st_logl[slot_j] = logl;
                A.st_logprior[slot_j] = lp;
                A.accepted[t_idx * A.W + j_idx] += 1;
            }
        }
        __syncthreads();
        if (active && misc[1] != 0.0) {
            double* dst = A.st_theta + (size_t)slot_j * n_free;
            for (int d = r; d < n_free; d += L) dst[d] = thp[d];
        }
    }
}

}  // namespace emp
