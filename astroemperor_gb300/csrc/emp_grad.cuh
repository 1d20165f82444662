// emp_grad.cuh -- adjoint kernel: d logL / d theta and d logprior / d theta.
//
// The reference has no gradient; this is the reverse mode of its
// my_likelihood (support/likelihoods/00.like:3-5) through my_model
// (emp_model.py:706-781): Keplerians of every parameterisation
// (kep00-kep07.model), the sinusoid and magnetic-cycle terms
// (sinusoid00.model, magneticcycle00.model), acceleration (acc.model),
// offsets, jitters and the moving average (moav01.model's recurrence,
// globally or on each instrument's run).
//
// One walker per group of L lanes; the CTA stages the series one epoch tile
// at a time (lane-chunk layout as in k_logpost) and each group keeps the
// tile's residuals r and adjoints in shared memory.
//
//   forward, tiles in order: mean model in float-float planet constants
//     (the same accurate steps as the mixed log-posterior kernel, with the
//     constants formed in FP64), b = y - offset - model; with MA the
//     recurrence r_i = b_i - sum_c a_{c,i} r_{i-1-c} runs per lane from a
//     zero state, an affine-map scan joins the lanes and the tiles, and a
//     second pass writes r; log L accumulates.  Without MA the adjoint
//     dL/dmodel_i = w_i r_i is local, and each tile's gradient terms follow
//     at once.
//   backward (MA only), tiles in reverse: lambda_i = dL/db_i =
//     -w_i r_i - sum_c a_{c,i+1+c} lambda_{i+1+c} by the same lane-chunk
//     scheme run backwards (reverse scan, carry to the earlier tile); the
//     noise-model gradients; then the tile's gradient terms.  When the
//     series spans several tiles, r goes through a per-walker buffer in
//     device memory between the passes.
//   gradient terms, per planet and tile: E recomputed (not stored),
//     dE/dM = 1/(1 - e cos E) and dE/de = sin E/(1 - e cos E) by the
//     implicit function theorem; five sums per planet against
//     lambda' = dL/dmodel: sum lambda' dRV/dM, sum lambda' dRV/dM t,
//     sum lambda' dRV/dA, sum lambda' dRV/dB and sum lambda' dRV/de at
//     fixed M, with RV = A((cos E - e)/D + e) - B sqrt(1-e^2) sin E/D,
//     A = K cos w, B = K sin w, D = 1 - e cos E.
//   chain rule (FP64, one lane per planet): the five sums to the
//     parameterisation's theta (period or log period, amplitude or the
//     (As, Ac) pair, phase or time of periastron, e and w or (S, C)).
// Per-epoch terms are FP32; every sum is a compensated (TwoSum) lane sum,
// float-float across lanes, finished in FP64.
#pragma once
#include "emp_kernels.cuh"

namespace emp {

constexpr int kGradMaxIns = 4;
constexpr int kGPC = 20;      // floats per planet: the forward kernel's 16, then B, q, 1 - e^2
constexpr int kGInsW = 4 + 3 * kMaxQ;   // offset, J^2, offset low part, J, then (Phi, -log2(e)/tau, tau)

struct GArgs {
    const emp_model_desc* md;
    DevData d;
    int nwalk;
    int tile;                 // epochs per staged tile (a multiple of L)
    const double* theta;      // [B][n_free]
    double* logl;             // [B]
    double* logprior;         // [B]
    double* grad_logl;        // [B][n_free]
    double* grad_logprior;    // [B][n_free]
    float* resid;             // [B][resid_stride]: r between the passes (MA over several tiles)
    int64_t resid_stride;     // tiles * tile
};

struct GSmem {
    int tile_bytes, group_bytes, total;
    int off_full, off_pc, off_ins, off_acc, off_red, off_scan, off_pterm, off_gfull, off_ug,
        off_misc, off_r, off_l;
    __host__ __device__ void build(int q, int L, int G, int tile, int n_full, int n_free, int n_planets,
                                   int n_ins, int acc_order) {
        tile_bytes = Smem::align16((6 * 4 + 4 * q) * tile);
        const int np = n_planets > 0 ? n_planets : 1;
        int o = 0;
        off_full = o;  o += Smem::align16(8 * n_full);
        off_pc = o;    o += Smem::align16(4 * kGPC * np);
        off_ins = o;   o += Smem::align16(4 * kGInsW * (n_ins > 0 ? n_ins : 1));
        off_acc = o;   o += Smem::align16(8 * (acc_order > 0 ? acc_order : 1));
        off_red = o;   o += Smem::align16(8 * 4 * ((L + 31) / 32));
        off_scan = o;  o += Smem::align16(4 * (kMaxQ + kMaxQ * kMaxQ) * ((L + 31) / 32));
        off_pterm = o; o += Smem::align16(8 * (n_free + 2 * n_planets + 1));
        off_gfull = o; o += Smem::align16(8 * n_full);
        off_ug = o;    o += Smem::align16(8 * 5 * np);
        off_misc = o;  o += 64;
        off_r = o;     o += Smem::align16(4 * tile);
        off_l = o;     o += Smem::align16(4 * tile);
        group_bytes = Smem::align16(o);
        total = tile_bytes + G * group_bytes;
    }
};

// gradient of a prior term (Normal, Beta; constant priors give 0)
__device__ __forceinline__ double prior_var_grad(const emp_prior& p, double x) {
    if (p.kind == EMP_PRIOR_NORMAL) return -(x - p.a0) * p.a1 * p.a1;
    if (p.kind == EMP_PRIOR_BETA) return (p.a0 - 1.0) / x - (p.a1 - 1.0) / (1.0 - x);
    if (p.kind == EMP_PRIOR_ISOTROPIC) return cos(x) / sin(x);
    return 0.0;
}

// Planet constants of the adjoint kernel, formed in FP64 from the planet's
// elements and split into float-float pairs (a rounded constant would shift
// every epoch's model alike, an error that adds up coherently in the
// gradient sums): [0..15] as planet_consts_mixed, [16] = K sin w,
// [17] = sqrt(1 - e^2), [18] = 1 - e^2.
__device__ __forceinline__ void grad_planet_consts(int par, const double* v, float* pc) {
    const Elements el = planet_elements(par, v);
    const double f = 1.0 / el.per;
    double cyc = el.use_tp ? -el.tp * f : el.phase * (1.0 / kTwoPi);
    cyc -= rint(cyc);
    const double q2 = fma(-el.e, el.e, 1.0);
    const double q = sqrt(q2);
    const double A = el.K * el.cw;
    split_ff(f, pc[0], pc[1]);
    split_ff(cyc, pc[2], pc[3]);
    split_ff(el.e, pc[4], pc[8]);
    split_ff(A, pc[5], pc[9]);
    split_ff(el.K * q * el.sw, pc[6], pc[10]);
    split_ff(A * el.e, pc[7], pc[11]);
    const float ef = pc[4];
    const float den = __fdividef(1.f, 4.f * ef + 0.5f);
    const float a = (1.f - ef) * den;
    pc[12] = a;
    pc[13] = a * a * a;
    pc[14] = 0.5f * den;
    pc[15] = __fdividef(0.078f, 1.f + ef);
    pc[16] = (float)(el.K * el.sw);
    pc[17] = (float)q;
    pc[18] = (float)q2;
}

// Chain rule of one planet (FP64): u = (sum lambda' dRV/dM, sum lambda' dRV/dM t,
// sum lambda' dRV/dA, sum lambda' dRV/dB, sum lambda' dRV/de) to the
// gradient with respect to its block's slots gf[0..4] (written; the two
// magnetic-cycle terms share one block, so the caller adds them up).
// M = 2 pi f t + phase or 2 pi f (t - tp), f = 1 / period.
__device__ __forceinline__ void grad_planet_chain(int par, const double* v, const double* u, double* gf) {
    const double SM = u[0], SMt = u[1], SA = u[2], SB = u[3], SE = u[4];
#pragma unroll
    for (int j = 0; j < 5; ++j) gf[j] = 0.0;
    const Elements el = planet_elements(par, v);
    const double f = 1.0 / el.per;
    const double tp = el.use_tp ? el.tp : 0.0;
    const double dLdf = kTwoPi * (SMt - tp * SM);
    const double dLdK = SA * el.cw + SB * el.sw;
    const double dLdw = el.K * (SB * el.cw - SA * el.sw);
    if (par == EMP_TERM_SINUSOID) {                     // (P, A, phase)
        gf[0] += -dLdf * f * f;
        gf[1] += SA;
        gf[2] += SM;
        return;
    }
    if (par == EMP_TERM_CYCLE_1) {                      // per' = 2 P: df/dP = -2 f^2
        gf[0] += -2.0 * dLdf * f * f;
        gf[1] += SA;
        gf[3] += SM;
        return;
    }
    if (par == EMP_TERM_CYCLE_2) {
        gf[0] += -dLdf * f * f;
        gf[2] += SA;
        gf[4] += SM;
        return;
    }
    double g0 = -dLdf * f * f;                          // d/dP
    if (par == 2 || par == 6 || par == 7) g0 *= el.per; // d/d ln P
    gf[0] += g0;
    if (par == 2) {
        // K = As^2 + Ac^2, phase = the angle of (Ac, As)
        const double As = v[1], Ac = v[2], K = el.K;
        gf[1] += dLdK * 2.0 * As + SM * Ac / K;
        gf[2] += dLdK * 2.0 * Ac - SM * As / K;
    } else {
        gf[1] += dLdK;
        gf[2] += el.use_tp ? -kTwoPi * f * SM : SM;
    }
    if (par == 0 || par == 3 || par == 6) {
        gf[3] += SE;
        gf[4] += dLdw;
    } else {
        // (S, C): e = S^2 + C^2, cos w = C / sqrt(e), sin w = S / sqrt(e)
        const double S = v[3], C = v[4], e = el.e;
        const double thr = (par == 2 || par == 4) ? 1e-5 : 1e-6;
        double gS = 2.0 * S * SE, gC = 2.0 * C * SE;
        if (e >= thr) {
            const double r3 = el.K / (e * sqrt(e));
            gS += SA * (-C * S * r3) + SB * (C * C * r3);
            gC += SA * (S * S * r3) + SB * (-S * C * r3);
        }
        gf[3] += gS;
        gf[4] += gC;
    }
}

template <int Q, int L, int NT>
__global__ void __launch_bounds__(NT) k_grad(GArgs A) {
    constexpr int G = NT / L;
    constexpr int NQ = Q > 0 ? Q : 1;
    constexpr int NE = 4;
    constexpr int NP = NE / 2;
    constexpr int IW = kGInsW;
    constexpr int KI = kGradMaxIns;
    constexpr int MS = NQ + NQ * NQ;
    constexpr int WL = L < 32 ? L : 32;
    extern __shared__ __align__(16) unsigned char smem[];

    const emp_model_desc* md = A.md;
    const int n_full = md->n_full, n_free = md->n_free, n_planets = md->n_planets;
    const int n_ins = md->n_ins, acc_order = md->acc_order;
    const int n = A.d.n;
    const int tile = A.tile;
    GSmem lay;
    lay.build(Q, L, G, tile, n_full, n_free, n_planets, n_ins, acc_order);

    const int tid = threadIdx.x;
    const int g = tid / L;
    const int r = tid - g * L;
    const int lw = r & (WL - 1);
    const int wk = blockIdx.x * G + g;
    const bool active = wk < A.nwalk;
    unsigned char* gs = smem + lay.tile_bytes + g * lay.group_bytes;
    double* full = reinterpret_cast<double*>(gs + lay.off_full);
    float* pcs = reinterpret_cast<float*>(gs + lay.off_pc);
    float* insc = reinterpret_cast<float*>(gs + lay.off_ins);
    double* accc = reinterpret_cast<double*>(gs + lay.off_acc);
    double* red = reinterpret_cast<double*>(gs + lay.off_red);
    float* scan = reinterpret_cast<float*>(gs + lay.off_scan);
    double* pterm = reinterpret_cast<double*>(gs + lay.off_pterm);
    double* gfull = reinterpret_cast<double*>(gs + lay.off_gfull);
    double* ug = reinterpret_cast<double*>(gs + lay.off_ug);
    double* misc = reinterpret_cast<double*>(gs + lay.off_misc);
    int* flag = reinterpret_cast<int*>(misc + 4);
    float* rb = reinterpret_cast<float*>(gs + lay.off_r);
    float* lb = reinterpret_cast<float*>(gs + lay.off_l);
    float* s_th = reinterpret_cast<float*>(smem);
    float* s_tl = s_th + tile;
    float* s_y = s_tl + tile;
    float* s_yl = s_y + tile;
    float* s_s2 = s_yl + tile;
    int* s_in = reinterpret_cast<int*>(s_s2 + tile);
    float* s_dt = reinterpret_cast<float*>(s_in + tile);

    // ---------------- theta, prior and its gradient, constants -------------
    if (active) {
        if (r == 0) flag[0] = 0;
        for (int s = r; s < n_full; s += L) {
            const int src = md->full_src[s];
            const double v = src >= 0 ? A.theta[(size_t)wk * n_free + src] : md->full_fixed[s];
            full[s] = v;
            gfull[s] = 0.0;
        }
        for (int j = r; j < 5 * n_planets; j += L) ug[j] = 0.0;
    }
    __syncthreads();
    if (active) {
        for (int d = r; d < n_free; d += L) {
            const emp_prior& p = md->prior[d];
            const double x = full[md->prior_slot[d]];
            double gp = 0.0;
            if (!in_support(x, p.lo, p.hi)) flag[0] = 1;
            else if (prior_varies(p.kind)) {
                pterm[d] = prior_var_term(p, x);
                gp = prior_var_grad(p, x);
            }
            A.grad_logprior[(size_t)wk * n_free + d] = gp;
        }
        for (int p = r; p < n_planets; p += L)
            grad_planet_consts(md->kep_param[p], full + md->kep_slot[p], pcs + p * kGPC);
        for (int k = r; k < n_ins; k += L) {
            float* ic = insc + k * IW;
            const double off = md->offset_slot >= 0 ? full[md->offset_slot + k] : 0.0;
            const float jf = (float)(md->jitter_slot >= 0 ? full[md->jitter_slot + k] : 0.0);
            ic[0] = (float)off;
            ic[1] = jf * jf;
            ic[2] = (float)(off - (double)(float)off);
            ic[3] = jf;
#pragma unroll
            for (int c = 0; c < Q; ++c) {
                const int base = md->ma_global ? md->ma_slot + 2 * c : md->ma_slot + 2 * Q * k + 2 * c;
                const float tau = (float)full[base + 1];
                ic[4 + 3 * c] = (float)full[base];
                ic[5 + 3 * c] = -1.44269504f / tau;
                ic[6 + 3 * c] = tau;
            }
        }
        for (int j = r; j < acc_order; j += L) accc[j] = full[md->acc_slot + j];
    }
    __syncthreads();
    if (active) {
        // derived priors (value and gradient through th[3], th[4] or th[1], th[2])
        for (int q2 = r; q2 < 2 * n_planets; q2 += L) {
            const int p = q2 >> 1, k = q2 & 1;
            const emp_prior& dp = md->derived[p][k];
            if (dp.kind == EMP_PRIOR_NONE) continue;
            const double* th = full + md->kep_slot[p];
            const double x = derived_x(th, k);
            if (!in_support(x, dp.lo, dp.hi)) { flag[0] = 1; continue; }
            if (prior_varies(dp.kind)) {
                pterm[n_free + q2] = prior_var_term(dp, x);
                const double gx = prior_var_grad(dp, x);
                const int i0 = k == 0 ? 3 : 1;
                for (int m = 0; m < 2; ++m) {
                    const int slot = md->kep_slot[p] + i0 + m;
                    const int src = md->full_src[slot];
                    if (src >= 0) atomicAdd(&A.grad_logprior[(size_t)wk * n_free + src], gx * 2.0 * th[i0 + m]);
                }
            }
        }
    }
    __syncthreads();
    if (active && r == 0) {
        double lp = -INFINITY;
        if (flag[0] == 0 && (md->hill_mask == 0 || hill_stable(md, full))) {
            lp = md->prior_const;
            for (int i = 0; i < md->n_prior_var; ++i) lp += pterm[md->prior_var[i]];
        }
        misc[0] = lp;
    }
    __syncthreads();
    const double lp = active ? misc[0] : -INFINITY;
    const bool valid = active && lp > -INFINITY;
    const double t0 = A.d.t0;
    const int ntiles = (n + tile - 1) / tile;
    const bool multi = ntiles > 1;
    float* rrow = A.resid != nullptr ? A.resid + (size_t)wk * A.resid_stride : nullptr;

    auto posof = [&](int C, int rr, int kk) { return kk * L + ((rr + kk) & (L - 1)); };
    auto tile_n = [&](int ti) { return min(tile, n - ti * tile); };
    auto stage = [&](int base, int nt) {
        const int C = (nt + L - 1) / L;
        for (int idx = tid; idx < nt; idx += NT) {
            const int rr = idx / C;
            const int kk = idx - rr * C;
            const int pos = kk * L + ((rr + kk) & (L - 1));
            const int gi = base + idx;
            s_th[pos] = A.d.t_hi[gi];
            s_tl[pos] = A.d.t_lo[gi];
            s_y[pos] = A.d.y32[gi];
            s_yl[pos] = A.d.y_lo[gi];
            s_s2[pos] = A.d.s2_32[gi];
            s_in[pos] = A.d.inst[gi];
#pragma unroll
            for (int c = 0; c < Q; ++c) s_dt[c * tile + pos] = A.d.dt32[(size_t)c * n + gi];
        }
    };
    // MA coefficient a_{c,i} = Phi exp(-dt/tau) from an epoch's gap and instrument
    auto ma_a = [&](float dt, int ins, int c, float& ef) -> float {
        const float* ic = insc + ins * IW;
        ef = ex2_fast(dt * ic[5 + 3 * c]);
        return ic[4 + 3 * c] * ef;
    };
    // coefficient of the epoch idx (tile-relative, may lie in the next tile)
    auto a_at = [&](int base, int nt, int C, int idx, int c, float& ef) -> float {
        if (idx < nt) {
            const int rr = idx / C, kk = idx - rr * C;
            const int ps = posof(C, rr, kk);
            return ma_a(s_dt[c * tile + ps], s_in[ps], c, ef);
        }
        const int gi = base + idx;
        if (gi >= n) { ef = 0.f; return 0.f; }
        return ma_a(A.d.dt32[(size_t)c * n + gi], A.d.inst[gi], c, ef);
    };
    // residual of the epoch idx (tile-relative, may lie in an earlier tile)
    auto r_at = [&](int base, int C, int idx) -> float {
        if (idx >= 0) {
            const int rr = idx / C, kk = idx - rr * C;
            return rb[posof(C, rr, kk)];
        }
        const int gi = base + idx;
        if (gi < 0 || rrow == nullptr) return 0.f;
        const int b2 = (gi / tile) * tile;
        const int n2 = tile_n(gi / tile);
        const int C2 = (n2 + L - 1) / L;
        const int i2 = gi - b2, rr = i2 / C2, kk = i2 - rr * C2;
        return rrow[b2 + posof(C2, rr, kk)];
    };

    // per-lane noise-model gradient sums (kept across tiles)
    LaneAcc<EMP_PREC_MIXED> g_off[KI], g_jit[KI], g_phi[KI][NQ], g_tau[KI][NQ];
#pragma unroll
    for (int k = 0; k < KI; ++k) {
        g_off[k].init(); g_jit[k].init();
#pragma unroll
        for (int c = 0; c < NQ; ++c) { g_phi[k][c].init(); g_tau[k][c].init(); }
    }
    LaneAcc<EMP_PREC_MIXED> lacc;
    lacc.init();

    // gradient terms of one staged tile from lambda' = dL/dmodel in lb
    auto tile_terms = [&](int nt) {
        const int C = (nt + L - 1) / L;
        const int nr = max(0, min(C, nt - r * C));
        for (int p = 0; p < n_planets; ++p) {
            const float* pc = pcs + p * kGPC;
            LaneAcc<EMP_PREC_MIXED> gM, gMt, gA, gB, gE;
            gM.init(); gMt.init(); gA.init(); gB.init(); gE.init();
            if (valid) {
                const float ec = pc[4], el = pc[8], Ah = pc[5], Bqh = pc[6], Bh = pc[16];
                const float q = pc[17], q2 = pc[18];
                const float eoq = q > 0.f ? ec / q : 0.f;
                for (int k0 = 0; k0 < nr; k0 += NE) {
                    float2 th2[NP], tl2[NP], lam2[NP];
#pragma unroll
                    for (int j = 0; j < NP; ++j) {
                        int ps[2];
                        float lv[2];
#pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            const int e = 2 * j + h;
                            const int kk = k0 + e < nr ? k0 + e : nr - 1;
                            ps[h] = posof(C, r, kk);
                            lv[h] = k0 + e < nr ? lb[ps[h]] : 0.f;
                        }
                        th2[j] = make_float2(s_th[ps[0]], s_th[ps[1]]);
                        tl2[j] = make_float2(s_tl[ps[0]], s_tl[ps[1]]);
                        lam2[j] = make_float2(lv[0], lv[1]);
                    }
                    float2 M[NP], ml[NP], sn[NP], cs[NP];
#pragma unroll
                    for (int j = 0; j < NP; ++j) M[j] = mean_anomaly_pair(pc, th2[j], tl2[j], ml[j]);
                    kepler_pairs<NP>(M, ml, ec, el, pc + 12, sn, cs);
                    float2 tM = bc2(0.f), tMt = bc2(0.f), tA = bc2(0.f), tB = bc2(0.f), tE = bc2(0.f);
#pragma unroll
                    for (int j = 0; j < NP; ++j) {
                        const float2 D = fma2(bc2(-el), cs[j], fma2(bc2(-ec), cs[j], bc2(1.f)));
                        const float2 iD = rcp_nr2(D);
                        const float2 iD2 = mul2(iD, iD);
                        const float2 cme = sub2(cs[j], bc2(ec));
                        // dRV/dE = -(A sin E (1 - e^2) + B q (cos E - e)) / D^2
                        const float2 dE = mul2(fma2(bc2(-Ah * q2), sn[j], mul2(bc2(-Bqh), cme)), iD2);
                        const float2 dM = mul2(dE, iD);
                        const float2 dA = fma2(cme, iD, bc2(ec));
                        const float2 dB = mul2(mul2(bc2(-q), sn[j]), iD);
                        // dRV/de at fixed M: explicit part plus dRV/dE sin E / D
                        const float2 s2 = mul2(sn[j], sn[j]);
                        const float2 ex1 = mul2(bc2(Ah), fma2(mul2(s2, iD2), bc2(-1.f), bc2(1.f)));
                        const float2 ex2 = mul2(mul2(bc2(-Bh), sn[j]),
                                                mul2(fma2(bc2(q), cs[j], mul2(bc2(-eoq), D)), iD2));
                        const float2 de = fma2(mul2(dE, sn[j]), iD, add2(ex1, ex2));
                        const float2 lm = lam2[j];
                        const float2 t = add2(th2[j], tl2[j]);
                        const float2 a = mul2(lm, dM);
                        tM = add2(tM, a);
                        tMt = fma2(a, t, tMt);
                        tA = fma2(lm, dA, tA);
                        tB = fma2(lm, dB, tB);
                        tE = fma2(lm, de, tE);
                    }
                    gM.add(tM.x + tM.y);
                    gMt.add(tMt.x + tMt.y);
                    gA.add(tA.x + tA.y);
                    gB.add(tB.x + tB.y);
                    gE.add(tE.x + tE.y);
                }
            }
            // the tile's five sums accumulate across tiles as float-float pairs
            // (FP64 instructions only in the chain rule at the end)
            const LaneAcc<EMP_PREC_MIXED>* gv[5] = {&gM, &gMt, &gA, &gB, &gE};
            FF* ugf = reinterpret_cast<FF*>(ug);
#pragma unroll
            for (int j = 0; j < 5; ++j) {
                const FF sj = gv[j]->template group_sum_ff<L>();
                if (r == 0 && valid) ugf[p * 5 + j] = ff_add(ugf[p * 5 + j], sj);
            }
            __syncwarp();
        }
        for (int j = 0; j < acc_order; ++j) {
            LaneAcc<EMP_PREC_MIXED> ga;
            ga.init();
            if (valid) {
                for (int kk = 0; kk < nr; ++kk) {
                    const int ps = posof(C, r, kk);
                    const float x = (s_th[ps] - (float)t0) + s_tl[ps];
                    float pw = 1.f;
                    for (int m = 0; m < acc_order - j; ++m) pw *= x;
                    ga.add(lb[ps] * pw);
                }
            }
            const double sj = ga.template group_sum<L>(red, r);
            if (r == 0 && valid) gfull[md->acc_slot + j] += sj;
            if (L <= 32) __syncwarp();
            else __syncthreads();
        }
    };

    // ================= forward: model, residuals, log L =====================
    float carry[NQ];                       // r_{base-1-m}: residuals before the tile
#pragma unroll
    for (int m = 0; m < NQ; ++m) carry[m] = 0.f;
    for (int ti = 0; ti < ntiles; ++ti) {
        const int base = ti * tile, nt = tile_n(ti);
        const int C = (nt + L - 1) / L;
        const int nr = max(0, min(C, nt - r * C));
        __syncthreads();
        stage(base, nt);
        __syncthreads();
        float xh[NQ], gh[NQ][NQ];
#pragma unroll
        for (int m = 0; m < NQ; ++m) {
            xh[m] = 0.f;
#pragma unroll
            for (int q2 = 0; q2 < NQ; ++q2) gh[m][q2] = m == q2 ? 1.f : 0.f;
        }
        if (valid) {
            for (int k0 = 0; k0 < nr; k0 += NE) {
                int pos[NE];
                bool ok[NE];
                float th[NE], tl[NE];
#pragma unroll
                for (int e = 0; e < NE; ++e) {
                    const int kk = k0 + e < nr ? k0 + e : nr - 1;
                    ok[e] = k0 + e < nr;
                    pos[e] = posof(C, r, kk);
                    th[e] = s_th[pos[e]];
                    tl[e] = s_tl[pos[e]];
                }
                float2 th2[NP], tl2[NP], mh[NP], mlo2[NP];
#pragma unroll
                for (int j = 0; j < NP; ++j) {
                    th2[j] = make_float2(th[2 * j], th[2 * j + 1]);
                    tl2[j] = make_float2(tl[2 * j], tl[2 * j + 1]);
                    mh[j] = bc2(0.f);
                    mlo2[j] = bc2(0.f);
                }
                for (int p = 0; p < n_planets; ++p) {
                    const float* pc = pcs + p * kGPC;
                    float2 M[NP], ml[NP], sn[NP], cs[NP];
#pragma unroll
                    for (int j = 0; j < NP; ++j) M[j] = mean_anomaly_pair(pc, th2[j], tl2[j], ml[j]);
                    const float ec = pc[4], el = pc[8];
                    kepler_pairs<NP>(M, ml, ec, el, pc + 12, sn, cs);
#pragma unroll
                    for (int j = 0; j < NP; ++j) {
                        const float2 cme = sub2(sub2(cs[j], bc2(ec)), bc2(el));
                        const float2 inv = rcp_nr2(fma2(bc2(-el), cs[j], fma2(bc2(-ec), cs[j], bc2(1.f))));
                        const float2 hi = fma2(fma2(bc2(pc[5]), cme, mul2(bc2(-pc[6]), sn[j])), inv, bc2(pc[7]));
                        const float2 lo = fma2(fma2(bc2(pc[9]), cme, mul2(bc2(-pc[10]), sn[j])), inv, bc2(pc[11]));
                        // the model as a float-float sum over planets
                        const float2 s = add2(mh[j], hi);
                        const float2 bb = sub2(s, mh[j]);
                        const float2 err = add2(sub2(mh[j], sub2(s, bb)), sub2(hi, bb));
                        mh[j] = s;
                        mlo2[j] = add2(mlo2[j], add2(err, lo));
                    }
                }
                float model[NE], mlo[NE];
#pragma unroll
                for (int j = 0; j < NP; ++j) {
                    model[2 * j] = mh[j].x; model[2 * j + 1] = mh[j].y;
                    mlo[2 * j] = mlo2[j].x; mlo[2 * j + 1] = mlo2[j].y;
                }
#pragma unroll
                for (int e = 0; e < NE; ++e) {
                    if (!ok[e]) continue;
                    if (acc_order > 0) {
                        const float x = (th[e] - (float)t0) + tl[e];
                        float pv = 0.f;
                        for (int j = 0; j < acc_order; ++j) pv = pv * x + (float)accc[j];
                        mlo[e] += pv * x;
                    }
                    const int ps = pos[e];
                    const int ki = s_in[ps];
                    const float* ic = insc + ki * IW;
                    const float b = ((s_y[ps] - ic[0]) - model[e]) + ((s_yl[ps] - ic[2]) - mlo[e]);
                    if (Q == 0) {
                        const float err2 = s_s2[ps] + ic[1];
                        const float w = rcp_nr(err2);
                        const float lam = w * b;                      // dL/dmodel
                        lb[ps] = lam;
                        lacc.add(lam * b + lg2_fast(err2) * 0.69314718055994531f);
                        const float gj = (w * w * b * b - w) * ic[3];
#pragma unroll
                        for (int k = 0; k < KI; ++k)
                            if (k == ki) { g_off[k].add(lam); g_jit[k].add(gj); }
                    } else {
                        rb[ps] = b;
                        float x = b, gn[NQ];
#pragma unroll
                        for (int q2 = 0; q2 < NQ; ++q2) gn[q2] = 0.f;
#pragma unroll
                        for (int c = 0; c < Q; ++c) {
                            float ef;
                            const float a = ma_a(s_dt[c * tile + ps], ki, c, ef);
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
                    }
                }
            }
        }
        if (Q == 0) {
            __syncthreads();
            tile_terms(nt);
            continue;
        }
        // join the lane chunks: inclusive scan of the maps u -> G u + x, then
        // the incoming state of each lane from the tile's incoming state
        float u[NQ];
        {
            float mv[MS];
#pragma unroll
            for (int m = 0; m < NQ; ++m) {
                mv[m] = xh[m];
#pragma unroll
                for (int q2 = 0; q2 < NQ; ++q2) mv[NQ + m * NQ + q2] = gh[m][q2];
            }
#pragma unroll
            for (int off = 1; off < WL; off <<= 1) {
                float pv[MS];
#pragma unroll
                for (int k = 0; k < MS; ++k) pv[k] = __shfl_up_sync(0xffffffffu, mv[k], off, WL);
                if (lw >= off) map_compose<float, NQ>(mv, pv);
            }
            float ex[MS];
#pragma unroll
            for (int k = 0; k < MS; ++k) ex[k] = __shfl_up_sync(0xffffffffu, mv[k], 1, WL);
            if (lw == 0) map_identity<float, NQ>(ex);
            float wpre[MS];
            map_identity<float, NQ>(wpre);
            if (L > 32) {
                if (lw == WL - 1) {
#pragma unroll
                    for (int k = 0; k < MS; ++k) scan[(r >> 5) * MS + k] = mv[k];
                }
                __syncthreads();
                for (int k = 0; k < (r >> 5); ++k) map_compose_left<float, NQ>(scan + k * MS, wpre);
                __syncthreads();
            }
            float cw_[NQ];
            map_apply<float, NQ>(wpre, carry, cw_);
            map_apply<float, NQ>(ex, cw_, u);
        }
        if (valid) {
            float hist[NQ];
#pragma unroll
            for (int m = 0; m < NQ; ++m) hist[m] = u[m];
            for (int kk = 0; kk < nr; ++kk) {
                const int ps = posof(C, r, kk);
                const int ki = s_in[ps];
                float x = rb[ps];
#pragma unroll
                for (int c = 0; c < Q; ++c) {
                    float ef;
                    x -= ma_a(s_dt[c * tile + ps], ki, c, ef) * hist[c];
                }
#pragma unroll
                for (int m = NQ - 1; m > 0; --m) hist[m] = hist[m - 1];
                hist[0] = x;
                rb[ps] = x;
                const float err2 = s_s2[ps] + insc[ki * IW + 1];
                lacc.add(x * x * rcp_nr(err2) + lg2_fast(err2) * 0.69314718055994531f);
            }
        }
        __syncthreads();
        // residuals before the next tile, most recent first
        float nc[NQ];
#pragma unroll
        for (int m = 0; m < NQ; ++m) {
            const int idx = nt - 1 - m;
            nc[m] = idx >= 0 ? r_at(base, C, idx) : carry[m - nt];
        }
#pragma unroll
        for (int m = 0; m < NQ; ++m) carry[m] = nc[m];
        if (multi && valid)
            for (int i = r; i < C * L; i += L) rrow[base + i] = rb[i];
    }
    const double sumL = lacc.template group_sum<L>(red, r);
    __syncthreads();

    // ================= backward (MA): adjoints, noise gradients ==============
    if (Q > 0) {
        float vcarry[NQ];                  // lambda_{end + m}: adjoints after the tile
#pragma unroll
        for (int m = 0; m < NQ; ++m) vcarry[m] = 0.f;
        for (int ti = ntiles - 1; ti >= 0; --ti) {
            const int base = ti * tile, nt = tile_n(ti);
            const int C = (nt + L - 1) / L;
            const int nr = max(0, min(C, nt - r * C));
            if (multi) {
                __syncthreads();
                stage(base, nt);
                if (valid)
                    for (int i = r; i < C * L; i += L) rb[i] = rrow[base + i];
                __syncthreads();
            }
            // per lane, backwards from a zero state after the chunk:
            // lambda_i = -w_i r_i - sum_c a_{c,i+1+c} lambda_{i+1+c}
            float lh[NQ], hh[NQ][NQ];
#pragma unroll
            for (int m = 0; m < NQ; ++m) {
                lh[m] = 0.f;
#pragma unroll
                for (int q2 = 0; q2 < NQ; ++q2) hh[m][q2] = m == q2 ? 1.f : 0.f;
            }
            if (valid) {
                for (int kk = nr - 1; kk >= 0; --kk) {
                    const int ps = posof(C, r, kk);
                    const float w = rcp_nr(s_s2[ps] + insc[s_in[ps] * IW + 1]);
                    float lam = -w * rb[ps];
                    float hn[NQ];
#pragma unroll
                    for (int q2 = 0; q2 < NQ; ++q2) hn[q2] = 0.f;
#pragma unroll
                    for (int c = 0; c < Q; ++c) {
                        float ef;
                        const float a = a_at(base, nt, C, r * C + kk + 1 + c, c, ef);
                        lam -= a * lh[c];
#pragma unroll
                        for (int q2 = 0; q2 < NQ; ++q2) hn[q2] -= a * hh[c][q2];
                    }
#pragma unroll
                    for (int m = NQ - 1; m > 0; --m) {
                        lh[m] = lh[m - 1];
#pragma unroll
                        for (int q2 = 0; q2 < NQ; ++q2) hh[m][q2] = hh[m - 1][q2];
                    }
                    lh[0] = lam;
#pragma unroll
                    for (int q2 = 0; q2 < NQ; ++q2) hh[0][q2] = hn[q2];
                }
            }
            // inclusive suffix scan S_r = map_r o S_{r+1}; incoming state of a
            // lane = the exclusive suffix applied to the tile's state after it
            float v[NQ];
            {
                float mv[MS];
#pragma unroll
                for (int m = 0; m < NQ; ++m) {
                    mv[m] = lh[m];
#pragma unroll
                    for (int q2 = 0; q2 < NQ; ++q2) mv[NQ + m * NQ + q2] = hh[m][q2];
                }
#pragma unroll
                for (int off = 1; off < WL; off <<= 1) {
                    float pv[MS];
#pragma unroll
                    for (int k = 0; k < MS; ++k) pv[k] = __shfl_down_sync(0xffffffffu, mv[k], off, WL);
                    if (lw + off < WL) map_compose<float, NQ>(mv, pv);
                }
                float ex[MS];
#pragma unroll
                for (int k = 0; k < MS; ++k) ex[k] = __shfl_down_sync(0xffffffffu, mv[k], 1, WL);
                if (lw == WL - 1) map_identity<float, NQ>(ex);
                float wsuf[MS];
                map_identity<float, NQ>(wsuf);
                if (L > 32) {
                    if (lw == 0) {
#pragma unroll
                        for (int k = 0; k < MS; ++k) scan[(r >> 5) * MS + k] = mv[k];
                    }
                    __syncthreads();
                    for (int k = L / 32 - 1; k > (r >> 5); --k) map_compose_left<float, NQ>(scan + k * MS, wsuf);
                    __syncthreads();
                }
                float cw_[NQ];
                map_apply<float, NQ>(wsuf, vcarry, cw_);
                map_apply<float, NQ>(ex, cw_, v);
            }
            if (valid) {
                float st[NQ];
#pragma unroll
                for (int m = 0; m < NQ; ++m) st[m] = v[m];
                for (int kk = nr - 1; kk >= 0; --kk) {
                    const int ps = posof(C, r, kk);
                    const int ki = s_in[ps];
                    const float* ic = insc + ki * IW;
                    const float w = rcp_nr(s_s2[ps] + ic[1]);
                    const float ri = rb[ps];
                    float lam = -w * ri;
#pragma unroll
                    for (int c = 0; c < Q; ++c) {
                        float ef;
                        lam -= a_at(base, nt, C, r * C + kk + 1 + c, c, ef) * st[c];
                    }
                    lb[ps] = -lam;                                   // dL/dmodel
                    const float gj = (w * w * ri * ri - w) * ic[3];
                    float gp[NQ], gt[NQ];
#pragma unroll
                    for (int c = 0; c < NQ; ++c) { gp[c] = 0.f; gt[c] = 0.f; }
#pragma unroll
                    for (int c = 0; c < Q; ++c) {
                        float ef;
                        const float dt = s_dt[c * tile + ps];
                        const float a = ma_a(dt, ki, c, ef);
                        if (ef > 0.f) {
                            const float rp = r_at(base, C, r * C + kk - 1 - c);
                            const float tau = ic[6 + 3 * c];
                            gp[c] = -lam * rp * ef;
                            gt[c] = -lam * rp * a * dt / (tau * tau);
                        }
                    }
#pragma unroll
                    for (int k = 0; k < KI; ++k) {
                        if (k == ki) {
                            g_off[k].add(-lam);
                            g_jit[k].add(gj);
#pragma unroll
                            for (int c = 0; c < Q; ++c) { g_phi[k][c].add(gp[c]); g_tau[k][c].add(gt[c]); }
                        }
                    }
#pragma unroll
                    for (int m = NQ - 1; m > 0; --m) st[m] = st[m - 1];
                    st[0] = lam;
                }
            }
            __syncthreads();
            // adjoints of the tile's first epochs carry to the earlier tile
            float nv[NQ];
#pragma unroll
            for (int m = 0; m < NQ; ++m) {
                if (m < nt) {
                    const int rr = m / C, kk = m - rr * C;
                    nv[m] = -lb[posof(C, rr, kk)];
                } else {
                    nv[m] = vcarry[m - nt];
                }
            }
#pragma unroll
            for (int m = 0; m < NQ; ++m) vcarry[m] = nv[m];
            tile_terms(nt);
        }
    }

    // ---------------- noise-model gradients into gfull --------------------
    for (int k = 0; k < min(n_ins, KI); ++k) {
        const double s_off = g_off[k].template group_sum<L>(red, r);
        const double s_jit = g_jit[k].template group_sum<L>(red, r);
        if (r == 0 && valid) {
            if (md->offset_slot >= 0) gfull[md->offset_slot + k] += s_off;
            if (md->jitter_slot >= 0) gfull[md->jitter_slot + k] += s_jit;
        }
#pragma unroll
        for (int c = 0; c < Q; ++c) {
            const double s_phi = g_phi[k][c].template group_sum<L>(red, r);
            const double s_tau = g_tau[k][c].template group_sum<L>(red, r);
            if (r == 0 && valid) {
                const int base = md->ma_global ? md->ma_slot + 2 * c : md->ma_slot + 2 * Q * k + 2 * c;
                gfull[base] += s_phi;
                gfull[base + 1] += s_tau;
            }
        }
        __syncthreads();
    }
    // ---------------- planets: chain rule to theta -------------------------
    __syncthreads();
    if (valid)
        for (int p = r; p < n_planets; p += L) {
            const FF* ugf = reinterpret_cast<const FF*>(ug);
            double u5[5], o[5];
#pragma unroll
            for (int j = 0; j < 5; ++j) u5[j] = (double)ugf[p * 5 + j].hi + (double)ugf[p * 5 + j].lo;
            grad_planet_chain(md->kep_param[p], full + md->kep_slot[p], u5, o);
#pragma unroll
            for (int j = 0; j < 5; ++j) ug[p * 5 + j] = o[j];
        }
    __syncthreads();
    if (valid && r == 0)
        for (int p = 0; p < n_planets; ++p) {
            const int nb = md->kep_param[p] == EMP_TERM_SINUSOID ? 3 : 5;   // slots of the block
            for (int j = 0; j < nb; ++j) gfull[md->kep_slot[p] + j] += ug[p * 5 + j];
        }
    __syncthreads();

    // ---------------- outputs ---------------------------------------------
    if (active) {
        if (r == 0) {
            A.logl[wk] = valid ? -0.5 * sumL + md->loglike_const : -INFINITY;
            A.logprior[wk] = lp;
        }
        for (int d = r; d < n_free; d += L)
            A.grad_logl[(size_t)wk * n_free + d] = valid ? gfull[md->prior_slot[d]] : 0.0;
    }
}

}  // namespace emp
