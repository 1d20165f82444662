// emp_am.cuh -- astrometric term of the joint RV + astrometry likelihood.
//
// support/likelihoods/a00.like adds loglike_AM(theta) to the RV Gaussian
// log-likelihood; its functions are written by ReddModel._write_model_AM
// (emp_model.py:1232-1675) with the helpers of support/astrometry/
// constants.scr.  Per walker row:
//   * the barycentre at the Hipparcos epoch (model_barycenter /
//     obs_lin_prop_PA): the DR3 solution minus the five offsets, propagated
//     linearly in Cartesian coordinates; at the DR3 epoch the propagation
//     time is zero and the barycentre is that solution itself, used as
//     offsets from the DR3 position;
//   * every Keplerian's sky-plane offsets at every Hipparcos and Gaia scan
//     epoch (calc_astro_new: Kepler solve, Thiele-Innes constants), lanes
//     over epochs;
//   * Hipparcos: along-scan abscissae against the residuals, iid Gaussian
//     with the jitter added in quadrature (compute_abs_signal_hipp);
//   * Gaia: the abscissae of each release's scans projected on its
//     five-parameter solution vectors (the pseudo-inverse of its design
//     matrix), compared with the catalogue solution under its covariance
//     scaled by the jitter squared (compute_abs_signal_gost,
//     gaussian_loglike_mvn).
// Everything is FP64 in both precisions.  The reference handles absolute
// positions in degrees (one FP64 ulp of 60 degrees is 2.5e-8 mas, and the
// Gaia term is sensitive at that level); here the scan positions are formed
// as offsets from the DR3 position, which keeps them to ~1e-16 of the
// offsets themselves.  k_logpost has written the RV part (logL of the row,
// or for a stretch half-step the proposal, its prior and RV logL); this
// kernel adds the astrometric term and finishes the mode (gp_finish).
#pragma once
#include "emp_gp.cuh"

namespace emp {

constexpr double kMasPerDeg = 3.6e6;
constexpr double kDayPerYear = 365.25;
constexpr double kPc2Au = 206265.0;
constexpr double kAuYr2Kms = 4.74047;
constexpr double kLog2Pi = 1.8378770664093453;
constexpr int kAmPC = 12;                      // doubles per planet

struct AmSmem {                                // per warp
    double full[EMP_MAX_PARAMS];
    double pc[EMP_MAX_PLANETS][kAmPC];
    double bary[1][6];                         // the Hipparcos epoch
};

// one catalogue epoch of the barycentre: ra, dec (deg), parallax, pmra,
// pmdec, rv (obs_lin_prop_PA on the DR3 solution minus the offsets)
__device__ inline void am_barycentre(const AmDev& d, const double* off, int c, double* out) {
    const double* ref = d.catalogs + 2 * 7 + 1;          // DR3: ra, dec, plx, pmra, pmdec, rv
    const double RA = ref[0] - off[0] / kMasPerDeg / cos(ref[1] * (kPi / 180.0));
    const double DE = ref[1] - off[1] / kMasPerDeg;
    const double PLX = ref[2] - off[2], PMRA = ref[3] - off[3], PMDE = ref[4] - off[4], RV = ref[5];
    const double ra = RA * (kPi / 180.0), de = DE * (kPi / 180.0);
    double sinde, cosde, sinra, cosra;
    sincos(de, &sinde, &cosde);
    sincos(ra, &sinra, &cosra);
    const double dist = 1.0 / PLX;                       // kpc
    const double x = cosde * cosra * dist * 1e3, y = cosde * sinra * dist * 1e3, z = sinde * dist * 1e3;
    const double vra = PMRA * dist, vde = PMDE * dist, vr = RV / kAuYr2Kms;
    const double vx = vr * cosde * cosra - vde * sinde * cosra - vra * sinra;
    const double vy = vr * cosde * sinra - vde * sinde * sinra + vra * cosra;
    const double vz = vr * sinde + vde * cosde;
    const double tf = (d.catalogs[c * 7] - d.catalogs[2 * 7]) / (kDayPerYear * kPc2Au);
    const double x1 = x + vx * tf, y1 = y + vy * tf, z1 = z + vz * tf;
    double de1 = atan2(z1, sqrt(x1 * x1 + y1 * y1));
    if (de1 > kPi / 2) de1 -= kPi;
    double ra1 = atan2(y1, x1);
    ra1 = fmod(ra1, 2.0 * kPi);
    if (ra1 < 0.0) ra1 += 2.0 * kPi;
    const double d1 = sqrt(x1 * x1 + y1 * y1 + z1 * z1) * 1e-3;
    double s1, c1, sd1, cd1;
    sincos(ra1, &s1, &c1);
    sincos(de1, &sd1, &cd1);
    const double u0 = c1 * vx + s1 * vy, u1 = -s1 * vx + c1 * vy, u2 = vz;
    const double v0 = cd1 * u0 + sd1 * u2, v2 = -sd1 * u0 + cd1 * u2;
    out[0] = ra1 * (180.0 / kPi);
    out[1] = de1 * (180.0 / kPi);
    out[2] = 1.0 / d1;
    out[3] = u1 / d1;
    out[4] = v2 / d1;
    out[5] = v0 * kAuYr2Kms;
}

// per-planet constants: [0] 2 pi / P, [1] phase, [2] e, [3] sqrt(1 - e^2),
// [4..9] beta B, beta G, beta A, beta F, -beta C plx/206265e3, -beta H plx/206265e3
__device__ inline void am_planet(const double* v, double plx, double* pc) {
    const double per = v[0], K = v[1], pha = v[2], e = v[3], om = v[4], I = v[5], Om = v[6];
    double sI, cI, sO, cO, so, co;
    sincos(I, &sI, &cI);
    sincos(Om, &sO, &cO);
    sincos(om, &so, &co);
    const double A = co * cO - so * sO * cI, B = co * sO + so * cO * cI;
    const double F = -so * cO - co * sO * cI, G = -so * sO + co * cO * cI;
    const double C = so * sI, H = co * sI;
    const double sq = sqrt(1.0 - e * e);
    const double beta0 = per / kDayPerYear * (K / 1e3 / kAuYr2Kms) * sq / (2.0 * kPi) / sI;
    const double beta = -beta0 * plx;
    pc[0] = 2.0 * kPi / per;
    pc[1] = pha;
    pc[2] = e;
    pc[3] = sq;
    pc[4] = beta * B; pc[5] = beta * G;
    pc[6] = beta * A; pc[7] = beta * F;
    pc[8] = -beta * C * plx / 206265e3;
    pc[9] = -beta * H * plx / 206265e3;
}

// PREC = EMP_PREC_MIXED solves Kepler's equation of each planet-epoch in
// FP32 (kepler_f32_n: Halley iterations on the special function unit's
// sin/cos, then one Newton step with an accurate sin/cos and the low parts
// of the FP64-reduced mean anomaly and of e, E to ~1e-11); the
// orbit enters the abscissae through amplitudes of a few mas, so its error
// there stays below 1e-7 mas.  Everything else is FP64 in both precisions.
template <int PREC>
__global__ void __launch_bounds__(kAmThreads) k_am(KArgs A0) {
    // system blockIdx.y of a batch handle as a one-system launch
    KArgs A = sys_rows(A0, blockIdx.y);
    if (A0.sys_off != nullptr && A0.am_rv != nullptr) A.am_rv = A0.am_rv + (size_t)blockIdx.y * A0.nwalk;
    __shared__ AmSmem sm[kAmThreads / 32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rowr = blockIdx.x * (kAmThreads / 32) + warp;
    const bool live = rowr < A.nwalk;
    const int row = live ? rowr : A.nwalk - 1;
    const emp_model_desc* md = A.md;
    const AmDev d = A0.am_sys != nullptr ? A0.am_sys[blockIdx.y] : A0.am;
    AmSmem& S = sm[warp];
    const double* th;
    const double lp = gp_row(A, row, &th);
    const bool valid = live && (lp > -INFINITY);
    const double rv_ll = A.mode == kModeStretch ? A.am_rv[row]
                       : (A.mode == kModeSlots ? A.st_logl[row] : A.logl[row]);
    for (int s = lane; s < md->n_full; s += 32) {
        const int src = md->full_src[s];
        S.full[s] = src >= 0 ? th[src] : md->full_fixed[s];
    }
    __syncwarp();
    const double* off = S.full + md->am_offset_slot;
    const double plx0 = d.catalogs[2 * 7 + 3] - off[2];
    if (lane == 0) am_barycentre(d, off, 0, S.bary[0]);
    if (lane >= 8 && lane - 8 < md->n_planets) am_planet(S.full + md->kep_slot[lane - 8], plx0, S.pc[lane - 8]);
    __syncwarp();
    // Hipparcos: the barycentre at the Hipparcos epoch against its solution
    const double* hc = d.catalogs + 1;                    // Hipparcos ra, dec, plx, pmra, pmdec
    const double* b0 = S.bary[0];
    const double mean_dec = 0.5 * (hc[1] + b0[1]);
    const double dra_h = (b0[0] - hc[0]) * cos(mean_dec * (kPi / 180.0)) * kMasPerDeg;
    const double dde_h = (b0[1] - hc[1]) * kMasPerDeg;
    const double dplx_h = b0[2] - hc[2], dpmra_h = b0[3] - hc[3], dpmde_h = b0[4] - hc[4];
    // the barycentre at the DR3 epoch: model_barycenter propagates the DR3
    // solution minus the offsets over zero time, which returns it unchanged
    // (position, parallax, proper motion); taken as offsets from the DR3
    // position in degrees, without the round trip through Cartesian
    // coordinates that rounds ~60-degree angles
    const double* r3 = d.catalogs + 2 * 7;                // epoch, ra, dec, plx, pmra, pmdec
    const double ref_dec3 = r3[2], t3 = r3[0];
    const double dde3 = -off[1] / kMasPerDeg;
    const double dra3 = -off[0] / kMasPerDeg / cos(ref_dec3 * (kPi / 180.0));
    const double plx3 = r3[3] - off[2], pmra3 = r3[4] - off[3], pmde3 = r3[5] - off[4];
    const double dec3r = (ref_dec3 + dde3) * (kPi / 180.0);
    const double jh = S.full[md->am_jitter_slot], jg = S.full[md->am_jitter_slot + 1];
    const int nh = d.n_hipp, ng = d.n_gost;
    double sh = 0.0, pr[2][5];
#pragma unroll
    for (int c = 0; c < 2; ++c)
#pragma unroll
        for (int k = 0; k < 5; ++k) pr[c][k] = 0.0;
    if (valid) {
        for (int i = lane; i < nh + ng; i += 32) {
            const double t = i < nh ? d.hipp[i] : d.gost[i - nh];
            double c0 = 0.0, c1 = 0.0, c2 = 0.0;
            for (int p = 0; p < md->n_planets; ++p) {
                const double* pc = S.pc[p];
                const double M = pc[0] * (t - d.common_t) + pc[1];
                double Mr = fmod(M + kPi, kTwoPi);
                if (Mr < 0.0) Mr += kTwoPi;
                Mr -= kPi;
                double sE, cE;
                if constexpr (PREC == EMP_PREC_MIXED) {
                    const float mh = (float)Mr, eh = (float)pc[2];
                    const float M1[1] = {mh}, L1[1] = {(float)(Mr - (double)mh)};
                    float s1[1], c1[1];
                    kepler_f32_n<1>(M1, L1, eh, (float)(pc[2] - (double)eh), s1, c1);
                    sE = s1[0];
                    cE = c1[0];
                } else {
                    kepler_f64(Mr, pc[2], sE, cE);
                }
                const double X = cE - pc[2], Y = pc[3] * sE;
                c0 += pc[4] * X + pc[5] * Y;
                c1 += pc[6] * X + pc[7] * Y;
                c2 += pc[8] * X + pc[9] * Y;
            }
            if (i < nh) {
                const double ep = d.hipp[nh + i];
                const double ab = d.hipp[3 * nh + i] * (c0 + dra_h + dpmra_h * ep) +
                                  d.hipp[4 * nh + i] * (c1 + dde_h + dpmde_h * ep) + d.hipp[2 * nh + i] * dplx_h;
                const double r = d.hipp[5 * nh + i] - ab;
                const double sr = d.hipp[6 * nh + i];
                const double var = sr * sr + jh * jh;
                sh += r * r / var + log(var);
            } else {
                const int j = i - nh;
                const double tg = (t - t3) / kDayPerYear / 206265e3;
                const double decs = dec3r + pmde3 * tg;
                const double dras = pmra3 * tg / cos(decs);                 // ras - RA3, rad
                const double ddeg = dde3 + pmde3 * tg * (180.0 / kPi) + c1 / kMasPerDeg;
                const double dec = ref_dec3 + ddeg;
                const double dra = (dra3 + dras * (180.0 / kPi)) * cos(dec * (kPi / 180.0)) * kMasPerDeg + c0;
                const double ddec = ddeg * kMasPerDeg;
                const double dplx = plx3 + c2;
                const double ab = d.gost[ng + j] * ddec + d.gost[2 * ng + j] * dra + d.gost[3 * ng + j] * dplx;
#pragma unroll
                for (int c = 0; c < 2; ++c)
#pragma unroll
                    for (int k = 0; k < 5; ++k) pr[c][k] = fma(d.gsv[(c * 5 + k) * ng + j], ab, pr[c][k]);
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sh += __shfl_xor_sync(0xffffffffu, sh, o);
#pragma unroll
        for (int c = 0; c < 2; ++c)
#pragma unroll
            for (int k = 0; k < 5; ++k) pr[c][k] += __shfl_xor_sync(0xffffffffu, pr[c][k], o);
    }
    double ll = -INFINITY;
    if (valid) {
        ll = -0.5 * (sh + nh * kLog2Pi);
        const double jg2 = jg * jg;
        for (int c = 0; c < 2; ++c) {
            double r[5];
            for (int k = 0; k < 5; ++k) r[k] = d.astro_gost[c * 5 + k] - pr[c][k];
            const double* ic = d.inv_cov + (c + 1) * 25;
            double quad = 0.0;
            for (int a = 0; a < 5; ++a) {
                double s = 0.0;
                for (int b = 0; b < 5; ++b) s = fma(ic[a * 5 + b], r[b], s);
                quad = fma(r[a], s, quad);
            }
            ll += -0.5 * (quad / jg2 + 5.0 * log(jg2) + d.log_det_cov[c + 1] + 5.0 * kLog2Pi);
        }
        ll += rv_ll;
        if (!(ll > -INFINITY) || isnan(ll)) ll = -INFINITY;
    }
    gp_finish<32>(A, row, lane, live, valid, lp, th, ll);
}

}  // namespace emp
