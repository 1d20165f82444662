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
// k_logpost writes each valid row's residuals and err2 (epoch-major, so the
// threads of a warp -- one row each -- read consecutive addresses) and the
// prior; k_gp runs the recursion in FP64, one thread per row, and finishes the
// mode: log-posterior rows, state slots, or the stretch move's Metropolis test.
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

// log-likelihood of one row; r and e are the row's residuals and err2 with
// stride ld between epochs
template <int M>
__device__ double gp_loglike(const emp_model_desc* md, const double* th, const double* t, int n,
                             const double* r, const double* e, int ld) {
    double pa[M], pb[M], pc[M], pd[M], pv[M];
    bool ps[M];
    double asum = 0.0;
    {
        GPDim dm[M];
#pragma unroll
        for (int k = 0; k < M; ++k) dm[k] = GPDim{0.0, 0.0, 0.0, 0.0, 0, 0};
        gp_fill(md, th, dm);
#pragma unroll
        for (int k = 0; k < M; ++k) {
            pa[k] = dm[k].a; pb[k] = dm[k].b; pc[k] = dm[k].c; pd[k] = dm[k].d;
            ps[k] = dm[k].sinpart != 0;
            pv[k] = dm[k].live ? 1.0 : 0.0;
            if (!ps[k]) asum += dm[k].a;
            if (!(isfinite(dm[k].a) && isfinite(dm[k].b) && isfinite(dm[k].c) && isfinite(dm[k].d)))
                return -INFINITY;
        }
    }
    // S is symmetric: the upper triangle is kept
    double S[M][M], f[M], W[M];
#pragma unroll
    for (int i = 0; i < M; ++i) {
        f[i] = 0.0; W[i] = 0.0;
#pragma unroll
        for (int j = 0; j < M; ++j) S[i][j] = 0.0;
    }
    double Dp = 0.0, zp = 0.0, tp = 0.0, quad = 0.0, logdet = 0.0;
    for (int i = 0; i < n; ++i) {
        const double ti = t[i];
        const double ri = r[(size_t)i * ld];
        const double ei = e[(size_t)i * ld];
        double U[M], V[M];
#pragma unroll
        for (int k = 0; k < M; ++k) {
            double sn, cs;
            sincos(pd[k] * ti, &sn, &cs);
            U[k] = ps[k] ? pa[k] * sn - pb[k] * cs : pa[k] * cs + pb[k] * sn;
            V[k] = pv[k] * (ps[k] ? sn : cs);
        }
        if (i > 0) {
            const double dt = ti - tp;
            double ph[M];
#pragma unroll
            for (int k = 0; k < M; ++k) ph[k] = exp(-pc[k] * dt);
#pragma unroll
            for (int a = 0; a < M; ++a) {
#pragma unroll
                for (int b = a; b < M; ++b) S[a][b] = ph[a] * ph[b] * fma(Dp * W[a], W[b], S[a][b]);
                f[a] = ph[a] * fma(W[a], zp, f[a]);
            }
        }
        double SU[M];
#pragma unroll
        for (int a = 0; a < M; ++a) {
            double s = 0.0;
#pragma unroll
            for (int b = 0; b < M; ++b) s = fma(a <= b ? S[a][b] : S[b][a], U[b], s);
            SU[a] = s;
        }
        double uSu = 0.0, uf = 0.0;
#pragma unroll
        for (int a = 0; a < M; ++a) { uSu = fma(U[a], SU[a], uSu); uf = fma(U[a], f[a], uf); }
        const double D = ei + asum - uSu;
        if (!(D > 0.0)) return -INFINITY;
        const double iD = 1.0 / D;
#pragma unroll
        for (int a = 0; a < M; ++a) W[a] = (V[a] - SU[a]) * iD;
        const double z = ri - uf;
        quad = fma(z * z, iD, quad);
        logdet += log(D);
        Dp = D; zp = z; tp = ti;
    }
    return -0.5 * (quad + logdet) + md->loglike_const;
}

// one thread per walker row of the preceding k_logpost launch (same KArgs)
template <int M>
__global__ void __launch_bounds__(32) k_gp(KArgs A) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= A.nwalk) return;
    const emp_model_desc* md = A.md;
    const int ds = A.dstride;
    double lp;
    const double* free_th;
    GPMeta m{};
    if (A.mode == kModeLogpost) {
        lp = A.logprior[row];
        free_th = A.theta + (size_t)row * ds;
    } else if (A.mode == kModeSlots) {
        lp = A.st_logprior[row];
        free_th = A.st_theta + (size_t)row * ds;
    } else {
        m = A.gp_meta[row];
        lp = m.lp;
        free_th = A.gp_prop + (size_t)row * ds;
    }
    double ll = -INFINITY;
    if (lp > -INFINITY)
        ll = gp_loglike<M>(md, free_th, A.d.t, A.d.n, A.gp_r + row, A.gp_e + row, A.nwalk);
    if (A.mode == kModeLogpost) {
        A.logl[row] = lp > -INFINITY ? ll : -INFINITY;
        if (A.logp != nullptr && A.beta != nullptr)
            A.logp[row] = (lp > -INFINITY && ll > -INFINITY) ? __dadd_rn(__dmul_rn(A.beta[row], ll), lp)
                                                              : -INFINITY;
    } else if (A.mode == kModeSlots) {
        A.st_logl[row] = ll;
    } else if (lp > -INFINITY && ll > -INFINITY) {
        const double beta = A.betas[m.t];
        const double lpj = A.st_logprior[m.slot];
        const double llj = A.st_logl[m.slot];
        const double cur = lpj > -INFINITY ? __dadd_rn(__dmul_rn(beta, llj), lpj) : -INFINITY;
        const double nlp = __dadd_rn(__dmul_rn(beta, ll), lp);
        if (metropolis(nlp, cur, m.z, md->n_free - 1, m.uword)) {
            A.st_logl[m.slot] = ll;
            A.st_logprior[m.slot] = lp;
            A.accepted[m.pos] += 1;
            double* dst = A.st_theta + (size_t)m.slot * ds;
            for (int d = 0; d < md->n_free; ++d) dst[d] = free_th[d];
        }
    }
}

}  // namespace emp
