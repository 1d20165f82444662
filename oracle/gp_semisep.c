/* Celerite GP log-likelihood, compiled restatement (oracle; TEST
 * INFRASTRUCTURE ONLY: the CPU baseline's stand-in for celerite2's C++ core).
 *
 * The reference's GP likelihood (support/likelihoods/02.like) calls celerite2,
 * which factorises K = k(|t_i - t_j|) + diag with the O(N J^2) semiseparable
 * recursion of Foreman-Mackey et al. (2017, AJ 154, 220).  This file states
 * the same recursion as oracle/gp.py's semisep_loglike in plain C, with a real
 * component taking one state dimension and a complex component two (the
 * celerite2 layout), so that a per-walker evaluation on the host costs what
 * the reference's compiled library costs.  Built by oracle/gp.py with gcc.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* kernel k(tau) = sum_j ar_j exp(-cr_j tau)
 *               + sum_j exp(-c_j tau) (a_j cos(d_j tau) + b_j sin(d_j tau));
 * returns -0.5 (r^T K^-1 r + log det K + n log 2 pi), or -inf when K is not
 * positive definite (or n < 1). */
double emp_oracle_gp_loglike(int n, const double* t, const double* r, const double* diag,
                             int jr, const double* ar, const double* cr,
                             int jc, const double* a, const double* b, const double* c,
                             const double* d) {
    const int M = jr + 2 * jc;
    if (n < 1) return -INFINITY;
    double asum = 0.0;
    for (int j = 0; j < jr; ++j) asum += ar[j];
    for (int j = 0; j < jc; ++j) asum += a[j];
    double* S = (double*)calloc((size_t)M * M + 5 * (size_t)M, sizeof(double));
    if (!S) return NAN;
    double* f = S + (size_t)M * M;
    double* W = f + M;
    double* U = W + M;
    double* V = U + M;
    double* ph = V + M;
    double Dp = 0.0, zp = 0.0, quad = 0.0, logdet = 0.0, out;
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < jr; ++j) { U[j] = ar[j]; V[j] = 1.0; }
        for (int j = 0; j < jc; ++j) {
            const double cs = cos(d[j] * t[i]), sn = sin(d[j] * t[i]);
            U[jr + 2 * j] = a[j] * cs + b[j] * sn;
            U[jr + 2 * j + 1] = a[j] * sn - b[j] * cs;
            V[jr + 2 * j] = cs;
            V[jr + 2 * j + 1] = sn;
        }
        if (i > 0) {
            const double dt = t[i] - t[i - 1];
            for (int j = 0; j < jr; ++j) ph[j] = exp(-cr[j] * dt);
            for (int j = 0; j < jc; ++j) ph[jr + 2 * j] = ph[jr + 2 * j + 1] = exp(-c[j] * dt);
            for (int p = 0; p < M; ++p) {
                for (int q = 0; q < M; ++q)
                    S[p * M + q] = ph[p] * ph[q] * (S[p * M + q] + Dp * W[p] * W[q]);
                f[p] = ph[p] * (f[p] + W[p] * zp);
            }
        }
        double uSu = 0.0, uf = 0.0;
        for (int p = 0; p < M; ++p) {
            double su = 0.0;
            for (int q = 0; q < M; ++q) su += S[p * M + q] * U[q];
            W[p] = su;                                   /* S U for now */
            uSu += U[p] * su;
            uf += U[p] * f[p];
        }
        const double D = diag[i] + asum - uSu;
        if (!(D > 0.0)) {
            free(S);
            return -INFINITY;
        }
        for (int p = 0; p < M; ++p) W[p] = (V[p] - W[p]) / D;
        const double z = r[i] - uf;
        quad += z * z / D;
        logdet += log(D);
        Dp = D;
        zp = z;
    }
    free(S);
    out = -0.5 * (quad + logdet) - 0.5 * n * 1.8378770664093453;   /* log(2 pi) */
    return out;
}
