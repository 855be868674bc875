/*
 * pdhg_ref.c — TEST INFRASTRUCTURE ONLY: C + OpenMP restatement of the
 * reference's restarted PDHG iteration (solver/lp/pdhg.py:168-244) on a
 * standard-form problem min c^T z, A z = b, z >= 0 that the caller already
 * built (oracle/pdhg_ref.py:to_standard_form restates pdhg.py:62-125).
 *
 * Used as the timed CPU baseline of the benchmark (all host threads) and
 * checked against oracle/pdhg_ref.py by tests/test_oracle_c.py.
 *
 *   z' = max(0, z - tau (c - A^T w));  zbar = 2 z' - z;  w += sigma (b - A zbar)
 *   ergodic sums; every 50 iterations the KKT error of the average
 *   (pdhg.py:184-196); stop below tol (return the average), restart to the
 *   average when the error halves.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define CHECK_INTERVAL 50

static void spmv(int rows, const int *p, const int *ix, const double *v, const double *x, double *y) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < rows; ++i) {
        double s = 0.0;
        for (int k = p[i]; k < p[i + 1]; ++k) s += v[k] * x[ix[k]];
        y[i] = s;
    }
}

static double kkt(int m, int n, const int *Ap, const int *Ai, const double *Ax, const int *Tp, const int *Ti,
                  const double *Tx, const double *b, const double *c, const double *z, const double *w,
                  double nb, double nc, double *tm, double *tn) {
    spmv(m, Ap, Ai, Ax, z, tm);
    spmv(n, Tp, Ti, Tx, w, tn);
    double rp = 0.0, rd = 0.0, po = 0.0, dob = 0.0;
#pragma omp parallel for reduction(+ : rp, dob) schedule(static)
    for (int i = 0; i < m; ++i) {
        const double r = tm[i] - b[i];
        rp += r * r;
        dob += b[i] * w[i];
    }
#pragma omp parallel for reduction(+ : rd, po) schedule(static)
    for (int j = 0; j < n; ++j) {
        const double r = fmin(c[j] - tn[j], 0.0);
        rd += r * r;
        po += c[j] * z[j];
    }
    const double e_p = sqrt(rp) / nb, e_d = sqrt(rd) / nc;
    const double gap = fabs(po - dob) / (1.0 + fabs(po) + fabs(dob));
    return fmax(e_p, fmax(e_d, gap));
}

/* Returns 0 = optimal, 1 = iteration limit.  z_out (n), w_out (m). */
int oracle_pdhg_ref(int m, int n, const int *Ap, const int *Ai, const double *Ax, const int *Tp, const int *Ti,
                    const double *Tx, const double *b, const double *c, long max_iters, double tol,
                    double *z_out, double *w_out, long *iters_out, int *restarts_out) {
    double *tau = malloc(sizeof(double) * n), *sig = malloc(sizeof(double) * m);
    double *z = calloc(n, sizeof(double)), *w = calloc(m, sizeof(double));
    double *zb = malloc(sizeof(double) * n), *zs = calloc(n, sizeof(double)), *ws = calloc(m, sizeof(double));
    double *tm = malloc(sizeof(double) * m), *tn = malloc(sizeof(double) * n);
    double *za = malloc(sizeof(double) * n), *wa = malloc(sizeof(double) * m);
    /* tau_j = 0.999 / max(sum_i |A_ij|, 1e-4), sigma_i likewise over rows */
#pragma omp parallel for schedule(static)
    for (int j = 0; j < n; ++j) {
        double s = 0.0;
        for (int k = Tp[j]; k < Tp[j + 1]; ++k) s += fabs(Tx[k]);
        tau[j] = 0.999 / fmax(s, 1e-4);
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < m; ++i) {
        double s = 0.0;
        for (int k = Ap[i]; k < Ap[i + 1]; ++k) s += fabs(Ax[k]);
        sig[i] = 0.999 / fmax(s, 1e-4);
    }
    double nb2 = 0.0, nc2 = 0.0;
    for (int i = 0; i < m; ++i) nb2 += b[i] * b[i];
    for (int j = 0; j < n; ++j) nc2 += c[j] * c[j];
    const double nb = fmax(1.0, sqrt(nb2)), nc = fmax(1.0, sqrt(nc2));
    double last = kkt(m, n, Ap, Ai, Ax, Tp, Ti, Tx, b, c, z, w, nb, nc, tm, tn);
    int status = 1, restarts = 0;
    long win = 0, it = 0;
    for (it = 1; it <= max_iters; ++it) {
        spmv(n, Tp, Ti, Tx, w, tn);
#pragma omp parallel for schedule(static)
        for (int j = 0; j < n; ++j) {
            const double zn = fmax(z[j] - tau[j] * (c[j] - tn[j]), 0.0);
            zb[j] = 2.0 * zn - z[j];
            z[j] = zn;
            zs[j] += zn;
        }
        spmv(m, Ap, Ai, Ax, zb, tm);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < m; ++i) {
            w[i] = w[i] + sig[i] * (b[i] - tm[i]);
            ws[i] += w[i];
        }
        ++win;
        if (win % CHECK_INTERVAL == 0) {
            for (int j = 0; j < n; ++j) za[j] = zs[j] / (double)win;
            for (int i = 0; i < m; ++i) wa[i] = ws[i] / (double)win;
            const double err = kkt(m, n, Ap, Ai, Ax, Tp, Ti, Tx, b, c, za, wa, nb, nc, tm, tn);
            if (err < tol) {
                memcpy(z, za, sizeof(double) * n);
                memcpy(w, wa, sizeof(double) * m);
                status = 0;
                break;
            }
            if (err < 0.5 * last) {
                memcpy(z, za, sizeof(double) * n);
                memcpy(w, wa, sizeof(double) * m);
                memset(zs, 0, sizeof(double) * n);
                memset(ws, 0, sizeof(double) * m);
                win = 0;
                last = err;
                ++restarts;
            }
        }
    }
    if (it > max_iters) it = max_iters;
    memcpy(z_out, z, sizeof(double) * n);
    memcpy(w_out, w, sizeof(double) * m);
    *iters_out = it;
    *restarts_out = restarts;
    free(tau); free(sig); free(z); free(w); free(zb); free(zs); free(ws); free(tm); free(tn); free(za); free(wa);
    return status;
}
