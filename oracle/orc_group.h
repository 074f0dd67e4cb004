/*
 * ORACLE (test infrastructure only): FP64 group and algebra primitives for the
 * CPU restatement of the reference's real-time hot path.
 *
 * Conventions follow the reference exactly, because the oracle reads and
 * writes the reference's own array layouts:
 *   SU(2): 4 reals, U = u3*1 + i u_k sigma_k   (SUNc/SU2/GroupOperations.cpp:4-9)
 *   SU(3): 9 complex, column-major (i,j) -> i + 3j (SUNc/SU3/GroupOperations.cpp:8-30)
 *   algebra: E = E^a t^a with t^a = sigma^a/2 (SU(2)) or lambda^a/2 (SU(3)),
 *            3 or 8 reals (SUNc/SU2/AlgebraOperations.cpp:4-7, SUNc/SU3/AlgebraOperations.cpp:6-7)
 *   proj(V)^a = Re tr(i t^a V) = -Im tr(t^a V)   (ReTrIGenU, SU2/GroupOperations.cpp:78-84,
 *                                                 SU3/GroupOperations.cpp:108-118)
 * The formulas are derived here from those definitions (quaternion algebra for
 * SU(2), explicit Gell-Mann contractions for SU(3)); the SU(3) exponential uses
 * a complex Jacobi eigen-decomposition, the same "diagonalise then exponentiate"
 * route as SUNc/SU3/AlgebraOperations.cpp:141-182 with a different eigensolver.
 */
#ifndef ORC_GROUP_H
#define ORC_GROUP_H

#include <complex.h>
#include <math.h>
#include <string.h>

typedef double complex cplx;

/* ------------------------------------------------------------------ SU(2) */
/* Quaternion product: (u3 + i u.s)(v3 + i v.s) = u3 v3 - u.v + i (u3 v + v3 u - u x v).s */
static inline void su2_mul(const double *u, const double *v, double *w) {
    double w0 = u[3] * v[0] + v[3] * u[0] - (u[1] * v[2] - u[2] * v[1]);
    double w1 = u[3] * v[1] + v[3] * u[1] - (u[2] * v[0] - u[0] * v[2]);
    double w2 = u[3] * v[2] + v[3] * u[2] - (u[0] * v[1] - u[1] * v[0]);
    double w3 = u[3] * v[3] - (u[0] * v[0] + u[1] * v[1] + u[2] * v[2]);
    w[0] = w0; w[1] = w1; w[2] = w2; w[3] = w3;
}
static inline void su2_dag(const double *u, double *d) { d[0] = -u[0]; d[1] = -u[1]; d[2] = -u[2]; d[3] = u[3]; }
static inline void su2_identity(double *u) { u[0] = u[1] = u[2] = 0.0; u[3] = 1.0; }
static inline void su2_proj(const double *v, double *p) { p[0] = -v[0]; p[1] = -v[1]; p[2] = -v[2]; }
/* Re tr(1 - V) for the 2x2 matrix */
static inline double su2_retr_one_minus(const double *v) { return 2.0 * (1.0 - v[3]); }
/* exp(i c t^a alpha^a) = cos(d/2) + i sin(d/2) (c alpha / d).sigma, d = |c alpha| */
static inline void su2_iexp(double c, const double *alpha, double *out) {
    double x0 = c * alpha[0], x1 = c * alpha[1], x2 = c * alpha[2];
    double d = sqrt(x0 * x0 + x1 * x1 + x2 * x2);
    if (d == 0.0) { su2_identity(out); return; }
    double s = sin(0.5 * d) / d;
    out[0] = s * x0; out[1] = s * x1; out[2] = s * x2; out[3] = cos(0.5 * d);
}
/* V (E^a t^a) V^dagger in components: i e.sigma is the pure quaternion (e, 0). */
static inline void su2_adjoint(const double *v, const double *e, double *out) {
    double q[4] = {e[0], e[1], e[2], 0.0}, vd[4], t[4];
    su2_dag(v, vd);
    su2_mul(v, q, t);
    su2_mul(t, vd, t);
    out[0] = t[0]; out[1] = t[1]; out[2] = t[2];
}
static inline void su2_inverse_adjoint(const double *v, const double *e, double *out) {
    double vd[4];
    su2_dag(v, vd);
    su2_adjoint(vd, e, out);
}
/* || V V^dagger - 1 || over the four stored components (SU2/GroupOperations.cpp:172-184) */
static inline double su2_unitarity_norm(const double *v) {
    double vd[4], c[4];
    su2_dag(v, vd);
    su2_mul(v, vd, c);
    return sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2] + (c[3] - 1.0) * (c[3] - 1.0));
}

/* ------------------------------------------------------------------ SU(3) */
#define M3(i, j) ((i) + 3 * (j))

static inline void su3_mul(const cplx *a, const cplx *b, cplx *c) {
    cplx r[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            r[M3(i, j)] = a[M3(i, 0)] * b[M3(0, j)] + a[M3(i, 1)] * b[M3(1, j)] + a[M3(i, 2)] * b[M3(2, j)];
    memcpy(c, r, sizeof(r));
}
static inline void su3_dag(const cplx *a, cplx *d) {
    cplx r[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r[M3(i, j)] = conj(a[M3(j, i)]);
    memcpy(d, r, sizeof(r));
}
static inline void su3_identity(cplx *u) {
    for (int k = 0; k < 9; ++k) u[k] = 0.0;
    u[0] = u[4] = u[8] = 1.0;
}
/* Hermitian H = sum_a x^a t^a with t^a = lambda^a / 2 */
static inline void su3_algebra_matrix(const double *x, cplx *h) {
    const double is3 = 0.57735026918962576450914878050196;
    h[M3(0, 0)] = 0.5 * (x[2] + x[7] * is3);
    h[M3(1, 1)] = 0.5 * (-x[2] + x[7] * is3);
    h[M3(2, 2)] = -x[7] * is3;
    h[M3(1, 0)] = 0.5 * (x[0] + I * x[1]);
    h[M3(0, 1)] = 0.5 * (x[0] - I * x[1]);
    h[M3(2, 0)] = 0.5 * (x[3] + I * x[4]);
    h[M3(0, 2)] = 0.5 * (x[3] - I * x[4]);
    h[M3(2, 1)] = 0.5 * (x[5] + I * x[6]);
    h[M3(1, 2)] = 0.5 * (x[5] - I * x[6]);
}
/* tr(t^a M) for all a, contracted against the Gell-Mann matrices directly. */
static inline void su3_tr_gen(const cplx *m, cplx *t) {
    const double is3 = 0.57735026918962576450914878050196;
    t[0] = 0.5 * (m[M3(1, 0)] + m[M3(0, 1)]);
    t[1] = 0.5 * I * (m[M3(0, 1)] - m[M3(1, 0)]);
    t[2] = 0.5 * (m[M3(0, 0)] - m[M3(1, 1)]);
    t[3] = 0.5 * (m[M3(2, 0)] + m[M3(0, 2)]);
    t[4] = 0.5 * I * (m[M3(0, 2)] - m[M3(2, 0)]);
    t[5] = 0.5 * (m[M3(2, 1)] + m[M3(1, 2)]);
    t[6] = 0.5 * I * (m[M3(1, 2)] - m[M3(2, 1)]);
    t[7] = 0.5 * is3 * (m[M3(0, 0)] + m[M3(1, 1)] - 2.0 * m[M3(2, 2)]);
}
static inline void su3_proj(const cplx *v, double *p) {
    cplx t[8];
    su3_tr_gen(v, t);
    for (int a = 0; a < 8; ++a) p[a] = -cimag(t[a]);
}
static inline double su3_retr_one_minus(const cplx *v) { return 3.0 - creal(v[0] + v[4] + v[8]); }

/* Complex Hermitian Jacobi eigen-decomposition: A = W diag(w) W^dagger.
 * Each sweep zeroes the off-diagonal (p,q) entries with a unitary 2x2 rotation. */
static inline void su3_hermitian_eigen(const cplx *a_in, double *w, cplx *wv) {
    cplx a[9];
    memcpy(a, a_in, sizeof(a));
    su3_identity(wv);
    for (int sweep = 0; sweep < 50; ++sweep) {
        double off = cabs(a[M3(0, 1)]) + cabs(a[M3(0, 2)]) + cabs(a[M3(1, 2)]);
        double scale = fabs(creal(a[0])) + fabs(creal(a[4])) + fabs(creal(a[8])) + off;
        if (off <= 1e-300 || off <= 1e-18 * scale) break;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                cplx apq = a[M3(p, q)];
                double r = cabs(apq);
                if (r == 0.0) continue;
                cplx ph = apq / r; /* a_pq = r e^{i phi} */
                double app = creal(a[M3(p, p)]), aqq = creal(a[M3(q, q)]);
                double th = 0.5 * atan2(2.0 * r, aqq - app);
                double c = cos(th), s = sin(th);
                /* G: columns p,q mixed as  col_p' = c col_p - s conj(ph) col_q ; col_q' = s ph col_p + c col_q */
                cplx gpp = c, gqp = -s * conj(ph), gpq = s * ph, gqq = c;
                for (int k = 0; k < 3; ++k) { /* A <- A G */
                    cplx akp = a[M3(k, p)], akq = a[M3(k, q)];
                    a[M3(k, p)] = akp * gpp + akq * gqp;
                    a[M3(k, q)] = akp * gpq + akq * gqq;
                    cplx vkp = wv[M3(k, p)], vkq = wv[M3(k, q)];
                    wv[M3(k, p)] = vkp * gpp + vkq * gqp;
                    wv[M3(k, q)] = vkp * gpq + vkq * gqq;
                }
                for (int k = 0; k < 3; ++k) { /* A <- G^dagger A */
                    cplx apk = a[M3(p, k)], aqk = a[M3(q, k)];
                    a[M3(p, k)] = conj(gpp) * apk + conj(gqp) * aqk;
                    a[M3(q, k)] = conj(gpq) * apk + conj(gqq) * aqk;
                }
            }
    }
    w[0] = creal(a[0]); w[1] = creal(a[4]); w[2] = creal(a[8]);
}
/* exp(i c t^a alpha^a) = W diag(e^{i c w_j}) W^dagger */
static inline void su3_iexp(double c, const double *alpha, cplx *out) {
    cplx h[9], wv[9];
    double w[3];
    su3_algebra_matrix(alpha, h);
    su3_hermitian_eigen(h, w, wv);
    cplx ph[3];
    for (int j = 0; j < 3; ++j) ph[j] = cos(c * w[j]) + I * sin(c * w[j]);
    for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 3; ++k) {
            cplx s = 0.0;
            for (int j = 0; j < 3; ++j) s += wv[M3(i, j)] * ph[j] * conj(wv[M3(k, j)]);
            out[M3(i, k)] = s;
        }
}
/* components of V (E^a t^a) V^dagger: x'^a = 2 tr(t^a V H V^dagger) */
static inline void su3_adjoint(const cplx *v, const double *e, double *out) {
    cplx h[9], vd[9], t[8];
    su3_algebra_matrix(e, h);
    su3_dag(v, vd);
    su3_mul(v, h, h);
    su3_mul(h, vd, h);
    su3_tr_gen(h, t);
    for (int a = 0; a < 8; ++a) out[a] = 2.0 * creal(t[a]);
}
static inline void su3_inverse_adjoint(const cplx *v, const double *e, double *out) {
    cplx vd[9];
    su3_dag(v, vd);
    su3_adjoint(vd, e, out);
}
/* || V V^dagger - 1 ||_F (SU3/GroupOperations.cpp:351-363) */
static inline double su3_unitarity_norm(const cplx *v) {
    cplx vd[9], c[9];
    su3_dag(v, vd);
    su3_mul(v, vd, c);
    double n = 0.0;
    for (int k = 0; k < 9; ++k) {
        cplx d = c[k] - ((k == 0 || k == 4 || k == 8) ? 1.0 : 0.0);
        n += creal(d) * creal(d) + cimag(d) * cimag(d);
    }
    return sqrt(n);
}


/* ---------------------------------------------------------------- matrix logs
 * A^a with exp(i c A^a t^a) = V for a group element V and c = +-1 (the
 * reference calls it with c = -1, SUNc/AdvancedOperations.cpp:432-442), using
 * the principal logarithm: eigenphases in (-pi, pi].
 *   SU(2) (MatrixILog, SU2/AlgebraOperations.cpp:56-74): V = cos(t) + i sin(t) n.sigma,
 *         t = atan2(|v|, v3), A = 2 t n / c.
 *   SU(3) (MatrixILog, SU3/AlgebraOperations.cpp:186-233, there via LAPACK zgeev):
 *         V is normal, so it shares its eigenvectors with the commuting Hermitian
 *         matrices (V + V^dag)/2 and (V - V^dag)/(2i); they are found as those of
 *         C = (V + V^dag)/2 + g (V - V^dag)/(2i), g = 0.6180339887 (eigenvalues
 *         cos t + g sin t separate the pairs t, -t that share a cosine), and
 *         H = W diag(arg(w_k^dag V w_k)) W^dag, A^a = 2 tr(t^a H) / c. */
static inline void su2_ilog(double c, const double *v, double *out) {
    double d = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (d == 0.0) { out[0] = out[1] = out[2] = 0.0; return; }
    double m = 2.0 * atan2(d, v[3]) / (c * d);
    out[0] = m * v[0]; out[1] = m * v[1]; out[2] = m * v[2];
}
static inline void su3_ilog(double c, const cplx *v, double *out) {
    const double g = 0.6180339887498949;
    cplx h[9], wv[9];
    double w[3];
    for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 3; ++k) {
            cplx a = v[M3(i, k)], b = conj(v[M3(k, i)]);
            h[M3(i, k)] = 0.5 * (a + b) + g * (a - b) / (2.0 * I);
        }
    su3_hermitian_eigen(h, w, wv);
    double th[3];
    for (int j = 0; j < 3; ++j) {
        cplx z = 0.0;  /* w_j^dag V w_j */
        for (int i = 0; i < 3; ++i)
            for (int k = 0; k < 3; ++k) z += conj(wv[M3(i, j)]) * v[M3(i, k)] * wv[M3(k, j)];
        th[j] = atan2(cimag(z), creal(z));
    }
    cplx hm[9], t[8];
    for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 3; ++k) {
            cplx s = 0.0;
            for (int j = 0; j < 3; ++j) s += wv[M3(i, j)] * th[j] * conj(wv[M3(k, j)]);
            hm[M3(i, k)] = s;
        }
    su3_tr_gen(hm, t);
    for (int a = 0; a < 8; ++a) out[a] = 2.0 * creal(t[a]) / c;
}

#endif
