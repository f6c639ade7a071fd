/* The oracle (test infrastructure only; see anifem_oracle.h).  Plain C restatement of
 * the reference's element-matrix engine and global assembly rules.  Every function
 * cites the reference lines it restates.  The quadrature rules come from the table
 * the product also uses (generated by inmost-fem_gb300/csrc/gen_quadrature.py); the
 * tests pin that table against the reference's own tetrahedron_quadrature_formulas
 * and against polynomial exactness. */
#define _POSIX_C_SOURCE 199309L
#include "anifem_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "../inmost-fem_gb300/csrc/quad_tables.h"
#include "../inmost-fem_gb300/csrc/tri_quad_tables.h"

#define MAXNF 30
#define MAXDIM 9

/* ---------------------------------------------------------------- bases */

/* edge (I,J) order of P2/P3 edge DOFs: poly_2.h:34,76 and poly_3.h:36,86 */
static const int EI[6] = {0, 0, 0, 1, 1, 2}, EJ[6] = {1, 2, 3, 2, 3, 3};
/* P3 face DOF vertex triples: poly_3.h:33 (IPF) */
static const int FV[4][3] = {{0, 1, 2}, {1, 2, 3}, {0, 2, 3}, {0, 1, 3}};
/* d(lambda_i)/d(xi_d): lambda_0 = 1 - xi1 - xi2 - xi3, lambda_k = xi_k (poly_2.h:68 GRAD_P1) */
static double dl(int i, int d) { return i == 0 ? -1.0 : (i - 1 == d ? 1.0 : 0.0); }

/* values and reference gradients of a scalar space at barycentric point l[4] */
static int scalar_basis(int space, const double* l, double* val, double (*g)[3]) {
    int d, i, e;
    switch (space) {
        case 0: /* P0: poly_0.h */
            val[0] = 1;
            for (d = 0; d < 3; ++d) g[0][d] = 0;
            return 1;
        case 1: /* P1: poly_1.h:12-30, :91-120 */
            for (i = 0; i < 4; ++i) {
                val[i] = l[i];
                for (d = 0; d < 3; ++d) g[i][d] = dl(i, d);
            }
            return 4;
        case 2: /* P2: poly_2.h:12-100 */
            for (i = 0; i < 4; ++i) {
                val[i] = l[i] * (2 * l[i] - 1);
                for (d = 0; d < 3; ++d) g[i][d] = dl(i, d) * (4 * l[i] - 1);
            }
            for (e = 0; e < 6; ++e) {
                double a = l[EI[e]], b = l[EJ[e]];
                val[4 + e] = 4 * a * b;
                for (d = 0; d < 3; ++d) g[4 + e][d] = 4 * (dl(EJ[e], d) * a + dl(EI[e], d) * b);
            }
            return 10;
        case 3: /* P3: poly_3.h:12-110 */
            for (i = 0; i < 4; ++i) {
                double s = l[i];
                val[i] = s * (3 * s - 1) * (3 * s - 2) / 2;
                for (d = 0; d < 3; ++d) g[i][d] = dl(i, d) * ((13.5 * s - 9) * s + 1);
            }
            for (e = 0; e < 6; ++e) {
                int I = EI[e], J = EJ[e];
                double s1 = l[I], s2 = l[J];
                val[4 + 2 * e] = s1 * (3 * s1 - 1) * s2 * 4.5;
                val[4 + 2 * e + 1] = s1 * (3 * s2 - 1) * s2 * 4.5;
                for (d = 0; d < 3; ++d) {
                    g[4 + 2 * e][d] = (dl(I, d) * (6 * s1 - 1) * s2 + dl(J, d) * (3 * s1 - 1) * s1) * 4.5;
                    g[4 + 2 * e + 1][d] = (dl(J, d) * (6 * s2 - 1) * s1 + dl(I, d) * (3 * s2 - 1) * s2) * 4.5;
                }
            }
            for (i = 0; i < 4; ++i) {
                int a = FV[i][0], b = FV[i][1], c = FV[i][2];
                double s1 = l[a], s2 = l[b], s3 = l[c];
                val[16 + i] = 27 * s1 * s2 * s3;
                for (d = 0; d < 3; ++d)
                    g[16 + i][d] = 27 * (dl(a, d) * s2 * s3 + s1 * dl(b, d) * s3 + s1 * s2 * dl(c, d));
            }
            return 20;
        case 6: /* CR1: crouzeix_raviart_1.h:34-38 (IPF3 = {3,0,1,2}), :68-80 */
            for (i = 0; i < 4; ++i) {
                int o = (i + 3) % 4;
                val[i] = 1 - 3 * l[o];
                for (d = 0; d < 3; ++d) g[i][d] = -3 * dl(o, d);
            }
            return 4;
        case 7: /* B2: bubble_2.h:34-38 */
            for (e = 0; e < 6; ++e) {
                double a = l[EI[e]], b = l[EJ[e]];
                val[e] = 4 * a * b;
                for (d = 0; d < 3; ++d) g[e][d] = 4 * (dl(EI[e], d) * b + dl(EJ[e], d) * a);
            }
            return 6;
        case 8: /* B4: bubble_4.h:30-34, :65-75 */
            val[0] = 256 * l[0] * l[1] * l[2] * l[3];
            for (d = 0; d < 3; ++d)
                g[0][d] = 256 * (dl(0, d) * l[1] * l[2] * l[3] + dl(1, d) * l[0] * l[2] * l[3] +
                                 dl(2, d) * l[0] * l[1] * l[3] + dl(3, d) * l[0] * l[1] * l[2]);
            return 1;
    }
    return -1;
}

static int scalar_nf(int space) {
    static const int nf[9] = {1, 4, 10, 20, -1, -1, 4, 6, 1};
    return (space >= 0 && space < 9) ? nf[space] : -1;
}

int orc_op_info(int code, int* nf, int* dim) {
    int space = code / 10, op = code % 10;
    if (space == 9 || space == 10) { /* ND0 / RT0: IDEN 3, GRAD 9, DIV 1, CURL 3 */
        static const int dims[5] = {0, 3, 9, 1, 3};
        if (op < 1 || op > 4) return -1;
        *nf = space == 9 ? 6 : 4;
        *dim = dims[op];
        return 0;
    }
    int vec = (space == 4 || space == 5), base = vec ? space - 3 : space;
    int n = scalar_nf(base);
    if (n < 0 || (op != 1 && op != 2)) return -1;
    int dm = (op == 1) ? 1 : 3;
    *nf = vec ? 3 * n : n;
    *dim = vec ? 3 * dm : dm;
    return 0;
}

/* (a - c) x (b - c) (geometry.h:57-64) */
static void cross3(const double* a, const double* b, const double* c, double* r) {
    double u[3] = {a[0] - c[0], a[1] - c[1], a[2] - c[2]}, v[3] = {b[0] - c[0], b[1] - c[1], b[2] - c[2]};
    r[0] = u[1] * v[2] - u[2] * v[1];
    r[1] = -u[0] * v[2] + u[2] * v[0];
    r[2] = u[0] * v[1] - u[1] * v[0];
}

/* physical gradient of lambda_v, component k: sum_m GRAD_P1(m, v) PSI(m, k) */
static double glam(const double* PSI, int v, int k) {
    return dl(v, 0) * PSI[0 + 3 * k] + dl(v, 1) * PSI[1 + 3 * k] + dl(v, 2) * PSI[2 + 3 * k];
}

/* ND0 (spaces/nedelec_0.h:12-183) and RT0 (spaces/raviant_thomas_0.h:12-190) at one point,
 * U[k + dim*i]; P = vertex coordinates relative to X0 (the reference's XYP), det signed */
static void apply_vec_space(int space, int op, const double* l, const double* PSI, const double* P, double det,
                            double* U) {
    static const int IPR[24] = {0, 1, 2, 3, 0, 2, 3, 1, 0, 3, 1, 2, 1, 2, 0, 3, 1, 3, 2, 0, 2, 3, 0, 1};
    static const int IPF[16] = {0, 1, 2, 3, 1, 2, 3, 0, 0, 2, 3, 1, 0, 1, 3, 2};
    int dim, nf;
    orc_op_info(10 * space + op, &nf, &dim);
    for (int i = 0; i < nf; ++i) {
        double* u = U + dim * i;
        if (space == 9) {
            const int* ip = IPR + 4 * i;
            double sq = 0, xn[3], xm[3], curl[3];
            for (int k = 0; k < 3; ++k) sq += (P[3 * ip[0] + k] - P[3 * ip[1] + k]) * (P[3 * ip[0] + k] - P[3 * ip[1] + k]);
            double s = sqrt(sq) / det;
            cross3(P + 3 * ip[2], P + 3 * ip[3], P + 3 * ip[0], xn);
            cross3(P + 3 * ip[2], P + 3 * ip[3], P + 3 * ip[1], xm);
            for (int k = 0; k < 3; ++k) {
                int k1 = (k + 1) % 3, k2 = (k + 2) % 3;
                curl[k] = s * ((glam(PSI, ip[0], k1) * xn[k2] + glam(PSI, ip[1], k1) * xm[k2]) -
                               (glam(PSI, ip[0], k2) * xn[k1] + glam(PSI, ip[1], k2) * xm[k1]));
            }
            if (op == 1)
                for (int k = 0; k < 3; ++k) u[k] = s * (xn[k] * l[ip[0]] + xm[k] * l[ip[1]]);
            else if (op == 3)
                u[0] = 0;
            else if (op == 4)
                for (int k = 0; k < 3; ++k) u[k] = curl[k];
            else { /* GRAD: nedelec_0.h:172-177 */
                double a0 = curl[0] / 2, a1 = curl[1] / 2, a2 = curl[2] / 2;
                u[0] = 0; u[3] = a2;  u[6] = -a1;
                u[1] = -a2; u[4] = 0; u[7] = a0;
                u[2] = a1; u[5] = -a0; u[8] = 0;
            }
        } else {
            const int* ip = IPF + 4 * i;
            double cr[3];
            cross3(P + 3 * ip[0], P + 3 * ip[1], P + 3 * ip[2], cr);
            double s = (sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]) / 2) / (fabs(det) / 2);
            if (op == 1) {
                for (int j = 0; j < 3; ++j) {
                    double v = 0;
                    for (int a = 0; a < 3; ++a) v += l[ip[a]] * (P[3 * ip[a] + j] - P[3 * ip[3] + j]);
                    u[j] = s * v;
                }
            } else if (op == 4) {
                for (int k = 0; k < 3; ++k) u[k] = 0;
            } else if (op == 2) {
                for (int j = 0; j < 3; ++j)
                    for (int k = 0; k < 3; ++k) {
                        double v = 0;
                        for (int a = 0; a < 3; ++a) v += glam(PSI, ip[a], k) * (P[3 * ip[a] + j] - P[3 * ip[3] + j]);
                        u[k + 3 * j] = s * v;
                    }
            } else {
                double v = 0;
                for (int j = 0; j < 3; ++j)
                    for (int a = 0; a < 3; ++a) v += glam(PSI, ip[a], j) * (P[3 * ip[a] + j] - P[3 * ip[3] + j]);
                u[0] = s * v;
            }
        }
    }
}

/* Operator application at one point: U[k + dim*i] (operators.h:127-155 for FemVec:
 * component c occupies rows [c*bdim, (c+1)*bdim) and columns [c*nfs, (c+1)*nfs)).
 * P (relative vertex coordinates) and det serve the geometry-dependent ND0 / RT0. */
static void apply_op(int code, const double* l, const double* PSI, const double* P, double det, double* U) {
    int space = code / 10, op = code % 10;
    if (space == 9 || space == 10) {
        apply_vec_space(space, op, l, PSI, P, det, U);
        return;
    }
    int vec = (space == 4 || space == 5), base = vec ? space - 3 : space;
    double val[20], g[20][3];
    int nfs = scalar_basis(base, l, val, g);
    int bdim = (op == 1) ? 1 : 3;
    int ncomp = vec ? 3 : 1;
    int dim = bdim * ncomp, nf = nfs * ncomp;
    memset(U, 0, sizeof(double) * dim * nf);
    for (int c = 0; c < ncomp; ++c)
        for (int i = 0; i < nfs; ++i) {
            int col = c * nfs + i;
            if (op == 1) {
                U[c + dim * col] = val[i];
            } else {
                for (int k = 0; k < 3; ++k) {
                    double s = 0; /* U_k = sum_j PSI(j,k) ghat_j  (poly_2.h:91-97) */
                    for (int j = 0; j < 3; ++j) s += PSI[j + 3 * k] * g[i][j];
                    U[c * 3 + k + dim * col] = s;
                }
            }
        }
}

/* ---------------------------------------------------------------- geometry */

/* Ani::inverse3x3 (geometry.h:26-44): col-major m, returns det */
static double inverse3x3(const double* m, double* inv) {
#define M(I, J) m[(I) + 3 * (J)]
    double da = M(1, 1) * M(2, 2) - M(1, 2) * M(2, 1);
    double db = M(1, 2) * M(2, 0) - M(1, 0) * M(2, 2);
    double dc = M(1, 0) * M(2, 1) - M(1, 1) * M(2, 0);
    double det = M(0, 0) * da + M(0, 1) * db + M(0, 2) * dc;
    inv[0] = da / det;
    inv[1] = db / det;
    inv[2] = dc / det;
    for (int i = 1; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            inv[j + 3 * i] = (M((i + 1) % 3, (j + 1) % 3) * M((i + 2) % 3, (j + 2) % 3) -
                              M((i + 1) % 3, (j + 2) % 3) * M((i + 2) % 3, (j + 1) % 3)) / det;
#undef M
    return det;
}

/* internalFem3DtetGeomInit_Tet (core.inl:217-247): edges from X0, PSI = inv, MES = |det|/6 */
static double tet_geom(const double* X, double* PSI, double* mes) {
    double J[9];
    for (int c = 0; c < 3; ++c)
        for (int i = 0; i < 3; ++i) J[i + 3 * c] = X[3 * (c + 1) + i] - X[i];
    double det = inverse3x3(J, PSI);
    *mes = fabs(det) / 6;
    return det;
}

int orc_quad_rule(int order, double* p, double* w, int cap) {
    const double *pp, *ww;
    int np;
    if (!anigpu_quad_rule(order, &pp, &ww, &np)) return -1;
    if (np > cap) return -np;
    if (p) memcpy(p, pp, sizeof(double) * 4 * np);
    if (w) memcpy(w, ww, sizeof(double) * np);
    return np;
}

/* physical points: X0 + sum_l xi_l (X_l - X0) (core.inl:249-269) */
int orc_quad_points(int order, long nt, const double* XY, double* XYG) {
    const double *pp, *ww;
    int q;
    if (!anigpu_quad_rule(order, &pp, &ww, &q)) return -1;
    for (long t = 0; t < nt; ++t) {
        const double* X = XY + 12 * t;
        for (int n = 0; n < q; ++n)
            for (int k = 0; k < 3; ++k) {
                double s = X[k];
                for (int l = 0; l < 3; ++l) s += pp[l + 1 + 4 * n] * (X[3 * (l + 1) + k] - X[k]);
                XYG[3 * (n + (long)q * t) + k] = s;
            }
    }
    return q;
}

/* ---------------------------------------------------------------- element matrices */

/* expand one tensor sample into a full col-major dimB x dimA matrix D(k,j) with the
 * semantics of internal_Dfunc::applyDU (diff_tensor.h:275-552): NULL -> identity (or a
 * column of ones when dimA == 1), SCALAR -> s * identity (or a column of s). */
static void expand_tensor(int kind, const double* src, int dA, int dB, double* D) {
    memset(D, 0, sizeof(double) * dA * dB);
    switch (kind) {
        case ORC_NULL:
        case ORC_CONST_SCALAR:
        case ORC_TET_SCALAR: {
            double s = (kind == ORC_NULL) ? 1.0 : src[0];
            if (dA == dB)
                for (int i = 0; i < dA; ++i) D[i + dB * i] = s;
            else
                for (int k = 0; k < dB; ++k) D[k] = s; /* dimA == 1 (P0 right-hand side) */
            break;
        }
        case ORC_TET_SYM: { /* d00 d01 d02 d11 d12 d22 */
            double m[9] = {src[0], src[1], src[2], src[1], src[3], src[4], src[2], src[4], src[5]};
            memcpy(D, m, sizeof m);
            break;
        }
        default:
            memcpy(D, src, sizeof(double) * dA * dB);
    }
}

/* GRAD.GRAD of one scalar space with a per-tet symmetric tensor: the same steps as the
 * reference's template path for one tet (core.inl:277-367): U = PSI^T ghat at every point
 * (poly_2.h:52-100), DU = w |T| D U (diff_tensor.h:275-310), A = U^T DU (core.inl:28-60). */
static void gradgrad_sym(int space, int order, long nt, const double* XY, const double* D6, double* A) {
    const double *pp, *ww;
    int q;
    anigpu_quad_rule(order, &pp, &ww, &q);
    int nf = scalar_nf(space);
    double val[20], g[20][3];
    /* rules of up to ANIGPU_QUAD_MAX_POINTS points: buffers on the heap */
    double* U = (double*)malloc(sizeof(double) * 3 * 20 * (size_t)q);
    double* DU = (double*)malloc(sizeof(double) * 3 * 20 * (size_t)q);
    double (*G)[20][3] = (double (*)[20][3])malloc(sizeof(double) * 60 * (size_t)q);
    for (long t = 0; t < nt; ++t) {
        double PSI[9], mes;
        tet_geom(XY + 12 * t, PSI, &mes);
        const double* s = D6 + 6 * t;
        const double Dm[9] = {s[0], s[1], s[2], s[1], s[3], s[4], s[2], s[4], s[5]};
        for (int n = 0; n < q; ++n) scalar_basis(space, pp + 4 * n, val, G[n]);
        for (int i = 0; i < nf; ++i)
            for (int n = 0; n < q; ++n)
                for (int k = 0; k < 3; ++k)
                    U[k + 3 * (n + q * i)] = PSI[0 + 3 * k] * G[n][i][0] + PSI[1 + 3 * k] * G[n][i][1] + PSI[2 + 3 * k] * G[n][i][2];
        for (int i = 0; i < nf; ++i)
            for (int n = 0; n < q; ++n) {
                const double wv = ww[n] * mes;
                const double* u = U + 3 * (n + q * i);
                for (int k = 0; k < 3; ++k)
                    DU[k + 3 * (n + q * i)] = wv * (Dm[k + 0] * u[0] + Dm[k + 3] * u[1] + Dm[k + 6] * u[2]);
            }
        double* At = A + (size_t)t * nf * nf;
        const int nr = 3 * q;
        for (int ia = 0; ia < nf; ++ia)
            for (int ib = 0; ib < nf; ++ib) {
                double acc = 0;
                const double* v = U + nr * ib;
                const double* du = DU + nr * ia;
                for (int j = 0; j < nr; ++j) acc += v[j] * du[j];
                At[ib + nf * ia] = acc;
            }
    }
    free(U);
    free(DU);
    free(G);
    (void)g;
}

/* triangle area (Ani::tri_area, geometry.h:67-72) of face k = vertices k, k+1, k+2 (mod 4),
 * from the coordinates relative to X0 as in the reference's XYP (int_face.inl:40-43) */
static double face_area(const double* X, int face) {
    double P[3][3];
    for (int v = 0; v < 3; ++v) {
        int node = (face + v) % 4;
        for (int i = 0; i < 3; ++i) P[v][i] = node == 0 ? 0.0 : X[3 * node + i] - X[i];
    }
    double a[3] = {P[0][0] - P[2][0], P[0][1] - P[2][1], P[0][2] - P[2][2]};
    double b[3] = {P[1][0] - P[2][0], P[1][1] - P[2][1], P[1][2] - P[2][2]};
    double c[3] = {a[1] * b[2] - a[2] * b[1], -a[0] * b[2] + a[2] * b[0], a[0] * b[1] - a[1] * b[0]};
    return sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]) / 2;
}

/* outward unit normal and area of face k (Ani::face_normal, geometry.h:77-93) on the coordinates
 * relative to X0 (int_face.inl:72-76); the fourth vertex decides the orientation */
static double face_normal(const double* X, int face, double* nrm) {
    double P[4][3];
    for (int v = 0; v < 4; ++v) {
        int node = (face + v) % 4;
        for (int i = 0; i < 3; ++i) P[v][i] = node == 0 ? 0.0 : X[3 * node + i] - X[i];
    }
    double a[3] = {P[1][0] - P[0][0], P[1][1] - P[0][1], P[1][2] - P[0][2]};
    double b[3] = {P[2][0] - P[0][0], P[2][1] - P[0][1], P[2][2] - P[0][2]};
    nrm[0] = a[1] * b[2] - a[2] * b[1];
    nrm[1] = -a[0] * b[2] + a[2] * b[0];
    nrm[2] = a[0] * b[1] - a[1] * b[0];
    double len = sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
    for (int i = 0; i < 3; ++i) a[i] = P[3][i] - P[0][i];
    double vol = nrm[0] * a[0] + nrm[1] * a[1] + nrm[2] * a[2];
    for (int i = 0; i < 3; ++i) nrm[i] /= (vol > 0 ? -len : len);
    return len / 2;
}

/* points of the triangle rule mapped onto face k (int_face.inl:31-36): 4 barycentric each */
static int face_points(int order, int face, double* pts, const double** ww) {
    const double* p3;
    int q;
    if (order < 0 || order > ANIGPU_TRI_MAX_ORDER || !anigpu_tri_rule(order, &p3, ww, &q)) return -1;
    for (int n = 0; n < q; ++n) {
        pts[4 * n + face] = p3[3 * n + 0];
        pts[4 * n + (face + 1) % 4] = p3[3 * n + 1];
        pts[4 * n + (face + 2) % 4] = p3[3 * n + 2];
        pts[4 * n + (face + 3) % 4] = 0.0;
    }
    return q;
}

/* A(ib, ia) = sum_n w_n mes sum_k V_k(ib) sum_j D(k,j) U_j(ia)
 * (core.inl:277-367: U = OpA(apply), DU (diff_tensor.h:488-552), A = V^T DU (core.inl:28-60));
 * mes = |T| for the tet integral (face < 0), the face area for fem3Dface (int_face.inl:12-44) */
/* normal != 0 (fem3DfaceN, int_face.inl:48-78): the tensor has 3*dB rows; DU's rows l + 3k are
 * contracted with the outward normal (DotWithNormalHelper::ProcessNormal, core.h:175-190), which
 * is the same as contracting the tensor's rows first; mes = the area from face_normal */
static int elem_core(int codeA, int codeB, int kind, const double* pp, const double* ww, int q, int face, int normal,
                     long nt, const double* XY, const double* D, double* A) {
    int nfA, dA, nfB, dB;
    if (orc_op_info(codeA, &nfA, &dA) || orc_op_info(codeB, &nfB, &dB)) return -1;
    int dBt = normal ? 3 * dB : dB;
    if ((kind == ORC_TET_SYM) && (dA != 3 || dBt != 3)) return -1;
    if ((kind == ORC_NULL || kind == ORC_CONST_SCALAR || kind == ORC_TET_SCALAR) && dA != dBt && dA != 1) return -1;
    double U[MAXDIM * MAXNF], V[MAXDIM * MAXNF], Dm[MAXDIM * MAXDIM], DU[MAXDIM * MAXNF];
    double Dfull[3 * MAXDIM * MAXDIM];
    for (long t = 0; t < nt; ++t) {
        double PSI[9], mes, nrm[3], P[12];
        double det = tet_geom(XY + 12 * t, PSI, &mes);
        for (int v = 0; v < 4; ++v)
            for (int i = 0; i < 3; ++i) P[3 * v + i] = v == 0 ? 0.0 : XY[12 * t + 3 * v + i] - XY[12 * t + i];
        if (normal) mes = face_normal(XY + 12 * t, face, nrm);
        else if (face >= 0) mes = face_area(XY + 12 * t, face);
        double* At = A + (size_t)t * nfA * nfB;
        memset(At, 0, sizeof(double) * nfA * nfB);
        for (int n = 0; n < q; ++n) {
            const double* l = pp + 4 * n;
            apply_op(codeA, l, PSI, P, det, U); /* l = (lambda_0..lambda_3) as tabulated (int_tet.inl:116-121) */
            apply_op(codeB, l, PSI, P, det, V);
            const double* src = NULL;
            switch (kind) {
                case ORC_CONST_SCALAR: src = D; break;
                case ORC_TET_SCALAR: src = D + t; break;
                case ORC_TET_SYM: src = D + 6 * t; break;
                case ORC_TET_GENERAL: src = D + (size_t)dA * dBt * t; break;
                case ORC_POINT: src = D + (size_t)dA * dBt * (n + (size_t)q * t); break;
            }
            if (!normal) {
                expand_tensor(kind, src, dA, dB, Dm);
            } else {
                expand_tensor(kind, src, dA, dBt, Dfull);
                for (int k = 0; k < dB; ++k)
                    for (int j = 0; j < dA; ++j)
                        Dm[k + dB * j] = Dfull[(0 + 3 * k) + dBt * j] * nrm[0] + Dfull[(1 + 3 * k) + dBt * j] * nrm[1] +
                                         Dfull[(2 + 3 * k) + dBt * j] * nrm[2];
            }
            double wv = ww[n] * mes;
            for (int ia = 0; ia < nfA; ++ia)
                for (int k = 0; k < dB; ++k) {
                    double s = 0;
                    for (int j = 0; j < dA; ++j) s += Dm[k + dB * j] * U[j + dA * ia];
                    DU[k + dB * ia] = wv * s;
                }
            for (int ia = 0; ia < nfA; ++ia)
                for (int ib = 0; ib < nfB; ++ib) {
                    double s = 0;
                    for (int k = 0; k < dB; ++k) s += V[k + dB * ib] * DU[k + dB * ia];
                    At[ib + nfB * ia] += s;
                }
        }
    }
    return 0;
}

int orc_fem3dtet(int codeA, int codeB, int kind, int order, long nt, const double* XY, const double* D, double* A) {
    const double *pp, *ww;
    int q;
    if (!anigpu_quad_rule(order, &pp, &ww, &q)) return -1;
    return elem_core(codeA, codeB, kind, pp, ww, q, -1, 0, nt, XY, D, A);
}

int orc_fem3dface(int codeA, int codeB, int kind, int order, int face, long nt, const double* XY, const double* D,
                  double* A) {
    double pts[4 * ANIGPU_TRI_MAX_POINTS];
    const double* ww;
    if (face < 0 || face > 3) return -1;
    int q = face_points(order, face, pts, &ww);
    if (q < 0) return -1;
    return elem_core(codeA, codeB, kind, pts, ww, q, face, 0, nt, XY, D, A);
}

int orc_fem3dface_n(int codeA, int codeB, int kind, int order, int face, long nt, const double* XY, const double* D,
                    double* A) {
    double pts[4 * ANIGPU_TRI_MAX_POINTS];
    const double* ww;
    if (face < 0 || face > 3) return -1;
    int q = face_points(order, face, pts, &ww);
    if (q < 0) return -1;
    return elem_core(codeA, codeB, kind, pts, ww, q, face, 1, nt, XY, D, A);
}

int orc_tri_rule(int order, double* p, double* w, int cap) {
    const double *pp, *ww;
    int np;
    if (order < 0 || order > ANIGPU_TRI_MAX_ORDER || !anigpu_tri_rule(order, &pp, &ww, &np)) return -1;
    if (np > cap) return -np;
    memcpy(p, pp, sizeof(double) * 3 * np);
    memcpy(w, ww, sizeof(double) * np);
    return np;
}

int orc_face_quad_points(int order, int face, long nt, const double* XY, double* XYG) {
    double pts[4 * ANIGPU_TRI_MAX_POINTS];
    const double* ww;
    if (face < 0 || face > 3) return -1;
    int q = face_points(order, face, pts, &ww);
    if (q < 0) return -1;
    for (long t = 0; t < nt; ++t) {
        const double* X = XY + 12 * t;
        for (int n = 0; n < q; ++n)
            for (int k = 0; k < 3; ++k) {
                double s = X[k];
                for (int l = 0; l < 3; ++l) s += pts[l + 1 + 4 * n] * (X[3 * (l + 1) + k] - X[k]);
                XYG[3 * (n + (size_t)q * t) + k] = s;
            }
    }
    return q;
}

/* ---------------------------------------------------------------- evaluation */

/* Op(u) at points of each tet (fem3DapplyL, eval.inl:93-111 -> core.inl:370-404; fem3DapplyX,
 * eval.inl:127-151 with getBaryCoord, core.inl:120-137).  phys = 0: pts are npts barycentric
 * points [npts][4] shared by every tet; phys = 1: pts are per-tet physical points [nt][npts][3],
 * turned into barycentric coordinates with the tet's PSI.  dofs[nt][nf]; opU[nt][npts][dim]
 * (opU[t][k + dim*n], the reference's vec(opU at point n) blocks).  Sums over the local DOFs
 * in ascending order (fusive_A_mul_B, core.inl:382). */
int orc_fem3d_apply(int code, long nt, const double* XY, int npts, const double* pts, int phys,
                    const double* dofs, double* opU) {
    int nf, dim;
    if (orc_op_info(code, &nf, &dim) != 0 || npts < 1) return -1;
    double U[MAXDIM * MAXNF];
    for (long t = 0; t < nt; ++t) {
        const double* X = XY + 12 * t;
        double PSI[9], mes, P[12];
        double det = tet_geom(X, PSI, &mes);
        for (int v = 0; v < 4; ++v)
            for (int i = 0; i < 3; ++i) P[3 * v + i] = v == 0 ? 0.0 : X[3 * v + i] - X[i];
        for (int n = 0; n < npts; ++n) {
            double l[4];
            if (phys) {
                const double* x = pts + 3 * ((size_t)npts * t + n);
                double dr[3] = {x[0] - X[0], x[1] - X[1], x[2] - X[2]};
                l[1] = l[2] = l[3] = 0;
                for (int j = 0; j < 3; ++j)
                    for (int i = 0; i < 3; ++i) l[i + 1] += PSI[i + 3 * j] * dr[j];
                l[0] = 1 - l[1] - l[2] - l[3];
            } else {
                for (int k = 0; k < 4; ++k) l[k] = pts[4 * n + k];
            }
            apply_op(code, l, PSI, P, det, U);
            for (int k = 0; k < dim; ++k) {
                double s = 0;
                for (int i = 0; i < nf; ++i) s += U[k + dim * i] * dofs[(size_t)nf * t + i];
                opU[((size_t)npts * t + n) * dim + k] = s;
            }
        }
    }
    return 0;
}

/* Ani::applyDir (dc_on_dof.h:39-45) */
void orc_apply_dir(int n, double* A, double* F, int k, double bc) {
    for (int i = 0; i < n; ++i) F[i] -= A[i + n * k] * bc;
    F[k] = bc;
    for (int i = 0; i < n; ++i) A[i + n * k] = 0; /* column k */
    for (int i = 0; i < n; ++i) A[k + n * i] = 0; /* row k */
    A[k + n * k] = 1.0;
}

/* ---------------------------------------------------------------- mesh topology */

/* reorderNodesOnTetrahedron (ordering.inl:9-26): swap local nodes 2,3 when
 * det(X0-X3, X1-X3, X2-X3) < 0 */
void orc_orient(const double* xyz, long nt, int32_t* tets) {
    for (long t = 0; t < nt; ++t) {
        int32_t* v = tets + 4 * t;
        double m[3][3];
        for (int j = 0; j < 3; ++j) {
            m[0][j] = xyz[3 * v[0] + j] - xyz[3 * v[3] + j];
            m[1][j] = xyz[3 * v[1] + j] - xyz[3 * v[3] + j];
            m[2][j] = xyz[3 * v[2] + j] - xyz[3 * v[3] + j];
        }
        double det = 0;
        det += m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]);
        det += m[0][1] * (m[1][2] * m[2][0] - m[1][0] * m[2][2]);
        det += m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
        if (det < 0) {
            int32_t s = v[2];
            v[2] = v[3];
            v[3] = s;
        }
    }
}

static int cmp_u64(const void* a, const void* b) {
    uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return (x > y) - (x < y);
}
static int cmp_i32(const void* a, const void* b) {
    int32_t x = *(const int32_t*)a, y = *(const int32_t*)b;
    return (x > y) - (x < y);
}

/* Edge numbering: the NATURAL enumeration (global_enumerator.h:392-404) orders edge
 * DOFs by edge id; this library defines the edge id as the rank of the edge's
 * (min vertex, max vertex) pair in lexicographic order. */
long orc_edges(long nv, long nt, const int32_t* tets, int32_t* tet_edges) {
    (void)nv;
    uint64_t* keys = (uint64_t*)malloc(sizeof(uint64_t) * 6 * (size_t)nt);
    for (long t = 0; t < nt; ++t)
        for (int e = 0; e < 6; ++e) {
            uint32_t a = (uint32_t)tets[4 * t + EI[e]], b = (uint32_t)tets[4 * t + EJ[e]];
            uint32_t lo = a < b ? a : b, hi = a < b ? b : a;
            keys[6 * t + e] = ((uint64_t)lo << 32) | hi;
        }
    uint64_t* u = (uint64_t*)malloc(sizeof(uint64_t) * 6 * (size_t)nt);
    memcpy(u, keys, sizeof(uint64_t) * 6 * (size_t)nt);
    qsort(u, 6 * (size_t)nt, sizeof(uint64_t), cmp_u64);
    long ne = 0;
    for (long i = 0; i < 6 * nt; ++i)
        if (i == 0 || u[i] != u[i - 1]) u[ne++] = u[i];
    for (long i = 0; i < 6 * nt; ++i) {
        long lo = 0, hi = ne - 1;
        while (lo < hi) {
            long mid = (lo + hi) / 2;
            if (u[mid] < keys[i]) lo = mid + 1;
            else hi = mid;
        }
        tet_edges[i] = (int32_t)lo;
    }
    free(keys);
    free(u);
    return ne;
}

/* NATURAL numbering (global_enumerator.h:392-404): vertex DOFs by vertex id, then edge
 * DOFs by edge id; Vec3P2 is component-major (component c block of ndof_scalar). */
long orc_element_dofs(int space, long nv, long ne, long nt, const int32_t* tets, const int32_t* tet_edges,
                      int32_t* edofs) {
    long nd = (space == 1) ? nv : nv + ne;
    for (long t = 0; t < nt; ++t) {
        int32_t loc[10];
        for (int i = 0; i < 4; ++i) loc[i] = tets[4 * t + i];
        if (space != 1)
            for (int e = 0; e < 6; ++e) loc[4 + e] = (int32_t)(nv + tet_edges[6 * t + e]);
        if (space == 1) {
            for (int i = 0; i < 4; ++i) edofs[4 * t + i] = loc[i];
        } else if (space == 2) {
            for (int i = 0; i < 10; ++i) edofs[10 * t + i] = loc[i];
        } else {
            for (int c = 0; c < 3; ++c)
                for (int i = 0; i < 10; ++i) edofs[30 * t + 10 * c + i] = (int32_t)(c * nd + loc[i]);
        }
    }
    return (space == 5) ? 3 * nd : nd;
}

/* dof -> incident (tet) lists, tets ascending */
static void incidence(long ndof, long nt, int nloc, const int32_t* edofs, int64_t** iptr, int32_t** itet) {
    int64_t* p = (int64_t*)calloc((size_t)ndof + 1, sizeof(int64_t));
    for (long t = 0; t < nt; ++t)
        for (int i = 0; i < nloc; ++i) p[edofs[(size_t)nloc * t + i] + 1]++;
    for (long r = 0; r < ndof; ++r) p[r + 1] += p[r];
    int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (size_t)ndof);
    memcpy(fill, p, sizeof(int64_t) * (size_t)ndof);
    int32_t* it = (int32_t*)malloc(sizeof(int32_t) * (size_t)(p[ndof] > 0 ? p[ndof] : 1));
    for (long t = 0; t < nt; ++t)
        for (int i = 0; i < nloc; ++i) it[fill[edofs[(size_t)nloc * t + i]]++] = (int32_t)t;
    free(fill);
    *iptr = p;
    *itet = it;
}

long orc_csr_template(long ndof, long nt, int nloc, const int32_t* edofs, int64_t* rowptr, int32_t* col) {
    int64_t* ip;
    int32_t* itet;
    incidence(ndof, nt, nloc, edofs, &ip, &itet);
    int32_t* buf = (int32_t*)malloc(sizeof(int32_t) * (64 * nloc + 8));
    int cap = 64 * nloc + 8;
    long nnz = 0;
    rowptr[0] = 0;
    for (long r = 0; r < ndof; ++r) {
        long m = 0;
        long deg = ip[r + 1] - ip[r];
        if (deg * nloc + 1 > cap) {
            cap = (int)(deg * nloc + 1);
            buf = (int32_t*)realloc(buf, sizeof(int32_t) * cap);
        }
        buf[m++] = (int32_t)r; /* diagonal forced (assembler.inl:114-135) */
        for (int64_t k = ip[r]; k < ip[r + 1]; ++k)
            for (int j = 0; j < nloc; ++j) buf[m++] = edofs[(size_t)nloc * itet[k] + j];
        qsort(buf, m, sizeof(int32_t), cmp_i32);
        long u = 0;
        for (long k = 0; k < m; ++k)
            if (k == 0 || buf[k] != buf[k - 1]) buf[u++] = buf[k];
        if (col) memcpy(col + nnz, buf, sizeof(int32_t) * u);
        nnz += u;
        rowptr[r + 1] = nnz;
    }
    free(buf);
    free(ip);
    free(itet);
    return nnz;
}

static long find_slot(const int64_t* rowptr, const int32_t* col, long r, int32_t c) {
    long lo = rowptr[r], hi = rowptr[r + 1] - 1;
    while (lo < hi) {
        long mid = (lo + hi) / 2;
        if (col[mid] < c) lo = mid + 1;
        else hi = mid;
    }
    return (lo <= hi && col[lo] == c) ? lo : -1;
}

int orc_scatter(long ndof, const int64_t* rowptr, const int32_t* col, long nt, int nloc, const int32_t* edofs,
                const double* Aelem, const double* Felem, double drop, double* vals, double* rhs, uint8_t* touched) {
    (void)ndof;
    for (long t = 0; t < nt; ++t) {
        const int32_t* ed = edofs + (size_t)nloc * t;
        const double* Ae = Aelem + (size_t)nloc * nloc * t;
        for (int i = 0; i < nloc; ++i) {
            long r = ed[i];
            if (Felem) {
                if (!isfinite(Felem[(size_t)nloc * t + i])) return -1;
                rhs[r] += Felem[(size_t)nloc * t + i];
            }
            for (int j = 0; j < nloc; ++j) {
                double a = Ae[i + nloc * j]; /* element matrix column-major: A(i,j) = Ae[j*n + i] */
                if (!isfinite(a)) return -1;
                if (fabs(a) > drop) {
                    long s = find_slot(rowptr, col, r, ed[j]);
                    if (s < 0) return -2;
                    vals[s] += a;
                    if (touched) touched[s] = 1;
                }
            }
        }
    }
    return 0;
}

long orc_csr_compact(long ndof, int64_t* rowptr, int32_t* col, double* vals, const uint8_t* touched) {
    long w = 0;
    int64_t start = rowptr[0];
    for (long r = 0; r < ndof; ++r) {
        int64_t end = rowptr[r + 1];
        for (int64_t k = start; k < end; ++k)
            if (touched[k] || col[k] == r) {
                col[w] = col[k];
                if (vals) vals[w] = vals[k];
                ++w;
            }
        start = end;
        rowptr[r + 1] = w;
    }
    return w;
}

/* ---------------------------------------------------------------- solver */

void orc_spmv(long n, const int64_t* rowptr, const int32_t* col, const double* vals, const double* x, double* y) {
    for (long r = 0; r < n; ++r) {
        double s = 0;
        for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) s += vals[k] * x[col[k]];
        y[r] = s;
    }
}

static double dot(long n, const double* a, const double* b) {
    double s = 0;
    for (long i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

double orc_true_residual(long n, const int64_t* rowptr, const int32_t* col, const double* vals, const double* x,
                         const double* b) {
    double* r = (double*)malloc(sizeof(double) * n);
    orc_spmv(n, rowptr, col, vals, x, r);
    for (long i = 0; i < n; ++i) r[i] = b[i] - r[i];
    double res = sqrt(dot(n, r, r)) / sqrt(dot(n, b, b));
    free(r);
    return res;
}

long orc_jacobi_pcg(long n, const int64_t* rowptr, const int32_t* col, const double* vals, const double* b,
                    double* x, double rtol, long maxit, double* final_rel) {
    double* r = (double*)malloc(sizeof(double) * n);
    double* z = (double*)malloc(sizeof(double) * n);
    double* p = (double*)malloc(sizeof(double) * n);
    double* q = (double*)malloc(sizeof(double) * n);
    double* dinv = (double*)malloc(sizeof(double) * n);
    for (long i = 0; i < n; ++i) {
        long s = find_slot(rowptr, col, i, (int32_t)i);
        double d = s >= 0 ? vals[s] : 0.0;
        dinv[i] = d != 0 ? 1.0 / d : 1.0;
    }
    orc_spmv(n, rowptr, col, vals, x, q);
    for (long i = 0; i < n; ++i) r[i] = b[i] - q[i];
    double bn = sqrt(dot(n, b, b));
    if (bn == 0) bn = 1;
    for (long i = 0; i < n; ++i) z[i] = dinv[i] * r[i];
    memcpy(p, z, sizeof(double) * n);
    double rz = dot(n, r, z);
    long it = 0;
    double rel = sqrt(dot(n, r, r)) / bn;
    while (rel > rtol && it < maxit) {
        orc_spmv(n, rowptr, col, vals, p, q);
        double alpha = rz / dot(n, p, q);
        for (long i = 0; i < n; ++i) {
            x[i] += alpha * p[i];
            r[i] -= alpha * q[i];
        }
        for (long i = 0; i < n; ++i) z[i] = dinv[i] * r[i];
        double rz1 = dot(n, r, z);
        double beta = rz1 / rz;
        rz = rz1;
        for (long i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
        ++it;
        rel = sqrt(dot(n, r, r)) / bn;
    }
    if (final_rel) *final_rel = rel;
    free(r);
    free(z);
    free(p);
    free(q);
    free(dinv);
    return rel <= rtol ? it : -1;
}

/* ---------------------------------------------------------------- CPU baseline */

struct chunk {
    long nt;
    const double *XY, *D6;
    int order;
    double* A;
};
static void* run_chunk(void* arg) {
    struct chunk* c = (struct chunk*)arg;
    gradgrad_sym(2, c->order, c->nt, c->XY, c->D6, c->A);
    return NULL;
}

double orc_time_p2_sym(long nt, const double* XY, const double* D6, int order, int nthreads, double* A) {
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    if (nthreads <= 1) {
        gradgrad_sym(2, order, nt, XY, D6, A);
    } else {
        pthread_t th[256];
        struct chunk cs[256];
        if (nthreads > 256) nthreads = 256;
        long per = (nt + nthreads - 1) / nthreads;
        int k = 0;
        for (int i = 0; i < nthreads; ++i) {
            long b = i * per, e = b + per < nt ? b + per : nt;
            if (b >= e) break;
            cs[k].nt = e - b;
            cs[k].XY = XY + 12 * b;
            cs[k].D6 = D6 + 6 * b;
            cs[k].order = order;
            cs[k].A = A + 100 * b;
            pthread_create(&th[k], NULL, run_chunk, &cs[k]);
            ++k;
        }
        for (int i = 0; i < k; ++i) pthread_join(th[i], NULL);
    }
    clock_gettime(CLOCK_MONOTONIC, &t1);
    return (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);
}

/* ---------------------------------------------------------------- multi-threaded drivers
 * The same restatements split over host threads, for full-size parity checks and the CPU
 * baselines.  Every output value is computed with the same arithmetic and summation order as the
 * serial functions above (threads own disjoint tets or rows), so the results are bitwise equal. */

typedef void (*range_fn)(long b, long e, void* ctx);
struct par_arg {
    range_fn fn;
    long b, e;
    void* ctx;
};
static void* par_run(void* a) {
    struct par_arg* p = (struct par_arg*)a;
    p->fn(p->b, p->e, p->ctx);
    return NULL;
}
static void par_for(long n, int nthreads, range_fn fn, void* ctx) {
    if (nthreads <= 1 || n < 2) {
        fn(0, n, ctx);
        return;
    }
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    struct par_arg args[256];
    long per = (n + nthreads - 1) / nthreads;
    int k = 0;
    for (int i = 0; i < nthreads; ++i) {
        long b = i * per, e = b + per < n ? b + per : n;
        if (b >= e) break;
        args[k].fn = fn;
        args[k].b = b;
        args[k].e = e;
        args[k].ctx = ctx;
        pthread_create(&th[k], NULL, par_run, &args[k]);
        ++k;
    }
    for (int i = 0; i < k; ++i) pthread_join(th[i], NULL);
}

struct elem_ctx {
    int codeA, codeB, kind, q, nfA, nfB, dA, dB;
    const double *pp, *ww, *XY, *D;
    double* A;
    int rc;
};
static void elem_range(long b, long e, void* c) {
    struct elem_ctx* x = (struct elem_ctx*)c;
    const double* D = x->D;
    size_t per = 0;
    switch (x->kind) {
        case ORC_TET_SCALAR: per = 1; break;
        case ORC_TET_SYM: per = 6; break;
        case ORC_TET_GENERAL: per = (size_t)x->dA * x->dB; break;
        case ORC_POINT: per = (size_t)x->dA * x->dB * x->q; break;
    }
    if (D) D += per * (size_t)b;
    int rc = elem_core(x->codeA, x->codeB, x->kind, x->pp, x->ww, x->q, -1, 0, e - b, x->XY + 12 * b, D,
                       x->A + (size_t)x->nfA * x->nfB * b);
    if (rc) x->rc = rc;
}

/* orc_fem3dtet over nthreads host threads (contiguous tet chunks) */
int orc_fem3dtet_mt(int codeA, int codeB, int kind, int order, long nt, const double* XY, const double* D, double* A,
                    int nthreads) {
    struct elem_ctx c;
    if (!anigpu_quad_rule(order, &c.pp, &c.ww, &c.q)) return -1;
    if (orc_op_info(codeA, &c.nfA, &c.dA) || orc_op_info(codeB, &c.nfB, &c.dB)) return -1;
    c.codeA = codeA, c.codeB = codeB, c.kind = kind, c.XY = XY, c.D = D, c.A = A, c.rc = 0;
    par_for(nt, nthreads, elem_range, &c);
    return c.rc;
}

struct dir_ctx {
    int nloc;
    double *A, *F;
    const int32_t* edofs;
    const uint8_t* mask;
    const double* bc;
};
static void dir_range(long b, long e, void* c) {
    struct dir_ctx* x = (struct dir_ctx*)c;
    for (long t = b; t < e; ++t)
        for (int k = 0; k < x->nloc; ++k) {
            const int32_t d = x->edofs[(size_t)x->nloc * t + k];
            if (x->mask[d])
                orc_apply_dir(x->nloc, x->A + (size_t)x->nloc * x->nloc * t, x->F + (size_t)x->nloc * t, k,
                              x->bc ? x->bc[d] : 0.0);
        }
}

/* applyDir on every element DOF whose global DOF is masked, local DOFs in ascending order (the
 * element loop of a local assembler, dc_on_dof.h:24-45) */
void orc_apply_dir_elems(long nt, int nloc, double* A, double* F, const int32_t* edofs, const uint8_t* mask,
                         const double* bc, int nthreads) {
    struct dir_ctx c = {nloc, A, F, edofs, mask, bc};
    par_for(nt, nthreads, dir_range, &c);
}

struct tmpl_ctx {
    int nloc;
    const int32_t* edofs;
    const int64_t *ip;
    const int32_t* itet;
    int64_t* rowptr; /* pass 1: counts in rowptr[r + 1]; pass 2: offsets */
    int32_t* col;
};
static long row_columns(const struct tmpl_ctx* x, long r, int32_t** buf, long* cap) {
    long deg = x->ip[r + 1] - x->ip[r];
    if (deg * x->nloc + 1 > *cap) {
        *cap = deg * x->nloc + 1;
        *buf = (int32_t*)realloc(*buf, sizeof(int32_t) * (size_t)*cap);
    }
    long m = 0;
    (*buf)[m++] = (int32_t)r;
    for (int64_t k = x->ip[r]; k < x->ip[r + 1]; ++k)
        for (int j = 0; j < x->nloc; ++j) (*buf)[m++] = x->edofs[(size_t)x->nloc * x->itet[k] + j];
    qsort(*buf, m, sizeof(int32_t), cmp_i32);
    long u = 0;
    for (long k = 0; k < m; ++k)
        if (k == 0 || (*buf)[k] != (*buf)[k - 1]) (*buf)[u++] = (*buf)[k];
    return u;
}
static void tmpl_count(long b, long e, void* c) {
    struct tmpl_ctx* x = (struct tmpl_ctx*)c;
    long cap = 0;
    int32_t* buf = NULL;
    for (long r = b; r < e; ++r) x->rowptr[r + 1] = row_columns(x, r, &buf, &cap);
    free(buf);
}
static void tmpl_fill(long b, long e, void* c) {
    struct tmpl_ctx* x = (struct tmpl_ctx*)c;
    long cap = 0;
    int32_t* buf = NULL;
    for (long r = b; r < e; ++r) {
        long u = row_columns(x, r, &buf, &cap);
        memcpy(x->col + x->rowptr[r], buf, sizeof(int32_t) * (size_t)u);
    }
    free(buf);
}

/* orc_csr_template over nthreads threads: the same rows (sorted unique DOFs of the incident
 * tets plus the diagonal); pass 1 counts, pass 2 fills (col NULL: counts only, returns nnz) */
long orc_csr_template_mt(long ndof, long nt, int nloc, const int32_t* edofs, int64_t* rowptr, int32_t* col,
                         int nthreads) {
    int64_t* ip;
    int32_t* itet;
    incidence(ndof, nt, nloc, edofs, &ip, &itet);
    struct tmpl_ctx c = {nloc, edofs, ip, itet, rowptr, col};
    rowptr[0] = 0;
    par_for(ndof, nthreads, tmpl_count, &c);
    for (long r = 0; r < ndof; ++r) rowptr[r + 1] += rowptr[r];
    if (col) par_for(ndof, nthreads, tmpl_fill, &c);
    long nnz = rowptr[ndof];
    free(ip);
    free(itet);
    return nnz;
}

struct scat_ctx {
    int nloc;
    const int64_t *rowptr, *ip;
    const int32_t *col, *edofs, *itet;
    const double *Aelem, *Felem;
    double drop;
    double *vals, *rhs;
    uint8_t* touched;
    int rc;
};
static void scat_range(long b, long e, void* c) {
    struct scat_ctx* x = (struct scat_ctx*)c;
    const int n = x->nloc;
    for (long r = b; r < e; ++r)
        for (int64_t k = x->ip[r]; k < x->ip[r + 1]; ++k) { /* incident tets in ascending order */
            const long t = x->itet[k];
            const int32_t* ed = x->edofs + (size_t)n * t;
            int i = 0;
            while (i < n && ed[i] != r) ++i;
            if (x->Felem) {
                const double f = x->Felem[(size_t)n * t + i];
                if (!isfinite(f)) x->rc = -1;
                x->rhs[r] += f;
            }
            const double* Ae = x->Aelem + (size_t)n * n * t;
            for (int j = 0; j < n; ++j) {
                const double a = Ae[i + n * j];
                if (!isfinite(a)) x->rc = -1;
                if (fabs(a) > x->drop) {
                    long s = find_slot(x->rowptr, x->col, r, ed[j]);
                    if (s < 0) {
                        x->rc = -2;
                        continue;
                    }
                    x->vals[s] += a;
                    if (x->touched) x->touched[s] = 1;
                }
            }
        }
}

/* orc_scatter over nthreads threads: threads own rows and add each row's element rows in
 * ascending tet order, the per-slot order of the serial tet loop (so the sums are bitwise equal) */
int orc_scatter_mt(long ndof, const int64_t* rowptr, const int32_t* col, long nt, int nloc, const int32_t* edofs,
                   const double* Aelem, const double* Felem, double drop, double* vals, double* rhs,
                   uint8_t* touched, int nthreads) {
    int64_t* ip;
    int32_t* itet;
    incidence(ndof, nt, nloc, edofs, &ip, &itet);
    struct scat_ctx c = {nloc, rowptr, ip, col, edofs, itet, Aelem, Felem, drop, vals, rhs, touched, 0};
    par_for(ndof, nthreads, scat_range, &c);
    free(ip);
    free(itet);
    return c.rc;
}

struct vec_ctx {
    long n;
    const int64_t* rowptr;
    const int32_t* col;
    const double* vals;
    double *x, *r, *z, *p, *q, *dinv;
    double alpha, beta;
    int op;
    double part[256];
    int nthreads;
};
static void pcg_range(long b, long e, void* c) {
    struct vec_ctx* x = (struct vec_ctx*)c;
    const long per = (x->n + x->nthreads - 1) / x->nthreads;
    const int slot = (int)(b / (per > 0 ? per : 1));
    double s = 0;
    if (x->op == 0) { /* q = A p, partial p.q */
        for (long i = b; i < e; ++i) {
            double v = 0;
            for (int64_t k = x->rowptr[i]; k < x->rowptr[i + 1]; ++k) v += x->vals[k] * x->p[x->col[k]];
            x->q[i] = v;
            s += x->p[i] * v;
        }
    } else if (x->op == 1) { /* x += a p, r -= a q, z = D^-1 r, partial r.z */
        for (long i = b; i < e; ++i) {
            x->x[i] += x->alpha * x->p[i];
            x->r[i] -= x->alpha * x->q[i];
            x->z[i] = x->dinv[i] * x->r[i];
            s += x->r[i] * x->z[i];
        }
    } else { /* p = z + b p */
        for (long i = b; i < e; ++i) x->p[i] = x->z[i] + x->beta * x->p[i];
    }
    x->part[slot] = s;
}

/* Seconds of `iters` Jacobi-PCG iterations (FP64, from x = 0) over nthreads threads: the CPU
 * baseline of the solve (a restatement: the reference solves through INMOST).  Dot products are
 * per-thread partial sums added in thread order. */
double orc_pcg_time_mt(long n, const int64_t* rowptr, const int32_t* col, const double* vals, const double* b,
                       long iters, int nthreads) {
    if (nthreads > 256) nthreads = 256;
    if (nthreads < 1) nthreads = 1;
    struct vec_ctx c;
    memset(&c, 0, sizeof(c));
    c.n = n, c.rowptr = rowptr, c.col = col, c.vals = vals, c.nthreads = nthreads;
    c.x = (double*)calloc(n, sizeof(double));
    c.r = (double*)malloc(sizeof(double) * n);
    c.z = (double*)malloc(sizeof(double) * n);
    c.p = (double*)malloc(sizeof(double) * n);
    c.q = (double*)malloc(sizeof(double) * n);
    c.dinv = (double*)malloc(sizeof(double) * n);
    for (long i = 0; i < n; ++i) {
        long s = find_slot(rowptr, col, i, (int32_t)i);
        double d = s >= 0 ? vals[s] : 0.0;
        c.dinv[i] = d != 0 ? 1.0 / d : 1.0;
        c.r[i] = b[i];
        c.z[i] = c.dinv[i] * b[i];
        c.p[i] = c.z[i];
    }
    double rz = dot(n, c.r, c.z);
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    for (long it = 0; it < iters; ++it) {
        memset(c.part, 0, sizeof(c.part));
        c.op = 0;
        par_for(n, nthreads, pcg_range, &c);
        double pq = 0;
        for (int k = 0; k < nthreads; ++k) pq += c.part[k];
        c.alpha = rz / pq;
        memset(c.part, 0, sizeof(c.part));
        c.op = 1;
        par_for(n, nthreads, pcg_range, &c);
        double rz1 = 0;
        for (int k = 0; k < nthreads; ++k) rz1 += c.part[k];
        c.beta = rz1 / rz;
        rz = rz1;
        c.op = 2;
        par_for(n, nthreads, pcg_range, &c);
    }
    clock_gettime(CLOCK_MONOTONIC, &t1);
    free(c.x), free(c.r), free(c.z), free(c.p), free(c.q), free(c.dinv);
    return (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);
}
