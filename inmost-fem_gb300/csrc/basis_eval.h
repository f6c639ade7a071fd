// Basis values and reference gradients of the Lagrange spaces P0..P3 at one barycentric
// point, for host and device code.
//
// Basis definitions and DOF order follow the reference's spaces:
//   P0  anifem++/fem/spaces/poly_0.h         constant
//   P1  anifem++/fem/spaces/poly_1.h:12,91   lambda_i
//   P2  anifem++/fem/spaces/poly_2.h:12-100  vertices lambda_i(2 lambda_i - 1), then edges
//       4 lambda_I lambda_J in edge order (0,1),(0,2),(0,3),(1,2),(1,3),(2,3)
//   P3  anifem++/fem/spaces/poly_3.h:12-110  vertices, two DOFs per edge (same edge order),
//       faces 27 lambda_a lambda_b lambda_c for faces {0,1,2},{1,2,3},{0,2,3},{0,1,3}
//   CR1 crouzeix_raviart_1.h:12-80, B2 bubble_2.h:12-80, B4 bubble_4.h:11-84
// Reference gradients are d/dxi_d with lambda_0 = 1 - xi_1 - xi_2 - xi_3, lambda_k = xi_k.
#pragma once
#include "anigpu.h"

#ifdef __CUDACC__
#define ANI_HD __host__ __device__
#else
#define ANI_HD
#endif

ANI_HD inline double ani_dlam(int i, int d) { return i == 0 ? -1.0 : (i - 1 == d ? 1.0 : 0.0); }

// values v[nf] and reference gradients g[nf][3] at barycentric l[4]; returns nf (-1: unknown space)
ANI_HD inline int ani_eval_space(int space, const double* l, double* v, double (*g)[3]) {
    const int kEI[6] = {0, 0, 0, 1, 1, 2}, kEJ[6] = {1, 2, 3, 2, 3, 3};
    const int kFace[4][3] = {{0, 1, 2}, {1, 2, 3}, {0, 2, 3}, {0, 1, 3}};

    switch (space) {
        case ANIGPU_P0:
            v[0] = 1;
            g[0][0] = g[0][1] = g[0][2] = 0;
            return 1;
        case ANIGPU_P1:
            for (int i = 0; i < 4; ++i) {
                v[i] = l[i];
                for (int d = 0; d < 3; ++d) g[i][d] = ani_dlam(i, d);
            }
            return 4;
        case ANIGPU_P2:
            for (int i = 0; i < 4; ++i) {
                v[i] = l[i] * (2 * l[i] - 1);
                for (int d = 0; d < 3; ++d) g[i][d] = ani_dlam(i, d) * (4 * l[i] - 1);
            }
            for (int e = 0; e < 6; ++e) {
                const double a = l[kEI[e]], b = l[kEJ[e]];
                v[4 + e] = 4 * a * b;
                for (int d = 0; d < 3; ++d) g[4 + e][d] = 4 * (ani_dlam(kEI[e], d) * b + ani_dlam(kEJ[e], d) * a);
            }
            return 10;
        case ANIGPU_P3:
            for (int i = 0; i < 4; ++i) {
                const double s = l[i];
                v[i] = s * (3 * s - 1) * (3 * s - 2) / 2;
                for (int d = 0; d < 3; ++d) g[i][d] = ani_dlam(i, d) * ((13.5 * s - 9) * s + 1);
            }
            for (int e = 0; e < 6; ++e) {
                const int I = kEI[e], J = kEJ[e];
                const double a = l[I], b = l[J];
                v[4 + 2 * e] = 4.5 * a * (3 * a - 1) * b;
                v[5 + 2 * e] = 4.5 * a * (3 * b - 1) * b;
                for (int d = 0; d < 3; ++d) {
                    g[4 + 2 * e][d] = 4.5 * (ani_dlam(I, d) * (6 * a - 1) * b + ani_dlam(J, d) * (3 * a - 1) * a);
                    g[5 + 2 * e][d] = 4.5 * (ani_dlam(J, d) * (6 * b - 1) * a + ani_dlam(I, d) * (3 * b - 1) * b);
                }
            }
            for (int f = 0; f < 4; ++f) {
                const int a = kFace[f][0], b = kFace[f][1], c = kFace[f][2];
                v[16 + f] = 27 * l[a] * l[b] * l[c];
                for (int d = 0; d < 3; ++d)
                    g[16 + f][d] = 27 * (ani_dlam(a, d) * l[b] * l[c] + l[a] * ani_dlam(b, d) * l[c] + l[a] * l[b] * ani_dlam(c, d));
            }
            return 20;
        case ANIGPU_CR1:  // crouzeix_raviart_1.h: DOF i on the face opposite vertex {3,0,1,2}[i]
            for (int i = 0; i < 4; ++i) {
                const int o = (i + 3) & 3;
                v[i] = 1 - 3 * l[o];
                for (int d = 0; d < 3; ++d) g[i][d] = -3 * ani_dlam(o, d);
            }
            return 4;
        case ANIGPU_B2:  // bubble_2.h: 4 lambda_I lambda_J on edge (I,J), edge order as P2
            for (int e = 0; e < 6; ++e) {
                const double a = l[kEI[e]], b = l[kEJ[e]];
                v[e] = 4 * a * b;
                for (int d = 0; d < 3; ++d) g[e][d] = 4 * (ani_dlam(kEI[e], d) * b + ani_dlam(kEJ[e], d) * a);
            }
            return 6;
        case ANIGPU_B4:  // bubble_4.h: 256 lambda_0 lambda_1 lambda_2 lambda_3
            v[0] = 256 * l[0] * l[1] * l[2] * l[3];
            for (int d = 0; d < 3; ++d)
                g[0][d] = 256 * (ani_dlam(0, d) * l[1] * l[2] * l[3] + ani_dlam(1, d) * l[0] * l[2] * l[3] +
                                 ani_dlam(2, d) * l[0] * l[1] * l[3] + ani_dlam(3, d) * l[0] * l[1] * l[2]);
            return 1;
    }
    return -1;
}

// ---- vector-valued lowest-order spaces (geometry dependent)
//   ND0 (spaces/nedelec_0.h:12-183): DOF i on edge (ip0, ip1) of IPR = {0,1,2,3, 0,2,3,1, 0,3,1,2,
//       1,2,0,3, 1,3,2,0, 2,3,0,1}; with P = vertex coordinates relative to X0, s = |P_ip0 - P_ip1| / det
//       (signed det), n = (P_ip2 - P_ip0) x (P_ip3 - P_ip0), m = (P_ip2 - P_ip1) x (P_ip3 - P_ip1):
//       IDEN = s (n lambda_ip0 + m lambda_ip1), CURL_k = s ((g_ip0 (k+1) n_(k+2) + g_ip1 (k+1) m_(k+2))
//       - (g_ip0 (k+2) n_(k+1) + g_ip1 (k+2) m_(k+1))), DIV = 0, GRAD = the skew matrix of CURL / 2.
//   RT0 (spaces/raviant_thomas_0.h:12-190): DOF i on face (ip0, ip1, ip2) of IPF = {0,1,2,3, 1,2,3,0,
//       0,2,3,1, 0,1,3,2}, opposite vertex ip3; s = area(P_ip0, P_ip1, P_ip2) / (|det| / 2):
//       IDEN_j = s sum_{a<3} lambda_ipa (P_ipa - P_ip3)_j, GRAD_(k + 3j) = s sum_a g_ipa(k) (P_ipa - P_ip3)_j,
//       DIV = sum_j GRAD_(j + 3j), CURL = 0.
// g_v(k) = d lambda_v / dx_k = sum_m dlam(v, m) PSI(m, k).  Returns the value of row `k` of operator
// `op` (ANIGPU_IDEN, GRAD, DIV, CURL) for DOF `i` at barycentric l.

ANI_HD inline double ani_glam(const double* PSI, int v, int k) {
    return ani_dlam(v, 0) * PSI[0 + 3 * k] + ani_dlam(v, 1) * PSI[1 + 3 * k] + ani_dlam(v, 2) * PSI[2 + 3 * k];
}

ANI_HD inline void ani_sub_cross(const double* p0, const double* p1, const double* p2, double* c) {
    // (p0 - p2) x (p1 - p2), geometry.h:57-64
    const double a[3] = {p0[0] - p2[0], p0[1] - p2[1], p0[2] - p2[2]};
    const double b[3] = {p1[0] - p2[0], p1[1] - p2[1], p1[2] - p2[2]};
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = -a[0] * b[2] + a[2] * b[0];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

// P: vertex coordinates relative to X0 (P[3v + k]); det: signed determinant of [P1 P2 P3]
ANI_HD inline double ani_vec_space_value(int space, int op, const double* l, const double* PSI, const double* P,
                                         double det, int i, int k) {
    if (space == ANIGPU_ND0) {
        const unsigned char IPR[24] = {0, 1, 2, 3, 0, 2, 3, 1, 0, 3, 1, 2, 1, 2, 0, 3, 1, 3, 2, 0, 2, 3, 0, 1};
        const unsigned char* ip = IPR + 4 * i;
        double sq = 0.0;
        for (int c = 0; c < 3; ++c) {
            const double t = P[3 * ip[0] + c] - P[3 * ip[1] + c];
            sq += t * t;
        }
        const double s = sqrt(sq) / det;
        double xn[3], xm[3];
        ani_sub_cross(P + 3 * ip[2], P + 3 * ip[3], P + 3 * ip[0], xn);
        ani_sub_cross(P + 3 * ip[2], P + 3 * ip[3], P + 3 * ip[1], xm);
        if (op == ANIGPU_IDEN) return s * (xn[k] * l[ip[0]] + xm[k] * l[ip[1]]);
        if (op == ANIGPU_DIV) return 0.0;
        auto curl = [&](int kk) {
            const int k1 = (kk + 1) % 3, k2 = (kk + 2) % 3;
            return s * ((ani_glam(PSI, ip[0], k1) * xn[k2] + ani_glam(PSI, ip[1], k1) * xm[k2]) -
                        (ani_glam(PSI, ip[0], k2) * xn[k1] + ani_glam(PSI, ip[1], k2) * xm[k1]));
        };
        if (op == ANIGPU_CURL) return curl(k);
        // GRAD: 3x3 column-major skew matrix of a = curl/2 (nedelec_0.h:172-177)
        const int r = k % 3, c = k / 3;
        if (r == c) return 0.0;
        const int t = 3 - r - c;            // the third index
        const double a = curl(t) / 2;
        return r == (c + 1) % 3 ? -a : a;  // entries (1,0), (2,1), (0,2) carry -a_t, the others +a_t
    }
    // RT0
    const unsigned char IPF[16] = {0, 1, 2, 3, 1, 2, 3, 0, 0, 2, 3, 1, 0, 1, 3, 2};
    const unsigned char* ip = IPF + 4 * i;
    double cr[3];
    ani_sub_cross(P + 3 * ip[0], P + 3 * ip[1], P + 3 * ip[2], cr);
    const double area = sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]) / 2;
    const double s = area / (fabs(det) / 2);
    if (op == ANIGPU_IDEN) {
        double v = 0.0;
        for (int a = 0; a < 3; ++a) v += l[ip[a]] * (P[3 * ip[a] + k] - P[3 * ip[3] + k]);
        return s * v;
    }
    if (op == ANIGPU_CURL) return 0.0;
    if (op == ANIGPU_GRAD) {
        const int kk = k % 3, j = k / 3;
        double v = 0.0;
        for (int a = 0; a < 3; ++a) v += ani_glam(PSI, ip[a], kk) * (P[3 * ip[a] + j] - P[3 * ip[3] + j]);
        return s * v;
    }
    double v = 0.0;  // DIV
    for (int j = 0; j < 3; ++j)
        for (int a = 0; a < 3; ++a) v += ani_glam(PSI, ip[a], j) * (P[3 * ip[a] + j] - P[3 * ip[3] + j]);
    return s * v;
}
