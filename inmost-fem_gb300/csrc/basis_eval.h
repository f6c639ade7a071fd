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
