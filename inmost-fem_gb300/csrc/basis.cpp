// Host-side reference-element tables: basis values and reference gradients of the
// Lagrange spaces P0..P3 at the points of a quadrature rule.
//
// Basis definitions and DOF order follow the reference's spaces:
//   P0  anifem++/fem/spaces/poly_0.h         constant
//   P1  anifem++/fem/spaces/poly_1.h:12,91   lambda_i
//   P2  anifem++/fem/spaces/poly_2.h:12-100  vertices lambda_i(2 lambda_i - 1), then edges
//       4 lambda_I lambda_J in edge order (0,1),(0,2),(0,3),(1,2),(1,3),(2,3)
//   P3  anifem++/fem/spaces/poly_3.h:12-110  vertices, two DOFs per edge (same edge order),
//       faces 27 lambda_a lambda_b lambda_c for faces {0,1,2},{1,2,3},{0,2,3},{0,1,3}
// Reference gradients are d/dxi_d with lambda_0 = 1 - xi_1 - xi_2 - xi_3, lambda_k = xi_k.
#include <cmath>

#include "anigpu_internal.h"
#include "quad_tables.h"

namespace {
const int kEI[6] = {0, 0, 0, 1, 1, 2}, kEJ[6] = {1, 2, 3, 2, 3, 3};
const int kFace[4][3] = {{0, 1, 2}, {1, 2, 3}, {0, 2, 3}, {0, 1, 3}};

inline double dlam(int i, int d) { return i == 0 ? -1.0 : (i - 1 == d ? 1.0 : 0.0); }

int eval_space(int space, const double* l, double* v, double (*g)[3]) {
    switch (space) {
        case ANIGPU_P0:
            v[0] = 1;
            g[0][0] = g[0][1] = g[0][2] = 0;
            return 1;
        case ANIGPU_P1:
            for (int i = 0; i < 4; ++i) {
                v[i] = l[i];
                for (int d = 0; d < 3; ++d) g[i][d] = dlam(i, d);
            }
            return 4;
        case ANIGPU_P2:
            for (int i = 0; i < 4; ++i) {
                v[i] = l[i] * (2 * l[i] - 1);
                for (int d = 0; d < 3; ++d) g[i][d] = dlam(i, d) * (4 * l[i] - 1);
            }
            for (int e = 0; e < 6; ++e) {
                const double a = l[kEI[e]], b = l[kEJ[e]];
                v[4 + e] = 4 * a * b;
                for (int d = 0; d < 3; ++d) g[4 + e][d] = 4 * (dlam(kEI[e], d) * b + dlam(kEJ[e], d) * a);
            }
            return 10;
        case ANIGPU_P3:
            for (int i = 0; i < 4; ++i) {
                const double s = l[i];
                v[i] = s * (3 * s - 1) * (3 * s - 2) / 2;
                for (int d = 0; d < 3; ++d) g[i][d] = dlam(i, d) * ((13.5 * s - 9) * s + 1);
            }
            for (int e = 0; e < 6; ++e) {
                const int I = kEI[e], J = kEJ[e];
                const double a = l[I], b = l[J];
                v[4 + 2 * e] = 4.5 * a * (3 * a - 1) * b;
                v[5 + 2 * e] = 4.5 * a * (3 * b - 1) * b;
                for (int d = 0; d < 3; ++d) {
                    g[4 + 2 * e][d] = 4.5 * (dlam(I, d) * (6 * a - 1) * b + dlam(J, d) * (3 * a - 1) * a);
                    g[5 + 2 * e][d] = 4.5 * (dlam(J, d) * (6 * b - 1) * a + dlam(I, d) * (3 * b - 1) * b);
                }
            }
            for (int f = 0; f < 4; ++f) {
                const int a = kFace[f][0], b = kFace[f][1], c = kFace[f][2];
                v[16 + f] = 27 * l[a] * l[b] * l[c];
                for (int d = 0; d < 3; ++d)
                    g[16 + f][d] = 27 * (dlam(a, d) * l[b] * l[c] + l[a] * dlam(b, d) * l[c] + l[a] * l[b] * dlam(c, d));
            }
            return 20;
    }
    return -1;
}
}  // namespace

int scalar_space_nf(int space) {
    switch (space) {
        case ANIGPU_P0: return 1;
        case ANIGPU_P1: return 4;
        case ANIGPU_P2: return 10;
        case ANIGPU_P3: return 20;
    }
    return -1;
}

bool op_info(int code, int* nf, int* dim, int* base_space, int* ncomp, int* op) {
    const int space = code / 10, o = code % 10;
    if (o != ANIGPU_IDEN && o != ANIGPU_GRAD) return false;
    int base = space, nc = 1;
    if (space == ANIGPU_VEC3_P1 || space == ANIGPU_VEC3_P2) {
        base = space - 3;
        nc = 3;
    }
    const int n = scalar_space_nf(base);
    if (n < 0) return false;
    const int bd = (o == ANIGPU_IDEN) ? 1 : 3;
    *nf = n * nc;
    *dim = bd * nc;
    *base_space = base;
    *ncomp = nc;
    *op = o;
    return true;
}

bool make_scalar_basis(int space, int order, ScalarBasisTable* t) {
    const double *p, *w;
    int q;
    if (!anigpu_quad_rule(order, &p, &w, &q)) return false;
    const int nf = scalar_space_nf(space);
    if (nf < 0) return false;
    t->space = space;
    t->order = order;
    t->q = q;
    t->nf = nf;
    t->pts.assign(p, p + 4 * q);
    t->wts.assign(w, w + q);
    t->val.assign((size_t)q * nf, 0.0);
    t->grad.assign((size_t)q * nf * 3, 0.0);
    for (int n = 0; n < q; ++n) {
        double v[20], g[20][3];
        eval_space(space, p + 4 * n, v, g);
        for (int i = 0; i < nf; ++i) {
            t->val[(size_t)n * nf + i] = v[i];
            for (int d = 0; d < 3; ++d) t->grad[((size_t)n * nf + i) * 3 + d] = g[i][d];
        }
    }
    return true;
}

// Basis values and reference gradients at one barycentric point, without any allocation
// (for callers that must not allocate).  Returns the number of basis functions or -1.
int eval_scalar_basis_at(int space, const double* l, double* val, double (*grad)[3]) {
    return eval_space(space, l, val, grad);
}
