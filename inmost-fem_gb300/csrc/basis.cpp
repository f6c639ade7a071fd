// Host-side reference-element tables: basis values and reference gradients of the
// Lagrange spaces P0..P3 at the points of a quadrature rule (the basis itself is in
// basis_eval.h, shared with the device code).
#include <cmath>

#include "anigpu_internal.h"
#include "quad_tables.h"
#include "tri_quad_tables.h"
#include "basis_eval.h"

namespace {
int eval_space(int space, const double* l, double* v, double (*g)[3]) { return ani_eval_space(space, l, v, g); }
}  // namespace

int scalar_space_nf(int space) {
    switch (space) {
        case ANIGPU_P0: return 1;
        case ANIGPU_P1: return 4;
        case ANIGPU_P2: return 10;
        case ANIGPU_P3: return 20;
        case ANIGPU_CR1: return 4;
        case ANIGPU_B2: return 6;
        case ANIGPU_B4: return 1;
    }
    return -1;
}

bool op_info(int code, int* nf, int* dim, int* base_space, int* ncomp, int* op) {
    const int space = code / 10, o = code % 10;
    if (space == ANIGPU_ND0 || space == ANIGPU_RT0) {  // vector-valued: IDEN, GRAD, DIV, CURL
        if (o < ANIGPU_IDEN || o > ANIGPU_CURL) return false;
        static const int dims[5] = {0, 3, 9, 1, 3};
        *nf = space == ANIGPU_ND0 ? 6 : 4;
        *dim = dims[o];
        *base_space = space;
        *ncomp = 1;
        *op = o;
        return true;
    }
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

bool make_scalar_basis_face(int space, int order, int face, ScalarBasisTable* t) {
    const double *p3, *w;
    int q;
    if (face < 0 || face > 3 || order < 0 || order > ANIGPU_TRI_MAX_ORDER) return false;
    if (!anigpu_tri_rule(order, &p3, &w, &q)) return false;
    const int nf = scalar_space_nf(space);
    if (nf < 0) return false;
    t->space = space;
    t->order = order;
    t->q = q;
    t->nf = nf;
    t->pts.assign((size_t)4 * q, 0.0);
    for (int n = 0; n < q; ++n) {  // int_face.inl:31-36
        t->pts[4 * n + face] = p3[3 * n + 0];
        t->pts[4 * n + (face + 1) % 4] = p3[3 * n + 1];
        t->pts[4 * n + (face + 2) % 4] = p3[3 * n + 2];
        t->pts[4 * n + (face + 3) % 4] = 0.0;
    }
    t->wts.assign(w, w + q);
    t->val.assign((size_t)q * nf, 0.0);
    t->grad.assign((size_t)q * nf * 3, 0.0);
    for (int n = 0; n < q; ++n) {
        double v[20], g[20][3];
        eval_space(space, t->pts.data() + 4 * n, v, g);
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
