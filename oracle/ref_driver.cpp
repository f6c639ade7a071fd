// Test infrastructure only (the oracle): a C driver around the reference
// library's own element-matrix routine, compiled from the reference sources in
// place by oracle/Makefile into oracle/_ref/libanifem_ref.so.  Nothing here is
// product code; only tests/, the smoke check and bench.py's CPU-baseline leg use it.
//
// It instantiates Ani::fem3Dtet (anifem++/fem/operations/int_tet.inl:93-122, the
// memoryless stack overload; and :30-57 for the PlainMemory overload used above
// order 6) for the operator pairs the parity tests need, and exposes
// Ani::tetrahedron_quadrature_formulas (anifem++/fem/quadrature_formulas.cpp:526)
// Ani::applyDir (anifem++/fem/operations/dc_on_dof.h:39-45) and Ani::fem3DapplyL/X
// (anifem++/fem/operations/eval.h, eval.inl:93-151).
#include "anifem++/fem/operations/operations.h"
#include "anifem++/fem/operators.h"
#include "anifem++/fem/spaces/spaces.h"

#include <chrono>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

using namespace Ani;

namespace {

// analytic per-point tensor fields shared with tests/ (same formulas in numpy)
// fn 0: the reference test field D(i,j) = (i*x0 + j*x1 + (i%2)*x2) * cnt++, TENSOR_GENERAL
//       (tests/fem/operations/int_tet_test.cpp:208-219)
// fn 1: scalar 1 + x0^2 (examples/tutorials/ex1.cpp:61-65)
// fn 2: symmetric 3x3 [[1+x^2, xy/2, 0],[xy/2, 1+y^2, z/3],[0, z/3, 2+z^2]]
// fn 3: scalar x0^2 (int_tet_test.cpp:405-409)
TensorType eval_fn(int fn, const std::array<double, 3>& x, double* D, size_t nr, size_t nc) {
    switch (fn) {
        case 0: {
            int cnt = 0;
            for (size_t i = 0; i < nr; ++i)
                for (size_t j = 0; j < nc; ++j)
                    D[i + nr * j] = (i * x[0] + j * x[1] + (i % 2) * x[2]) * (cnt++);
            return TENSOR_GENERAL;
        }
        case 1: D[0] = 1 + x[0] * x[0]; return TENSOR_SCALAR;
        case 2: {
            double m[9] = {1 + x[0] * x[0], x[0] * x[1] / 2, 0,
                           x[0] * x[1] / 2, 1 + x[1] * x[1], x[2] / 3,
                           0, x[2] / 3, 2 + x[2] * x[2]};
            for (int i = 0; i < 9; ++i) D[i] = m[i];
            return TENSOR_SYMMETRIC;
        }
        case 3: D[0] = x[0] * x[0]; return TENSOR_SCALAR;
    }
    return TENSOR_NULL;
}

// tensor kinds understood by ref_fem3dtet
enum { K_NULL = 0, K_CONST_SCALAR = 1, K_TET_SCALAR = 2, K_TET_SYM = 3, K_TET_GENERAL = 4, K_POINT_FN = 5 };

struct Req {
    int kind, order, fn;
    long nt;
    const double* XY;  // nt * 12 (X0 X1 X2 X3)
    const double* D;
    double* A;
};

// face of the fem3Dface requests (-1: fem3Dtet); g_normal: fem3DfaceN (tensor rows x 3)
int g_face = -1;
int g_normal = 0;

template <typename OpA, typename OpB, typename Traits, typename F>
void run_pairs(const Req& r, const F& functor_for_tet) {
    constexpr int nfA = OpA::Nfa::value, nfB = OpB::Nfa::value;
    for (long t = 0; t < r.nt; ++t) {
        const double* X = r.XY + 12 * t;
        DenseMatrix<> XY0(const_cast<double*>(X + 0), 3, 1), XY1(const_cast<double*>(X + 3), 3, 1),
            XY2(const_cast<double*>(X + 6), 3, 1), XY3(const_cast<double*>(X + 9), 3, 1);
        DenseMatrix<> A(r.A + (size_t)t * nfA * nfB, nfB, nfA, nfA * nfB);
        auto f = functor_for_tet(t);
        if (g_face >= 0 && r.order > 9) {  // the PlainMemory overloads take triangle orders up to 20
            auto req = g_normal ? fem3DfaceN_memory_requirements<OpA, OpB>(r.order, 1)
                                : fem3Dface_memory_requirements<OpA, OpB>(r.order, 1);
            std::vector<char> raw(req.enoughRawSize());
            req.allocateFromRaw(raw.data(), raw.size());
            if (g_normal)
                fem3DfaceN<OpA, OpB, Traits>(make_tetras(X, X + 3, X + 6, X + 9, 1), g_face, f, A, req, r.order);
            else
                fem3Dface<OpA, OpB, Traits>(make_tetras(X, X + 3, X + 6, X + 9, 1), g_face, f, A, req, r.order);
        } else if (g_face >= 0 && g_normal) {
            fem3DfaceN<OpA, OpB, Traits>(make_tetras(X, X + 3, X + 6, X + 9, 1), g_face, f, A, r.order);
        } else if (g_face >= 0) {
            fem3Dface<OpA, OpB, Traits>(make_tetras(X, X + 3, X + 6, X + 9, 1), g_face, f, A, r.order);
        } else if (r.order <= 6) {
            fem3Dtet<OpA, OpB, Traits>(XY0, XY1, XY2, XY3, f, A, r.order);
        } else {
            auto req = fem3Dtet_memory_requirements<OpA, OpB>(r.order, 1);
            std::vector<char> raw(req.enoughRawSize());
            req.allocateFromRaw(raw.data(), raw.size());
            fem3Dtet<OpA, OpB, Traits>(XY0, XY1, XY2, XY3, f, A, req, r.order);
        }
    }
}

template <typename OpA, typename OpB>
int run(const Req& r) {
    constexpr int dA = OpA::Dim::value, dB = OpB::Dim::value;
    const size_t nD = (size_t)dA * dB * (g_normal ? 3 : 1);
    switch (r.kind) {
        case K_NULL:
            run_pairs<OpA, OpB, DfuncTraits<TENSOR_NULL, true>>(r, [](long) { return TensorNull<>; });
            return 0;
        case K_CONST_SCALAR:
            run_pairs<OpA, OpB, DfuncTraits<TENSOR_SCALAR, true>>(r, [&](long) {
                double v = r.D[0];
                return [v](const std::array<double, 3>&, double* D, TensorDims, void*, int) { D[0] = v; return TENSOR_SCALAR; };
            });
            return 0;
        case K_TET_SCALAR:
            run_pairs<OpA, OpB, DfuncTraits<PerTetra, false>>(r, [&](long t) {
                double v = r.D[t];
                return [v](const std::array<double, 3>&, double* D, TensorDims, void*, int) { D[0] = v; return TENSOR_SCALAR; };
            });
            return 0;
        case K_TET_SYM:
            run_pairs<OpA, OpB, DfuncTraits<TENSOR_SYMMETRIC, false>>(r, [&](long t) {
                const double* s = r.D + 6 * t;  // d00 d01 d02 d11 d12 d22
                return [s](const std::array<double, 3>&, double* D, TensorDims, void*, int) {
                    double m[9] = {s[0], s[1], s[2], s[1], s[3], s[4], s[2], s[4], s[5]};
                    for (int i = 0; i < 9; ++i) D[i] = m[i];
                    return TENSOR_SYMMETRIC;
                };
            });
            return 0;
        case K_TET_GENERAL:
            run_pairs<OpA, OpB, DfuncTraits<PerTetra, false>>(r, [&](long t) {
                const double* s = r.D + nD * t;
                return [s, nD](const std::array<double, 3>&, double* D, TensorDims, void*, int) {
                    for (size_t i = 0; i < nD; ++i) D[i] = s[i];
                    return TENSOR_GENERAL;
                };
            });
            return 0;
        case K_POINT_FN:
            run_pairs<OpA, OpB, DfuncTraits<PerPoint, false>>(r, [&](long) {
                int fn = r.fn;
                return [fn](const std::array<double, 3>& x, double* D, TensorDims dims, void*, int) {
                    return eval_fn(fn, x, D, dims.first, dims.second);
                };
            });
            return 0;
    }
    return -1;
}

// operator codes: 10*space + op, op: 1 IDEN, 2 GRAD; space: 0 P0, 1 P1, 2 P2, 3 P3, 4 Vec3P1, 5 Vec3P2
#define P0 FemFix<FEM_P0>
#define P1 FemFix<FEM_P1>
#define P2 FemFix<FEM_P2>
#define P3 FemFix<FEM_P3>
#define V1 FemVec<3, FEM_P1>
#define V2 FemVec<3, FEM_P2>
#define CR FemFix<FEM_CR1>
#define BB2 FemFix<FEM_B2>
#define BB4 FemFix<FEM_B4>
#define ND FemFix<FEM_ND0>
#define RT FemFix<FEM_RT0>

// Ani::fem3DapplyL (eval.inl:93-111) for phys == 0: npts shared barycentric points [npts][4];
// Ani::fem3DapplyX (eval.inl:103-125) for phys == 1: per-tet physical points [nt][npts][3].
// dofs[nt][nf]; opU[nt][npts*dim].  One tet per call (fusion 1), at most 24 points.
template <typename Op>
int apply_tets(long nt, const double* XY, int npts, const double* pts, int phys, const double* dofs, double* opU) {
    constexpr int nf = Op::Nfa::value, dim = Op::Dim::value;
    if (npts < 1 || npts > 24) return -3;
    std::vector<double> l(pts, pts + (phys ? 0 : 4 * npts));
    for (long t = 0; t < nt; ++t) {
        const double* X = XY + 12 * t;
        std::vector<double> d(dofs + (size_t)nf * t, dofs + (size_t)nf * (t + 1));
        double* out = opU + (size_t)npts * dim * t;
        if (phys) {
            ArrayView<const double> Xv(pts + (size_t)3 * npts * t, 3 * npts);
            fem3DapplyX<Op>(X, X + 3, X + 6, X + 9, Xv, ArrayView<double>(d.data(), nf),
                            ArrayView<double>(out, (size_t)npts * dim));
        } else {
            DenseMatrix<const double> XY0(X, 3, 1), XY1(X + 3, 3, 1), XY2(X + 6, 3, 1), XY3(X + 9, 3, 1);
            DenseMatrix<> dm(d.data(), nf, 1), om(out, (size_t)npts * dim, 1);
            fem3DapplyL<Op>(XY0, XY1, XY2, XY3, ArrayView<double>(l.data(), 4 * npts), dm, om);
        }
    }
    return 0;
}

}  // namespace

extern "C" {

int ref_fem3dtet(int codeA, int codeB, int kind, int order, long nt, const double* XY, const double* D,
                 int fn, double* A) {
    Req r{kind, order, fn, nt, XY, D, A};
    try {
#define PAIR(ca, cb, OA, OB) if (codeA == (ca) && codeB == (cb)) return run<OA, OB>(r);
        using G1 = Operator<GRAD, P1>; using G2 = Operator<GRAD, P2>; using G3 = Operator<GRAD, P3>;
        using GV1 = Operator<GRAD, V1>; using GV2 = Operator<GRAD, V2>;
        using I0 = Operator<IDEN, P0>; using I1 = Operator<IDEN, P1>; using I2 = Operator<IDEN, P2>;
        using I3 = Operator<IDEN, P3>; using IV2 = Operator<IDEN, V2>;
        PAIR(12, 12, G1, G1)
        PAIR(22, 22, G2, G2)
        PAIR(32, 32, G3, G3)
        PAIR(42, 42, GV1, GV1)
        PAIR(52, 52, GV2, GV2)
        PAIR(32, 42, G3, GV1)
        PAIR(11, 11, I1, I1)
        PAIR(21, 21, I2, I2)
        PAIR(31, 31, I3, I3)
        PAIR(1, 11, I0, I1)
        PAIR(1, 21, I0, I2)
        PAIR(1, 31, I0, I3)
        PAIR(1, 51, I0, IV2)
        PAIR(12, 22, G1, G2)
        PAIR(22, 12, G2, G1)
        PAIR(22, 21, G2, I2)
        PAIR(12, 11, G1, I1)
        using ICR = Operator<IDEN, CR>; using GCR = Operator<GRAD, CR>;
        using IB2 = Operator<IDEN, BB2>; using GB2 = Operator<GRAD, BB2>;
        using IB4 = Operator<IDEN, BB4>; using GB4 = Operator<GRAD, BB4>;
        PAIR(61, 61, ICR, ICR)
        PAIR(62, 62, GCR, GCR)
        PAIR(1, 61, I0, ICR)
        PAIR(71, 71, IB2, IB2)
        PAIR(72, 72, GB2, GB2)
        PAIR(81, 81, IB4, IB4)
        PAIR(82, 82, GB4, GB4)
        PAIR(11, 81, I1, IB4)
        PAIR(81, 11, IB4, I1)
        using IND = Operator<IDEN, ND>; using CND = Operator<CURL, ND>; using GND = Operator<GRAD, ND>;
        using IRT = Operator<IDEN, RT>; using DRT = Operator<DIV, RT>; using GRT = Operator<GRAD, RT>;
        PAIR(91, 91, IND, IND)
        PAIR(94, 94, CND, CND)
        PAIR(92, 92, GND, GND)
        PAIR(101, 101, IRT, IRT)
        PAIR(103, 103, DRT, DRT)
        PAIR(102, 102, GRT, GRT)
        PAIR(103, 1, DRT, I0)
        PAIR(91, 101, IND, IRT)
#undef PAIR
    } catch (const std::exception&) {
        return -2;
    }
    return -1;
}

int ref_fem3d_apply(int code, long nt, const double* XY, int npts, const double* pts, int phys,
                    const double* dofs, double* opU) {
    try {
#define OP(c, OPT) if (code == (c)) return apply_tets<OPT>(nt, XY, npts, pts, phys, dofs, opU);
        using I0 = Operator<IDEN, P0>; using I1 = Operator<IDEN, P1>; using G1 = Operator<GRAD, P1>;
        using I2 = Operator<IDEN, P2>; using G2 = Operator<GRAD, P2>; using I3 = Operator<IDEN, P3>;
        using G3 = Operator<GRAD, P3>; using IV1 = Operator<IDEN, V1>; using GV1 = Operator<GRAD, V1>;
        using IV2 = Operator<IDEN, V2>; using GV2 = Operator<GRAD, V2>;
        OP(1, I0)
        OP(11, I1)
        OP(12, G1)
        OP(21, I2)
        OP(22, G2)
        OP(31, I3)
        OP(32, G3)
        OP(41, IV1)
        OP(42, GV1)
        OP(51, IV2)
        OP(52, GV2)
        using ICR = Operator<IDEN, CR>; using GCR = Operator<GRAD, CR>;
        using IB2 = Operator<IDEN, BB2>; using GB2 = Operator<GRAD, BB2>;
        using IB4 = Operator<IDEN, BB4>; using GB4 = Operator<GRAD, BB4>;
        OP(61, ICR)
        OP(62, GCR)
        OP(71, IB2)
        OP(72, GB2)
        OP(81, IB4)
        OP(82, GB4)
        using IND = Operator<IDEN, ND>; using CND = Operator<CURL, ND>; using GND = Operator<GRAD, ND>;
        using DND = Operator<DIV, ND>;
        using IRT = Operator<IDEN, RT>; using DRT = Operator<DIV, RT>; using GRT = Operator<GRAD, RT>;
        using CRT = Operator<CURL, RT>;
        OP(91, IND)
        OP(92, GND)
        OP(93, DND)
        OP(94, CND)
        OP(101, IRT)
        OP(102, GRT)
        OP(103, DRT)
        OP(104, CRT)
#undef OP
    } catch (const std::exception&) {
        return -2;
    }
    return -1;
}

// Ani::fem3Dface (anifem++/fem/operations/int_face.inl:12-44) for the same operator pairs,
// face `face` of every tet of the batch
int ref_fem3dface(int codeA, int codeB, int kind, int order, int face, long nt, const double* XY, const double* D,
                  int fn, double* A) {
    g_face = face;
    const int rc = ref_fem3dtet(codeA, codeB, kind, order, nt, XY, D, fn, A);
    g_face = -1;
    return rc;
}

// Ani::fem3DfaceN (anifem++/fem/operations/int_face.inl:48-78): tensors of 3*dimB x dimA
int ref_fem3dface_n(int codeA, int codeB, int kind, int order, int face, long nt, const double* XY,
                    const double* D, int fn, double* A) {
    g_normal = 1;
    const int rc = ref_fem3dface(codeA, codeB, kind, order, face, nt, XY, D, fn, A);
    g_normal = 0;
    return rc;
}

int ref_quadrature(int order, double* p, double* w, int cap) {
    auto f = tetrahedron_quadrature_formulas(order);
    int np = f.GetNumPoints();
    if (np > cap) return -np;
    for (int i = 0; i < np; ++i) {
        auto pw = f.GetPointWeight<double>(i);
        for (int k = 0; k < 4; ++k) p[4 * i + k] = f.p[4 * i + k];
        w[i] = pw.w;
    }
    return np;
}

// Ani::triangle_quadrature_formulas (anifem++/fem/quadrature_formulas.cpp:109): points as 3
// barycentric coordinates, weights; returns the number of points (-np when cap is short);
// sym receives the orbit counts (#s1, #s3, #s6)
int ref_tri_quadrature(int order, double* p, double* w, int cap, int* sym) {
    auto f = triangle_quadrature_formulas(order);
    int np = f.GetNumPoints();
    if (np > cap) return -np;
    for (int i = 0; i < np; ++i) {
        for (int k = 0; k < 3; ++k) p[3 * i + k] = f.p[3 * i + k];
        w[i] = f.w[i];
    }
    for (int k = 0; k < 3; ++k) sym[k] = f.sym[k];
    return np;
}

void ref_applyDir(double* A, double* F, int n, int k, double bc) {
    DenseMatrix<> Am(A, n, n), Fm(F, n, 1);
    applyDir(Am, Fm, k, bc);
}

// CPU baseline: P2 GRAD.GRAD with a per-tet symmetric tensor (TENSOR_SYMMETRIC traits),
// one fem3Dtet call per tet, split into contiguous chunks over nthreads std::threads
// like ThreadPar STD (anifem++/fem/mutex_type.h:106-128).  Returns elapsed seconds.
double ref_time_p2_sym(long nt, const double* XY, const double* D6, int order, int nthreads, double* A) {
    Req r{K_TET_SYM, order, 0, nt, XY, D6, A};
    auto t0 = std::chrono::steady_clock::now();
    if (nthreads <= 1) {
        run<Operator<GRAD, P2>, Operator<GRAD, P2>>(r);
    } else {
        std::vector<std::thread> th;
        long chunk = (nt + nthreads - 1) / nthreads;
        for (int i = 0; i < nthreads; ++i) {
            long b = i * chunk, e = std::min(nt, b + chunk);
            if (b >= e) break;
            th.emplace_back([&, b, e]() {
                Req q = r;
                q.nt = e - b;
                q.XY = XY + 12 * b;
                q.D = D6 + 6 * b;
                q.A = A + 100 * b;
                run<Operator<GRAD, P2>, Operator<GRAD, P2>>(q);
            });
        }
        for (auto& t : th) t.join();
    }
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // extern "C"
