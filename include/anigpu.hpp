/* C++ runtime-space layer over the anigpu C ABI (header only).
 *
 * Mirrors the reference's runtime operator / space interface, so that code written against
 *   Ani::ApplyOp / Ani::ApplyOpBase   (anifem++/fem/operators.h:418-450)
 *   Ani::FemSpace::getOP(OperatorType) (anifem++/fem/fem_space.h:404-589)
 *   Ani::fem3Dtet / fem3Dface / fem3DfaceN / fem3DapplyL / fem3DapplyX with runtime operators
 *     (anifem++/fem/operations/int_tet.h:111-147, int_face.h, eval.h:80-87)
 * finds the same names: an ApplyOp is an operator code (10*space + op) with Nfa(), Dim() and
 * Order(); a FemSpace hands out its operators; the integrals run the library's batched kernels on
 * device arrays.  Errors come back as std::runtime_error, as the reference throws them.
 *
 * Spaces: P0, P1, P2, P3, CR1, B2, B4, ND0, RT0 and FemVec<3, P1 | P2> (component-major DOF
 * blocks, the reference's FemVec order).  Operators: IDEN, GRAD; DIV and CURL for ND0 / RT0;
 * user-defined operators (ApplyOpCustom) whose values the caller's device code supplies. */
#ifndef ANIGPU_HPP
#define ANIGPU_HPP

#include <climits>
#include <cstdint>
#include <functional>
#include <stdexcept>
#include <string>

#include "anigpu.h"

namespace anigpu {

enum OperatorType { IDEN = ANIGPU_IDEN, GRAD = ANIGPU_GRAD, DIV = ANIGPU_DIV, CURL = ANIGPU_CURL };

inline void check(anigpu_handle h, int rc) {
    if (rc != ANIGPU_OK) {
        const char* msg = h ? anigpu_last_error(h) : "";
        throw std::runtime_error("anigpu error " + std::to_string(rc) + ": " + (msg ? msg : ""));
    }
}

/* An operator applied to a space: Operator<OP, FEM> as a runtime value. */
class ApplyOp {
public:
    ApplyOp() = default;
    explicit ApplyOp(int code) : code_(code) {
        const int space = code / 10, op = code % 10;
        const bool vec = space == ANIGPU_ND0 || space == ANIGPU_RT0;
        const bool ok = vec ? (op >= ANIGPU_IDEN && op <= ANIGPU_CURL)
                            : ((op == ANIGPU_IDEN || op == ANIGPU_GRAD) && space >= ANIGPU_P0 && space <= ANIGPU_B4);
        if (!ok) throw std::invalid_argument("unknown operator code " + std::to_string(code));
    }
    int code() const { return code_; }
    int space() const { return code_ / 10; }
    OperatorType type() const { return static_cast<OperatorType>(code_ % 10); }
    unsigned ncomp() const { return space() == ANIGPU_VEC3_P1 || space() == ANIGPU_VEC3_P2 ? 3u : 1u; }
    unsigned base_space() const { return ncomp() == 3 ? (unsigned)space() - 3u : (unsigned)space(); }
    /* local DOFs of the operator's space (Operator::Nfa) */
    bool vector_valued() const { return space() == ANIGPU_ND0 || space() == ANIGPU_RT0; }
    unsigned Nfa() const {
        static const unsigned nfs[11] = {1, 4, 10, 20, 0, 0, 4, 6, 1, 6, 4};
        return nfs[base_space()] * ncomp();
    }
    /* rows of the operator's value at a point (Operator::Dim) */
    unsigned Dim() const {
        if (vector_valued()) {
            static const unsigned dims[5] = {0, 3, 9, 1, 3};
            return dims[type()];
        }
        return (type() == IDEN ? 1u : 3u) * ncomp();
    }
    /* polynomial order of the operator's value */
    unsigned Order() const {
        static const unsigned deg[11] = {0, 1, 2, 3, 1, 2, 1, 2, 4, 1, 1};
        const unsigned p = deg[space()];
        return type() == IDEN ? p : (p > 0 ? p - 1 : 0);
    }
    bool operator==(const ApplyOp& o) const { return code_ == o.code_; }
    bool operator!=(const ApplyOp& o) const { return code_ != o.code_; }

private:
    int code_ = 10 * ANIGPU_P1 + ANIGPU_IDEN;
};

/* A finite element space as a runtime value (Ani::FemSpace). */
class FemSpace {
public:
    FemSpace() = default;
    static FemSpace P0() { return FemSpace(ANIGPU_P0); }
    static FemSpace P1() { return FemSpace(ANIGPU_P1); }
    static FemSpace P2() { return FemSpace(ANIGPU_P2); }
    static FemSpace P3() { return FemSpace(ANIGPU_P3); }
    static FemSpace CR1() { return FemSpace(ANIGPU_CR1); }
    static FemSpace B2() { return FemSpace(ANIGPU_B2); }
    static FemSpace B4() { return FemSpace(ANIGPU_B4); }
    static FemSpace ND0() { return FemSpace(ANIGPU_ND0); }
    static FemSpace RT0() { return FemSpace(ANIGPU_RT0); }
    /* FemVec<3, base> for base P1 or P2 */
    static FemSpace Vec3(const FemSpace& base) {
        if (base.space_ == ANIGPU_P1) return FemSpace(ANIGPU_VEC3_P1);
        if (base.space_ == ANIGPU_P2) return FemSpace(ANIGPU_VEC3_P2);
        throw std::invalid_argument("FemVec<3, .> of P1 or P2 only");
    }
    int space() const { return space_; }
    ApplyOp getOP(OperatorType op) const { return ApplyOp(10 * space_ + op); }
    /* local DOFs per tet (dofMap().NumDofsOnTet()) */
    unsigned NumDofsOnTet() const { return getOP(IDEN).Nfa(); }
    std::string typeName() const {
        static const char* names[11] = {"P0", "P1", "P2", "P3", "P1^3", "P2^3", "CR1", "B2", "B4", "ND0", "RT0"};
        return names[space_];
    }
    bool operator==(const FemSpace& o) const { return space_ == o.space_; }

private:
    explicit FemSpace(int s) : space_(s) {}
    int space_ = ANIGPU_P1;
};

/* A = int over each tet of (D OpA(u)) . OpB(v): nt element matrices, column-major nfB x nfA per
 * tet (device arrays; XY: nt x 4 vertices x 3 coordinates). */
inline void fem3Dtet(anigpu_handle h, int64_t nt, const double* XY, const ApplyOp& opA, const ApplyOp& opB,
                     int tensor_kind, const double* D, void* A, int order = 5, int precision = ANIGPU_F64) {
    check(h, anigpu_fem3dtet(h, opA.code(), opB.code(), tensor_kind, order, precision, nt, XY, D, A));
}

/* the same over face `face` of every tet (fem3Dface) or with the outward normal (fem3DfaceN) */
inline void fem3Dface(anigpu_handle h, int64_t nt, const double* XY, int face, const ApplyOp& opA,
                      const ApplyOp& opB, int tensor_kind, const double* D, void* A, int order = 5,
                      int precision = ANIGPU_F64) {
    check(h, anigpu_fem3dface(h, opA.code(), opB.code(), tensor_kind, order, precision, nt, XY, face, D, A));
}
inline void fem3DfaceN(anigpu_handle h, int64_t nt, const double* XY, int face, const ApplyOp& opA,
                       const ApplyOp& opB, int tensor_kind, const double* D, void* A, int order = 5,
                       int precision = ANIGPU_F64) {
    check(h, anigpu_fem3dface_n(h, opA.code(), opB.code(), tensor_kind, order, precision, nt, XY, face, D, A));
}

/* Op(u) at shared barycentric points XYL[npts][4] (fem3DapplyL) or per-tet physical points
 * X[nt][npts][3] (fem3DapplyX); dofs[nt][Nfa]; opU[nt][npts][Dim] */
inline void fem3DapplyL(anigpu_handle h, int64_t nt, const double* XY, int npts, const double* XYL,
                        const ApplyOp& op, const double* dofs, double* opU) {
    check(h, anigpu_fem3d_apply(h, op.code(), nt, XY, npts, XYL, dofs, opU));
}
inline void fem3DapplyX(anigpu_handle h, int64_t nt, const double* XY, int npts, const double* X, const ApplyOp& op,
                        const double* dofs, double* opU) {
    check(h, anigpu_fem3d_apply_x(h, op.code(), nt, XY, npts, X, dofs, opU));
}

/* A user-defined operator (Ani::ApplyOpCustom, anifem++/fem/operators.h:450-471): a unique label
 * (operators with equal labels are the same operator), Dim, Nfa, Order and a functor that writes
 * the operator's values at the points of the quadrature rule of `order` for a batch of tets on the
 * device: U[((t*q + n)*Nfa + i)*Dim + k], q = the rule's points (anigpu_quadrature).  The functor
 * replaces the reference's applyOp(mem, U); it runs the caller's own device code. */
class ApplyOpCustom {
public:
    using Fill = std::function<void(anigpu_handle h, int64_t nt, const double* XY, int order, double* U)>;
    ApplyOpCustom(unsigned unique_label, Fill fill, unsigned dim, unsigned nfa, unsigned order = UINT_MAX)
        : fill_(std::move(fill)), dim_(dim), nfa_(nfa), order_(order), label_(unique_label) {
        if (dim < 1 || dim > 9 || nfa < 1) throw std::invalid_argument("custom operator: 1 <= Dim <= 9, Nfa >= 1");
    }
    unsigned Nfa() const { return nfa_; }
    unsigned Dim() const { return dim_; }
    unsigned Order() const { return order_; }
    unsigned label() const { return label_; }
    bool operator==(const ApplyOpCustom& o) const { return label_ == o.label_; }
    bool operator!=(const ApplyOpCustom& o) const { return label_ != o.label_; }
    void fill(anigpu_handle h, int64_t nt, const double* XY, int order, double* U) const { fill_(h, nt, XY, order, U); }
    /* doubles of the device buffer that holds the operator's values for nt tets */
    size_t values_size(int64_t nt, int order) const {
        const int q = anigpu_quadrature(order, nullptr, nullptr, 1 << 20);
        if (q <= 0) throw std::invalid_argument("no quadrature rule of order " + std::to_string(order));
        return (size_t)nt * (size_t)q * nfa_ * dim_;
    }

private:
    Fill fill_;
    unsigned dim_, nfa_, order_, label_;
};

/* fem3Dtet with user-defined operators: fills UA (and VB when opB is another operator) through the
 * operators' functors, then integrates; UA / VB hold values_size(nt, order) doubles each */
inline void fem3Dtet(anigpu_handle h, int64_t nt, const double* XY, const ApplyOpCustom& opA,
                     const ApplyOpCustom& opB, int tensor_kind, const double* D, void* A, double* UA, double* VB,
                     int order = 5, int precision = ANIGPU_F64) {
    opA.fill(h, nt, XY, order, UA);
    const bool same = opA == opB;
    if (!same) {
        if (!VB) throw std::invalid_argument("a second operator needs its own value buffer");
        opB.fill(h, nt, XY, order, VB);
    }
    check(h, anigpu_fem3dtet_custom(h, (int)opA.Dim(), (int)opA.Nfa(), UA, (int)opB.Dim(), (int)opB.Nfa(),
                                    same ? nullptr : VB, tensor_kind, order, precision, nt, XY, D, A));
}

/* owning handle */
class Context {
public:
    explicit Context(int device = 0) { check(nullptr, anigpu_create(&h_, device)); }
    ~Context() {
        if (h_) anigpu_destroy(h_);
    }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    anigpu_handle get() const { return h_; }

private:
    anigpu_handle h_ = nullptr;
};

}  // namespace anigpu

#endif
