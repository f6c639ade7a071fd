/* Drop-in template interface of AniFem++'s element level and local-assembler contract, over the
 * anigpu C ABI (header only; link libanigpu and cudart).
 *
 * Code written against the reference's
 *   Ani::fem3Dtet<Operator<OpA, Space>, Operator<OpB, Space>, DfuncTraits<...>, FUSION>(XYZ, Dfnc, A,
 *       order, user_data)                              (anifem++/fem/operations/int_tet.h:16-77)
 *   Ani::fem3Dface / fem3DfaceN<OpA, OpB, Traits>      (anifem++/fem/operations/int_face.h:15-48)
 *   DfuncTraits / DfuncTraitsFusive, TensorType        (anifem++/fem/diff_tensor.h:17-53)
 *   DenseMatrix, ArrayView, Tetra / make_tetras        (anifem++/fem/fem_memory.h:26-90, geometry.h:96-200)
 *   applyDir                                           (anifem++/fem/operations/dc_on_dof.h:24-45)
 *   GenerateElemMatRhs + Assembler::SetMatRHSFunc / PrepareProblem / Assemble
 *                                                      (anifem++/inmost_interface/func_wrap.h:311-317,
 *                                                       assembler.h:316-386)
 * compiles unchanged against this header: the same names, template parameters, argument order,
 * layouts (column-major element matrices A(i_test, j_trial), the tensor functor's column-major
 * D with Ddims = {dim OpB, dim OpA}) and errors (std::runtime_error for the reference's throws).
 *
 * Where the work runs.  Every element integral is computed by the library's CUDA kernels
 * (anigpu_fem3dtet / anigpu_fem3dface / anigpu_fem3dface_n); the coefficient functor is the
 * caller's host code and is evaluated on the host, at the physical quadrature points
 * (internalFem3DtetGeomInit_XYG, core.inl:249-269) with the reference's call pattern per traits
 * (diff_tensor.h:279-994: one call for constant tensors, per point otherwise, the PerTetra /
 * PerSelection type probes, one batched call for fusive tensors); its values travel to the device
 * as per-tet or per-point tensor data.
 *   - A plain call of fem3Dtet is one GPU batch of the call's FUSION tets (synchronous).
 *   - Assembler::Assemble runs the caller's local assembler twice per element: a recording pass in
 *     which every fem3Dtet / fem3Dface call records its request (operators, order, coordinates,
 *     functor values) and returns zeros, one batched GPU launch per distinct request signature over
 *     a chunk of elements, then a replay pass in which each call returns its computed matrix, so
 *     that the local assembler's own host code (sums, applyDir, ...) runs on the real values.  The
 *     element matrices and right-hand sides are then scattered on the GPU by
 *     anigpu_assemble_elements.  The local assembler must issue the same calls in the same order
 *     on both passes (a std::runtime_error reports a mismatch).
 *
 * Spaces: P0, P1, P2, P3, CR1, B2, B4, ND0, RT0 (FemFix) and FemVec<3, P1 | P2>; operators IDEN,
 * GRAD (and DIV, CURL of ND0 / RT0).  Quadrature orders 0-6 for the memoryless overloads (the
 * reference's limit, int_tet.inl:98-99), 0-20 with PlainMemory; triangle orders 0-9 / 0-20. */
#ifndef ANIGPU_FEM_HPP
#define ANIGPU_FEM_HPP

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cassert>
#include <cstdint>
#include <cstring>
#include <functional>
#include <limits>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#include "anigpu.h"

namespace Ani {

// ------------------------------------------------------------------ spaces and operators
enum FiniteElement { FEM_P0 = 1, FEM_P1 = 2, FEM_P2 = 3, FEM_P3 = 4, FEM_RT0 = 21, FEM_ND0 = 25, FEM_CR1 = 31,
                     FEM_B2 = 1002, FEM_B4 = 1004 };
enum OperatorType { IDEN = 1, GRAD = 2, DIV = 3, CURL = 4, DUDX = 6, DUDY = 7, DUDZ = 8 };

template <int OP>
using FemFix = std::integral_constant<int, OP>;

template <int DIM, int OP>
struct FemVec {
    using Dim = std::integral_constant<int, DIM>;
    using Base = FemFix<OP>;
};

namespace gpu_detail {
constexpr int space_of(int fem) {
    return fem == FEM_P0 ? ANIGPU_P0 : fem == FEM_P1 ? ANIGPU_P1 : fem == FEM_P2 ? ANIGPU_P2 : fem == FEM_P3 ? ANIGPU_P3
         : fem == FEM_CR1 ? ANIGPU_CR1 : fem == FEM_B2 ? ANIGPU_B2 : fem == FEM_B4 ? ANIGPU_B4
         : fem == FEM_ND0 ? ANIGPU_ND0 : fem == FEM_RT0 ? ANIGPU_RT0 : -1;
}
constexpr int nf_of(int space) {
    return space == ANIGPU_P0 ? 1 : space == ANIGPU_P1 ? 4 : space == ANIGPU_P2 ? 10 : space == ANIGPU_P3 ? 20
         : space == ANIGPU_CR1 ? 4 : space == ANIGPU_B2 ? 6 : space == ANIGPU_B4 ? 1 : space == ANIGPU_ND0 ? 6
         : space == ANIGPU_RT0 ? 4 : 0;
}
constexpr bool vector_space(int space) { return space == ANIGPU_ND0 || space == ANIGPU_RT0; }
constexpr int dim_of(int space, int op) {
    return vector_space(space) ? (op == IDEN ? 3 : op == GRAD ? 9 : op == DIV ? 1 : op == CURL ? 3 : 0)
                               : (op == IDEN ? 1 : op == GRAD ? 3 : 0);
}
constexpr int degree_of(int space) {
    return space == ANIGPU_P0 ? 0 : space == ANIGPU_P1 ? 1 : space == ANIGPU_P2 ? 2 : space == ANIGPU_P3 ? 3
         : space == ANIGPU_CR1 ? 1 : space == ANIGPU_B2 ? 2 : space == ANIGPU_B4 ? 4 : 1;
}
}  // namespace gpu_detail

template <int OPERATOR, typename FEMTYPE>
struct Operator;

/* Operator<OP, FemFix<FEM>>: Nfa, Dim, Order as the reference's specialisations (the spaces/ headers);
 * `code` is the library's operator code (10 * space + operator) */
template <int OPERATOR, int FEM>
struct Operator<OPERATOR, FemFix<FEM>> {
    static constexpr int space = gpu_detail::space_of(FEM);
    static_assert(space >= 0, "finite element type not provided by the GPU library");
    static_assert(gpu_detail::dim_of(space, OPERATOR) > 0,
                  "operator not provided by the GPU library for this space (IDEN, GRAD; DIV, CURL of ND0/RT0)");
    static constexpr int code = 10 * space + OPERATOR;
    using Nfa = std::integral_constant<int, gpu_detail::nf_of(space)>;
    using Dim = std::integral_constant<int, gpu_detail::dim_of(space, OPERATOR)>;
    using Order = std::integral_constant<int, OPERATOR == IDEN ? gpu_detail::degree_of(space)
                                                               : (gpu_detail::degree_of(space) > 0 ? gpu_detail::degree_of(space) - 1 : 0)>;
};

/* Operator<OP, FemVec<3, P1 | P2>>: component-major DOF blocks (operators.h:127-155) */
template <int OPERATOR, int DIM, int FEM>
struct Operator<OPERATOR, FemVec<DIM, FEM>> {
    static_assert(DIM == 3 && (FEM == FEM_P1 || FEM == FEM_P2) && (OPERATOR == IDEN || OPERATOR == GRAD),
                  "the GPU library provides FemVec<3, FEM_P1 | FEM_P2> with IDEN and GRAD");
    static constexpr int space = FEM == FEM_P1 ? ANIGPU_VEC3_P1 : ANIGPU_VEC3_P2;
    static constexpr int code = 10 * space + OPERATOR;
    using Nfa = std::integral_constant<int, 3 * gpu_detail::nf_of(FEM == FEM_P1 ? ANIGPU_P1 : ANIGPU_P2)>;
    using Dim = std::integral_constant<int, 3 * (OPERATOR == IDEN ? 1 : 3)>;
    using Order = std::integral_constant<int, OPERATOR == IDEN ? (FEM == FEM_P1 ? 1 : 2) : (FEM == FEM_P1 ? 0 : 1)>;
};

// ------------------------------------------------------------------ tensor traits (diff_tensor.h:17-53)
enum TensorType { TENSOR_NULL = 1, TENSOR_SCALAR = 2, TENSOR_SYMMETRIC = 3, TENSOR_GENERAL = 4 };
enum TensorTypeSparsity { PerPoint = 0, PerTetra = -1, PerSelection = -2 };
enum TensorTypeAggregate { OnePointTensor = 0, FusiveTensor = 1 };

template <int TensorTypeSparse = PerPoint, bool isConstant = false, long idim = -1, long jdim = -1,
          int aggregateType = OnePointTensor>
struct DfuncTraitsCommon {
    using AggregateType = std::integral_constant<int, aggregateType>;
    using IsConstant = std::integral_constant<bool, isConstant>;
    using TensorSparsity = std::integral_constant<int, TensorTypeSparse>;
    using iD = std::integral_constant<long, idim>;
    using jD = std::integral_constant<long, jdim>;
};
template <int TensorTypeSparse = PerPoint, bool isConstant = false, long idim = -1, long jdim = -1>
using DfuncTraits = DfuncTraitsCommon<TensorTypeSparse, isConstant, idim, jdim>;
template <long idim = -1, long jdim = -1>
using DfuncTraitsFusive = DfuncTraitsCommon<PerSelection, false, idim, jdim, FusiveTensor>;

template <typename Scalar = double>
using Coord = std::array<Scalar, 3>;
using TensorDims = std::pair<std::size_t, std::size_t>;

// ------------------------------------------------------------------ memory views (fem_memory.h)
template <typename ScalarType = double>
struct ArrayView {
    using Scalar = ScalarType;
    Scalar* data = nullptr;
    std::size_t size = 0;
    ArrayView() = default;
    ArrayView(Scalar* data, std::size_t size) : data{data}, size{size} {}
    void Init(Scalar* d, std::size_t s) { data = d, size = s; }
    void SetZero() { std::fill(data, data + size, Scalar(0)); }
    Scalar& operator[](std::size_t i) { return data[i]; }
    Scalar operator[](std::size_t i) const { return data[i]; }
    bool empty() const { return size == 0 || data == nullptr; }
};

/* column-major dense matrix view: A(i, j) = data[i + nRow * j] */
template <typename ScalarType = double>
struct DenseMatrix {
    using Scalar = ScalarType;
    Scalar* data = nullptr;
    std::size_t nRow = 0, nCol = 0;
    std::size_t size = 0;
    DenseMatrix() = default;
    DenseMatrix(Scalar* data, std::size_t nRow, std::size_t nCol) : data{data}, nRow{nRow}, nCol{nCol}, size{nRow * nCol} {}
    DenseMatrix(Scalar* data, std::size_t nRow, std::size_t nCol, std::size_t size)
        : data{data}, nRow{nRow}, nCol{nCol}, size{size} {}
    void Init(Scalar* d, std::size_t r, std::size_t c, std::size_t s) { data = d, nRow = r, nCol = c, size = s; }
    Scalar& operator()(std::size_t i, std::size_t j) { return data[i + nRow * j]; }
    Scalar operator()(std::size_t i, std::size_t j) const { return data[i + nRow * j]; }
    Scalar& operator[](std::size_t i) { return data[i]; }
    Scalar operator[](std::size_t i) const { return data[i]; }
    template <typename RT>
    DenseMatrix& operator+=(const DenseMatrix<RT>& o) {
        for (std::size_t i = 0; i < nRow * nCol; ++i) data[i] += o.data[i];
        return *this;
    }
    template <typename RT>
    DenseMatrix& operator-=(const DenseMatrix<RT>& o) {
        for (std::size_t i = 0; i < nRow * nCol; ++i) data[i] -= o.data[i];
        return *this;
    }
    template <typename RT>
    DenseMatrix& operator*=(RT v) {
        for (std::size_t i = 0; i < nRow * nCol; ++i) data[i] *= v;
        return *this;
    }
    void SetZero() { std::fill(data, data + nRow * nCol, Scalar(0)); }
};

/* coordinates of a fused batch of tets: four 3 x f column-major matrices (geometry.h:96-200) */
template <typename ScalarType = const double>
struct Tetras {
    DenseMatrix<ScalarType> XY0, XY1, XY2, XY3;
    int fusion = 0;
    Tetras() = default;
    Tetras(ScalarType* a, ScalarType* b, ScalarType* c, ScalarType* d, int count = 1)
        : XY0(a, 3, count), XY1(b, 3, count), XY2(c, 3, count), XY3(d, 3, count), fusion(count) {}
    Tetras(const DenseMatrix<ScalarType>& a, const DenseMatrix<ScalarType>& b, const DenseMatrix<ScalarType>& c,
           const DenseMatrix<ScalarType>& d)
        : XY0(a), XY1(b), XY2(c), XY3(d), fusion((int)a.nCol) {}
};
template <typename ScalarType = const double>
struct Tetra : public Tetras<ScalarType> {
    Tetra(ScalarType* a, ScalarType* b, ScalarType* c, ScalarType* d) : Tetras<ScalarType>(a, b, c, d, 1) {}
    Tetra() : Tetras<ScalarType>(nullptr, nullptr, nullptr, nullptr, 0) {}
};
template <typename ScalarType>
Tetras<const ScalarType> make_tetras(const ScalarType* a, const ScalarType* b, const ScalarType* c, const ScalarType* d,
                                     int count = 1) {
    return {a, b, c, d, count};
}
template <typename ScalarType>
Tetras<ScalarType> make_tetras(ScalarType* a, ScalarType* b, ScalarType* c, ScalarType* d, int count = 1) {
    return {a, b, c, d, count};
}

/* what a fusive tensor functor sees of the element engine's memory (fem_memory.h:196-212):
 * q, f, the quadrature rule (XYL, WG), the physical points (XYG) and the coordinates relative to
 * the first node (XYP); the engine's other work arrays live on the device and are left empty */
template <typename ScalarType = double, typename IndexType = int>
struct AniMemory {
    using Scalar = ScalarType;
    ArrayView<Scalar> XYP, PSI, XYG, DET, MES, NRM, U, V, DIFF, DU, XYL, WG, extraR;
    ArrayView<IndexType> extraI;
    std::size_t q = 0, f = 1;
};

/* caller-provided host memory of the PlainMemory overloads (fem_memory.h:266-300).  The GPU
 * engine needs none: the requirement is one scalar, kept so that callers' allocation code runs. */
template <typename ScalarType = double, typename IndexType = int>
struct PlainMemory {
    ScalarType* ddata = nullptr;
    IndexType* idata = nullptr;
    std::size_t dSize = 0, iSize = 0;
    void* allocateFromRaw(void* mem_in, std::size_t mem_sz) {
        void* p = mem_in;
        std::size_t remain = mem_sz;
        if (dSize > 0) {
            ddata = static_cast<ScalarType*>(std::align(alignof(ScalarType), sizeof(ScalarType) * dSize, p, remain));
            if (!ddata) return nullptr;
            p = ddata + dSize;
            remain = mem_sz - (static_cast<char*>(p) - static_cast<char*>(mem_in));
        }
        if (iSize > 0) {
            idata = static_cast<IndexType*>(std::align(alignof(IndexType), sizeof(IndexType) * iSize, p, remain));
            if (!idata) return nullptr;
            p = idata + iSize;
        }
        return p;
    }
    std::size_t enoughRawSize() const {
        return sizeof(ScalarType) * dSize + sizeof(IndexType) * iSize + alignof(ScalarType) + alignof(IndexType);
    }
};
template <typename OpA, typename OpB, typename ScalarType = double, typename IndexType = int>
PlainMemory<ScalarType, IndexType> fem3Dtet_memory_requirements(int order, int fusion = 1) {
    (void)order, (void)fusion;
    PlainMemory<ScalarType, IndexType> m;
    m.dSize = 1;
    return m;
}
template <typename OpA, typename OpB, typename ScalarType = double, typename IndexType = int>
PlainMemory<ScalarType, IndexType> fem3Dface_memory_requirements(int order, int fusion = 1) {
    return fem3Dtet_memory_requirements<OpA, OpB, ScalarType, IndexType>(order, fusion);
}
template <typename OpA, typename OpB, typename ScalarType = double, typename IndexType = int>
PlainMemory<ScalarType, IndexType> fem3DfaceN_memory_requirements(int order, int fusion = 1) {
    return fem3Dtet_memory_requirements<OpA, OpB, ScalarType, IndexType>(order, fusion);
}

// ------------------------------------------------------------------ tensor helpers (diff_tensor.h:215-260)
template <typename Scalar = double>
TensorType TensorNull(const Coord<Scalar>& X, Scalar* D, TensorDims Ddims, void* user_data, int iTet) {
    (void)X, (void)D, (void)Ddims, (void)user_data, (void)iTet;
    return TENSOR_NULL;
}
template <typename Scalar = double>
auto makeConstantTensorScalar(double val) {
    return [val](const Coord<Scalar>& X, Scalar* D, TensorDims Ddims, void* user_data, int iTet) {
        (void)X, (void)Ddims, (void)user_data, (void)iTet;
        D[0] = val;
        return TENSOR_SCALAR;
    };
}

// ------------------------------------------------------------------ element-level Dirichlet (dc_on_dof.h:24-45)
template <typename Scalar>
inline void applyDirMatrix(DenseMatrix<Scalar>& A, int k) {
    std::fill(A.data + k * A.nRow, A.data + (k + 1) * A.nRow, Scalar(0));
    for (std::size_t i = 0; i < A.nCol; ++i) A(k, i) = 0;
    A(k, k) = 1.0;
}
template <typename Scalar>
inline void applyDir(DenseMatrix<Scalar>& A, DenseMatrix<Scalar>& F, int k, Scalar bc) {
    for (std::size_t i = 0; i < A.nRow; ++i) F(i, 0) -= A(i, k) * bc;
    F(k, 0) = bc;
    applyDirMatrix<Scalar>(A, k);
}
template <typename Scalar>
inline void applyDirResidual(DenseMatrix<Scalar>& F, int k) {
    F(k, 0) = 0.0;
}

// ------------------------------------------------------------------ the GPU session
namespace gpu {
/* Eager: each fem3Dtet call is one GPU batch.  Record / Replay: the two passes of
 * Assembler::Assemble (see the file comment). */
enum class Mode { Eager, Record, Replay };
}  // namespace gpu

namespace gpu_detail {

inline void check_rc(anigpu_handle h, int rc, const char* what) {
    if (rc != ANIGPU_OK) {
        const char* msg = h ? anigpu_last_error(h) : "";
        throw std::runtime_error(std::string(what) + ": " + (msg && *msg ? msg : ("anigpu error " + std::to_string(rc))));
    }
}
inline void check_cuda(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}
inline cudaStream_t handle_stream(anigpu_handle h) {
    void* s = nullptr;
    check_rc(h, anigpu_get_stream(h, &s), "anigpu_get_stream");
    return static_cast<cudaStream_t>(s);
}
/* host <-> device copies ordered on the handle's stream, then waited for */
inline void copy_on(anigpu_handle h, void* dst, const void* src, std::size_t bytes, cudaMemcpyKind kind) {
    cudaStream_t st = handle_stream(h);
    check_cuda(cudaMemcpyAsync(dst, src, bytes, kind, st), "cudaMemcpyAsync");
    check_cuda(cudaStreamSynchronize(st), "cudaStreamSynchronize");
}

/* one element-integral request: a batch of f tets with one operator pair, rule and face */
struct Request {
    int codeA, codeB, order, face, normal;  // face -1: the tet integral
    int kind;                               // ANIGPU_TENSOR_* of the tensor data
    int nfA, nfB, dA, dBt;                  // dBt: tensor rows (3 dB with the normal)
    int f;
    std::size_t xy_off, d_off, d_len, a_off;
};

/* device buffers that only grow */
struct DevBuf {
    void* p = nullptr;
    std::size_t cap = 0;
    void* get(std::size_t bytes) {
        if (bytes > cap) {
            if (p) cudaFree(p);
            p = nullptr;
            cap = 0;
            check_cuda(cudaMalloc(&p, std::max<std::size_t>(bytes, 256)), "cudaMalloc");
            cap = std::max<std::size_t>(bytes, 256);
        }
        return p;
    }
    ~DevBuf() {
        if (p) cudaFree(p);
    }
};

class Session {
public:
    static Session& get() {
        thread_local Session s;
        return s;
    }
    ~Session() {
        if (own_ && h_) anigpu_destroy(h_);
    }
    anigpu_handle handle() {
        if (!h_) {
            check_rc(nullptr, anigpu_create(&h_, device_), "anigpu_create");
            own_ = true;
        }
        return h_;
    }
    void set_device(int device) {
        if (own_ && h_) anigpu_destroy(h_);
        h_ = nullptr;
        own_ = false;
        device_ = device;
    }
    /* run this thread's element integrals on another handle (not owned) until restored */
    anigpu_handle swap_handle(anigpu_handle h, bool& owned) {
        anigpu_handle old = h_;
        owned = own_;
        h_ = h;
        own_ = false;
        return old;
    }
    void restore_handle(anigpu_handle h, bool owned) {
        h_ = h;
        own_ = owned;
    }

    gpu::Mode mode = gpu::Mode::Eager;

    /* eager: one request now */
    void run_now(const Request& r, const double* xy, const double* d, double* out) {
        Request rr = r;
        rr.xy_off = rr.d_off = 0;
        launch(rr, xy, d, out, r.f);
    }
    /* record: keep the request and its inputs; results are filled by flush() */
    void record(Request r, const double* xy, const double* d) {
        r.xy_off = xy_.size();
        xy_.insert(xy_.end(), xy, xy + 12 * (std::size_t)r.f);
        r.d_off = d_.size();
        if (r.d_len) d_.insert(d_.end(), d, d + r.d_len);
        r.a_off = nres_;
        nres_ += (std::size_t)r.nfA * r.nfB * r.f;
        reqs_.push_back(r);
    }
    /* every recorded request computed: one GPU launch per signature */
    void flush() {
        results_.assign(nres_, 0.0);
        std::map<std::tuple<int, int, int, int, int, int>, std::vector<std::size_t>> groups;
        for (std::size_t i = 0; i < reqs_.size(); ++i) {
            const Request& r = reqs_[i];
            groups[std::make_tuple(r.codeA, r.codeB, r.order, r.face, r.normal, r.kind)].push_back(i);
        }
        std::vector<double> xy, d, out;
        for (auto& g : groups) {
            const Request& r0 = reqs_[g.second.front()];
            std::size_t nt = 0;
            xy.clear();
            d.clear();
            for (std::size_t i : g.second) {
                const Request& r = reqs_[i];
                xy.insert(xy.end(), xy_.begin() + r.xy_off, xy_.begin() + r.xy_off + 12 * (std::size_t)r.f);
                d.insert(d.end(), d_.begin() + r.d_off, d_.begin() + r.d_off + r.d_len);
                nt += (std::size_t)r.f;
            }
            const std::size_t per = (std::size_t)r0.nfA * r0.nfB;
            out.resize(per * nt);
            Request rr = r0;
            launch(rr, xy.data(), d.data(), out.data(), (int64_t)nt);
            std::size_t pos = 0;
            for (std::size_t i : g.second) {
                const Request& r = reqs_[i];
                std::copy(out.begin() + pos, out.begin() + pos + per * r.f, results_.begin() + r.a_off);
                pos += per * r.f;
            }
        }
        next_ = 0;
    }
    /* replay: the next request's result, checked against what the call asks for now */
    const double* replay(const Request& now, const double* xy) {
        if (next_ >= reqs_.size())
            throw std::runtime_error("fem3Dtet replay: more element integrals than recorded (the local assembler "
                                     "must make the same calls on both passes)");
        const Request& r = reqs_[next_++];
        if (r.codeA != now.codeA || r.codeB != now.codeB || r.order != now.order || r.face != now.face ||
            r.normal != now.normal || r.f != now.f ||
            std::memcmp(xy_.data() + r.xy_off, xy, sizeof(double) * 12 * (std::size_t)r.f) != 0)
            throw std::runtime_error("fem3Dtet replay: the call differs from the recorded one (the local assembler "
                                     "must make the same calls on both passes)");
        return results_.data() + r.a_off;
    }
    void clear_records() {
        reqs_.clear();
        xy_.clear();
        d_.clear();
        results_.clear();
        nres_ = 0;
        next_ = 0;
    }
    std::size_t recorded() const { return reqs_.size(); }
    std::size_t replayed() const { return next_; }

private:
    void launch(const Request& r, const double* xy, const double* d, double* out, int64_t nt) {
        anigpu_handle h = handle();
        const std::size_t nxy = 12 * (std::size_t)nt, nout = (std::size_t)r.nfA * r.nfB * nt;
        std::size_t nd = 0;
        switch (r.kind) {
            case ANIGPU_TENSOR_NULL: nd = 0; break;
            case ANIGPU_TENSOR_TET_SCALAR: nd = nt; break;
            case ANIGPU_TENSOR_TET_SYM: nd = 6 * nt; break;
            case ANIGPU_TENSOR_TET_GENERAL: nd = (std::size_t)r.dA * r.dBt * nt; break;
            default: nd = r.d_len == 0 ? 0 : r.d_len / (std::size_t)r.f * nt; break;
        }
        cudaStream_t st = handle_stream(h);
        double* dxy = static_cast<double*>(bxy_.get(sizeof(double) * nxy));
        double* dd = nd ? static_cast<double*>(bd_.get(sizeof(double) * nd)) : nullptr;
        double* da = static_cast<double*>(ba_.get(sizeof(double) * nout));
        // every copy on the handle's stream: it does not synchronise with the legacy default stream
        check_cuda(cudaMemcpyAsync(dxy, xy, sizeof(double) * nxy, cudaMemcpyHostToDevice, st), "cudaMemcpyAsync");
        if (nd) check_cuda(cudaMemcpyAsync(dd, d, sizeof(double) * nd, cudaMemcpyHostToDevice, st), "cudaMemcpyAsync");
        int rc;
        if (r.face < 0)
            rc = anigpu_fem3dtet(h, r.codeA, r.codeB, r.kind, r.order, ANIGPU_F64, nt, dxy, dd, da);
        else if (r.normal)
            rc = anigpu_fem3dface_n(h, r.codeA, r.codeB, r.kind, r.order, ANIGPU_F64, nt, dxy, r.face, dd, da);
        else
            rc = anigpu_fem3dface(h, r.codeA, r.codeB, r.kind, r.order, ANIGPU_F64, nt, dxy, r.face, dd, da);
        if (rc == ANIGPU_ERR_ARG || rc == ANIGPU_ERR_UNSUPPORTED) check_rc(h, rc, "fem3Dtet");
        check_rc(h, rc, "fem3Dtet (GPU)");
        check_cuda(cudaMemcpyAsync(out, da, sizeof(double) * nout, cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
        check_cuda(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    }

    anigpu_handle h_ = nullptr;
    bool own_ = false;
    int device_ = 0;
    DevBuf bxy_, bd_, ba_;
    std::vector<Request> reqs_;
    std::vector<double> xy_, d_, results_;
    std::size_t nres_ = 0, next_ = 0;
};

/* the quadrature rule's barycentric points: the tet rule, or the triangle rule mapped onto face k
 * (int_face.inl:31-36) */
inline int rule_points(int order, int face, std::vector<double>& lam, std::vector<double>& w) {
    if (face < 0) {
        lam.assign(4 * 1024, 0.0);
        w.assign(1024, 0.0);
        const int n = anigpu_quadrature(order, lam.data(), w.data(), 1024);
        if (n <= 0) throw std::runtime_error("tetrahedron quadrature order " + std::to_string(order) + " is not provided (0..20)");
        lam.resize(4 * (std::size_t)n);
        w.resize(n);
        return n;
    }
    std::vector<double> p3(3 * 1024), w3(1024);
    const int n = anigpu_face_quadrature(order, p3.data(), w3.data(), 1024);
    if (n <= 0) throw std::runtime_error("triangle quadrature order " + std::to_string(order) + " is not provided (0..20)");
    lam.assign(4 * (std::size_t)n, 0.0);
    w.assign(w3.begin(), w3.begin() + n);
    for (int i = 0; i < n; ++i) {
        lam[4 * i + face] = p3[3 * i + 0];
        lam[4 * i + (face + 1) % 4] = p3[3 * i + 1];
        lam[4 * i + (face + 2) % 4] = p3[3 * i + 2];
        lam[4 * i + (face + 3) % 4] = 0.0;
    }
    return n;
}

/* XYG[3 (n + q r)]: the physical points as internalFem3DtetGeomInit_XYG (core.inl:249-269) */
inline void physical_points(const double* xy, int f, int q, const double* lam, double* xyg) {
    for (int r = 0; r < f; ++r) {
        const double* X = xy + 12 * r;
        double P[3][3];
        for (int l = 0; l < 3; ++l)
            for (int k = 0; k < 3; ++k) P[l][k] = X[3 * (l + 1) + k] - X[k];
        for (int n = 0; n < q; ++n)
            for (int k = 0; k < 3; ++k) {
                double s = X[k];
                for (int l = 0; l < 3; ++l) s += lam[l + 1 + 4 * n] * P[l][k];
                xyg[k + 3 * (n + (std::size_t)q * r)] = s;
            }
    }
}

/* the tensor of one point as the engine uses it, column-major jdim x idim (D(k, j) maps component j
 * of OpA(u) to component k of the OpB side), from the functor's return type and output
 * (_internal_DFunc_common_memoryless, diff_tensor.h:62-95, and the applyDU variants): GENERAL as
 * written, SYMMETRIC as the engine reads it (untransposed), SCALAR / NULL as s I, or a column of s
 * for the P0 right-hand side (idim = 1, nfa = 1) */
inline void to_engine(TensorType t, const double* buf, std::size_t jdim, std::size_t idim, int nfa, double* out) {
    if (t == TENSOR_GENERAL) {
        std::copy(buf, buf + jdim * idim, out);
        return;
    }
    if (t == TENSOR_SYMMETRIC) {
        for (std::size_t k = 0; k < jdim; ++k)
            for (std::size_t j = 0; j < idim; ++j) out[k + jdim * j] = buf[j + idim * k];
        return;
    }
    if (jdim != idim && (nfa != 1 || idim != 1))
        throw std::runtime_error("Identity tensor defined only for compatible (with same dimensions) operators A and B");
    const double s = t == TENSOR_SCALAR ? buf[0] : 1.0;
    std::fill(out, out + jdim * idim, 0.0);
    if (jdim == idim)
        for (std::size_t k = 0; k < jdim; ++k) out[k + jdim * k] = s;
    else
        for (std::size_t k = 0; k < jdim; ++k) out[k] = s;
}

/* per-point tensors (q per tet, engine layout) -> the most specific kind of the library:
 * identical points of every tet -> per-tet data (SCALAR / SYM / GENERAL), else POINT */
inline void compress(const std::vector<double>& pts, const std::vector<char>& scalar_like, int f, int q,
                     std::size_t jdim, std::size_t idim, int& kind, std::vector<double>& d) {
    const std::size_t m = jdim * idim;
    bool per_tet = true;
    for (int r = 0; r < f && per_tet; ++r)
        for (int n = 1; n < q && per_tet; ++n)
            per_tet = std::memcmp(&pts[m * ((std::size_t)q * r)], &pts[m * (n + (std::size_t)q * r)], sizeof(double) * m) == 0;
    if (!per_tet) {
        kind = ANIGPU_TENSOR_POINT;
        d = pts;
        return;
    }
    bool all_scalar = true;
    for (char c : scalar_like) all_scalar = all_scalar && c;
    d.clear();
    if (all_scalar) {
        kind = ANIGPU_TENSOR_TET_SCALAR;
        for (int r = 0; r < f; ++r) d.push_back(pts[m * ((std::size_t)q * r)]);
        return;
    }
    bool sym3 = jdim == 3 && idim == 3;
    for (int r = 0; r < f && sym3; ++r) {
        const double* D = &pts[m * ((std::size_t)q * r)];
        sym3 = D[1] == D[3] && D[2] == D[6] && D[5] == D[7];
    }
    if (sym3) {
        kind = ANIGPU_TENSOR_TET_SYM;
        for (int r = 0; r < f; ++r) {
            const double* D = &pts[m * ((std::size_t)q * r)];
            const double s6[6] = {D[0], D[3], D[6], D[4], D[7], D[8]};
            d.insert(d.end(), s6, s6 + 6);
        }
        return;
    }
    kind = ANIGPU_TENSOR_TET_GENERAL;
    for (int r = 0; r < f; ++r) {
        const double* D = &pts[m * ((std::size_t)q * r)];
        d.insert(d.end(), D, D + m);
    }
}

/* the per-point tensors of a batch, in the engine layout, and which are scalar multiples of I */
struct PointTensors {
    std::size_t jdim, idim, m;
    int f, q, nfa;
    std::vector<double> xyg, pts, buf;
    std::vector<char> scalar_like;
    PointTensors(const double* xy, int f_, int q_, const std::vector<double>& lam, std::size_t jd, std::size_t id, int nfa_)
        : jdim(jd), idim(id), m(jd * id), f(f_), q(q_), nfa(nfa_), xyg(3 * (std::size_t)q_ * f_),
          pts(jd * id * (std::size_t)q_ * f_), buf(std::max<std::size_t>(jd * id, 1) + 8, 0.0),
          scalar_like((std::size_t)q_ * f_, 0) {
        physical_points(xy, f, q, lam.data(), xyg.data());
    }
    std::array<double, 3> X(int r, int n) const {
        const double* p = &xyg[3 * (n + (std::size_t)q * r)];
        return std::array<double, 3>{p[0], p[1], p[2]};
    }
    void put(int r, int n, TensorType t) {
        to_engine(t, buf.data(), jdim, idim, nfa, &pts[m * (n + (std::size_t)q * r)]);
        scalar_like[n + (std::size_t)q * r] = (t == TENSOR_SCALAR || t == TENSOR_NULL);
    }
};

/* fusive traits: one call for the whole batch, TensorType(ArrayView X, ArrayView D, TensorDims,
 * void*, const AniMemory&) (diff_tensor.h:900-994); GENERAL blocks as written, SYMMETRIC untransposed,
 * SCALAR from the first entry of each block */
template <typename Traits, typename Functor>
void eval_tensor_batch(std::integral_constant<int, FusiveTensor>, const Functor& Dfnc, const double* xy,
                       const std::vector<double>& lam, const std::vector<double>& w, PointTensors& P, void* user_data) {
    const int f = P.f, q = P.q;
    const std::size_t m = P.m;
    constexpr bool constant = Traits::IsConstant::value;
    std::vector<double> D(m * (std::size_t)q * f + 8, 0.0);
    {
        std::vector<double> XYP(12 * (std::size_t)f), XYL(lam), WG(w);
        for (int r = 0; r < f; ++r)
            for (int l = 0; l < 4; ++l)
                for (int k = 0; k < 3; ++k) XYP[k + 3 * l + 12 * r] = l == 0 ? 0.0 : xy[12 * r + 3 * l + k] - xy[12 * r + k];
        AniMemory<double, int> mem;
        mem.q = q;
        mem.f = f;
        mem.XYG.Init(P.xyg.data(), P.xyg.size());
        mem.XYL.Init(XYL.data(), XYL.size());
        mem.WG.Init(WG.data(), WG.size());
        mem.XYP.Init(XYP.data(), XYP.size());
        mem.DIFF.Init(D.data(), m * (std::size_t)q * f);
        const TensorType t = static_cast<TensorType>(
            Dfnc(ArrayView<double>(P.xyg.data(), P.xyg.size()), ArrayView<double>(D.data(), m * (std::size_t)q * f),
                 TensorDims{P.jdim, P.idim}, user_data, mem));
        for (int r = 0; r < f; ++r)
            for (int n = 0; n < q; ++n) {
                const std::size_t blk = constant ? 0 : m * (n + (std::size_t)q * r);
                std::copy(D.begin() + blk, D.begin() + blk + m, P.buf.begin());
                P.put(r, n, t);
            }
    }
}

/* one-point traits: the reference's call pattern per traits (diff_tensor.h:279-898); returns false
 * when the whole batch is the identity (no tensor data) */
template <typename Traits, typename Functor>
bool eval_tensor_points(std::integral_constant<int, OnePointTensor>, const Functor& Dfnc, PointTensors& P,
                        void* user_data) {
    constexpr int sparsity = Traits::TensorSparsity::value;
    constexpr bool constant = Traits::IsConstant::value;
    const int f = P.f, q = P.q;
    auto call = [&](const std::array<double, 3>& x, int iTet) {
        std::fill(P.buf.begin(), P.buf.end(), 0.0);
        return static_cast<TensorType>(Dfnc(x, P.buf.data(), TensorDims{P.jdim, P.idim}, user_data, iTet));
    };
    if (constant) {  // one call at the origin, iTet 0 (diff_tensor.h:279-300, 409-470)
        const TensorType t = call({0.0, 0.0, 0.0}, 0);
        P.put(0, 0, t);  // (also the identity compatibility check)
        if (t == TENSOR_NULL) return false;
        for (int r = 0; r < f; ++r)
            for (int n = 0; n < q; ++n) P.put(r, n, t);
        return true;
    }
    if (sparsity == PerTetra) {  // type from the first point of each tet (diff_tensor.h:553-656)
        bool any = false;
        for (int r = 0; r < f; ++r) {
            const TensorType t = call(P.X(r, 0), r);
            P.put(r, 0, t);
            if (t != TENSOR_NULL) any = true;
            for (int n = 1; n < q; ++n) {
                if (t != TENSOR_NULL) call(P.X(r, n), r);
                P.put(r, n, t);
            }
        }
        return any;
    }
    if (sparsity == PerSelection) {  // type from the batch's first point (diff_tensor.h:657-775)
        const TensorType t = call(P.X(0, 0), 0);
        P.put(0, 0, t);
        if (t == TENSOR_NULL) return false;
        for (int n = 1; n < q; ++n) {
            call(P.X(0, n), 0);
            P.put(0, n, t);
        }
        for (int r = 1; r < f; ++r)
            for (int n = 0; n < q; ++n) {
                call(P.X(r, n), t == TENSOR_SCALAR ? r : 0);
                P.put(r, n, t);
            }
        return true;
    }
    // PerPoint and fixed non-constant types: one call per point (diff_tensor.h:488-552, 776-861)
    for (int r = 0; r < f; ++r)
        for (int n = 0; n < q; ++n) P.put(r, n, call(P.X(r, n), r));
    return true;
}

template <typename Traits, typename Functor>
void eval_dispatch(std::integral_constant<int, FusiveTensor> tag, const Functor& Dfnc, const double* xy,
                   const std::vector<double>& lam, const std::vector<double>& w, PointTensors& P, void* user_data,
                   bool& any) {
    eval_tensor_batch<Traits>(tag, Dfnc, xy, lam, w, P, user_data);
    any = true;
}
template <typename Traits, typename Functor>
void eval_dispatch(std::integral_constant<int, OnePointTensor> tag, const Functor& Dfnc, const double* xy,
                   const std::vector<double>& lam, const std::vector<double>& w, PointTensors& P, void* user_data,
                   bool& any) {
    (void)xy, (void)lam, (void)w;
    any = eval_tensor_points<Traits>(tag, Dfnc, P, user_data);
}

/* evaluate the caller's functor for a fused batch of f tets with the reference's call pattern for
 * the traits; results as (kind, data) for the library */
template <typename Traits, typename Functor>
void eval_tensor(const Functor& Dfnc, const double* xy, int f, int q, const std::vector<double>& lam,
                 const std::vector<double>& w, std::size_t jdim, std::size_t idim, int nfa, void* user_data, int& kind,
                 std::vector<double>& d) {
    d.clear();
    if (Traits::TensorSparsity::value == TENSOR_NULL) {  // no call (diff_tensor.h:373-407, 862-898)
        if (jdim != idim && (nfa != 1 || idim != 1))
            throw std::runtime_error("Identity tensor defined only for compatible (with same dimensions) operators A and B");
        kind = ANIGPU_TENSOR_NULL;
        return;
    }
    PointTensors P(xy, f, q, lam, jdim, idim, nfa);
    bool any = true;
    eval_dispatch<Traits>(typename Traits::AggregateType{}, Dfnc, xy, lam, w, P, user_data, any);
    if (!any) {
        kind = ANIGPU_TENSOR_NULL;
        return;
    }
    compress(P.pts, P.scalar_like, f, q, jdim, idim, kind, d);
}

template <typename MatrT>
inline void gather_coords(const Tetras<MatrT>& XYZ, std::vector<double>& xy) {
    const int f = XYZ.fusion;
    xy.resize(12 * (std::size_t)f);
    for (int r = 0; r < f; ++r)
        for (int k = 0; k < 3; ++k) {
            xy[12 * r + 0 + k] = XYZ.XY0.data[k + 3 * r];
            xy[12 * r + 3 + k] = XYZ.XY1.data[k + 3 * r];
            xy[12 * r + 6 + k] = XYZ.XY2.data[k + 3 * r];
            xy[12 * r + 9 + k] = XYZ.XY3.data[k + 3 * r];
        }
}

/* one element integral (tet or face) through the session */
template <typename FuncTraits, typename Functor, typename MatrT>
void integral(int codeA, int nfA, int dA, int codeB, int nfB, int dB, const Tetras<MatrT>& XYZ, const Functor& Dfnc,
              DenseMatrix<double>& A, int order, void* user_data, int face, int normal) {
    const int f = XYZ.fusion;
    if (f <= 0) return;
    if (A.size < (std::size_t)nfA * nfB * f)
        throw std::runtime_error("Not enough memory for local matrix, expected size = " + std::to_string(nfA * nfB * f) +
                                 " but A has size = " + std::to_string(A.size));
    A.nRow = nfB;
    A.nCol = (std::size_t)nfA * f;
    std::vector<double> xy;
    gather_coords(XYZ, xy);
    Session& s = Session::get();
    Request r{};
    r.codeA = codeA, r.codeB = codeB, r.order = order, r.face = face, r.normal = normal;
    r.nfA = nfA, r.nfB = nfB, r.dA = dA, r.dBt = normal ? 3 * dB : dB, r.f = f;
    if (s.mode == gpu::Mode::Replay) {
        const double* res = s.replay(r, xy.data());
        std::copy(res, res + (std::size_t)nfA * nfB * f, A.data);
        return;
    }
    std::vector<double> lam, w;
    const int q = rule_points(order, face, lam, w);
    std::vector<double> d;
    int kind = ANIGPU_TENSOR_NULL;
    eval_tensor<FuncTraits>(Dfnc, xy.data(), f, q, lam, w, (std::size_t)r.dBt, (std::size_t)dA, nfA, user_data, kind, d);
    r.kind = kind;
    r.d_len = d.size();
    if (s.mode == gpu::Mode::Record) {
        s.record(r, xy.data(), d.data());
        std::fill(A.data, A.data + (std::size_t)nfA * nfB * f, 0.0);
        return;
    }
    s.run_now(r, xy.data(), d.data(), A.data);
}

}  // namespace gpu_detail

namespace gpu {
/* the device this thread's element integrals run on (default 0) */
inline void set_device(int device) { gpu_detail::Session::get().set_device(device); }
inline Mode mode() { return gpu_detail::Session::get().mode; }
}  // namespace gpu

// ------------------------------------------------------------------ fem3Dtet (int_tet.h:16-77)
/* A = integral over each tet of (D OpA(u)) . OpB(v): memoryless overload, order <= 6, at most
 * FUSION tets (int_tet.inl:93-122) */
template <typename OpA, typename OpB, typename FuncTraits = DfuncTraits<>, int FUSION = 1, typename ScalarType = double,
          typename IndexType = int, typename Functor, typename TetrasT>
void fem3Dtet(const TetrasT& XYZ, const Functor& Dfnc, DenseMatrix<ScalarType>& A, int order = 5,
              void* user_data = nullptr) {
    static_assert(std::is_same<ScalarType, double>::value, "the GPU element engine computes in double");
    if (A.size < (std::size_t)OpB::Nfa::value * OpA::Nfa::value * XYZ.fusion)
        throw std::runtime_error("Expected dimensions of A is " + std::to_string(OpB::Nfa::value) + "x" +
                                 std::to_string(OpA::Nfa::value * XYZ.fusion) + ", but A has size = " + std::to_string(A.size));
    if (order > 6)
        throw std::runtime_error("Quadratures more than 6-th order are not supported for stack memory version of the function");
    if (XYZ.fusion > FUSION)
        throw std::runtime_error("This version of the function not supported fusion that more than " + std::to_string(FUSION));
    gpu_detail::integral<FuncTraits>(OpA::code, OpA::Nfa::value, OpA::Dim::value, OpB::code, OpB::Nfa::value,
                                     OpB::Dim::value, XYZ, Dfnc, A, order, user_data, -1, 0);
}

/* the PlainMemory overload: any fusion, orders 0..20 (int_tet.inl:30-57) */
template <typename OpA, typename OpB, typename FuncTraits = DfuncTraits<>, typename ScalarType = double,
          typename IndexType = int, typename Functor, typename TetrasT>
void fem3Dtet(const TetrasT& XYZ, const Functor& Dfnc, DenseMatrix<ScalarType>& A,
              PlainMemory<ScalarType, IndexType> plainMemory, int order = 5, void* user_data = nullptr) {
    static_assert(std::is_same<ScalarType, double>::value, "the GPU element engine computes in double");
    (void)plainMemory;
    gpu_detail::integral<FuncTraits>(OpA::code, OpA::Nfa::value, OpA::Dim::value, OpB::code, OpB::Nfa::value,
                                     OpB::Dim::value, XYZ, Dfnc, A, order, user_data, -1, 0);
}

/* overloads on four 3 x f coordinate matrices (int_tet.h:48-77, 94-121) */
template <typename OpA, typename OpB, typename FuncTraits = DfuncTraits<>, int FUSION = 1, typename ScalarType = double,
          typename IndexType = int, typename Functor>
void fem3Dtet(const DenseMatrix<ScalarType>& XY0, const DenseMatrix<ScalarType>& XY1, const DenseMatrix<ScalarType>& XY2,
              const DenseMatrix<ScalarType>& XY3, const Functor& Dfnc, DenseMatrix<ScalarType>& A, int order = 5,
              void* user_data = nullptr) {
    fem3Dtet<OpA, OpB, FuncTraits, FUSION, ScalarType, IndexType>(
        make_tetras(XY0.data, XY1.data, XY2.data, XY3.data, (int)XY0.nCol), Dfnc, A, order, user_data);
}
template <typename OpA, typename OpB, typename FuncTraits = DfuncTraits<>, int FUSION = 1, typename ScalarType = double,
          typename IndexType = int, typename Functor>
void fem3Dtet(const DenseMatrix<const ScalarType>& XY0, const DenseMatrix<const ScalarType>& XY1,
              const DenseMatrix<const ScalarType>& XY2, const DenseMatrix<const ScalarType>& XY3, const Functor& Dfnc,
              DenseMatrix<ScalarType>& A, int order = 5, void* user_data = nullptr) {
    fem3Dtet<OpA, OpB, FuncTraits, FUSION, ScalarType, IndexType>(
        make_tetras(XY0.data, XY1.data, XY2.data, XY3.data, (int)XY0.nCol), Dfnc, A, order, user_data);
}
template <typename OpA, typename OpB, typename FuncTraits = DfuncTraits<>, typename ScalarType = double,
          typename IndexType = int, typename Functor>
void fem3Dtet(const DenseMatrix<ScalarType>& XY0, const DenseMatrix<ScalarType>& XY1, const DenseMatrix<ScalarType>& XY2,
              const DenseMatrix<ScalarType>& XY3, const Functor& Dfnc, DenseMatrix<ScalarType>& A,
              PlainMemory<ScalarType, IndexType> plainMemory, int order = 5, void* user_data = nullptr) {
    fem3Dtet<OpA, OpB, FuncTraits, ScalarType, IndexType>(make_tetras(XY0.data, XY1.data, XY2.data, XY3.data, (int)XY0.nCol),
                                                          Dfnc, A, plainMemory, order, user_data);
}

// ------------------------------------------------------------------ fem3Dface / fem3DfaceN (int_face.h:15-48)
/* A = integral over face `face_num` (nodes face, face+1, face+2 mod 4) of (D OpA(u)) . OpB(v) */
template <typename OpA, typename OpB, typename FuncTraits = DfuncTraits<>, int FUSION = 1, typename ScalarType = double,
          typename IndexType = int, typename Functor, typename TetrasT>
void fem3Dface(const TetrasT& XYZ, int face_num, const Functor& Dfnc, DenseMatrix<ScalarType>& A, int order = 5,
               void* user_data = nullptr) {
    if (order > 9)
        throw std::runtime_error("Quadratures more than 9-th order are not supported for stack memory version of the function");
    if (XYZ.fusion > FUSION)
        throw std::runtime_error("This version of the function not supported fusion that more than " + std::to_string(FUSION));
    gpu_detail::integral<FuncTraits>(OpA::code, OpA::Nfa::value, OpA::Dim::value, OpB::code, OpB::Nfa::value,
                                     OpB::Dim::value, XYZ, Dfnc, A, order, user_data, face_num, 0);
}
template <typename OpA, typename OpB, typename FuncTraits = DfuncTraits<>, typename ScalarType = double,
          typename IndexType = int, typename Functor, typename TetrasT>
void fem3Dface(const TetrasT& XYZ, int face_num, const Functor& Dfnc, DenseMatrix<ScalarType>& A,
               PlainMemory<ScalarType, IndexType> plainMemory, int order = 5, void* user_data = nullptr) {
    (void)plainMemory;
    gpu_detail::integral<FuncTraits>(OpA::code, OpA::Nfa::value, OpA::Dim::value, OpB::code, OpB::Nfa::value,
                                     OpB::Dim::value, XYZ, Dfnc, A, order, user_data, face_num, 0);
}
/* the same with the tensor's 3 dim(OpB) rows contracted with the outward normal (fem3DfaceN) */
template <typename OpA, typename OpB, typename FuncTraits = DfuncTraits<>, int FUSION = 1, typename ScalarType = double,
          typename IndexType = int, typename Functor, typename TetrasT>
void fem3DfaceN(const TetrasT& XYZ, int face_num, const Functor& Dfnc, DenseMatrix<ScalarType>& A, int order = 5,
                void* user_data = nullptr) {
    if (order > 9)
        throw std::runtime_error("Quadratures more than 9-th order are not supported for stack memory version of the function");
    if (XYZ.fusion > FUSION)
        throw std::runtime_error("This version of the function not supported fusion that more than " + std::to_string(FUSION));
    gpu_detail::integral<FuncTraits>(OpA::code, OpA::Nfa::value, OpA::Dim::value, OpB::code, OpB::Nfa::value,
                                     OpB::Dim::value, XYZ, Dfnc, A, order, user_data, face_num, 1);
}
template <typename OpA, typename OpB, typename FuncTraits = DfuncTraits<>, typename ScalarType = double,
          typename IndexType = int, typename Functor, typename TetrasT>
void fem3DfaceN(const TetrasT& XYZ, int face_num, const Functor& Dfnc, DenseMatrix<ScalarType>& A,
                PlainMemory<ScalarType, IndexType> plainMemory, int order = 5, void* user_data = nullptr) {
    (void)plainMemory;
    gpu_detail::integral<FuncTraits>(OpA::code, OpA::Nfa::value, OpA::Dim::value, OpB::code, OpB::Nfa::value,
                                     OpB::Dim::value, XYZ, Dfnc, A, order, user_data, face_num, 1);
}

// ------------------------------------------------------------------ local-assembler contract (func_wrap.h:311-317)
/* a wrapped local assembler: element matrix nRow x nCol and right-hand side nRow */
struct ElemMatRhsFunc {
    std::function<void(const double**, double*, double*, void*)> f;
    std::size_t nRow = 0, nCol = 0;
};
inline ElemMatRhsFunc GenerateElemMatRhs(std::function<void(const double**, double*, double*, void*)> f, std::size_t nRow,
                                         std::size_t nCol) {
    return {std::move(f), nRow, nCol};
}
inline ElemMatRhsFunc GenerateElemMatRhs(std::function<void(const double**, double*, double*)> f, std::size_t nRow,
                                         std::size_t nCol) {
    return {[f](const double** XY, double* A, double* F, void*) { f(XY, A, F); }, nRow, nCol};
}
inline ElemMatRhsFunc GenerateElemMat(std::function<void(const double**, double*, void*)> f, std::size_t nRow,
                                      std::size_t nCol) {
    return {[f](const double** XY, double* A, double*, void* u) { f(XY, A, u); }, nRow, nCol};
}
inline ElemMatRhsFunc GenerateElemMat(std::function<void(const double**, double*)> f, std::size_t nRow, std::size_t nCol) {
    return {[f](const double** XY, double* A, double*, void*) { f(XY, A); }, nRow, nCol};
}

/* the problem's one unknown: trial and test functions of one space (FemExprDescr /
 * GenerateHelper, fem.h) */
struct VarHelper {
    int space = -1;
};
template <typename FEMTYPE>
struct HelperOf;
template <int FEM>
struct HelperOf<FemFix<FEM>> {
    static constexpr int space = gpu_detail::space_of(FEM);
};
template <int DIM, int FEM>
struct HelperOf<FemVec<DIM, FEM>> {
    static_assert(DIM == 3 && FEM == FEM_P2, "the GPU global assembly takes FemVec<3, FEM_P2>");
    static constexpr int space = ANIGPU_VEC3_P2;
};
template <typename FEMTYPE>
VarHelper GenerateHelper() {
    return VarHelper{HelperOf<FEMTYPE>::space};
}
struct FemExprDescr {
    std::vector<std::pair<VarHelper, std::string>> trial, test;
    void PushTrialFunc(VarHelper h, std::string name) { trial.emplace_back(h, std::move(name)); }
    void PushTestFunc(VarHelper h, std::string name) { test.emplace_back(h, std::move(name)); }
};

/* what the data gatherer sees of one element: its oriented nodes (coordinates and mesh node ids)
 * and compute(), which runs the local assembler (ElementalAssembler, elemental_assembler.h:118-219) */
struct ElementalAssembler {
    const double* xy = nullptr;      // 12 doubles: nodes 0..3 of the oriented tet
    const int32_t* node_ids = nullptr;
    int64_t cell = 0;
    const ElemMatRhsFunc* func = nullptr;
    double* A = nullptr;
    double* F = nullptr;
    double nodes_copy[12];
    double* get_nodes() {
        std::copy(xy, xy + 12, nodes_copy);
        return nodes_copy;
    }
    int32_t node_id(int i) const { return node_ids[i]; }
    void compute(const double** args, void* user_data = nullptr) { func->f(args, A, F, user_data); }
};

/* assembled system on the device: CSR template (rowptr i64, col i32) with FP64 values, and vectors */
struct SparseMatrix {
    int64_t n = 0, nnz = 0;
    int64_t* rowptr = nullptr;
    int32_t* col = nullptr;
    double* vals = nullptr;
    SparseMatrix() = default;
    SparseMatrix(const SparseMatrix&) = delete;
    SparseMatrix& operator=(const SparseMatrix&) = delete;
    ~SparseMatrix() { release(); }
    void release() {
        if (rowptr) cudaFree(rowptr);
        if (col) cudaFree(col);
        if (vals) cudaFree(vals);
        rowptr = nullptr, col = nullptr, vals = nullptr, n = nnz = 0;
    }
    void resize(int64_t nrow, int64_t nz) {
        if (nrow == n && nz == nnz && rowptr) return;
        release();
        gpu_detail::check_cuda(cudaMalloc((void**)&rowptr, sizeof(int64_t) * (nrow + 1)), "cudaMalloc");
        gpu_detail::check_cuda(cudaMalloc((void**)&col, sizeof(int32_t) * std::max<int64_t>(nz, 1)), "cudaMalloc");
        gpu_detail::check_cuda(cudaMalloc((void**)&vals, sizeof(double) * std::max<int64_t>(nz, 1)), "cudaMalloc");
        n = nrow, nnz = nz;
    }
    /* host copies (after the device work of the assembly that filled the matrix) */
    void download(std::vector<int64_t>& rp, std::vector<int32_t>& c, std::vector<double>& v) const {
        rp.resize(n + 1), c.resize(nnz), v.resize(nnz);
        gpu_detail::check_cuda(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
        gpu_detail::check_cuda(cudaMemcpy(rp.data(), rowptr, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost), "cudaMemcpy");
        gpu_detail::check_cuda(cudaMemcpy(c.data(), col, sizeof(int32_t) * nnz, cudaMemcpyDeviceToHost), "cudaMemcpy");
        gpu_detail::check_cuda(cudaMemcpy(v.data(), vals, sizeof(double) * nnz, cudaMemcpyDeviceToHost), "cudaMemcpy");
    }
};
struct Vector {
    int64_t n = 0;
    double* data = nullptr;
    Vector() = default;
    Vector(const Vector&) = delete;
    Vector& operator=(const Vector&) = delete;
    ~Vector() {
        if (data) cudaFree(data);
    }
    void resize(int64_t m) {
        if (m == n && data) return;
        if (data) cudaFree(data);
        data = nullptr;
        gpu_detail::check_cuda(cudaMalloc((void**)&data, sizeof(double) * std::max<int64_t>(m, 1)), "cudaMalloc");
        n = m;
        gpu_detail::check_cuda(cudaMemset(data, 0, sizeof(double) * std::max<int64_t>(m, 1)), "cudaMemset");
    }
    void download(std::vector<double>& v) const {
        v.resize(n);
        gpu_detail::check_cuda(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
        gpu_detail::check_cuda(cudaMemcpy(v.data(), data, sizeof(double) * n, cudaMemcpyDeviceToHost), "cudaMemcpy");
    }
};

/* The global assembler (AssemblerT, assembler.h:316-386) on a tetrahedral mesh given as arrays:
 * coordinates xyz[nv*3] and tets[nt*4] (host).  SetMatRHSFunc / SetProbDescr / SetDataGatherer /
 * PrepareProblem / Assemble as the reference; the DOF numbering is NATURAL (vertex DOFs by node,
 * then edge DOFs, FemVec component-major) and the matrix is the topological CSR template. */
class Assembler {
public:
    Assembler(const double* xyz, int64_t nv, const int32_t* tets, int64_t nt, int device = 0)
        : nv_(nv), nt_(nt), xyz_(xyz, xyz + 3 * nv), tets_(tets, tets + 4 * nt) {
        gpu_detail::check_rc(nullptr, anigpu_create(&h_, device), "anigpu_create");
    }
    ~Assembler() {
        if (h_) anigpu_destroy(h_);
    }
    Assembler(const Assembler&) = delete;
    Assembler& operator=(const Assembler&) = delete;

    void SetMatRHSFunc(ElemMatRhsFunc f) { func_ = std::move(f); }
    void SetProbDescr(FemExprDescr d) {
        if (d.trial.size() != 1 || d.test.size() != 1 || d.trial[0].first.space != d.test[0].first.space)
            throw std::runtime_error("the GPU assembler takes one unknown with the same trial and test space");
        space_ = d.trial[0].first.space;
    }
    void SetDataGatherer(std::function<void(ElementalAssembler&)> g) { gather_ = std::move(g); }
    /* elements per record / compute / replay round (host memory of the recorded requests) */
    void SetChunkSize(int64_t n) { chunk_ = std::max<int64_t>(1, n); }

    void PrepareProblem() {
        if (space_ < 0) throw std::runtime_error("SetProbDescr was not called");
        double* dxyz = nullptr;
        int32_t* dtets = nullptr;
        gpu_detail::check_cuda(cudaMalloc((void**)&dxyz, sizeof(double) * 3 * nv_), "cudaMalloc");
        gpu_detail::check_cuda(cudaMalloc((void**)&dtets, sizeof(int32_t) * 4 * nt_), "cudaMalloc");
        gpu_detail::copy_on(h_, dxyz, xyz_.data(), sizeof(double) * 3 * nv_, cudaMemcpyHostToDevice);
        gpu_detail::copy_on(h_, dtets, tets_.data(), sizeof(int32_t) * 4 * nt_, cudaMemcpyHostToDevice);
        int rc = anigpu_mesh_upload(h_, nv_, dxyz, nt_, dtets);
        gpu_detail::check_cuda(cudaStreamSynchronize(gpu_detail::handle_stream(h_)), "cudaStreamSynchronize");
        cudaFree(dxyz);
        cudaFree(dtets);
        gpu_detail::check_rc(h_, rc, "mesh upload");
        gpu_detail::check_rc(h_, anigpu_problem_setup(h_, space_), "PrepareProblem");
        int64_t ne = 0;
        gpu_detail::check_rc(h_, anigpu_problem_info(h_, &ndof_, &nnz_, &ne), "PrepareProblem");
        // the oriented tets the local assembler sees: coordinates and node ids
        double* dxy = nullptr;
        int32_t* dn = nullptr;
        gpu_detail::check_cuda(cudaMalloc((void**)&dxy, sizeof(double) * 12 * nt_), "cudaMalloc");
        gpu_detail::check_cuda(cudaMalloc((void**)&dn, sizeof(int32_t) * 4 * nt_), "cudaMalloc");
        rc = anigpu_element_coords(h_, dxy);
        if (rc == ANIGPU_OK) rc = anigpu_element_nodes(h_, dn);
        elem_xy_.resize(12 * nt_);
        elem_nodes_.resize(4 * nt_);
        if (rc == ANIGPU_OK) {
            gpu_detail::copy_on(h_, elem_xy_.data(), dxy, sizeof(double) * 12 * nt_, cudaMemcpyDeviceToHost);
            gpu_detail::copy_on(h_, elem_nodes_.data(), dn, sizeof(int32_t) * 4 * nt_, cudaMemcpyDeviceToHost);
        }
        cudaFree(dxy);
        cudaFree(dn);
        gpu_detail::check_rc(h_, rc, "PrepareProblem");
        prepared_ = true;
    }

    /* A, b: the assembled system (FP64) in the CSR template; returns 0, or -1 when a value is not
     * finite (AssemblerT::Assemble status, assembler.inl:306-313) */
    int Assemble(SparseMatrix& A, Vector& b) {
        if (!prepared_) throw std::runtime_error("PrepareProblem was not called");
        if (!func_.f) throw std::runtime_error("SetMatRHSFunc was not called");
        const std::size_t nA = func_.nRow * func_.nCol, nF = func_.nRow;
        double *dA = nullptr, *dF = nullptr;
        gpu_detail::check_cuda(cudaMalloc((void**)&dA, sizeof(double) * nA * nt_), "cudaMalloc");
        gpu_detail::check_cuda(cudaMalloc((void**)&dF, sizeof(double) * nF * nt_), "cudaMalloc");
        gpu_detail::Session& s = gpu_detail::Session::get();
        bool owned = false;
        anigpu_handle saved = s.swap_handle(h_, owned);
        int status = 0;
        try {
            std::vector<double> Ae, Fe;
            for (int64_t e0 = 0; e0 < nt_; e0 += chunk_) {
                const int64_t e1 = std::min<int64_t>(nt_, e0 + chunk_);
                Ae.assign(nA * (e1 - e0), 0.0);
                Fe.assign(nF * (e1 - e0), 0.0);
                s.clear_records();
                s.mode = gpu::Mode::Record;
                run_pass(e0, e1, Ae, Fe);
                s.mode = gpu::Mode::Eager;
                s.flush();
                s.mode = gpu::Mode::Replay;
                std::fill(Ae.begin(), Ae.end(), 0.0);
                std::fill(Fe.begin(), Fe.end(), 0.0);
                run_pass(e0, e1, Ae, Fe);
                s.mode = gpu::Mode::Eager;
                if (s.replayed() != s.recorded())
                    throw std::runtime_error("fem3Dtet replay: fewer element integrals than recorded (the local assembler "
                                             "must make the same calls on both passes)");
                s.clear_records();
                gpu_detail::copy_on(h_, dA + nA * e0, Ae.data(), sizeof(double) * nA * (e1 - e0), cudaMemcpyHostToDevice);
                gpu_detail::copy_on(h_, dF + nF * e0, Fe.data(), sizeof(double) * nF * (e1 - e0), cudaMemcpyHostToDevice);
            }
            A.resize(ndof_, nnz_);
            b.resize(ndof_);
            gpu_detail::check_rc(h_, anigpu_csr_template(h_, A.rowptr, A.col), "Assemble");
            const int rc = anigpu_assemble_elements(h_, dA, dF, A.vals, b.data);
            gpu_detail::check_cuda(cudaStreamSynchronize(gpu_detail::handle_stream(h_)), "cudaStreamSynchronize");
            if (rc == ANIGPU_ERR_NONFINITE)
                status = -1;
            else
                gpu_detail::check_rc(h_, rc, "Assemble");
        } catch (...) {
            s.mode = gpu::Mode::Eager;
            s.clear_records();
            s.restore_handle(saved, owned);
            cudaFree(dA);
            cudaFree(dF);
            throw;
        }
        s.restore_handle(saved, owned);
        cudaFree(dA);
        cudaFree(dF);
        return status;
    }

    int64_t getMatrixSize() const { return ndof_; }
    int64_t getBegInd() const { return 0; }
    int64_t getEndInd() const { return ndof_; }
    int64_t nnz() const { return nnz_; }
    anigpu_handle handle() const { return h_; }

private:
    void run_pass(int64_t e0, int64_t e1, std::vector<double>& Ae, std::vector<double>& Fe) {
        const std::size_t nA = func_.nRow * func_.nCol, nF = func_.nRow;
        for (int64_t e = e0; e < e1; ++e) {
            ElementalAssembler p;
            p.xy = elem_xy_.data() + 12 * e;
            p.node_ids = elem_nodes_.data() + 4 * e;
            p.cell = e;
            p.func = &func_;
            p.A = Ae.data() + nA * (e - e0);
            p.F = Fe.data() + nF * (e - e0);
            if (gather_) {
                gather_(p);
            } else {
                const double* args[4] = {p.xy, p.xy + 3, p.xy + 6, p.xy + 9};
                p.compute(args, nullptr);
            }
        }
    }

    anigpu_handle h_ = nullptr;
    int64_t nv_, nt_;
    std::vector<double> xyz_;
    std::vector<int32_t> tets_;
    ElemMatRhsFunc func_;
    std::function<void(ElementalAssembler&)> gather_;
    int space_ = -1;
    bool prepared_ = false;
    int64_t ndof_ = 0, nnz_ = 0, chunk_ = 65536;
    std::vector<double> elem_xy_;
    std::vector<int32_t> elem_nodes_;
};

}  // namespace Ani

#endif
