// Global assembly: GRAD.GRAD stiffness + P0 x IDEN right-hand side of a scalar
// Lagrange space, with element-level Dirichlet elimination, written straight into the
// CSR template.  Replaces the per-cell loop of AssemblerT::Assemble
// (anifem++/inmost_interface/assembler.inl:314-487) that calls fem3Dtet per cell and
// scatters into INMOST row lists.
//
// Formulation.  For a tensor that is constant on a tet (NULL, SCALAR, SYMMETRIC kinds)
// the quadrature sum of fem3Dtet factorises:
//     A_ij = sum_n w_n |T| (PSI^T g_i(n))^T D (PSI^T g_j(n)) = sum_{a<=b} K_ab Tsym^{ab}_ij
//     K = |T| PSI D PSI^T (3x3 symmetric, 6 numbers per tet)
//     Tsym^{aa} = S^{aa}, Tsym^{ab} = S^{ab} + S^{ba},  S^{ab}_ij = sum_n w_n g_i^a(n) g_j^b(n)
// where g are the reference gradients and S is computed once on the host with the same
// quadrature rule the caller asked for.  Phase 1 computes K (and f|T|) once per tet;
// phase 2 is a row gather: every CSR row is owned by one group of NLOC lanes, which walks
// the row's incident tets in ascending tet order, computes that tet's row of A (lane j
// computes A(i, j)) and adds it into a shared-memory copy of the row at the offsets held
// by the scatter record.  Each value is therefore summed in the same order as the
// reference's serial cell loop, without atomics, and written to HBM once, coalesced.
#include <mutex>

#include "anigpu_internal.h"
#include "quad_tables.h"

namespace {

constexpr int kChunk = 16;  // incidences staged per group per step

// ---------------------------------------------------------------- phase 1
// FP64 -> FP32 with round-to-nearest-even in integer arithmetic.  GB300 runs FP64 (and
// the F64->F32 conversion) at a small fraction of its FP32 rate, so the FP32 path keeps
// every FP64 instruction off its common path; zero, subnormal and out-of-range inputs go
// through the hardware conversion.
__device__ __forceinline__ float d2f_rn(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const int e = (int)((hi >> 20) & 0x7ffu) - 1023 + 127;
    if (e <= 0 || e >= 255) return (b << 1) == 0 ? __uint_as_float(hi & 0x80000000u) : __double2float_rn(x);
    const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const unsigned rest = lo & 0x1fffffffu;
    unsigned f = (hi & 0x80000000u) | ((unsigned)e << 23) | m;
    if (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) f += 1u;
    return __uint_as_float(f);
}

// K = |T| PSI D PSI^T (k00 k11 k22 k01 k02 k12), then f|T| and 0: 8 values per tet.
// PSI(a,a') = PSI[a + 3a'] (inverse3x3, geometry.h:26-44; core.inl:217-247).
template <typename R>
__device__ __forceinline__ void k_from_psi(const R* PSI, const R* d, R mes, R* K) {
    const R Dm[9] = {d[0], d[1], d[2], d[1], d[3], d[4], d[2], d[4], d[5]};
    R M[9];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) M[a + 3 * b] = PSI[a] * Dm[3 * b] + PSI[a + 3] * Dm[1 + 3 * b] + PSI[a + 6] * Dm[2 + 3 * b];
    auto kab = [&](int a, int b) { return mes * (M[a] * PSI[b] + M[a + 3] * PSI[b + 3] + M[a + 6] * PSI[b + 6]); };
    K[0] = kab(0, 0);
    K[1] = kab(1, 1);
    K[2] = kab(2, 2);
    K[3] = kab(0, 1);
    K[4] = kab(0, 2);
    K[5] = kab(1, 2);
}

template <typename R>
__device__ __forceinline__ R inverse3(const R* m, R* inv) {
#define M(I, J) m[(I) + 3 * (J)]
    const R da = M(1, 1) * M(2, 2) - M(1, 2) * M(2, 1);
    const R db = M(1, 2) * M(2, 0) - M(1, 0) * M(2, 2);
    const R dc = M(1, 0) * M(2, 1) - M(1, 1) * M(2, 0);
    const R det = M(0, 0) * da + M(0, 1) * db + M(0, 2) * dc;
    const R r = R(1) / det;
    inv[0] = da * r;
    inv[1] = db * r;
    inv[2] = dc * r;
#pragma unroll
    for (int i = 1; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
            inv[j + 3 * i] = (M((i + 1) % 3, (j + 1) % 3) * M((i + 2) % 3, (j + 2) % 3) -
                              M((i + 1) % 3, (j + 2) % 3) * M((i + 2) % 3, (j + 1) % 3)) * r;
#undef M
    return det;
}

__device__ __forceinline__ void load_sym(int kind, const double* __restrict__ D, int64_t t, double* d) {
    switch (kind) {
        case ANIGPU_TENSOR_NULL: d[0] = d[3] = d[5] = 1; d[1] = d[2] = d[4] = 0; break;
        case ANIGPU_TENSOR_CONST_SCALAR: d[0] = d[3] = d[5] = D[0]; d[1] = d[2] = d[4] = 0; break;
        case ANIGPU_TENSOR_TET_SCALAR: d[0] = d[3] = d[5] = D[t]; d[1] = d[2] = d[4] = 0; break;
        default:
#pragma unroll
            for (int k = 0; k < 6; ++k) d[k] = D[6 * t + k];
    }
}

// FP64 path (parity arithmetic): everything in FP64, as the reference.
__global__ void tet_prepare_f64_kernel(int64_t nt, const double* __restrict__ xyz, const int32_t* __restrict__ tets,
                                       int kind, const double* __restrict__ D, const double* __restrict__ f,
                                       double f_const, double* __restrict__ out, int* __restrict__ status) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const int4 v = reinterpret_cast<const int4*>(tets)[t];
    double e[9];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double x0 = xyz[3 * (int64_t)v.x + k];
        e[k + 0] = xyz[3 * (int64_t)v.y + k] - x0;  // columns X1-X0, X2-X0, X3-X0 (core.inl:230-236)
        e[k + 3] = xyz[3 * (int64_t)v.z + k] - x0;
        e[k + 6] = xyz[3 * (int64_t)v.w + k] - x0;
    }
    double d[6], PSI[9], K[8];
    load_sym(kind, D, t, d);
    const double det = inverse3(e, PSI);
    const double mes = fabs(det) / 6.0;
    k_from_psi(PSI, d, mes, K);
    K[6] = (f ? f[t] : f_const) * mes;
    K[7] = 0;
    bool bad = !(det != 0.0);
#pragma unroll
    for (int k = 0; k < 7; ++k) bad |= !isfinite(K[k]);
    if (bad) atomicExch(status, ANIGPU_ERR_NONFINITE);
    double2* o = reinterpret_cast<double2*>(out + 8 * t);
#pragma unroll
    for (int q = 0; q < 4; ++q) o[q] = make_double2(K[2 * q], K[2 * q + 1]);
}

// FP32 path: FP32 geometry from the (hi, lo) coordinate pairs; the edge vectors carry one
// FP32 rounding.  A tet whose |det| is small against its edge lengths (badly shaped,
// |det| <= 0.05 |e1||e2||e3|) is redone in FP64 from the FP64 coordinates.
__global__ void tet_prepare_f32_kernel(int64_t nt, const double* __restrict__ xyz, const float2* __restrict__ xyz2,
                                       const int32_t* __restrict__ tets, int kind, const double* __restrict__ D,
                                       const double* __restrict__ f, double f_const, float* __restrict__ out,
                                       int* __restrict__ status) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const int4 v = reinterpret_cast<const int4*>(tets)[t];
    float e[9];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float2 x0 = xyz2[3 * (int64_t)v.x + k];
        const float2 x1 = xyz2[3 * (int64_t)v.y + k];
        const float2 x2 = xyz2[3 * (int64_t)v.z + k];
        const float2 x3 = xyz2[3 * (int64_t)v.w + k];
        e[k + 0] = (x1.x - x0.x) + (x1.y - x0.y);
        e[k + 3] = (x2.x - x0.x) + (x2.y - x0.y);
        e[k + 6] = (x3.x - x0.x) + (x3.y - x0.y);
    }
    float d[6];
    if (kind == ANIGPU_TENSOR_TET_SYM) {
        const double2* Dp = reinterpret_cast<const double2*>(D + 6 * t);
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const double2 w = Dp[q];
            d[2 * q] = d2f_rn(w.x);
            d[2 * q + 1] = d2f_rn(w.y);
        }
    } else {
        const float s = kind == ANIGPU_TENSOR_NULL ? 1.f : d2f_rn(kind == ANIGPU_TENSOR_CONST_SCALAR ? D[0] : D[t]);
        d[0] = d[3] = d[5] = s;
        d[1] = d[2] = d[4] = 0.f;
    }
    const float fv = d2f_rn(f ? f[t] : f_const);
    float PSI[9], K[8];
    const float det = inverse3(e, PSI);
    const float l0 = e[0] * e[0] + e[1] * e[1] + e[2] * e[2];
    const float l1 = e[3] * e[3] + e[4] * e[4] + e[5] * e[5];
    const float l2 = e[6] * e[6] + e[7] * e[7] + e[8] * e[8];
    float mes;
    if (det * det > 0.0025f * l0 * l1 * l2) {
        mes = fabsf(det) * (1.0f / 6.0f);
        k_from_psi(PSI, d, mes, K);
    } else {
        // badly shaped (or degenerate) tet: Jacobian and inverse in FP64
        double ed[9], P64[9], dd[6];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const double x0 = xyz[3 * (int64_t)v.x + k];
            ed[k + 0] = xyz[3 * (int64_t)v.y + k] - x0;
            ed[k + 3] = xyz[3 * (int64_t)v.z + k] - x0;
            ed[k + 6] = xyz[3 * (int64_t)v.w + k] - x0;
        }
        load_sym(kind, D, t, dd);
        const double det64 = inverse3(ed, P64);
        const double mes64 = fabs(det64) / 6.0;
        double K64[6];
        k_from_psi(P64, dd, mes64, K64);
#pragma unroll
        for (int k = 0; k < 6; ++k) K[k] = (float)K64[k];
        mes = (float)mes64;
        if (!(det64 != 0.0)) atomicExch(status, ANIGPU_ERR_NONFINITE);
    }
    K[6] = fv * mes;
    K[7] = 0.f;
    bool bad = false;
#pragma unroll
    for (int k = 0; k < 7; ++k) bad |= !isfinite(K[k]);
    if (bad) atomicExch(status, ANIGPU_ERR_NONFINITE);
    float4* o = reinterpret_cast<float4*>(out + 8 * t);
    o[0] = make_float4(K[0], K[1], K[2], K[3]);
    o[1] = make_float4(K[4], K[5], K[6], K[7]);
}

// ---------------------------------------------------------------- phase 2
struct RowParams {
    int64_t row_begin;  // first row of this launch
    int64_t nrows;      // one past the last row of this launch
    const int64_t* inc_ptr;
    const ScatterRec* recs;
    const int64_t* rowptr;
    const uint8_t* dir_mask;
    const double* dir_bc;
    const int32_t* edofs;
    int cap;  // row buffer capacity (>= longest row)
    double drop;
};

__device__ __forceinline__ uint32_t rec_off(const ScatterRec& r, int j) {
    const uint32_t w = j < 4 ? r.off03 : (j < 8 ? r.off47 : (r.meta >> 16));
    return (w >> (8 * (j & 3))) & 0xffu;
}

template <typename Real>
struct KVec;
template <>
struct KVec<float> {
    float4 a, b;
    __device__ __forceinline__ void load(const float* p) {
        a = reinterpret_cast<const float4*>(p)[0];
        b = reinterpret_cast<const float4*>(p)[1];
    }
    __device__ __forceinline__ float k(int i) const {
        return i == 0 ? a.x : i == 1 ? a.y : i == 2 ? a.z : i == 3 ? a.w : i == 4 ? b.x : i == 5 ? b.y : b.z;
    }
    __device__ __forceinline__ void zero() { a = b = make_float4(0.f, 0.f, 0.f, 0.f); }
};
template <>
struct KVec<double> {
    double2 a, b, c, d;
    __device__ __forceinline__ void load(const double* p) {
        const double2* q = reinterpret_cast<const double2*>(p);
        a = q[0];
        b = q[1];
        c = q[2];
        d = q[3];
    }
    __device__ __forceinline__ double k(int i) const {
        return i == 0 ? a.x : i == 1 ? a.y : i == 2 ? b.x : i == 3 ? b.y : i == 4 ? c.x : i == 5 ? c.y : d.x;
    }
    __device__ __forceinline__ void zero() { a = b = c = d = make_double2(0.0, 0.0); }
};

// Row gather.  One lane owns one CSR row.  It walks the row's incident tets in ascending
// tet order (the order of the reference's serial cell loop), computes the tet's element
// row A_t(i, 0..NLOC-1) = sum_k K_t[k] Tsym[i][j][k] in registers and adds it into its own
// copy of the row in shared memory, lane-interleaved and rotated (see rot()).  The
// record and the per-tet block of the next incidence are prefetched.  At the end the warp
// writes its 32 rows cooperatively (each row contiguous, coalesced).  No atomics: every
// CSR value is produced by exactly one lane with a fixed summation order.
// slot s of lane l lives at s*33 + l (rows padded to 33 words): every lane touching its
// own slot and the transposed read of one row by the whole warp are both free of bank
// conflicts when the lanes' slots are equal (structured meshes), and at most a few-way
// otherwise.
__device__ __forceinline__ int rot(int s, int l) { return s * 33 + l; }

template <typename Real, int NLOC>
struct RowTab {
    // per-i stride padded so that lanes holding different i read distinct banks
    static constexpr int TS = NLOC * 8 + (16 / (int)sizeof(Real));
    static constexpr int SIZE = NLOC * TS + NLOC;  // then m[i]
};

template <typename Real, int NLOC, bool DIR, bool BCNZ, bool TOUCH, bool DROPCHK>
__global__ void __launch_bounds__(64) row_gather_kernel(RowParams p, const Real* __restrict__ tables,
                                                        const Real* __restrict__ tetK, Real* __restrict__ vals,
                                                        double* __restrict__ rhs, uint8_t* __restrict__ touched_out,
                                                        int* __restrict__ status) {
    using Tab = RowTab<Real, NLOC>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    Real* sT = reinterpret_cast<Real*>(smem_raw);
    // host layout [i][j][8] -> padded stride TS per i
    for (int k = threadIdx.x; k < NLOC * NLOC * 8; k += blockDim.x) {
        const int i = k / (NLOC * 8), rem = k - i * NLOC * 8;
        sT[i * Tab::TS + rem] = tables[k];
    }
    for (int k = threadIdx.x; k < NLOC; k += blockDim.x) sT[NLOC * Tab::TS + k] = tables[NLOC * NLOC * 8 + k];
    const Real* sM = sT + NLOC * Tab::TS;
    const size_t tab_bytes = ((sizeof(Real) * Tab::SIZE + 15) / 16) * 16;
    // per warp: row metadata (32 x {row start, length}), the rows, the touched map
    const size_t meta_bytes = 32 * 16;
    const size_t row_bytes = (((size_t)p.cap * 33 * sizeof(Real)) + 15) / 16 * 16;
    const size_t touch_bytes = TOUCH ? (((size_t)p.cap * 33) + 15) / 16 * 16 : 0;
    unsigned char* wbase = smem_raw + tab_bytes + (meta_bytes + row_bytes + touch_bytes) * warp;
    longlong2* sMeta = reinterpret_cast<longlong2*>(wbase);
    Real* sRow = reinterpret_cast<Real*>(wbase + meta_bytes);
    uint8_t* sTouch = reinterpret_cast<uint8_t*>(wbase + meta_bytes + row_bytes);
    // zero this warp's rows (and touched map), 16 bytes per store
    for (size_t k = lane; k < (row_bytes + touch_bytes) / 16; k += 32)
        reinterpret_cast<int4*>(sRow)[k] = make_int4(0, 0, 0, 0);

    const int64_t row0 = p.row_begin + ((int64_t)blockIdx.x * nwarps + warp) * 32;
    const int64_t row = row0 + lane;
    const bool valid = row < p.nrows;
    int64_t ib = 0, rb = 0;
    int len = 0, deg = 0;
    bool isdir = false;
    if (valid) {
        ib = p.inc_ptr[row];
        deg = (int)(p.inc_ptr[row + 1] - ib);
        rb = p.rowptr[row];
        len = (int)(p.rowptr[row + 1] - rb);
        if (DIR) isdir = p.dir_mask[row] != 0;
    }
    sMeta[lane] = make_longlong2(rb, len);
    __syncthreads();
    Real* myRow = sRow + lane;  // slot s at myRow[s * 33]
    uint8_t* myTouch = sTouch + lane;
    const Real drop = Real(p.drop);
    Real racc = Real(0);
    // software pipeline over the incidences: r0/K0 current, r1 next; indices are clamped
    // to the last incidence so that the loop body has no branches
    ScatterRec r0 = {0u, 0u, 0u, 0u}, r1 = {0u, 0u, 0u, 0u};
    KVec<Real> K0, K1;
    K0.zero();
    if (deg > 0) {
        r0 = p.recs[ib];
        K0.load(tetK + 8 * (int64_t)r0.tet);
        r1 = p.recs[ib + (deg > 1 ? 1 : 0)];
    }
    const int last = deg - 1;
    for (int k = 0; k < deg; ++k) {
        K1.load(tetK + 8 * (int64_t)r1.tet);
        const ScatterRec r2 = p.recs[ib + min(k + 2, last)];
        const int i = r0.meta & 15;
        const Real* T = sT + i * Tab::TS;
        const uint32_t dm = DIR ? (r0.meta >> 4) & 0x3ffu : 0u;
        const Real k0 = K0.k(0), k1 = K0.k(1), k2 = K0.k(2), k3 = K0.k(3), k4 = K0.k(4), k5 = K0.k(5);
        Real F = K0.k(6) * sM[i];
        Real a[NLOC];
        int addr[NLOC];
        uint32_t addbits = 0;
#pragma unroll
        for (int j = 0; j < NLOC; ++j) {
            Real v;
            if (sizeof(Real) == 4) {
                const float4 t0 = reinterpret_cast<const float4*>(T + j * 8)[0];
                const float4 t1 = reinterpret_cast<const float4*>(T + j * 8)[1];
                v = k0 * Real(t0.x);
                v = fma(k1, Real(t0.y), v);
                v = fma(k2, Real(t0.z), v);
                v = fma(k3, Real(t0.w), v);
                v = fma(k4, Real(t1.x), v);
                v = fma(k5, Real(t1.y), v);
            } else {
                const double2 t0 = reinterpret_cast<const double2*>(T + j * 8)[0];
                const double2 t1 = reinterpret_cast<const double2*>(T + j * 8)[1];
                const double2 t2 = reinterpret_cast<const double2*>(T + j * 8)[2];
                v = k0 * Real(t0.x);
                v = fma(k1, Real(t0.y), v);
                v = fma(k2, Real(t1.x), v);
                v = fma(k3, Real(t1.y), v);
                v = fma(k4, Real(t2.x), v);
                v = fma(k5, Real(t2.y), v);
            }
            const bool colDir = DIR && ((dm >> j) & 1u);
            if (BCNZ && colDir)  // applyDir on Dirichlet column j, ascending j (dc_on_dof.h:39-45)
                F -= v * Real(p.dir_bc[p.edofs[(int64_t)r0.tet * NLOC + j]]);
            // the drop rule |a| > drop_val (assembler.inl:416-418).  Without a touched map and
            // with a drop value that rounds to zero in FP32 the rule only skips exact zeros,
            // which cannot change a sum: that variant is compiled without the test.
            bool add = !colDir && (!DROPCHK || fabs(v) > drop);
            if (DIR) {  // a Dirichlet row: applyDir makes the element row e_i
                add = isdir ? (j == i) : add;
                v = isdir ? Real(1) : v;
            }
            a[j] = add ? v : Real(0);
            if (TOUCH) addbits |= (add ? 1u : 0u) << j;
            addr[j] = (int)rec_off(r0, j) * 33;
        }
        // the NLOC slots of one element row are distinct columns: independent updates
        Real cur[NLOC];
#pragma unroll
        for (int j = 0; j < NLOC; ++j) cur[j] = myRow[addr[j]];
#pragma unroll
        for (int j = 0; j < NLOC; ++j) myRow[addr[j]] = cur[j] + a[j];
        if (TOUCH) {
#pragma unroll
            for (int j = 0; j < NLOC; ++j)
                myTouch[addr[j]] |= (uint8_t)((addbits >> j) & 1u);
        }
        racc += (DIR && isdir) ? Real(0) : F;
        r0 = r1;
        K0 = K1;
        r1 = r2;
    }
    bool bad = false;
    if (valid) {
        double F;
        if (DIR && isdir) {
            const double bcr = p.dir_bc[row];
            F = 0;
            for (int q = 0; q < deg; ++q) F += bcr;  // sum of bc over the incident tets
        } else {
            F = (double)racc;
        }
        bad |= !isfinite(F);
        rhs[row] = F;
    }
    __syncwarp();
    // cooperative write-out: row by row, all lanes, contiguous stores
    const int64_t rem_rows = p.nrows - row0;
    const int nrow = rem_rows < 32 ? (int)rem_rows : 32;
    for (int w = 0; w < nrow; ++w) {
        const longlong2 m = sMeta[w];
        const Real* src = sRow + w;
        for (int s = lane; s < (int)m.y; s += 32) {
            const Real v = src[s * 33];
            bad |= !isfinite(v);
            vals[m.x + s] = v;
            if (TOUCH) touched_out[m.x + s] = sTouch[s * 33 + w];
        }
    }
    if (bad) atomicExch(status, ANIGPU_ERR_NONFINITE);
}

// ---------------------------------------------------------------- CSR compaction
__global__ void compact_count_kernel(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                     const uint8_t* __restrict__ touched, unsigned long long* __restrict__ cnt) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= n) return;
    unsigned long long c = 0;
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) c += (touched[k] || col[k] == r) ? 1 : 0;
    cnt[r] = c;
}
template <typename Real>
__global__ void compact_fill_kernel(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                    const Real* __restrict__ vals, const uint8_t* __restrict__ touched,
                                    const int64_t* __restrict__ nptr, int32_t* __restrict__ ncol,
                                    Real* __restrict__ nvals) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= n) return;
    int64_t w = nptr[r];
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k)
        if (touched[k] || col[k] == r) {
            ncol[w] = col[k];
            if (vals) nvals[w] = vals[k];
            ++w;
        }
}

}  // namespace

// host: Tsym tables and m for (space, order) in precision
static int get_row_tables(anigpu_ctx* h, int space, int order, int precision, const void** dev) {
    const int key = 1000 * precision + 100 * space + order + 100000;
    for (auto& kv : h->basis_dev)
        if (kv.first == key) {
            *dev = kv.second;
            return ANIGPU_OK;
        }
    ScalarBasisTable tb;
    if (!make_scalar_basis(space, order, &tb)) return set_err(h, ANIGPU_ERR_UNSUPPORTED, "unsupported space/order");
    const int nf = tb.nf, q = tb.q;
    // Tsym[i][j][k] (k = 00 11 22 01 02 12, padded to 8) then m[i]
    std::vector<double> T((size_t)nf * nf * 8 + nf, 0.0);
    const int A[6] = {0, 1, 2, 0, 0, 1}, B[6] = {0, 1, 2, 1, 2, 2};
    for (int k = 0; k < 6; ++k)
        for (int i = 0; i < nf; ++i)
            for (int j = 0; j < nf; ++j) {
                double s = 0;
                for (int n = 0; n < q; ++n) {
                    const double* gi = &tb.grad[((size_t)n * nf + i) * 3];
                    const double* gj = &tb.grad[((size_t)n * nf + j) * 3];
                    double v = gi[A[k]] * gj[B[k]];
                    if (A[k] != B[k]) v += gi[B[k]] * gj[A[k]];
                    s += tb.wts[n] * v;
                }
                T[((size_t)i * nf + j) * 8 + k] = s;
            }
    for (int i = 0; i < nf; ++i) {
        double s = 0;
        for (int n = 0; n < q; ++n) s += tb.wts[n] * tb.val[(size_t)n * nf + i];
        T[(size_t)nf * nf * 8 + i] = s;
    }
    void* d = nullptr;
    if (precision == ANIGPU_F32) {
        std::vector<float> Tf(T.begin(), T.end());
        ANI_CUDA(h, cudaMalloc(&d, Tf.size() * sizeof(float)));
        ANI_CUDA(h, cudaMemcpy(d, Tf.data(), Tf.size() * sizeof(float), cudaMemcpyHostToDevice));
    } else {
        ANI_CUDA(h, cudaMalloc(&d, T.size() * sizeof(double)));
        ANI_CUDA(h, cudaMemcpy(d, T.data(), T.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    h->basis_dev.push_back({key, (double*)d});
    *dev = d;
    return ANIGPU_OK;
}

template <typename Real, int NLOC, bool DIR, bool BCNZ, bool TOUCH, bool DROPCHK>
static int launch_rows_t(anigpu_ctx* h, const RowParams& p, const void* tables, void* vals, double* rhs,
                         uint8_t* touched, cudaStream_t st) {
    const int warps = 2;
    const size_t tab_bytes = ((sizeof(Real) * RowTab<Real, NLOC>::SIZE + 15) / 16) * 16;
    const size_t row_bytes = (((size_t)p.cap * 33 * sizeof(Real)) + 15) / 16 * 16;
    const size_t touch_bytes = TOUCH ? (((size_t)p.cap * 33) + 15) / 16 * 16 : 0;
    const size_t smem = tab_bytes + (32 * 16 + row_bytes + touch_bytes) * warps;
    auto kern = row_gather_kernel<Real, NLOC, DIR, BCNZ, TOUCH, DROPCHK>;
    ANI_CUDA(h, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<grid_for(p.nrows - p.row_begin, 32 * warps), 32 * warps, smem, st>>>(
        p, (const Real*)tables, (const Real*)h->tetdata, (Real*)vals, rhs, touched, h->d_status);
    ANI_LAUNCHED(h);
    return ANIGPU_OK;
}

template <typename Real, int NLOC>
static int launch_rows(anigpu_ctx* h, const RowParams& p, const void* tables, void* vals, double* rhs,
                       uint8_t* touched, cudaStream_t st) {
    const bool dir = h->has_dirichlet, bcnz = h->bc_nonzero, tch = touched != nullptr;
    // FP32 template assembly with a drop value that is zero in FP32 needs no drop test
    const bool dchk = tch || sizeof(Real) == 8 || (float)p.drop != 0.0f;
#define LR(D, B, T, C) return launch_rows_t<Real, NLOC, D, B, T, C>(h, p, tables, vals, rhs, touched, st)
    if (tch) {
        if (!dir) LR(false, false, true, true);
        if (bcnz) LR(true, true, true, true);
        LR(true, false, true, true);
    }
    if (dchk) {
        if (!dir) LR(false, false, false, true);
        if (bcnz) LR(true, true, false, true);
        LR(true, false, false, true);
    }
    if (!dir) LR(false, false, false, false);
    if (bcnz) LR(true, true, false, false);
    LR(true, false, false, false);
#undef LR
}

int run_assemble(anigpu_ctx* h, int kind, const double* D, const double* f, double f_const, int order,
                 int precision, void* vals, double* rhs, uint8_t* touched, double drop_val) {
    if (h->space < 0) return set_err(h, ANIGPU_ERR_STATE, "anigpu_problem_setup not called");
    if (h->space == ANIGPU_VEC3_P2) return set_err(h, ANIGPU_ERR_UNSUPPORTED, "vector assembly not built yet");
    if (kind != ANIGPU_TENSOR_NULL && kind != ANIGPU_TENSOR_CONST_SCALAR && kind != ANIGPU_TENSOR_TET_SCALAR &&
        kind != ANIGPU_TENSOR_TET_SYM)
        return set_err(h, ANIGPU_ERR_UNSUPPORTED, "assembly tensor kind must be NULL, CONST_SCALAR, TET_SCALAR or TET_SYM");
    if (kind != ANIGPU_TENSOR_NULL && !D) return set_err(h, ANIGPU_ERR_ARG, "tensor data is NULL");
    if (!vals || !rhs) return set_err(h, ANIGPU_ERR_ARG, "NULL output");
    if (precision != ANIGPU_F32 && precision != ANIGPU_F64) return set_err(h, ANIGPU_ERR_ARG, "precision");
    const void* tables = nullptr;
    int rc = get_row_tables(h, h->space, order, precision, &tables);
    if (rc) return rc;
    const size_t rsz = precision == ANIGPU_F32 ? 4 : 8;
    const size_t need = (size_t)h->nt * 8 * rsz;
    if (h->tetdata_bytes < need) {
        if (h->tetdata) cudaFree(h->tetdata);
        h->tetdata = nullptr;
        ANI_CUDA(h, cudaMalloc(&h->tetdata, need));
        h->tetdata_bytes = need;
    }
    time_mark(h, 0);
    if (precision == ANIGPU_F32)
        tet_prepare_f32_kernel<<<grid_for(h->nt, 256), 256, 0, h->stream>>>(
            h->nt, h->xyz, h->xyz2, h->tets, kind, D, f, f_const, (float*)h->tetdata, h->d_status);
    else
        tet_prepare_f64_kernel<<<grid_for(h->nt, 256), 256, 0, h->stream>>>(
            h->nt, h->xyz, h->tets, kind, D, f, f_const, (double*)h->tetdata, h->d_status);
    ANI_LAUNCHED(h);
    time_mark(h, 1);
    RowParams p;
    p.inc_ptr = h->inc_ptr;
    p.recs = h->recs;
    p.rowptr = h->rowptr_s;
    p.dir_mask = h->dir_mask;
    p.dir_bc = h->dir_bc;
    p.edofs = h->edofs;
    p.drop = drop_val;
    // one launch per row range (vertex rows, edge rows) so that the shared-memory row
    // buffer fits the longest row of that range; the two run concurrently (the vertex
    // range on a side stream) so that the tail of one overlaps the other
    cudaStream_t side = h->side_stream ? h->side_stream : h->stream;
    if (side != h->stream) {
        ANI_CUDA(h, cudaEventRecord(h->fork_ev, h->stream));
        ANI_CUDA(h, cudaStreamWaitEvent(side, h->fork_ev, 0));
    }
    for (int rg = 0; rg < 2; ++rg) {
        p.row_begin = h->row_range[rg];
        p.nrows = h->row_range[rg + 1];
        p.cap = h->row_range_cap[rg];
        if (p.nrows <= p.row_begin) continue;
        cudaStream_t st = rg == 0 ? side : h->stream;
        if (h->nloc_s == 10) {
            rc = precision == ANIGPU_F32 ? launch_rows<float, 10>(h, p, tables, vals, rhs, touched, st)
                                         : launch_rows<double, 10>(h, p, tables, vals, rhs, touched, st);
        } else {
            rc = precision == ANIGPU_F32 ? launch_rows<float, 4>(h, p, tables, vals, rhs, touched, st)
                                         : launch_rows<double, 4>(h, p, tables, vals, rhs, touched, st);
        }
        if (rc) return rc;
    }
    if (side != h->stream) {
        ANI_CUDA(h, cudaEventRecord(h->join_ev, side));
        ANI_CUDA(h, cudaStreamWaitEvent(h->stream, h->join_ev, 0));
    }
    time_mark(h, 2);
    return rc;
}

int run_compact(anigpu_ctx* h, int64_t* rowptr, int32_t* col, void* vals, int precision, const uint8_t* touched,
                int64_t* nnz_out) {
    if (h->space < 0) return set_err(h, ANIGPU_ERR_STATE, "anigpu_problem_setup not called");
    const int64_t n = h->ndof;
    cudaStream_t s = h->stream;
    int64_t nnz_old = 0;
    ANI_CUDA(h, cudaMemcpyAsync(&nnz_old, rowptr + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    ANI_CUDA(h, cudaStreamSynchronize(s));
    unsigned long long* cnt = nullptr;
    int64_t* nptr = nullptr;
    int32_t* ncol = nullptr;
    void* nvals = nullptr;
    const size_t rsz = precision == ANIGPU_F32 ? 4 : 8;
    ANI_CUDA(h, cudaMallocAsync((void**)&cnt, sizeof(unsigned long long) * (n + 1), s));
    ANI_CUDA(h, cudaMallocAsync((void**)&nptr, sizeof(int64_t) * (n + 1), s));
    ANI_CUDA(h, cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * (n + 1), s));
    compact_count_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, rowptr, col, touched, cnt);
    ANI_LAUNCHED(h);
    {
        int rc = scan_counts(h, cnt, n, nptr);
        if (rc) return rc;
        ANI_CUDA(h, cudaMemcpyAsync(nnz_out, nptr + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        ANI_CUDA(h, cudaStreamSynchronize(s));
    }
    ANI_CUDA(h, cudaMallocAsync((void**)&ncol, sizeof(int32_t) * std::max<int64_t>(*nnz_out, 1), s));
    ANI_CUDA(h, cudaMallocAsync(&nvals, rsz * std::max<int64_t>(*nnz_out, 1), s));
    if (precision == ANIGPU_F32)
        compact_fill_kernel<float><<<grid_for(n, 256), 256, 0, s>>>(n, rowptr, col, (const float*)vals, touched, nptr,
                                                                   ncol, (float*)nvals);
    else
        compact_fill_kernel<double><<<grid_for(n, 256), 256, 0, s>>>(n, rowptr, col, (const double*)vals, touched,
                                                                    nptr, ncol, (double*)nvals);
    ANI_LAUNCHED(h);
    ANI_CUDA(h, cudaMemcpyAsync(rowptr, nptr, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToDevice, s));
    ANI_CUDA(h, cudaMemcpyAsync(col, ncol, sizeof(int32_t) * *nnz_out, cudaMemcpyDeviceToDevice, s));
    if (vals) ANI_CUDA(h, cudaMemcpyAsync(vals, nvals, rsz * *nnz_out, cudaMemcpyDeviceToDevice, s));
    ANI_CUDA(h, cudaFreeAsync(cnt, s));
    ANI_CUDA(h, cudaFreeAsync(nptr, s));
    ANI_CUDA(h, cudaFreeAsync(ncol, s));
    ANI_CUDA(h, cudaFreeAsync(nvals, s));
    ANI_CUDA(h, cudaStreamSynchronize(s));
    (void)nnz_old;
    return ANIGPU_OK;
}

// ---------------------------------------------------------------- allocation-free assembly
// anigpu_assemble_noalloc: the same two kernels as anigpu_assemble, with their scratch (the
// per-tet K blocks and the reference-element tables) in a fixed device array that the
// library owns for its lifetime instead of memory from cudaMalloc.  It exists for callers
// that cannot allocate device memory at the moment they assemble: code whose device memory
// is fully reserved by another allocator (for example a framework's caching allocator), and
// latency-critical loops where cudaMalloc's implicit device-wide synchronisation is not
// acceptable.  The array is a file-scope __device__ variable, so every GPU that loads the
// library holds it (kNoallocScratchBytes) until the process exits.
namespace {
constexpr size_t kNoallocTableBytes = 16u << 10;  // reference tables, at the start
constexpr size_t kNoallocScratchBytes = 16u << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];
constexpr int kNoallocMaxDevices = 64;
void* g_noalloc_dev_ptr[kNoallocMaxDevices] = {};
std::mutex g_noalloc_mu;

// host address of the array is only a stand-in: the device address comes from
// cudaGetSymbolAddress, once per device, with that device current
int noalloc_scratch(anigpu_ctx* h, unsigned char** out) {
    int dev = -1;
    ANI_CUDA(h, cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoallocMaxDevices) return set_err(h, ANIGPU_ERR_UNSUPPORTED, "device index above 63");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_dev_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return cuda_check(h, e != cudaSuccess ? e : cudaErrorInvalidSymbol, "cudaGetSymbolAddress");
        g_noalloc_dev_ptr[dev] = p;
    }
    *out = static_cast<unsigned char*>(g_noalloc_dev_ptr[dev]);
    return ANIGPU_OK;
}

// Tsym[i][j][8] and m[i] for (space, order), computed into caller storage (no allocation)
bool noalloc_tables(int space, int order, double* T, int* nf_out) {
    const double *pp, *ww;
    int q;
    if (!anigpu_quad_rule(order, &pp, &ww, &q)) return false;
    double val[ANIGPU_MAX_Q][20], grad[ANIGPU_MAX_Q][20][3];
    int nf = -1;
    for (int n = 0; n < q; ++n) nf = eval_scalar_basis_at(space, pp + 4 * n, val[n], grad[n]);
    if (nf != 4 && nf != 10) return false;
    const int A[6] = {0, 1, 2, 0, 0, 1}, B[6] = {0, 1, 2, 1, 2, 2};
    for (int i = 0; i < nf; ++i)
        for (int j = 0; j < nf; ++j)
            for (int k = 0; k < 8; ++k) {
                double s = 0;
                if (k < 6)
                    for (int n = 0; n < q; ++n) {
                        double v = grad[n][i][A[k]] * grad[n][j][B[k]];
                        if (A[k] != B[k]) v += grad[n][i][B[k]] * grad[n][j][A[k]];
                        s += ww[n] * v;
                    }
                T[((size_t)i * nf + j) * 8 + k] = s;
            }
    for (int i = 0; i < nf; ++i) {
        double s = 0;
        for (int n = 0; n < q; ++n) s += ww[n] * val[n][i];
        T[(size_t)nf * nf * 8 + i] = s;
    }
    *nf_out = nf;
    return true;
}

template <typename Real, int NLOC, bool DIR, bool BCNZ, bool DROPCHK>
int noalloc_rows(anigpu_ctx* h, const RowParams& p, const Real* tables, const Real* tetK, Real* vals, double* rhs) {
    const int warps = 2;
    const size_t tab_bytes = ((sizeof(Real) * RowTab<Real, NLOC>::SIZE + 15) / 16) * 16;
    const size_t row_bytes = (((size_t)p.cap * 33 * sizeof(Real)) + 15) / 16 * 16;
    const size_t smem = tab_bytes + (32 * 16 + row_bytes) * warps;
    auto kern = row_gather_kernel<Real, NLOC, DIR, BCNZ, false, DROPCHK>;
    ANI_CUDA(h, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<grid_for(p.nrows - p.row_begin, 32 * warps), 32 * warps, smem, h->stream>>>(p, tables, tetK, vals, rhs,
                                                                                        nullptr, h->d_status);
    ANI_LAUNCHED(h);
    return ANIGPU_OK;
}

template <typename Real, int NLOC>
int noalloc_rows_dispatch(anigpu_ctx* h, const RowParams& p, const Real* tables, const Real* tetK, Real* vals,
                          double* rhs) {
    const bool dir = h->has_dirichlet, bcnz = h->bc_nonzero;
    const bool dchk = sizeof(Real) == 8 || (float)p.drop != 0.0f;
#define NR(D, B, C) return noalloc_rows<Real, NLOC, D, B, C>(h, p, tables, tetK, vals, rhs)
    if (dchk) {
        if (!dir) NR(false, false, true);
        if (bcnz) NR(true, true, true);
        NR(true, false, true);
    }
    if (!dir) NR(false, false, false);
    if (bcnz) NR(true, true, false);
    NR(true, false, false);
#undef NR
}
}  // namespace

extern "C" int anigpu_assemble_noalloc(anigpu_handle h, int tensor_kind, const double* D, const double* f,
                                       double f_const, int order, int precision, void* vals, double* rhs,
                                       double drop_val) {
    if (!h) return ANIGPU_ERR_ARG;
    (void)cudaGetLastError();
    cudaSetDevice(h->device);
    if (h->space < 0) return set_err(h, ANIGPU_ERR_STATE, "anigpu_problem_setup not called");
    if (h->space == ANIGPU_VEC3_P2) return set_err(h, ANIGPU_ERR_UNSUPPORTED, "vector assembly not built yet");
    if (tensor_kind != ANIGPU_TENSOR_NULL && tensor_kind != ANIGPU_TENSOR_CONST_SCALAR &&
        tensor_kind != ANIGPU_TENSOR_TET_SCALAR && tensor_kind != ANIGPU_TENSOR_TET_SYM)
        return set_err(h, ANIGPU_ERR_UNSUPPORTED, "assembly tensor kind must be NULL, CONST_SCALAR, TET_SCALAR or TET_SYM");
    if (tensor_kind != ANIGPU_TENSOR_NULL && !D) return set_err(h, ANIGPU_ERR_ARG, "tensor data is NULL");
    if (!vals || !rhs) return set_err(h, ANIGPU_ERR_ARG, "NULL output");
    if (precision != ANIGPU_F32 && precision != ANIGPU_F64) return set_err(h, ANIGPU_ERR_ARG, "precision");
    const size_t rsz = precision == ANIGPU_F32 ? 4 : 8;
    const size_t need = (size_t)h->nt * 8 * rsz;
    if (need > kNoallocScratchBytes - kNoallocTableBytes)
        return set_err(h, ANIGPU_ERR_ARG,
                       "anigpu_assemble_noalloc: mesh too large for the fixed scratch (" +
                           std::to_string(h->nt) + " tets need " + std::to_string(need) + " bytes, limit " +
                           std::to_string(kNoallocScratchBytes - kNoallocTableBytes) +
                           " bytes: 524288 tets in FP32, 262144 in FP64)");
    unsigned char* scratch = nullptr;
    int rc = noalloc_scratch(h, &scratch);
    if (rc) return rc;
    // reference tables: computed on the host into fixed storage, copied to the array's head
    double T64[10 * 10 * 8 + 10];
    int nf = 0;
    if (!noalloc_tables(h->space, order, T64, &nf) || nf != h->nloc_s)
        return set_err(h, ANIGPU_ERR_UNSUPPORTED, "unsupported space/order");
    const size_t ntab = (size_t)nf * nf * 8 + nf;
    static thread_local float T32[10 * 10 * 8 + 10];
    static thread_local double T64s[10 * 10 * 8 + 10];
    if (precision == ANIGPU_F32) {
        for (size_t k = 0; k < ntab; ++k) T32[k] = (float)T64[k];
        ANI_CUDA(h, cudaMemcpyAsync(scratch, T32, ntab * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    } else {
        for (size_t k = 0; k < ntab; ++k) T64s[k] = T64[k];
        ANI_CUDA(h, cudaMemcpyAsync(scratch, T64s, ntab * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    }
    void* tetK = scratch + kNoallocTableBytes;
    if (precision == ANIGPU_F32)
        tet_prepare_f32_kernel<<<grid_for(h->nt, 256), 256, 0, h->stream>>>(
            h->nt, h->xyz, h->xyz2, h->tets, tensor_kind, D, f, f_const, (float*)tetK, h->d_status);
    else
        tet_prepare_f64_kernel<<<grid_for(h->nt, 256), 256, 0, h->stream>>>(
            h->nt, h->xyz, h->tets, tensor_kind, D, f, f_const, (double*)tetK, h->d_status);
    ANI_LAUNCHED(h);
    RowParams p;
    p.inc_ptr = h->inc_ptr;
    p.recs = h->recs;
    p.rowptr = h->rowptr_s;
    p.dir_mask = h->dir_mask;
    p.dir_bc = h->dir_bc;
    p.edofs = h->edofs;
    p.drop = drop_val;
    for (int rg = 0; rg < 2; ++rg) {
        p.row_begin = h->row_range[rg];
        p.nrows = h->row_range[rg + 1];
        p.cap = h->row_range_cap[rg];
        if (p.nrows <= p.row_begin) continue;
        if (h->nloc_s == 10)
            rc = precision == ANIGPU_F32
                     ? noalloc_rows_dispatch<float, 10>(h, p, (const float*)scratch, (const float*)tetK, (float*)vals, rhs)
                     : noalloc_rows_dispatch<double, 10>(h, p, (const double*)scratch, (const double*)tetK,
                                                         (double*)vals, rhs);
        else
            rc = precision == ANIGPU_F32
                     ? noalloc_rows_dispatch<float, 4>(h, p, (const float*)scratch, (const float*)tetK, (float*)vals, rhs)
                     : noalloc_rows_dispatch<double, 4>(h, p, (const double*)scratch, (const double*)tetK,
                                                        (double*)vals, rhs);
        if (rc) return rc;
    }
    int st = 0;
    ANI_CUDA(h, cudaMemcpyAsync(&st, h->d_status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    ANI_CUDA(h, cudaStreamSynchronize(h->stream));
    if (st) {
        ANI_CUDA(h, cudaMemsetAsync(h->d_status, 0, sizeof(int), h->stream));
        return set_err(h, st, "non-finite value in assembly (AssemblerT status -1)");
    }
    return ANIGPU_OK;
}
