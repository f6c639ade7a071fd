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
// quadrature rule the caller asked for ("table" form, any quadrature order).
//
// When the quadrature integrates the element integrals exactly (P1: any order; P2: order
// >= 2, whose rules are exact for the degree-2 integrands of GRAD.GRAD and of the P0 x P2
// right-hand side) the "Gram" form is used instead: with G_pq = |T| grad(l_p)^T D grad(l_q)
// (the 4x4 Gram matrix of the barycentric gradients) and the barycentric moments
// E[l_p] = 1/4, E[l_p^2] = 1/10, E[l_p l_q] = 1/20, one row of the P2 element matrix in the
// canonical column order of its row (canon_local) is a fixed combination of 4 (vertex row)
// or 7 (edge row) entries of G, e.g. for vertex row i with others o1 < o2 < o3
//     A(i,i) = 0.6 G_ii,  A(i,o) = -0.2 G_io,  A(i, edge(i,o)) = 0.6 G_io - 0.2 G_ii,
//     A(i, edge(o,o')) = -0.2 (G_io + G_io')
// so the gather needs no tables.  The values agree with the quadrature sums of fem3Dtet to
// rounding (FP64: ~1e-15 relative).
//
// Phase 1 computes K or G (and f|T|) once per tet; phase 2 is a row gather: every CSR row
// is owned by one lane, which walks the row's incident tets in ascending tet order, computes
// that tet's row of A and adds it into a shared-memory copy of the row at the offsets held
// by the scatter record.  Each value is therefore summed in the same order as the
// reference's serial cell loop, without atomics, and written to HBM once, coalesced.
#include <mutex>
#include <type_traits>

#include "anigpu_internal.h"
#include "fp_convert.cuh"
#include "quad_tables.h"

namespace {


// Programmatic dependent launch between the phases of one assembly: the per-tet kernel lets the
// gathers launch once each of its blocks has stored its blocks, and a gather waits for the
// per-tet kernel's completion (and memory) only before its first per-tet block load, so its
// set-up (zeroing, row pointers, records) overlaps the per-tet kernel's last wave.  Both are no-ops
// for launches without a programmatic dependency.
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// ---------------------------------------------------------------- phase 1
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

// Gram form: G = |T| g^T D g for the four barycentric gradients g_0..g_3 (g_{a+1} = row a of
// PSI, g_0 = -(g_1 + g_2 + g_3), poly_1.h).  Stored: the six off-diagonal entries by local
// edge, G01 G02 G03 G12 G13 G23, then f|T| and 0 (8 values, two 16-byte loads per tet).  The
// diagonal is not stored: the gradients sum to zero, so G_pp = -sum_{q != p} G_pq, which
// the row gather forms from the off-diagonal entries of the row it is computing anyway.
template <typename R>
__device__ __forceinline__ void gram_from_psi(const R* PSI, const R* d, R mes, R* out) {
    R g[4][3], Dg[4][3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        g[a + 1][0] = PSI[a];
        g[a + 1][1] = PSI[a + 3];
        g[a + 1][2] = PSI[a + 6];
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) g[0][c] = -(g[1][c] + g[2][c] + g[3][c]);
#pragma unroll
    for (int p = 0; p < 4; ++p) {
        Dg[p][0] = d[0] * g[p][0] + d[1] * g[p][1] + d[2] * g[p][2];
        Dg[p][1] = d[1] * g[p][0] + d[3] * g[p][1] + d[4] * g[p][2];
        Dg[p][2] = d[2] * g[p][0] + d[4] * g[p][1] + d[5] * g[p][2];
    }
    auto dot = [&](int p, int q) { return mes * (g[p][0] * Dg[q][0] + g[p][1] * Dg[q][1] + g[p][2] * Dg[q][2]); };
    out[0] = dot(0, 1);
    out[1] = dot(0, 2);
    out[2] = dot(0, 3);
    out[3] = dot(1, 2);
    out[4] = dot(1, 3);
    out[5] = dot(2, 3);
}

__global__ void tet_gram_f64_kernel(int64_t nt, const double* __restrict__ xyz, const int32_t* __restrict__ tets,
                                    int kind, const double* __restrict__ D, const double* __restrict__ f,
                                    double f_const, double* __restrict__ out, int* __restrict__ status) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const int4 v = reinterpret_cast<const int4*>(tets)[t];
    double e[9];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double x0 = xyz[3 * (int64_t)v.x + k];
        e[k + 0] = xyz[3 * (int64_t)v.y + k] - x0;
        e[k + 3] = xyz[3 * (int64_t)v.z + k] - x0;
        e[k + 6] = xyz[3 * (int64_t)v.w + k] - x0;
    }
    double d[6], PSI[9], G[8];
    load_sym(kind, D, t, d);
    const double det = inverse3(e, PSI);
    const double mes = fabs(det) / 6.0;
    gram_from_psi(PSI, d, mes, G);
    G[6] = (f ? f[t] : f_const) * mes;
    G[7] = 0;
    bool bad = !(det != 0.0);
#pragma unroll
    for (int k = 0; k < 7; ++k) bad |= !isfinite(G[k]);
    if (bad) atomicExch(status, ANIGPU_ERR_NONFINITE);
    double2* o = reinterpret_cast<double2*>(out + 8 * t);
#pragma unroll
    for (int q = 0; q < 4; ++q) o[q] = make_double2(G[2 * q], G[2 * q + 1]);
    pdl_launch_dependents();
}

// six 256-thread blocks per SM (40 registers): the loads of more tets in flight; the few values
// this moves to local memory belong to the FP64 redo of badly shaped tets
#ifndef TET_GRAM_MINB
#define TET_GRAM_MINB 6
#endif
#define TET_GRAM_BOUNDS __launch_bounds__(256, TET_GRAM_MINB)
__global__ void TET_GRAM_BOUNDS tet_gram_f32_kernel(int64_t nt, const double* __restrict__ xyz, const float2* __restrict__ xyz2,
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
    float PSI[9], G[8];
    const float det = inverse3(e, PSI);
    const float l0 = e[0] * e[0] + e[1] * e[1] + e[2] * e[2];
    const float l1 = e[3] * e[3] + e[4] * e[4] + e[5] * e[5];
    const float l2 = e[6] * e[6] + e[7] * e[7] + e[8] * e[8];
    float mes;
    if (det * det > 0.0025f * l0 * l1 * l2) {
        mes = fabsf(det) * (1.0f / 6.0f);
        gram_from_psi(PSI, d, mes, G);
    } else {
        // badly shaped (or degenerate) tet: Jacobian, inverse and Gram matrix in FP64
        double ed[9], P64[9], dd[6], G64[6];
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
        gram_from_psi(P64, dd, mes64, G64);
#pragma unroll
        for (int k = 0; k < 6; ++k) G[k] = (float)G64[k];
        mes = (float)mes64;
        if (!(det64 != 0.0)) atomicExch(status, ANIGPU_ERR_NONFINITE);
    }
    G[6] = fv * mes;
    G[7] = 0.f;
    bool bad = false;
#pragma unroll
    for (int k = 0; k < 7; ++k) bad |= !isfinite(G[k]);
    if (bad) atomicExch(status, ANIGPU_ERR_NONFINITE);
    float4* o = reinterpret_cast<float4*>(out + 8 * t);
    o[0] = make_float4(G[0], G[1], G[2], G[3]);
    o[1] = make_float4(G[4], G[5], G[6], G[7]);
    pdl_launch_dependents();
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
    const int64_t* dir_cptr;  // Dirichlet columns of each non-Dirichlet row ...
    const uint16_t* dir_coff;  // ... as offsets within the row
    int cap;  // row buffer capacity (>= longest row)
    int vec_ok;  // the value array is 16-byte aligned: vector stores
    double drop;
    const int32_t* vcol;  // vector template columns (non-zero boundary values of the vector path)
    int bcnz;             // vector path: non-zero boundary values
    int64_t wstride = 0;  // lane-interleaved records: slots per warp when uniform, else 0 (per-warp offsets)
};


// per-tet block of N = 8 values (32-byte aligned: 32 bytes FP32, 64 bytes FP64), read with
// 256-bit loads through the read-only path: one L1 wavefront per lane and block (FP32)
template <typename Real, int N>
struct KVec {
    Real v[N];
    __device__ __forceinline__ void load(const Real* p) {
        if (N == 8 && sizeof(Real) == 4) {
            float* f = reinterpret_cast<float*>(v);
            asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                : "=f"(f[0]), "=f"(f[1]), "=f"(f[2]), "=f"(f[3]), "=f"(f[4]), "=f"(f[5]), "=f"(f[6]), "=f"(f[7])
                : "l"(p));
        } else if (N == 8) {
            double* d = reinterpret_cast<double*>(v);
            asm("ld.global.nc.v4.f64 {%0,%1,%2,%3}, [%4];"
                : "=d"(d[0]), "=d"(d[1]), "=d"(d[2]), "=d"(d[3])
                : "l"(p));
            asm("ld.global.nc.v4.f64 {%0,%1,%2,%3}, [%4];"
                : "=d"(d[4]), "=d"(d[5]), "=d"(d[6]), "=d"(d[7])
                : "l"(p + 4));
        } else if (sizeof(Real) == 4) {
#pragma unroll
            for (int q = 0; q < N / 4; ++q) {
                const float4 w = reinterpret_cast<const float4*>(p)[q];
                v[4 * q] = w.x;
                v[4 * q + 1] = w.y;
                v[4 * q + 2] = w.z;
                v[4 * q + 3] = w.w;
            }
        } else {
#pragma unroll
            for (int q = 0; q < N / 2; ++q) {
                const double2 w = reinterpret_cast<const double2*>(p)[q];
                v[2 * q] = w.x;
                v[2 * q + 1] = w.y;
            }
        }
    }
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int q = 0; q < N; ++q) v[q] = Real(0);
    }
};

// Gram-form element rows in canonical column order (FORM 1: vertex rows, FORM 2: P2 edge
// rows); G = K.v: G01 G02 G03 G12 G13 G23, f|T|.  The diagonal entries come from the
// off-diagonal ones of the same row (G_pp = -sum_{q != p} G_pq).  Returns f|T| E[phi_i].
template <typename Real, int NLOC, int FORM>
__device__ __forceinline__ Real gram_row(const Real* G, int i, Real* a) {
    const Real e0 = G[0], e1 = G[1], e2 = G[2], e3 = G[3], e4 = G[4], e5 = G[5];
    if (FORM == 1) {
        // vertex i and the others o1 < o2 < o3: G_io1, G_io2, G_io3 and G_ii
        const Real g1 = i <= 1 ? e0 : i == 2 ? e1 : e2;
        const Real g2 = i == 0 ? e1 : i <= 2 ? e3 : e4;
        const Real g3 = i == 0 ? e2 : i == 1 ? e4 : e5;
        const Real gii = -((g1 + g2) + g3);
        if (NLOC == 4) {
            a[0] = gii;
            a[1] = g1;
            a[2] = g2;
            a[3] = g3;
            return Real(0.25) * G[6];
        } else {
            const Real m2 = Real(-0.2), p6 = Real(0.6);
            a[0] = p6 * gii;
            a[1] = m2 * g1;
            a[2] = m2 * g2;
            a[3] = m2 * g3;
            const Real t = m2 * gii;
            a[4] = fma(p6, g1, t);
            a[5] = fma(p6, g2, t);
            a[6] = fma(p6, g3, t);
            a[7] = m2 * (g1 + g2);
            a[8] = m2 * (g1 + g3);
            a[9] = m2 * (g2 + g3);
            return Real(-0.05) * G[6];
        }
    } else {
        // edge k = (a,b) with the other vertices c < d
        const int k = i - 4;
        const Real gab = k == 0 ? e0 : k == 1 ? e1 : k == 2 ? e2 : k == 3 ? e3 : k == 4 ? e4 : e5;
        const Real gac = (k == 0 || k == 5) ? e1 : e0;
        const Real gad = k <= 1 ? e2 : k == 2 ? e1 : k == 3 ? e4 : e3;
        const Real gbc = k <= 1 ? e3 : k == 2 ? e4 : k == 3 ? e1 : e2;
        const Real gbd = (k == 0 || k == 5) ? e4 : e5;
        const Real gaa = -((gab + gac) + gad);
        const Real gbb = -((gab + gbc) + gbd);
        const Real m2 = Real(-0.2), p6 = Real(0.6), p8 = Real(0.8), p16 = Real(1.6);
        a[0] = fma(m2, gaa, p6 * gab);
        a[1] = fma(m2, gbb, p6 * gab);
        a[2] = m2 * (gac + gbc);
        a[3] = m2 * (gad + gbd);
        a[4] = p16 * (gaa + gbb + gab);
        const Real sa = gaa + gab, sb = gab + gbb;
        a[5] = fma(p8, sa + gac, p16 * gbc);
        a[6] = fma(p8, sa + gad, p16 * gbd);
        a[7] = fma(p8, sb + gbc, p16 * gac);
        a[8] = fma(p8, sb + gbd, p16 * gad);
        a[9] = p8 * ((gac + gad) + (gbc + gbd));
        return Real(0.2) * G[6];
    }
}

// Row gather.  One lane owns one CSR row.  It walks the row's incident tets in ascending
// tet order (the order of the reference's serial cell loop), computes the tet's element
// row A_t(i, .) in canonical column order in registers and adds it into the row's values in
// shared memory at the offsets held by the scatter record.  The 32 rows of a warp are
// consecutive, so their values are one contiguous range of the CSR value array; the warp
// keeps that range in shared memory in CSR order (lane l's row at rowptr[row] - rowptr[row0])
// and writes it back with one contiguous, vectorised copy.  Loads of later incidences (tet
// ids, per-tet blocks, records) are in flight while one is computed.  A Dirichlet row does not walk
// its incidences: applyDir makes each of its element rows e_i, so the row is zero except the
// diagonal, which is the number of incident tets.  No atomics: every CSR value is produced by
// exactly one lane with a fixed summation order.
template <typename Real, int NLOC>
struct RowTab {
    // per-i stride padded so that lanes holding different i read distinct banks
    static constexpr int TS = NLOC * 8 + (16 / (int)sizeof(Real));
    static constexpr int SIZE = NLOC * TS + NLOC;  // then m[i]
};

// shared memory of one row-gather block: tables (table form), then per warp the value
// range (32 rows of at most cap values, shifted by up to one 16-byte vector so that shared
// and global addresses have the same alignment) and, with a touched map, its bytes
template <typename Real, int NLOC, int FORM, bool TOUCH>
struct RowSmem {
    static constexpr int VEC = 16 / (int)sizeof(Real);
    __host__ __device__ static size_t tab_bytes() { return FORM == 0 ? ((sizeof(Real) * RowTab<Real, NLOC>::SIZE + 15) / 16) * 16 : 0; }
    __host__ __device__ static size_t chunk_bytes(int cap) { return (((size_t)32 * cap + VEC) * sizeof(Real) + 15) / 16 * 16; }
    __host__ __device__ static size_t touch_bytes(int cap) { return TOUCH ? ((size_t)32 * cap + 16 + 15) / 16 * 16 : 0; }
    __host__ __device__ static size_t warp_bytes(int cap) { return chunk_bytes(cap) + touch_bytes(cap); }
    __host__ __device__ static size_t total(int cap, int warps) { return tab_bytes() + warp_bytes(cap) * warps; }
};

// prefetch depths of the row gather (per-tet blocks, records)
#ifndef ROW_KD
#define ROW_KD 3
#endif
#ifndef ROW_RD
#define ROW_RD 5
#endif
#ifndef ROW_UNROLL
#define ROW_UNROLL 4
#endif
#ifndef ROW_RED
#define ROW_RED 0
#endif
#ifdef ROW_MINB
#define ROW_BOUNDS __launch_bounds__(64, ROW_MINB)
#else
#define ROW_BOUNDS __launch_bounds__(64)
#endif
constexpr int kRowUnroll = ROW_UNROLL;

// records k and k+1 (k even; the record array has one record of padding at its end)
__device__ __forceinline__ void load_rec_pair(const ScatterRec* p, ScatterRec& lo, ScatterRec& hi) {
    asm("ld.global.nc.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=r"(lo.tet), "=r"(lo.meta), "=r"(lo.off03), "=r"(lo.off47), "=r"(hi.tet), "=r"(hi.meta), "=r"(hi.off03),
          "=r"(hi.off47)
        : "l"(p));
}

// byte c & 3 of w, zero-extended
__device__ __forceinline__ uint32_t byte_of(uint32_t w, int c) { return __byte_perm(w, 0u, 0x4440u + (uint32_t)(c & 3)); }

// contiguous write-out of a warp's value range (shared index k <-> vals[cbase + k], same 16-byte
// alignment): single values up to the first aligned vector, vectors over the middle, single values
// at the end.  Returns a sum of value * 0 over the values written: non-finite iff one of them is.
template <typename Real>
__device__ __forceinline__ Real write_out_range(const Real* sC, int shift, int clen, int64_t cbase,
                                                Real* __restrict__ vals, int vec_ok, int lane) {
    constexpr int VEC = 16 / (int)sizeof(Real);
    Real fin = Real(0);
    const int head = shift == 0 ? 0 : (VEC - shift < clen ? VEC - shift : clen);
    if (lane < head) {
        const Real v = sC[lane];
        fin = fma(v, Real(0), fin);
        vals[cbase + lane] = v;
    }
    const int nbody = (clen - head) / VEC;
    using V = typename std::conditional<sizeof(Real) == 4, float4, double2>::type;
    const V* sv = reinterpret_cast<const V*>(sC + head);
    V* gv = reinterpret_cast<V*>(vals + cbase + head);
    for (int k = lane; k < (vec_ok ? nbody : 0); k += 32) {
        const V v = sv[k];
        if (sizeof(Real) == 4) {
            const float4 f = *reinterpret_cast<const float4*>(&v);
            fin = fma(Real(f.x), Real(0), fin);
            fin = fma(Real(f.y), Real(0), fin);
            fin = fma(Real(f.z), Real(0), fin);
            fin = fma(Real(f.w), Real(0), fin);
        } else {
            const double2 f = *reinterpret_cast<const double2*>(&v);
            fin = fma(Real(f.x), Real(0), fin);
            fin = fma(Real(f.y), Real(0), fin);
        }
        gv[k] = v;
    }
    for (int k = (vec_ok ? head + nbody * VEC : head) + lane; k < clen; k += 32) {
        const Real v = sC[k];
        fin = fma(v, Real(0), fin);
        vals[cbase + k] = v;
    }
    return fin;
}

// FORM 0: table form (any row kind); FORM 1: Gram form, vertex rows; FORM 2: Gram form, P2 edge rows
template <typename Real, int NLOC, int FORM, bool DIR, bool BCNZ, bool TOUCH, bool DROPCHK>
__global__ void ROW_BOUNDS row_gather_kernel(RowParams p, const Real* __restrict__ tables,
                                                        const Real* __restrict__ tetK, Real* __restrict__ vals,
                                                        double* __restrict__ rhs, uint8_t* __restrict__ touched_out,
                                                        int* __restrict__ status) {
    using Tab = RowTab<Real, NLOC>;
    using Sm = RowSmem<Real, NLOC, FORM, TOUCH>;
    constexpr int KS = 8;  // values per tet block (K or G, then f|T|)
    // Dirichlet columns: masked per element value where the masked value is needed (the
    // rhs update of a non-zero boundary value, the touched map); otherwise every value is
    // added and the Dirichlet columns of the row are set to zero at the end
    constexpr bool MASKCOLS = DIR && (BCNZ || TOUCH);
    constexpr int VEC = Sm::VEC;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    Real* sT = reinterpret_cast<Real*>(smem_raw);
    if (FORM == 0) {
        // host layout [i][c][8] -> padded stride TS per i
        for (int k = threadIdx.x; k < NLOC * NLOC * 8; k += blockDim.x) {
            const int i = k / (NLOC * 8), rem = k - i * NLOC * 8;
            sT[i * Tab::TS + rem] = tables[k];
        }
        for (int k = threadIdx.x; k < NLOC; k += blockDim.x) sT[NLOC * Tab::TS + k] = tables[NLOC * NLOC * 8 + k];
        __syncthreads();
    }
    const Real* sM = sT + NLOC * Tab::TS;
    const int64_t row0 = p.row_begin + ((int64_t)blockIdx.x * nwarps + warp) * 32;
    if (row0 >= p.nrows) return;  // warp-uniform; no block-wide barrier follows
    const int64_t rend = row0 + 32 < p.nrows ? row0 + 32 : p.nrows;
    const int64_t cbase = p.rowptr[row0];
    const int clen = (int)(p.rowptr[rend] - cbase);
    const int shift = (int)(cbase & (VEC - 1));  // shared index s <-> global cbase + s, same alignment
    unsigned char* wbase = smem_raw + Sm::tab_bytes() + Sm::warp_bytes(p.cap) * warp;
    Real* sC = reinterpret_cast<Real*>(wbase) + shift;
    uint8_t* sTouch = wbase + Sm::chunk_bytes(p.cap) + shift;
    // zero [0, shift + clen) of this warp's range, 16 bytes per store
    {
        const int nvec = (shift + clen + VEC - 1) / VEC;
        int4* z = reinterpret_cast<int4*>(wbase);
        for (int k = lane; k < nvec; k += 32) z[k] = make_int4(0, 0, 0, 0);
        if (TOUCH) {
            int4* zt = reinterpret_cast<int4*>(wbase + Sm::chunk_bytes(p.cap));
            for (int k = lane; k < (shift + clen + 15) / 16; k += 32) zt[k] = make_int4(0, 0, 0, 0);
        }
    }
    const int64_t row = row0 + lane;
    const bool valid = row < p.nrows;
    int64_t ib = 0;
    int deg = 0, base = 0;
    bool isdir = false;
    if (valid) {
        ib = p.inc_ptr[row];
        deg = (int)(p.inc_ptr[row + 1] - ib);
        base = (int)(p.rowptr[row] - cbase);
        if (DIR) isdir = p.dir_mask[row] != 0;
    }
    __syncwarp();
    Real* myRow = sC + base;
    uint8_t* myTouch = sTouch + base;
    const Real drop = Real(p.drop);
    Real racc = Real(0);
    const int nloop = isdir ? 0 : deg;
    // software pipeline over the incidences, indices clamped to the last incidence so that the
    // loop body has no branches: per-tet blocks KD incidences ahead, records RD ahead, so that
    // the record that addresses a block arrived RD - KD iterations before the block is requested
    constexpr int KD = ROW_KD, RD = ROW_RD;
    static_assert(RD > KD, "records must run ahead of the blocks they address");
    KVec<Real, KS> Kq[KD];
    ScatterRec Rq[RD];
    const int last = nloop - 1;
#pragma unroll
    for (int j = 0; j < KD; ++j) Kq[j].zero();
#pragma unroll
    for (int j = 0; j < RD; ++j) Rq[j] = ScatterRec{0u, 0u, 0u, 0u};
    // records ahead of the queue are read in aligned pairs: when the next index is even the
    // pair is loaded and its second record kept for the following iteration
    ScatterRec pend = ScatterRec{0u, 0u, 0u, 0u};
    // loads past the row's last incidence are skipped (their values are never used)
#pragma unroll
    for (int j = 0; j < RD; ++j)
        if (j <= last) Rq[j] = p.recs[ib + j];
#pragma unroll
    for (int j = 0; j < KD; ++j)
        if (j <= last) Kq[j].load(tetK + KS * (int64_t)Rq[j].tet);
    if (RD <= last && ((ib + RD) & 1)) pend = p.recs[ib + RD];
#pragma unroll kRowUnroll
    for (int k = 0; k < nloop; ++k) {
        KVec<Real, KS> Kn;
        if (k + KD <= last) Kn.load(tetK + KS * (int64_t)Rq[KD].tet);
        const int64_t ridx = ib + k + RD;
        ScatterRec Rn = pend;
        if (k + RD <= last && !(ridx & 1)) load_rec_pair(p.recs + ridx, Rn, pend);
        const ScatterRec r0 = Rq[0];
        const KVec<Real, KS>& K0 = Kq[0];
        const int i = r0.meta & 15;
        const uint32_t dm = MASKCOLS ? (r0.meta >> 4) & 0x3ffu : 0u;
        Real F;
        Real a[NLOC];
        if (FORM != 0) {
            F = gram_row<Real, NLOC, FORM>(K0.v, i, a);
        } else {
            const Real* T = sT + i * Tab::TS;
            const Real k0 = K0.v[0], k1 = K0.v[1], k2 = K0.v[2], k3 = K0.v[3], k4 = K0.v[4], k5 = K0.v[5];
            F = K0.v[6] * sM[i];
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
                a[j] = v;
            }
        }
        int o[NLOC];
#pragma unroll
        for (int j = 0; j < NLOC; ++j) {
            const uint32_t w = j < 4 ? r0.off03 : (j < 8 ? r0.off47 : (r0.meta >> 16));
            o[j] = (int)byte_of(w, j);
            const Real v = a[j];
            const bool colDir = MASKCOLS && ((dm >> j) & 1u);
            if (BCNZ && colDir)  // applyDir on a Dirichlet column (dc_on_dof.h:39-45), canonical order
                F -= v * Real(p.dir_bc[p.edofs[(int64_t)r0.tet * NLOC + canon_local(NLOC, i, j)]]);
            // the drop rule |a| > drop_val (assembler.inl:416-418).  Without a touched map and
            // with a drop value that rounds to zero in FP32 the rule only skips exact zeros,
            // which cannot change a sum: that variant is compiled without the test.
            const bool add = !colDir && (!DROPCHK || fabs(v) > drop);
            a[j] = add ? v : Real(0);
            if (TOUCH) myTouch[o[j]] |= (uint8_t)(add ? 1 : 0);
        }
        // the NLOC slots of one element row are distinct columns: independent updates; every
        // slot of the row belongs to this lane alone, so the order of its additions is fixed
        if (ROW_RED && sizeof(Real) == 4) {
#pragma unroll
            for (int j = 0; j < NLOC; ++j) atomicAdd(&myRow[o[j]], a[j]);
        } else {
            Real cur[NLOC];
#pragma unroll
            for (int j = 0; j < NLOC; ++j) cur[j] = myRow[o[j]];
#pragma unroll
            for (int j = 0; j < NLOC; ++j) myRow[o[j]] = cur[j] + a[j];
        }
        racc += F;
#pragma unroll
        for (int j = 0; j + 1 < KD; ++j) Kq[j] = Kq[j + 1];
        Kq[KD - 1] = Kn;
#pragma unroll
        for (int j = 0; j + 1 < RD; ++j) Rq[j] = Rq[j + 1];
        Rq[RD - 1] = Rn;
    }
    bool bad = false;
    if (valid) {
        double F;
        if (DIR && isdir) {
            // diagonal = number of incident tets (a sum of ones, exact); rhs = sum of bc over them
            if (deg > 0) {
                const ScatterRec rd = p.recs[ib];
                const int dc = canon_diag(NLOC, rd.meta & 15);
                const uint32_t w = dc < 4 ? rd.off03 : rd.off47;
                const int od = (int)byte_of(w, dc);
                myRow[od] = Real(deg);
                if (TOUCH) myTouch[od] = 1;
            }
            const double bcr = p.dir_bc[row];
            F = 0;
            for (int q = 0; q < deg; ++q) F += bcr;
        } else {
            F = (double)racc;
            if (DIR && !MASKCOLS)
                for (int64_t q = p.dir_cptr[row]; q < p.dir_cptr[row + 1]; ++q) myRow[p.dir_coff[q]] = Real(0);
        }
        bad |= !isfinite(F);
        rhs[row] = F;
    }
    __syncwarp();
    Real fin = write_out_range<Real>(sC, shift, clen, cbase, vals, p.vec_ok, lane);
    if (TOUCH)
        for (int k = lane; k < clen; k += 32) touched_out[cbase + k] = sTouch[k];
    bad |= !isfinite(fin);
    if (bad) atomicExch(status, ANIGPU_ERR_NONFINITE);
}

// ---------------------------------------------------------------- P2 edge rows by rings
// The tets around an edge (A, B) form a ring (a path for a boundary edge): consecutive tets
// share a face (A, B, v).  Of the columns of the edge row, A, B and the edge itself collect every
// tet of the ring; the ring vertex v and the edges (A, v), (B, v) collect the two tets on the face
// (A, B, v) (one at the end of a path); the edge (P, N) opposite to (A, B) in a tet collects that
// tet alone.  Walking the ring in order, a lane keeps A, B and the edge in registers and carries
// the three columns of the face it is on from one tet to the next, so every value of the row is
// written to shared memory exactly once, with no read-modify-write and no zeroing pass over the
// columns the walk covers.  Each value is still the sum of its tets' contributions in a fixed
// order (the ring order from the smallest tet id).
//
// Ring record (8 bytes), one per (edge row, incident tet), in ring order:
//   x: tet id (bits 0-26), local edge k of (A, B) in the tet (27-29), A is the tet's local b (30),
//      P is the tet's local d (31)  [local a < b: the edge's vertices, c < d: the other two]
//   y: offsets within the row of N, (A, N), (B, N), (P, N), 8 bits each
// Header (one per row, before its records):
//   x: offsets of A, B, the edge (8 bits each), bit 24: closed ring
//   y: offsets of the first face's vertex P0, (A, P0), (B, P0)
// For warp w of the edge range the slots are ring[woff[w] + 32 s + lane]: the header at s = 0,
// record j at s = j + 1, so the 32 lanes read 256 contiguous bytes per step.
constexpr uint32_t kRingTetMask = (1u << 27) - 1;
constexpr int kRingMax = 32;  // incident tets of an edge that the ring build takes

// the gathers of one assembly on the per-tet kernel's stream with programmatic dependencies (1) or
// on two streams (0)
#ifndef ASM_SEQ
#define ASM_SEQ 1
#endif
// the plain edge walk writes every column of its row (checked when the rings are built), so its
// row buffer is not zeroed first; Dirichlet rows (no walk) zero their own row (1)
#ifndef RING_NOZERO
#define RING_NOZERO 1
#endif
// the lane-interleaved layouts end in kRecPad slots of padding, so that a walk's first records
// are loaded without waiting for the row's incidence count (1): slots past the lane's own records
// belong to other lanes or to the padding and are never used; or only the lane's own (0)
#ifndef REC_AHEAD
#define REC_AHEAD 1
#endif
constexpr int64_t kRecPad = 32 * 16;  // prefetch depths below 16

// with ASM_SEQ and P2: the vertex rows behind the per-tet kernel and the edge rows concurrently on
// the side stream (1), or edge rows then vertex rows behind the per-tet kernel (0)
#ifndef ASM_SPLIT
#define ASM_SPLIT 1
#endif

// prefetch depths of the ring gather (per-tet blocks, records)
#ifndef RING_KD
#define RING_KD 2
#endif
#ifndef RING_RD
#define RING_RD 4
#endif
#ifndef RING_U
#define RING_U 4
#endif
// FP32: sixteen 64-thread blocks per SM (64 registers; a few bytes of spill) for more loads in
// flight; FP64 keeps its registers
#ifndef RING_MINB
#define RING_MINB 16
#endif
#define RING_BOUNDS __launch_bounds__(64, sizeof(Real) == 4 ? RING_MINB : 1)

template <typename Real, bool DIR, bool DROPCHK>
__global__ void RING_BOUNDS edge_ring_kernel(RowParams p, const uint2* __restrict__ ring,
                                            const int64_t* __restrict__ woff, const Real* __restrict__ tetK,
                                            Real* __restrict__ vals, double* __restrict__ rhs,
                                            int* __restrict__ status) {
    using Sm = RowSmem<Real, 10, 2, false>;
    constexpr int KS = 8;
    constexpr int VEC = Sm::VEC;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    const int64_t wg = (int64_t)blockIdx.x * nwarps + warp;
    const int64_t row0 = p.row_begin + wg * 32;
    if (row0 >= p.nrows) return;  // warp-uniform; no block-wide barrier follows
    const int64_t rend = row0 + 32 < p.nrows ? row0 + 32 : p.nrows;
    const int64_t cbase = p.rowptr[row0];
    const int clen = (int)(p.rowptr[rend] - cbase);
    const int shift = (int)(cbase & (VEC - 1));
    unsigned char* wbase = smem_raw + Sm::warp_bytes(p.cap) * warp;
    Real* sC = reinterpret_cast<Real*>(wbase) + shift;
    if (!RING_NOZERO) {
        const int nvec = (shift + clen + VEC - 1) / VEC;
        int4* z = reinterpret_cast<int4*>(wbase);
        for (int k = lane; k < nvec; k += 32) z[k] = make_int4(0, 0, 0, 0);
    }
    const int64_t row = row0 + lane;
    const bool valid = row < p.nrows;
    const uint2* rr = ring + (p.wstride > 0 ? wg * p.wstride : woff[wg]) + lane;
    int deg = 0, base = 0;
    bool isdir = false;
    uint2 hd = make_uint2(0u, 0u);
    if (valid) {
        deg = (int)(p.inc_ptr[row + 1] - p.inc_ptr[row]);
        base = (int)(p.rowptr[row] - cbase);
        if (DIR) isdir = p.dir_mask[row] != 0;
        hd = rr[0];
    }
    __syncwarp();
    Real* myRow = sC + base;
    const Real drop = Real(p.drop);
    const int nloop = isdir ? 0 : deg;
    const int last = nloop - 1;
    constexpr int KD = RING_KD, RD = RING_RD;
    static_assert(RD > KD, "records must run ahead of the blocks they address");
    static_assert(RD < 16, "the first records may reach RD slots past the lane's own (kRecPad)");
    KVec<Real, KS> Kq[KD];
    uint2 Rq[RD];
#pragma unroll
    for (int j = 0; j < KD; ++j) Kq[j].zero();
#pragma unroll
    for (int j = 0; j < RD; ++j) Rq[j] = make_uint2(0u, 0u);
#pragma unroll
    for (int j = 0; j < RD; ++j)
        if (REC_AHEAD || j <= last) Rq[j] = rr[32 * (j + 1)];
    pdl_wait();  // the per-tet blocks of this assembly
#pragma unroll
    for (int j = 0; j < KD; ++j)
        if (j <= last) Kq[j].load(tetK + KS * (int64_t)(Rq[j].x & kRingTetMask));
    const bool closed = (hd.x >> 24) & 1u;
    Real cP = Real(0), cAP = Real(0), cBP = Real(0);  // the face carried to the next tet
    Real fP = Real(0), fAP = Real(0), fBP = Real(0);  // the first face of a closed ring
    uint32_t coff = hd.y;                             // offsets of the carried face's columns
    Real accA = Real(0), accB = Real(0), accE = Real(0), racc = Real(0);
    // the walk with its prefetch in fixed slots (blocks of incidences k.. in Kq[k % KD], records in
    // Rq[k % RD]), unrolled by RING_U (a multiple of both) so that no prefetched value is moved
    constexpr int U = RING_U;
    static_assert(U % KD == 0 && U % RD == 0, "slot walk");
    auto step = [&](const int k, const uint2 r0, const Real* G) {
        // the Gram entries of the edge (A, B) and of its four neighbours in the tet, in ring roles:
        // local edge le = (a, b) with the other vertices c < d, then A = b if bit 30, P = d if bit 31
        const int le = (int)((r0.x >> 27) & 7u);
        const Real gab = le == 0 ? G[0] : le == 1 ? G[1] : le == 2 ? G[2] : le == 3 ? G[3] : le == 4 ? G[4] : G[5];
        const Real gac = (le == 0 || le == 5) ? G[1] : G[0];
        const Real gad = le <= 1 ? G[2] : le == 2 ? G[1] : le == 3 ? G[4] : G[3];
        const Real gbc = le <= 1 ? G[3] : le == 2 ? G[4] : le == 3 ? G[1] : G[2];
        const Real gbd = (le == 0 || le == 5) ? G[4] : G[5];
        const bool sab = (r0.x >> 30) & 1u, scd = (r0.x >> 31) & 1u;
        const Real x1 = scd ? gad : gac, x2 = scd ? gac : gad;  // a with P, a with N
        const Real y1 = scd ? gbd : gbc, y2 = scd ? gbc : gbd;  // b with P, b with N
        const Real gAP = sab ? y1 : x1, gAN = sab ? y2 : x2;
        const Real gBP = sab ? x1 : y1, gBN = sab ? x2 : y2;
        // the element row of the edge (the Gram form of fem3Dtet's P2 GRAD.GRAD row, with
        // G_AA = -(G_AB + G_AP + G_AN) and G_BB likewise eliminated)
        const Real sA = gAP + gAN, sB = gBP + gBN;
        const Real c2 = Real(0.2), c8 = Real(0.8), c16 = Real(1.6);
        Real vA = fma(c2, sA, c8 * gab), vB = fma(c2, sB, c8 * gab);
        Real vE = -c16 * ((gab + sA) + sB);
        Real vP = -c2 * (gAP + gBP), vN = -c2 * (gAN + gBN);
        Real vAP = fma(c16, gBP, -c8 * gAN), vAN = fma(c16, gBN, -c8 * gAP);
        Real vBP = fma(c16, gAP, -c8 * gBN), vBN = fma(c16, gAN, -c8 * gBP);
        Real vPN = c8 * (sA + sB);
        const Real F = c2 * G[6];
        if (DROPCHK) {
            auto keep = [&](Real v) { return fabs(v) > drop ? v : Real(0); };
            vA = keep(vA); vB = keep(vB); vE = keep(vE); vP = keep(vP); vN = keep(vN);
            vAP = keep(vAP); vAN = keep(vAN); vBP = keep(vBP); vBN = keep(vBN); vPN = keep(vPN);
        }
        accA += vA;
        accB += vB;
        accE += vE;
        racc += F;
        // face P: the carried tet's part plus this tet's; final except the first face of a closed ring
        const Real oP = cP + vP, oAP = cAP + vAP, oBP = cBP + vBP;
        if (k == 0 && closed) {
            fP = oP;
            fAP = oAP;
            fBP = oBP;
        } else {
            myRow[coff & 255u] = oP;
            myRow[(coff >> 8) & 255u] = oAP;
            myRow[(coff >> 16) & 255u] = oBP;
        }
        myRow[r0.y >> 24] = vPN;
        cP = vN;
        cAP = vAN;
        cBP = vBN;
        coff = r0.y;
    };
    int k = 0;
    for (; k + U <= nloop; k += U) {
#pragma unroll
        for (int u = 0; u < U; ++u) {
            step(k + u, Rq[u % RD], Kq[u % KD].v);
            if (k + u + KD <= last) Kq[u % KD].load(tetK + KS * (int64_t)(Rq[(u + KD) % RD].x & kRingTetMask));
            if (k + u + RD <= last) Rq[u % RD] = rr[32 * (k + u + RD + 1)];
        }
    }
#pragma unroll
    for (int u = 0; u + 1 < U; ++u) {
        if (k + u < nloop) {
            step(k + u, Rq[u % RD], Kq[u % KD].v);
            if (k + u + KD <= last) Kq[u % KD].load(tetK + KS * (int64_t)(Rq[(u + KD) % RD].x & kRingTetMask));
        }
    }
    bool bad = false;
    if (valid) {
        double F;
        if (DIR && isdir) {
            if (RING_NOZERO) {  // the walk did not run: the row is its diagonal alone
                const int len = (int)(p.rowptr[row + 1] - p.rowptr[row]);
                for (int q = 0; q < len; ++q) myRow[q] = Real(0);
            }
            if (deg > 0) myRow[(hd.x >> 16) & 255u] = Real(deg);
            const double bcr = p.dir_bc[row];
            F = 0;
            for (int q = 0; q < deg; ++q) F += bcr;
        } else {
            if (nloop > 0) {
                // the last face: a closed ring ends on its first face
                myRow[coff & 255u] = cP + fP;
                myRow[(coff >> 8) & 255u] = cAP + fAP;
                myRow[(coff >> 16) & 255u] = cBP + fBP;
                myRow[hd.x & 255u] = accA;
                myRow[(hd.x >> 8) & 255u] = accB;
                myRow[(hd.x >> 16) & 255u] = accE;
            }
            F = (double)racc;
            if (DIR)
                for (int64_t q = p.dir_cptr[row]; q < p.dir_cptr[row + 1]; ++q) myRow[p.dir_coff[q]] = Real(0);
        }
        bad |= !isfinite(F);
        rhs[row] = F;
    }
    __syncwarp();
    const Real fin = write_out_range<Real>(sC, shift, clen, cbase, vals, p.vec_ok, lane);
    bad |= !isfinite(fin);
    if (bad) atomicExch(status, ANIGPU_ERR_NONFINITE);
    pdl_launch_dependents();
}

// The edge walk that also builds the vertex rows by symmetry (used for FP64): every value of this
// row that belongs to a vertex column (A, B, the ring vertices) is also stored at its transposed
// position in that vertex row, together with the vertex-vertex entry (A, B); Dirichlet edge rows
// walk too (for that entry) but write only their diagonal here.  A separate function so that the
// plain walk above keeps its own code.
template <typename Real, bool DIR, bool DROPCHK, bool TR = true>
__global__ void RING_BOUNDS edge_ring_tr_kernel(RowParams p, const uint2* __restrict__ ring,
                                            const int64_t* __restrict__ woff, const Real* __restrict__ tetK,
                                            Real* __restrict__ vals, double* __restrict__ rhs,
                                            int* __restrict__ status, const int32_t* __restrict__ tpos,
                                               const int64_t* __restrict__ twoff, int64_t tstride) {
    using Sm = RowSmem<Real, 10, 2, false>;
    constexpr int KS = 8;
    constexpr int VEC = Sm::VEC;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    const int64_t wg = (int64_t)blockIdx.x * nwarps + warp;
    const int64_t row0 = p.row_begin + wg * 32;
    if (row0 >= p.nrows) return;  // warp-uniform; no block-wide barrier follows
    const int64_t rend = row0 + 32 < p.nrows ? row0 + 32 : p.nrows;
    const int64_t cbase = p.rowptr[row0];
    const int clen = (int)(p.rowptr[rend] - cbase);
    const int shift = (int)(cbase & (VEC - 1));
    unsigned char* wbase = smem_raw + Sm::warp_bytes(p.cap) * warp;
    Real* sC = reinterpret_cast<Real*>(wbase) + shift;
    {
        const int nvec = (shift + clen + VEC - 1) / VEC;
        int4* z = reinterpret_cast<int4*>(wbase);
        for (int k = lane; k < nvec; k += 32) z[k] = make_int4(0, 0, 0, 0);
    }
    const int64_t row = row0 + lane;
    const bool valid = row < p.nrows;
    const uint2* rr = ring + (p.wstride > 0 ? wg * p.wstride : woff[wg]) + lane;
    int deg = 0, base = 0;
    bool isdir = false;
    uint2 hd = make_uint2(0u, 0u);
    if (valid) {
        deg = (int)(p.inc_ptr[row + 1] - p.inc_ptr[row]);
        base = (int)(p.rowptr[row] - cbase);
        if (DIR) isdir = p.dir_mask[row] != 0;
        hd = rr[0];
    }
    __syncwarp();
    Real* myRow = sC + base;
    const Real drop = Real(p.drop);
    const int nloop = isdir && !TR ? 0 : deg;
    const int last = nloop - 1;
    constexpr int KD = RING_KD, RD = RING_RD;
    static_assert(RD > KD, "records must run ahead of the blocks they address");
    // TR: transposed positions, (N,E) of incidence j in slot 5 + j, prefetched like the records
    const int32_t* tr = TR ? tpos + (tstride > 0 ? wg * tstride : twoff[wg]) + lane : nullptr;
    int32_t Tq[TR ? RD : 1];
    int32_t tprev = 0;  // (N,E) of the previous incidence: where this step's completed face goes
    Real tf0 = Real(0), accAB = Real(0);
    if (TR) {
#pragma unroll
        for (int j = 0; j < RD; ++j) Tq[j] = tr[32 * (5 + j)];
    }
    static_assert(RD < 16, "the first records may reach RD slots past the lane's own (kRecPad)");
    KVec<Real, KS> Kq[KD];
    uint2 Rq[RD];
#pragma unroll
    for (int j = 0; j < KD; ++j) Kq[j].zero();
#pragma unroll
    for (int j = 0; j < RD; ++j) Rq[j] = make_uint2(0u, 0u);
#pragma unroll
    for (int j = 0; j < RD; ++j)
        if (REC_AHEAD || j <= last) Rq[j] = rr[32 * (j + 1)];
    pdl_wait();  // the per-tet blocks of this assembly
#pragma unroll
    for (int j = 0; j < KD; ++j)
        if (j <= last) Kq[j].load(tetK + KS * (int64_t)(Rq[j].x & kRingTetMask));
    const bool closed = (hd.x >> 24) & 1u;
    Real cP = Real(0), cAP = Real(0), cBP = Real(0);  // the face carried to the next tet
    Real fP = Real(0), fAP = Real(0), fBP = Real(0);  // the first face of a closed ring
    uint32_t coff = hd.y;                             // offsets of the carried face's columns
    Real accA = Real(0), accB = Real(0), accE = Real(0), racc = Real(0);
    // the walk with its prefetch in fixed slots (blocks of incidences k.. in Kq[k % KD], records in
    // Rq[k % RD]), unrolled by RING_U (a multiple of both) so that no prefetched value is moved
    constexpr int U = RING_U;
    static_assert(U % KD == 0 && U % RD == 0, "slot walk");
    auto step = [&](const int k, const uint2 r0, const Real* G) {
        // the Gram entries of the edge (A, B) and of its four neighbours in the tet, in ring roles:
        // local edge le = (a, b) with the other vertices c < d, then A = b if bit 30, P = d if bit 31
        const int le = (int)((r0.x >> 27) & 7u);
        const Real gab = le == 0 ? G[0] : le == 1 ? G[1] : le == 2 ? G[2] : le == 3 ? G[3] : le == 4 ? G[4] : G[5];
        const Real gac = (le == 0 || le == 5) ? G[1] : G[0];
        const Real gad = le <= 1 ? G[2] : le == 2 ? G[1] : le == 3 ? G[4] : G[3];
        const Real gbc = le <= 1 ? G[3] : le == 2 ? G[4] : le == 3 ? G[1] : G[2];
        const Real gbd = (le == 0 || le == 5) ? G[4] : G[5];
        const bool sab = (r0.x >> 30) & 1u, scd = (r0.x >> 31) & 1u;
        const Real x1 = scd ? gad : gac, x2 = scd ? gac : gad;  // a with P, a with N
        const Real y1 = scd ? gbd : gbc, y2 = scd ? gbc : gbd;  // b with P, b with N
        const Real gAP = sab ? y1 : x1, gAN = sab ? y2 : x2;
        const Real gBP = sab ? x1 : y1, gBN = sab ? x2 : y2;
        // the element row of the edge (the Gram form of fem3Dtet's P2 GRAD.GRAD row, with
        // G_AA = -(G_AB + G_AP + G_AN) and G_BB likewise eliminated)
        const Real sA = gAP + gAN, sB = gBP + gBN;
        const Real c2 = Real(0.2), c8 = Real(0.8), c16 = Real(1.6);
        Real vA = fma(c2, sA, c8 * gab), vB = fma(c2, sB, c8 * gab);
        Real vE = -c16 * ((gab + sA) + sB);
        Real vP = -c2 * (gAP + gBP), vN = -c2 * (gAN + gBN);
        Real vAP = fma(c16, gBP, -c8 * gAN), vAN = fma(c16, gBN, -c8 * gAP);
        Real vBP = fma(c16, gAP, -c8 * gBN), vBN = fma(c16, gAN, -c8 * gBP);
        Real vPN = c8 * (sA + sB);
        const Real F = c2 * G[6];
        if (DROPCHK) {
            auto keep = [&](Real v) { return fabs(v) > drop ? v : Real(0); };
            vA = keep(vA); vB = keep(vB); vE = keep(vE); vP = keep(vP); vN = keep(vN);
            vAP = keep(vAP); vAN = keep(vAN); vBP = keep(vBP); vBN = keep(vBN); vPN = keep(vPN);
        }
        accA += vA;
        accB += vB;
        accE += vE;
        racc += F;
        // face P: the carried tet's part plus this tet's; final except the first face of a closed ring
        const Real oP = cP + vP, oAP = cAP + vAP, oBP = cBP + vBP;
        if (TR) {
            // the vertex-vertex entry (A, B) of fem3Dtet's P2 GRAD.GRAD matrix: -0.2 G_AB per tet
            const Real vAB = Real(-0.2) * gab;
            accAB += DROPCHK ? (fabs(vAB) > drop ? vAB : Real(0)) : vAB;
            if (k == 0) tf0 = oP;
            else if (!isdir) vals[tprev] = oP;  // the completed face's vertex row, column E
        }
        if (k == 0 && closed) {
            fP = oP;
            fAP = oAP;
            fBP = oBP;
        } else if (!TR || !isdir) {
            myRow[coff & 255u] = oP;
            myRow[(coff >> 8) & 255u] = oAP;
            myRow[(coff >> 16) & 255u] = oBP;
        }
        if (!TR || !isdir) myRow[r0.y >> 24] = vPN;
        cP = vN;
        cAP = vAN;
        cBP = vBN;
        coff = r0.y;
    };
    int k = 0;
    for (; k + U <= nloop; k += U) {
#pragma unroll
        for (int u = 0; u < U; ++u) {
            step(k + u, Rq[u % RD], Kq[u % KD].v);
            if (TR) tprev = Tq[u % RD];
            if (k + u + KD <= last) Kq[u % KD].load(tetK + KS * (int64_t)(Rq[(u + KD) % RD].x & kRingTetMask));
            if (k + u + RD <= last) {
                Rq[u % RD] = rr[32 * (k + u + RD + 1)];
                if (TR) Tq[u % RD] = tr[32 * (5 + k + u + RD)];
            }
        }
    }
#pragma unroll
    for (int u = 0; u + 1 < U; ++u) {
        if (k + u < nloop) {
            step(k + u, Rq[u % RD], Kq[u % KD].v);
            if (TR) tprev = Tq[u % RD];
            if (k + u + KD <= last) Kq[u % KD].load(tetK + KS * (int64_t)(Rq[(u + KD) % RD].x & kRingTetMask));
        }
    }
    bool bad = false;
    if (TR && valid && nloop > 0) {
        // transposed: the last face, the first face of a path, (A,E), (B,E) and (A,B), (B,A)
        if (!isdir) {
            vals[tprev] = cP + fP;
            if (!closed) vals[tr[128]] = tf0;
            vals[tr[0]] = accA;
            vals[tr[32]] = accB;
        }
        vals[tr[64]] = accAB;
        vals[tr[96]] = accAB;
        bad |= !isfinite(accAB);
    }
    if (valid) {
        double F;
        if (DIR && isdir) {
            if (deg > 0) myRow[(hd.x >> 16) & 255u] = Real(deg);
            const double bcr = p.dir_bc[row];
            F = 0;
            for (int q = 0; q < deg; ++q) F += bcr;
        } else {
            if (nloop > 0) {
                // the last face: a closed ring ends on its first face
                myRow[coff & 255u] = cP + fP;
                myRow[(coff >> 8) & 255u] = cAP + fAP;
                myRow[(coff >> 16) & 255u] = cBP + fBP;
                myRow[hd.x & 255u] = accA;
                myRow[(hd.x >> 8) & 255u] = accB;
                myRow[(hd.x >> 16) & 255u] = accE;
            }
            F = (double)racc;
            if (DIR)
                for (int64_t q = p.dir_cptr[row]; q < p.dir_cptr[row + 1]; ++q) myRow[p.dir_coff[q]] = Real(0);
        }
        bad |= !isfinite(F);
        rhs[row] = F;
    }
    __syncwarp();
    const Real fin = write_out_range<Real>(sC, shift, clen, cbase, vals, p.vec_ok, lane);
    bad |= !isfinite(fin);
    if (bad) atomicExch(status, ANIGPU_ERR_NONFINITE);
    pdl_launch_dependents();
}

// vertex rows: per-tet blocks four incidences ahead, records eight (127 registers, eight 64-thread
// blocks per SM: the loads in flight per warp matter more than the warps)
#ifndef VILV_KD
#define VILV_KD 4
#endif
#ifndef VILV_RD
#define VILV_RD 8
#endif
#ifndef VILV_U
#define VILV_U 8
#endif
#ifdef VILV_MINB
#define VILV_BOUNDS __launch_bounds__(64, VILV_MINB)
#else
#define VILV_BOUNDS __launch_bounds__(64)
#endif

// Vertex rows (Gram form) from lane-interleaved records: record j of lane l of warp w at
// vrec[woff[w] + 32 j + l], so a warp reads one contiguous 512-byte range per step instead of 32
// scattered records.  The diagonal (every incident tet) is summed in a register and written once;
// the other columns of an element row are added into the shared-memory row as in row_gather_kernel.
template <typename Real, int NLOC, bool DIR, bool DROPCHK>
__global__ void VILV_BOUNDS vertex_ilv_kernel(RowParams p, const ScatterRec* __restrict__ vrec,
                                             const int64_t* __restrict__ woff, const Real* __restrict__ tetK,
                                             Real* __restrict__ vals, double* __restrict__ rhs,
                                             int* __restrict__ status) {
    using Sm = RowSmem<Real, NLOC, 1, false>;
    constexpr int KS = 8;
    constexpr int VEC = Sm::VEC;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    const int64_t wg = (int64_t)blockIdx.x * nwarps + warp;
    const int64_t row0 = p.row_begin + wg * 32;
    if (row0 >= p.nrows) return;  // warp-uniform; no block-wide barrier follows
    const int64_t rend = row0 + 32 < p.nrows ? row0 + 32 : p.nrows;
    const int64_t cbase = p.rowptr[row0];
    const int clen = (int)(p.rowptr[rend] - cbase);
    const int shift = (int)(cbase & (VEC - 1));
    unsigned char* wbase = smem_raw + Sm::warp_bytes(p.cap) * warp;
    Real* sC = reinterpret_cast<Real*>(wbase) + shift;
    {
        const int nvec = (shift + clen + VEC - 1) / VEC;
        int4* z = reinterpret_cast<int4*>(wbase);
        for (int k = lane; k < nvec; k += 32) z[k] = make_int4(0, 0, 0, 0);
    }
    const int64_t row = row0 + lane;
    const bool valid = row < p.nrows;
    const ScatterRec* rr = vrec + (p.wstride > 0 ? wg * p.wstride : woff[wg]) + lane;
    int deg = 0, base = 0;
    bool isdir = false;
    if (valid) {
        deg = (int)(p.inc_ptr[row + 1] - p.inc_ptr[row]);
        base = (int)(p.rowptr[row] - cbase);
        if (DIR) isdir = p.dir_mask[row] != 0;
    }
    __syncwarp();
    Real* myRow = sC + base;
    const Real drop = Real(p.drop);
    const int nloop = isdir ? 0 : deg;
    const int last = nloop - 1;
    // the walk with its prefetch in fixed slots (blocks of incidences k.. in Kq[k % KD], records in
    // Rq[k % RD]), unrolled by U (a multiple of both) so that no prefetched value is moved
    constexpr int KD = VILV_KD, RD = VILV_RD, U = VILV_U;
    static_assert(RD > KD && U % KD == 0 && U % RD == 0, "slot walk");
    static_assert(RD <= 16, "the first records may reach RD - 1 slots past the lane's own (kRecPad)");
    KVec<Real, KS> Kq[KD];
    ScatterRec Rq[RD];
#pragma unroll
    for (int j = 0; j < KD; ++j) Kq[j].zero();
#pragma unroll
    for (int j = 0; j < RD; ++j) Rq[j] = ScatterRec{0u, 0u, 0u, 0u};
#pragma unroll
    for (int j = 0; j < RD; ++j)
        if (REC_AHEAD || j <= last) Rq[j] = rr[32 * j];
    pdl_wait();  // the per-tet blocks of this assembly
#pragma unroll
    for (int j = 0; j < KD; ++j)
        if (j <= last) Kq[j].load(tetK + KS * (int64_t)Rq[j].tet);
    // the diagonal's offset: column 0 of every record of the row (its own vertex)
    int odiag = 0;
    if (deg > 0) odiag = (int)((isdir ? rr[0].off03 : Rq[0].off03) & 255u);
    Real accD = Real(0), racc = Real(0);
    auto step = [&](const ScatterRec r0, const Real* G) {
        Real a[NLOC];
        const Real F = gram_row<Real, NLOC, 1>(G, (int)(r0.meta & 15u), a);
        if (DROPCHK) {
#pragma unroll
            for (int j = 0; j < NLOC; ++j) a[j] = fabs(a[j]) > drop ? a[j] : Real(0);
        }
        accD += a[0];
        racc += F;
        int o[NLOC];
        Real cur[NLOC];
#pragma unroll
        for (int j = 1; j < NLOC; ++j) {
            const uint32_t w = j < 4 ? r0.off03 : (j < 8 ? r0.off47 : (r0.meta >> 16));
            o[j] = (int)byte_of(w, j);
            cur[j] = myRow[o[j]];
        }
#pragma unroll
        for (int j = 1; j < NLOC; ++j) myRow[o[j]] = cur[j] + a[j];
    };
    int k = 0;
    for (; k + U <= nloop; k += U) {
#pragma unroll
        for (int u = 0; u < U; ++u) {
            step(Rq[u % RD], Kq[u % KD].v);
            if (k + u + KD <= last) Kq[u % KD].load(tetK + KS * (int64_t)Rq[(u + KD) % RD].tet);
            if (k + u + RD <= last) Rq[u % RD] = rr[32 * (k + u + RD)];
        }
    }
#pragma unroll
    for (int u = 0; u + 1 < U; ++u) {
        if (k + u < nloop) {
            step(Rq[u % RD], Kq[u % KD].v);
            if (k + u + KD <= last) Kq[u % KD].load(tetK + KS * (int64_t)Rq[(u + KD) % RD].tet);
        }
    }
    bool bad = false;
    if (valid) {
        double F;
        if (DIR && isdir) {
            if (deg > 0) myRow[odiag] = Real(deg);
            const double bcr = p.dir_bc[row];
            F = 0;
            for (int q = 0; q < deg; ++q) F += bcr;
        } else {
            if (nloop > 0) myRow[odiag] = accD;
            F = (double)racc;
            if (DIR)
                for (int64_t q = p.dir_cptr[row]; q < p.dir_cptr[row + 1]; ++q) myRow[p.dir_coff[q]] = Real(0);
        }
        bad |= !isfinite(F);
        rhs[row] = F;
    }
    __syncwarp();
    const Real fin = write_out_range<Real>(sC, shift, clen, cbase, vals, p.vec_ok, lane);
    bad |= !isfinite(fin);
    if (bad) atomicExch(status, ANIGPU_ERR_NONFINITE);
    pdl_launch_dependents();
}

// The vertex rows when the edge walks have stored their off-diagonal entries (TR): per row the
// diagonal (the sum of 0.6 G_ii over the incident tets, fem3Dtet's P2 GRAD.GRAD diagonal) and the
// right-hand side (-0.05 f|T| per tet), from the incidence words in the interleaved layout; a
// Dirichlet row is rewritten as its diagonal (the number of incident tets), a row with Dirichlet
// columns has them zeroed.  Runs after the edge walks (their stores into these rows come first).
#ifndef VTR_KD
#define VTR_KD 4
#endif
#ifndef VTR_RD
#define VTR_RD 8
#endif
template <typename Real, bool DIR, bool DROPCHK>
__global__ void __launch_bounds__(128) vertex_tr_kernel(RowParams p, const uint32_t* __restrict__ vrec4,
                                                        const int64_t* __restrict__ woff,
                                                        const int32_t* __restrict__ vdiag,
                                                        const Real* __restrict__ tetK, Real* __restrict__ vals,
                                                        double* __restrict__ rhs, int* __restrict__ status) {
    constexpr int KS = 8, KD = VTR_KD, RD = VTR_RD;
    static_assert(RD > KD && RD <= 16, "prefetch depths (kRecPad)");
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t wg = t >> 5;
    const int lane = (int)(t & 31);
    const int64_t row = p.row_begin + t;
    if (row >= p.nrows) return;  // no warp-wide operation follows
    const uint32_t* rr = vrec4 + (p.wstride > 0 ? wg * p.wstride : woff[wg]) + lane;
    const int deg = (int)(p.inc_ptr[row + 1] - p.inc_ptr[row]);
    const bool isdir = DIR && p.dir_mask[row] != 0;
    const int nloop = isdir ? 0 : deg;
    const int last = nloop - 1;
    const Real drop = Real(p.drop);
    uint32_t Rq[RD];
#pragma unroll
    for (int j = 0; j < RD; ++j) Rq[j] = rr[32 * j];
    pdl_wait();  // the per-tet blocks and the edge walks' stores
    KVec<Real, KS> Kq[KD];
#pragma unroll
    for (int j = 0; j < KD; ++j) {
        Kq[j].zero();
        if (j <= last) Kq[j].load(tetK + KS * (int64_t)(Rq[j] & kRingTetMask));
    }
    Real accD = Real(0), racc = Real(0);
    auto step = [&](const uint32_t r0, const Real* G) {
        Real a[10];
        const Real F = gram_row<Real, 10, 1>(G, (int)(r0 >> 27), a);
        accD += DROPCHK ? (fabs(a[0]) > drop ? a[0] : Real(0)) : a[0];
        racc += F;
    };
    // prefetch in fixed slots (blocks of incidence k in Kq[k % KD], words in Rq[k % RD]), unrolled
    // by RD so that no prefetched value is moved
    constexpr int U = RD;
    static_assert(U % KD == 0, "slot walk");
    int k = 0;
    for (; k + U <= nloop; k += U) {
#pragma unroll
        for (int u = 0; u < U; ++u) {
            step(Rq[u % RD], Kq[u % KD].v);
            if (k + u + KD <= last) Kq[u % KD].load(tetK + KS * (int64_t)(Rq[(u + KD) % RD] & kRingTetMask));
            if (k + u + RD <= last) Rq[u % RD] = rr[32 * (k + u + RD)];
        }
    }
#pragma unroll
    for (int u = 0; u + 1 < U; ++u) {
        if (k + u < nloop) {
            step(Rq[u % RD], Kq[u % KD].v);
            if (k + u + KD <= last) Kq[u % KD].load(tetK + KS * (int64_t)(Rq[(u + KD) % RD] & kRingTetMask));
        }
    }
    const int64_t rb = p.rowptr[row];
    double F;
    if (DIR && isdir) {
        const int64_t re = p.rowptr[row + 1];
        for (int64_t q = rb; q < re; ++q) vals[q] = Real(0);
        if (deg > 0) vals[vdiag[row]] = Real(deg);
        const double bcr = p.dir_bc[row];
        F = 0;
        for (int q = 0; q < deg; ++q) F += bcr;
    } else {
        vals[vdiag[row]] = accD;
        F = (double)racc;
        if (DIR)
            for (int64_t q = p.dir_cptr[row]; q < p.dir_cptr[row + 1]; ++q) vals[rb + p.dir_coff[q]] = Real(0);
    }
    rhs[row] = F;
    if (!isfinite(F) || !isfinite((double)accD)) atomicExch(status, ANIGPU_ERR_NONFINITE);
}

// slots of each warp of 32 rows in a lane-interleaved layout: 32 x (head + its largest
// incident-tet count)
__global__ void warp_slots_kernel(int64_t rb, int64_t re, int head, const int64_t* __restrict__ inc_ptr,
                                  unsigned long long* __restrict__ cnt, unsigned long long* __restrict__ cmax) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;  // blockDim: a multiple of 32
    const int64_t r = rb + t;
    const int deg = r < re ? (int)(inc_ptr[r + 1] - inc_ptr[r]) : 0;
    const int m = __reduce_max_sync(0xffffffffu, deg);
    if ((threadIdx.x & 31) == 0 && rb + t < re) {
        const unsigned long long c = 32ull * (unsigned long long)(m + head);
        cnt[t >> 5] = c;
        atomicMax(cmax, c);
    }
}

__global__ void uniform_offsets_kernel(int64_t nw, int64_t ws, int64_t* __restrict__ woff) {
    const int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (w <= nw) woff[w] = w * ws;
}

// vertex rows' records in the lane-interleaved layout: record j of row rb + 32 w + l at
// vrec[woff[w] + 32 j + l]
__global__ void vertex_ilv_build_kernel(int64_t rb, int64_t re, const int64_t* __restrict__ inc_ptr,
                                        const ScatterRec* __restrict__ recs, const int64_t* __restrict__ woff,
                                        ScatterRec* __restrict__ vrec) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t r = rb + t;
    if (r >= re) return;
    ScatterRec* out = vrec + woff[t >> 5] + (t & 31);
    const int64_t ib = inc_ptr[r];
    const int deg = (int)(inc_ptr[r + 1] - ib);
    for (int j = 0; j < deg; ++j) out[32 * j] = recs[ib + j];
}

// canonical column c of an edge row's scatter record: its offset within the row
__device__ __forceinline__ uint32_t rec_off(const ScatterRec& r, int c) {
    const uint32_t w = c < 4 ? r.off03 : (c < 8 ? r.off47 : (r.meta >> 16));
    return (w >> (8 * (c & 3))) & 255u;
}

// ring build, pass 2: one thread per edge row orders the row's incident tets into its ring and
// writes the header and the records; a row whose tets do not form one ring (a non-manifold edge,
// more than kRingMax tets, an inconsistent record) sets *fail, and the mesh keeps the record gather
__global__ void ring_build_kernel(int64_t rb, int64_t re, const int64_t* __restrict__ inc_ptr,
                                  const ScatterRec* __restrict__ recs, const int32_t* __restrict__ tets,
                                  const int64_t* __restrict__ rowptr, const int64_t* __restrict__ woff,
                                  uint2* __restrict__ ring, int* __restrict__ fail) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t r = rb + t;
    if (r >= re) return;
    uint2* out = ring + woff[t >> 5] + (t & 31);
    const int64_t ib = inc_ptr[r];
    const int deg = (int)(inc_ptr[r + 1] - ib);
    if (deg < 1 || deg > kRingMax) {
        atomicOr(fail, 1);
        return;
    }
    const int EI[6] = {0, 0, 0, 1, 1, 2}, EJ[6] = {1, 2, 3, 2, 3, 3};
    int32_t gc[kRingMax], gd[kRingMax];
    int32_t vA = -1, vB = -1;
    for (int j = 0; j < deg; ++j) {
        const ScatterRec rec = recs[ib + j];
        const int i = (int)(rec.meta & 15u);
        if (i < 4 || i > 9 || rec.tet > kRingTetMask) {
            atomicOr(fail, 1);
            return;
        }
        const int k = i - 4, la = EI[k], lb = EJ[k];
        int lc = -1, ld = -1;
        for (int l = 0; l < 4; ++l)
            if (l != la && l != lb) {
                if (lc < 0) lc = l;
                else ld = l;
            }
        const int32_t* tv = tets + 4 * (int64_t)rec.tet;
        const int32_t ga = tv[la], gb = tv[lb];
        if (j == 0) {
            vA = ga < gb ? ga : gb;
            vB = ga < gb ? gb : ga;
        } else if ((ga < gb ? ga : gb) != vA || (ga < gb ? gb : ga) != vB) {
            atomicOr(fail, 1);
            return;
        }
        gc[j] = tv[lc];
        gd[j] = tv[ld];
    }
    // each ring vertex lies on two tets (one at the two ends of a path)
    int ones = 0;
    int32_t end0 = -1;
    for (int j = 0; j < deg; ++j)
        for (int h = 0; h < 2; ++h) {
            const int32_t v = h ? gd[j] : gc[j];
            int n = 0;
            for (int q = 0; q < deg; ++q) n += (gc[q] == v) + (gd[q] == v);
            if (n < 1 || n > 2) {
                atomicOr(fail, 1);
                return;
            }
            if (n == 1) {
                ++ones;
                if (end0 < 0) end0 = v;  // in the smallest tet that has an end
            }
        }
    const bool closed = ones == 0;
    if (!(ones == 0 || ones == 2) || (closed && deg < 3)) {
        atomicOr(fail, 1);
        return;
    }
    // the walk writes every column of the row: A, B, the edge, three per ring vertex (the vertex and
    // its edges to A and B) and one per tet (the opposite edge)
    const int nverts = closed ? deg : deg + 1;
    if (rowptr[r + 1] - rowptr[r] != 3 + 3 * nverts + deg) {
        atomicOr(fail, 1);
        return;
    }
    // walk: start at the smallest tet (closed) or at the path end in the smallest tet
    int order[kRingMax];
    int32_t pv[kRingMax];
    int j0 = 0;
    int32_t P0 = gc[0];
    if (!closed) {
        for (int j = 0; j < deg; ++j)
            if (gc[j] == end0 || gd[j] == end0) {
                j0 = j;
                break;
            }
        P0 = end0;
    }
    uint32_t used = 1u << j0;
    order[0] = j0;
    pv[0] = P0;
    int32_t N = gc[j0] == P0 ? gd[j0] : gc[j0];
    for (int s = 1; s < deg; ++s) {
        int js = -1;
        for (int j = 0; j < deg; ++j)
            if (!((used >> j) & 1u) && (gc[j] == N || gd[j] == N)) {
                js = j;
                break;
            }
        if (js < 0) {
            atomicOr(fail, 1);
            return;
        }
        used |= 1u << js;
        order[s] = js;
        pv[s] = N;
        N = gc[js] == N ? gd[js] : gc[js];
    }
    if (closed ? N != P0 : N == P0) {
        atomicOr(fail, 1);
        return;
    }
    // records in ring order; the face offsets of consecutive tets must agree
    uint32_t hx = 0, hy = 0, prevN = 0;
    for (int s = 0; s < deg; ++s) {
        const int j = order[s];
        const ScatterRec rec = recs[ib + j];
        const int k = (int)(rec.meta & 15u) - 4;
        const int32_t* tv = tets + 4 * (int64_t)rec.tet;
        const uint32_t sab = tv[EI[k]] != vA ? 1u : 0u;
        const uint32_t scd = gc[j] != pv[s] ? 1u : 0u;
        uint32_t o[10];
        for (int c = 0; c < 10; ++c) o[c] = rec_off(rec, c);
        const uint32_t oA = sab ? o[1] : o[0], oB = sab ? o[0] : o[1];
        const uint32_t oP = scd ? o[3] : o[2], oN = scd ? o[2] : o[3];
        const uint32_t aP = scd ? o[6] : o[5], aN = scd ? o[5] : o[6];
        const uint32_t bP = scd ? o[8] : o[7], bN = scd ? o[7] : o[8];
        const uint32_t oAP = sab ? bP : aP, oBP = sab ? aP : bP;
        const uint32_t oAN = sab ? bN : aN, oBN = sab ? aN : bN;
        const uint32_t face = oP | (oAP << 8) | (oBP << 16);
        const uint32_t ends = oA | (oB << 8) | (o[4] << 16);
        if (s == 0) {
            hx = ends | (closed ? 1u << 24 : 0u);
            hy = face;
        } else if (face != prevN || ends != (hx & 0xffffffu)) {
            atomicOr(fail, 1);
            return;
        }
        prevN = oN | (oAN << 8) | (oBN << 16);
        out[32 * (s + 1)] = make_uint2(rec.tet | ((uint32_t)k << 27) | (sab << 30) | (scd << 31),
                                       prevN | (o[9] << 24));
    }
    if (closed && prevN != hy) {
        atomicOr(fail, 1);
        return;
    }
    out[0] = make_uint2(hx, hy);
}

// ---------------------------------------------------------------- P2 vertex rows by symmetry
// position of column c in row x of the template (-1 when absent)
__device__ __forceinline__ int32_t col_pos(const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                           int64_t x, int32_t c) {
    int64_t lo = rowptr[x], hi = rowptr[x + 1];
    const int64_t end = hi;
    while (lo < hi) {
        const int64_t m = (lo + hi) >> 1;
        if (col[m] < c) lo = m + 1;
        else hi = m;
    }
    return lo < end && col[lo] == c ? (int32_t)lo : -1;
}

// transposed positions of edge row r = E in the lane-interleaved layout (head 5): (A,E), (B,E),
// (A,B), (B,A), the first ring vertex's (P0,E) for a path, then (N,E) of each incidence of the ring
__global__ void tpos_build_kernel(int64_t rb, int64_t re, const int64_t* __restrict__ inc_ptr,
                                  const uint2* __restrict__ ring, const int64_t* __restrict__ ring_woff,
                                  const int32_t* __restrict__ tets, const int64_t* __restrict__ rowptr,
                                  const int32_t* __restrict__ col, const int64_t* __restrict__ twoff,
                                  int32_t* __restrict__ tpos, int* __restrict__ fail) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t r = rb + t;
    if (r >= re) return;
    const uint2* rr = ring + ring_woff[t >> 5] + (t & 31);
    int32_t* out = tpos + twoff[t >> 5] + (t & 31);
    const int deg = (int)(inc_ptr[r + 1] - inc_ptr[r]);
    const bool closed = (rr[0].x >> 24) & 1u;
    const int32_t E = (int32_t)r;
    const int EI[6] = {0, 0, 0, 1, 1, 2}, EJ[6] = {1, 2, 3, 2, 3, 3};
    int32_t vA = -1, vB = -1, P0 = -1;
    bool bad = deg < 1;
    for (int s = 0; s < deg && !bad; ++s) {
        const uint2 rec = rr[32 * (s + 1)];
        const int32_t* tv = tets + 4 * (int64_t)(rec.x & kRingTetMask);
        const int k = (int)((rec.x >> 27) & 7u), la = EI[k], lb = EJ[k];
        int lc = -1, ld = -1;
        for (int l = 0; l < 4; ++l)
            if (l != la && l != lb) {
                if (lc < 0) lc = l;
                else ld = l;
            }
        const bool sab = (rec.x >> 30) & 1u, scd = (rec.x >> 31) & 1u;
        const int32_t A = sab ? tv[lb] : tv[la], B = sab ? tv[la] : tv[lb];
        const int32_t P = scd ? tv[ld] : tv[lc], N = scd ? tv[lc] : tv[ld];
        if (s == 0) {
            vA = A;
            vB = B;
            P0 = P;
        }
        const int32_t q = col_pos(rowptr, col, N, E);
        bad |= q < 0 || A != vA || B != vB;
        out[32 * (5 + s)] = q;
    }
    if (!bad) {
        const int32_t h0 = col_pos(rowptr, col, vA, E), h1 = col_pos(rowptr, col, vB, E);
        const int32_t h2 = col_pos(rowptr, col, vA, vB), h3 = col_pos(rowptr, col, vB, vA);
        const int32_t h4 = closed ? 0 : col_pos(rowptr, col, P0, E);
        bad = h0 < 0 || h1 < 0 || h2 < 0 || h3 < 0 || h4 < 0;
        out[0] = h0;
        out[32] = h1;
        out[64] = h2;
        out[96] = h3;
        out[128] = h4;
    }
    if (bad) atomicOr(fail, 1);
}

// the vertex rows' incidences (tet | local vertex << 27) in the interleaved layout of vrec, and the
// position of each vertex row's diagonal
__global__ void vertex4_build_kernel(int64_t rb, int64_t re, const int64_t* __restrict__ inc_ptr,
                                     const ScatterRec* __restrict__ recs, const int64_t* __restrict__ rowptr,
                                     const int32_t* __restrict__ col, const int64_t* __restrict__ woff,
                                     uint32_t* __restrict__ vrec4, int32_t* __restrict__ vdiag,
                                     int* __restrict__ fail) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t r = rb + t;
    if (r >= re) return;
    uint32_t* out = vrec4 + woff[t >> 5] + (t & 31);
    const int64_t ib = inc_ptr[r];
    const int deg = (int)(inc_ptr[r + 1] - ib);
    bool bad = false;
    for (int j = 0; j < deg; ++j) {
        const ScatterRec rec = recs[ib + j];
        const uint32_t i = rec.meta & 15u;
        bad |= i > 3u || rec.tet > kRingTetMask;
        out[32 * j] = rec.tet | (i << 27);
    }
    const int32_t d = col_pos(rowptr, col, r, (int32_t)r);
    vdiag[r] = d;
    if (bad || d < 0) atomicOr(fail, 1);
}

// ---------------------------------------------------------------- vector P2 (linear elasticity)
// Operator<GRAD, FemVec<3, FEM_P2>> with the isotropic Lame tensor
//     D[(j,c),(l,d)] = lambda delta_jc delta_ld + mu (delta_cd delta_jl + delta_cl delta_jd)
// (gradient index j + 3 c for derivative j of component c; lin_elast.cpp:100-118).  With exact
// integration (order >= 2) the block (row component c, column component d) of an element row is the
// scalar Gram formula of its row kind with G_pq replaced by
//     B^{cd}_pq = |T| (lambda g_p^c g_q^d + mu (delta_cd g_p.g_q + g_p^d g_q^c))
// (p on the row side: B is not symmetric in p, q for c != d); rows of B also sum to zero over q.
// Per tet: g_1, g_2, g_3 (g_0 = -(g_1 + g_2 + g_3)), lambda|T|, mu|T|, f|T|: a 16-value block.
template <typename R>
__device__ __forceinline__ void lame_block(const R* PSI, R lam, R mu, R mes, R fm, R* out) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        out[3 * a] = PSI[a];
        out[3 * a + 1] = PSI[a + 3];
        out[3 * a + 2] = PSI[a + 6];
    }
    out[9] = lam * mes;
    out[10] = mu * mes;
    out[11] = fm * mes;
    out[12] = out[13] = out[14] = out[15] = R(0);
}

__global__ void tet_lame_f64_kernel(int64_t nt, const double* __restrict__ xyz, const int32_t* __restrict__ tets,
                                    const double* __restrict__ D, const double* __restrict__ f, double f_const,
                                    double* __restrict__ out, int* __restrict__ status) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const int4 v = reinterpret_cast<const int4*>(tets)[t];
    double e[9], PSI[9], B[16];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double x0 = xyz[3 * (int64_t)v.x + k];
        e[k + 0] = xyz[3 * (int64_t)v.y + k] - x0;
        e[k + 3] = xyz[3 * (int64_t)v.z + k] - x0;
        e[k + 6] = xyz[3 * (int64_t)v.w + k] - x0;
    }
    const double det = inverse3(e, PSI);
    lame_block(PSI, D[2 * t], D[2 * t + 1], fabs(det) / 6.0, f ? f[t] : f_const, B);
    bool bad = !(det != 0.0);
#pragma unroll
    for (int k = 0; k < 12; ++k) bad |= !isfinite(B[k]);
    if (bad) atomicExch(status, ANIGPU_ERR_NONFINITE);
    double2* o = reinterpret_cast<double2*>(out + 16 * t);
#pragma unroll
    for (int q = 0; q < 8; ++q) o[q] = make_double2(B[2 * q], B[2 * q + 1]);
}

__global__ void tet_lame_f32_kernel(int64_t nt, const double* __restrict__ xyz, const float2* __restrict__ xyz2,
                                    const int32_t* __restrict__ tets, const double* __restrict__ D,
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
    const double2 lm = reinterpret_cast<const double2*>(D)[t];
    const float lam = d2f_rn(lm.x), mu = d2f_rn(lm.y), fv = d2f_rn(f ? f[t] : f_const);
    float PSI[9], B[16];
    const float det = inverse3(e, PSI);
    const float l0 = e[0] * e[0] + e[1] * e[1] + e[2] * e[2];
    const float l1 = e[3] * e[3] + e[4] * e[4] + e[5] * e[5];
    const float l2 = e[6] * e[6] + e[7] * e[7] + e[8] * e[8];
    if (det * det > 0.0025f * l0 * l1 * l2) {
        lame_block(PSI, lam, mu, fabsf(det) * (1.0f / 6.0f), fv, B);
    } else {  // badly shaped tet: Jacobian and inverse in FP64
        double ed[9], P64[9];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const double x0 = xyz[3 * (int64_t)v.x + k];
            ed[k + 0] = xyz[3 * (int64_t)v.y + k] - x0;
            ed[k + 3] = xyz[3 * (int64_t)v.z + k] - x0;
            ed[k + 6] = xyz[3 * (int64_t)v.w + k] - x0;
        }
        const double det64 = inverse3(ed, P64);
        double B64[16];
        lame_block(P64, lm.x, lm.y, fabs(det64) / 6.0, f ? f[t] : f_const, B64);
#pragma unroll
        for (int k = 0; k < 16; ++k) B[k] = (float)B64[k];
        if (!(det64 != 0.0)) atomicExch(status, ANIGPU_ERR_NONFINITE);
    }
    bool bad = false;
#pragma unroll
    for (int k = 0; k < 12; ++k) bad |= !isfinite(B[k]);
    if (bad) atomicExch(status, ANIGPU_ERR_NONFINITE);
    float4* o = reinterpret_cast<float4*>(out + 16 * t);
#pragma unroll
    for (int q = 0; q < 4; ++q) o[q] = make_float4(B[4 * q], B[4 * q + 1], B[4 * q + 2], B[4 * q + 3]);
}

// prefetch depths of the vector gathers (16-value per-tet blocks, records)
#ifndef VEC_KD
#define VEC_KD 2
#endif
#ifndef VEC_RD
#define VEC_RD 4
#endif
#ifndef VRING_KD
#define VRING_KD 2
#endif
#ifndef VRING_RD
#define VRING_RD 4
#endif

template <typename Real>
struct VBlock {
    Real v[16];
    __device__ __forceinline__ void load(const Real* p) {
        KVec<Real, 8> a, b;
        a.load(p);
        b.load(p + 8);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            v[k] = a.v[k];
            v[8 + k] = b.v[k];
        }
    }
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int k = 0; k < 16; ++k) v[k] = Real(0);
    }
};

template <typename Real>
__device__ __forceinline__ void gvec(const Real* v, int p, Real* g) {
    // gradient of barycentric p from the block: g_1..g_3 stored, g_0 = -(g_1 + g_2 + g_3)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const Real g1 = v[c], g2 = v[3 + c], g3 = v[6 + c];
        g[c] = p == 0 ? -((g1 + g2) + g3) : p == 1 ? g1 : p == 2 ? g2 : g3;
    }
}

template <typename Real>
__device__ __forceinline__ Real sel3(const Real* g, int c) {
    return c == 0 ? g[0] : c == 1 ? g[1] : g[2];
}

// B^{cd}_pq from the row-side gradient gp (gpc = gp[c]) and the column-side gq (gqc = gq[c])
template <typename Real>
__device__ __forceinline__ Real lameB(Real lam, Real mu, const Real* gp, Real gpc, const Real* gq, Real gqc,
                                      Real dot, int c, int d) {
    const Real gpd = sel3(gp, d), gqd = sel3(gq, d);
    Real b = lam * gpc * gqd + mu * gpd * gqc;
    if (c == d) b += mu * dot;
    return b;
}

// one lane per vector row (component c = blockIdx.y, scalar row r); FORM 1 vertex rows, 2 edge rows
template <typename Real, int FORM, bool DIR>
__global__ void __launch_bounds__(64) vec_row_gather_kernel(RowParams p, int64_t nds, const int64_t* __restrict__ vrowptr,
                                                            const Real* __restrict__ tetB, Real* __restrict__ vals,
                                                            double* __restrict__ rhs, int* __restrict__ status) {
    constexpr int VEC = 16 / (int)sizeof(Real);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    const int c = blockIdx.y;
    const int64_t row0 = p.row_begin + ((int64_t)blockIdx.x * nwarps + warp) * 32;
    if (row0 >= p.nrows) return;
    const int64_t rend = row0 + 32 < p.nrows ? row0 + 32 : p.nrows;
    const int64_t cbase = vrowptr[c * nds + row0];
    const int clen = (int)(vrowptr[c * nds + rend] - cbase);
    const int shift = (int)(cbase & (VEC - 1));
    const size_t chunk_bytes = (((size_t)32 * 3 * p.cap + VEC) * sizeof(Real) + 15) / 16 * 16;
    unsigned char* wbase = smem_raw + chunk_bytes * warp;
    Real* sC = reinterpret_cast<Real*>(wbase) + shift;
    {
        const int nvec = (shift + clen + VEC - 1) / VEC;
        int4* z = reinterpret_cast<int4*>(wbase);
        for (int k = lane; k < nvec; k += 32) z[k] = make_int4(0, 0, 0, 0);
    }
    const int64_t r = row0 + lane;
    const int64_t R = c * nds + r;
    const bool valid = r < p.nrows;
    int64_t ib = 0;
    int deg = 0, base = 0, L = 0;
    bool isdir = false;
    if (valid) {
        ib = p.inc_ptr[r];
        deg = (int)(p.inc_ptr[r + 1] - ib);
        base = (int)(vrowptr[R] - cbase);
        L = (int)(p.rowptr[r + 1] - p.rowptr[r]);
        if (DIR) isdir = p.dir_mask[R] != 0;
    }
    __syncwarp();
    Real* myRow = sC + base;
    Real racc = Real(0);
    const int nloop = isdir ? 0 : deg;
    const int last = nloop - 1;
    constexpr int KD = VEC_KD, RD = VEC_RD;
    VBlock<Real> Kq[KD];
    ScatterRec Rq[RD];
#pragma unroll
    for (int j = 0; j < KD; ++j) Kq[j].zero();
#pragma unroll
    for (int j = 0; j < RD; ++j) Rq[j] = ScatterRec{0u, 0u, 0u, 0u};
    if (nloop > 0) {
#pragma unroll
        for (int j = 0; j < RD; ++j) Rq[j] = p.recs[ib + min(j, last)];
#pragma unroll
        for (int j = 0; j < KD; ++j) Kq[j].load(tetB + 16 * (int64_t)Rq[j].tet);
    }
    const Real m2 = Real(-0.2), p6 = Real(0.6), p8 = Real(0.8), p16 = Real(1.6);
    for (int k = 0; k < nloop; ++k) {
        VBlock<Real> Kn;
        Kn.load(tetB + 16 * (int64_t)Rq[KD].tet);
        const ScatterRec Rn = p.recs[ib + min(k + RD, last)];
        const ScatterRec r0 = Rq[0];
        const Real* bv = Kq[0].v;
        const int i = r0.meta & 15;
        const Real lam = bv[9], mu = bv[10];
        int o[10];
#pragma unroll
        for (int j = 0; j < 10; ++j) {
            const uint32_t w = j < 4 ? r0.off03 : (j < 8 ? r0.off47 : (r0.meta >> 16));
            o[j] = (int)byte_of(w, j);
        }
        if (FORM == 1) {
            // vertex i, others o1 < o2 < o3
            const int q1 = i == 0 ? 1 : 0, q2 = i <= 1 ? 2 : 1, q3 = i <= 2 ? 3 : 2;
            Real gi[3], g1[3], g2[3], g3[3];
            gvec(bv, i, gi);
            gvec(bv, q1, g1);
            gvec(bv, q2, g2);
            gvec(bv, q3, g3);
            const Real gic = sel3(gi, c), g1c = sel3(g1, c), g2c = sel3(g2, c), g3c = sel3(g3, c);
            const Real d1 = gi[0] * g1[0] + gi[1] * g1[1] + gi[2] * g1[2];
            const Real d2 = gi[0] * g2[0] + gi[1] * g2[1] + gi[2] * g2[2];
            const Real d3 = gi[0] * g3[0] + gi[1] * g3[1] + gi[2] * g3[2];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const Real b1 = lameB(lam, mu, gi, gic, g1, g1c, d1, c, d);
                const Real b2 = lameB(lam, mu, gi, gic, g2, g2c, d2, c, d);
                const Real b3 = lameB(lam, mu, gi, gic, g3, g3c, d3, c, d);
                const Real bii = -((b1 + b2) + b3);
                Real a[10];
                a[0] = p6 * bii;
                a[1] = m2 * b1;
                a[2] = m2 * b2;
                a[3] = m2 * b3;
                const Real t = m2 * bii;
                a[4] = fma(p6, b1, t);
                a[5] = fma(p6, b2, t);
                a[6] = fma(p6, b3, t);
                a[7] = m2 * (b1 + b2);
                a[8] = m2 * (b1 + b3);
                a[9] = m2 * (b2 + b3);
                Real* rowd = myRow + d * L;
                Real cur[10];
#pragma unroll
                for (int j = 0; j < 10; ++j) cur[j] = rowd[o[j]];
#pragma unroll
                for (int j = 0; j < 10; ++j) rowd[o[j]] = cur[j] + a[j];
            }
            racc += Real(-0.05) * bv[11];
        } else {
            // edge k = (a,b), others c_ < d_
            const int e = i - 4;
            const int va = e <= 2 ? 0 : e <= 4 ? 1 : 2;
            const int vb = e == 0 ? 1 : (e == 1 || e == 3) ? 2 : 3;
            const int vc = (e <= 2) ? (e == 0 ? 2 : 1) : 0;
            const int vd = e == 0 ? 3 : e == 1 ? 3 : e == 2 ? 2 : e == 3 ? 3 : e == 4 ? 2 : 1;
            Real ga[3], gb[3], gc[3], gd[3];
            gvec(bv, va, ga);
            gvec(bv, vb, gb);
            gvec(bv, vc, gc);
            gvec(bv, vd, gd);
            const Real gac_ = sel3(ga, c), gbc_ = sel3(gb, c), gcc_ = sel3(gc, c), gdc_ = sel3(gd, c);
            const Real dab = ga[0] * gb[0] + ga[1] * gb[1] + ga[2] * gb[2];
            const Real dac = ga[0] * gc[0] + ga[1] * gc[1] + ga[2] * gc[2];
            const Real dad = ga[0] * gd[0] + ga[1] * gd[1] + ga[2] * gd[2];
            const Real dbc = gb[0] * gc[0] + gb[1] * gc[1] + gb[2] * gc[2];
            const Real dbd = gb[0] * gd[0] + gb[1] * gd[1] + gb[2] * gd[2];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const Real Bab = lameB(lam, mu, ga, gac_, gb, gbc_, dab, c, d);
                const Real Bba = lameB(lam, mu, gb, gbc_, ga, gac_, dab, c, d);
                const Real Bac = lameB(lam, mu, ga, gac_, gc, gcc_, dac, c, d);
                const Real Bad = lameB(lam, mu, ga, gac_, gd, gdc_, dad, c, d);
                const Real Bbc = lameB(lam, mu, gb, gbc_, gc, gcc_, dbc, c, d);
                const Real Bbd = lameB(lam, mu, gb, gbc_, gd, gdc_, dbd, c, d);
                const Real Baa = -((Bab + Bac) + Bad), Bbb = -((Bba + Bbc) + Bbd);
                Real a[10];
                a[0] = fma(m2, Baa, p6 * Bba);
                a[1] = fma(p6, Bab, m2 * Bbb);
                a[2] = m2 * (Bac + Bbc);
                a[3] = m2 * (Bad + Bbd);
                a[4] = fma(p16, Baa + Bbb, p8 * (Bab + Bba));
                a[5] = fma(p8, (Baa + Bac) + Bba, p16 * Bbc);
                a[6] = fma(p8, (Baa + Bad) + Bba, p16 * Bbd);
                a[7] = fma(p8, (Bab + Bbb) + Bbc, p16 * Bac);
                a[8] = fma(p8, (Bab + Bbb) + Bbd, p16 * Bad);
                a[9] = p8 * ((Bac + Bad) + (Bbc + Bbd));
                Real* rowd = myRow + d * L;
                Real cur[10];
#pragma unroll
                for (int j = 0; j < 10; ++j) cur[j] = rowd[o[j]];
#pragma unroll
                for (int j = 0; j < 10; ++j) rowd[o[j]] = cur[j] + a[j];
            }
            racc += Real(0.2) * bv[11];
        }
#pragma unroll
        for (int j = 0; j + 1 < KD; ++j) Kq[j] = Kq[j + 1];
        Kq[KD - 1] = Kn;
#pragma unroll
        for (int j = 0; j + 1 < RD; ++j) Rq[j] = Rq[j + 1];
        Rq[RD - 1] = Rn;
    }
    bool bad = false;
    if (valid) {
        double F;
        if (DIR && isdir) {
            if (deg > 0) {  // diagonal = number of incident tets
                const ScatterRec rd = p.recs[ib];
                const int dc = canon_diag(10, rd.meta & 15);
                const int od = (int)byte_of(dc < 4 ? rd.off03 : rd.off47, dc);
                myRow[c * L + od] = Real(deg);
            }
            // rhs = bc per incident tet (applyDir sets F(k) = bc in every element, dc_on_dof.h:39-45)
            const double bcr = p.bcnz ? p.dir_bc[R] : 0.0;
            F = 0;
            for (int q = 0; q < deg; ++q) F += bcr;
        } else {
            F = (double)racc;
            if (DIR) {
                // Dirichlet columns: F -= A(i,k) bc_k with the assembled A(i,k) (the sum over the tets of
                // applyDir's per-element F -= A(:,k) bc), then the column is eliminated
                const int64_t vb = vrowptr[R];
                for (int64_t q = p.dir_cptr[R]; q < p.dir_cptr[R + 1]; ++q) {
                    const int off = p.dir_coff[q];
                    if (p.bcnz) F -= (double)myRow[off] * p.dir_bc[p.vcol[vb + off]];
                    myRow[off] = Real(0);
                }
            }
        }
        bad |= !isfinite(F);
        rhs[R] = F;
    }
    __syncwarp();
    const Real fin = write_out_range<Real>(sC, shift, clen, cbase, vals, p.vec_ok, lane);
    bad |= !isfinite(fin);
    if (bad) atomicExch(status, ANIGPU_ERR_NONFINITE);
}

// Vector P2 edge rows (component c = blockIdx.y) in ring order: the scalar rings, each column of the
// scalar row standing for its three component columns d L + offset (the vector row repeats the
// scalar row's columns once per column component d).  Per tet and d the element row is the scalar
// edge row's Gram formula with G replaced by B^{cd} in ring roles; A, B and the edge are summed in
// registers and the face columns carried, as in edge_ring_kernel, so every value is written once.
template <typename Real, bool DIR>
__global__ void __launch_bounds__(64) vec_edge_ring_kernel(RowParams p, int64_t nds, const int64_t* __restrict__ vrowptr,
                                                           const uint2* __restrict__ ring,
                                                           const int64_t* __restrict__ woff,
                                                           const Real* __restrict__ tetB, Real* __restrict__ vals,
                                                           double* __restrict__ rhs, int* __restrict__ status) {
    constexpr int VEC = 16 / (int)sizeof(Real);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    const int c = blockIdx.y;
    const int64_t wg = (int64_t)blockIdx.x * nwarps + warp;
    const int64_t row0 = p.row_begin + wg * 32;
    if (row0 >= p.nrows) return;  // warp-uniform; no block-wide barrier follows
    const int64_t rend = row0 + 32 < p.nrows ? row0 + 32 : p.nrows;
    const int64_t cbase = vrowptr[c * nds + row0];
    const int clen = (int)(vrowptr[c * nds + rend] - cbase);
    const int shift = (int)(cbase & (VEC - 1));
    const size_t chunk_bytes = (((size_t)32 * 3 * p.cap + VEC) * sizeof(Real) + 15) / 16 * 16;
    unsigned char* wbase = smem_raw + chunk_bytes * warp;
    Real* sC = reinterpret_cast<Real*>(wbase) + shift;
    if (!RING_NOZERO) {  // every column is written by the walk (or, in a Dirichlet row, cleared below)
        const int nvec = (shift + clen + VEC - 1) / VEC;
        int4* z = reinterpret_cast<int4*>(wbase);
        for (int k = lane; k < nvec; k += 32) z[k] = make_int4(0, 0, 0, 0);
    }
    const int64_t r = row0 + lane;
    const int64_t R = c * nds + r;
    const bool valid = r < p.nrows;
    const uint2* rr = ring + (p.wstride > 0 ? wg * p.wstride : woff[wg]) + lane;
    int deg = 0, base = 0, L = 0;
    bool isdir = false;
    uint2 hd = make_uint2(0u, 0u);
    if (valid) {
        deg = (int)(p.inc_ptr[r + 1] - p.inc_ptr[r]);
        base = (int)(vrowptr[R] - cbase);
        L = (int)(p.rowptr[r + 1] - p.rowptr[r]);
        if (DIR) isdir = p.dir_mask[R] != 0;
        hd = rr[0];
    }
    __syncwarp();
    Real* myRow = sC + base;
    const int nloop = isdir ? 0 : deg;
    const int last = nloop - 1;
    constexpr int KD = VRING_KD, RD = VRING_RD;
    static_assert(RD < 16, "the first records may reach RD slots past the lane's own (kRecPad)");
    VBlock<Real> Kq[KD];
    uint2 Rq[RD];
#pragma unroll
    for (int j = 0; j < KD; ++j) Kq[j].zero();
#pragma unroll
    for (int j = 0; j < RD; ++j) Rq[j] = make_uint2(0u, 0u);
#pragma unroll
    for (int j = 0; j < RD; ++j)
        if (REC_AHEAD || j <= last) Rq[j] = rr[32 * (j + 1)];
#pragma unroll
    for (int j = 0; j < KD; ++j)
        if (j <= last) Kq[j].load(tetB + 16 * (int64_t)(Rq[j].x & kRingTetMask));
    const bool closed = (hd.x >> 24) & 1u;
    Real cP[3], cAP[3], cBP[3], fP[3], fAP[3], fBP[3], accA[3], accB[3], accE[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) cP[d] = cAP[d] = cBP[d] = fP[d] = fAP[d] = fBP[d] = accA[d] = accB[d] = accE[d] = Real(0);
    uint32_t coff = hd.y;
    Real racc = Real(0);
    const Real m2 = Real(-0.2), p6 = Real(0.6), p8 = Real(0.8), p16 = Real(1.6);
    for (int k = 0; k < nloop; ++k) {
        VBlock<Real> Kn;
        if (k + KD <= last) Kn.load(tetB + 16 * (int64_t)(Rq[KD].x & kRingTetMask));
        uint2 Rn = make_uint2(0u, 0u);
        if (k + RD <= last) Rn = rr[32 * (k + RD + 1)];
        const uint2 r0 = Rq[0];
        const Real* bv = Kq[0].v;
        const Real lam = bv[9], mu = bv[10];
        // local vertices of the ring roles: local edge le = (a, b), others c_ < d_
        const int le = (int)((r0.x >> 27) & 7u);
        const int la = le <= 2 ? 0 : (le <= 4 ? 1 : 2);
        const int lb = le == 0 ? 1 : ((le == 1 || le == 3) ? 2 : 3);
        const int lc = le <= 2 ? (le == 0 ? 2 : 1) : 0;
        const int ld = 6 - la - lb - lc;
        const bool sab = (r0.x >> 30) & 1u, scd = (r0.x >> 31) & 1u;
        Real gA[3], gB[3], gP[3], gN[3];
        gvec(bv, sab ? lb : la, gA);
        gvec(bv, sab ? la : lb, gB);
        gvec(bv, scd ? ld : lc, gP);
        gvec(bv, scd ? lc : ld, gN);
        const Real gAc = sel3(gA, c), gBc = sel3(gB, c), gPc = sel3(gP, c), gNc = sel3(gN, c);
        const Real dAB = gA[0] * gB[0] + gA[1] * gB[1] + gA[2] * gB[2];
        const Real dAP = gA[0] * gP[0] + gA[1] * gP[1] + gA[2] * gP[2];
        const Real dAN = gA[0] * gN[0] + gA[1] * gN[1] + gA[2] * gN[2];
        const Real dBP = gB[0] * gP[0] + gB[1] * gP[1] + gB[2] * gP[2];
        const Real dBN = gB[0] * gN[0] + gB[1] * gN[1] + gB[2] * gN[2];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const Real BAB = lameB(lam, mu, gA, gAc, gB, gBc, dAB, c, d);
            const Real BBA = lameB(lam, mu, gB, gBc, gA, gAc, dAB, c, d);
            const Real BAP = lameB(lam, mu, gA, gAc, gP, gPc, dAP, c, d);
            const Real BAN = lameB(lam, mu, gA, gAc, gN, gNc, dAN, c, d);
            const Real BBP = lameB(lam, mu, gB, gBc, gP, gPc, dBP, c, d);
            const Real BBN = lameB(lam, mu, gB, gBc, gN, gNc, dBN, c, d);
            const Real BAA = -((BAB + BAP) + BAN), BBB = -((BBA + BBP) + BBN);
            accA[d] += fma(m2, BAA, p6 * BBA);
            accB[d] += fma(p6, BAB, m2 * BBB);
            accE[d] += fma(p16, BAA + BBB, p8 * (BAB + BBA));
            const Real vP = m2 * (BAP + BBP), vN = m2 * (BAN + BBN);
            const Real vAP = fma(p8, (BAA + BAP) + BBA, p16 * BBP), vAN = fma(p8, (BAA + BAN) + BBA, p16 * BBN);
            const Real vBP = fma(p8, (BAB + BBB) + BBP, p16 * BAP), vBN = fma(p8, (BAB + BBB) + BBN, p16 * BAN);
            const Real oP = cP[d] + vP, oAP = cAP[d] + vAP, oBP = cBP[d] + vBP;
            Real* rowd = myRow + d * L;
            if (k == 0 && closed) {
                fP[d] = oP;
                fAP[d] = oAP;
                fBP[d] = oBP;
            } else {
                rowd[coff & 255u] = oP;
                rowd[(coff >> 8) & 255u] = oAP;
                rowd[(coff >> 16) & 255u] = oBP;
            }
            rowd[r0.y >> 24] = p8 * ((BAP + BAN) + (BBP + BBN));
            cP[d] = vN;
            cAP[d] = vAN;
            cBP[d] = vBN;
        }
        racc += Real(0.2) * bv[11];
        coff = r0.y;
#pragma unroll
        for (int j = 0; j + 1 < KD; ++j) Kq[j] = Kq[j + 1];
        Kq[KD - 1] = Kn;
#pragma unroll
        for (int j = 0; j + 1 < RD; ++j) Rq[j] = Rq[j + 1];
        Rq[RD - 1] = Rn;
    }
    bool bad = false;
    if (valid) {
        double F;
        if (DIR && isdir) {
            if (RING_NOZERO)
                for (int q = 0; q < 3 * L; ++q) myRow[q] = Real(0);
            if (deg > 0) myRow[c * L + (int)((hd.x >> 16) & 255u)] = Real(deg);  // diagonal: the edge itself
            const double bcr = p.bcnz ? p.dir_bc[R] : 0.0;
            F = 0;
            for (int q = 0; q < deg; ++q) F += bcr;
        } else {
            if (nloop > 0) {
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    Real* rowd = myRow + d * L;
                    rowd[coff & 255u] = cP[d] + fP[d];
                    rowd[(coff >> 8) & 255u] = cAP[d] + fAP[d];
                    rowd[(coff >> 16) & 255u] = cBP[d] + fBP[d];
                    rowd[hd.x & 255u] = accA[d];
                    rowd[(hd.x >> 8) & 255u] = accB[d];
                    rowd[(hd.x >> 16) & 255u] = accE[d];
                }
            }
            F = (double)racc;
            if (DIR) {
                // Dirichlet columns: F -= A(i,k) bc_k with the assembled A(i,k), then the column is eliminated
                const int64_t vb = vrowptr[R];
                for (int64_t q = p.dir_cptr[R]; q < p.dir_cptr[R + 1]; ++q) {
                    const int off = p.dir_coff[q];
                    if (p.bcnz) F -= (double)myRow[off] * p.dir_bc[p.vcol[vb + off]];
                    myRow[off] = Real(0);
                }
            }
        }
        bad |= !isfinite(F);
        rhs[R] = F;
    }
    __syncwarp();
    const Real fin = write_out_range<Real>(sC, shift, clen, cbase, vals, p.vec_ok, lane);
    bad |= !isfinite(fin);
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
// Scatter of caller-computed element matrices (P1, P2, FemVec<3,P2>; the local-assembler contract):
// one warp per row; for every incidence in the records' order (ascending tets) lane d*nloc + c adds
// the element row's entry at component d, canonical column c: A_t(ci, d canon_local(i, c)), at the
// record's offset of that column in block d of the row (a vector row (c, r) holds block d = the
// scalar row's columns of component d).  The columns of one incidence are distinct, so every entry
// sums its contributions in tet order.  Dirichlet rows: zero except the diagonal = number of
// incident tets; Dirichlet columns of the other rows: A(i, k) bc_k moved to the right-hand side,
// then zeroed.
__global__ void elements_gather_kernel(int64_t nds, int ncomp, int nloc, int cap, const int64_t* __restrict__ rowptr,
                                       const int32_t* __restrict__ col, const int64_t* __restrict__ rowptr_s,
                                       const int64_t* __restrict__ inc_ptr, const ScatterRec* __restrict__ recs,
                                       const double* __restrict__ A, const double* __restrict__ F,
                                       const uint8_t* __restrict__ dir_mask, const double* __restrict__ dir_bc,
                                       int dir, int bcnz, double* __restrict__ vals, double* __restrict__ rhs,
                                       int* __restrict__ status) {
    extern __shared__ double erow[];  // per warp: the row being summed (cap values)
    __shared__ int8_t canon[100];     // canon_local(nloc, i, c) at i * nloc + c
    for (int k = threadIdx.x; k < nloc * nloc; k += blockDim.x) canon[k] = (int8_t)canon_local(nloc, k / nloc, k % nloc);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t R = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (R >= nds * ncomp) return;  // warp-uniform; no block-wide barrier follows
    double* row = erow + (size_t)(threadIdx.x >> 5) * cap;
    const int c = (int)(R / nds);
    const int64_t r = R - (int64_t)c * nds;
    const int NL = ncomp * nloc;
    const int64_t b = rowptr[R];
    const int len = (int)(rowptr[R + 1] - b);
    const int L = (int)(rowptr_s[r + 1] - rowptr_s[r]);
    for (int k = lane; k < len; k += 32) row[k] = 0.0;
    __syncwarp();
    const int64_t q0 = inc_ptr[r], q1 = inc_ptr[r + 1];
    const bool isdir = dir && dir_mask[R];
    double f = 0.0, fd = 0.0;
    if (!isdir) {
        const int d = lane / nloc, cc = lane - d * nloc;
        for (int64_t q = q0; q < q1; ++q) {
            const ScatterRec rec = recs[q];
            const int64_t t = rec.tet;
            const int i = (int)(rec.meta & 15u);
            if (lane < NL) {
                const uint32_t w = cc < 4 ? rec.off03 : (cc < 8 ? rec.off47 : (rec.meta >> 16));
                const int o = (int)byte_of(w, cc);
                row[d * L + o] += A[(size_t)NL * NL * t + (c * nloc + i) + (size_t)NL * (d * nloc + canon[i * nloc + cc])];
            }
            __syncwarp();
            if (F) f += F[(int64_t)NL * t + c * nloc + i];
        }
        if (dir) {
            for (int k = lane; k < len; k += 32)
                if (dir_mask[col[b + k]]) {
                    if (bcnz) fd += row[k] * dir_bc[col[b + k]];
                    row[k] = 0.0;
                }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) fd += __shfl_xor_sync(0xffffffffu, fd, o);
            f -= fd;
        }
    } else {
        if (lane == 0 && q1 > q0) {
            const ScatterRec rd = recs[q0];
            const int dc = canon_diag(nloc, (int)(rd.meta & 15u));
            row[c * L + (int)byte_of(dc < 4 ? rd.off03 : rd.off47, dc)] = (double)(q1 - q0);
        }
        const double bcr = bcnz ? dir_bc[R] : 0.0;
        for (int64_t q = q0; q < q1; ++q) f += bcr;
    }
    __syncwarp();
    bool bad = !isfinite(f);
    for (int k = lane; k < len; k += 32) {
        const double v = row[k];
        bad |= !isfinite(v);
        vals[b + k] = v;
    }
    if (__any_sync(0xffffffffu, bad) && lane == 0) atomicExch(status, ANIGPU_ERR_NONFINITE);
    if (rhs && lane == 0) rhs[R] = f;
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

// columns of every row i of the [i][j][8] tables into the canonical order of row i
static void to_canonical(int nf, double* T) {
    std::vector<double> row((size_t)nf * 8);
    for (int i = 0; i < nf; ++i) {
        double* Ti = T + (size_t)i * nf * 8;
        for (int c = 0; c < nf; ++c)
            for (int k = 0; k < 8; ++k) row[(size_t)c * 8 + k] = Ti[(size_t)canon_local(nf, i, c) * 8 + k];
        std::copy(row.begin(), row.end(), Ti);
    }
}

// host: Tsym tables (canonical columns) and m for (space, order) in precision
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
    to_canonical(nf, T.data());
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

template <typename Real, int NLOC, int FORM, bool DIR, bool BCNZ, bool TOUCH, bool DROPCHK>
static int launch_rows_t(anigpu_ctx* h, const RowParams& p, const void* tables, void* vals, double* rhs,
                         uint8_t* touched, cudaStream_t st) {
    const int warps = h->row_warps == 1 ? 1 : 2;  // at most 64 threads (the kernel's launch bounds)
    const size_t smem = RowSmem<Real, NLOC, FORM, TOUCH>::total(p.cap, warps);
    auto kern = row_gather_kernel<Real, NLOC, FORM, DIR, BCNZ, TOUCH, DROPCHK>;
    static int smem_set[64] = {};  // per device: the largest dynamic shared memory set so far
    const int slot = h->device >= 0 && h->device < 64 ? h->device : 0;
    if ((int)smem > smem_set[slot]) {
        ANI_CUDA(h, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        smem_set[slot] = (int)smem;
    }
    kern<<<grid_for(p.nrows - p.row_begin, 32 * warps), 32 * warps, smem, st>>>(
        p, (const Real*)tables, (const Real*)h->tetdata, (Real*)vals, rhs, touched, h->d_status);
    ANI_LAUNCHED(h);
    return ANIGPU_OK;
}

template <typename Real, bool DIR, bool DROPCHK, bool TR = false>
static int launch_ring_t(anigpu_ctx* h, const RowParams& p, void* vals, double* rhs, cudaStream_t st) {
    const int warps = h->row_warps == 1 ? 1 : 2;
    const size_t smem = RowSmem<Real, 10, 2, false>::total(p.cap, warps);
    auto kern = edge_ring_kernel<Real, DIR, DROPCHK>;
    static int smem_set[64] = {};
    const int slot = h->device >= 0 && h->device < 64 ? h->device : 0;
    if ((int)smem > smem_set[slot]) {
        if constexpr (TR)
            ANI_CUDA(h, cudaFuncSetAttribute(edge_ring_tr_kernel<Real, DIR, DROPCHK>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        else
            ANI_CUDA(h, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        smem_set[slot] = (int)smem;
    }
    // launched right behind the per-tet kernel on the same stream (h->asm_pdl): a programmatic
    // dependency, so that its blocks start (and set up) while that kernel's last wave runs
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid_for(p.nrows - p.row_begin, 32 * warps));
    cfg.blockDim = dim3(32 * warps);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = h->asm_pdl ? 1 : 0;
    RowParams q = p;
    q.wstride = h->ring_ws;
    if constexpr (TR)
        ANI_CUDA(h, cudaLaunchKernelEx(&cfg, edge_ring_tr_kernel<Real, DIR, DROPCHK>, q, (const uint2*)h->ring,
                                       (const int64_t*)h->ring_woff, (const Real*)h->tetdata, (Real*)vals, rhs,
                                       h->d_status, (const int32_t*)h->tpos, (const int64_t*)h->tpos_woff,
                                       h->tpos_ws));
    else
        ANI_CUDA(h, cudaLaunchKernelEx(&cfg, kern, q, (const uint2*)h->ring, (const int64_t*)h->ring_woff,
                                       (const Real*)h->tetdata, (Real*)vals, rhs, h->d_status));
    ANI_LAUNCHED(h);
    return ANIGPU_OK;
}

// the vertex pass behind the edge walks that stored the vertex rows' off-diagonal entries
template <typename Real, bool DIR, bool DROPCHK>
static int launch_vtr_t(anigpu_ctx* h, const RowParams& p, void* vals, double* rhs, cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid_for(p.nrows - p.row_begin, 128));
    cfg.blockDim = dim3(128);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = h->asm_pdl ? 1 : 0;
    RowParams q = p;
    q.wstride = h->vrec_ws;
    ANI_CUDA(h, cudaLaunchKernelEx(&cfg, vertex_tr_kernel<Real, DIR, DROPCHK>, q, (const uint32_t*)h->vrec4,
                                   (const int64_t*)h->vrec_woff, (const int32_t*)h->vdiag, (const Real*)h->tetdata,
                                   (Real*)vals, rhs, h->d_status));
    ANI_LAUNCHED(h);
    return ANIGPU_OK;
}

// P2 vertex rows by symmetry: the edge walks with their transposed stores, then the vertex pass,
// both behind the per-tet kernel on its stream
template <typename Real>
static int launch_tr(anigpu_ctx* h, const RowParams& p0, void* vals, double* rhs) {
    const bool dir = h->has_dirichlet;
    const bool dchk = sizeof(Real) == 8 || (float)p0.drop != 0.0f;
    RowParams p = p0;
    p.row_begin = h->row_range[1];
    p.nrows = h->row_range[2];
    p.cap = h->row_range_cap[1];
    int rc;
    if (dchk) rc = dir ? launch_ring_t<Real, true, true, true>(h, p, vals, rhs, h->stream)
                       : launch_ring_t<Real, false, true, true>(h, p, vals, rhs, h->stream);
    else rc = dir ? launch_ring_t<Real, true, false, true>(h, p, vals, rhs, h->stream)
                  : launch_ring_t<Real, false, false, true>(h, p, vals, rhs, h->stream);
    if (rc) return rc;
    p.row_begin = h->row_range[0];
    p.nrows = h->row_range[1];
    p.cap = h->row_range_cap[0];
    if (dchk) return dir ? launch_vtr_t<Real, true, true>(h, p, vals, rhs, h->stream)
                         : launch_vtr_t<Real, false, true>(h, p, vals, rhs, h->stream);
    return dir ? launch_vtr_t<Real, true, false>(h, p, vals, rhs, h->stream)
               : launch_vtr_t<Real, false, false>(h, p, vals, rhs, h->stream);
}

template <typename Real, int NLOC, bool DIR, bool DROPCHK>
static int launch_vilv_t(anigpu_ctx* h, const RowParams& p, void* vals, double* rhs, cudaStream_t st) {
    const int warps = h->row_warps == 1 ? 1 : 2;
    const size_t smem = RowSmem<Real, NLOC, 1, false>::total(p.cap, warps);
    auto kern = vertex_ilv_kernel<Real, NLOC, DIR, DROPCHK>;
    static int smem_set[64] = {};
    const int slot = h->device >= 0 && h->device < 64 ? h->device : 0;
    if ((int)smem > smem_set[slot]) {
        ANI_CUDA(h, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        smem_set[slot] = (int)smem;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid_for(p.nrows - p.row_begin, 32 * warps));
    cfg.blockDim = dim3(32 * warps);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = h->asm_pdl ? 1 : 0;
    RowParams q = p;
    q.wstride = h->vrec_ws;
    ANI_CUDA(h, cudaLaunchKernelEx(&cfg, kern, q, (const ScatterRec*)h->vrec, (const int64_t*)h->vrec_woff,
                                   (const Real*)h->tetdata, (Real*)vals, rhs, h->d_status));
    ANI_LAUNCHED(h);
    return ANIGPU_OK;
}

// vertex rows (Gram form) from the interleaved records under the same conditions as the rings;
// returns 1 when it did not launch
template <typename Real, int NLOC>
static int launch_vilv(anigpu_ctx* h, const RowParams& p, void* vals, double* rhs, uint8_t* touched,
                       cudaStream_t st, int* rc) {
    if (!h->vrec || !h->ring_enabled || touched || (h->has_dirichlet && h->bc_nonzero) || p.row_begin != 0) return 1;
    const bool dir = h->has_dirichlet;
    const bool dchk = sizeof(Real) == 8 || (float)p.drop != 0.0f;
    if (dchk) *rc = dir ? launch_vilv_t<Real, NLOC, true, true>(h, p, vals, rhs, st)
                        : launch_vilv_t<Real, NLOC, false, true>(h, p, vals, rhs, st);
    else *rc = dir ? launch_vilv_t<Real, NLOC, true, false>(h, p, vals, rhs, st)
                   : launch_vilv_t<Real, NLOC, false, false>(h, p, vals, rhs, st);
    return 0;
}

// P2 edge rows in ring order where the mesh has rings and the call needs neither a touched map nor
// per-value Dirichlet masks (non-zero boundary values); returns 1 when it did not launch
template <typename Real>
static int launch_ring(anigpu_ctx* h, const RowParams& p, void* vals, double* rhs, uint8_t* touched,
                       cudaStream_t st, int* rc) {
    if (!h->ring_ok || !h->ring_enabled || touched || (h->has_dirichlet && h->bc_nonzero) || p.row_begin != h->row_range[1]) return 1;
    const bool dir = h->has_dirichlet;
    const bool dchk = sizeof(Real) == 8 || (float)p.drop != 0.0f;
    if (dchk) *rc = dir ? launch_ring_t<Real, true, true>(h, p, vals, rhs, st) : launch_ring_t<Real, false, true>(h, p, vals, rhs, st);
    else *rc = dir ? launch_ring_t<Real, true, false>(h, p, vals, rhs, st) : launch_ring_t<Real, false, false>(h, p, vals, rhs, st);
    return 0;
}

// lane-interleaved records of the vertex rows [0, row_range[1]) (P1: every row)
#ifndef WS_UNIFORM
#define WS_UNIFORM 1
#endif

// slots of the lane-interleaved layout of rows [rb, re) (head + incidences per lane, 32 lanes per
// warp): per-warp offsets (*woff, nwarps + 1 entries) and the total.  When a uniform stride (every
// warp the largest warp's slots) costs at most a quarter more slots, the offsets are w * stride and
// *ws = stride: a warp then finds its records without loading its offset first.
static int warp_layout(anigpu_ctx* h, int64_t rb, int64_t re, int head, int64_t** woff, int64_t* total,
                       int64_t* ws) {
    cudaStream_t s = h->stream;
    const int64_t n = re - rb, nw = (n + 31) / 32;
    *ws = 0;
    unsigned long long* cnt = nullptr;  // nw counts, the scan's zero, the largest count
    ANI_CUDA(h, cudaMallocAsync((void**)&cnt, sizeof(unsigned long long) * (nw + 2), s));
    ANI_CUDA(h, cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * (nw + 2), s));
    warp_slots_kernel<<<grid_for(n, 256), 256, 0, s>>>(rb, re, head, h->inc_ptr, cnt, cnt + nw + 1);
    ANI_LAUNCHED(h);
    int rc = dev_alloc(h, woff, (size_t)nw + 1);
    if (!rc) rc = scan_counts(h, cnt, nw, *woff);
    int64_t tot = 0;
    unsigned long long mx = 0;
    if (!rc) {
        ANI_CUDA(h, cudaMemcpyAsync(&tot, *woff + nw, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        ANI_CUDA(h, cudaMemcpyAsync(&mx, cnt + nw + 1, sizeof(mx), cudaMemcpyDeviceToHost, s));
        ANI_CUDA(h, cudaStreamSynchronize(s));
    }
    ANI_CUDA(h, cudaFreeAsync(cnt, s));
    if (rc) return rc;
    if (WS_UNIFORM && nw * (int64_t)mx <= tot + tot / 4) {
        uniform_offsets_kernel<<<grid_for(nw + 1, 256), 256, 0, s>>>(nw, (int64_t)mx, *woff);
        ANI_LAUNCHED(h);
        tot = nw * (int64_t)mx;
        *ws = (int64_t)mx;
    }
    *total = tot;
    return ANIGPU_OK;
}

static int setup_vertex_ilv(anigpu_ctx* h) {
    if (h->vrec) cudaFree(h->vrec);
    if (h->vrec_woff) cudaFree(h->vrec_woff);
    h->vrec = nullptr;
    h->vrec_woff = nullptr;
    h->vrec_ws = 0;
    if (h->space != ANIGPU_P1 && h->space != ANIGPU_P2) return ANIGPU_OK;
    const int64_t rb = h->row_range[0], re = h->row_range[1];
    if (re <= rb) return ANIGPU_OK;
    cudaStream_t s = h->stream;
    const int64_t n = re - rb;
    int64_t total = 0;
    int rc = warp_layout(h, rb, re, 0, &h->vrec_woff, &total, &h->vrec_ws);
    if (rc) return rc;
    rc = dev_alloc(h, &h->vrec, (size_t)(total + kRecPad));
    if (rc) return rc;
    ANI_CUDA(h, cudaMemsetAsync(h->vrec, 0, sizeof(ScatterRec) * (size_t)(total + kRecPad), s));
    vertex_ilv_build_kernel<<<grid_for(n, 128), 128, 0, s>>>(rb, re, h->inc_ptr, h->recs, h->vrec_woff, h->vrec);
    ANI_LAUNCHED(h);
    return ANIGPU_OK;
}

#ifndef VERTEX_TR
#define VERTEX_TR 1
#endif

// the transposed positions and the vertex rows' incidence words (P2 with rings); left out (and the
// vertex rows gathered by their own walk) when a position is missing or the values do not fit
static int setup_vertex_tr(anigpu_ctx* h) {
    void* ptrs[] = {h->tpos, h->tpos_woff, h->vrec4, h->vdiag};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    h->tpos = nullptr;
    h->tpos_woff = nullptr;
    h->vrec4 = nullptr;
    h->vdiag = nullptr;
    h->tpos_ws = 0;
    h->tr_ok = false;
    if (!VERTEX_TR || h->space != ANIGPU_P2 || !h->ring_ok || !h->vrec || h->nnz_s >= (int64_t)INT32_MAX) return ANIGPU_OK;
    const int64_t vb = h->row_range[0], ve = h->row_range[1], rb = h->row_range[1], re = h->row_range[2];
    if (ve <= vb || re <= rb) return ANIGPU_OK;
    cudaStream_t s = h->stream;
    int64_t total = 0;
    int rc = warp_layout(h, rb, re, 5, &h->tpos_woff, &total, &h->tpos_ws);
    if (rc) return rc;
    rc = dev_alloc(h, &h->tpos, (size_t)(total + kRecPad));
    if (rc) return rc;
    ANI_CUDA(h, cudaMemsetAsync(h->tpos, 0, sizeof(int32_t) * (size_t)(total + kRecPad), s));
    const int64_t nwv = (ve - vb + 31) / 32;
    int64_t vtotal = 0;
    ANI_CUDA(h, cudaMemcpyAsync(&vtotal, h->vrec_woff + nwv, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    ANI_CUDA(h, cudaStreamSynchronize(s));
    rc = dev_alloc(h, &h->vrec4, (size_t)(vtotal + kRecPad));
    if (rc) return rc;
    ANI_CUDA(h, cudaMemsetAsync(h->vrec4, 0, sizeof(uint32_t) * (size_t)(vtotal + kRecPad), s));
    rc = dev_alloc(h, &h->vdiag, (size_t)(ve - vb));
    if (rc) return rc;
    int* fail = nullptr;
    ANI_CUDA(h, cudaMallocAsync((void**)&fail, sizeof(int), s));
    ANI_CUDA(h, cudaMemsetAsync(fail, 0, sizeof(int), s));
    tpos_build_kernel<<<grid_for(re - rb, 128), 128, 0, s>>>(rb, re, h->inc_ptr, h->ring, h->ring_woff, h->tets,
                                                             h->rowptr_s, h->col_s, h->tpos_woff, h->tpos, fail);
    ANI_LAUNCHED(h);
    vertex4_build_kernel<<<grid_for(ve - vb, 128), 128, 0, s>>>(vb, ve, h->inc_ptr, h->recs, h->rowptr_s, h->col_s,
                                                                h->vrec_woff, h->vrec4, h->vdiag, fail);
    ANI_LAUNCHED(h);
    int hf = 0;
    ANI_CUDA(h, cudaMemcpyAsync(&hf, fail, sizeof(int), cudaMemcpyDeviceToHost, s));
    ANI_CUDA(h, cudaStreamSynchronize(s));
    ANI_CUDA(h, cudaFreeAsync(fail, s));
    if (hf) {
        void* q2[] = {h->tpos, h->tpos_woff, h->vrec4, h->vdiag};
        for (void* q : q2) cudaFree(q);
        h->tpos = nullptr;
        h->tpos_woff = nullptr;
        h->vrec4 = nullptr;
        h->vdiag = nullptr;
        h->tpos_ws = 0;
        return ANIGPU_OK;
    }
    h->tr_ok = true;
    return ANIGPU_OK;
}

int setup_row_layouts(anigpu_ctx* h) {
    int rc = setup_vertex_ilv(h);
    if (rc) return rc;
    h->ring_ok = false;
    h->tr_ok = false;
    if (h->ring) cudaFree(h->ring);
    if (h->ring_woff) cudaFree(h->ring_woff);
    h->ring = nullptr;
    h->ring_woff = nullptr;
    h->ring_ws = 0;
    if ((h->space != ANIGPU_P2 && h->space != ANIGPU_VEC3_P2) || h->nt - 1 > (int64_t)kRingTetMask) return ANIGPU_OK;
    const int64_t rb = h->row_range[1], re = h->row_range[2];
    if (re <= rb) return ANIGPU_OK;
    cudaStream_t s = h->stream;
    const int64_t n = re - rb;
    int64_t total = 0;
    rc = warp_layout(h, rb, re, 1, &h->ring_woff, &total, &h->ring_ws);
    if (rc) return rc;
    rc = dev_alloc(h, &h->ring, (size_t)(total + kRecPad));
    if (rc) return rc;
    ANI_CUDA(h, cudaMemsetAsync(h->ring, 0, sizeof(uint2) * (size_t)(total + kRecPad), s));
    int* fail = nullptr;
    ANI_CUDA(h, cudaMallocAsync((void**)&fail, sizeof(int), s));
    ANI_CUDA(h, cudaMemsetAsync(fail, 0, sizeof(int), s));
    ring_build_kernel<<<grid_for(n, 128), 128, 0, s>>>(rb, re, h->inc_ptr, h->recs, h->tets, h->rowptr_s,
                                                       h->ring_woff, h->ring, fail);
    ANI_LAUNCHED(h);
    int hf = 0;
    ANI_CUDA(h, cudaMemcpyAsync(&hf, fail, sizeof(int), cudaMemcpyDeviceToHost, s));
    ANI_CUDA(h, cudaStreamSynchronize(s));
    ANI_CUDA(h, cudaFreeAsync(fail, s));
    if (hf) {
        cudaFree(h->ring);
        cudaFree(h->ring_woff);
        h->ring = nullptr;
        h->ring_woff = nullptr;
        h->ring_ws = 0;
        return ANIGPU_OK;
    }
    h->ring_ok = true;
    return setup_vertex_tr(h);
}

template <typename Real, int NLOC, int FORM>
static int launch_rows(anigpu_ctx* h, const RowParams& p, const void* tables, void* vals, double* rhs,
                       uint8_t* touched, cudaStream_t st) {
    const bool dir = h->has_dirichlet, bcnz = h->bc_nonzero, tch = touched != nullptr;
    // FP32 template assembly with a drop value that is zero in FP32 needs no drop test
    const bool dchk = tch || sizeof(Real) == 8 || (float)p.drop != 0.0f;
#define LR(D, B, T, C) return launch_rows_t<Real, NLOC, FORM, D, B, T, C>(h, p, tables, vals, rhs, touched, st)
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

// vector P2 with the Lame tensor: tet blocks, then vertex-row and edge-row gathers (x 3 components)
static int run_assemble_vec(anigpu_ctx* h, int kind, const double* D, const double* f, double f_const, int order,
                            int precision, void* vals, double* rhs, uint8_t* touched, double drop_val) {
    (void)drop_val;
    if (kind != ANIGPU_TENSOR_LAME)
        return set_err(h, ANIGPU_ERR_UNSUPPORTED, "vector P2 assembly takes ANIGPU_TENSOR_LAME (lambda, mu per tet)");
    if (order < 2)
        return set_err(h, ANIGPU_ERR_UNSUPPORTED, "vector P2 assembly needs quadrature order >= 2 (exact integration)");
    if (!D) return set_err(h, ANIGPU_ERR_ARG, "tensor data is NULL");
    if (!vals || !rhs) return set_err(h, ANIGPU_ERR_ARG, "NULL output");
    if (touched) return set_err(h, ANIGPU_ERR_UNSUPPORTED, "no touched map for vector P2 assembly");
    if (precision != ANIGPU_F32 && precision != ANIGPU_F64) return set_err(h, ANIGPU_ERR_ARG, "precision");
    const double *pp, *ww;
    int q;
    if (!anigpu_quad_rule(order, &pp, &ww, &q)) return set_err(h, ANIGPU_ERR_UNSUPPORTED, "quadrature order");
    const size_t rsz = precision == ANIGPU_F32 ? 4 : 8;
    const size_t need = (size_t)h->nt * 16 * rsz;
    if (h->tetdata_bytes < need) {
        if (h->tetdata) cudaFree(h->tetdata);
        h->tetdata = nullptr;
        ANI_CUDA(h, cudaMalloc(&h->tetdata, need));
        h->tetdata_bytes = need;
    }
    time_mark(h, 0);
    if (precision == ANIGPU_F32)
        tet_lame_f32_kernel<<<grid_for(h->nt, 256), 256, 0, h->stream>>>(h->nt, h->xyz, h->xyz2, h->tets, D, f, f_const,
                                                                       (float*)h->tetdata, h->d_status);
    else
        tet_lame_f64_kernel<<<grid_for(h->nt, 256), 256, 0, h->stream>>>(h->nt, h->xyz, h->tets, D, f, f_const,
                                                                       (double*)h->tetdata, h->d_status);
    ANI_LAUNCHED(h);
    time_mark(h, 1);
    RowParams p{};
    p.inc_ptr = h->inc_ptr;
    p.recs = h->recs;
    p.rowptr = h->rowptr_s;
    p.dir_mask = h->dir_mask;
    p.dir_bc = h->dir_bc;
    p.edofs = h->edofs;
    p.drop = 0;
    p.vec_ok = ((uintptr_t)vals % 16) == 0 ? 1 : 0;
    p.dir_cptr = h->dir_cptr;
    p.dir_coff = h->dir_coff;
    p.vcol = h->col;
    p.bcnz = h->bc_nonzero ? 1 : 0;
    p.wstride = h->ring_ws;
    cudaStream_t side = h->side_stream ? h->side_stream : h->stream;
    if (side != h->stream) {
        ANI_CUDA(h, cudaEventRecord(h->fork_ev, h->stream));
        ANI_CUDA(h, cudaStreamWaitEvent(side, h->fork_ev, 0));
    }
    const bool dir = h->has_dirichlet;
    for (int rg = 0; rg < 2; ++rg) {
        p.row_begin = h->row_range[rg];
        p.nrows = h->row_range[rg + 1];
        p.cap = h->row_range_cap[rg];
        if (p.nrows <= p.row_begin) continue;
        cudaStream_t st = rg == 0 ? side : h->stream;
        const int warps = 2;
        const size_t smem = ((((size_t)32 * 3 * p.cap + 16 / rsz) * rsz + 15) / 16 * 16) * warps;
        const dim3 grid(grid_for(p.nrows - p.row_begin, 32 * warps), 3);
#define VLAUNCH(R, F, DD)                                                                                          do {                                                                                                               auto kern = vec_row_gather_kernel<R, F, DD>;                                                                   ANI_CUDA(h, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));              kern<<<grid, 32 * warps, smem, st>>>(p, h->nds, h->rowptr, (const R*)h->tetdata, (R*)vals, rhs,                                                     h->d_status);                                                         } while (0)
        const bool ring = rg == 1 && h->ring_ok && h->ring_enabled;
#define VRING(R, DD)                                                                                               \
    do {                                                                                                           \
        auto kern = vec_edge_ring_kernel<R, DD>;                                                                   \
        ANI_CUDA(h, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));          \
        kern<<<grid, 32 * warps, smem, st>>>(p, h->nds, h->rowptr, h->ring, h->ring_woff, (const R*)h->tetdata,    \
                                             (R*)vals, rhs, h->d_status);                                          \
    } while (0)
        if (ring) {
            if (precision == ANIGPU_F32) { if (dir) VRING(float, true); else VRING(float, false); }
            else { if (dir) VRING(double, true); else VRING(double, false); }
        } else if (precision == ANIGPU_F32) {
            if (rg == 0) { if (dir) VLAUNCH(float, 1, true); else VLAUNCH(float, 1, false); }
            else { if (dir) VLAUNCH(float, 2, true); else VLAUNCH(float, 2, false); }
        } else {
            if (rg == 0) { if (dir) VLAUNCH(double, 1, true); else VLAUNCH(double, 1, false); }
            else { if (dir) VLAUNCH(double, 2, true); else VLAUNCH(double, 2, false); }
        }
#undef VLAUNCH
#undef VRING
        ANI_LAUNCHED(h);
    }
    if (side != h->stream) {
        ANI_CUDA(h, cudaEventRecord(h->join_ev, side));
        ANI_CUDA(h, cudaStreamWaitEvent(h->stream, h->join_ev, 0));
    }
    time_mark(h, 2);
    return ANIGPU_OK;
}

int run_assemble(anigpu_ctx* h, int kind, const double* D, const double* f, double f_const, int order,
                 int precision, void* vals, double* rhs, uint8_t* touched, double drop_val) {
    if (h->space < 0) return set_err(h, ANIGPU_ERR_STATE, "anigpu_problem_setup not called");
    if (is_general_space(h->space))
        return set_err(h, ANIGPU_ERR_UNSUPPORTED, "this space assembles through anigpu_assemble_general");
    if (h->space == ANIGPU_VEC3_P2)
        return run_assemble_vec(h, kind, D, f, f_const, order, precision, vals, rhs, touched, drop_val);
    if (kind != ANIGPU_TENSOR_NULL && kind != ANIGPU_TENSOR_CONST_SCALAR && kind != ANIGPU_TENSOR_TET_SCALAR &&
        kind != ANIGPU_TENSOR_TET_SYM)
        return set_err(h, ANIGPU_ERR_UNSUPPORTED, "assembly tensor kind must be NULL, CONST_SCALAR, TET_SCALAR or TET_SYM");
    if (kind != ANIGPU_TENSOR_NULL && !D) return set_err(h, ANIGPU_ERR_ARG, "tensor data is NULL");
    if (!vals || !rhs) return set_err(h, ANIGPU_ERR_ARG, "NULL output");
    if (precision != ANIGPU_F32 && precision != ANIGPU_F64) return set_err(h, ANIGPU_ERR_ARG, "precision");
    // Gram form where the quadrature is exact for the element integrals, table form otherwise
    const bool gram = h->space == ANIGPU_P1 || (h->space == ANIGPU_P2 && order >= 2);
    const void* tables = nullptr;
    int rc = ANIGPU_OK;
    if (!gram) {
        rc = get_row_tables(h, h->space, order, precision, &tables);
        if (rc) return rc;
    } else {
        const double *pp, *ww;
        int q;
        if (!anigpu_quad_rule(order, &pp, &ww, &q)) return set_err(h, ANIGPU_ERR_UNSUPPORTED, "quadrature order");
    }
    const size_t rsz = precision == ANIGPU_F32 ? 4 : 8;
    const size_t need = (size_t)h->nt * 8 * rsz;
    if (h->tetdata_bytes < need) {
        if (h->tetdata) cudaFree(h->tetdata);
        h->tetdata = nullptr;
        ANI_CUDA(h, cudaMalloc(&h->tetdata, need));
        h->tetdata_bytes = need;
    }
    time_mark(h, 0);
    if (gram) {
        if (precision == ANIGPU_F32)
            tet_gram_f32_kernel<<<grid_for(h->nt, 256), 256, 0, h->stream>>>(
                h->nt, h->xyz, h->xyz2, h->tets, kind, D, f, f_const, (float*)h->tetdata, h->d_status);
        else
            tet_gram_f64_kernel<<<grid_for(h->nt, 256), 256, 0, h->stream>>>(
                h->nt, h->xyz, h->tets, kind, D, f, f_const, (double*)h->tetdata, h->d_status);
    } else if (precision == ANIGPU_F32) {
        tet_prepare_f32_kernel<<<grid_for(h->nt, 256), 256, 0, h->stream>>>(
            h->nt, h->xyz, h->xyz2, h->tets, kind, D, f, f_const, (float*)h->tetdata, h->d_status);
    } else {
        tet_prepare_f64_kernel<<<grid_for(h->nt, 256), 256, 0, h->stream>>>(
            h->nt, h->xyz, h->tets, kind, D, f, f_const, (double*)h->tetdata, h->d_status);
    }
    ANI_LAUNCHED(h);
    time_mark(h, 1);
    RowParams p{};
    p.inc_ptr = h->inc_ptr;
    p.recs = h->recs;
    p.rowptr = h->rowptr_s;
    p.dir_mask = h->dir_mask;
    p.dir_bc = h->dir_bc;
    p.edofs = h->edofs;
    p.drop = drop_val;
    p.vec_ok = ((uintptr_t)vals % 16) == 0 ? 1 : 0;
    p.dir_cptr = h->dir_cptr;
    p.dir_coff = h->dir_coff;
    // one launch per row range (vertex rows, edge rows) so that the shared-memory row
    // buffer fits the longest row of that range.  With the ring and interleaved layouts the vertex
    // rows follow the per-tet kernel on its stream with a programmatic dependency and the edge rows
    // run concurrently on the side stream: the vertex rows' long walks are dispatched first and the
    // short edge-row blocks fill the SMs as they end (0.197 vs 0.205 ms per 64^3 FP32 assembly
    // against edge rows then vertex rows on one stream).  Otherwise the two ranges run concurrently
    // (the vertex range on the side stream) so that the tail of one overlaps the other.
    const bool seq = ASM_SEQ && gram && h->ring_enabled && !touched && !(h->has_dirichlet && h->bc_nonzero) &&
                     (h->nloc_s == 4 || h->ring_ok) && h->vrec;
    // FP64: the vertex rows by symmetry (their own walk is FP64-bound: 1.53 vs 1.78 ms per 64^3
    // assembly); FP32 keeps the vertex walk (the transposed stores cost more: 0.248 vs 0.195 ms)
    if (seq && h->tr_ok && precision == ANIGPU_F64 && h->nloc_s == 10 && h->row_range[1] > h->row_range[0] &&
        h->row_range[2] > h->row_range[1]) {
        h->asm_pdl = true;
        rc = launch_tr<double>(h, p, vals, rhs);
        h->asm_pdl = false;
        time_mark(h, 2);
        return rc;
    }
    const bool split = seq && ASM_SPLIT && h->nloc_s == 10 && h->side_stream;
    cudaStream_t side = h->side_stream && (!seq || split) ? h->side_stream : h->stream;
    if (side != h->stream) {
        ANI_CUDA(h, cudaEventRecord(h->fork_ev, h->stream));
        ANI_CUDA(h, cudaStreamWaitEvent(side, h->fork_ev, 0));
    }
    for (int it = 0; it < 2; ++it) {
        const int rg = seq && !split ? 1 - it : it;
        p.row_begin = h->row_range[rg];
        p.nrows = h->row_range[rg + 1];
        p.cap = h->row_range_cap[rg];
        if (p.nrows <= p.row_begin) continue;
        cudaStream_t st = seq ? (split && rg == 1 ? side : h->stream) : (rg == 0 ? side : h->stream);
        h->asm_pdl = seq && st == h->stream;
        const bool f32 = precision == ANIGPU_F32;
        if (h->nloc_s == 10) {
            if (!gram)
                rc = f32 ? launch_rows<float, 10, 0>(h, p, tables, vals, rhs, touched, st)
                         : launch_rows<double, 10, 0>(h, p, tables, vals, rhs, touched, st);
            else if (rg == 0) {
                if ((f32 ? launch_vilv<float, 10>(h, p, vals, rhs, touched, st, &rc)
                         : launch_vilv<double, 10>(h, p, vals, rhs, touched, st, &rc)) != 0)
                    rc = f32 ? launch_rows<float, 10, 1>(h, p, tables, vals, rhs, touched, st)
                             : launch_rows<double, 10, 1>(h, p, tables, vals, rhs, touched, st);
            }
            else if ((f32 ? launch_ring<float>(h, p, vals, rhs, touched, st, &rc)
                          : launch_ring<double>(h, p, vals, rhs, touched, st, &rc)) != 0)
                rc = f32 ? launch_rows<float, 10, 2>(h, p, tables, vals, rhs, touched, st)
                         : launch_rows<double, 10, 2>(h, p, tables, vals, rhs, touched, st);
        } else {
            if (!gram)
                rc = f32 ? launch_rows<float, 4, 0>(h, p, tables, vals, rhs, touched, st)
                         : launch_rows<double, 4, 0>(h, p, tables, vals, rhs, touched, st);
            else if ((f32 ? launch_vilv<float, 4>(h, p, vals, rhs, touched, st, &rc)
                          : launch_vilv<double, 4>(h, p, vals, rhs, touched, st, &rc)) != 0)
                rc = f32 ? launch_rows<float, 4, 1>(h, p, tables, vals, rhs, touched, st)
                         : launch_rows<double, 4, 1>(h, p, tables, vals, rhs, touched, st);
        }
        if (rc) {
            h->asm_pdl = false;
            return rc;
        }
    }
    h->asm_pdl = false;
    if (side != h->stream) {
        ANI_CUDA(h, cudaEventRecord(h->join_ev, side));
        ANI_CUDA(h, cudaStreamWaitEvent(h->stream, h->join_ev, 0));
    }
    time_mark(h, 2);
    return rc;
}

int elements_scatter(anigpu_ctx* h, const double* A, const double* F, double* vals, double* rhs) {
    if (h->space != ANIGPU_P1 && h->space != ANIGPU_P2 && h->space != ANIGPU_VEC3_P2)
        return set_err(h, ANIGPU_ERR_UNSUPPORTED, "element-matrix assembly: P1, P2, vector P2 or a general-path space");
    if (!A || !vals) return set_err(h, ANIGPU_ERR_ARG, "NULL element matrices or values");
    const int cap = h->max_row_len_s * h->ncomp;  // the longest row of the template
    const size_t smem = sizeof(double) * 8 * (size_t)cap;
    if (smem > 227 * 1024) return set_err(h, ANIGPU_ERR_UNSUPPORTED, "template rows too long for the element scatter");
    ANI_CUDA(h, cudaFuncSetAttribute(elements_gather_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    elements_gather_kernel<<<grid_for(h->nds * h->ncomp * 32, 256), 256, smem, h->stream>>>(
        h->nds, h->ncomp, h->nloc_s, cap, h->rowptr, h->col, h->rowptr_s, h->inc_ptr, h->recs, A, F, h->dir_mask,
        h->dir_bc, h->has_dirichlet ? 1 : 0, h->bc_nonzero ? 1 : 0, vals, rhs, h->d_status);
    ANI_LAUNCHED(h);
    return ANIGPU_OK;
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
constexpr size_t kNoallocBlockBytes = 16u << 20;  // per-tet blocks: 524,288 tets in FP32, 262,144 in FP64
constexpr size_t kNoallocScratchBytes = kNoallocTableBytes + kNoallocBlockBytes;
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
    double val[20], grad[20][3];
    const int nf = eval_scalar_basis_at(space, pp, val, grad);
    if (nf != 4 && nf != 10) return false;
    const int A[6] = {0, 1, 2, 0, 0, 1}, B[6] = {0, 1, 2, 1, 2, 2};
    for (size_t k = 0; k < (size_t)nf * nf * 8 + nf; ++k) T[k] = 0.0;
    // point by point (rules of up to 552 points), each sum in ascending point order
    for (int n = 0; n < q; ++n) {
        eval_scalar_basis_at(space, pp + 4 * n, val, grad);
        for (int i = 0; i < nf; ++i)
            for (int j = 0; j < nf; ++j)
                for (int k = 0; k < 6; ++k) {
                    double v = grad[i][A[k]] * grad[j][B[k]];
                    if (A[k] != B[k]) v += grad[i][B[k]] * grad[j][A[k]];
                    T[((size_t)i * nf + j) * 8 + k] += ww[n] * v;
                }
        for (int i = 0; i < nf; ++i) T[(size_t)nf * nf * 8 + i] += ww[n] * val[i];
    }
    // columns into canonical order, in place (fixed storage: one row of 10 x 8 at a time)
    for (int i = 0; i < nf; ++i) {
        double row[10 * 8];
        double* Ti = T + (size_t)i * nf * 8;
        for (int c = 0; c < nf; ++c)
            for (int k = 0; k < 8; ++k) row[c * 8 + k] = Ti[canon_local(nf, i, c) * 8 + k];
        for (int k = 0; k < nf * 8; ++k) Ti[k] = row[k];
    }
    *nf_out = nf;
    return true;
}

template <typename Real, int NLOC, bool DIR, bool BCNZ, bool DROPCHK>
int noalloc_rows(anigpu_ctx* h, const RowParams& p, const Real* tables, const Real* tetK, Real* vals, double* rhs) {
    const int warps = 2;
    const size_t smem = RowSmem<Real, NLOC, 0, false>::total(p.cap, warps);
    auto kern = row_gather_kernel<Real, NLOC, 0, DIR, BCNZ, false, DROPCHK>;
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
    if (need > kNoallocBlockBytes)
        return set_err(h, ANIGPU_ERR_ARG,
                       "anigpu_assemble_noalloc: mesh too large for the fixed scratch (" +
                           std::to_string(h->nt) + " tets need " + std::to_string(need) + " bytes, limit " +
                           std::to_string(kNoallocBlockBytes) + " bytes: " +
                           std::to_string(kNoallocBlockBytes / 32) + " tets in FP32, " +
                           std::to_string(kNoallocBlockBytes / 64) + " in FP64)");
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
    RowParams p{};
    p.inc_ptr = h->inc_ptr;
    p.recs = h->recs;
    p.rowptr = h->rowptr_s;
    p.dir_mask = h->dir_mask;
    p.dir_bc = h->dir_bc;
    p.edofs = h->edofs;
    p.drop = drop_val;
    p.vec_ok = ((uintptr_t)vals % 16) == 0 ? 1 : 0;
    p.dir_cptr = h->dir_cptr;
    p.dir_coff = h->dir_coff;
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
