// Learned preconditioner for flexible CG (a new component: the reference has no learned
// part; its solver is INMOST's ILU-Krylov, examples/tutorials/ex1.cpp:161-163).
//
// Preconditioner (additive two-level, symmetric positive definite by construction):
//     M r = D^-1 r + P Dc^-1/2 B B^T Dc^-1/2 P^T r,      B = sum_{k<K} diag(a_k) A_hat^k
// P interpolates vertex values onto the P2 DOFs (vertex DOF = its vertex, edge DOF = mean of
// the two end vertices); P^T is its transpose.  A_hat_vw = -A_vw / sqrt(A_vv A_ww) over the
// vertex-vertex entries of the P2 matrix (no self loop), Dc = diag(A_vv).  The per-vertex
// coefficients a_k come from a message-passing network run once per system:
//     h0 = relu(F W0 + b0)                     F: log A_vv, mean log(trace D / 3) (centred)
//     h_l = h_{l-1} + relu((A_hat h_{l-1}) W_l + b_l),  l = 1..L
//     a = h_L W_out + b_out                      (K outputs per vertex)
// Activations and the weights the kernels use are BF16 (FP32 for gradient checks); every
// accumulation is FP32.  Training minimises the relative energy-norm error against pairs
// (r, e = A^-1 r):   L = (M r - e)^T A (M r - e) / (e^T A e), with hand-written backward
// kernels (through the polynomial and the network) and Adam.  Every reduction is two-stage
// with a fixed order, so runs reproduce bit for bit.
#include <cuda_bf16.h>

#include <atomic>
#include <cmath>
#include <vector>

#include "coarse_chain.cuh"
#include "learned.h"

namespace {

constexpr int C = 64;           // hidden channels
constexpr int K = kChainK;     // polynomial terms of B (A_hat^0 .. A_hat^3)
constexpr int NF = 2;           // input features
constexpr int kMaxLayers = 8;
constexpr int kBlk = 256;
constexpr int kMaxPart = 1024;  // block partials of reductions

template <typename A>
__device__ __forceinline__ float ld(const A* p) {
    return (float)*p;
}
template <>
__device__ __forceinline__ float ld<__nv_bfloat16>(const __nv_bfloat16* p) {
    return __bfloat162float(*p);
}
template <typename A>
__device__ __forceinline__ A cvt(float v) {
    return (A)v;
}
template <>
__device__ __forceinline__ __nv_bfloat16 cvt<__nv_bfloat16>(float v) {
    return __float2bfloat16_rn(v);
}

struct Gnn {
    int layers = 4, act = ANIGPU_BF16;  // act: ANIGPU_F32 or ANIGPU_BF16
    int64_t nparam = 0;
    float* w = nullptr;      // FP32 master parameters
    float* g = nullptr;      // FP32 gradient accumulator
    float* m1 = nullptr;     // Adam moments
    float* m2 = nullptr;
    float* wk = nullptr;     // parameters as the kernels see them (rounded to BF16 when act is BF16)
    // bound system
    int64_t nc = 0;          // coarse nodes (vertex DOFs of every component)
    CMap map{0, 0};
    int64_t nf = 0;          // fine DOFs
    int64_t* crow = nullptr; // coarse graph CSR
    int32_t* ccol = nullptr;
    float* cval = nullptr;
    int64_t cnnz = 0;
    // the coarse graph again in slices of 32 rows (entry j of row 32 s + l at sbase[s] + 32 j + l,
    // padded with zero entries to the slice's longest row) for the fused coarse chain
    int64_t* sbase = nullptr;
    int32_t* scol = nullptr;
    float* sval = nullptr;
    int64_t snnz = 0;
    unsigned int* bar = nullptr;  // grid barrier of the fused chain: arrivals, generation, expired
    int chain_grid = 0;           // co-resident blocks of the fused chain; 0: separate launches
    float* diag_f = nullptr;    // fine diagonal
    float* isd_c = nullptr;     // 1/sqrt(A_vv)
    float* feat = nullptr;      // static features [nc][NF]
    int32_t* edge_ends = nullptr;  // [ne][2]
    int64_t* vrow = nullptr;       // vertex -> incident edge DOFs (CSR, ascending)
    int32_t* vedge = nullptr;
    double* dpart = nullptr;       // [2][kMaxPart] dot partials of the standalone FP32 apply
    float* coef = nullptr;      // a [nc][K] (network output)
    // activations: H_l (l=0..L), G_l (l=1..L), Z_l (l=0..L) -- each nc*C of act type
    void* act_buf = nullptr;
    size_t act_bytes = 0;
    float* u = nullptr;         // Dc^-1/2 P^T r            [nc]
    float* pw = nullptr;        // A_hat^k w, k = 0..K-1    [K][nc]
    float* qv = nullptr;        // A_hat^k v, k = 0..K-1    [K][nc]
    float* t0 = nullptr;        // scratch [nc]
    float* t1 = nullptr;        // scratch [nc]
    float* cc = nullptr;        // coarse correction [nc]
    float* ga = nullptr;        // dL/da [nc][K]
    float* dH = nullptr;        // backward buffers [nc][C] fp32
    float* dG = nullptr;
    float* dZ = nullptr;
    float* part = nullptr;      // reduction partials
    float* wpart = nullptr;     // weight-gradient partials [kMaxPart][C*C]
    double* fine_tmp = nullptr;   // [nf] f64
    double* fine_tmp2 = nullptr;  // [nf]
    int64_t bind_gen = 0;       // incremented by every bind (solver graphs bake the buffers in)
    const void* bound_vals = nullptr;
    int bound_prec = -1;
    bool bound = false;
};

// ------------------------------------------------------------ parameter layout
struct Layout {
    int64_t W0, b0, W[kMaxLayers], b[kMaxLayers], wout, bout, total;
};
Layout layout(int L) {
    Layout o;
    int64_t p = 0;
    o.W0 = p; p += NF * C;
    o.b0 = p; p += C;
    for (int l = 0; l < L; ++l) {
        o.W[l] = p; p += C * C;
        o.b[l] = p; p += C;
    }
    o.wout = p; p += C * K;
    o.bout = p; p += K;
    o.total = p;
    return o;
}

// ------------------------------------------------------------ bind: coarse graph and features
__global__ void fine_diag_kernel(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                 const void* __restrict__ vals, int f32, float* __restrict__ diag) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= n) return;
    float d = 0.f;
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k)
        if (col[k] == r) {
            d = f32 ? ((const float*)vals)[k] : (float)((const double*)vals)[k];
            break;
        }
    diag[r] = d;
}

__global__ void coarse_count_kernel(int64_t nc, CMap m, const int64_t* __restrict__ rowptr,
                                    const int32_t* __restrict__ col, unsigned long long* __restrict__ cnt) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= nc) return;
    const int64_t fr = m.fine_of(r);
    unsigned long long c = 0;
    for (int64_t k = rowptr[fr]; k < rowptr[fr + 1]; ++k) c += (col[k] != fr && m.coarse_of(col[k]) >= 0) ? 1 : 0;
    cnt[r] = c;
}

__global__ void coarse_fill_kernel(int64_t nc, CMap m, const int64_t* __restrict__ rowptr,
                                   const int32_t* __restrict__ col, const void* __restrict__ vals, int f32,
                                   const float* __restrict__ diag, const int64_t* __restrict__ crow,
                                   int32_t* __restrict__ ccol, float* __restrict__ cval, float* __restrict__ isd) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= nc) return;
    const int64_t fr = m.fine_of(r);
    int64_t w = crow[r];
    const float dr = diag[fr];
    isd[r] = dr > 0.f ? rsqrtf(dr) : 0.f;
    for (int64_t k = rowptr[fr]; k < rowptr[fr + 1]; ++k) {
        const int32_t c = col[k];
        const int64_t cc = m.coarse_of(c);
        if (c != fr && cc >= 0) {
            const float a = f32 ? ((const float*)vals)[k] : (float)((const double*)vals)[k];
            const float dd = dr * diag[c];
            ccol[w] = (int32_t)cc;
            cval[w] = dd > 0.f ? -a * rsqrtf(dd) : 0.f;
            ++w;
        }
    }
}

// static features: log(A_vv), mean over incident tets of log(trace(D)/3) (Lame: of lambda + 2 mu)
__global__ void static_feat_kernel(int64_t nc, CMap m, const float* __restrict__ diag_f,
                                   const int64_t* __restrict__ inc_ptr, const ScatterRec* __restrict__ recs, int kind,
                                   const double* __restrict__ D, float* __restrict__ feat) {
    const int64_t cid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (cid >= nc) return;
    const int64_t v = cid % m.nv;
    const float d = diag_f[m.fine_of(cid)];
    feat[NF * cid] = d > 0.f ? logf(d) : 0.f;
    float s = 0.f;
    const int64_t b = inc_ptr[v], e = inc_ptr[v + 1];
    for (int64_t k = b; k < e; ++k) {
        const int64_t t = recs[k].tet;
        float tr = 1.f;
        if (kind == ANIGPU_TENSOR_TET_SYM) tr = (float)((D[6 * t] + D[6 * t + 3] + D[6 * t + 5]) / 3.0);
        else if (kind == ANIGPU_TENSOR_TET_SCALAR) tr = (float)D[t];
        else if (kind == ANIGPU_TENSOR_CONST_SCALAR) tr = (float)D[0];
        else if (kind == ANIGPU_TENSOR_LAME) tr = (float)(D[2 * t] + 2.0 * D[2 * t + 1]);
        s += logf(fmaxf(tr, 1e-30f));
    }
    feat[NF * cid + 1] = e > b ? s / (float)(e - b) : 0.f;
}

__global__ void edge_ends_kernel(int64_t ne, int64_t nv, const int64_t* __restrict__ inc_ptr,
                                 const ScatterRec* __restrict__ recs, const int32_t* __restrict__ tets,
                                 int32_t* __restrict__ ends) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int64_t row = nv + e;
    const int64_t b = inc_ptr[row];
    const ScatterRec r = recs[b];
    const int i = (r.meta & 15) - 4;
    const int I[6] = {0, 0, 0, 1, 1, 2}, J[6] = {1, 2, 3, 2, 3, 3};
    ends[2 * e] = tets[4 * (int64_t)r.tet + I[i]];
    ends[2 * e + 1] = tets[4 * (int64_t)r.tet + J[i]];
}

// vertex -> edge adjacency: counts, fill (any order), then an ascending sort of every row so
// that sums over it have a fixed order
__global__ void vedge_count_kernel(int64_t ne, const int32_t* __restrict__ ends, unsigned long long* __restrict__ cnt) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= ne) return;
    atomicAdd(cnt + ends[2 * e], 1ull);
    atomicAdd(cnt + ends[2 * e + 1], 1ull);
}
__global__ void vedge_fill_kernel(int64_t ne, int64_t nv, const int32_t* __restrict__ ends,
                                  const int64_t* __restrict__ vrow, unsigned long long* __restrict__ fill,
                                  int32_t* __restrict__ vedge) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= ne) return;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const int32_t v = ends[2 * e + q];
        const unsigned long long k = atomicAdd(fill + v, 1ull);
        vedge[vrow[v] + (int64_t)k] = (int32_t)(nv + e);
    }
}
__global__ void vedge_sort_kernel(int64_t nc, const int64_t* __restrict__ vrow, int32_t* __restrict__ vedge) {
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= nc) return;
    const int64_t b = vrow[v], e = vrow[v + 1];
    for (int64_t i = b + 1; i < e; ++i) {
        const int32_t key = vedge[i];
        int64_t j = i - 1;
        while (j >= b && vedge[j] > key) {
            vedge[j + 1] = vedge[j];
            --j;
        }
        vedge[j + 1] = key;
    }
}

// fixed-order block reduction helper (float)
__device__ __forceinline__ float block_sum(float v, float* sh) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    float s = 0.f;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i];
    return s;
}

// centre the feature columns (partial sums, then apply)
__global__ void feat_partial_kernel(int64_t nc, const float* __restrict__ feat, float* __restrict__ part) {
    __shared__ float sh[32];
    float a0 = 0.f, a1 = 0.f;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nc; v += (int64_t)gridDim.x * blockDim.x) {
        a0 += feat[NF * v];
        a1 += feat[NF * v + 1];
    }
    const float s0 = block_sum(a0, sh);
    __syncthreads();
    const float s1 = block_sum(a1, sh);
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = s0;
        part[2 * blockIdx.x + 1] = s1;
    }
}
__global__ void feat_center_kernel(int64_t nc, int nb, const float* __restrict__ part, float* __restrict__ feat) {
    __shared__ float m[2];
    if (threadIdx.x < 2) {
        double s = 0;
        for (int b = 0; b < nb; ++b) s += part[2 * b + threadIdx.x];
        m[threadIdx.x] = (float)(s / (double)nc);
    }
    __syncthreads();
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nc; v += (int64_t)gridDim.x * blockDim.x) {
        feat[NF * v] -= m[0];
        feat[NF * v + 1] -= m[1];
    }
}

// ------------------------------------------------------------ transfers
// out_v = isd_v * (x_v + 1/2 sum over the edge DOFs e of v of x_e)        (Dc^-1/2 P^T x)
// (v a coarse node; the edges are those of v's vertex, in v's component)
template <typename T>
__global__ void restrict_kernel(int64_t nc, CMap m, const T* __restrict__ x, const int64_t* __restrict__ vrow,
                                const int32_t* __restrict__ vedge, const float* __restrict__ isd,
                                float* __restrict__ out) {
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= nc) return;
    const int c = m.comp_coarse(v);
    const int64_t vs = v - c * m.nv;
    const T* xc = x + c * m.nds;
    float s = 0.f;
    for (int64_t k = vrow[vs]; k < vrow[vs + 1]; ++k) s += (float)xc[vedge[k]];
    out[v] = isd[v] * fmaf(0.5f, s, (float)xc[vs]);
}

// z = dinv .* r + P c
template <typename T>
__global__ void prolong_kernel(int64_t nf, CMap m, const T* __restrict__ r, const float* __restrict__ diag_f,
                               const float* __restrict__ c, const int32_t* __restrict__ ends, T* __restrict__ z) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= nf) return;
    const float d = diag_f[i];
    T v = d != 0.f ? r[i] / (T)d : r[i];
    const int comp = m.comp_fine(i);
    const int64_t s = i - comp * m.nds;
    const float* cc = c + comp * m.nv;
    if (s < m.nv) v += (T)cc[s];
    else {
        const int64_t e = s - m.nv;
        v += (T)0.5 * ((T)cc[ends[2 * e]] + (T)cc[ends[2 * e + 1]]);
    }
    z[i] = v;
}

// scalar coarse SpMV: y = A_hat x (+ coef_k .* s when s given)   (one thread per row)
__global__ void cspmv_kernel(int64_t nc, const int64_t* __restrict__ crow, const int32_t* __restrict__ ccol,
                             const float* __restrict__ cval, const float* __restrict__ x,
                             const float* __restrict__ coef, int k, const float* __restrict__ s,
                             float* __restrict__ y) {
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= nc) return;
    float a = 0.f;
    for (int64_t q = crow[v]; q < crow[v + 1]; ++q) a = fmaf(cval[q], x[ccol[q]], a);
    if (s) a = fmaf(coef[K * v + k], s[v], a);
    y[v] = a;
}

// y = coef_k .* s   (start of a Horner chain)
__global__ void cscale_kernel(int64_t nc, const float* __restrict__ coef, int k, const float* __restrict__ s,
                              float* __restrict__ y) {
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v < nc) y[v] = coef[K * v + k] * s[v];
}

// c = isd .* sum_k coef_k .* pw_k
__global__ void combine_kernel(int64_t nc, const float* __restrict__ coef, const float* __restrict__ pw,
                               const float* __restrict__ isd, float* __restrict__ c) {
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= nc) return;
    float a = 0.f;
#pragma unroll
    for (int k = 0; k < K; ++k) a = fmaf(coef[K * v + k], pw[k * nc + v], a);
    c[v] = isd[v] * a;
}

// dL/da_k = g' .* P_k + u .* Q_k
__global__ void coef_grad_kernel(int64_t nc, const float* __restrict__ gp, const float* __restrict__ pw,
                                 const float* __restrict__ u, const float* __restrict__ qv, float* __restrict__ ga) {
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= nc) return;
#pragma unroll
    for (int k = 0; k < K; ++k) ga[K * v + k] = gp[v] * pw[k * nc + v] + u[v] * qv[k * nc + v];
}

// ------------------------------------------------------------ fused FP32 apply (the solver's path)
// CW lanes per coarse row; every kernel returns at once when *stop is set (a converged or
// stopped batch of solver iterations).
constexpr int CW = 4;

__device__ __forceinline__ float cw_sum(float s) {
#pragma unroll
    for (int o = CW / 2; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, CW);
    return s;
}

// u = Dc^-1/2 P^T r ; t = a_{K-1} .* u
__global__ void __launch_bounds__(256) restrict_scale_kernel(int64_t nc, CMap m, const float* __restrict__ r,
                                                             const int64_t* __restrict__ vrow,
                                                             const int32_t* __restrict__ vedge,
                                                             const float* __restrict__ isd,
                                                             const float* __restrict__ coef, float* __restrict__ u,
                                                             float* __restrict__ t, const int* __restrict__ stop) {
    if (stop && *stop) return;
    const int64_t v = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / CW;
    const int lane = threadIdx.x & (CW - 1);
    const int c = m.comp_coarse(v);
    const int64_t vs = v - c * m.nv;
    const float* rc = r + c * m.nds;
    float s = 0.f;
    if (v < nc)
        for (int64_t k = vrow[vs] + lane; k < vrow[vs + 1]; k += CW) s += rc[vedge[k]];
    s = cw_sum(s);
    if (v < nc && lane == 0) {
        const float uu = isd[v] * fmaf(0.5f, s, rc[vs]);
        u[v] = uu;
        t[v] = coef[K * v + K - 1] * uu;
    }
}

// y = A_hat x (+ a_k .* s when s is given)
__global__ void __launch_bounds__(256) cspmv4_kernel(int64_t nc, const int64_t* __restrict__ crow,
                                                     const int32_t* __restrict__ ccol, const float* __restrict__ cval,
                                                     const float* __restrict__ x, const float* __restrict__ coef, int k,
                                                     const float* __restrict__ sv, float* __restrict__ y,
                                                     const int* __restrict__ stop) {
    if (stop && *stop) return;
    const int64_t v = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / CW;
    const int lane = threadIdx.x & (CW - 1);
    float a = 0.f;
    if (v < nc)
        for (int64_t q = crow[v] + lane; q < crow[v + 1]; q += CW) a = fmaf(cval[q], x[ccol[q]], a);
    a = cw_sum(a);
    if (v < nc && lane == 0) y[v] = sv ? fmaf(coef[K * v + k], sv[v], a) : a;
}

// P_{K-1} = A_hat P_{K-2};  c = isd .* sum_k a_k .* P_k
__global__ void __launch_bounds__(256) combine4_kernel(int64_t nc, const int64_t* __restrict__ crow,
                                                       const int32_t* __restrict__ ccol,
                                                       const float* __restrict__ cval, const float* __restrict__ pw,
                                                       const float* __restrict__ coef, const float* __restrict__ isd,
                                                       float* __restrict__ c, const int* __restrict__ stop) {
    if (stop && *stop) return;
    const int64_t v = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / CW;
    const int lane = threadIdx.x & (CW - 1);
    const float* x = pw + (int64_t)(K - 2) * nc;
    float a = 0.f;
    if (v < nc)
        for (int64_t q = crow[v] + lane; q < crow[v + 1]; q += CW) a = fmaf(cval[q], x[ccol[q]], a);
    a = cw_sum(a);
    if (v < nc && lane == 0) {
        float s = coef[K * v + K - 1] * a;
#pragma unroll
        for (int k = K - 2; k >= 0; --k) s = fmaf(coef[K * v + k], pw[(int64_t)k * nc + v], s);
        c[v] = isd[v] * s;
    }
}

// z = D^-1 r + P c ; block partials of r.z and z.qold (FP32 per thread, FP64 across the block)
__global__ void __launch_bounds__(256) prolong_dot_kernel(int64_t nf, CMap m, const float* __restrict__ r,
                                                          const float* __restrict__ diag_f,
                                                          const float* __restrict__ c,
                                                          const int32_t* __restrict__ ends,
                                                          const float* __restrict__ qold, float* __restrict__ z,
                                                          double* __restrict__ part_rz, double* __restrict__ part_zq,
                                                          const int* __restrict__ stop) {
    __shared__ double sh[32];
    if (stop && *stop) return;
    float arz = 0.f, azq = 0.f;
    const ProlongArgs pa{nf, m, diag_f, c, ends};
    prolong_rows(pa, r, z, qold, blockIdx.x * (int64_t)blockDim.x + threadIdx.x, (int64_t)gridDim.x * blockDim.x, arz,
                 azq);
    double a = arz, b = azq;
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if ((threadIdx.x & 31) == 0) {
        sh[threadIdx.x >> 5] = a;
        sh[16 + (threadIdx.x >> 5)] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ta = 0, tb = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            ta += sh[w];
            tb += sh[16 + w];
        }
        part_rz[blockIdx.x] = ta;
        part_zq[blockIdx.x] = tb;
    }
}

// ------------------------------------------------------------ fused coarse chain (one cooperative launch)
// The coarse part of M r as one kernel: restriction, the three Horner products, the two powers and
// the combination (the work of restrict_scale, cspmv4 x 5 and combine4 above), separated by grid
// barriers instead of kernel boundaries (chain_stages, coarse_chain.cuh).
// threads per block of the chain: large blocks, few arrivals per barrier; two blocks per SM (32
// registers) so that every coarse row has its own thread at 64^3
#ifndef CHAIN_THREADS
#define CHAIN_THREADS 1024
#endif
#ifndef CHAIN_MINB
#define CHAIN_MINB 2
#endif
constexpr int kChainThreads = CHAIN_THREADS;

__global__ void __launch_bounds__(kChainThreads, CHAIN_MINB) coarse_chain_kernel(ChainArgs a) {
    if (a.stop && *a.stop) return;  // the same value for every block: no barrier is entered
    if (barrier_expired(a.bar)) {  // an earlier launch's wait expired: the barrier is unusable
        for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < a.nc; v += (int64_t)gridDim.x * blockDim.x)
            a.cc[v] = __int_as_float(0x7fc00000);
        return;
    }
    chain_stages(a, blockIdx.x * (int64_t)blockDim.x + threadIdx.x, (int64_t)gridDim.x * blockDim.x);
}

// slices: 32 x (the longest row of each 32-row slice) entries
__global__ void sell_count_kernel(int64_t nc, const int64_t* __restrict__ crow, unsigned long long* __restrict__ cnt) {
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;  // blockDim: a multiple of 32
    const int len = v < nc ? (int)(crow[v + 1] - crow[v]) : 0;
    const int m = __reduce_max_sync(0xffffffffu, len);
    if ((threadIdx.x & 31) == 0 && v < nc) cnt[v >> 5] = 32ull * (unsigned long long)m;
}

__global__ void sell_fill_kernel(int64_t nc, const int64_t* __restrict__ crow, const int32_t* __restrict__ ccol,
                                 const float* __restrict__ cval, const int64_t* __restrict__ sbase,
                                 int32_t* __restrict__ scol, float* __restrict__ sval) {
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= nc) return;
    const int64_t s = v >> 5, b = crow[v];
    const int len = (int)(crow[v + 1] - b), w = (int)((sbase[s + 1] - sbase[s]) >> 5);
    for (int j = 0; j < w; ++j) {
        const int64_t q = sbase[s] + 32 * j + (v & 31);
        scol[q] = j < len ? ccol[b + j] : (int32_t)v;
        sval[q] = j < len ? cval[b + j] : 0.f;
    }
}

__global__ void chain_probe_kernel(int* out) {
    if (out && threadIdx.x == 0 && blockIdx.x == 0) *out = 1;
}

// ------------------------------------------------------------ network forward
// one warp per node; lane owns channels lane and lane + 32
template <typename A>
__global__ void input_layer_kernel(int64_t nc, const float* __restrict__ feat, const float* __restrict__ W0,
                                   const float* __restrict__ b0, A* __restrict__ Z, A* __restrict__ H) {
    const int64_t v = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (v >= nc) return;
    const float f1 = feat[NF * v], f2 = feat[NF * v + 1];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int c = lane + 32 * h;
        const float z = b0[c] + f1 * W0[c] + f2 * W0[C + c];
        Z[v * C + c] = cvt<A>(z);
        H[v * C + c] = cvt<A>(fmaxf(z, 0.f));
    }
}

// G = A_hat H   (rows of the coarse graph)
template <typename In, typename Out>
__global__ void spmm_kernel(int64_t nc, const int64_t* __restrict__ crow, const int32_t* __restrict__ ccol,
                            const float* __restrict__ cval, const In* __restrict__ H, Out* __restrict__ G,
                            int accumulate) {
    const int64_t v = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (v >= nc) return;
    float a0 = 0.f, a1 = 0.f;
    for (int64_t k = crow[v]; k < crow[v + 1]; ++k) {
        const float w = cval[k];
        const In* hr = H + (int64_t)ccol[k] * C;
        a0 = fmaf(w, ld(hr + lane), a0);
        a1 = fmaf(w, ld(hr + lane + 32), a1);
    }
    if (accumulate) {
        a0 += ld(G + v * C + lane);
        a1 += ld(G + v * C + lane + 32);
    }
    G[v * C + lane] = cvt<Out>(a0);
    G[v * C + lane + 32] = cvt<Out>(a1);
}

// Z = G W + b ; Hout = Hin + relu(Z)
template <typename A>
__global__ void __launch_bounds__(kBlk) dense_kernel(int64_t nc, const A* __restrict__ G, const float* __restrict__ W,
                                                     const float* __restrict__ b, const A* __restrict__ Hin,
                                                     A* __restrict__ Z, A* __restrict__ Hout) {
    __shared__ float sW[C * C];
    for (int k = threadIdx.x; k < C * C; k += blockDim.x) sW[k] = W[k];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t v = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (v >= nc) return;
    const float g0 = ld(G + v * C + lane), g1 = ld(G + v * C + lane + 32);
    float z0 = b[lane], z1 = b[lane + 32];
#pragma unroll 8
    for (int k = 0; k < 32; ++k) {
        const float ga = __shfl_sync(0xffffffffu, g0, k), gb = __shfl_sync(0xffffffffu, g1, k);
        z0 = fmaf(ga, sW[k * C + lane], z0);
        z1 = fmaf(ga, sW[k * C + lane + 32], z1);
        z0 = fmaf(gb, sW[(k + 32) * C + lane], z0);
        z1 = fmaf(gb, sW[(k + 32) * C + lane + 32], z1);
    }
    Z[v * C + lane] = cvt<A>(z0);
    Z[v * C + lane + 32] = cvt<A>(z1);
    Hout[v * C + lane] = cvt<A>(ld(Hin + v * C + lane) + fmaxf(z0, 0.f));
    Hout[v * C + lane + 32] = cvt<A>(ld(Hin + v * C + lane + 32) + fmaxf(z1, 0.f));
}

// The BF16 layer on the tensor cores: Z = G W + b, Hout = Hin + relu(Z) with
// mma.sync.m16n8k16 (BF16 inputs, FP32 accumulation).  One warp computes a 16-node x 64-channel
// tile: 4 k-steps x 8 n-tiles of 8 channels = 32 MMAs; A fragments (16 x 16 of G) are read straight
// from global memory as BF16 pairs, B fragments from W^T staged once per block in shared memory as
// BF16 (row n holds the 64 k of output channel n, padded to 72 so that the 8 rows of a fragment load
// fall on distinct banks); the accumulators start at the bias.
constexpr int kMmaWarps = 4;  // warps per block: 64 nodes
constexpr int kWtStride = C + 8;

__device__ __forceinline__ void mma_bf16_16816(float* d, const uint32_t* a, const uint32_t* b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__global__ void __launch_bounds__(kMmaWarps * 32) dense_mma_bf16_kernel(int64_t nc, const __nv_bfloat16* __restrict__ G,
                                                                         const float* __restrict__ W,
                                                                         const float* __restrict__ b,
                                                                         const __nv_bfloat16* __restrict__ Hin,
                                                                         __nv_bfloat16* __restrict__ Z,
                                                                         __nv_bfloat16* __restrict__ Hout) {
    // per warp: its 16 x 64 tile of G (then of Hin) as BF16 and the 16 x 64 FP32 pre-activations,
    // moved between global and shared memory with coalesced 16-byte accesses
    constexpr int kAS = C + 8;  // BF16 row stride: 144 bytes, fragment loads on distinct banks
    constexpr int kZS = C + 4;  // FP32 row stride
    __shared__ __align__(16) __nv_bfloat16 sWt[C * kWtStride];
    __shared__ __align__(16) __nv_bfloat16 sA[kMmaWarps][16 * kAS];
    __shared__ __align__(16) float sZf[kMmaWarps][16 * kZS];
    for (int k = threadIdx.x; k < C * C; k += blockDim.x) {
        const int kk = k / C, n = k - kk * C;  // W[kk][n] -> Wt[n][kk]
        sWt[n * kWtStride + kk] = __float2bfloat16_rn(W[k]);
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int64_t v0 = ((int64_t)blockIdx.x * kMmaWarps + warp) * 16;
    if (v0 >= nc) return;
    __nv_bfloat16* A = sA[warp];
    float* Zf = sZf[warp];
    // 16 rows x 8 vectors of 8 BF16: lane handles vectors lane + 32 j
    auto load_tile = [&](const __nv_bfloat16* src) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int idx = lane + 32 * j, r = idx >> 3, c8 = (idx & 7) * 8;
            const int64_t v = v0 + r;
            const uint4 val = v < nc ? __ldg(reinterpret_cast<const uint4*>(src + v * C + c8)) : make_uint4(0, 0, 0, 0);
            *reinterpret_cast<uint4*>(A + r * kAS + c8) = val;
        }
        __syncwarp();
    };
    load_tile(G);
    float acc[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const float b0 = b[nt * 8 + 2 * t], b1 = b[nt * 8 + 2 * t + 1];
        acc[nt][0] = b0;
        acc[nt][1] = b1;
        acc[nt][2] = b0;
        acc[nt][3] = b1;
    }
#pragma unroll
    for (int ks = 0; ks < C / 16; ++ks) {
        // A: rows g / g+8, columns ks*16 + 2t (+1) and + 8 (32-bit BF16 pairs)
        const uint32_t* a0p = reinterpret_cast<const uint32_t*>(A + g * kAS + ks * 16 + 2 * t);
        const uint32_t* a1p = reinterpret_cast<const uint32_t*>(A + (g + 8) * kAS + ks * 16 + 2 * t);
        const uint32_t a[4] = {a0p[0], a1p[0], a0p[4], a1p[4]};
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            // B: k = ks*16 + 2t (+1) and + 8, n = nt*8 + g
            const uint32_t* wt = reinterpret_cast<const uint32_t*>(sWt + (nt * 8 + g) * kWtStride + ks * 16 + 2 * t);
            const uint32_t bb[2] = {wt[0], wt[4]};
            mma_bf16_16816(acc[nt], a, bb);
        }
    }
    // pre-activations to shared memory (FP32), then Hin over the G tile
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const int col = nt * 8 + 2 * t;
        *reinterpret_cast<float2*>(Zf + g * kZS + col) = make_float2(acc[nt][0], acc[nt][1]);
        *reinterpret_cast<float2*>(Zf + (g + 8) * kZS + col) = make_float2(acc[nt][2], acc[nt][3]);
    }
    __syncwarp();
    load_tile(Hin);
    // epilogue, coalesced: Z = bf16(z), Hout = bf16(Hin + relu(z)), 8 channels per vector
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int idx = lane + 32 * j, r = idx >> 3, c8 = (idx & 7) * 8;
        const int64_t v = v0 + r;
        if (v >= nc) continue;
        const float* z = Zf + r * kZS + c8;
        const __nv_bfloat162* hi = reinterpret_cast<const __nv_bfloat162*>(A + r * kAS + c8);
        __align__(16) __nv_bfloat162 zo[4], ho[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float z0 = z[2 * q], z1 = z[2 * q + 1];
            const float2 hf = __bfloat1622float2(hi[q]);
            zo[q] = __floats2bfloat162_rn(z0, z1);
            ho[q] = __floats2bfloat162_rn(hf.x + fmaxf(z0, 0.f), hf.y + fmaxf(z1, 0.f));
        }
        *reinterpret_cast<uint4*>(Z + v * C + c8) = *reinterpret_cast<const uint4*>(zo);
        *reinterpret_cast<uint4*>(Hout + v * C + c8) = *reinterpret_cast<const uint4*>(ho);
    }
}

// a = H W_out + b_out   (K outputs per node)
template <typename A>
__global__ void output_kernel(int64_t nc, const A* __restrict__ H, const float* __restrict__ wout,
                              const float* __restrict__ bout, float* __restrict__ coef) {
    const int64_t v = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (v >= nc) return;
    const float h0 = ld(H + v * C + lane), h1 = ld(H + v * C + lane + 32);
#pragma unroll
    for (int k = 0; k < K; ++k) {
        float s = h0 * wout[lane * K + k] + h1 * wout[(lane + 32) * K + k];
#pragma unroll
        for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) coef[K * v + k] = s + bout[k];
    }
}

// ------------------------------------------------------------ network backward
// dH_L = ga W_out^T ; partials of dW_out (C x K) and db_out (K)
template <typename A>
__global__ void output_bwd_kernel(int64_t nc, const A* __restrict__ H, const float* __restrict__ wout,
                                  const float* __restrict__ ga, float* __restrict__ dH, float* __restrict__ part) {
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    float acc0[K], acc1[K], accb[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc0[k] = acc1[k] = accb[k] = 0.f;
    for (int64_t v = (int64_t)blockIdx.x * wpb + (threadIdx.x >> 5); v < nc; v += (int64_t)gridDim.x * wpb) {
        float d0 = 0.f, d1 = 0.f;
        const float h0 = ld(H + v * C + lane), h1 = ld(H + v * C + lane + 32);
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const float g = ga[K * v + k];
            d0 = fmaf(g, wout[lane * K + k], d0);
            d1 = fmaf(g, wout[(lane + 32) * K + k], d1);
            acc0[k] = fmaf(g, h0, acc0[k]);
            acc1[k] = fmaf(g, h1, acc1[k]);
            accb[k] += g;
        }
        dH[v * C + lane] = d0;
        dH[v * C + lane + 32] = d1;
    }
    // fixed-order combination over the warps of the block: [C*K] weights then [K] biases
    __shared__ float red[8][C * K + K];
    const int w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        red[w][lane * K + k] = acc0[k];
        red[w][(lane + 32) * K + k] = acc1[k];
    }
    if (lane < K) red[w][C * K + lane] = accb[lane];
    __syncthreads();
    for (int q = threadIdx.x; q < C * K + K; q += blockDim.x) {
        float s = 0.f;
        for (int u = 0; u < wpb; ++u) s += red[u][q];
        part[(int64_t)blockIdx.x * (C * K + K) + q] = s;
    }
}

// dZ = dH * (Z > 0); dG = dZ W^T ; dW partial = G^T dZ (per block); db partial
template <typename A>
__global__ void __launch_bounds__(kBlk) dense_bwd_kernel(int64_t nc, const float* __restrict__ dH,
                                                         const A* __restrict__ Z, const A* __restrict__ G,
                                                         const float* __restrict__ W, float* __restrict__ dZout,
                                                         float* __restrict__ dG, float* __restrict__ wpart,
                                                         float* __restrict__ bpart, int rows_per_block) {
    __shared__ float sW[C * C];
    __shared__ float sG[32][C + 1];
    __shared__ float sZ[32][C + 1];
    for (int k = threadIdx.x; k < C * C; k += blockDim.x) sW[k] = W[k];
    // each thread owns 16 entries of dW: rows (tid / 16) * 4 .. +4, cols (tid % 16) * 4 .. +4
    const int tr = (threadIdx.x >> 4) * 4, tc = (threadIdx.x & 15) * 4;
    float acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[a][q] = 0.f;
    float bacc = 0.f;
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t v0 = (int64_t)blockIdx.x * rows_per_block;
    const int64_t vend = (v0 + rows_per_block < nc) ? v0 + rows_per_block : nc;
    for (int64_t base = v0; base < vend; base += 32) {
        for (int r = w; r < 32; r += kBlk / 32) {
            const int64_t v = base + r;
            float z0 = 0.f, z1 = 0.f, g0 = 0.f, g1 = 0.f;
            if (v < vend) {
                const float h0 = dH[v * C + lane], h1 = dH[v * C + lane + 32];
                z0 = ld(Z + v * C + lane) > 0.f ? h0 : 0.f;
                z1 = ld(Z + v * C + lane + 32) > 0.f ? h1 : 0.f;
                g0 = ld(G + v * C + lane);
                g1 = ld(G + v * C + lane + 32);
                dZout[v * C + lane] = z0;
                dZout[v * C + lane + 32] = z1;
                float d0 = 0.f, d1 = 0.f;
#pragma unroll 8
                for (int c = 0; c < 32; ++c) {
                    const float za = __shfl_sync(0xffffffffu, z0, c), zb = __shfl_sync(0xffffffffu, z1, c);
                    d0 = fmaf(za, sW[lane * C + c], d0);
                    d0 = fmaf(zb, sW[lane * C + c + 32], d0);
                    d1 = fmaf(za, sW[(lane + 32) * C + c], d1);
                    d1 = fmaf(zb, sW[(lane + 32) * C + c + 32], d1);
                }
                dG[v * C + lane] = d0;
                dG[v * C + lane + 32] = d1;
            }
            sZ[r][lane] = z0;
            sZ[r][lane + 32] = z1;
            sG[r][lane] = g0;
            sG[r][lane + 32] = g1;
        }
        __syncthreads();
        for (int r = 0; r < 32; ++r) {
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[a][q] = fmaf(sG[r][tr + a], sZ[r][tc + q], acc[a][q]);
        }
        if (threadIdx.x < C)
            for (int r = 0; r < 32; ++r) bacc += sZ[r][threadIdx.x];
        __syncthreads();
    }
    float* wp = wpart + (int64_t)blockIdx.x * C * C;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int q = 0; q < 4; ++q) wp[(tr + a) * C + tc + q] = acc[a][q];
    if (threadIdx.x < C) bpart[(int64_t)blockIdx.x * C + threadIdx.x] = bacc;
}

// The same backward step on the tensor cores for BF16 activations (TF32 inputs, FP32 accumulation,
// mma.sync m16n8k8): 32 nodes per chunk, staged in shared memory as FP32 (dZ, G); 4 warps.
//   dG = dZ W^T : warp w computes nodes (w & 1)*16 .. +16 x output columns (w >> 1)*32 .. +32
//   dW += G^T dZ: warp w owns the 16 rows w*16 .. +16 of dW (all 64 columns), K = the chunk's nodes
// Row strides 68 (W) and 72 (dZ, G) keep the fragment loads on distinct banks (dZ's A-loads of dG
// meet at most two-way conflicts).
constexpr int kTcWarps = 4, kTcChunk = 32, kSW = C + 4, kSZ = C + 8;

__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ void mma_tf32_1688(float* d, const uint32_t* a, const uint32_t* b) {
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__global__ void __launch_bounds__(kTcWarps * 32) dense_bwd_tc_kernel(int64_t nc, const float* __restrict__ dH,
                                                                      const __nv_bfloat16* __restrict__ Z,
                                                                      const __nv_bfloat16* __restrict__ G,
                                                                      const float* __restrict__ W,
                                                                      float* __restrict__ dZout, float* __restrict__ dG,
                                                                      float* __restrict__ wpart,
                                                                      float* __restrict__ bpart, int rows_per_block) {
    __shared__ float sW[C * kSW];
    __shared__ float sZ[kTcChunk * kSZ];
    __shared__ float sG[kTcChunk * kSZ];
    for (int k = threadIdx.x; k < C * C; k += blockDim.x) sW[(k / C) * kSW + (k % C)] = W[k];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    float accW[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int q = 0; q < 4; ++q) accW[nt][q] = 0.f;
    float bacc = 0.f;
    const int64_t v0 = (int64_t)blockIdx.x * rows_per_block;
    const int64_t vend = (v0 + rows_per_block < nc) ? v0 + rows_per_block : nc;
    for (int64_t base = v0; base < vend; base += kTcChunk) {
        __syncthreads();  // sW staged / the previous chunk's readers done
        for (int e = threadIdx.x; e < kTcChunk * C; e += blockDim.x) {
            const int r = e / C, c = e - r * C;
            const int64_t v = base + r;
            float z = 0.f, gg = 0.f;
            if (v < vend) {
                z = __bfloat162float(Z[v * C + c]) > 0.f ? dH[v * C + c] : 0.f;
                gg = __bfloat162float(G[v * C + c]);
                dZout[v * C + c] = z;
            }
            sZ[r * kSZ + c] = z;
            sG[r * kSZ + c] = gg;
        }
        __syncthreads();
        // dG = dZ W^T for this warp's 16 nodes x 32 columns
        {
            const int mt = w & 1, nh = w >> 1;
            float acc[4][4];
#pragma unroll
            for (int nt = 0; nt < 4; ++nt)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[nt][q] = 0.f;
            const float* zr0 = sZ + (mt * 16 + g) * kSZ;
            const float* zr1 = zr0 + 8 * kSZ;
#pragma unroll
            for (int ks = 0; ks < C / 8; ++ks) {
                const uint32_t a[4] = {to_tf32(zr0[ks * 8 + t]), to_tf32(zr1[ks * 8 + t]), to_tf32(zr0[ks * 8 + t + 4]),
                                       to_tf32(zr1[ks * 8 + t + 4])};
#pragma unroll
                for (int nt = 0; nt < 4; ++nt) {
                    const float* wr = sW + (nh * 32 + nt * 8 + g) * kSW + ks * 8 + t;  // W[j][n], n = k index
                    const uint32_t b[2] = {to_tf32(wr[0]), to_tf32(wr[4])};
                    mma_tf32_1688(acc[nt], a, b);
                }
            }
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                const int col = nh * 32 + nt * 8 + 2 * t;
                const int64_t ra = base + mt * 16 + g, rb = ra + 8;
                if (ra < vend) *reinterpret_cast<float2*>(dG + ra * C + col) = make_float2(acc[nt][0], acc[nt][1]);
                if (rb < vend) *reinterpret_cast<float2*>(dG + rb * C + col) = make_float2(acc[nt][2], acc[nt][3]);
            }
        }
        // dW += G^T dZ: rows w*16 .. +16 of dW, K = the chunk's 32 nodes
#pragma unroll
        for (int ks = 0; ks < kTcChunk / 8; ++ks) {
            const float* g0 = sG + (ks * 8 + t) * kSZ + w * 16 + g;
            const float* g1 = sG + (ks * 8 + t + 4) * kSZ + w * 16 + g;
            const uint32_t a[4] = {to_tf32(g0[0]), to_tf32(g0[8]), to_tf32(g1[0]), to_tf32(g1[8])};
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                const uint32_t b[2] = {to_tf32(sZ[(ks * 8 + t) * kSZ + nt * 8 + g]),
                                       to_tf32(sZ[(ks * 8 + t + 4) * kSZ + nt * 8 + g])};
                mma_tf32_1688(accW[nt], a, b);
            }
        }
        if (threadIdx.x < C)
            for (int r = 0; r < kTcChunk; ++r) bacc += sZ[r * kSZ + threadIdx.x];
    }
    float* wp = wpart + (int64_t)blockIdx.x * C * C;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const int col = nt * 8 + 2 * t, row = w * 16 + g;
        *reinterpret_cast<float2*>(wp + row * C + col) = make_float2(accW[nt][0], accW[nt][1]);
        *reinterpret_cast<float2*>(wp + (row + 8) * C + col) = make_float2(accW[nt][2], accW[nt][3]);
    }
    if (threadIdx.x < C) bpart[(int64_t)blockIdx.x * C + threadIdx.x] = bacc;
}

// input layer: dZ0 = dH0 * (Z0 > 0); dW0 partial = F^T dZ0 (NF x C); db0 partial
template <typename A>
__global__ void input_bwd_kernel(int64_t nc, const float* __restrict__ dH, const A* __restrict__ Z,
                                 const float* __restrict__ feat, float* __restrict__ part, int rows_per_block) {
    const int c = threadIdx.x;
    if (c >= C) return;
    float a1 = 0.f, a2 = 0.f, ab = 0.f;
    const int64_t v0 = (int64_t)blockIdx.x * rows_per_block;
    const int64_t v1 = (v0 + rows_per_block < nc) ? v0 + rows_per_block : nc;
    for (int64_t v = v0; v < v1; ++v) {
        const float d = ld(Z + v * C + c) > 0.f ? dH[v * C + c] : 0.f;
        a1 = fmaf(feat[NF * v], d, a1);
        a2 = fmaf(feat[NF * v + 1], d, a2);
        ab += d;
    }
    float* p = part + (int64_t)blockIdx.x * 3 * C;
    p[c] = a1;
    p[C + c] = a2;
    p[2 * C + c] = ab;
}

// out[k] += sum_b part[b * stride + k]  (fixed order over blocks)
__global__ void reduce_parts_kernel(int n, int nb, int64_t stride, const float* __restrict__ part,
                                    float* __restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    float s = 0.f;
    for (int b = 0; b < nb; ++b) s += part[(int64_t)b * stride + k];
    out[k] += s;
}

// ------------------------------------------------------------ loss pieces
// out = a - b elementwise (out may be a)
__global__ void sub_kernel(int64_t n, const double* a, const double* __restrict__ b, double* out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = a[i] - b[i];
}
__global__ void dot_partial_kernel(int64_t n, const double* __restrict__ a, const double* __restrict__ b,
                                   double* __restrict__ part) {
    __shared__ double sh[32];
    double acc = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        acc += a[i] * b[i];
#pragma unroll
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i];
        part[blockIdx.x] = s;
    }
}
__global__ void scale_kernel(int64_t n, float a, float* __restrict__ x) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) x[i] *= a;
}

__global__ void adam_kernel(int64_t n, float* __restrict__ w, float* __restrict__ g, float* __restrict__ m1,
                            float* __restrict__ m2, float* __restrict__ wk, float lr, float b1, float b2, float eps,
                            float c1, float c2, float gscale, int bf16) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i] * gscale;
    const float a = b1 * m1[i] + (1.f - b1) * gi;
    const float b = b2 * m2[i] + (1.f - b2) * gi * gi;
    m1[i] = a;
    m2[i] = b;
    const float wi = w[i] - lr * (a / c1) / (sqrtf(b / c2) + eps);
    w[i] = wi;
    wk[i] = bf16 ? __bfloat162float(__float2bfloat16_rn(wi)) : wi;
    g[i] = 0.f;
}

__global__ void round_params_kernel(int64_t n, const float* __restrict__ w, float* __restrict__ wk, int bf16) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) wk[i] = bf16 ? __bfloat162float(__float2bfloat16_rn(w[i])) : w[i];
}

// ------------------------------------------------------------ host helpers
#define RC(x)                \
    do {                     \
        int _rc = (x);       \
        if (_rc) return _rc; \
    } while (0)

Gnn* gnn(anigpu_ctx* h) { return static_cast<Gnn*>(h->learned); }

std::atomic<int64_t> g_bind_counter{0};

unsigned nblk(int64_t n, int threads) { return grid_for(n, threads); }

size_t act_size(const Gnn* g) { return g->act == ANIGPU_BF16 ? 2 : 4; }

// activation arrays: H_l (L+1), G_l (L), Z_l (L+1)
void* act_ptr(Gnn* g, int which, int l) {
    const size_t sz = (size_t)g->nc * C * act_size(g);
    int idx = which == 0 ? l : (which == 1 ? (g->layers + 1) + (l - 1) : (2 * g->layers + 1) + l);
    return static_cast<char*>(g->act_buf) + sz * idx;
}

template <typename A>
int forward_t(anigpu_ctx* h, Gnn* g, const Layout& L) {
    cudaStream_t s = h->stream;
    const int64_t nc = g->nc;
    const unsigned wb = nblk(nc * 32, kBlk);
    input_layer_kernel<A><<<wb, kBlk, 0, s>>>(nc, g->feat, g->wk + L.W0, g->wk + L.b0, (A*)act_ptr(g, 2, 0),
                                             (A*)act_ptr(g, 0, 0));
    ANI_LAUNCHED(h);
    for (int l = 1; l <= g->layers; ++l) {
        spmm_kernel<A, A><<<wb, kBlk, 0, s>>>(nc, g->crow, g->ccol, g->cval, (const A*)act_ptr(g, 0, l - 1),
                                              (A*)act_ptr(g, 1, l), 0);
        ANI_LAUNCHED(h);
        if (sizeof(A) == 2)  // BF16 activations: the tensor-core layer
            dense_mma_bf16_kernel<<<(unsigned)((nc + 16 * kMmaWarps - 1) / (16 * kMmaWarps)), 32 * kMmaWarps, 0, s>>>(
                nc, (const __nv_bfloat16*)act_ptr(g, 1, l), g->wk + L.W[l - 1], g->wk + L.b[l - 1],
                (const __nv_bfloat16*)act_ptr(g, 0, l - 1), (__nv_bfloat16*)act_ptr(g, 2, l),
                (__nv_bfloat16*)act_ptr(g, 0, l));
        else
            dense_kernel<A><<<wb, kBlk, 0, s>>>(nc, (const A*)act_ptr(g, 1, l), g->wk + L.W[l - 1],
                                                g->wk + L.b[l - 1], (const A*)act_ptr(g, 0, l - 1),
                                                (A*)act_ptr(g, 2, l), (A*)act_ptr(g, 0, l));
        ANI_LAUNCHED(h);
    }
    output_kernel<A><<<wb, kBlk, 0, s>>>(nc, (const A*)act_ptr(g, 0, g->layers), g->wk + L.wout, g->wk + L.bout,
                                         g->coef);
    ANI_LAUNCHED(h);
    return ANIGPU_OK;
}

template <typename A>
int backward_t(anigpu_ctx* h, Gnn* g, const Layout& L) {
    cudaStream_t s = h->stream;
    const int64_t nc = g->nc;
    int nb = (int)std::min<int64_t>(kMaxPart, (int64_t)nblk(nc * 32, kBlk));
    output_bwd_kernel<A><<<nb, kBlk, 0, s>>>(nc, (const A*)act_ptr(g, 0, g->layers), g->wk + L.wout, g->ga, g->dH,
                                             g->part);
    ANI_LAUNCHED(h);
    reduce_parts_kernel<<<1, C * K + K, 0, s>>>(C * K, nb, C * K + K, g->part, g->g + L.wout);
    ANI_LAUNCHED(h);
    reduce_parts_kernel<<<1, K, 0, s>>>(K, nb, C * K + K, g->part + C * K, g->g + L.bout);
    ANI_LAUNCHED(h);
    const int64_t rpb = std::max<int64_t>(32, ((nc + kMaxPart - 1) / kMaxPart + 31) / 32 * 32);
    const int nbw = (int)((nc + rpb - 1) / rpb);
    for (int l = g->layers; l >= 1; --l) {
        if (sizeof(A) == 2)  // BF16 activations: the tensor-core step
            dense_bwd_tc_kernel<<<nbw, kTcWarps * 32, 0, s>>>(nc, g->dH, (const __nv_bfloat16*)act_ptr(g, 2, l),
                                                              (const __nv_bfloat16*)act_ptr(g, 1, l), g->wk + L.W[l - 1],
                                                              g->dZ, g->dG, g->wpart, g->part, (int)rpb);
        else
            dense_bwd_kernel<A><<<nbw, kBlk, 0, s>>>(nc, g->dH, (const A*)act_ptr(g, 2, l), (const A*)act_ptr(g, 1, l),
                                                     g->wk + L.W[l - 1], g->dZ, g->dG, g->wpart, g->part, (int)rpb);
        ANI_LAUNCHED(h);
        reduce_parts_kernel<<<nblk(C * C, 256), 256, 0, s>>>(C * C, nbw, (int64_t)C * C, g->wpart, g->g + L.W[l - 1]);
        ANI_LAUNCHED(h);
        reduce_parts_kernel<<<1, C, 0, s>>>(C, nbw, C, g->part, g->g + L.b[l - 1]);
        ANI_LAUNCHED(h);
        // dH_{l-1} = dH_l + A_hat dG   (A_hat symmetric)
        spmm_kernel<float, float><<<nblk(nc * 32, kBlk), kBlk, 0, s>>>(nc, g->crow, g->ccol, g->cval, g->dG, g->dH, 1);
        ANI_LAUNCHED(h);
    }
    input_bwd_kernel<A><<<nbw, C, 0, s>>>(nc, g->dH, (const A*)act_ptr(g, 2, 0), g->feat, g->part, (int)rpb);
    ANI_LAUNCHED(h);
    reduce_parts_kernel<<<1, NF * C, 0, s>>>(NF * C, nbw, 3 * C, g->part, g->g + L.W0);
    ANI_LAUNCHED(h);
    reduce_parts_kernel<<<1, C, 0, s>>>(C, nbw, 3 * C, g->part + NF * C, g->g + L.b0);
    ANI_LAUNCHED(h);
    return ANIGPU_OK;
}

// Horner: out = sum_k A_hat^k (coef_k .* s)   (K-1 SpMVs)
int horner(anigpu_ctx* h, Gnn* g, const float* sv, float* out) {
    cudaStream_t st = h->stream;
    const unsigned b = nblk(g->nc, 256);
    cscale_kernel<<<b, 256, 0, st>>>(g->nc, g->coef, K - 1, sv, g->t0);
    ANI_LAUNCHED(h);
    float* cur = g->t0;
    float* nxt = g->t1;
    for (int k = K - 2; k >= 0; --k) {
        float* dst = k == 0 ? out : nxt;
        cspmv_kernel<<<b, 256, 0, st>>>(g->nc, g->crow, g->ccol, g->cval, cur, g->coef, k, sv, dst);
        ANI_LAUNCHED(h);
        std::swap(cur, nxt);
    }
    return ANIGPU_OK;
}

// powers: P_0 = x, P_k = A_hat P_{k-1}, stored in pw[k*nc]
int powers(anigpu_ctx* h, Gnn* g, const float* x, float* pw) {
    cudaStream_t st = h->stream;
    const unsigned b = nblk(g->nc, 256);
    ANI_CUDA(h, cudaMemcpyAsync(pw, x, sizeof(float) * g->nc, cudaMemcpyDeviceToDevice, st));
    for (int k = 1; k < K; ++k) {
        cspmv_kernel<<<b, 256, 0, st>>>(g->nc, g->crow, g->ccol, g->cval, pw + (k - 1) * g->nc, nullptr, 0, nullptr,
                                        pw + k * g->nc);
        ANI_LAUNCHED(h);
    }
    return ANIGPU_OK;
}

// z = M r (and keeps u, w powers for the backward pass)
template <typename T>
int apply_impl(anigpu_ctx* h, Gnn* g, const T* r, T* z) {
    cudaStream_t s = h->stream;
    restrict_kernel<T><<<nblk(g->nc, 256), 256, 0, s>>>(g->nc, g->map, r, g->vrow, g->vedge, g->isd_c, g->u);
    ANI_LAUNCHED(h);
    // w = B^T u = sum_k A_hat^k (a_k .* u); then P_k = A_hat^k w; c = isd .* sum_k a_k .* P_k
    float* wv = g->qv;  // w lives in qv[0..nc) until the backward pass needs qv
    RC(horner(h, g, g->u, wv));
    RC(powers(h, g, wv, g->pw));
    combine_kernel<<<nblk(g->nc, 256), 256, 0, s>>>(g->nc, g->coef, g->pw, g->isd_c, g->cc);
    ANI_LAUNCHED(h);
    prolong_kernel<T><<<nblk(g->nf, 256), 256, 0, s>>>(g->nf, g->map, r, g->diag_f, g->cc, g->edge_ends, z);
    ANI_LAUNCHED(h);
    return ANIGPU_OK;
}

}  // namespace

// Whether a cooperative launch can be captured into a CUDA graph here (the solver's iterations
// are graph-captured): a one-block launch of an empty kernel captured, instantiated and run on a
// private stream, once per process.
bool chain_capture_ok() {
    static int known = -1;
    if (known >= 0) return known == 1;
    cudaStream_t st = nullptr;
    cudaGraph_t gr = nullptr;
    cudaGraphExec_t ge = nullptr;
    bool ok = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess;
    if (ok) {
        int* nul = nullptr;
        void* args[] = {&nul};
        ok = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        if (ok) {
            const cudaError_t e1 = cudaLaunchCooperativeKernel((const void*)chain_probe_kernel, dim3(1), dim3(32), args, 0, st);
            const cudaError_t e2 = cudaStreamEndCapture(st, &gr);
            ok = e1 == cudaSuccess && e2 == cudaSuccess && gr;
        }
        if (ok) ok = cudaGraphInstantiate(&ge, gr, 0) == cudaSuccess;
        if (ok) ok = cudaGraphLaunch(ge, st) == cudaSuccess && cudaStreamSynchronize(st) == cudaSuccess;
    }
    if (ge) cudaGraphExecDestroy(ge);
    if (gr) cudaGraphDestroy(gr);
    if (st) cudaStreamDestroy(st);
    (void)cudaGetLastError();
    known = ok ? 1 : 0;
    return ok;
}

// the slices of the coarse graph and the grid of the fused chain (0: the separate launches)
int chain_setup(anigpu_ctx* h, Gnn* g) {
    cudaStream_t s = h->stream;
    const int64_t ns = (g->nc + 31) / 32;
    unsigned long long* cnt = nullptr;
    ANI_CUDA(h, cudaMallocAsync((void**)&cnt, sizeof(unsigned long long) * (ns + 1), s));
    ANI_CUDA(h, cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * (ns + 1), s));
    sell_count_kernel<<<nblk(g->nc, 256), 256, 0, s>>>(g->nc, g->crow, cnt);
    ANI_LAUNCHED(h);
    RC(dev_alloc(h, &g->sbase, (size_t)ns + 1));
    RC(scan_counts(h, cnt, ns, g->sbase));
    int64_t snnz = 0;
    ANI_CUDA(h, cudaMemcpyAsync(&snnz, g->sbase + ns, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    ANI_CUDA(h, cudaStreamSynchronize(s));
    ANI_CUDA(h, cudaFreeAsync(cnt, s));
    if (snnz != g->snnz || !g->scol) {
        RC(dev_alloc(h, &g->scol, (size_t)std::max<int64_t>(snnz, 1)));
        RC(dev_alloc(h, &g->sval, (size_t)std::max<int64_t>(snnz, 1)));
        g->snnz = snnz;
    }
    sell_fill_kernel<<<nblk(g->nc, 256), 256, 0, s>>>(g->nc, g->crow, g->ccol, g->cval, g->sbase, g->scol, g->sval);
    ANI_LAUNCHED(h);
    if (!g->bar) RC(dev_alloc(h, &g->bar, 3));
    ANI_CUDA(h, cudaMemsetAsync(g->bar, 0, 3 * sizeof(unsigned int), s));
    g->chain_grid = 0;
    int coop = 0, nsm = 0, per_sm = 0;
    ANI_CUDA(h, cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, h->device));
    ANI_CUDA(h, cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, h->device));
    ANI_CUDA(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, coarse_chain_kernel, kChainThreads, 0));
    if (coop && per_sm > 0 && h->chain_enabled && chain_capture_ok())
        g->chain_grid = (int)std::min<int64_t>((int64_t)per_sm * nsm,
                                               std::max<int64_t>(1, (g->nc + kChainThreads - 1) / kChainThreads));
    return ANIGPU_OK;
}

// z = M r in FP32 with fused kernels; nb blocks of partials for r.z and z.qold.  No
// allocation and no synchronisation, so solver iterations around it can be graph-captured.
int gnn_precond_f32(anigpu_ctx* h, const float* r, float* z, const float* qold, double* part_rz, double* part_zq,
                    int nb, const int* stop) {
    Gnn* g = gnn(h);
    cudaStream_t s = h->stream;
    if (g->chain_grid > 0) {
        ChainArgs a{g->nc, g->map, r, g->vrow, g->vedge, g->isd_c, g->coef, g->sbase, g->scol, g->sval,
                    g->u, g->t0, g->t1, g->pw, g->cc, g->bar, h->d_status, stop};
        void* args[] = {&a};
        ANI_CUDA(h, cudaLaunchCooperativeKernel((const void*)coarse_chain_kernel, dim3(g->chain_grid), dim3(kChainThreads),
                                                args, 0, s));
        ANI_LAUNCHED(h);
        prolong_dot_kernel<<<nb, 256, 0, s>>>(g->nf, g->map, r, g->diag_f, g->cc, g->edge_ends, qold, z, part_rz,
                                              part_zq, stop);
        ANI_LAUNCHED(h);
        return ANIGPU_OK;
    }
    const unsigned bc = nblk(g->nc * CW, 256);
    restrict_scale_kernel<<<bc, 256, 0, s>>>(g->nc, g->map, r, g->vrow, g->vedge, g->isd_c, g->coef, g->u, g->t0, stop);
    ANI_LAUNCHED(h);
    float* cur = g->t0;
    float* nxt = g->t1;
    for (int k = K - 2; k >= 0; --k) {  // Horner: w = sum_k A_hat^k (a_k .* u), into pw[0]
        float* dst = k == 0 ? g->pw : nxt;
        cspmv4_kernel<<<bc, 256, 0, s>>>(g->nc, g->crow, g->ccol, g->cval, cur, g->coef, k, g->u, dst, stop);
        ANI_LAUNCHED(h);
        std::swap(cur, nxt);
    }
    for (int k = 1; k <= K - 2; ++k) {  // P_k = A_hat^k w
        cspmv4_kernel<<<bc, 256, 0, s>>>(g->nc, g->crow, g->ccol, g->cval, g->pw + (k - 1) * g->nc, nullptr, 0,
                                         nullptr, g->pw + k * g->nc, stop);
        ANI_LAUNCHED(h);
    }
    combine4_kernel<<<bc, 256, 0, s>>>(g->nc, g->crow, g->ccol, g->cval, g->pw, g->coef, g->isd_c, g->cc, stop);
    ANI_LAUNCHED(h);
    prolong_dot_kernel<<<nb, 256, 0, s>>>(g->nf, g->map, r, g->diag_f, g->cc, g->edge_ends, qold, z, part_rz, part_zq,
                                          stop);
    ANI_LAUNCHED(h);
    return ANIGPU_OK;
}

int64_t gnn_bind_generation(anigpu_ctx* h) { return gnn(h) ? gnn(h)->bind_gen : -1; }
int gnn_chain_active(anigpu_ctx* h) { return gnn(h) && gnn(h)->bound && gnn(h)->chain_grid > 0 ? 1 : 0; }

// ------------------------------------------------------------ entry points
int gnn_init(anigpu_ctx* h, int layers, int act, uint64_t seed) {
    if (layers < 1 || layers > kMaxLayers) return set_err(h, ANIGPU_ERR_ARG, "layers must be 1..8");
    if (act != ANIGPU_F32 && act != ANIGPU_BF16) return set_err(h, ANIGPU_ERR_ARG, "activation precision");
    free_learned(h);
    Gnn* g = new Gnn();
    h->learned = g;
    g->layers = layers;
    g->act = act;
    const Layout L = layout(layers);
    g->nparam = L.total;
    RC(dev_alloc(h, &g->w, L.total));
    RC(dev_alloc(h, &g->g, L.total));
    RC(dev_alloc(h, &g->m1, L.total));
    RC(dev_alloc(h, &g->m2, L.total));
    RC(dev_alloc(h, &g->wk, L.total));
    // deterministic init (splitmix64 -> uniform): He-uniform hidden weights, zero biases, small
    // output weights, b_out = (1, 0, ...) so that the untrained B is the identity
    std::vector<float> w(L.total, 0.f);
    uint64_t st = seed;
    auto next = [&]() {
        uint64_t z = (st += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
    };
    for (int k = 0; k < NF * C; ++k) w[L.W0 + k] = (float)(next() * std::sqrt(6.0 / NF));
    for (int l = 0; l < layers; ++l)
        for (int k = 0; k < C * C; ++k) w[L.W[l] + k] = (float)(next() * std::sqrt(6.0 / C) * 0.3);
    for (int k = 0; k < C * K; ++k) w[L.wout + k] = (float)(next() * std::sqrt(3.0 / C) * 0.01);
    w[L.bout] = 1.f;
    ANI_CUDA(h, cudaMemcpyAsync(g->w, w.data(), sizeof(float) * L.total, cudaMemcpyHostToDevice, h->stream));
    ANI_CUDA(h, cudaMemsetAsync(g->g, 0, sizeof(float) * L.total, h->stream));
    ANI_CUDA(h, cudaMemsetAsync(g->m1, 0, sizeof(float) * L.total, h->stream));
    ANI_CUDA(h, cudaMemsetAsync(g->m2, 0, sizeof(float) * L.total, h->stream));
    round_params_kernel<<<nblk(L.total, 256), 256, 0, h->stream>>>(L.total, g->w, g->wk, act == ANIGPU_BF16);
    ANI_LAUNCHED(h);
    ANI_CUDA(h, cudaStreamSynchronize(h->stream));
    return ANIGPU_OK;
}

int64_t gnn_num_params(anigpu_ctx* h) { return gnn(h) ? gnn(h)->nparam : -1; }

int gnn_forward_coefs(anigpu_ctx* h) {
    Gnn* g = gnn(h);
    const Layout L = layout(g->layers);
    if (g->act == ANIGPU_BF16) return forward_t<__nv_bfloat16>(h, g, L);
    return forward_t<float>(h, g, L);
}

int gnn_params(anigpu_ctx* h, float* host, int64_t n, int set, int which) {
    Gnn* g = gnn(h);
    if (!g) return set_err(h, ANIGPU_ERR_STATE, "anigpu_gnn_init not called");
    if (n != g->nparam) return set_err(h, ANIGPU_ERR_ARG, "parameter count mismatch");
    float* dev = which == 0 ? g->w : g->g;
    if (set) {
        ANI_CUDA(h, cudaMemcpyAsync(dev, host, sizeof(float) * n, cudaMemcpyHostToDevice, h->stream));
        if (which == 0) {
            round_params_kernel<<<nblk(n, 256), 256, 0, h->stream>>>(n, g->w, g->wk, g->act == ANIGPU_BF16);
            ANI_LAUNCHED(h);
            if (g->bound) RC(gnn_forward_coefs(h));  // new parameters: new coefficients
        }
    } else {
        ANI_CUDA(h, cudaMemcpyAsync(host, dev, sizeof(float) * n, cudaMemcpyDeviceToHost, h->stream));
    }
    ANI_CUDA(h, cudaStreamSynchronize(h->stream));
    return ANIGPU_OK;
}

int gnn_bind(anigpu_ctx* h, const void* vals, int precision, int kind, const double* D) {
    Gnn* g = gnn(h);
    if (!g) return set_err(h, ANIGPU_ERR_STATE, "anigpu_gnn_init not called");
    if (h->space != ANIGPU_P2 && h->space != ANIGPU_VEC3_P2)
        return set_err(h, ANIGPU_ERR_UNSUPPORTED, "the learned preconditioner needs a P2 or vector P2 problem");
    if (!vals) return set_err(h, ANIGPU_ERR_ARG, "NULL values");
    if (kind != ANIGPU_TENSOR_NULL && !D) return set_err(h, ANIGPU_ERR_ARG, "NULL tensor");
    cudaStream_t s = h->stream;
    const int f32 = precision == ANIGPU_F32;
    const int64_t nc = h->ncomp * h->nv;
    const bool resize = g->nc != nc || g->nf != h->ndof || g->map.nv != h->nv || g->map.nds != h->nds;
    g->nc = nc;
    g->map = CMap{h->nv, h->nds};
    g->nf = h->ndof;
    if (resize) {
        RC(dev_alloc(h, &g->crow, g->nc + 1));
        RC(dev_alloc(h, &g->diag_f, g->nf));
        RC(dev_alloc(h, &g->isd_c, g->nc));
        RC(dev_alloc(h, &g->feat, NF * g->nc));
        RC(dev_alloc(h, &g->edge_ends, 2 * std::max<int64_t>(h->ne, 1)));
        RC(dev_alloc(h, &g->vrow, h->nv + 1));
        RC(dev_alloc(h, &g->vedge, 2 * std::max<int64_t>(h->ne, 1)));
        RC(dev_alloc(h, &g->dpart, 2 * kMaxPart));
        RC(dev_alloc(h, &g->coef, (size_t)K * g->nc));
        RC(dev_alloc(h, &g->u, g->nc));
        RC(dev_alloc(h, &g->pw, (size_t)K * g->nc));
        RC(dev_alloc(h, &g->qv, (size_t)K * g->nc));
        RC(dev_alloc(h, &g->t0, g->nc));
        RC(dev_alloc(h, &g->t1, g->nc));
        RC(dev_alloc(h, &g->cc, g->nc));
        RC(dev_alloc(h, &g->ga, (size_t)K * g->nc));
        RC(dev_alloc(h, &g->dH, g->nc * C));
        RC(dev_alloc(h, &g->dG, g->nc * C));
        RC(dev_alloc(h, &g->dZ, g->nc * C));
        RC(dev_alloc(h, &g->part, (size_t)kMaxPart * (C * K + K)));
        RC(dev_alloc(h, &g->wpart, (size_t)kMaxPart * C * C));
        RC(dev_alloc(h, &g->fine_tmp, g->nf));
        RC(dev_alloc(h, &g->fine_tmp2, g->nf));
        g->act_bytes = (size_t)g->nc * C * act_size(g) * (3 * g->layers + 2);
        if (g->act_buf) cudaFree(g->act_buf);
        g->act_buf = nullptr;
        ANI_CUDA(h, cudaMalloc(&g->act_buf, g->act_bytes));
    }
    fine_diag_kernel<<<nblk(g->nf, 256), 256, 0, s>>>(g->nf, h->rowptr, h->col, vals, f32, g->diag_f);
    ANI_LAUNCHED(h);
    unsigned long long* cnt = nullptr;
    ANI_CUDA(h, cudaMallocAsync((void**)&cnt, sizeof(unsigned long long) * (g->nc + 1), s));
    ANI_CUDA(h, cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * (g->nc + 1), s));
    coarse_count_kernel<<<nblk(g->nc, 256), 256, 0, s>>>(g->nc, g->map, h->rowptr, h->col, cnt);
    ANI_LAUNCHED(h);
    RC(scan_counts(h, cnt, g->nc, g->crow));
    int64_t cnnz = 0;
    ANI_CUDA(h, cudaMemcpyAsync(&cnnz, g->crow + g->nc, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    ANI_CUDA(h, cudaStreamSynchronize(s));
    ANI_CUDA(h, cudaFreeAsync(cnt, s));
    if (cnnz != g->cnnz || !g->ccol) {
        RC(dev_alloc(h, &g->ccol, std::max<int64_t>(cnnz, 1)));
        RC(dev_alloc(h, &g->cval, std::max<int64_t>(cnnz, 1)));
        g->cnnz = cnnz;
    }
    coarse_fill_kernel<<<nblk(g->nc, 256), 256, 0, s>>>(g->nc, g->map, h->rowptr, h->col, vals, f32, g->diag_f, g->crow,
                                                        g->ccol, g->cval, g->isd_c);
    ANI_LAUNCHED(h);
    RC(chain_setup(h, g));
    static_feat_kernel<<<nblk(g->nc, 256), 256, 0, s>>>(g->nc, g->map, g->diag_f, h->inc_ptr, h->recs, kind, D, g->feat);
    ANI_LAUNCHED(h);
    const int nb = (int)std::min<int64_t>(kMaxPart, nblk(g->nc, 256));
    feat_partial_kernel<<<nb, 256, 0, s>>>(g->nc, g->feat, g->part);
    ANI_LAUNCHED(h);
    feat_center_kernel<<<nb, 256, 0, s>>>(g->nc, nb, g->part, g->feat);
    ANI_LAUNCHED(h);
    edge_ends_kernel<<<nblk(std::max<int64_t>(h->ne, 1), 256), 256, 0, s>>>(h->ne, h->nv, h->inc_ptr, h->recs, h->tets,
                                                                          g->edge_ends);
    ANI_LAUNCHED(h);
    {
        unsigned long long* vc = nullptr;
        ANI_CUDA(h, cudaMallocAsync((void**)&vc, sizeof(unsigned long long) * 2 * (h->nv + 1), s));
        ANI_CUDA(h, cudaMemsetAsync(vc, 0, sizeof(unsigned long long) * 2 * (h->nv + 1), s));
        const unsigned eb = nblk(std::max<int64_t>(h->ne, 1), 256);
        vedge_count_kernel<<<eb, 256, 0, s>>>(h->ne, g->edge_ends, vc);
        ANI_LAUNCHED(h);
        RC(scan_counts(h, vc, h->nv, g->vrow));
        vedge_fill_kernel<<<eb, 256, 0, s>>>(h->ne, h->nv, g->edge_ends, g->vrow, vc + h->nv + 1, g->vedge);
        ANI_LAUNCHED(h);
        vedge_sort_kernel<<<nblk(h->nv, 256), 256, 0, s>>>(h->nv, g->vrow, g->vedge);
        ANI_LAUNCHED(h);
        ANI_CUDA(h, cudaFreeAsync(vc, s));
    }
    g->bound_vals = vals;
    g->bound_prec = precision;
    g->bound = true;
    g->bind_gen = ++g_bind_counter;  // unique over every state of every handle
    RC(gnn_forward_coefs(h));
    ANI_CUDA(h, cudaStreamSynchronize(s));
    return ANIGPU_OK;
}

int gnn_apply(anigpu_ctx* h, const double* r, double* z) {
    Gnn* g = gnn(h);
    if (!g || !g->bound) return set_err(h, ANIGPU_ERR_STATE, "anigpu_gnn_bind not called");
    return apply_impl<double>(h, g, r, z);
}

int gnn_coefficients(anigpu_ctx* h, float* coef) {
    Gnn* g = gnn(h);
    if (!g || !g->bound) return set_err(h, ANIGPU_ERR_STATE, "anigpu_gnn_bind not called");
    if (!coef) return set_err(h, ANIGPU_ERR_ARG, "NULL output");
    ANI_CUDA(h, cudaMemcpyAsync(coef, g->coef, sizeof(float) * K * g->nc, cudaMemcpyDeviceToDevice, h->stream));
    ANI_CUDA(h, cudaStreamSynchronize(h->stream));
    return ANIGPU_OK;
}

int gnn_apply_f32(anigpu_ctx* h, const float* r, float* z) {
    Gnn* g = gnn(h);
    if (!g || !g->bound) return set_err(h, ANIGPU_ERR_STATE, "anigpu_gnn_bind not called");
    const int nb = (int)std::min<int64_t>(kMaxPart, nblk(g->nf, 256));
    return gnn_precond_f32(h, r, z, nullptr, g->dpart, g->dpart + kMaxPart, nb, nullptr);
}

// forward + backward for one pair; accumulates gradients; loss to host
int gnn_loss_grad(anigpu_ctx* h, const double* r, const double* e, double* loss) {
    Gnn* g = gnn(h);
    if (!g || !g->bound) return set_err(h, ANIGPU_ERR_STATE, "anigpu_gnn_bind not called");
    cudaStream_t s = h->stream;
    const Layout L = layout(g->layers);
    double* m = g->fine_tmp;
    double* q = g->fine_tmp2;
    RC(apply_impl<double>(h, g, r, m));
    // d = m - e (into m), q = A d
    sub_kernel<<<nblk(g->nf, 256), 256, 0, s>>>(g->nf, m, e, m);
    ANI_LAUNCHED(h);
    RC(run_spmv(h, g->bound_vals, g->bound_prec, m, q));
    const int nb = (int)std::min<int64_t>(kMaxPart, nblk(g->nf, 256));
    double* dpart = reinterpret_cast<double*>(g->wpart);
    dot_partial_kernel<<<nb, 256, 0, s>>>(g->nf, m, q, dpart);
    ANI_LAUNCHED(h);
    RC(run_spmv(h, g->bound_vals, g->bound_prec, e, m));
    dot_partial_kernel<<<nb, 256, 0, s>>>(g->nf, e, m, dpart + kMaxPart);
    ANI_LAUNCHED(h);
    std::vector<double> hp(2 * kMaxPart);
    ANI_CUDA(h, cudaMemcpyAsync(hp.data(), dpart, sizeof(double) * 2 * kMaxPart, cudaMemcpyDeviceToHost, s));
    ANI_CUDA(h, cudaStreamSynchronize(s));
    double dq = 0, eae = 0;
    for (int b = 0; b < nb; ++b) {
        dq += hp[b];
        eae += hp[kMaxPart + b];
    }
    if (!(eae > 0)) return set_err(h, ANIGPU_ERR_ARG, "e^T A e is not positive");
    *loss = dq / eae;
    // dL/dc = 2/eAe P^T q ; g' = Dc^-1/2 dL/dc = 2/eAe * restrict(q) (restrict includes Dc^-1/2)
    float* gp = g->cc;
    restrict_kernel<double><<<nblk(g->nc, 256), 256, 0, s>>>(g->nc, g->map, q, g->vrow, g->vedge, g->isd_c, gp);
    ANI_LAUNCHED(h);
    scale_kernel<<<nblk(g->nc, 256), 256, 0, s>>>(g->nc, (float)(2.0 / eae), gp);
    ANI_LAUNCHED(h);
    // v = B^T g' = sum_k A_hat^k (a_k .* g'); Q_k = A_hat^k v; dL/da_k = g' .* P_k + u .* Q_k
    float* vv = g->ga;  // v staged in ga (overwritten by the gradient below)
    RC(horner(h, g, gp, vv));
    RC(powers(h, g, vv, g->qv));
    coef_grad_kernel<<<nblk(g->nc, 256), 256, 0, s>>>(g->nc, gp, g->pw, g->u, g->qv, g->ga);
    ANI_LAUNCHED(h);
    if (g->act == ANIGPU_BF16) RC(backward_t<__nv_bfloat16>(h, g, L));
    else RC(backward_t<float>(h, g, L));
    ANI_CUDA(h, cudaStreamSynchronize(s));
    return ANIGPU_OK;
}

int gnn_adam(anigpu_ctx* h, float lr, float b1, float b2, float eps, int step, float gscale) {
    Gnn* g = gnn(h);
    if (!g) return set_err(h, ANIGPU_ERR_STATE, "anigpu_gnn_init not called");
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    adam_kernel<<<nblk(g->nparam, 256), 256, 0, h->stream>>>(g->nparam, g->w, g->g, g->m1, g->m2, g->wk, lr, b1, b2,
                                                             eps, c1, c2, gscale, g->act == ANIGPU_BF16);
    ANI_LAUNCHED(h);
    if (g->bound) RC(gnn_forward_coefs(h));
    return ANIGPU_OK;
}

int gnn_zero_grads(anigpu_ctx* h) {
    Gnn* g = gnn(h);
    if (!g) return set_err(h, ANIGPU_ERR_STATE, "anigpu_gnn_init not called");
    ANI_CUDA(h, cudaMemsetAsync(g->g, 0, sizeof(float) * g->nparam, h->stream));
    return ANIGPU_OK;
}

bool gnn_bound_to(anigpu_ctx* h, const void* vals) {
    Gnn* g = gnn(h);
    return g && g->bound && g->bound_vals == vals;
}

const float* gnn_fine_diag(anigpu_ctx* h) { return gnn(h) ? gnn(h)->diag_f : nullptr; }

void learned_invalidate(anigpu_ctx* h) {
    free_fcg(h);
    if (Gnn* g = gnn(h)) {
        g->bound = false;
        g->bound_vals = nullptr;
    }
}

void free_learned(anigpu_ctx* h) {
    free_fcg(h);
    Gnn* g = gnn(h);
    if (!g) return;
    void* ptrs[] = {g->w,      g->g,  g->m1, g->m2, g->wk, g->crow, g->ccol, g->cval, g->diag_f, g->isd_c,
                    g->feat,   g->edge_ends, g->vrow, g->vedge, g->dpart, g->coef, g->act_buf, g->u, g->pw, g->qv, g->t0, g->t1,
                    g->cc,     g->ga, g->dH, g->dG, g->dZ, g->part, g->wpart, g->fine_tmp, g->fine_tmp2,
                    g->sbase,  g->scol, g->sval, g->bar};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete g;
    h->learned = nullptr;
}
