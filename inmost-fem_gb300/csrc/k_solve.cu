// Krylov solve of the assembled system (the reference hands its Sparse::Matrix to
// INMOST's Solver, examples/tutorials/ex1.cpp:161-163; that solver is external to the
// reference, so this file is the replacement named by the path, not a restatement).
//
//   * CSR SpMV: a group of W lanes per row (W = 8 for P2-like rows, 4 for P1), FP64 or
//     FP32 values, FP64 or FP32 vectors, accumulation in the vector type.
//   * Jacobi-PCG: five kernels per iteration
//       spmv_dot   q = A p, block partials of p.q
//       alpha      (one block) alpha = rz / pq
//       update     x += alpha p; r -= alpha q; z = Dinv r; partials r.z, r.r
//       beta       (one block) beta = rz_new / rz; convergence flag
//       pupdate    p = z + beta p
//     Every global reduction is two-stage with a fixed order (per-block tree, then one block
//     sums the block partials in index order), so runs are bitwise reproducible.  The scalars live on the device; a converged solve sets a device flag
//     after which the remaining kernels of a batch return immediately, so batches of
//     iterations run from a captured CUDA graph without host round trips.
//   * IR_CG32: FP32-SpMV Jacobi-CG on FP32 vectors inside FP64 iterative refinement
//     (outer residual b - A x in FP64 arithmetic).
#include <cmath>

#include "anigpu_internal.h"
#include "learned.h"
#include "spmv_vec3.cuh"

namespace {

constexpr int kBlock = 256;
constexpr int kMaxBlocks = 2048;
#ifndef SOLVE_W_P2
#define SOLVE_W_P2 4
#endif

struct PcgScalars {
    double rz[2];     // r.z by iteration parity
    double alpha;     // step length of the current iteration
    double bb;        // ||b||^2 (or of the refinement rhs)
    double tol2;      // (rtol * ||b||)^2
    double rr;        // last ||r||^2
    double beta;      // direction update of the current iteration
    long long iter;   // completed iterations
    long long maxit;
    int done;         // 1 converged, 2 breakdown / maxit
    int pad;
};

template <typename T>
__device__ inline T block_reduce_sum(T v, T* sh) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    T s = 0;
    if (threadIdx.x == 0) {
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i];
    }
    return s;  // valid in thread 0
}

// fixed-order sum of nb partials, result broadcast to the whole block
__device__ inline double sum_partials(const double* part, int nb, double* sh) {
    double v = 0;
    // each thread sums a strided subset in index order; then a fixed tree
    for (int i = threadIdx.x; i < nb; i += blockDim.x) v += part[i];
    double s = block_reduce_sum(v, sh);
    __syncthreads();
    if (threadIdx.x == 0) sh[32] = s;
    __syncthreads();
    return sh[32];
}

template <typename VR, typename T, int W>
__global__ void __launch_bounds__(kBlock) spmv_kernel(int64_t n, const int64_t* __restrict__ rowptr,
                                                      const int32_t* __restrict__ col, const VR* __restrict__ vals,
                                                      const T* __restrict__ x, T* __restrict__ y) {
    const int64_t gid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t row = gid / W;
    const int lane = threadIdx.x & (W - 1);
    T s = 0;
    if (row < n) {
        const int64_t b = rowptr[row], e = rowptr[row + 1];
        for (int64_t k = b + lane; k < e; k += W) s += T(vals[k]) * x[col[k]];
    }
#pragma unroll
    for (int o = W / 2; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, W);
    if (row < n && lane == 0) y[row] = s;
}

// q = A p ; partial p.q
template <typename VR, typename T, int W>
__global__ void __launch_bounds__(kBlock) spmv_dot_kernel(int64_t n, const int64_t* __restrict__ rowptr,
                                                          const int32_t* __restrict__ col, const VR* __restrict__ vals,
                                                          const T* __restrict__ p, T* __restrict__ q,
                                                          double* __restrict__ part, const PcgScalars* __restrict__ sc) {
    __shared__ double sh[33];
    if (sc->done) return;
    const int64_t rows_per_block = kBlock / W;
    // per-thread partial in the vector type (a few rows per thread), block sum in FP64:
    // the FP32 solve keeps FP64 instructions off its per-row path
    T acc = 0;
    for (int64_t base = blockIdx.x * rows_per_block; base < n; base += (int64_t)gridDim.x * rows_per_block) {
        const int64_t row = base + threadIdx.x / W;
        const int lane = threadIdx.x & (W - 1);
        T s = 0;
        if (row < n) {
            const int64_t b = rowptr[row], e = rowptr[row + 1];
            for (int64_t k = b + lane; k < e; k += W) s += T(vals[k]) * p[col[k]];
        }
#pragma unroll
        for (int o = W / 2; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, W);
        if (row < n && lane == 0) {
            q[row] = s;
            acc += s * p[row];
        }
    }
    const double tot = block_reduce_sum((double)acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

// q = A p ; partial p.q -- vector (3-component) template, W lanes per scalar row
template <typename VR, typename T, int W>
__global__ void __launch_bounds__(kBlock, SPMV3_MINB) spmv3_dot_kernel(int64_t nds, int64_t nnz_s,
                                                           const int64_t* __restrict__ rowptr_s,
                                                           const int32_t* __restrict__ col_s,
                                                           const VR* __restrict__ vals, const T* __restrict__ p,
                                                           T* __restrict__ q, double* __restrict__ part,
                                                           const PcgScalars* __restrict__ sc) {
    __shared__ double sh[33];
    if (sc->done) return;
    const int64_t rows_per_block = kBlock / W;
    const int lane = threadIdx.x & (W - 1);
    T acc = 0;
    for (int64_t base = blockIdx.x * rows_per_block; base < nds; base += (int64_t)gridDim.x * rows_per_block) {
        const int64_t r = base + threadIdx.x / W;
        T s0, s1, s2;
        vec3_rows<W>(r, lane, nds, nnz_s, rowptr_s, col_s, vals, p, s0, s1, s2);
        if (r < nds && lane == 0) {
            q[r] = s0;
            q[nds + r] = s1;
            q[2 * nds + r] = s2;
            acc += s0 * p[r] + s1 * p[nds + r] + s2 * p[2 * nds + r];
        }
    }
    const double tot = block_reduce_sum((double)acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

// q = A p ; partial p.q with the kernel that fits the template; returns the partial count
template <typename VR, typename T, int W>
int launch_spmv_dot(anigpu_ctx* h, int nb_rows, int nb3, const VR* vals, const T* p, T* q, double* part,
                    const PcgScalars* sc) {
    if (h->ncomp == 3) {
        spmv3_dot_kernel<VR, T, SPMV3_W><<<nb3, kBlock, 0, h->stream>>>(h->nds, h->nnz_s, h->rowptr_s, h->col_s,
                                                                        vals, p, q, part, sc);
        return nb3;
    }
    spmv_dot_kernel<VR, T, W><<<nb_rows, kBlock, 0, h->stream>>>(h->ndof, h->rowptr, h->col, vals, p, q, part, sc);
    return nb_rows;
}

// alpha = rz / pq, once (one block); the vector kernels read it
__global__ void alpha_kernel(int parity, const double* __restrict__ part_pq, int nb, PcgScalars* __restrict__ sc) {
    __shared__ double sh[33];
    if (sc->done) return;
    const double pq = sum_partials(part_pq, nb, sh);
    if (threadIdx.x == 0) sc->alpha = sc->rz[parity] / pq;
}

// x += alpha p ; r -= alpha q ; z = dinv r ; partials r.z and r.r
template <typename T, typename X>
__global__ void __launch_bounds__(kBlock) update_kernel(int64_t n, X* __restrict__ x, T* __restrict__ r,
                                                        T* __restrict__ z, const T* __restrict__ p,
                                                        const T* __restrict__ q, const T* __restrict__ dinv,
                                                        double* __restrict__ part_rz, double* __restrict__ part_rr,
                                                        const PcgScalars* __restrict__ sc) {
    __shared__ double sh[33];
    if (sc->done) return;
    const double alpha = sc->alpha;
    const T a = (T)alpha;
    const X ax = (X)alpha;
    T arz = 0, arr = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x[i] += ax * (X)p[i];
        const T ri = r[i] - a * q[i];
        r[i] = ri;
        const T zi = dinv[i] * ri;
        z[i] = zi;
        arz += ri * zi;
        arr += ri * ri;
    }
    const double trz = block_reduce_sum((double)arz, sh);
    __syncthreads();
    const double trr = block_reduce_sum((double)arr, sh);
    if (threadIdx.x == 0) {
        part_rz[blockIdx.x] = trz;
        part_rr[blockIdx.x] = trr;
    }
}

// beta = rz_new / rz and the convergence / breakdown flags, once (one block)
__global__ void beta_kernel(int parity, const double* __restrict__ part_rz, const double* __restrict__ part_rr, int nb,
                            PcgScalars* __restrict__ sc) {
    __shared__ double sh[33];
    if (sc->done) return;
    const double rz_new = sum_partials(part_rz, nb, sh);
    const double rr = sum_partials(part_rr, nb, sh);
    if (threadIdx.x == 0) {
        const double beta = rz_new / sc->rz[parity];
        sc->beta = beta;
        sc->rz[parity ^ 1] = rz_new;
        sc->rr = rr;
        sc->iter += 1;
        if (rr <= sc->tol2) sc->done = 1;
        else if (!isfinite(rr) || !isfinite(beta) || sc->iter >= sc->maxit) sc->done = 2;
    }
}

// p = z + beta p
template <typename T>
__global__ void __launch_bounds__(kBlock) pupdate_kernel(int64_t n, T* __restrict__ p, const T* __restrict__ z,
                                                         const PcgScalars* __restrict__ sc) {
    if (sc->done) return;
    const T b = (T)sc->beta;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = z[i] + b * p[i];
}

// r = b - A x (FP64 vectors), z = dinv r, p = z; partials r.z, r.r, b.b
template <typename VR, typename T, int W>
__global__ void __launch_bounds__(kBlock) init_kernel(int64_t n, const int64_t* __restrict__ rowptr,
                                                      const int32_t* __restrict__ col, const VR* __restrict__ vals,
                                                      const double* __restrict__ xin, const double* __restrict__ b,
                                                      T* __restrict__ r, T* __restrict__ z, T* __restrict__ p,
                                                      const T* __restrict__ dinv, double* __restrict__ part_rz,
                                                      double* __restrict__ part_rr, double* __restrict__ part_bb,
                                                      int x_is_zero) {
    __shared__ double sh[33];
    const int64_t rows_per_block = kBlock / W;
    double arz = 0, arr = 0, abb = 0;
    for (int64_t base = blockIdx.x * rows_per_block; base < n; base += (int64_t)gridDim.x * rows_per_block) {
        const int64_t row = base + threadIdx.x / W;
        const int lane = threadIdx.x & (W - 1);
        double s = 0;
        if (row < n && !x_is_zero) {
            const int64_t bb = rowptr[row], e = rowptr[row + 1];
            for (int64_t k = bb + lane; k < e; k += W) s += (double)vals[k] * xin[col[k]];
        }
#pragma unroll
        for (int o = W / 2; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, W);
        if (row < n && lane == 0) {
            const double ri = b[row] - s;
            const T rt = (T)ri;
            const T zt = dinv[row] * rt;
            r[row] = rt;
            z[row] = zt;
            p[row] = zt;
            arz += (double)rt * (double)zt;
            arr += ri * ri;
            abb += b[row] * b[row];
        }
    }
    double t = block_reduce_sum(arz, sh);
    __syncthreads();
    if (threadIdx.x == 0) part_rz[blockIdx.x] = t;
    t = block_reduce_sum(arr, sh);
    __syncthreads();
    if (threadIdx.x == 0) part_rr[blockIdx.x] = t;
    t = block_reduce_sum(abb, sh);
    if (threadIdx.x == 0) part_bb[blockIdx.x] = t;
}

__global__ void init_scalars_kernel(PcgScalars* sc, const double* part_rz, const double* part_rr,
                                    const double* part_bb, int nb, double rtol, long long maxit, int use_bb_of_rhs,
                                    double bb_ext) {
    __shared__ double sh[33];
    const double rz = sum_partials(part_rz, nb, sh);
    const double rr = sum_partials(part_rr, nb, sh);
    const double bb = sum_partials(part_bb, nb, sh);
    if (threadIdx.x == 0) {
        sc->rz[0] = rz;
        sc->rz[1] = rz;
        sc->rr = rr;
        sc->bb = use_bb_of_rhs ? bb : bb_ext;
        sc->tol2 = rtol * rtol * sc->bb;
        sc->iter = 0;
        sc->maxit = maxit;
        sc->done = (rr <= sc->tol2) ? 1 : 0;
    }
}

template <typename VR, typename T>
__global__ void diag_inv_kernel(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                const VR* __restrict__ vals, T* __restrict__ dinv) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= n) return;
    double d = 0;
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k)
        if (col[k] == r) {
            d = (double)vals[k];
            break;
        }
    dinv[r] = (T)(d != 0 ? 1.0 / d : 1.0);
}

// y (f64) = b - A x with f64 arithmetic; partial ||y||^2
template <typename VR, int W>
__global__ void __launch_bounds__(kBlock) residual_kernel(int64_t n, const int64_t* __restrict__ rowptr,
                                                          const int32_t* __restrict__ col, const VR* __restrict__ vals,
                                                          const double* __restrict__ x, const double* __restrict__ b,
                                                          double* __restrict__ y, double* __restrict__ part) {
    __shared__ double sh[33];
    const int64_t rows_per_block = kBlock / W;
    double acc = 0;
    for (int64_t base = blockIdx.x * rows_per_block; base < n; base += (int64_t)gridDim.x * rows_per_block) {
        const int64_t row = base + threadIdx.x / W;
        const int lane = threadIdx.x & (W - 1);
        double s = 0;
        if (row < n) {
            const int64_t bb = rowptr[row], e = rowptr[row + 1];
            for (int64_t k = bb + lane; k < e; k += W) s += (double)vals[k] * x[col[k]];
        }
#pragma unroll
        for (int o = W / 2; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, W);
        if (row < n && lane == 0) {
            const double ri = b[row] - s;
            y[row] = ri;
            acc += ri * ri;
        }
    }
    const double t = block_reduce_sum(acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

__global__ void sum_kernel(const double* part, int nb, double* out) {
    __shared__ double sh[33];
    const double s = sum_partials(part, nb, sh);
    if (threadIdx.x == 0) *out = s;
}

// x (f64) += d (f32)
__global__ void axpy_mixed_kernel(int64_t n, double* __restrict__ x, const float* __restrict__ d) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) x[i] += (double)d[i];
}

// ---------------------------------------------------------------- workspace
struct SolveWs {
    int64_t n = 0;
    // f64 vectors
    double *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr, *dinv = nullptr, *res = nullptr;
    // f32 vectors
    float *r32 = nullptr, *z32 = nullptr, *p32 = nullptr, *q32 = nullptr, *dinv32 = nullptr, *d32 = nullptr;
    float* vals32 = nullptr;  // f32 copy of f64 values when needed
    double* part = nullptr;   // 4 * kMaxBlocks
    double* scal = nullptr;   // misc scalars
    PcgScalars* sc = nullptr;
};

int ensure_ws(anigpu_ctx* h, SolveWs** out) {
    SolveWs* w = (SolveWs*)h->solve_ws;
    if (w && w->n == h->ndof) {
        *out = w;
        return ANIGPU_OK;
    }
    if (w) {
        void* ptrs[] = {w->r, w->z, w->p, w->q, w->dinv, w->res, w->r32, w->z32, w->p32, w->q32, w->dinv32, w->d32,
                        w->vals32, w->part, w->scal, w->sc};
        for (void* q : ptrs)
            if (q) cudaFree(q);
        delete w;
        h->solve_ws = nullptr;
    }
    w = new SolveWs();
    w->n = h->ndof;
    const size_t n = (size_t)h->ndof;
    int rc = 0;
    rc |= dev_alloc(h, &w->r, n);
    rc |= dev_alloc(h, &w->z, n);
    rc |= dev_alloc(h, &w->p, n);
    rc |= dev_alloc(h, &w->q, n);
    rc |= dev_alloc(h, &w->dinv, n);
    rc |= dev_alloc(h, &w->res, n);
    rc |= dev_alloc(h, &w->r32, n);
    rc |= dev_alloc(h, &w->z32, n);
    rc |= dev_alloc(h, &w->p32, n);
    rc |= dev_alloc(h, &w->q32, n);
    rc |= dev_alloc(h, &w->dinv32, n);
    rc |= dev_alloc(h, &w->d32, n);
    rc |= dev_alloc(h, &w->part, 4 * kMaxBlocks);
    rc |= dev_alloc(h, &w->scal, 16);
    rc |= dev_alloc(h, &w->sc, 1);
    h->solve_ws = w;
    if (rc) return rc;
    *out = w;
    return ANIGPU_OK;
}

// lanes per CSR row of the SpMV kernels (2, 4 or 8)
int row_width(anigpu_ctx* h) {
#ifdef SOLVE_W_FORCE
    (void)h;
    return SOLVE_W_FORCE;
#else
    const double avg = h->ndof ? (double)h->nnz / (double)h->ndof : 1.0;
    return avg > 48 ? 8 : (avg > 12 ? SOLVE_W_P2 : 2);
#endif
}

int nblocks_for(anigpu_ctx* h, int64_t work_items) {
    int sms = 148;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
    int64_t nb = (work_items + kBlock - 1) / kBlock;
    nb = std::min<int64_t>(nb, (int64_t)sms * 8);
    nb = std::min<int64_t>(nb, kMaxBlocks);
    return (int)std::max<int64_t>(nb, 1);
}

// one PCG solve; VR = matrix values, T = vector type, X = solution type
template <typename VR, typename T, typename X, int W>
int pcg_core(anigpu_ctx* h, SolveWs* w, const VR* vals, const double* b, X* x, T* r, T* z, T* p, T* q, T* dinv,
             double rtol, int64_t maxit, bool x_zero, double bb_ext, int64_t* iters, int* done_out) {
    const int64_t n = h->ndof;
    cudaStream_t s = h->stream;
    const int nb_rows = nblocks_for(h, n * W);
    const int nb3 = nblocks_for(h, h->nds * SPMV3_W);
    const int nb_pq = h->ncomp == 3 ? nb3 : nb_rows;
    const int nb_vec = nblocks_for(h, n);
    double* part_pq = w->part;
    double* part_rz = w->part + kMaxBlocks;
    double* part_rr = w->part + 2 * kMaxBlocks;
    double* part_bb = w->part + 3 * kMaxBlocks;
    // initial residual: x is f64 for the outer solve; for the inner IR solve x (f32 d) is zero
    init_kernel<VR, T, W><<<nb_rows, kBlock, 0, s>>>(n, h->rowptr, h->col, vals, (const double*)(x_zero ? nullptr : (const void*)x),
                                                     b, r, z, p, dinv, part_rz, part_rr, part_bb, x_zero ? 1 : 0);
    ANI_LAUNCHED(h);
    init_scalars_kernel<<<1, kBlock, 0, s>>>(w->sc, part_rz, part_rr, part_bb, nb_rows, rtol, (long long)maxit,
                                             bb_ext < 0 ? 1 : 0, bb_ext);
    ANI_LAUNCHED(h);
    // batches of iterations, replayed from a CUDA graph when the stream can be captured
    const int kBatch = 16;  // even: parities alternate 0,1,...
    cudaGraphExec_t exec = nullptr;
    {
        cudaGraph_t graph = nullptr;
        if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
            for (int it = 0; it < kBatch; ++it) {
                const int par = it & 1;
                launch_spmv_dot<VR, T, W>(h, nb_rows, nb3, vals, p, q, part_pq, w->sc);
                alpha_kernel<<<1, kBlock, 0, s>>>(par, part_pq, nb_pq, w->sc);
                update_kernel<T, X><<<nb_vec, kBlock, 0, s>>>(n, x, r, z, p, q, dinv, part_rz, part_rr, w->sc);
                beta_kernel<<<1, kBlock, 0, s>>>(par, part_rz, part_rr, nb_vec, w->sc);
                pupdate_kernel<T><<<nb_vec, kBlock, 0, s>>>(n, p, z, w->sc);
            }
            if (cudaStreamEndCapture(s, &graph) == cudaSuccess && graph) {
                if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) exec = nullptr;
                cudaGraphDestroy(graph);
            }
        }
        cudaGetLastError();
    }
    PcgScalars hs;
    int64_t launched = 0;
    while (true) {
        if (exec) {
            ANI_CUDA(h, cudaGraphLaunch(exec, s));
            h->launches += 5 * kBatch;
        } else {
            for (int it = 0; it < kBatch; ++it) {
                const int par = it & 1;
                launch_spmv_dot<VR, T, W>(h, nb_rows, nb3, vals, p, q, part_pq, w->sc);
                alpha_kernel<<<1, kBlock, 0, s>>>(par, part_pq, nb_pq, w->sc);
                update_kernel<T, X><<<nb_vec, kBlock, 0, s>>>(n, x, r, z, p, q, dinv, part_rz, part_rr, w->sc);
                beta_kernel<<<1, kBlock, 0, s>>>(par, part_rz, part_rr, nb_vec, w->sc);
                pupdate_kernel<T><<<nb_vec, kBlock, 0, s>>>(n, p, z, w->sc);
                h->launches += 5;
            }
            ANI_CUDA(h, cudaGetLastError());
        }
        launched += kBatch;
        ANI_CUDA(h, cudaMemcpyAsync(&hs, w->sc, sizeof(PcgScalars), cudaMemcpyDeviceToHost, s));
        ANI_CUDA(h, cudaStreamSynchronize(s));
        if (hs.done || launched >= maxit + kBatch) break;
    }
    if (exec) cudaGraphExecDestroy(exec);
    *iters = hs.iter;
    *done_out = hs.done;
    return ANIGPU_OK;
}

template <typename VR, int W>
int true_residual(anigpu_ctx* h, SolveWs* w, const VR* vals, const double* x, const double* b, double* rr) {
    const int64_t n = h->ndof;
    const int nb = nblocks_for(h, n * W);
    residual_kernel<VR, W><<<nb, kBlock, 0, h->stream>>>(n, h->rowptr, h->col, vals, x, b, w->res, w->part);
    ANI_LAUNCHED(h);
    sum_kernel<<<1, kBlock, 0, h->stream>>>(w->part, nb, w->scal);
    ANI_LAUNCHED(h);
    ANI_CUDA(h, cudaMemcpyAsync(rr, w->scal, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    ANI_CUDA(h, cudaStreamSynchronize(h->stream));
    return ANIGPU_OK;
}

template <typename VR, int W>
int solve_jacobi_pcg(anigpu_ctx* h, SolveWs* w, const VR* vals, const double* b, double* x, double rtol,
                     int64_t maxit, anigpu_solve_stats* st) {
    const int64_t n = h->ndof;
    diag_inv_kernel<VR, double><<<grid_for(n, 256), 256, 0, h->stream>>>(n, h->rowptr, h->col, vals, w->dinv);
    ANI_LAUNCHED(h);
    double bb = 0;
    int64_t total = 0, outer = 0;
    double rel = 0;
    int done = 0;
    // restart from the true residual when the recursive residual drifted
    for (outer = 0; outer < 8; ++outer) {
        int64_t it = 0;
        int rc = pcg_core<VR, double, double, W>(h, w, vals, b, x, w->r, w->z, w->p, w->q, w->dinv, rtol,
                                                  maxit - total, false, -1.0, &it, &done);
        if (rc) return rc;
        total += it;
        PcgScalars hs;
        ANI_CUDA(h, cudaMemcpy(&hs, w->sc, sizeof(PcgScalars), cudaMemcpyDeviceToHost));
        bb = hs.bb;
        double rr;
        rc = true_residual<VR, W>(h, w, vals, x, b, &rr);
        if (rc) return rc;
        rel = bb > 0 ? std::sqrt(rr / bb) : std::sqrt(rr);
        if (rel <= rtol || done == 2 || total >= maxit) break;
    }
    st->iterations = total;
    st->outer_iterations = outer + 1;
    st->rel_residual = rel;
    return rel <= rtol ? ANIGPU_OK : set_err(h, ANIGPU_ERR_NOT_CONVERGED, "Jacobi-PCG did not reach the tolerance");
}

__global__ void cast_f64_f32_kernel(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) b[i] = (float)a[i];
}

// FP32-SpMV CG inside FP64 iterative refinement
// (inner32: the FP32 system of the inner solves when it is not the outer system's rounding, e.g. an
// FP32-assembled matrix under an FP64-assembled outer system)
template <typename VR, int W>
int solve_ir_cg32(anigpu_ctx* h, SolveWs* w, const VR* vals_in, const double* b, double* x, double rtol,
                  int64_t maxit, anigpu_solve_stats* st, const float* inner32 = nullptr) {
    const int64_t n = h->ndof;
    const float* vals32;
    if (inner32) {
        vals32 = inner32;
    } else if (sizeof(VR) == 4) {
        vals32 = (const float*)vals_in;
    } else {
        int rc = dev_alloc(h, &w->vals32, (size_t)h->nnz);
        if (rc) return rc;
        cast_f64_f32_kernel<<<grid_for(h->nnz, 256), 256, 0, h->stream>>>(h->nnz, (const double*)vals_in, w->vals32);
        ANI_LAUNCHED(h);
        vals32 = w->vals32;
    }
    diag_inv_kernel<float, float><<<grid_for(n, 256), 256, 0, h->stream>>>(n, h->rowptr, h->col, vals32, w->dinv32);
    ANI_LAUNCHED(h);
    // ||b||^2
    double bb = 0;
    {
        ANI_CUDA(h, cudaMemsetAsync(w->res, 0, sizeof(double) * n, h->stream));
        int nb = nblocks_for(h, n * W);
        residual_kernel<VR, W><<<nb, kBlock, 0, h->stream>>>(n, h->rowptr, h->col, vals_in, w->res, b, w->q,
                                                              w->part);
        ANI_LAUNCHED(h);
        sum_kernel<<<1, kBlock, 0, h->stream>>>(w->part, nb, w->scal);
        ANI_LAUNCHED(h);
        ANI_CUDA(h, cudaMemcpyAsync(&bb, w->scal, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        ANI_CUDA(h, cudaStreamSynchronize(h->stream));
    }
    const double inner_tol = 1e-4;
    int64_t total = 0, outer = 0;
    double rel = 1;
    for (outer = 0; outer < 64; ++outer) {
        double rr;
        int rc = true_residual<VR, W>(h, w, vals_in, x, b, &rr);  // w->res = b - A x (f64)
        if (rc) return rc;
        rel = bb > 0 ? std::sqrt(rr / bb) : std::sqrt(rr);
        if (rel <= rtol || total >= maxit) break;
        // inner: A d = res in f32, relative to ||res||
        ANI_CUDA(h, cudaMemsetAsync(w->d32, 0, sizeof(float) * n, h->stream));
        int64_t it = 0;
        int done = 0;
        rc = pcg_core<float, float, float, W>(h, w, vals32, w->res, w->d32, w->r32, w->z32, w->p32, w->q32,
                                              w->dinv32, inner_tol, maxit - total, true, -1.0, &it, &done);
        if (rc) return rc;
        total += it;
        axpy_mixed_kernel<<<grid_for(n, 256), 256, 0, h->stream>>>(n, x, w->d32);
        ANI_LAUNCHED(h);
        if (it == 0) break;
    }
    st->iterations = total;
    st->outer_iterations = outer;
    st->rel_residual = rel;
    return rel <= rtol ? ANIGPU_OK : set_err(h, ANIGPU_ERR_NOT_CONVERGED, "IR-CG32 did not reach the tolerance");
}

}  // namespace

int run_spmv(anigpu_ctx* h, const void* vals, int precision, const double* x, double* y) {
    if (h->space < 0) return set_err(h, ANIGPU_ERR_STATE, "anigpu_problem_setup not called");
    const int64_t n = h->ndof;
    const int W = row_width(h);
    const unsigned g = grid_for(n * W, kBlock);
#define SPMV(VR, WW) spmv_kernel<VR, double, WW><<<g, kBlock, 0, h->stream>>>(n, h->rowptr, h->col, (const VR*)vals, x, y)
    if (precision == ANIGPU_F32) {
        if (W == 8) SPMV(float, 8);
        else if (W == 2) SPMV(float, 2);
        else SPMV(float, 4);
    } else {
        if (W == 8) SPMV(double, 8);
        else if (W == 2) SPMV(double, 2);
        else SPMV(double, 4);
    }
#undef SPMV
    ANI_LAUNCHED(h);
    return ANIGPU_OK;
}

int run_solve_refined(anigpu_ctx* h, int method, const float* vals32, const double* vals64, const double* b, double* x,
                      double rtol, int64_t maxit, anigpu_solve_stats* st) {
    if (h->space < 0) return set_err(h, ANIGPU_ERR_STATE, "anigpu_problem_setup not called");
    if (!vals32 || !vals64 || !b || !x || !st) return set_err(h, ANIGPU_ERR_ARG, "NULL argument");
    SolveWs* w;
    int rc = ensure_ws(h, &w);
    if (rc) return rc;
    *st = anigpu_solve_stats{0, 0, 0.0, 0.0, 0};
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, h->stream);
    const int W = row_width(h);
    switch (method) {
        case ANIGPU_SOLVE_IR_CG32:
            rc = W == 8   ? solve_ir_cg32<double, 8>(h, w, vals64, b, x, rtol, maxit, st, vals32)
                 : W == 2 ? solve_ir_cg32<double, 2>(h, w, vals64, b, x, rtol, maxit, st, vals32)
                          : solve_ir_cg32<double, 4>(h, w, vals64, b, x, rtol, maxit, st, vals32);
            break;
        case ANIGPU_SOLVE_FCG_LEARNED:
            rc = run_fcg_learned(h, vals32, ANIGPU_F32, b, x, rtol, maxit, st, vals64);
            break;
        default:
            rc = set_err(h, ANIGPU_ERR_ARG, "refined solves take IR_CG32 or FCG_LEARNED");
    }
    cudaEventRecord(e1, h->stream);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    st->seconds = ms * 1e-3;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

int run_solve(anigpu_ctx* h, int method, const void* vals, int precision, const double* b, double* x, double rtol,
              int64_t maxit, anigpu_solve_stats* st) {
    if (h->space < 0) return set_err(h, ANIGPU_ERR_STATE, "anigpu_problem_setup not called");
    if (!vals || !b || !x || !st) return set_err(h, ANIGPU_ERR_ARG, "NULL argument");
    if (precision != ANIGPU_F32 && precision != ANIGPU_F64) return set_err(h, ANIGPU_ERR_ARG, "precision");
    SolveWs* w;
    int rc = ensure_ws(h, &w);
    if (rc) return rc;
    *st = anigpu_solve_stats{0, 0, 0.0, 0.0, 0};
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, h->stream);
    const int W = row_width(h);
    switch (method) {
#define BY_W(FN, VR)                                                                              \
    (W == 8 ? FN<VR, 8>(h, w, (const VR*)vals, b, x, rtol, maxit, st)                             \
            : W == 2 ? FN<VR, 2>(h, w, (const VR*)vals, b, x, rtol, maxit, st)                    \
                     : FN<VR, 4>(h, w, (const VR*)vals, b, x, rtol, maxit, st))
        case ANIGPU_SOLVE_JACOBI_PCG:
            rc = precision == ANIGPU_F64 ? BY_W(solve_jacobi_pcg, double) : BY_W(solve_jacobi_pcg, float);
            break;
        case ANIGPU_SOLVE_IR_CG32:
            rc = precision == ANIGPU_F64 ? BY_W(solve_ir_cg32, double) : BY_W(solve_ir_cg32, float);
            break;
#undef BY_W
        case ANIGPU_SOLVE_FCG_LEARNED:
            rc = run_fcg_learned(h, vals, precision, b, x, rtol, maxit, st);
            break;
        default:
            rc = set_err(h, ANIGPU_ERR_ARG, "unknown solve method");
    }
    cudaEventRecord(e1, h->stream);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    st->seconds = ms * 1e-3;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

void free_solver(anigpu_ctx* h) {
    SolveWs* w = (SolveWs*)h->solve_ws;
    if (!w) return;
    void* ptrs[] = {w->r, w->z, w->p, w->q, w->dinv, w->res, w->r32, w->z32, w->p32, w->q32, w->dinv32, w->d32,
                    w->vals32, w->part, w->scal, w->sc};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    delete w;
    h->solve_ws = nullptr;
}
