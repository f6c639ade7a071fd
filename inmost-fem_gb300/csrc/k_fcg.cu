// Flexible CG with the learned preconditioner: FP32 vectors and FP32 SpMV, FP64 solution,
// FP64 residual replacement (a new component: the reference hands its matrix to INMOST's
// ILU-Krylov solver, examples/tutorials/ex1.cpp:161-163).
//
// Iteration k (FCG(1): one A-orthogonalisation against the previous direction; the scalars of
// a step are formed once by one-block kernels that the vector kernels read):
//     q = A p ;  alpha = r.z / p.q ;  d += alpha p ;  r -= alpha q
//     z = M r ;  beta = -(z.q) / (p.q) ;  p = z + beta p
// d is an FP32 correction that is folded into the FP64 solution x at every residual
// replacement: when ||r|| fell below kDelta times its value at the last replacement (or the
// recursive residual says "converged"), x += d, d = 0 and r = b - A x is recomputed in FP64
// arithmetic; p is kept, z and r.z are recomputed.  The FP32 recursion therefore never has to
// resolve more than kDelta of relative reduction, and the final accuracy is that of the FP64
// residual.  Stopping: ||b - A x|| <= rtol ||b|| with the FP64 residual.
//
// Fallback: Jacobi (z = D^-1 r).  The solve switches to it for the rest of the call when a step
// breaks down (r.z <= 0 or p.q <= 0, non-finite values) or when the residual stops decreasing
// (no new smallest residual over max(kStallBatches, half the batches run so far) batches: the
// residual norm of CG is not monotone and its plateaus grow with the condition number); the
// direction restarts from z.  Steps
// taken with the Jacobi direction are counted in fallback_steps.
//
// The scalars live on the device.  Iterations run in captured batches of kBatch; each kernel
// of iteration k reads the status word written by iteration k-1 (two words, by parity, so that
// no kernel reads a word that another block of the same launch writes) and returns at once
// when it is set.  Dot products are FP32 per thread and FP64 across threads, two-stage with a
// fixed order, so runs reproduce bit for bit.
#include <algorithm>
#include <cmath>
#include <vector>

#include "learned.h"
#include "spmv_vec3.cuh"

#define RC_(x)               \
    do {                     \
        int _r = (x);        \
        if (_r) return _r;   \
    } while (0)

namespace {

constexpr int kB = 256;
constexpr int kMaxP = 1024;          // block partials per reduction
constexpr int kBatch = 16;           // even: the status parity of a batch starts at 0
constexpr double kDelta = 0.1;       // residual replacement threshold (ratio of norms)
constexpr int kStallBatches = 32;    // batches without a new smallest residual -> Jacobi (at least)
#ifndef FCG_W
#define FCG_W 4
#endif
constexpr int kW = FCG_W;            // lanes per CSR row

struct FcgScalars {
    double rz;        // r.z of the current direction
    double pq;        // p.q of the current step
    double alpha, beta;
    int brk;          // p.q of the current step is not positive (or not finite): no update
    int pad;
    double rr;        // recursive ||r||^2 after the last step
    double rrep2;     // kDelta^2 * ||r||^2 at the last replacement
    double tol2;      // (rtol ||b||)^2
    long long iter;   // steps of this solve
    long long maxit;
    int st[2];        // status by iteration parity: 0 running, 1 converged, 2 breakdown, 3 replace, 4 maxit
};

__device__ inline double block_sum_d(double v, double* sh) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i];
    return s;  // thread 0
}

// fixed-order sum of nb partials, broadcast to the block
__device__ inline double sum_parts_d(const double* part, int nb, double* sh) {
    double v = 0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) v += part[i];
    const double s = block_sum_d(v, sh);
    __syncthreads();
    if (threadIdx.x == 0) sh[32] = s;
    __syncthreads();
    return sh[32];
}

// q = A p ; partials of p.q
__global__ void __launch_bounds__(kB) spmv_dot_kernel(int64_t n, const int64_t* __restrict__ rowptr,
                                                      const int32_t* __restrict__ col,
                                                      const float* __restrict__ vals, const float* __restrict__ p,
                                                      float* __restrict__ q, double* __restrict__ part,
                                                      const int* __restrict__ stop) {
    __shared__ double sh[33];
    if (*stop) return;
    const int64_t rows_per_block = kB / kW;
    const int lane = threadIdx.x & (kW - 1);
    float acc = 0.f;
    for (int64_t base = blockIdx.x * rows_per_block; base < n; base += (int64_t)gridDim.x * rows_per_block) {
        const int64_t row = base + threadIdx.x / kW;
        float s = 0.f;
        if (row < n) {
            const int64_t b = rowptr[row], e = rowptr[row + 1];
            for (int64_t k = b + lane; k < e; k += kW) s = fmaf(vals[k], p[col[k]], s);
        }
#pragma unroll
        for (int o = kW / 2; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, kW);
        if (row < n && lane == 0) {
            q[row] = s;
            acc = fmaf(s, p[row], acc);
        }
    }
    const double t = block_sum_d((double)acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// q = A p ; partials of p.q -- vector (3-component) template, SPMV3_W lanes per scalar row
__global__ void __launch_bounds__(kB, SPMV3_MINB_F32) spmv3_dot_kernel(int64_t nds, int64_t nnz_s, const int64_t* __restrict__ rowptr_s,
                                                       const int32_t* __restrict__ col_s,
                                                       const float* __restrict__ vals, const float* __restrict__ p,
                                                       float* __restrict__ q, double* __restrict__ part,
                                                       const int* __restrict__ stop) {
    __shared__ double sh[33];
    if (*stop) return;
    constexpr int W = SPMV3_W;
    const int64_t rows_per_block = kB / W;
    const int lane = threadIdx.x & (W - 1);
    float acc = 0.f;
    for (int64_t base = blockIdx.x * rows_per_block; base < nds; base += (int64_t)gridDim.x * rows_per_block) {
        const int64_t r = base + threadIdx.x / W;
        float s0, s1, s2;
        vec3_rows<W>(r, lane, nds, nnz_s, rowptr_s, col_s, vals, p, s0, s1, s2);
        if (r < nds && lane == 0) {
            q[r] = s0;
            q[nds + r] = s1;
            q[2 * nds + r] = s2;
            acc = fmaf(s0, p[r], acc);
            acc = fmaf(s1, p[nds + r], acc);
            acc = fmaf(s2, p[2 * nds + r], acc);
        }
    }
    const double t = block_sum_d((double)acc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// alpha = rz / pq, once (one block): the update kernels read it
__global__ void alpha_kernel(const double* __restrict__ part_pq, int nb_pq, FcgScalars* __restrict__ sc,
                             const int* __restrict__ stop) {
    __shared__ double sh[33];
    if (*stop) return;
    const double pq = sum_parts_d(part_pq, nb_pq, sh);
    if (threadIdx.x == 0) {
        const double al = sc->rz / pq;
        sc->pq = pq;
        sc->brk = (!(pq > 0) || !isfinite(al)) ? 1 : 0;
        sc->alpha = sc->brk ? 0.0 : al;
    }
}

// d += alpha p ; r -= alpha q ; partials of r.r
__global__ void __launch_bounds__(kB) update_kernel(int64_t n, float* __restrict__ d, float* __restrict__ r,
                                                    const float* __restrict__ p, const float* __restrict__ q,
                                                    double* __restrict__ part_rr, const FcgScalars* __restrict__ sc,
                                                    const int* __restrict__ stop) {
    __shared__ double sh[33];
    if (*stop) return;
    if (sc->brk) {  // breakdown: no update; the status check stops the batch
        if (threadIdx.x == 0) part_rr[blockIdx.x] = 0;
        return;
    }
    const float a = (float)sc->alpha;
    float arr = 0.f;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        d[i] = fmaf(a, p[i], d[i]);
        const float ri = fmaf(-a, q[i], r[i]);
        r[i] = ri;
        arr = fmaf(ri, ri, arr);
    }
    const double t = block_sum_d((double)arr, sh);
    if (threadIdx.x == 0) part_rr[blockIdx.x] = t;
}

// Jacobi direction: z = D^-1 r ; partials of r.z and z.qold
__global__ void __launch_bounds__(kB) jacobi_dot_kernel(int64_t n, const float* __restrict__ r,
                                                        const float* __restrict__ dinv,
                                                        const float* __restrict__ qold, float* __restrict__ z,
                                                        double* __restrict__ part_rz, double* __restrict__ part_zq,
                                                        const int* __restrict__ stop) {
    __shared__ double sh[33];
    if (stop && *stop) return;
    float arz = 0.f, azq = 0.f;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float zi = dinv[i] * r[i];
        z[i] = zi;
        arz = fmaf(r[i], zi, arz);
        if (qold) azq = fmaf(zi, qold[i], azq);
    }
    double t = block_sum_d((double)arz, sh);
    if (threadIdx.x == 0) part_rz[blockIdx.x] = t;
    __syncthreads();
    t = block_sum_d((double)azq, sh);
    if (threadIdx.x == 0) part_zq[blockIdx.x] = t;
}

// beta = -(z.q)/(p.q) and the status of this step, once (one block)
__global__ void beta_kernel(const double* __restrict__ part_rz, const double* __restrict__ part_zq, int nb_prec,
                            const double* __restrict__ part_rr, int nb_vec, FcgScalars* __restrict__ sc, int par) {
    __shared__ double sh[33];
    const int prev = sc->st[par ^ 1];
    if (prev) {
        if (threadIdx.x == 0) sc->st[par] = prev;  // carry the stop through the batch
        return;
    }
    const double rz = sum_parts_d(part_rz, nb_prec, sh);
    const double zq = sum_parts_d(part_zq, nb_prec, sh);
    const double rr = sum_parts_d(part_rr, nb_vec, sh);
    if (threadIdx.x == 0) {
        const double pq = sc->pq;
        sc->beta = pq > 0 ? -zq / pq : 0.0;
        if (sc->brk || !(rz > 0) || !isfinite(rz) || !isfinite(rr) || !isfinite(zq)) {
            sc->st[par] = 2;  // breakdown: the step is not counted and the scalars stay
            return;
        }
        sc->rz = rz;
        sc->rr = rr;
        sc->iter += 1;
        int st = 0;
        if (rr <= sc->tol2) st = 1;
        else if (rr <= sc->rrep2) st = 3;
        else if (sc->iter >= sc->maxit) st = 4;
        sc->st[par] = st;
    }
}

// p = z + beta p (skipped when the previous step stopped the batch)
__global__ void __launch_bounds__(kB) pupdate_kernel(int64_t n, float* __restrict__ p, const float* __restrict__ z,
                                                     const FcgScalars* __restrict__ sc, int par) {
    if (sc->st[par ^ 1]) return;
    const float beta = (float)sc->beta;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = fmaf(beta, p[i], z[i]);
}

// x += d ; d = 0
__global__ void fold_kernel(int64_t n, double* __restrict__ x, float* __restrict__ d) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    x[i] += (double)d[i];
    d[i] = 0.f;
}

// r = b - A x in FP64 arithmetic (r stored FP32); partials of r.r (and b.b when part_bb); A is the
// FP32 system the iteration runs on, or the FP64-assembled system that judges convergence
template <typename VT>
__global__ void __launch_bounds__(kB) resid_kernel(int64_t n, const int64_t* __restrict__ rowptr,
                                                   const int32_t* __restrict__ col, const VT* __restrict__ vals,
                                                   const double* __restrict__ x, const double* __restrict__ b,
                                                   float* __restrict__ r, double* __restrict__ part_rr,
                                                   double* __restrict__ part_bb) {
    __shared__ double sh[33];
    const int64_t rows_per_block = kB / kW;
    const int lane = threadIdx.x & (kW - 1);
    double arr = 0, abb = 0;
    for (int64_t base = blockIdx.x * rows_per_block; base < n; base += (int64_t)gridDim.x * rows_per_block) {
        const int64_t row = base + threadIdx.x / kW;
        double s = 0;
        if (row < n) {
            const int64_t bb = rowptr[row], e = rowptr[row + 1];
            for (int64_t k = bb + lane; k < e; k += kW) s += (double)vals[k] * x[col[k]];
        }
#pragma unroll
        for (int o = kW / 2; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, kW);
        if (row < n && lane == 0) {
            const double ri = b[row] - s;
            r[row] = (float)ri;
            arr += ri * ri;
            abb += b[row] * b[row];
        }
    }
    double t = block_sum_d(arr, sh);
    if (threadIdx.x == 0) part_rr[blockIdx.x] = t;
    if (part_bb) {
        __syncthreads();
        t = block_sum_d(abb, sh);
        if (threadIdx.x == 0) part_bb[blockIdx.x] = t;
    }
}

// out[k] = fixed-order sum of the nb partials of part + k * kMaxP
__global__ void sums_kernel(const double* __restrict__ part, int nb, int m, double* __restrict__ out) {
    __shared__ double sh[33];
    for (int k = 0; k < m; ++k) {
        const double s = sum_parts_d(part + (size_t)k * kMaxP, nb, sh);
        if (threadIdx.x == 0) out[k] = s;
        __syncthreads();
    }
}

// after a replacement: r.z of the new z, ||r||^2, thresholds, status cleared
__global__ void restart_scalars_kernel(FcgScalars* __restrict__ sc, const double* __restrict__ part_rz, int nb_vec,
                                       double rr, double tol2, long long maxit, int first) {
    __shared__ double sh[33];
    const double rz = sum_parts_d(part_rz, nb_vec, sh);
    if (threadIdx.x == 0) {
        sc->rz = rz;
        sc->rr = rr;
        sc->rrep2 = kDelta * kDelta * rr;
        sc->tol2 = tol2;
        sc->maxit = maxit;
        sc->brk = 0;
        if (first) sc->iter = 0;
        sc->st[0] = 0;
        sc->st[1] = 0;
    }
}

__global__ void dinv_kernel(int64_t n, const float* __restrict__ diag, float* __restrict__ dinv) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) dinv[i] = diag[i] != 0.f ? 1.f / diag[i] : 1.f;
}

struct FcgWs {
    int64_t n = 0;
    float *r = nullptr, *d = nullptr, *z = nullptr, *p = nullptr, *q = nullptr, *dinv = nullptr;
    double* part = nullptr;  // [5][kMaxP]: pq, rr, bb, rz, zq
    double* sums = nullptr;  // [2]
    FcgScalars* sc = nullptr;
    // captured batches, valid for (vals, bind generation)
    cudaGraphExec_t exec[2] = {nullptr, nullptr};  // 0 learned, 1 Jacobi
    int64_t per_batch[2] = {0, 0};
    const void* key_vals = nullptr;
    int64_t key_gen = -1;
};

void drop_graphs(FcgWs* w) {
    for (auto& e : w->exec)
        if (e) {
            cudaGraphExecDestroy(e);
            e = nullptr;
        }
}

int ensure_ws(anigpu_ctx* h, FcgWs** out) {
    FcgWs* w = static_cast<FcgWs*>(h->fcg_ws);
    if (w && w->n == h->ndof) {
        *out = w;
        return ANIGPU_OK;
    }
    free_fcg(h);
    w = new FcgWs();
    h->fcg_ws = w;
    w->n = h->ndof;
    const size_t n = (size_t)h->ndof;
    int rc = 0;
    rc |= dev_alloc(h, &w->r, n);
    rc |= dev_alloc(h, &w->d, n);
    rc |= dev_alloc(h, &w->z, n);
    rc |= dev_alloc(h, &w->p, n);
    rc |= dev_alloc(h, &w->q, n);
    rc |= dev_alloc(h, &w->dinv, n);
    rc |= dev_alloc(h, &w->part, 5 * kMaxP);
    rc |= dev_alloc(h, &w->sums, 2);
    rc |= dev_alloc(h, &w->sc, 1);
    if (rc) return rc;
    *out = w;
    return ANIGPU_OK;
}

int nblocks(int64_t work) { return (int)std::min<int64_t>(kMaxP, std::max<int64_t>(1, (work + kB - 1) / kB)); }

struct Ctx {
    anigpu_ctx* h;
    FcgWs* w;
    const float* vals;
    const double* b;
    double* x;
    int64_t n;
    const double* vals64;  // FP64 system of the residual replacements (null: the FP32 one)
    int nb_rows, nb_vec, nb_prec;  // nb_prec: blocks (partials) of the preconditioner's r.z, z.q
    int nb_pq;                     // blocks (partials) of the SpMV's p.q
    double *part_pq, *part_rr, *part_bb, *part_rz, *part_zq;
};

// z = M r (mode 0) or D^-1 r (mode 1); partials of r.z (and z.qold)
int precond(Ctx& c, int mode, const float* qold, const int* stop) {
    if (mode == 0) return gnn_precond_f32(c.h, c.w->r, c.w->z, qold, c.part_rz, c.part_zq, c.nb_prec, stop);
    jacobi_dot_kernel<<<c.nb_prec, kB, 0, c.h->stream>>>(c.n, c.w->r, c.w->dinv, qold, c.w->z, c.part_rz, c.part_zq,
                                                         stop);
    ANI_LAUNCHED(c.h);
    return ANIGPU_OK;
}

int one_iteration(Ctx& c, int mode, int par) {
    anigpu_ctx* h = c.h;
    FcgWs* w = c.w;
    cudaStream_t s = h->stream;
    const int* stop = &w->sc->st[par ^ 1];
    if (h->ncomp == 3)
        spmv3_dot_kernel<<<c.nb_pq, kB, 0, s>>>(h->nds, h->nnz_s, h->rowptr_s, h->col_s, c.vals, w->p, w->q, c.part_pq,
                                                stop);
    else
        spmv_dot_kernel<<<c.nb_pq, kB, 0, s>>>(c.n, h->rowptr, h->col, c.vals, w->p, w->q, c.part_pq, stop);
    ANI_LAUNCHED(h);
    alpha_kernel<<<1, kB, 0, s>>>(c.part_pq, c.nb_pq, w->sc, stop);
    ANI_LAUNCHED(h);
    update_kernel<<<c.nb_vec, kB, 0, s>>>(c.n, w->d, w->r, w->p, w->q, c.part_rr, w->sc, stop);
    ANI_LAUNCHED(h);
    RC_(precond(c, mode, w->q, stop));
    beta_kernel<<<1, kB, 0, s>>>(c.part_rz, c.part_zq, c.nb_prec, c.part_rr, c.nb_vec, w->sc, par);
    ANI_LAUNCHED(h);
    pupdate_kernel<<<c.nb_vec, kB, 0, s>>>(c.n, w->p, w->z, w->sc, par);
    ANI_LAUNCHED(h);
    return ANIGPU_OK;
}

// kBatch iterations of one mode from a captured graph (captured on first use); uncaptured when
// the stream cannot be captured
int batch(Ctx& c, int mode) {
    anigpu_ctx* h = c.h;
    FcgWs* w = c.w;
    cudaStream_t s = h->stream;
    if (!w->exec[mode]) {
        const int64_t l0 = h->launches;
        cudaGraph_t graph = nullptr;
        if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
            int rc = 0;
            for (int it = 0; it < kBatch && !rc; ++it) rc = one_iteration(c, mode, it & 1);
            const cudaError_t e = cudaStreamEndCapture(s, &graph);
            if (!rc && e == cudaSuccess && graph) {
                if (cudaGraphInstantiate(&w->exec[mode], graph, 0) != cudaSuccess) w->exec[mode] = nullptr;
            }
            if (graph) cudaGraphDestroy(graph);
        }
        cudaGetLastError();
        w->per_batch[mode] = h->launches - l0;
        h->launches = l0;
    }
    if (w->exec[mode]) {
        ANI_CUDA(h, cudaGraphLaunch(w->exec[mode], s));
        h->launches += w->per_batch[mode];
        return ANIGPU_OK;
    }
    for (int it = 0; it < kBatch; ++it) RC_(one_iteration(c, mode, it & 1));
    return ANIGPU_OK;
}

// x += d, d = 0, r = b - A x (FP64 arithmetic); returns ||r||^2 (and ||b||^2 when asked)
int checkpoint(Ctx& c, double* rr, double* bb) {
    anigpu_ctx* h = c.h;
    cudaStream_t s = h->stream;
    fold_kernel<<<grid_for(c.n, kB), kB, 0, s>>>(c.n, c.x, c.w->d);
    ANI_LAUNCHED(h);
    if (c.vals64)
        resid_kernel<double><<<c.nb_rows, kB, 0, s>>>(c.n, h->rowptr, h->col, c.vals64, c.x, c.b, c.w->r, c.part_rr,
                                                      bb ? c.part_bb : nullptr);
    else
        resid_kernel<float><<<c.nb_rows, kB, 0, s>>>(c.n, h->rowptr, h->col, c.vals, c.x, c.b, c.w->r, c.part_rr,
                                                     bb ? c.part_bb : nullptr);
    ANI_LAUNCHED(h);
    sums_kernel<<<1, kB, 0, s>>>(c.part_rr, c.nb_rows, bb ? 2 : 1, c.w->sums);  // part_bb = part_rr + kMaxP
    ANI_LAUNCHED(h);
    double hs[2] = {0, 0};
    ANI_CUDA(h, cudaMemcpyAsync(hs, c.w->sums, sizeof(double) * 2, cudaMemcpyDeviceToHost, s));
    ANI_CUDA(h, cudaStreamSynchronize(s));
    *rr = hs[0];
    if (bb) *bb = hs[1];
    return ANIGPU_OK;
}

// new direction data after a checkpoint: z, r.z, thresholds; p = z when reset_p
int restart(Ctx& c, int mode, bool reset_p, double rr, double tol2, int64_t maxit, bool first) {
    anigpu_ctx* h = c.h;
    cudaStream_t s = h->stream;
    RC_(precond(c, mode, nullptr, nullptr));
    if (reset_p) ANI_CUDA(h, cudaMemcpyAsync(c.w->p, c.w->z, sizeof(float) * c.n, cudaMemcpyDeviceToDevice, s));
    restart_scalars_kernel<<<1, kB, 0, s>>>(c.w->sc, c.part_rz, c.nb_prec, rr, tol2, (long long)maxit, first ? 1 : 0);
    ANI_LAUNCHED(h);
    return ANIGPU_OK;
}

}  // namespace

void free_fcg(anigpu_ctx* h) {
    FcgWs* w = static_cast<FcgWs*>(h->fcg_ws);
    if (!w) return;
    drop_graphs(w);
    void* ptrs[] = {w->r, w->d, w->z, w->p, w->q, w->dinv, w->part, w->sums, w->sc};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete w;
    h->fcg_ws = nullptr;
}

int run_fcg_learned(anigpu_ctx* h, const void* vals, int precision, const double* b, double* x, double rtol,
                    int64_t maxit, anigpu_solve_stats* st, const double* vals64) {
    if (precision != ANIGPU_F32) return set_err(h, ANIGPU_ERR_UNSUPPORTED, "FCG_LEARNED takes FP32 values");
    if (!gnn_bound_to(h, vals)) return set_err(h, ANIGPU_ERR_STATE, "anigpu_gnn_bind not called for these values");
    FcgWs* w;
    RC_(ensure_ws(h, &w));
    if (w->key_vals != vals || w->key_gen != gnn_bind_generation(h)) {
        drop_graphs(w);
        w->key_vals = vals;
        w->key_gen = gnn_bind_generation(h);
    }
    Ctx c{h, w, (const float*)vals, b, x, h->ndof, vals64, 0, 0, 0, 0, nullptr, nullptr, nullptr, nullptr, nullptr};
    c.nb_rows = nblocks(c.n * kW);
    c.nb_pq = h->ncomp == 3 ? nblocks(h->nds * SPMV3_W) : c.nb_rows;
    c.nb_vec = nblocks(c.n);
    c.nb_prec = c.nb_vec;
    c.part_pq = w->part;
    c.part_rr = w->part + kMaxP;
    c.part_bb = w->part + 2 * kMaxP;  // follows part_rr: checkpoint sums both with one kernel
    c.part_rz = w->part + 3 * kMaxP;
    c.part_zq = w->part + 4 * kMaxP;
    cudaStream_t s = h->stream;
    dinv_kernel<<<grid_for(c.n, kB), kB, 0, s>>>(c.n, gnn_fine_diag(h), w->dinv);
    ANI_LAUNCHED(h);
    ANI_CUDA(h, cudaMemsetAsync(w->d, 0, sizeof(float) * c.n, s));
    double rr = 0, bb = 0;
    RC_(checkpoint(c, &rr, &bb));
    const double tol2 = rtol * rtol * (bb > 0 ? bb : 1.0);
    double rel = bb > 0 ? std::sqrt(rr / bb) : std::sqrt(rr);
    int mode = 0;
    int64_t fallback = 0, replacements = 0;
    FcgScalars hs{};
    if (rel > rtol && maxit > 0) {
        RC_(restart(c, mode, true, rr, tol2, maxit, true));
        double best = rr;
        int64_t stall = 0, nbatch = 0;
        int64_t last_iter = 0;
        while (true) {
            RC_(batch(c, mode));
            ++nbatch;
            ANI_CUDA(h, cudaMemcpyAsync(&hs, w->sc, sizeof(FcgScalars), cudaMemcpyDeviceToHost, s));
            ANI_CUDA(h, cudaStreamSynchronize(s));
            if (mode == 1) fallback += hs.iter - last_iter;
            last_iter = hs.iter;
            const int status = hs.st[1];
            bool to_jacobi = false;
            if (hs.rr < best) {
                best = hs.rr;
                stall = 0;
            } else if (++stall >= std::max<int64_t>(kStallBatches, nbatch / 2) && mode == 0) {
                to_jacobi = true;
            }
            if (status == 2 && mode == 0) to_jacobi = true;
            if (status == 0 && !to_jacobi) continue;
            RC_(checkpoint(c, &rr, nullptr));
            ++replacements;
            rel = bb > 0 ? std::sqrt(rr / bb) : std::sqrt(rr);
            if (rel <= rtol || hs.iter >= maxit) break;
            if (status == 2 && mode == 1) break;  // breakdown of the Jacobi fallback itself
            if (to_jacobi) {
                mode = 1;
                stall = 0;
                best = rr;
            }
            RC_(restart(c, mode, to_jacobi, rr, tol2, maxit, false));
        }
    }
    st->iterations = hs.iter;
    st->outer_iterations = replacements;
    st->rel_residual = rel;
    st->fallback_steps = fallback;
    return rel <= rtol ? ANIGPU_OK : set_err(h, ANIGPU_ERR_NOT_CONVERGED, "FCG did not reach the tolerance");
}
