// Batched uneven instances: many independent meshes assembled and solved as one problem (a new
// component; the reference assembles and solves one mesh at a time, examples/tutorials/ex1.cpp:
// 120-163).  The caller uploads the disjoint union of the meshes (vertex and tet ids offset per
// instance): the CSR template, the NATURAL numbering and the assembly kernels then cover every
// instance in one pass, and the matrix is block diagonal.  This file adds
//
//   * the instance map: the instance of every DOF (from the tet ranges of the instances) and row
//     tiles of at most kTileRows consecutive DOFs of one instance, so that every reduction of the
//     solver is a per-tile partial followed by a fixed-order per-instance sum (deterministic).
//     One warp works on one tile (a fixed shuffle tree for its partials, no block barrier), eight
//     tiles in flight per 256-thread block;
//   * Jacobi-PCG with per-instance scalars and convergence: five kernels per iteration (q = A p
//     with per-tile p.q; per-instance alpha; x, r, z update with per-tile r.z, r.r; per-instance
//     beta and convergence; p update).  Tiles of converged instances return at once, so the cost
//     of an iteration shrinks as instances converge;
//   * one CUDA graph for the whole job: the assembly and the solver initialisation, then a
//     device-side while loop (conditional graph node) whose body is kBatchIters iterations and a
//     check kernel that continues while any instance runs and fewer than maxit iterations were
//     taken.  One graph launch assembles and solves every instance;
//   * an autotuner: the lanes per CSR row of the SpMV (2, 4, 8, 16) are timed on the actual
//     matrix when the instances are set, and the fastest is used.
#include <algorithm>
#include <cmath>
#include <vector>

#include "anigpu_internal.h"

int run_assemble(anigpu_ctx* h, int kind, const double* D, const double* f, double f_const, int order,
                 int precision, void* vals, double* rhs, uint8_t* touched, double drop_val);

namespace {

constexpr int kTileRows = 64;
constexpr int kBatchIters = 16;

#define RC_(x)               \
    do {                     \
        int _r = (x);        \
        if (_r) return _r;   \
    } while (0)

struct InstScalars {
    double rz, rr, bb, tol2, alpha, beta;
    long long iters;
    int done;  // 0 running, 1 converged, 2 stopped (maxit or breakdown)
    int pad;
};

struct BatchCtl {
    long long iters;      // iterations taken by the batch (all instances advance together)
    long long maxit;
    int remaining;        // instances still running after the last check
    int pad;
};

__device__ inline double bsum(double v, double* sh) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i];
    __syncthreads();
    return s;  // thread 0
}

// one warp per tile: every reduction of a tile is a fixed shuffle tree, no block barrier
constexpr int kWarps = 8;  // warps (tiles in flight) per 256-thread block

__device__ inline double wsum(double v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ---------------------------------------------------------------- instance map
__global__ void dof_inst_kernel(int64_t nt, int nloc, const int32_t* __restrict__ edofs,
                                const int64_t* __restrict__ toff, int ninst, int32_t* __restrict__ inst,
                                int* __restrict__ status) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nt) return;
    int lo = 0, hi = ninst;  // toff[lo] <= t < toff[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (toff[mid] <= t) lo = mid;
        else hi = mid;
    }
    for (int j = 0; j < nloc; ++j) {
        const int32_t d = edofs[t * nloc + j];
        const int32_t prev = atomicExch(&inst[d], lo);
        if (prev != -1 && prev != lo) atomicExch(status, ANIGPU_ERR_ARG);  // meshes share a DOF
    }
}

// a tile starts where the instance changes and at every multiple of kTileRows
__global__ void tile_flag_kernel(int64_t n, const int32_t* __restrict__ inst, unsigned long long* __restrict__ flag) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= n) return;
    flag[p] = (p % kTileRows == 0 || inst[p] != inst[p - 1]) ? 1 : 0;
}

__global__ void tile_fill_kernel(int64_t n, const unsigned long long* __restrict__ flag,
                                 const int64_t* __restrict__ pos, const int32_t* __restrict__ inst,
                                 int64_t* __restrict__ tstart, int32_t* __restrict__ tinst) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= n || !flag[p]) return;
    const int64_t t = pos[p];
    tstart[t] = p;
    tinst[t] = inst[p];
}

// ---------------------------------------------------------------- solver kernels
__global__ void bdiag_kernel(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                             const double* __restrict__ vals, double* __restrict__ dinv) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= n) return;
    double d = 0;
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k)
        if (col[k] == r) {
            d = vals[k];
            break;
        }
    dinv[r] = d != 0 ? 1.0 / d : 1.0;
}

// x = 0, r = b, z = dinv r, p = z; partials r.z and b.b per tile (one warp per tile)
__global__ void __launch_bounds__(256) binit_kernel(int ntiles, const int64_t* __restrict__ tstart,
                                                    const double* __restrict__ b, const double* __restrict__ dinv,
                                                    double* __restrict__ x, double* __restrict__ r,
                                                    double* __restrict__ z, double* __restrict__ p,
                                                    double* __restrict__ part_rz, double* __restrict__ part_rr) {
    const int lane = threadIdx.x & 31;
    for (int t = blockIdx.x * kWarps + (threadIdx.x >> 5); t < ntiles; t += gridDim.x * kWarps) {
        const int64_t t0 = tstart[t], t1 = tstart[t + 1];
        double arz = 0, arr = 0;
        for (int64_t i = t0 + lane; i < t1; i += 32) {
            const double ri = b[i], zi = dinv[i] * ri;
            x[i] = 0;
            r[i] = ri;
            z[i] = zi;
            p[i] = zi;
            arz += ri * zi;
            arr += ri * ri;
        }
        arz = wsum(arz);
        arr = wsum(arr);
        if (lane == 0) {
            part_rz[t] = arz;
            part_rr[t] = arr;
        }
    }
}

// fixed-order sum over the tiles of instance i (inst_tiles sorted ascending)
__device__ inline double inst_reduce(const double* part, const int32_t* itp, const int32_t* it, int i, double* sh) {
    double v = 0;
    for (int k = itp[i] + threadIdx.x; k < itp[i + 1]; k += blockDim.x) v += part[it[k]];
    return bsum(v, sh);
}

__global__ void binst_init_kernel(int ninst, const int32_t* __restrict__ itp, const int32_t* __restrict__ it,
                                  const double* __restrict__ part_rz, const double* __restrict__ part_rr, double rtol,
                                  InstScalars* __restrict__ sc) {
    __shared__ double sh[32];
    const int i = blockIdx.x;
    const double rz = inst_reduce(part_rz, itp, it, i, sh);
    const double bb = inst_reduce(part_rr, itp, it, i, sh);
    if (threadIdx.x == 0) {
        InstScalars s{};
        s.rz = rz;
        s.rr = bb;
        s.bb = bb;
        s.tol2 = rtol * rtol * bb;
        s.iters = 0;
        s.done = (bb <= s.tol2) ? 1 : 0;
        sc[i] = s;
    }
}

// q = A p per tile, partial p.q (one warp per tile: 32/W rows per pass, W lanes per row)
template <int W>
__global__ void __launch_bounds__(256) bspmv_dot_kernel(int ntiles, const int64_t* __restrict__ tstart,
                                                        const int32_t* __restrict__ tinst,
                                                        const int64_t* __restrict__ rowptr,
                                                        const int32_t* __restrict__ col,
                                                        const double* __restrict__ vals, const double* __restrict__ p,
                                                        double* __restrict__ q, const InstScalars* __restrict__ sc,
                                                        double* __restrict__ part) {
    const int lane32 = threadIdx.x & 31, sub = lane32 / W, lane = lane32 & (W - 1);
    for (int t = blockIdx.x * kWarps + (threadIdx.x >> 5); t < ntiles; t += gridDim.x * kWarps) {
        if (sc[tinst[t]].done) {  // warp-uniform
            if (lane32 == 0) part[t] = 0;
            continue;
        }
        const int64_t t0 = tstart[t], t1 = tstart[t + 1];
        double acc = 0;
        for (int64_t base = t0; base < t1; base += 32 / W) {
            const int64_t row = base + sub;
            const bool ok = row < t1;
            double s = 0;
            if (ok)
                for (int64_t k = rowptr[row] + lane; k < rowptr[row + 1]; k += W) s += vals[k] * p[col[k]];
#pragma unroll
            for (int o = W / 2; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, W);
            if (ok && lane == 0) {
                q[row] = s;
                acc += s * p[row];
            }
        }
        acc = wsum(acc);
        if (lane32 == 0) part[t] = acc;
    }
}

__global__ void balpha_kernel(int ninst, const int32_t* __restrict__ itp, const int32_t* __restrict__ it,
                              const double* __restrict__ part_pq, InstScalars* __restrict__ sc) {
    __shared__ double sh[32];
    const int i = blockIdx.x;
    if (sc[i].done) return;  // block-uniform
    const double pq = inst_reduce(part_pq, itp, it, i, sh);
    if (threadIdx.x == 0) {
        if (pq > 0 && isfinite(pq)) sc[i].alpha = sc[i].rz / pq;
        else sc[i].done = 2;  // breakdown
    }
}

__global__ void __launch_bounds__(256) bupdate_kernel(int ntiles, const int64_t* __restrict__ tstart,
                                                      const int32_t* __restrict__ tinst, double* __restrict__ x,
                                                      double* __restrict__ r, double* __restrict__ z,
                                                      const double* __restrict__ p, const double* __restrict__ q,
                                                      const double* __restrict__ dinv,
                                                      const InstScalars* __restrict__ sc,
                                                      double* __restrict__ part_rz, double* __restrict__ part_rr) {
    const int lane = threadIdx.x & 31;
    for (int t = blockIdx.x * kWarps + (threadIdx.x >> 5); t < ntiles; t += gridDim.x * kWarps) {
        const InstScalars& s = sc[tinst[t]];
        if (s.done) {  // warp-uniform
            if (lane == 0) part_rz[t] = part_rr[t] = 0;
            continue;
        }
        const double a = s.alpha;
        const int64_t t0 = tstart[t], t1 = tstart[t + 1];
        double arz = 0, arr = 0;
        for (int64_t i = t0 + lane; i < t1; i += 32) {
            x[i] += a * p[i];
            const double ri = r[i] - a * q[i];
            const double zi = dinv[i] * ri;
            r[i] = ri;
            z[i] = zi;
            arz += ri * zi;
            arr += ri * ri;
        }
        arz = wsum(arz);
        arr = wsum(arr);
        if (lane == 0) {
            part_rz[t] = arz;
            part_rr[t] = arr;
        }
    }
}

__global__ void bbeta_kernel(int ninst, const int32_t* __restrict__ itp, const int32_t* __restrict__ it,
                             const double* __restrict__ part_rz, const double* __restrict__ part_rr, long long maxit,
                             InstScalars* __restrict__ sc) {
    __shared__ double sh[32];
    const int i = blockIdx.x;
    if (sc[i].done) return;
    const double rz = inst_reduce(part_rz, itp, it, i, sh);
    const double rr = inst_reduce(part_rr, itp, it, i, sh);
    if (threadIdx.x == 0) {
        InstScalars s = sc[i];
        s.iters += 1;
        s.rr = rr;
        s.beta = rz / s.rz;
        s.rz = rz;
        if (rr <= s.tol2) s.done = 1;
        else if (!isfinite(rr) || !isfinite(s.beta) || s.iters >= maxit) s.done = 2;
        sc[i] = s;
    }
}

__global__ void __launch_bounds__(256) bpupdate_kernel(int ntiles, const int64_t* __restrict__ tstart,
                                                       const int32_t* __restrict__ tinst, double* __restrict__ p,
                                                       const double* __restrict__ z,
                                                       const InstScalars* __restrict__ sc) {
    const int lane = threadIdx.x & 31;
    for (int t = blockIdx.x * kWarps + (threadIdx.x >> 5); t < ntiles; t += gridDim.x * kWarps) {
        const InstScalars& s = sc[tinst[t]];
        if (s.done) continue;
        const double beta = s.beta;
        for (int64_t i = tstart[t] + lane; i < tstart[t + 1]; i += 32) p[i] = z[i] + beta * p[i];
    }
}

// after a body of kBatchIters iterations: continue while an instance runs and iterations remain
__global__ void bcheck_kernel(int ninst, const InstScalars* __restrict__ sc, BatchCtl* __restrict__ ctl,
                              cudaGraphConditionalHandle handle, int use_handle) {
    __shared__ int cnt[32];
    int c = 0;
    for (int i = threadIdx.x; i < ninst; i += blockDim.x) c += sc[i].done == 0 ? 1 : 0;
#pragma unroll
    for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) cnt[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int tot = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += cnt[w];
        ctl->iters += kBatchIters;
        ctl->remaining = tot;
        const unsigned more = (tot > 0 && ctl->iters < ctl->maxit) ? 1u : 0u;
        if (use_handle) cudaGraphSetConditional(handle, more);
    }
}

// true residual b - A x per tile (FP64), partial ||r||^2
template <int W>
__global__ void __launch_bounds__(256) bresid_kernel(int ntiles, const int64_t* __restrict__ tstart,
                                                     const int64_t* __restrict__ rowptr,
                                                     const int32_t* __restrict__ col, const double* __restrict__ vals,
                                                     const double* __restrict__ x, const double* __restrict__ b,
                                                     double* __restrict__ part) {
    const int lane32 = threadIdx.x & 31, sub = lane32 / W, lane = lane32 & (W - 1);
    for (int t = blockIdx.x * kWarps + (threadIdx.x >> 5); t < ntiles; t += gridDim.x * kWarps) {
        const int64_t t0 = tstart[t], t1 = tstart[t + 1];
        double acc = 0;
        for (int64_t base = t0; base < t1; base += 32 / W) {
            const int64_t row = base + sub;
            const bool ok = row < t1;
            double s = 0;
            if (ok)
                for (int64_t k = rowptr[row] + lane; k < rowptr[row + 1]; k += W) s += vals[k] * x[col[k]];
#pragma unroll
            for (int o = W / 2; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, W);
            if (ok && lane == 0) {
                const double ri = b[row] - s;
                acc += ri * ri;
            }
        }
        acc = wsum(acc);
        if (lane32 == 0) part[t] = acc;
    }
}

__global__ void binst_sum_kernel(int ninst, const int32_t* __restrict__ itp, const int32_t* __restrict__ it,
                                 const double* __restrict__ part, double* __restrict__ out) {
    __shared__ double sh[32];
    const double s = inst_reduce(part, itp, it, blockIdx.x, sh);
    if (threadIdx.x == 0) out[blockIdx.x] = s;
}

// ---------------------------------------------------------------- workspace
struct BatchWs {
    int ninst = 0;
    int64_t n = 0;
    int ntiles = 0;
    int W = 4;                       // autotuned lanes per row
    int32_t* inst = nullptr;         // [n]
    int64_t* tstart = nullptr;       // [ntiles + 1]
    int32_t* tinst = nullptr;        // [ntiles]
    int32_t* itp = nullptr;          // [ninst + 1]
    int32_t* it = nullptr;           // [ntiles]
    double *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr, *dinv = nullptr;
    double* part = nullptr;          // [3][ntiles]
    double* isum = nullptr;          // [ninst]
    double* x = nullptr;             // the solution of the current run (caller memory)
    InstScalars* sc = nullptr;       // [ninst]
    BatchCtl* ctl = nullptr;
    std::vector<int64_t> toff;
    float tune_ms[5] = {0, 0, 0, 0, 0};
    int conditional = 0;             // the last job ran as one graph with a device-side loop
    int asm_tuned = 0;               // the assembly's rows per block were timed on this instance set
    float asm_tune_ms[2] = {0, 0};   // assembly with 1, 2 warps (32 rows each) per block
};

// blocks of 256 threads (8 tiles in flight each), at most 8 blocks per SM on 152 SMs
int grid_tiles(int ntiles) { return std::max(1, std::min((ntiles + kWarps - 1) / kWarps, 152 * 8)); }

template <int W>
void launch_spmv_dot(anigpu_ctx* h, BatchWs* w, const double* vals, cudaStream_t s) {
    bspmv_dot_kernel<W><<<grid_tiles(w->ntiles), 256, 0, s>>>(w->ntiles, w->tstart, w->tinst, h->rowptr,
                                                                       h->col, vals, w->p, w->q, w->sc, w->part);
}
void spmv_dot(anigpu_ctx* h, BatchWs* w, const double* vals, cudaStream_t s) {
    switch (w->W) {
        case 2: launch_spmv_dot<2>(h, w, vals, s); break;
        case 8: launch_spmv_dot<8>(h, w, vals, s); break;
        case 16: launch_spmv_dot<16>(h, w, vals, s); break;
        default: launch_spmv_dot<4>(h, w, vals, s);
    }
    h->launches++;
}

int one_iteration(anigpu_ctx* h, BatchWs* w, const double* vals, int64_t maxit, cudaStream_t s) {
    const int gt = grid_tiles(w->ntiles);
    spmv_dot(h, w, vals, s);
    balpha_kernel<<<w->ninst, 128, 0, s>>>(w->ninst, w->itp, w->it, w->part, w->sc);
    bupdate_kernel<<<gt, 256, 0, s>>>(w->ntiles, w->tstart, w->tinst, w->x, w->r, w->z, w->p, w->q, w->dinv,
                                            w->sc, w->part + w->ntiles, w->part + 2 * w->ntiles);
    bbeta_kernel<<<w->ninst, 128, 0, s>>>(w->ninst, w->itp, w->it, w->part + w->ntiles, w->part + 2 * w->ntiles,
                                          (long long)maxit, w->sc);
    bpupdate_kernel<<<gt, 256, 0, s>>>(w->ntiles, w->tstart, w->tinst, w->p, w->z, w->sc);
    h->launches += 4;
    ANI_CUDA(h, cudaGetLastError());
    return ANIGPU_OK;
}

BatchWs* ws(anigpu_ctx* h) { return static_cast<BatchWs*>(h->batch_ws); }

// the device status word after a setup kernel (waits for the stream)
int status_check(anigpu_ctx* h, const char* what) {
    int st = 0;
    ANI_CUDA(h, cudaMemcpyAsync(&st, h->d_status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    ANI_CUDA(h, cudaStreamSynchronize(h->stream));
    if (st != 0) {
        ANI_CUDA(h, cudaMemsetAsync(h->d_status, 0, sizeof(int), h->stream));
        return set_err(h, st, what);
    }
    return ANIGPU_OK;
}

}  // namespace

void free_batch(anigpu_ctx* h) {
    BatchWs* w = ws(h);
    if (!w) return;
    void* ptrs[] = {w->inst, w->tstart, w->tinst, w->itp, w->it, w->r, w->z, w->p, w->q, w->dinv, w->part, w->isum,
                    w->sc, w->ctl};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete w;
    h->batch_ws = nullptr;
}

int batch_set_instances(anigpu_ctx* h, int ninst, const int64_t* toff_host, const void* vals_for_tuning) {
    if (h->space < 0) return set_err(h, ANIGPU_ERR_STATE, "anigpu_problem_setup not called");
    if (h->space != ANIGPU_P1 && h->space != ANIGPU_P2)
        return set_err(h, ANIGPU_ERR_UNSUPPORTED, "batched instances need a P1 or P2 problem");
    if (ninst < 1 || ninst > (1 << 24) || !toff_host) return set_err(h, ANIGPU_ERR_ARG, "instances");
    if (toff_host[0] != 0 || toff_host[ninst] != h->nt) return set_err(h, ANIGPU_ERR_ARG, "tet offsets must span 0..nt");
    for (int i = 0; i < ninst; ++i)
        if (toff_host[i + 1] <= toff_host[i]) return set_err(h, ANIGPU_ERR_ARG, "every instance needs a tet");
    free_batch(h);
    BatchWs* w = new BatchWs();
    h->batch_ws = w;
    w->ninst = ninst;
    w->n = h->ndof;
    w->toff.assign(toff_host, toff_host + ninst + 1);
    cudaStream_t s = h->stream;
    const int64_t n = h->ndof;
    RC_(dev_alloc(h, &w->inst, n));
    ANI_CUDA(h, cudaMemsetAsync(w->inst, 0xff, sizeof(int32_t) * n, s));
    int64_t* dtoff = nullptr;
    ANI_CUDA(h, cudaMallocAsync((void**)&dtoff, sizeof(int64_t) * (ninst + 1), s));
    ANI_CUDA(h, cudaMemcpyAsync(dtoff, toff_host, sizeof(int64_t) * (ninst + 1), cudaMemcpyHostToDevice, s));
    dof_inst_kernel<<<grid_for(h->nt, 256), 256, 0, s>>>(h->nt, h->nloc_s, h->edofs, dtoff, ninst, w->inst,
                                                         h->d_status);
    ANI_LAUNCHED(h);
    RC_(status_check(h, "instance map: instances must not share vertices"));
    ANI_CUDA(h, cudaFreeAsync(dtoff, s));
    // tiles
    unsigned long long* flag = nullptr;
    int64_t* pos = nullptr;
    ANI_CUDA(h, cudaMallocAsync((void**)&flag, sizeof(unsigned long long) * (n + 1), s));
    ANI_CUDA(h, cudaMallocAsync((void**)&pos, sizeof(int64_t) * (n + 1), s));
    ANI_CUDA(h, cudaMemsetAsync(flag, 0, sizeof(unsigned long long) * (n + 1), s));
    tile_flag_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, w->inst, flag);
    ANI_LAUNCHED(h);
    RC_(scan_counts(h, flag, n, pos));
    int64_t nt64 = 0;
    ANI_CUDA(h, cudaMemcpyAsync(&nt64, pos + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    ANI_CUDA(h, cudaStreamSynchronize(s));
    if (nt64 <= 0 || nt64 > (int64_t)1 << 30) return set_err(h, ANIGPU_ERR_ARG, "tile count");
    w->ntiles = (int)nt64;
    RC_(dev_alloc(h, &w->tstart, (size_t)w->ntiles + 1));
    RC_(dev_alloc(h, &w->tinst, (size_t)w->ntiles));
    tile_fill_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, flag, pos, w->inst, w->tstart, w->tinst);
    ANI_LAUNCHED(h);
    ANI_CUDA(h, cudaMemcpyAsync(w->tstart + w->ntiles, &n, sizeof(int64_t), cudaMemcpyHostToDevice, s));
    ANI_CUDA(h, cudaFreeAsync(flag, s));
    ANI_CUDA(h, cudaFreeAsync(pos, s));
    // per-instance tile lists, ascending (host: a counting sort of the tile instances)
    std::vector<int32_t> tinst(w->ntiles);
    ANI_CUDA(h, cudaMemcpyAsync(tinst.data(), w->tinst, sizeof(int32_t) * w->ntiles, cudaMemcpyDeviceToHost, s));
    ANI_CUDA(h, cudaStreamSynchronize(s));
    std::vector<int32_t> itp(ninst + 1, 0), it(w->ntiles);
    for (int t = 0; t < w->ntiles; ++t) itp[tinst[t] + 1]++;
    for (int i = 0; i < ninst; ++i) itp[i + 1] += itp[i];
    {
        std::vector<int32_t> fill(itp.begin(), itp.end() - 1);
        for (int t = 0; t < w->ntiles; ++t) it[fill[tinst[t]]++] = t;
    }
    for (int i = 0; i < ninst; ++i)
        if (itp[i + 1] == itp[i]) return set_err(h, ANIGPU_ERR_ARG, "an instance has no DOF");
    RC_(dev_alloc(h, &w->itp, (size_t)ninst + 1));
    RC_(dev_alloc(h, &w->it, (size_t)w->ntiles));
    ANI_CUDA(h, cudaMemcpyAsync(w->itp, itp.data(), sizeof(int32_t) * (ninst + 1), cudaMemcpyHostToDevice, s));
    ANI_CUDA(h, cudaMemcpyAsync(w->it, it.data(), sizeof(int32_t) * w->ntiles, cudaMemcpyHostToDevice, s));
    RC_(dev_alloc(h, &w->r, n));
    RC_(dev_alloc(h, &w->z, n));
    RC_(dev_alloc(h, &w->p, n));
    RC_(dev_alloc(h, &w->q, n));
    RC_(dev_alloc(h, &w->dinv, n));
    RC_(dev_alloc(h, &w->part, (size_t)3 * w->ntiles));
    RC_(dev_alloc(h, &w->isum, (size_t)ninst));
    RC_(dev_alloc(h, &w->sc, (size_t)ninst));
    RC_(dev_alloc(h, &w->ctl, 1));
    ANI_CUDA(h, cudaStreamSynchronize(s));
    // autotune the lanes per row on the given values (q = A p with p = 1 on every DOF)
    w->W = h->nnz > 12 * h->ndof ? 8 : 4;
    if (vals_for_tuning) {
        bdiag_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, h->rowptr, h->col, (const double*)vals_for_tuning, w->p);
        ANI_LAUNCHED(h);
        ANI_CUDA(h, cudaMemsetAsync(w->sc, 0, sizeof(InstScalars) * ninst, s));
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        const int cand[4] = {2, 4, 8, 16};
        float best = 1e30f;
        int bestW = w->W;
        for (int c = 0; c < 4; ++c) {
            w->W = cand[c];
            spmv_dot(h, w, (const double*)vals_for_tuning, s);  // warm-up
            cudaEventRecord(e0, s);
            for (int rep = 0; rep < 5; ++rep) spmv_dot(h, w, (const double*)vals_for_tuning, s);
            cudaEventRecord(e1, s);
            cudaEventSynchronize(e1);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            w->tune_ms[c] = ms / 5;
            if (ms < best) {
                best = ms;
                bestW = cand[c];
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        w->W = bestW;
        ANI_CUDA(h, cudaGetLastError());
    }
    return ANIGPU_OK;
}

int batch_info(anigpu_ctx* h, int* ntiles, int* lanes, float* tune_ms, int* device_loop) {
    BatchWs* w = ws(h);
    if (!w) return set_err(h, ANIGPU_ERR_STATE, "anigpu_batch_set_instances not called");
    if (ntiles) *ntiles = w->ntiles;
    if (lanes) *lanes = w->W;
    if (device_loop) *device_loop = w->conditional;
    if (tune_ms)
        for (int c = 0; c < 4; ++c) tune_ms[c] = w->tune_ms[c];
    return ANIGPU_OK;
}

// the whole job: (optional) assembly, initialisation and every PCG iteration of every instance.
// Several jobs (handles on one device, e.g. the P1 instances and the P2 instances) go into one
// graph: per job a prologue (child graph) and a device-side while loop (conditional node) whose body
// is kBatchIters iterations and a check kernel; the jobs' node chains are independent, so they run
// concurrently within the one launch.  Where conditional nodes are unavailable the jobs run one after
// the other as host-driven launches of their captured bodies.
namespace {

struct Job {
    anigpu_ctx* h;
    BatchWs* w;
    int kind;
    const double* D;
    const double* f;
    double f_const;
    int order;
    double* vals;
    double* rhs_assembled;
    const double* b;
    double* x;
    anigpu_solve_stats* st;
    bool assemble;
};

int job_check(const Job& j, int64_t maxit) {
    anigpu_ctx* h = j.h;
    if (!j.w) return set_err(h, ANIGPU_ERR_STATE, "anigpu_batch_set_instances not called");
    if (!j.vals || !j.b || !j.x || !j.st) return set_err(h, ANIGPU_ERR_ARG, "NULL argument");
    if (maxit < 1) return set_err(h, ANIGPU_ERR_ARG, "maxit");
    return ANIGPU_OK;
}

// the assembly's rows per block (warps of 32 rows; the row gather is compiled for at most 64
// threads per block): timed on this job's tensor once per instance set
int tune_assembly(Job& j) {
    anigpu_ctx* h = j.h;
    BatchWs* w = j.w;
    if (!j.assemble || w->asm_tuned) return ANIGPU_OK;
    cudaStream_t s = h->stream;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int cand[2] = {1, 2};
    float best = 1e30f;
    int bestw = h->row_warps;
    for (int c = 0; c < 2; ++c) {
        h->row_warps = cand[c];
        RC_(run_assemble(h, j.kind, j.D, j.f, j.f_const, j.order, ANIGPU_F64, j.vals, j.rhs_assembled, nullptr, 1e-100));
        cudaEventRecord(e0, s);
        for (int rep = 0; rep < 3; ++rep)
            RC_(run_assemble(h, j.kind, j.D, j.f, j.f_const, j.order, ANIGPU_F64, j.vals, j.rhs_assembled, nullptr,
                             1e-100));
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        w->asm_tune_ms[c] = ms / 3;
        if (ms < best) {
            best = ms;
            bestw = cand[c];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    h->row_warps = bestw;
    w->asm_tuned = 1;
    RC_(status_check(h, "assembly"));
    return ANIGPU_OK;
}

int job_prepare(Job& j, int64_t maxit) {
    anigpu_ctx* h = j.h;
    BatchWs* w = j.w;
    if (j.assemble && h->tetdata_bytes < (size_t)h->nt * 8 * sizeof(double)) {
        // the per-tet blocks of the assembly: allocated before the graph is captured
        if (h->tetdata) cudaFree(h->tetdata);
        h->tetdata = nullptr;
        ANI_CUDA(h, cudaMalloc(&h->tetdata, (size_t)h->nt * 8 * sizeof(double)));
        h->tetdata_bytes = (size_t)h->nt * 8 * sizeof(double);
    }
    RC_(tune_assembly(j));
    BatchCtl c0{0, (long long)maxit, w->ninst, 0};
    ANI_CUDA(h, cudaMemcpyAsync(w->ctl, &c0, sizeof(BatchCtl), cudaMemcpyHostToDevice, h->stream));
    ANI_CUDA(h, cudaStreamSynchronize(h->stream));
    w->x = j.x;  // the iteration kernels update the caller's solution in place
    w->conditional = 0;
    return ANIGPU_OK;
}

// prologue: assembly, diagonal, initial residual
int job_prologue(Job& j, double rtol) {
    anigpu_ctx* h = j.h;
    BatchWs* w = j.w;
    cudaStream_t s = h->stream;
    const int gt = grid_tiles(w->ntiles);
    if (j.assemble) RC_(run_assemble(h, j.kind, j.D, j.f, j.f_const, j.order, ANIGPU_F64, j.vals, j.rhs_assembled, nullptr, 1e-100));
    bdiag_kernel<<<grid_for(w->n, 256), 256, 0, s>>>(w->n, h->rowptr, h->col, j.vals, w->dinv);
    binit_kernel<<<gt, 256, 0, s>>>(w->ntiles, w->tstart, j.b, w->dinv, j.x, w->r, w->z, w->p, w->part,
                                    w->part + w->ntiles);
    binst_init_kernel<<<w->ninst, 128, 0, s>>>(w->ninst, w->itp, w->it, w->part, w->part + w->ntiles, rtol, w->sc);
    h->launches += 3;
    ANI_CUDA(h, cudaGetLastError());
    return ANIGPU_OK;
}

int job_body(Job& j, int64_t maxit, cudaGraphConditionalHandle hd, int use) {
    anigpu_ctx* h = j.h;
    BatchWs* w = j.w;
    for (int k = 0; k < kBatchIters; ++k) RC_(one_iteration(h, w, j.vals, maxit, h->stream));
    bcheck_kernel<<<1, 256, 0, h->stream>>>(w->ninst, w->sc, w->ctl, hd, use);
    h->launches++;
    ANI_CUDA(h, cudaGetLastError());
    return ANIGPU_OK;
}

// job j's nodes in graph g: prologue child graph -> while(cond) { body }
bool job_add_to_graph(Job& j, cudaGraph_t g, double rtol, int64_t maxit, cudaGraph_t* pre_out) {
    anigpu_ctx* h = j.h;
    cudaStream_t s = h->stream;
    cudaGraph_t pre = nullptr;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return false;
    const int prc = job_prologue(j, rtol);
    cudaError_t e = cudaStreamEndCapture(s, &pre);
    *pre_out = pre;
    if (prc != ANIGPU_OK || e != cudaSuccess || !pre) return false;
    cudaGraphNode_t preNode;
    cudaGraphConditionalHandle hd;
    if (cudaGraphAddChildGraphNode(&preNode, g, nullptr, 0, pre) != cudaSuccess) return false;
    if (cudaGraphConditionalHandleCreate(&hd, g, 1, cudaGraphCondAssignDefault) != cudaSuccess) return false;
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = hd;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t cnode;
    if (cudaGraphAddNode(&cnode, g, &preNode, nullptr, 1, &np) != cudaSuccess) return false;
    cudaGraph_t bodyg = np.conditional.phGraph_out[0];
    if (cudaStreamBeginCaptureToGraph(s, bodyg, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return false;
    const int brc = job_body(j, maxit, hd, 1);
    cudaGraph_t outg = nullptr;
    e = cudaStreamEndCapture(s, &outg);
    return brc == ANIGPU_OK && e == cudaSuccess;
}

// host-driven fallback for one job: prologue, then captured bodies until the device says stop
int job_run_host(Job& j, double rtol, int64_t maxit) {
    anigpu_ctx* h = j.h;
    RC_(job_prologue(j, rtol));
    BatchCtl hc{};
    while (true) {
        RC_(job_body(j, maxit, 0, 0));
        ANI_CUDA(h, cudaMemcpyAsync(&hc, j.w->ctl, sizeof(BatchCtl), cudaMemcpyDeviceToHost, h->stream));
        ANI_CUDA(h, cudaStreamSynchronize(h->stream));
        if (hc.remaining == 0 || hc.iters >= hc.maxit) break;
    }
    return ANIGPU_OK;
}

// statistics: FP64 true residual per instance; launch count of the job
int job_finish(Job& j, double rtol, float ms, bool* all) {
    anigpu_ctx* h = j.h;
    BatchWs* w = j.w;
    cudaStream_t s = h->stream;
    const int gt = grid_tiles(w->ntiles);
    switch (w->W) {
        case 2: bresid_kernel<2><<<gt, 256, 0, s>>>(w->ntiles, w->tstart, h->rowptr, h->col, j.vals, j.x, j.b, w->part); break;
        case 8: bresid_kernel<8><<<gt, 256, 0, s>>>(w->ntiles, w->tstart, h->rowptr, h->col, j.vals, j.x, j.b, w->part); break;
        case 16: bresid_kernel<16><<<gt, 256, 0, s>>>(w->ntiles, w->tstart, h->rowptr, h->col, j.vals, j.x, j.b, w->part); break;
        default: bresid_kernel<4><<<gt, 256, 0, s>>>(w->ntiles, w->tstart, h->rowptr, h->col, j.vals, j.x, j.b, w->part);
    }
    binst_sum_kernel<<<w->ninst, 128, 0, s>>>(w->ninst, w->itp, w->it, w->part, w->isum);
    ANI_LAUNCHED(h);
    std::vector<double> rr(w->ninst);
    std::vector<InstScalars> hs(w->ninst);
    BatchCtl hc{};
    ANI_CUDA(h, cudaMemcpyAsync(rr.data(), w->isum, sizeof(double) * w->ninst, cudaMemcpyDeviceToHost, s));
    ANI_CUDA(h, cudaMemcpyAsync(hs.data(), w->sc, sizeof(InstScalars) * w->ninst, cudaMemcpyDeviceToHost, s));
    ANI_CUDA(h, cudaMemcpyAsync(&hc, w->ctl, sizeof(BatchCtl), cudaMemcpyDeviceToHost, s));
    ANI_CUDA(h, cudaStreamSynchronize(s));
    h->launches += (j.assemble ? 3 : 0) + 3 + (hc.iters / kBatchIters) * (5 * kBatchIters + 1);
    for (int i = 0; i < w->ninst; ++i) {
        const double rel = hs[i].bb > 0 ? std::sqrt(rr[i] / hs[i].bb) : std::sqrt(rr[i]);
        j.st[i] = anigpu_solve_stats{hs[i].iters, hc.iters, rel, ms * 1e-3, 0};
        *all &= rel <= rtol;
    }
    return ANIGPU_OK;
}

int run_jobs(std::vector<Job>& jobs, double rtol, int64_t maxit) {
    for (Job& j : jobs) RC_(job_check(j, maxit));
    for (size_t k = 1; k < jobs.size(); ++k)
        if (jobs[k].h->device != jobs[0].h->device)
            return set_err(jobs[k].h, ANIGPU_ERR_ARG, "batched jobs of one launch must share a device");
    for (Job& j : jobs) RC_(job_prepare(j, maxit));
    anigpu_ctx* h0 = jobs[0].h;
    cudaStream_t s0 = h0->stream;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int rc = ANIGPU_OK;
    cudaGraph_t g = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<cudaGraph_t> pres(jobs.size(), nullptr);
    bool ok = cudaGraphCreate(&g, 0) == cudaSuccess;
    for (size_t k = 0; k < jobs.size() && ok; ++k) {
        const int64_t l0 = jobs[k].h->launches;
        ok = job_add_to_graph(jobs[k], g, rtol, maxit, &pres[k]);
        jobs[k].h->launches = l0;  // counted from the device's iteration count after the run
    }
    ok = ok && cudaGraphInstantiate(&exec, g, 0) == cudaSuccess;
    cudaGetLastError();
    // every job's inputs are ready on its own stream before the launch on the first job's stream
    for (size_t k = 1; k < jobs.size(); ++k) {
        ANI_CUDA(h0, cudaEventRecord(jobs[k].h->fork_ev, jobs[k].h->stream));
        ANI_CUDA(h0, cudaStreamWaitEvent(s0, jobs[k].h->fork_ev, 0));
    }
    cudaEventRecord(e0, s0);
    if (ok) {
        for (Job& j : jobs) j.w->conditional = 1;
        const cudaError_t le = cudaGraphLaunch(exec, s0);
        if (le != cudaSuccess) rc = cuda_check(h0, le, "cudaGraphLaunch");
    } else {
        for (Job& j : jobs) {
            if (j.h != h0) {
                ANI_CUDA(h0, cudaEventRecord(h0->fork_ev, s0));
                ANI_CUDA(j.h, cudaStreamWaitEvent(j.h->stream, h0->fork_ev, 0));
            }
            rc = job_run_host(j, rtol, maxit);
            if (rc) break;
            if (j.h != h0) {
                ANI_CUDA(j.h, cudaEventRecord(j.h->join_ev, j.h->stream));
                ANI_CUDA(h0, cudaStreamWaitEvent(s0, j.h->join_ev, 0));
            }
        }
    }
    cudaEventRecord(e1, s0);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (exec) cudaGraphExecDestroy(exec);
    if (g) cudaGraphDestroy(g);
    for (cudaGraph_t p : pres)
        if (p) cudaGraphDestroy(p);
    if (rc) return rc;
    // the jobs' streams see the results: the launch ran on the first job's stream
    for (size_t k = 1; k < jobs.size(); ++k) {
        ANI_CUDA(h0, cudaEventRecord(h0->join_ev, s0));
        ANI_CUDA(jobs[k].h, cudaStreamWaitEvent(jobs[k].h->stream, h0->join_ev, 0));
    }
    bool all = true;
    for (Job& j : jobs) RC_(job_finish(j, rtol, ms, &all));
    return all ? ANIGPU_OK : set_err(h0, ANIGPU_ERR_NOT_CONVERGED, "some instances did not reach the tolerance");
}

}  // namespace

int batch_run(anigpu_ctx* h, int kind, const double* D, const double* f, double f_const, int order, double* vals,
              double* rhs_assembled, const double* b, double* x, double rtol, int64_t maxit, anigpu_solve_stats* st) {
    std::vector<Job> jobs{Job{h, ws(h), kind, D, f, f_const, order, vals, rhs_assembled, b, x, st, rhs_assembled != nullptr}};
    return run_jobs(jobs, rtol, maxit);
}

int batch_run_jobs(int njobs, const anigpu_batch_job* in, double rtol, int64_t maxit) {
    if (njobs < 1 || !in) return ANIGPU_ERR_ARG;
    std::vector<Job> jobs;
    for (int k = 0; k < njobs; ++k) {
        const anigpu_batch_job& a = in[k];
        if (!a.h) return ANIGPU_ERR_ARG;
        jobs.push_back(Job{a.h, ws(a.h), a.tensor_kind, a.D, a.f, a.f_const, a.order, a.vals, a.rhs_assembled, a.b,
                           a.x, a.stats, a.rhs_assembled != nullptr});
    }
    return run_jobs(jobs, rtol, maxit);
}

int batch_assembly_tuning(anigpu_ctx* h, int* row_warps, float* ms) {
    BatchWs* w = ws(h);
    if (!w) return set_err(h, ANIGPU_ERR_STATE, "anigpu_batch_set_instances not called");
    if (row_warps) *row_warps = h->row_warps;
    if (ms)
        for (int c = 0; c < 2; ++c) ms[c] = w->asm_tune_ms[c];
    return ANIGPU_OK;
}
