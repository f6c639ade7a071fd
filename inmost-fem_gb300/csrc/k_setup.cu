// Problem setup on the device: tet orientation, edge numbering, the NATURAL DOF
// numbering, the topological CSR template and the row-gather scatter records.
//
// Reference semantics restated here:
//   * reorderNodesOnTetrahedron (anifem++/inmost_interface/ordering.inl:9-26): swap local
//     nodes 2 and 3 when det(X0-X3, X1-X3, X2-X3) < 0.
//   * GlobEnumeration NATURAL (global_enumerator.h:392-404): vertex DOFs by vertex id, then
//     edge DOFs by edge id; FemVec components as consecutive blocks.  Edge ids are the rank
//     of (min vertex, max vertex) in lexicographic order.
//   * AssembleTemplate (assembler.inl:590-693): every pair of DOFs that share a tet, rows
//     sorted, diagonal always present (assembler.inl:114-135).
// Every list that is built with atomics is re-sorted per row, so the structures are
// identical from run to run.
#include <cub/cub.cuh>

#include "anigpu_internal.h"

namespace {

constexpr int kWarpsPerBlock = 8;

__global__ void orient_kernel(int64_t nt, const double* __restrict__ xyz, int32_t* __restrict__ tets) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nt) return;
    int4 v = reinterpret_cast<int4*>(tets)[t];
    double m[3][3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const double x3 = xyz[3 * (int64_t)v.w + j];
        m[0][j] = xyz[3 * (int64_t)v.x + j] - x3;
        m[1][j] = xyz[3 * (int64_t)v.y + j] - x3;
        m[2][j] = xyz[3 * (int64_t)v.z + j] - x3;
    }
    double det = 0;
    det += m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]);
    det += m[0][1] * (m[1][2] * m[2][0] - m[1][0] * m[2][2]);
    det += m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
    if (det < 0) {
        const int s = v.z;
        v.z = v.w;
        v.w = s;
        reinterpret_cast<int4*>(tets)[t] = v;
    }
}

__global__ void bad_index_kernel(int64_t n, const int32_t* __restrict__ idx, int64_t limit, int* __restrict__ status) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t v = idx[i];
    if (v < 0 || v >= limit) atomicExch(status, ANIGPU_ERR_BAD_ELEMENT);
}

// count[key[i]]++ for n entries with stride-free keys
__global__ void count_kernel(int64_t n, const int32_t* __restrict__ keys, unsigned long long* __restrict__ cnt) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    atomicAdd(&cnt[keys[i]], 1ull);
}

// list[cursor[key]++] = i  (unordered within a key; sorted afterwards)
__global__ void fill_kernel(int64_t n, const int32_t* __restrict__ keys, unsigned long long* __restrict__ cursor,
                            int32_t* __restrict__ list) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned long long p = atomicAdd(&cursor[keys[i]], 1ull);
    list[p] = (int32_t)i;
}

// Warp-cooperative "sorted unique" of a candidate list in shared memory.
// Step 1 keeps the first occurrence of every value (compacted into tmp with ballots),
// step 2 ranks the distinct values (rank = number of smaller distinct values) and
// writes them to out[rank].  Returns the number of distinct values.
__device__ inline int warp_sorted_unique(const int32_t* cand, int m, int lane, int32_t* tmp, int32_t* out) {
    int u = 0;
    for (int base = 0; base < m; base += 32) {
        const int a = base + lane;
        bool first = false;
        int32_t v = 0;
        if (a < m) {
            v = cand[a];
            first = true;
            for (int b = 0; b < a; ++b)
                if (cand[b] == v) {
                    first = false;
                    break;
                }
        }
        const unsigned bal = __ballot_sync(0xffffffffu, first);
        if (first) tmp[u + __popc(bal & ((1u << lane) - 1u))] = v;
        u += __popc(bal);
    }
    __syncwarp();
    if (out) {
        for (int a = lane; a < u; a += 32) {
            const int32_t v = tmp[a];
            int rank = 0;
            for (int b = 0; b < u; ++b) rank += tmp[b] < v;
            out[rank] = v;
        }
    }
    return u;
}

__global__ void div4_kernel(int64_t n, int32_t* __restrict__ a) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) a[i] >>= 2;
}

// ---------------------------------------------------------------- edges
// Per vertex v: the distinct neighbours w > v over its incident tets.  pass 0 counts,
// pass 1 writes them sorted into nbr[eptr[v] ...].
__global__ void vertex_edges_kernel(int pass, int64_t nv, const int64_t* __restrict__ vptr,
                                    const int32_t* __restrict__ vlist, const int32_t* __restrict__ tets, int cap,
                                    unsigned long long* __restrict__ ecount, const int64_t* __restrict__ eptr,
                                    int32_t* __restrict__ nbr, int* __restrict__ status) {
    extern __shared__ int32_t sh[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int32_t* cand = sh + warp * 2 * cap;
    int32_t* tmp = cand + cap;
    const int64_t v = blockIdx.x * (int64_t)kWarpsPerBlock + warp;
    if (v >= nv) return;
    const int64_t b = vptr[v], e = vptr[v + 1];
    if ((e - b) * 3 > cap) {
        if (lane == 0) atomicExch(status, ANIGPU_ERR_UNSUPPORTED);
        return;
    }
    // gather candidates w > v
    __shared__ int s_m[kWarpsPerBlock];
    if (lane == 0) s_m[warp] = 0;
    __syncwarp();
    for (int64_t k = b + lane; k < e; k += 32) {
        const int4 tv = reinterpret_cast<const int4*>(tets)[vlist[k]];
        const int32_t w[4] = {tv.x, tv.y, tv.z, tv.w};
#pragma unroll
        for (int i = 0; i < 4; ++i)
            if (w[i] > v) {
                const int p = atomicAdd(&s_m[warp], 1);
                cand[p] = w[i];
            }
    }
    __syncwarp();
    const int m = s_m[warp];
    const int c = warp_sorted_unique(cand, m, lane, tmp, pass == 0 ? nullptr : nbr + eptr[v]);
    if (pass == 0 && lane == 0) ecount[v] = (unsigned long long)c;
}

__device__ inline int64_t lower_bound_i32(const int32_t* a, int64_t lo, int64_t hi, int32_t key) {
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__global__ void tet_edges_kernel(int64_t nt, const int32_t* __restrict__ tets, const int64_t* __restrict__ eptr,
                                 const int32_t* __restrict__ nbr, int32_t* __restrict__ tet_edges) {
    const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= nt * 6) return;
    const int64_t t = idx / 6;
    const int e = (int)(idx - t * 6);
    const int I[6] = {0, 0, 0, 1, 1, 2}, J[6] = {1, 2, 3, 2, 3, 3};
    const int32_t a = tets[4 * t + I[e]], b = tets[4 * t + J[e]];
    const int32_t lo = a < b ? a : b, hi = a < b ? b : a;
    tet_edges[idx] = (int32_t)lower_bound_i32(nbr, eptr[lo], eptr[lo + 1], hi);
}

__global__ void element_dofs_kernel(int64_t nt, int nloc, int64_t nv, const int32_t* __restrict__ tets,
                                    const int32_t* __restrict__ tet_edges, int32_t* __restrict__ edofs) {
    const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= nt * nloc) return;
    const int64_t t = idx / nloc;
    const int i = (int)(idx - t * nloc);
    edofs[idx] = i < 4 ? tets[4 * t + i] : (int32_t)(nv + tet_edges[6 * t + (i - 4)]);
}

// ---------------------------------------------------------------- DOF incidence
// inc[k] holds tet*16 + local index; sort each row's list ascending (deterministic order)
__global__ void sort_rows_kernel(int64_t nrows, const int64_t* __restrict__ ptr, int32_t* __restrict__ list,
                                 int cap, int* __restrict__ status) {
    extern __shared__ int32_t sh[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int32_t* buf = sh + warp * cap;
    const int64_t r = blockIdx.x * (int64_t)kWarpsPerBlock + warp;
    if (r >= nrows) return;
    const int64_t b = ptr[r], e = ptr[r + 1];
    const int m = (int)(e - b);
    if (m > cap) {
        if (lane == 0) atomicExch(status, ANIGPU_ERR_UNSUPPORTED);
        return;
    }
    for (int k = lane; k < m; k += 32) buf[k] = list[b + k];
    __syncwarp();
    // values are distinct: rank = number of smaller values
    for (int k = lane; k < m; k += 32) {
        const int32_t v = buf[k];
        int rank = 0;
        for (int j = 0; j < m; ++j) rank += buf[j] < v;
        list[b + rank] = v;
    }
}

__global__ void dof_count_kernel(int64_t n, const int32_t* __restrict__ edofs, unsigned long long* __restrict__ cnt) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    atomicAdd(&cnt[edofs[i]], 1ull);
}
__global__ void dof_fill_kernel(int64_t n, int nloc, const int32_t* __restrict__ edofs,
                                unsigned long long* __restrict__ cursor, int32_t* __restrict__ inc) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t t = i / nloc;
    const int loc = (int)(i - t * nloc);
    const unsigned long long p = atomicAdd(&cursor[edofs[i]], 1ull);
    inc[p] = (int32_t)(t * 16 + loc);
}

// ---------------------------------------------------------------- CSR template
__global__ void template_rows_kernel(int pass, int64_t nrows, int nloc, const int64_t* __restrict__ iptr,
                                     const int32_t* __restrict__ inc, const int32_t* __restrict__ edofs, int cap,
                                     unsigned long long* __restrict__ rcount, const int64_t* __restrict__ rowptr,
                                     int32_t* __restrict__ col, int* __restrict__ status) {
    extern __shared__ int32_t sh[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int32_t* cand = sh + warp * 2 * cap;
    int32_t* tmp = cand + cap;
    const int64_t r = blockIdx.x * (int64_t)kWarpsPerBlock + warp;
    if (r >= nrows) return;
    const int64_t b = iptr[r], e = iptr[r + 1];
    const int m = (int)((e - b) * nloc + 1);
    if (m > cap) {
        if (lane == 0) atomicExch(status, ANIGPU_ERR_UNSUPPORTED);
        return;
    }
    if (lane == 0) cand[0] = (int32_t)r;  // diagonal forced
    for (int64_t k = lane; k < (e - b) * nloc; k += 32) {
        const int64_t kk = k / nloc;
        const int j = (int)(k - kk * nloc);
        const int32_t packed = inc[b + kk];
        cand[1 + k] = edofs[(int64_t)(packed >> 4) * nloc + j];
    }
    __syncwarp();
    const int c = warp_sorted_unique(cand, m, lane, tmp, pass == 0 ? nullptr : col + rowptr[r]);
    if (pass == 0 && lane == 0) rcount[r] = (unsigned long long)c;
}

// scatter records: for row r and incident (tet, i): offsets of the tet's DOFs in row r
__global__ void records_kernel(int64_t nrows, int nloc, const int64_t* __restrict__ iptr,
                               const int32_t* __restrict__ inc, const int32_t* __restrict__ edofs,
                               const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                               ScatterRec* __restrict__ recs) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= iptr[nrows]) return;
    // row of incidence k: binary search in iptr
    int64_t lo = 0, hi = nrows;
    while (hi - lo > 1) {
        const int64_t mid = (lo + hi) >> 1;
        if (iptr[mid] <= k) lo = mid;
        else hi = mid;
    }
    const int64_t r = lo;
    const int32_t packed = inc[k];
    const int64_t t = packed >> 4;
    const int i = packed & 15;
    const int64_t rb = rowptr[r], re = rowptr[r + 1];
    uint32_t off[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int j = 0; j < nloc; ++j) {  // canonical column j of row i
        const int32_t c = edofs[t * nloc + canon_local(nloc, i, j)];
        off[j] = (uint32_t)(lower_bound_i32(col, rb, re, c) - rb);
    }
    ScatterRec rec;
    rec.tet = (uint32_t)t;
    rec.meta = (uint32_t)i | (off[8] << 16) | (off[9] << 24);
    rec.off03 = off[0] | (off[1] << 8) | (off[2] << 16) | (off[3] << 24);
    rec.off47 = off[4] | (off[5] << 8) | (off[6] << 16) | (off[7] << 24);
    recs[k] = rec;
}

// Dirichlet bits of each record: bit 4+c set when the DOF of canonical column c is Dirichlet
__global__ void dirichlet_bits_kernel(int64_t nrec, int nloc, const int32_t* __restrict__ edofs,
                                      const uint8_t* __restrict__ mask, ScatterRec* __restrict__ recs) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= nrec) return;
    ScatterRec rec = recs[k];
    const int i = rec.meta & 15;
    uint32_t bits = 0;
    for (int c = 0; c < nloc; ++c)
        bits |= (mask[edofs[(int64_t)rec.tet * nloc + canon_local(nloc, i, c)]] ? 1u : 0u) << c;
    rec.meta = (rec.meta & ~(0x3ffu << 4)) | (bits << 4);
    recs[k] = rec;
}

// Dirichlet columns of the non-Dirichlet rows (offsets within the row, ascending)
__global__ void dircol_count_kernel(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                    const uint8_t* __restrict__ mask, unsigned long long* __restrict__ cnt) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= n || mask[r]) return;
    unsigned long long c = 0;
    for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) c += mask[col[k]] ? 1 : 0;
    cnt[r] = c;
}
__global__ void dircol_fill_kernel(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                   const uint8_t* __restrict__ mask, const int64_t* __restrict__ cptr,
                                   uint16_t* __restrict__ coff) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= n || mask[r]) return;
    int64_t w = cptr[r];
    const int64_t b = rowptr[r];
    for (int64_t k = b; k < rowptr[r + 1]; ++k)
        if (mask[col[k]]) coff[w++] = (uint16_t)(k - b);
}

// vector template: rows (c, r) -> c*nds + r; columns [c'*nds + col_s] for c' = 0..2
__global__ void vec_rowptr_kernel(int64_t nds, int64_t nnz_s, const int64_t* __restrict__ rowptr_s,
                                  int64_t* __restrict__ rowptr) {
    const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx > 3 * nds) return;
    if (idx == 3 * nds) {
        rowptr[idx] = 9 * nnz_s;
        return;
    }
    const int64_t c = idx / nds, r = idx - c * nds;
    rowptr[idx] = c * 3 * nnz_s + 3 * rowptr_s[r];
}
__global__ void vec_col_kernel(int64_t nds, const int64_t* __restrict__ rowptr_s, const int32_t* __restrict__ col_s,
                               const int64_t* __restrict__ rowptr, int32_t* __restrict__ col) {
    const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= 3 * nds) return;
    const int64_t c = idx / nds, r = idx - c * nds;
    (void)c;
    const int64_t b = rowptr_s[r], len = rowptr_s[r + 1] - b;
    int32_t* out = col + rowptr[idx];
    for (int cc = 0; cc < 3; ++cc)
        for (int64_t k = 0; k < len; ++k) out[cc * len + k] = (int32_t)(cc * nds + col_s[b + k]);
}

int max_count(anigpu_ctx* h, const unsigned long long* cnt, int64_t n, unsigned long long* out) {
    size_t bytes = 0;
    unsigned long long* d_out = nullptr;
    ANI_CUDA(h, cudaMallocAsync((void**)&d_out, sizeof(unsigned long long), h->stream));
    ANI_CUDA(h, cub::DeviceReduce::Max(nullptr, bytes, cnt, d_out, n, h->stream));
    void* tmp = nullptr;
    ANI_CUDA(h, cudaMallocAsync(&tmp, bytes, h->stream));
    ANI_CUDA(h, cub::DeviceReduce::Max(tmp, bytes, cnt, d_out, n, h->stream));
    ANI_CUDA(h, cudaMemcpyAsync(out, d_out, sizeof(unsigned long long), cudaMemcpyDeviceToHost, h->stream));
    ANI_CUDA(h, cudaFreeAsync(tmp, h->stream));
    ANI_CUDA(h, cudaFreeAsync(d_out, h->stream));
    ANI_CUDA(h, cudaStreamSynchronize(h->stream));
    h->launches++;
    return ANIGPU_OK;
}

int check_status(anigpu_ctx* h, const char* what) {
    int st = 0;
    ANI_CUDA(h, cudaMemcpyAsync(&st, h->d_status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    ANI_CUDA(h, cudaStreamSynchronize(h->stream));
    if (st != 0) {
        ANI_CUDA(h, cudaMemsetAsync(h->d_status, 0, sizeof(int), h->stream));
        return set_err(h, st, std::string(what) + " failed");
    }
    return ANIGPU_OK;
}

#define RC(x)                \
    do {                     \
        int _rc = (x);       \
        if (_rc) return _rc; \
    } while (0)

int round_cap(unsigned long long m) {
    int c = 32;
    while ((unsigned long long)c < m) c <<= 1;
    return c;
}

}  // namespace

int scan_counts(anigpu_ctx* h, unsigned long long* cnt, int64_t n, int64_t* ptr) {
    // exclusive scan of n+1 entries (cnt[n] must be 0): ptr[n] = total
    size_t bytes = 0;
    ANI_CUDA(h, cub::DeviceScan::ExclusiveSum(nullptr, bytes, cnt, (unsigned long long*)ptr, n + 1, h->stream));
    void* tmp = nullptr;
    ANI_CUDA(h, cudaMallocAsync(&tmp, bytes, h->stream));
    ANI_CUDA(h, cub::DeviceScan::ExclusiveSum(tmp, bytes, cnt, (unsigned long long*)ptr, n + 1, h->stream));
    ANI_CUDA(h, cudaFreeAsync(tmp, h->stream));
    h->launches++;
    return ANIGPU_OK;
}

int setup_orient(anigpu_ctx* h) {
    bad_index_kernel<<<grid_for(h->nt * 4, 256), 256, 0, h->stream>>>(h->nt * 4, h->tets, h->nv, h->d_status);
    ANI_LAUNCHED(h);
    RC(check_status(h, "tet vertex index out of range"));
    orient_kernel<<<grid_for(h->nt, 256), 256, 0, h->stream>>>(h->nt, h->xyz, h->tets);
    ANI_LAUNCHED(h);
    return ANIGPU_OK;
}

int setup_problem(anigpu_ctx* h, int space) {
    if (space != ANIGPU_P1 && space != ANIGPU_P2 && space != ANIGPU_VEC3_P2)
        return set_err(h, ANIGPU_ERR_UNSUPPORTED, "problem space must be P1, P2 or VEC3_P2");
    if (h->nt <= 0) return set_err(h, ANIGPU_ERR_STATE, "no mesh uploaded");
    cudaStream_t s = h->stream;
    const int64_t nv = h->nv, nt = h->nt;
    // drop the aliases of a previous scalar setup before the scalar arrays are reallocated
    if (h->rowptr == h->rowptr_s) h->rowptr = nullptr;
    if (h->col == h->col_s) h->col = nullptr;
    if (h->rowptr) {
        cudaFree(h->rowptr);
        h->rowptr = nullptr;
    }
    if (h->col) {
        cudaFree(h->col);
        h->col = nullptr;
    }
    h->space = space;
    h->nloc_s = space == ANIGPU_P1 ? 4 : 10;
    h->ncomp = space == ANIGPU_VEC3_P2 ? 3 : 1;
    const int nloc = h->nloc_s;

    // vertex -> tet incidence
    unsigned long long* cnt = nullptr;
    int64_t nmax = std::max<int64_t>(nv, 1) + 1;
    ANI_CUDA(h, cudaMallocAsync((void**)&cnt, sizeof(unsigned long long) * (nmax + 8), s));
    int64_t* vptr = nullptr;
    int32_t* vlist = nullptr;
    ANI_CUDA(h, cudaMallocAsync((void**)&vptr, sizeof(int64_t) * (nv + 1), s));
    ANI_CUDA(h, cudaMallocAsync((void**)&vlist, sizeof(int32_t) * nt * 4, s));
    ANI_CUDA(h, cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * (nv + 1), s));
    count_kernel<<<grid_for(nt * 4, 256), 256, 0, s>>>(nt * 4, h->tets, cnt);
    ANI_LAUNCHED(h);
    unsigned long long maxdeg_v = 0;
    RC(max_count(h, cnt, nv, &maxdeg_v));
    RC(scan_counts(h, cnt, nv, vptr));
    ANI_CUDA(h, cudaMemcpyAsync(cnt, vptr, sizeof(int64_t) * nv, cudaMemcpyDeviceToDevice, s));
    {
        // fill with tet ids: keys are the 4 vertices of every tet, value i/4
        // (fill_kernel writes i; divide afterwards)
        fill_kernel<<<grid_for(nt * 4, 256), 256, 0, s>>>(nt * 4, h->tets, cnt, vlist);
        ANI_LAUNCHED(h);
    }

    // edges (needed for P2 numbering)
    h->ne = 0;
    if (space != ANIGPU_P1) {
        const int cap = round_cap(maxdeg_v * 3 + 1);
        if (cap > 4096) return set_err(h, ANIGPU_ERR_UNSUPPORTED, "vertex degree too large for edge numbering");
        unsigned long long* ecnt = nullptr;
        int64_t* eptr = nullptr;
        ANI_CUDA(h, cudaMallocAsync((void**)&ecnt, sizeof(unsigned long long) * (nv + 1), s));
        ANI_CUDA(h, cudaMallocAsync((void**)&eptr, sizeof(int64_t) * (nv + 1), s));
        ANI_CUDA(h, cudaMemsetAsync(ecnt, 0, sizeof(unsigned long long) * (nv + 1), s));
        // vlist holds i = 4*tet + local: convert to tet ids in place
        div4_kernel<<<grid_for(nt * 4, 256), 256, 0, s>>>(nt * 4, vlist);
        ANI_LAUNCHED(h);
        const size_t shm = sizeof(int32_t) * 2 * cap * kWarpsPerBlock;
        ANI_CUDA(h, cudaFuncSetAttribute(vertex_edges_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
        vertex_edges_kernel<<<grid_for(nv, kWarpsPerBlock), 32 * kWarpsPerBlock, shm, s>>>(
            0, nv, vptr, vlist, h->tets, cap, ecnt, nullptr, nullptr, h->d_status);
        ANI_LAUNCHED(h);
        RC(check_status(h, "edge numbering"));
        RC(scan_counts(h, ecnt, nv, eptr));
        int64_t ne = 0;
        ANI_CUDA(h, cudaMemcpyAsync(&ne, eptr + nv, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        ANI_CUDA(h, cudaStreamSynchronize(s));
        h->ne = ne;
        int32_t* nbr = nullptr;
        ANI_CUDA(h, cudaMallocAsync((void**)&nbr, sizeof(int32_t) * std::max<int64_t>(ne, 1), s));
        vertex_edges_kernel<<<grid_for(nv, kWarpsPerBlock), 32 * kWarpsPerBlock, shm, s>>>(
            1, nv, vptr, vlist, h->tets, cap, nullptr, eptr, nbr, h->d_status);
        ANI_LAUNCHED(h);
        RC(dev_alloc(h, &h->tet_edges, (size_t)nt * 6));
        tet_edges_kernel<<<grid_for(nt * 6, 256), 256, 0, s>>>(nt, h->tets, eptr, nbr, h->tet_edges);
        ANI_LAUNCHED(h);
        ANI_CUDA(h, cudaFreeAsync(nbr, s));
        ANI_CUDA(h, cudaFreeAsync(ecnt, s));
        ANI_CUDA(h, cudaFreeAsync(eptr, s));
    }
    ANI_CUDA(h, cudaFreeAsync(cnt, s));
    ANI_CUDA(h, cudaFreeAsync(vptr, s));
    ANI_CUDA(h, cudaFreeAsync(vlist, s));

    // element DOFs (scalar)
    h->nds = space == ANIGPU_P1 ? nv : nv + h->ne;
    h->ndof = h->nds * h->ncomp;
    if (h->ndof >= (int64_t)INT32_MAX) return set_err(h, ANIGPU_ERR_UNSUPPORTED, "more than 2^31 DOFs");
    RC(dev_alloc(h, &h->edofs, (size_t)nt * nloc));
    element_dofs_kernel<<<grid_for(nt * nloc, 256), 256, 0, s>>>(nt, nloc, nv, h->tets, h->tet_edges, h->edofs);
    ANI_LAUNCHED(h);

    // DOF -> (tet, local) incidence, sorted per row
    const int64_t nds = h->nds;
    unsigned long long* dcnt = nullptr;
    ANI_CUDA(h, cudaMallocAsync((void**)&dcnt, sizeof(unsigned long long) * (nds + 1), s));
    ANI_CUDA(h, cudaMemsetAsync(dcnt, 0, sizeof(unsigned long long) * (nds + 1), s));
    dof_count_kernel<<<grid_for(nt * nloc, 256), 256, 0, s>>>(nt * nloc, h->edofs, dcnt);
    ANI_LAUNCHED(h);
    unsigned long long maxdeg = 0;
    RC(max_count(h, dcnt, nds, &maxdeg));
    h->max_deg = (int)maxdeg;
    RC(dev_alloc(h, &h->inc_ptr, (size_t)nds + 1));
    RC(scan_counts(h, dcnt, nds, h->inc_ptr));
    ANI_CUDA(h, cudaMemcpyAsync(dcnt, h->inc_ptr, sizeof(int64_t) * nds, cudaMemcpyDeviceToDevice, s));
    int32_t* inc = nullptr;
    ANI_CUDA(h, cudaMallocAsync((void**)&inc, sizeof(int32_t) * nt * nloc, s));
    dof_fill_kernel<<<grid_for(nt * nloc, 256), 256, 0, s>>>(nt * nloc, nloc, h->edofs, dcnt, inc);
    ANI_LAUNCHED(h);
    {
        const int cap = round_cap(maxdeg);
        if (cap > 4096) return set_err(h, ANIGPU_ERR_UNSUPPORTED, "DOF degree too large");
        const size_t shm = sizeof(int32_t) * cap * kWarpsPerBlock;
        ANI_CUDA(h, cudaFuncSetAttribute(sort_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
        sort_rows_kernel<<<grid_for(nds, kWarpsPerBlock), 32 * kWarpsPerBlock, shm, s>>>(nds, h->inc_ptr, inc, cap,
                                                                                         h->d_status);
        ANI_LAUNCHED(h);
    }

    // scalar CSR template
    {
        const int cap = round_cap(maxdeg * nloc + 1);
        if (cap > 4096) return set_err(h, ANIGPU_ERR_UNSUPPORTED, "row candidate list too large");
        const size_t shm = sizeof(int32_t) * 2 * cap * kWarpsPerBlock;
        ANI_CUDA(h, cudaFuncSetAttribute(template_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
        ANI_CUDA(h, cudaMemsetAsync(dcnt, 0, sizeof(unsigned long long) * (nds + 1), s));
        template_rows_kernel<<<grid_for(nds, kWarpsPerBlock), 32 * kWarpsPerBlock, shm, s>>>(
            0, nds, nloc, h->inc_ptr, inc, h->edofs, cap, dcnt, nullptr, nullptr, h->d_status);
        ANI_LAUNCHED(h);
        RC(check_status(h, "CSR template"));
        unsigned long long maxlen = 0;
        RC(max_count(h, dcnt, nds, &maxlen));
        h->max_row_len_s = (int)maxlen;
        // row ranges: vertex rows [0, nv) and (P2) edge rows [nv, nds), each with its longest row
        h->row_range[0] = 0;
        h->row_range[1] = space == ANIGPU_P1 ? nds : nv;
        h->row_range[2] = nds;
        for (int rg = 0; rg < 2; ++rg) {
            const int64_t b = h->row_range[rg], e = h->row_range[rg + 1];
            unsigned long long m = 0;
            if (e > b) RC(max_count(h, dcnt + b, e - b, &m));
            h->row_range_cap[rg] = (int)m;
        }
        if (maxlen > 256) return set_err(h, ANIGPU_ERR_UNSUPPORTED, "scalar row longer than 256 entries");
        RC(dev_alloc(h, &h->rowptr_s, (size_t)nds + 1));
        RC(scan_counts(h, dcnt, nds, h->rowptr_s));
        ANI_CUDA(h, cudaMemcpyAsync(&h->nnz_s, h->rowptr_s + nds, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        ANI_CUDA(h, cudaStreamSynchronize(s));
        RC(dev_alloc(h, &h->col_s, (size_t)h->nnz_s));
        template_rows_kernel<<<grid_for(nds, kWarpsPerBlock), 32 * kWarpsPerBlock, shm, s>>>(
            1, nds, nloc, h->inc_ptr, inc, h->edofs, cap, nullptr, h->rowptr_s, h->col_s, h->d_status);
        ANI_LAUNCHED(h);
    }

    // scatter records
    // one zero record of padding: the row gather reads records in aligned pairs
    RC(dev_alloc(h, &h->recs, (size_t)nt * nloc + 1));
    ANI_CUDA(h, cudaMemsetAsync(h->recs + (size_t)nt * nloc, 0, sizeof(ScatterRec), s));
    records_kernel<<<grid_for(nt * nloc, 256), 256, 0, s>>>(nds, nloc, h->inc_ptr, inc, h->edofs, h->rowptr_s,
                                                            h->col_s, h->recs);
    ANI_LAUNCHED(h);
    ANI_CUDA(h, cudaFreeAsync(inc, s));
    ANI_CUDA(h, cudaFreeAsync(dcnt, s));

    // full template
    if (h->ncomp == 1) {
        h->rowptr = h->rowptr_s;
        h->col = h->col_s;
        h->nnz = h->nnz_s;
    } else {
        h->nnz = 9 * h->nnz_s;
        RC(dev_alloc(h, &h->rowptr, (size_t)h->ndof + 1));
        RC(dev_alloc(h, &h->col, (size_t)h->nnz));
        vec_rowptr_kernel<<<grid_for(3 * nds + 1, 256), 256, 0, s>>>(nds, h->nnz_s, h->rowptr_s, h->rowptr);
        ANI_LAUNCHED(h);
        vec_col_kernel<<<grid_for(3 * nds, 256), 256, 0, s>>>(nds, h->rowptr_s, h->col_s, h->rowptr, h->col);
        ANI_LAUNCHED(h);
    }
    RC(dev_alloc(h, &h->dir_mask, (size_t)h->ndof));
    RC(dev_alloc(h, &h->dir_bc, (size_t)h->ndof));
    ANI_CUDA(h, cudaMemsetAsync(h->dir_mask, 0, h->ndof, s));
    ANI_CUDA(h, cudaMemsetAsync(h->dir_bc, 0, sizeof(double) * h->ndof, s));
    h->has_dirichlet = false;
    h->bc_nonzero = false;
    RC(check_status(h, "problem setup"));
    RC(setup_row_layouts(h));
    return ANIGPU_OK;
}

namespace {
__global__ void dof_coords_kernel(int64_t nt, int nloc, int64_t nds, int ncomp, const double* __restrict__ xyz,
                                  const int32_t* __restrict__ tets, const int32_t* __restrict__ edofs,
                                  double* __restrict__ out) {
    const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= nt * nloc) return;
    const int64_t t = idx / nloc;
    const int j = (int)(idx - t * nloc);
    const int I[6] = {0, 0, 0, 1, 1, 2}, J[6] = {1, 2, 3, 2, 3, 3};
    double c[3];
    if (j < 4) {
        const int64_t v = tets[4 * t + j];
        for (int k = 0; k < 3; ++k) c[k] = xyz[3 * v + k];
    } else {
        const int64_t a = tets[4 * t + I[j - 4]], b = tets[4 * t + J[j - 4]];
        for (int k = 0; k < 3; ++k) c[k] = 0.5 * (xyz[3 * a + k] + xyz[3 * b + k]);
    }
    const int64_t d = edofs[idx];
    for (int comp = 0; comp < ncomp; ++comp)
        for (int k = 0; k < 3; ++k) out[3 * (comp * nds + d) + k] = c[k];  // same value from every tet
}
}  // namespace

namespace {
__global__ void split_coords_kernel(int64_t n, const double* __restrict__ x, float2* __restrict__ out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = x[i];
    const float hi = __double2float_rn(v);
    const float lo = __double2float_rn(v - (double)hi);
    out[i] = make_float2(hi, lo);
}
}  // namespace

int setup_coords_split(anigpu_ctx* h) {
    if (!h->xyz2) {
        int rc = dev_alloc(h, &h->xyz2, (size_t)h->nv * 3);
        if (rc) return rc;
    }
    split_coords_kernel<<<grid_for(h->nv * 3, 256), 256, 0, h->stream>>>(h->nv * 3, h->xyz, h->xyz2);
    ANI_LAUNCHED(h);
    return ANIGPU_OK;
}

int setup_dof_coords(anigpu_ctx* h, double* out) {
    const int64_t n = h->nt * h->nloc_s;
    dof_coords_kernel<<<grid_for(n, 256), 256, 0, h->stream>>>(h->nt, h->nloc_s, h->nds, h->ncomp, h->xyz, h->tets,
                                                             h->edofs, out);
    ANI_LAUNCHED(h);
    return ANIGPU_OK;
}

int setup_dirichlet_bits(anigpu_ctx* h) {
    // for vector spaces the record bits use the component-0 mask (all components of a
    // node are constrained together for the scalar-structured records); the per-component
    // mask itself is used by the assembly for rows.
    const int64_t nrec = h->nt * h->nloc_s;
    if (!is_general_space(h->space)) {  // the record bits of the fast P1/P2 gathers
        dirichlet_bits_kernel<<<grid_for(nrec, 256), 256, 0, h->stream>>>(nrec, h->nloc_s, h->edofs, h->dir_mask,
                                                                          h->recs);
        ANI_LAUNCHED(h);
    }
    if (!h->has_dirichlet) return ANIGPU_OK;
    // per non-Dirichlet row (of the full template: vector rows for FemVec), the offsets of its
    // Dirichlet columns: the assembly adds every element value and zeroes these entries at the end
    // (applyDir zeroes column k of every element matrix, so their sums are exactly zero)
    cudaStream_t s = h->stream;
    const int64_t n = h->ndof;
    unsigned long long* cnt = nullptr;
    ANI_CUDA(h, cudaMallocAsync((void**)&cnt, sizeof(unsigned long long) * (n + 1), s));
    ANI_CUDA(h, cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * (n + 1), s));
    dircol_count_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, h->rowptr, h->col, h->dir_mask, cnt);
    ANI_LAUNCHED(h);
    RC(dev_alloc(h, &h->dir_cptr, (size_t)n + 1));
    RC(scan_counts(h, cnt, n, h->dir_cptr));
    int64_t total = 0;
    ANI_CUDA(h, cudaMemcpyAsync(&total, h->dir_cptr + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    ANI_CUDA(h, cudaStreamSynchronize(s));
    ANI_CUDA(h, cudaFreeAsync(cnt, s));
    RC(dev_alloc(h, &h->dir_coff, (size_t)std::max<int64_t>(total, 1)));
    dircol_fill_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, h->rowptr, h->col, h->dir_mask, h->dir_cptr, h->dir_coff);
    ANI_LAUNCHED(h);
    return ANIGPU_OK;
}
