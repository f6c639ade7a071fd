// Global assembly for the element spaces beyond the fast P1/P2 path: P0, P3, CR1, B2, B4, ND0, RT0,
// with the reference's oriented-DOF rules (AssemblerT::fill_assemble_templates,
// anifem++/inmost_interface/assembler.inl:136-190: sign-encoded indices, index_encode :48-54).
//
// NATURAL numbering (VAR DIM ELEM_TYPE ELEM_ID DOF_ID, global_enumerator.h:392-404): node DOFs, then
// edge DOFs, then face DOFs, then cell DOFs; the DOFs of one entity consecutive.  Edge ids rank the
// (min, max) vertex pairs, face ids the sorted vertex triples (radix sorts on the device).  Local
// DOFs of a tet and their entities:
//   P0  cell;  P3  4 nodes, 2 per edge (local 4+2e+k: k = 0 near the edge's first local vertex),
//   1 per face (16+f);  CR1, RT0  1 per face;  B2, ND0  1 per edge;  B4  cell.
// Local edges e: (0,1),(0,2),(0,3),(1,2),(1,3),(2,3); local faces f: {0,1,2},{1,2,3},{0,2,3},{0,1,3}
// (the P3 face order, the CR1 faces opposite vertices 3,0,1,2, the RT0 IPF faces).
// Orientation (this library's convention; the reference's follows INMOST's element orientation,
// which is not available here): a global edge runs from its smaller to its larger vertex id; the
// two P3 DOFs of an edge are stored in that direction, so a tet whose local edge runs the other way
// swaps them; an ND0 DOF gets the sign + when its local edge (ip0, ip1) runs the global way; an RT0
// DOF gets + when the tet's outward normal of the face agrees with the global face normal
// (X_b - X_a) x (X_c - X_a) of the sorted vertex triple a < b < c.
// Element matrices and right-hand sides come from the fem3Dtet kernel (FP64); one warp per row
// walks the row's incidences in ascending tet order, its lanes over the element row's columns, and
// adds s_i s_j A_t(i, j) into the row's slots (binary search in the sorted row): deterministic, no
// atomics.  Dirichlet rows and columns
// follow the vector path: diagonal = number of incident tets, rhs = that number times the value,
// A(i,k) bc_k moved to the right-hand side of the other rows.
#include <cub/cub.cuh>

#include <algorithm>
#include <vector>

#include "anigpu_internal.h"

#define RC_(x)             \
    do {                   \
        int _r = (x);      \
        if (_r) return _r; \
    } while (0)

namespace {

constexpr int kNode = 0, kEdge = 1, kFace = 2, kCell = 3;

// DOFs per entity type (node, edge, face, cell) and local DOFs per tet
struct SpaceLayout {
    int per[4];
    int nloc;
};

bool layout_of(int space, SpaceLayout* L) {
    switch (space) {
        case ANIGPU_P0: *L = {{0, 0, 0, 1}, 1}; return true;
        case ANIGPU_P3: *L = {{1, 2, 1, 0}, 20}; return true;
        case ANIGPU_CR1: *L = {{0, 0, 1, 0}, 4}; return true;
        case ANIGPU_B2: *L = {{0, 1, 0, 0}, 6}; return true;
        case ANIGPU_B4: *L = {{0, 0, 0, 1}, 1}; return true;
        case ANIGPU_ND0: *L = {{0, 1, 0, 0}, 6}; return true;
        case ANIGPU_RT0: *L = {{0, 0, 1, 0}, 4}; return true;
    }
    return false;
}

// entity type, local entity index and DOF index within the entity of local DOF i
__device__ inline void local_dof(int space, int i, int& type, int& ent, int& k) {
    k = 0;
    switch (space) {
        case ANIGPU_P3:
            if (i < 4) { type = kNode; ent = i; }
            else if (i < 16) { type = kEdge; ent = (i - 4) / 2; k = (i - 4) % 2; }
            else { type = kFace; ent = i - 16; }
            return;
        case ANIGPU_CR1:
        case ANIGPU_RT0: type = kFace; ent = i; return;
        case ANIGPU_B2:
        case ANIGPU_ND0: type = kEdge; ent = i; return;
        default: type = kCell; ent = 0; return;  // P0, B4
    }
}

__constant__ int cEI[6] = {0, 0, 0, 1, 1, 2}, cEJ[6] = {1, 2, 3, 2, 3, 3};
__constant__ int cFV[4][3] = {{0, 1, 2}, {1, 2, 3}, {0, 2, 3}, {0, 1, 3}};
__constant__ int cFopp[4] = {3, 0, 1, 2};

// sort keys of the 6 edges / 4 faces of every tet: (min, max) and the sorted vertex triple
__global__ void edge_keys_kernel(int64_t nt, const int32_t* __restrict__ tets, uint64_t* __restrict__ key,
                                 int64_t* __restrict__ val) {
    const int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (id >= nt * 6) return;
    const int64_t t = id / 6;
    const int e = (int)(id - t * 6);
    const uint64_t a = (uint32_t)tets[4 * t + cEI[e]], b = (uint32_t)tets[4 * t + cEJ[e]];
    key[id] = a < b ? (a << 32) | b : (b << 32) | a;
    val[id] = id;
}

__global__ void face_keys_kernel(int64_t nt, uint64_t nv, const int32_t* __restrict__ tets, uint64_t* __restrict__ key,
                                 int64_t* __restrict__ val) {
    const int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (id >= nt * 4) return;
    const int64_t t = id / 4;
    const int f = (int)(id - t * 4);
    uint64_t v[3] = {(uint32_t)tets[4 * t + cFV[f][0]], (uint32_t)tets[4 * t + cFV[f][1]],
                     (uint32_t)tets[4 * t + cFV[f][2]]};
    if (v[0] > v[1]) { const uint64_t x = v[0]; v[0] = v[1]; v[1] = x; }
    if (v[1] > v[2]) { const uint64_t x = v[1]; v[1] = v[2]; v[2] = x; }
    if (v[0] > v[1]) { const uint64_t x = v[0]; v[0] = v[1]; v[1] = x; }
    key[id] = (v[0] * nv + v[1]) * nv + v[2];
    val[id] = id;
}

// first occurrence flags of sorted keys
__global__ void head_flags_kernel(int64_t n, const uint64_t* __restrict__ key, unsigned long long* __restrict__ flag) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) flag[i] = (i == 0 || key[i] != key[i - 1]) ? 1ull : 0ull;
}

// entity id of every (tet, local entity): the rank of its key (inclusive scan of the flags - 1)
__global__ void entity_ids_kernel(int64_t n, const int64_t* __restrict__ rank_excl, const unsigned long long* __restrict__ flag,
                                  const int64_t* __restrict__ val, int32_t* __restrict__ ent) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) ent[val[i]] = (int32_t)(rank_excl[i] + (int64_t)flag[i] - 1);
}

struct DofOffsets {
    int per[4];
    int64_t off[4];  // first global DOF of each entity type
};

// global DOF and orientation sign of every (tet, local DOF)
__global__ void gdof_kernel(int64_t nt, int space, int nloc, DofOffsets o, const double* __restrict__ xyz,
                            const int32_t* __restrict__ tets, const int32_t* __restrict__ tedge,
                            const int32_t* __restrict__ tface, int32_t* __restrict__ gdof, int8_t* __restrict__ sign) {
    const int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (id >= nt * nloc) return;
    const int64_t t = id / nloc;
    const int i = (int)(id - t * nloc);
    int type, ent, k;
    local_dof(space, i, type, ent, k);
    const int32_t* tv = tets + 4 * t;
    int64_t g = 0;
    int sg = 1;
    if (type == kNode) {
        g = o.off[kNode] + (int64_t)tv[ent] * o.per[kNode] + k;
    } else if (type == kEdge) {
        const int32_t I = tv[cEI[ent]], J = tv[cEJ[ent]];
        const int kk = (o.per[kEdge] == 2 && I > J) ? 1 - k : k;  // P3: the pair in the global direction
        g = o.off[kEdge] + (int64_t)tedge[6 * t + ent] * o.per[kEdge] + kk;
        if (space == ANIGPU_ND0) sg = I < J ? 1 : -1;
    } else if (type == kFace) {
        g = o.off[kFace] + (int64_t)tface[4 * t + ent] * o.per[kFace] + k;
        if (space == ANIGPU_RT0) {
            int32_t a = tv[cFV[ent][0]], b = tv[cFV[ent][1]], c = tv[cFV[ent][2]];
            if (a > b) { const int32_t x = a; a = b; b = x; }
            if (b > c) { const int32_t x = b; b = c; c = x; }
            if (a > b) { const int32_t x = a; a = b; b = x; }
            const double* Xa = xyz + 3 * (int64_t)a;
            const double* Xb = xyz + 3 * (int64_t)b;
            const double* Xc = xyz + 3 * (int64_t)c;
            const double u[3] = {Xb[0] - Xa[0], Xb[1] - Xa[1], Xb[2] - Xa[2]};
            const double w[3] = {Xc[0] - Xa[0], Xc[1] - Xa[1], Xc[2] - Xa[2]};
            const double n[3] = {u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2], u[0] * w[1] - u[1] * w[0]};
            const double* X0 = xyz + 3 * (int64_t)tv[cFV[ent][0]];
            const double* Xo = xyz + 3 * (int64_t)tv[cFopp[ent]];
            const double dot = n[0] * (X0[0] - Xo[0]) + n[1] * (X0[1] - Xo[1]) + n[2] * (X0[2] - Xo[2]);
            sg = dot > 0 ? 1 : -1;
        }
    } else {
        g = o.off[kCell] + t * o.per[kCell] + k;
    }
    gdof[id] = (int32_t)g;
    sign[id] = (int8_t)sg;
}

// (row, col) keys of every element matrix entry, and (dof, slot) keys of every incidence
__global__ void pair_keys_kernel(int64_t nt, int nloc, uint64_t ndof, const int32_t* __restrict__ gdof,
                                 uint64_t* __restrict__ key) {
    const int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t per = (int64_t)nloc * nloc;
    if (id >= nt * per) return;
    const int64_t t = id / per;
    const int r = (int)(id - t * per);
    const int i = r / nloc, j = r - (r / nloc) * nloc;
    key[id] = (uint64_t)gdof[nloc * t + i] * ndof + (uint64_t)gdof[nloc * t + j];
}

__global__ void inc_keys_kernel(int64_t n, const int32_t* __restrict__ gdof, uint64_t* __restrict__ key) {
    const int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (id < n) key[id] = ((uint64_t)(uint32_t)gdof[id] << 32) | (uint64_t)id;
}

// rows of unique sorted keys: counts, columns; incidences: counts, slot ids
__global__ void row_count_kernel(int64_t n, const uint64_t* __restrict__ key, uint64_t div, int shift,
                                 unsigned long long* __restrict__ cnt) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) atomicAdd(cnt + (shift ? (key[i] >> 32) : key[i] / div), 1ull);
}

__global__ void col_of_key_kernel(int64_t n, const uint64_t* __restrict__ key, uint64_t ndof, int32_t* __restrict__ col) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) col[i] = (int32_t)(key[i] % ndof);
}

__global__ void low_word_kernel(int64_t n, const uint64_t* __restrict__ key, int32_t* __restrict__ out) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = (int32_t)(key[i] & 0xffffffffull);
}

// coordinates of every DOF: nodes, P3 edge points at 1/3 and 2/3 in the global direction, other
// edge DOFs at the midpoint, face centroids, cell centroids
__global__ void gdof_coords_kernel(int64_t nt, int space, int nloc, const double* __restrict__ xyz,
                                   const int32_t* __restrict__ tets, const int32_t* __restrict__ gdof,
                                   double* __restrict__ out) {
    const int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (id >= nt * nloc) return;
    const int64_t t = id / nloc;
    const int i = (int)(id - t * nloc);
    int type, ent, k;
    local_dof(space, i, type, ent, k);
    const int32_t* tv = tets + 4 * t;
    double c[3] = {0, 0, 0};
    if (type == kNode) {
        for (int d = 0; d < 3; ++d) c[d] = xyz[3 * (int64_t)tv[ent] + d];
    } else if (type == kEdge) {
        const double* XI = xyz + 3 * (int64_t)tv[cEI[ent]];
        const double* XJ = xyz + 3 * (int64_t)tv[cEJ[ent]];
        const double wI = space == ANIGPU_P3 ? (k == 0 ? 2.0 / 3.0 : 1.0 / 3.0) : 0.5;
        for (int d = 0; d < 3; ++d) c[d] = wI * XI[d] + (1.0 - wI) * XJ[d];
    } else if (type == kFace) {
        for (int v = 0; v < 3; ++v)
            for (int d = 0; d < 3; ++d) c[d] += xyz[3 * (int64_t)tv[cFV[ent][v]] + d] / 3.0;
    } else {
        for (int v = 0; v < 4; ++v)
            for (int d = 0; d < 3; ++d) c[d] += xyz[3 * (int64_t)tv[v] + d] / 4.0;
    }
    double* o = out + 3 * (int64_t)gdof[id];
    for (int d = 0; d < 3; ++d) o[d] = c[d];
}

// per-tet vertex coordinates for the element kernel
__global__ void tet_xy_kernel(int64_t nt, const double* __restrict__ xyz, const int32_t* __restrict__ tets,
                              double* __restrict__ XY) {
    const int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (id >= nt * 12) return;
    const int64_t t = id / 12;
    const int r = (int)(id - t * 12);
    XY[id] = xyz[3 * (int64_t)tets[4 * t + r / 3] + r % 3];
}

}  // namespace

namespace {

struct GenWs {
    int space = -1, nloc = 0;
    DofOffsets o{};
    int64_t nf = 0;                 // faces
    int32_t* tedge = nullptr;       // [nt][6]
    int32_t* tface = nullptr;       // [nt][4]
    int8_t* sign = nullptr;         // [nt][nloc]
    double* XY = nullptr;           // [nt][12]
    int64_t* inc_ptr = nullptr;     // [ndof + 1]
    int32_t* inc = nullptr;         // [nt * nloc] slots t*nloc + i, ascending per DOF
    double* A = nullptr;            // element matrices [nt][nloc][nloc]
    double* F = nullptr;            // element right-hand sides [nt][nloc]
};

GenWs* gws(anigpu_ctx* h) { return static_cast<GenWs*>(h->gen_ws); }

// sort the keys (with their slot values when val_in is given) and number the distinct keys:
// ent[val] = rank of the key; returns the number of distinct keys
int number_keys(anigpu_ctx* h, int64_t n, uint64_t* key_in, int64_t* val_in, int32_t* ent, int64_t* count) {
    cudaStream_t s = h->stream;
    uint64_t* key = nullptr;
    int64_t* val = nullptr;
    ANI_CUDA(h, cudaMallocAsync((void**)&key, sizeof(uint64_t) * n, s));
    ANI_CUDA(h, cudaMallocAsync((void**)&val, sizeof(int64_t) * n, s));
    size_t bytes = 0;
    ANI_CUDA(h, cub::DeviceRadixSort::SortPairs(nullptr, bytes, key_in, key, val_in, val, (int)n, 0, 64, s));
    void* tmp = nullptr;
    ANI_CUDA(h, cudaMallocAsync(&tmp, bytes, s));
    ANI_CUDA(h, cub::DeviceRadixSort::SortPairs(tmp, bytes, key_in, key, val_in, val, (int)n, 0, 64, s));
    ANI_CUDA(h, cudaFreeAsync(tmp, s));
    h->launches++;
    unsigned long long* flag = nullptr;
    int64_t* rank = nullptr;
    ANI_CUDA(h, cudaMallocAsync((void**)&flag, sizeof(unsigned long long) * (n + 1), s));
    ANI_CUDA(h, cudaMallocAsync((void**)&rank, sizeof(int64_t) * (n + 1), s));
    ANI_CUDA(h, cudaMemsetAsync(flag + n, 0, sizeof(unsigned long long), s));
    head_flags_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, key, flag);
    ANI_LAUNCHED(h);
    RC_(scan_counts(h, flag, n, rank));
    entity_ids_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, rank, flag, val, ent);
    ANI_LAUNCHED(h);
    ANI_CUDA(h, cudaMemcpyAsync(count, rank + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    ANI_CUDA(h, cudaStreamSynchronize(s));
    ANI_CUDA(h, cudaFreeAsync(flag, s));
    ANI_CUDA(h, cudaFreeAsync(rank, s));
    ANI_CUDA(h, cudaFreeAsync(key, s));
    ANI_CUDA(h, cudaFreeAsync(val, s));
    return ANIGPU_OK;
}

// CSR rows from sorted keys: counts per row (key / div, or key >> 32 when shift), exclusive scan
int rows_of_keys(anigpu_ctx* h, int64_t n, const uint64_t* key, int64_t nrows, uint64_t div, int shift, int64_t* ptr) {
    cudaStream_t s = h->stream;
    unsigned long long* cnt = nullptr;
    ANI_CUDA(h, cudaMallocAsync((void**)&cnt, sizeof(unsigned long long) * (nrows + 1), s));
    ANI_CUDA(h, cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * (nrows + 1), s));
    if (n > 0) {
        row_count_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, key, div, shift, cnt);
        ANI_LAUNCHED(h);
    }
    RC_(scan_counts(h, cnt, nrows, ptr));
    ANI_CUDA(h, cudaFreeAsync(cnt, s));
    return ANIGPU_OK;
}

}  // namespace

void free_general(anigpu_ctx* h) {
    GenWs* w = gws(h);
    if (!w) return;
    void* ptrs[] = {w->tedge, w->tface, w->sign, w->XY, w->inc_ptr, w->inc, w->A, w->F};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete w;
    h->gen_ws = nullptr;
}

bool is_general_space(int space) {
    SpaceLayout L;
    return layout_of(space, &L);
}

int general_setup(anigpu_ctx* h, int space) {
    SpaceLayout L;
    if (!layout_of(space, &L)) return set_err(h, ANIGPU_ERR_UNSUPPORTED, "not a general-path space");
    if (h->nt <= 0) return set_err(h, ANIGPU_ERR_STATE, "no mesh uploaded");
    const int64_t nt = h->nt, nv = h->nv, nloc = L.nloc;
    if ((double)nt * nloc * nloc >= 2.0e9) return set_err(h, ANIGPU_ERR_UNSUPPORTED, "mesh too large for the general path");
    cudaStream_t s = h->stream;
    free_general(h);
    GenWs* w = new GenWs();
    h->gen_ws = w;
    w->space = space;
    w->nloc = (int)nloc;
    // drop the aliases of a previous scalar setup before the template arrays are reallocated
    if (h->rowptr == h->rowptr_s) h->rowptr = nullptr;
    if (h->col == h->col_s) h->col = nullptr;
    if (h->rowptr) cudaFree(h->rowptr);
    if (h->col) cudaFree(h->col);
    h->rowptr = nullptr;
    h->col = nullptr;
    // topology: edges and faces numbered by their sorted vertex keys
    int64_t ne = 0, nf = 0;
    RC_(dev_alloc(h, &w->tedge, (size_t)nt * 6));
    RC_(dev_alloc(h, &w->tface, (size_t)nt * 4));
    {
        uint64_t* key = nullptr;
        int64_t* val = nullptr;
        ANI_CUDA(h, cudaMallocAsync((void**)&key, sizeof(uint64_t) * nt * 6, s));
        ANI_CUDA(h, cudaMallocAsync((void**)&val, sizeof(int64_t) * nt * 6, s));
        edge_keys_kernel<<<grid_for(nt * 6, 256), 256, 0, s>>>(nt, h->tets, key, val);
        ANI_LAUNCHED(h);
        RC_(number_keys(h, nt * 6, key, val, w->tedge, &ne));
        face_keys_kernel<<<grid_for(nt * 4, 256), 256, 0, s>>>(nt, (uint64_t)nv, h->tets, key, val);
        ANI_LAUNCHED(h);
        RC_(number_keys(h, nt * 4, key, val, w->tface, &nf));
        ANI_CUDA(h, cudaFreeAsync(key, s));
        ANI_CUDA(h, cudaFreeAsync(val, s));
    }
    w->nf = nf;
    DofOffsets o;
    for (int k = 0; k < 4; ++k) o.per[k] = L.per[k];
    o.off[kNode] = 0;
    o.off[kEdge] = nv * L.per[kNode];
    o.off[kFace] = o.off[kEdge] + ne * L.per[kEdge];
    o.off[kCell] = o.off[kFace] + nf * L.per[kFace];
    const int64_t ndof = o.off[kCell] + nt * L.per[kCell];
    if (ndof >= (int64_t)INT32_MAX) return set_err(h, ANIGPU_ERR_UNSUPPORTED, "more than 2^31 DOFs");
    w->o = o;
    h->space = space;
    h->nloc_s = (int)nloc;
    h->ncomp = 1;
    h->ne = ne;
    h->nds = ndof;
    h->ndof = ndof;
    // global DOFs with orientation
    RC_(dev_alloc(h, &h->edofs, (size_t)nt * nloc));
    RC_(dev_alloc(h, &w->sign, (size_t)nt * nloc));
    gdof_kernel<<<grid_for(nt * nloc, 256), 256, 0, s>>>(nt, space, (int)nloc, o, h->xyz, h->tets, w->tedge, w->tface,
                                                         h->edofs, w->sign);
    ANI_LAUNCHED(h);
    // template: sorted unique (row, col) keys of every element matrix entry
    {
        const int64_t n = nt * nloc * nloc;
        uint64_t *key = nullptr, *sorted = nullptr, *uniq = nullptr;
        int* nsel = nullptr;
        ANI_CUDA(h, cudaMallocAsync((void**)&key, sizeof(uint64_t) * n, s));
        ANI_CUDA(h, cudaMallocAsync((void**)&sorted, sizeof(uint64_t) * n, s));
        ANI_CUDA(h, cudaMallocAsync((void**)&uniq, sizeof(uint64_t) * n, s));
        ANI_CUDA(h, cudaMallocAsync((void**)&nsel, sizeof(int), s));
        pair_keys_kernel<<<grid_for(n, 256), 256, 0, s>>>(nt, (int)nloc, (uint64_t)ndof, h->edofs, key);
        ANI_LAUNCHED(h);
        size_t b1 = 0, b2 = 0;
        ANI_CUDA(h, cub::DeviceRadixSort::SortKeys(nullptr, b1, key, sorted, (int)n, 0, 64, s));
        ANI_CUDA(h, cub::DeviceSelect::Unique(nullptr, b2, sorted, uniq, nsel, (int)n, s));
        void* tmp = nullptr;
        ANI_CUDA(h, cudaMallocAsync(&tmp, std::max(b1, b2), s));
        ANI_CUDA(h, cub::DeviceRadixSort::SortKeys(tmp, b1, key, sorted, (int)n, 0, 64, s));
        ANI_CUDA(h, cub::DeviceSelect::Unique(tmp, b2, sorted, uniq, nsel, (int)n, s));
        h->launches += 2;
        int hsel = 0;
        ANI_CUDA(h, cudaMemcpyAsync(&hsel, nsel, sizeof(int), cudaMemcpyDeviceToHost, s));
        ANI_CUDA(h, cudaStreamSynchronize(s));
        const int64_t nnz = hsel;
        RC_(dev_alloc(h, &h->rowptr_s, (size_t)ndof + 1));
        RC_(dev_alloc(h, &h->col_s, (size_t)nnz));
        RC_(rows_of_keys(h, nnz, uniq, ndof, (uint64_t)ndof, 0, h->rowptr_s));
        col_of_key_kernel<<<grid_for(nnz, 256), 256, 0, s>>>(nnz, uniq, (uint64_t)ndof, h->col_s);
        ANI_LAUNCHED(h);
        h->nnz_s = nnz;
        h->nnz = nnz;
        h->rowptr = h->rowptr_s;
        h->col = h->col_s;
        // incidence: (dof, slot) keys sorted; slots ascending = tets ascending per DOF
        const int64_t m = nt * nloc;
        inc_keys_kernel<<<grid_for(m, 256), 256, 0, s>>>(m, h->edofs, key);
        ANI_LAUNCHED(h);
        size_t b3 = 0;
        ANI_CUDA(h, cub::DeviceRadixSort::SortKeys(nullptr, b3, key, sorted, (int)m, 0, 64, s));
        if (b3 > std::max(b1, b2)) {
            ANI_CUDA(h, cudaFreeAsync(tmp, s));
            ANI_CUDA(h, cudaMallocAsync(&tmp, b3, s));
        }
        ANI_CUDA(h, cub::DeviceRadixSort::SortKeys(tmp, b3, key, sorted, (int)m, 0, 64, s));
        h->launches++;
        RC_(dev_alloc(h, &w->inc_ptr, (size_t)ndof + 1));
        RC_(dev_alloc(h, &w->inc, (size_t)m));
        RC_(rows_of_keys(h, m, sorted, ndof, 0, 1, w->inc_ptr));
        low_word_kernel<<<grid_for(m, 256), 256, 0, s>>>(m, sorted, w->inc);
        ANI_LAUNCHED(h);
        ANI_CUDA(h, cudaFreeAsync(tmp, s));
        ANI_CUDA(h, cudaFreeAsync(key, s));
        ANI_CUDA(h, cudaFreeAsync(sorted, s));
        ANI_CUDA(h, cudaFreeAsync(uniq, s));
        ANI_CUDA(h, cudaFreeAsync(nsel, s));
    }
    RC_(dev_alloc(h, &w->XY, (size_t)nt * 12));
    tet_xy_kernel<<<grid_for(nt * 12, 256), 256, 0, s>>>(nt, h->xyz, h->tets, w->XY);
    ANI_LAUNCHED(h);
    RC_(dev_alloc(h, &h->dir_mask, (size_t)ndof));
    RC_(dev_alloc(h, &h->dir_bc, (size_t)ndof));
    ANI_CUDA(h, cudaMemsetAsync(h->dir_mask, 0, ndof, s));
    ANI_CUDA(h, cudaMemsetAsync(h->dir_bc, 0, sizeof(double) * ndof, s));
    h->has_dirichlet = false;
    h->bc_nonzero = false;
    ANI_CUDA(h, cudaStreamSynchronize(s));
    return ANIGPU_OK;
}

int general_dof_coords(anigpu_ctx* h, double* out) {
    GenWs* w = gws(h);
    if (!w) return set_err(h, ANIGPU_ERR_STATE, "general problem not set up");
    gdof_coords_kernel<<<grid_for(h->nt * w->nloc, 256), 256, 0, h->stream>>>(h->nt, w->space, w->nloc, h->xyz, h->tets,
                                                                              h->edofs, out);
    ANI_LAUNCHED(h);
    return ANIGPU_OK;
}

const int8_t* general_signs(anigpu_ctx* h) { return gws(h) ? gws(h)->sign : nullptr; }

bool general_dof_blocks(anigpu_ctx* h, int per[4], int64_t off[5]) {
    GenWs* w = gws(h);
    if (!w) return false;
    for (int T = 0; T < 4; ++T) {
        per[T] = w->o.per[T];
        off[T] = w->o.off[T];
    }
    off[4] = h->ndof;
    return true;
}

namespace {

// per row: the row's slots zeroed, then for every incidence (ascending tets) the signed element
// row added column by column (binary search of the column in the sorted row); Dirichlet rows and
// columns as in the other assembly paths
__global__ void general_gather_kernel(int64_t ndof, int nloc, const int64_t* __restrict__ rowptr,
                                      const int32_t* __restrict__ col, const int64_t* __restrict__ inc_ptr,
                                      const int32_t* __restrict__ inc, const int32_t* __restrict__ gdof,
                                      const int8_t* __restrict__ sign, const double* __restrict__ A,
                                      const double* __restrict__ F, const uint8_t* __restrict__ dir_mask,
                                      const double* __restrict__ dir_bc, int dir, int bcnz, double* __restrict__ vals,
                                      double* __restrict__ rhs, int* __restrict__ status) {
    // one warp per row: incidences in ascending order, lanes over the element row's columns (distinct
    // columns within one incidence), so every entry sums its contributions in incidence order
    const int lane = threadIdx.x & 31;
    const int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (r >= ndof) return;
    const int64_t b = rowptr[r], e = rowptr[r + 1];
    for (int64_t k = b + lane; k < e; k += 32) vals[k] = 0.0;
    __syncwarp();
    double f = 0.0, fd = 0.0;
    const int64_t q0 = inc_ptr[r], q1 = inc_ptr[r + 1];
    const bool isdir = dir && dir_mask[r];
    if (!isdir) {
        for (int64_t q = q0; q < q1; ++q) {
            const int64_t slot = inc[q];
            const int64_t t = slot / nloc;
            const int i = (int)(slot - t * nloc);
            const double si = sign[slot];
            const double* At = A + (size_t)nloc * nloc * t;
            for (int j = lane; j < nloc; j += 32) {
                const int32_t c = gdof[(int64_t)nloc * t + j];
                int64_t lo = b, hi = e;
                while (lo < hi) {
                    const int64_t mid = (lo + hi) >> 1;
                    if (col[mid] < c) lo = mid + 1;
                    else hi = mid;
                }
                vals[lo] += si * (double)sign[(int64_t)nloc * t + j] * At[i + nloc * j];
            }
            __syncwarp();
            if (F) f += si * F[(int64_t)nloc * t + i];
        }
        if (dir) {
            for (int64_t k = b + lane; k < e; k += 32)
                if (dir_mask[col[k]]) {
                    if (bcnz) fd += vals[k] * dir_bc[col[k]];
                    vals[k] = 0.0;
                }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) fd += __shfl_xor_sync(0xffffffffu, fd, o);
            f -= fd;
        }
    } else {
        for (int64_t k = b + lane; k < e; k += 32)
            if (col[k] == r) vals[k] = (double)(q1 - q0);
        for (int64_t q = q0; q < q1; ++q) f += bcnz ? dir_bc[r] : 0.0;
    }
    __syncwarp();
    bool bad = !isfinite(f);
    for (int64_t k = b + lane; k < e; k += 32) bad |= !isfinite(vals[k]);
    if (__any_sync(0xffffffffu, bad) && lane == 0) atomicExch(status, ANIGPU_ERR_NONFINITE);
    if (rhs && lane == 0) rhs[r] = f;
}

}  // namespace

int general_assemble(anigpu_ctx* h, int opA, int opB, int kind, const double* D, int rhs_kind, const double* Fdata,
                     int order, double* vals, double* rhs) {
    GenWs* w = gws(h);
    if (!w || h->space != w->space) return set_err(h, ANIGPU_ERR_STATE, "general problem not set up");
    if (opA / 10 != w->space || opB / 10 != w->space)
        return set_err(h, ANIGPU_ERR_ARG, "operators must act on the problem's space");
    if (!vals) return set_err(h, ANIGPU_ERR_ARG, "NULL values");
    const int64_t nt = h->nt, nloc = w->nloc;
    RC_(dev_alloc(h, &w->A, (size_t)nt * nloc * nloc));
    RC_(launch_fem3dtet(h, opA, opB, kind, order, ANIGPU_F64, nt, w->XY, D, w->A));
    const double* F = nullptr;
    if (rhs) {
        RC_(dev_alloc(h, &w->F, (size_t)nt * nloc));
        RC_(launch_fem3dtet(h, ANIGPU_OP(ANIGPU_P0, ANIGPU_IDEN), ANIGPU_OP(w->space, ANIGPU_IDEN), rhs_kind, order,
                            ANIGPU_F64, nt, w->XY, Fdata, w->F));
        F = w->F;
    }
    return general_gather(h, w->A, F, vals, rhs);
}

// the signed row gather of element matrices A [nt][nloc][nloc] (column-major per tet, the layout of
// fem3Dtet) and element right-hand sides F [nt][nloc] (or NULL) into the template
int general_gather(anigpu_ctx* h, const double* A, const double* F, double* vals, double* rhs) {
    GenWs* w = gws(h);
    if (!w || h->space != w->space) return set_err(h, ANIGPU_ERR_STATE, "general problem not set up");
    if (!A || !vals) return set_err(h, ANIGPU_ERR_ARG, "NULL element matrices or values");
    general_gather_kernel<<<grid_for(h->ndof * 32, 256), 256, 0, h->stream>>>(
        h->ndof, w->nloc, h->rowptr, h->col, w->inc_ptr, w->inc, h->edofs, w->sign, A, F, h->dir_mask, h->dir_bc,
        h->has_dirichlet ? 1 : 0, h->bc_nonzero ? 1 : 0, vals, rhs, h->d_status);
    ANI_LAUNCHED(h);
    return ANIGPU_OK;
}
