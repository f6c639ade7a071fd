// Global enumerations other than NATURAL (GlobEnumeration::ASSEMBLING_TYPE,
// anifem++/inmost_interface/global_enumerator.h:392-404): the assembled system in the numbering
// the caller asks for.
//
// Every enumeration orders the DOFs lexicographically by a permutation of the key
// (VAR, DIM, ELEM_TYPE, ELEM_ID, DOF_ID).  With one variable and one DOF per node (P1) or per
// node and edge (P2, vector P2) the six types give three numberings of DOF (component c, scalar
// DOF s), s < nv a node, s >= nv an edge:
//   NATURAL                            c*nds + s                       (VAR DIM ELEM_TYPE ELEM_ID DOF_ID)
//   ANITYPE, BYELEMTYPE                s < nv: c*nv + s;  else 3nv + c*ne + (s - nv)   (ELEM_TYPE VAR DIM ..)
//   MINIBLOCKS, DIMUNION, ETDIMBLOCKS  ncomp*s + c                     (ELEM_TYPE/VAR .. ELEM_ID DOF_ID DIM)
// (scalar spaces: all three are the identity).  The template in the new numbering has the rows
// permuted and each row's columns mapped and sorted; the new position of every template slot
// follows in closed form from the component-major block structure of the NATURAL vector row
// (block d holds the scalar row's columns t_0 < t_1 < ... shifted by d*nds):
//   MINIBLOCKS: slot (d, j) -> 3j + d
//   ANITYPE:    slot (d, j) -> j < Ln ? d*Ln + j : 3Ln + d*Le + (j - Ln)   (Ln node columns, Le edge columns)
// so that a renumbered assembly is one gather of the values.
//
// General-path spaces (one scalar variable; DOFs on nodes, edges, faces or cells, the DOFs of an
// entity consecutive in NATURAL): only ANITYPE, whose key puts DOF_ID before ELEM_ID, differs from
// NATURAL, and only where an entity holds several DOFs (P3: two per edge).  DOF k of entity E in the
// block of entity type T goes to off_T + k*count_T + E.  Every entity in a row brings all its DOFs,
// so the row's columns of type T are m_T entities x per_T DOFs starting at slot b_T, and slot
// b_T + p*per_T + k moves to b_T + k*m_T + p.
#include <algorithm>

#include "anigpu_internal.h"

#define RC_(x)             \
    do {                   \
        int _r = (x);      \
        if (_r) return _r; \
    } while (0)

namespace {

struct EnumWs {
    int type = ANIGPU_ENUM_NATURAL;
    int64_t n = 0, nnz = 0;
    int64_t* perm = nullptr;     // [ndof] new index of each NATURAL DOF
    int64_t* rowptr = nullptr;   // [ndof + 1] new template
    int32_t* col = nullptr;      // [nnz]
    int64_t* slot = nullptr;     // [nnz] new position of each NATURAL slot
};

EnumWs* ews(anigpu_ctx* h) { return static_cast<EnumWs*>(h->enum_ws); }

int kind_of(int type) {  // 0 identity, 1 type-major, 2 interleaved
    switch (type) {
        case ANIGPU_ENUM_ANITYPE:
        case ANIGPU_ENUM_BYELEMTYPE: return 1;
        case ANIGPU_ENUM_MINIBLOCKS:
        case ANIGPU_ENUM_DIMUNION:
        case ANIGPU_ENUM_ETDIMBLOCKS: return 2;
    }
    return 0;
}

__device__ __forceinline__ int64_t new_index(int kind, int64_t R, int64_t nds, int64_t nv, int ncomp) {
    const int64_t c = R / nds, s = R - c * nds;
    if (kind == 2) return ncomp * s + c;
    if (kind == 1) return s < nv ? c * nv + s : ncomp * nv + c * (nds - nv) + (s - nv);
    return R;
}

__global__ void perm_kernel(int64_t n, int kind, int64_t nds, int64_t nv, int ncomp, int64_t* __restrict__ perm,
                            const int64_t* __restrict__ rowptr, unsigned long long* __restrict__ len_new) {
    const int64_t R = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (R >= n) return;
    const int64_t P = new_index(kind, R, nds, nv, ncomp);
    perm[R] = P;
    len_new[P] = (unsigned long long)(rowptr[R + 1] - rowptr[R]);
}

// one block per NATURAL row: every slot's new column and new position
__global__ void slot_kernel(int64_t n, int kind, int64_t nds, int64_t nv, int ncomp, const int64_t* __restrict__ rowptr,
                            const int32_t* __restrict__ col, const int64_t* __restrict__ rowptr_s,
                            const int32_t* __restrict__ col_s, const int64_t* __restrict__ perm,
                            const int64_t* __restrict__ rowptr_new, int32_t* __restrict__ col_new,
                            int64_t* __restrict__ slot) {
    const int64_t R = blockIdx.x;  // one block per row (grid-stride)
    for (int64_t row = R; row < n; row += gridDim.x) {
        const int64_t s = row % nds;
        const int64_t b = rowptr[row], len = rowptr[row + 1] - b;
        const int64_t L = len / ncomp;  // scalar row length
        int64_t Ln = 0;
        if (kind == 1) {  // node columns of the scalar row: a prefix (columns sorted, nodes first)
            const int64_t bs = rowptr_s[s];
            int64_t lo = 0, hi = L;
            while (lo < hi) {
                const int64_t mid = (lo + hi) / 2;
                if (col_s[bs + mid] < nv) lo = mid + 1;
                else hi = mid;
            }
            Ln = lo;
        }
        const int64_t nb = rowptr_new[perm[row]];
        for (int64_t k = threadIdx.x; k < len; k += blockDim.x) {
            const int64_t d = k / L, j = k - d * L;
            int64_t pos;
            if (kind == 2) pos = ncomp * j + d;
            else if (kind == 1) pos = j < Ln ? d * Ln + j : ncomp * Ln + d * (L - Ln) + (j - Ln);
            else pos = k;
            slot[b + k] = nb + pos;
            col_new[nb + pos] = (int32_t)perm[col[b + k]];
        }
    }
}

struct GenBlocks {
    int per[4];
    int64_t off[5];  // off[4] = ndof
};

__device__ __forceinline__ int gen_type(const GenBlocks& g, int64_t s) {
    int T = 0;
#pragma unroll
    for (int q = 1; q < 4; ++q)
        if (s >= g.off[q] && g.off[q] < g.off[q + 1]) T = q;
    return T;
}

__device__ __forceinline__ int64_t gen_new_index(const GenBlocks& g, int anitype, int64_t s) {
    if (!anitype) return s;
    const int T = gen_type(g, s);
    const int p = g.per[T];
    if (p <= 1) return s;
    const int64_t cnt = (g.off[T + 1] - g.off[T]) / p, r = s - g.off[T];
    return g.off[T] + (r % p) * cnt + r / p;
}

__global__ void gen_perm_kernel(int64_t n, GenBlocks g, int anitype, int64_t* __restrict__ perm,
                                const int64_t* __restrict__ rowptr, unsigned long long* __restrict__ len_new) {
    const int64_t R = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (R >= n) return;
    const int64_t P = gen_new_index(g, anitype, R);
    perm[R] = P;
    len_new[P] = (unsigned long long)(rowptr[R + 1] - rowptr[R]);
}

// one block per NATURAL row (grid-stride): the row's type boundaries by binary search, then every
// slot's new position and column
__global__ void gen_slot_kernel(int64_t n, GenBlocks g, int anitype, const int64_t* __restrict__ rowptr,
                                const int32_t* __restrict__ col, const int64_t* __restrict__ perm,
                                const int64_t* __restrict__ rowptr_new, int32_t* __restrict__ col_new,
                                int64_t* __restrict__ slot) {
    for (int64_t row = blockIdx.x; row < n; row += gridDim.x) {
        const int64_t b = rowptr[row], len = rowptr[row + 1] - b;
        int64_t pos[5];
#pragma unroll
        for (int T = 0; T < 5; ++T) {
            int64_t lo = 0, hi = len;
            while (lo < hi) {
                const int64_t mid = (lo + hi) / 2;
                if (col[b + mid] < g.off[T]) lo = mid + 1;
                else hi = mid;
            }
            pos[T] = lo;
        }
        const int64_t nb = rowptr_new[perm[row]];
        for (int64_t k = threadIdx.x; k < len; k += blockDim.x) {
            int T = 0;
#pragma unroll
            for (int q = 1; q < 4; ++q)
                if (k >= pos[q]) T = q;
            const int p = g.per[T];
            int64_t j = k;
            if (anitype && p > 1) {
                const int64_t m = (pos[T + 1] - pos[T]) / p, r = k - pos[T];
                j = pos[T] + (r % p) * m + r / p;
            }
            slot[b + k] = nb + j;
            col_new[nb + j] = (int32_t)perm[col[b + k]];
        }
    }
}

template <typename Real>
__global__ void gather_vals_kernel(int64_t nnz, const int64_t* __restrict__ slot, const Real* __restrict__ in,
                                   Real* __restrict__ out) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k < nnz) out[slot[k]] = in[k];
}

__global__ void permute_vec_kernel(int64_t n, const int64_t* __restrict__ perm, const double* __restrict__ in,
                                   double* __restrict__ out, int to_natural) {
    const int64_t R = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (R >= n) return;
    if (to_natural) out[R] = in[perm[R]];
    else out[perm[R]] = in[R];
}

}  // namespace

void free_enum(anigpu_ctx* h) {
    EnumWs* w = ews(h);
    if (!w) return;
    void* ptrs[] = {w->perm, w->rowptr, w->col, w->slot};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete w;
    h->enum_ws = nullptr;
}

int enum_setup(anigpu_ctx* h, int type) {
    if (type < ANIGPU_ENUM_ANITYPE || type > ANIGPU_ENUM_ETDIMBLOCKS) return set_err(h, ANIGPU_ERR_ARG, "enumeration type");
    if (h->space < 0) return set_err(h, ANIGPU_ERR_STATE, "anigpu_problem_setup not called");
    const bool general = is_general_space(h->space);
    GenBlocks gb{};
    if (general && !general_dof_blocks(h, gb.per, gb.off)) return set_err(h, ANIGPU_ERR_STATE, "general problem not set up");
    free_enum(h);
    EnumWs* w = new EnumWs();
    h->enum_ws = w;
    w->type = type;
    w->n = h->ndof;
    w->nnz = h->nnz;
    RC_(dev_alloc(h, &w->perm, w->n));
    RC_(dev_alloc(h, &w->rowptr, w->n + 1));
    RC_(dev_alloc(h, &w->col, std::max<int64_t>(w->nnz, 1)));
    RC_(dev_alloc(h, &w->slot, std::max<int64_t>(w->nnz, 1)));
    cudaStream_t s = h->stream;
    const int kind = kind_of(type);
    unsigned long long* len = nullptr;
    ANI_CUDA(h, cudaMallocAsync((void**)&len, sizeof(unsigned long long) * (w->n + 1), s));
    ANI_CUDA(h, cudaMemsetAsync(len, 0, sizeof(unsigned long long) * (w->n + 1), s));
    const int anitype = type == ANIGPU_ENUM_ANITYPE ? 1 : 0;
    if (general)
        gen_perm_kernel<<<grid_for(w->n, 256), 256, 0, s>>>(w->n, gb, anitype, w->perm, h->rowptr, len);
    else
        perm_kernel<<<grid_for(w->n, 256), 256, 0, s>>>(w->n, kind, h->nds, h->nv, h->ncomp, w->perm, h->rowptr, len);
    ANI_LAUNCHED(h);
    RC_(scan_counts(h, len, w->n, w->rowptr));
    ANI_CUDA(h, cudaFreeAsync(len, s));
    const unsigned blocks = (unsigned)std::min<int64_t>(w->n, 152 * 32);
    if (general)
        gen_slot_kernel<<<blocks, 128, 0, s>>>(w->n, gb, anitype, h->rowptr, h->col, w->perm, w->rowptr, w->col, w->slot);
    else
        slot_kernel<<<blocks, 128, 0, s>>>(w->n, kind, h->nds, h->nv, h->ncomp, h->rowptr, h->col, h->rowptr_s,
                                           h->col_s, w->perm, w->rowptr, w->col, w->slot);
    ANI_LAUNCHED(h);
    ANI_CUDA(h, cudaStreamSynchronize(s));
    return ANIGPU_OK;
}

int enum_template(anigpu_ctx* h, int64_t* rowptr, int32_t* col, int64_t* perm) {
    EnumWs* w = ews(h);
    if (!w) return set_err(h, ANIGPU_ERR_STATE, "anigpu_enumeration_setup not called");
    cudaStream_t s = h->stream;
    if (rowptr) ANI_CUDA(h, cudaMemcpyAsync(rowptr, w->rowptr, sizeof(int64_t) * (w->n + 1), cudaMemcpyDeviceToDevice, s));
    if (col) ANI_CUDA(h, cudaMemcpyAsync(col, w->col, sizeof(int32_t) * w->nnz, cudaMemcpyDeviceToDevice, s));
    if (perm) ANI_CUDA(h, cudaMemcpyAsync(perm, w->perm, sizeof(int64_t) * w->n, cudaMemcpyDeviceToDevice, s));
    ANI_CUDA(h, cudaStreamSynchronize(s));
    return ANIGPU_OK;
}

int enum_apply(anigpu_ctx* h, const void* vals_in, int precision, const double* rhs_in, void* vals_out,
               double* rhs_out) {
    EnumWs* w = ews(h);
    if (!w) return set_err(h, ANIGPU_ERR_STATE, "anigpu_enumeration_setup not called");
    if (w->n != h->ndof || w->nnz != h->nnz) return set_err(h, ANIGPU_ERR_STATE, "problem changed since the setup");
    cudaStream_t s = h->stream;
    if (vals_in && vals_out) {
        if (vals_in == vals_out) return set_err(h, ANIGPU_ERR_ARG, "in-place renumbering is not supported");
        if (precision == ANIGPU_F32)
            gather_vals_kernel<float><<<grid_for(w->nnz, 256), 256, 0, s>>>(w->nnz, w->slot, (const float*)vals_in,
                                                                           (float*)vals_out);
        else if (precision == ANIGPU_F64)
            gather_vals_kernel<double><<<grid_for(w->nnz, 256), 256, 0, s>>>(w->nnz, w->slot, (const double*)vals_in,
                                                                            (double*)vals_out);
        else
            return set_err(h, ANIGPU_ERR_ARG, "precision");
        ANI_LAUNCHED(h);
    }
    if (rhs_in && rhs_out) {
        if (rhs_in == rhs_out) return set_err(h, ANIGPU_ERR_ARG, "in-place renumbering is not supported");
        permute_vec_kernel<<<grid_for(w->n, 256), 256, 0, s>>>(w->n, w->perm, rhs_in, rhs_out, 0);
        ANI_LAUNCHED(h);
    }
    return ANIGPU_OK;
}

int enum_to_natural(anigpu_ctx* h, const double* x_in, double* x_out) {
    EnumWs* w = ews(h);
    if (!w) return set_err(h, ANIGPU_ERR_STATE, "anigpu_enumeration_setup not called");
    if (!x_in || !x_out || x_in == x_out) return set_err(h, ANIGPU_ERR_ARG, "vectors");
    permute_vec_kernel<<<grid_for(w->n, 256), 256, 0, h->stream>>>(w->n, w->perm, x_in, x_out, 1);
    ANI_LAUNCHED(h);
    return ANIGPU_OK;
}
