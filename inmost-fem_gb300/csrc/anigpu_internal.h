// Internal declarations shared by the anigpu translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/anigpu.h"

#define ANIGPU_MAX_NF 30
#define ANIGPU_MAX_DIM 9

// ------------------------------------------------------------------ basis tables (host)
// Reference-element data of one scalar space at the points of one quadrature rule.
struct ScalarBasisTable {
    int space = -1, order = -1, q = 0, nf = 0;
    std::vector<double> pts, wts;   // 4*q barycentric, q weights (sum 1)
    std::vector<double> val;        // val[n*nf + i]
    std::vector<double> grad;       // grad[(n*nf + i)*3 + d]  d/dxi_d of phi_i
};
bool make_scalar_basis(int space, int order, ScalarBasisTable* t);
// the same at the points of the triangle rule of `order` mapped onto face `face` of the tet
// (face k = vertices k, k+1, k+2 mod 4, fem3Dface, int_face.inl:31-36); weights of that rule
bool make_scalar_basis_face(int space, int order, int face, ScalarBasisTable* t);
int eval_scalar_basis_at(int space, const double* l, double* val, double (*grad)[3]);
int scalar_space_nf(int space);
// op code helpers (code = 10*space + op)
bool op_info(int code, int* nf, int* dim, int* base_space, int* ncomp, int* op);

// ------------------------------------------------------------------ device records
// One scatter record per (row DOF, incident tet): the tet, the row's local index i in the
// tet, the Dirichlet flags and the column offsets of the tet's DOFs within the row, both
// in the canonical column order of row i (canon_local below):
//   x: tet id
//   y: bits 0-3 local index i, bits 4-13 Dirichlet flag of canonical column c (bit 4+c),
//      bits 16-31 offsets of canonical columns 8, 9
//   z: offsets of canonical columns 0..3, w: of columns 4..7 (8 bits each, little end first)
struct __align__(16) ScatterRec {
    uint32_t tet, meta, off03, off47;
};

// Canonical column order of element row i: the local DOF of canonical column c.
//   P1 vertex i:    i, then the other vertices ascending.
//   P2 vertex i:    i, the other vertices o1<o2<o3, edges (i,o1) (i,o2) (i,o3), then the
//                   opposite edges (o1,o2) (o1,o3) (o2,o3).
//   P2 edge (a,b):  a, b, the other vertices c<d, the edge itself, (a,c) (a,d) (b,c) (b,d), (c,d).
// Local edges are (0,1) (0,2) (0,3) (1,2) (1,3) (2,3) = local DOFs 4..9 (poly_2.h:76).
// In this order one element row is a fixed function of the tet's Gram matrix whatever i is,
// and the diagonal is column 0 (vertex rows) or 4 (P2 edge rows).
__host__ __device__ inline int canon_local(int nloc, int i, int c) {
    constexpr signed char k4[4][4] = {{0, 1, 2, 3}, {1, 0, 2, 3}, {2, 0, 1, 3}, {3, 0, 1, 2}};
    constexpr signed char k10[10][10] = {
        {0, 1, 2, 3, 4, 5, 6, 7, 8, 9}, {1, 0, 2, 3, 4, 7, 8, 5, 6, 9}, {2, 0, 1, 3, 5, 7, 9, 4, 6, 8},
        {3, 0, 1, 2, 6, 8, 9, 4, 5, 7}, {0, 1, 2, 3, 4, 5, 6, 7, 8, 9}, {0, 2, 1, 3, 5, 4, 6, 7, 9, 8},
        {0, 3, 1, 2, 6, 4, 5, 8, 9, 7}, {1, 2, 0, 3, 7, 4, 8, 5, 9, 6}, {1, 3, 0, 2, 8, 4, 7, 6, 9, 5},
        {2, 3, 0, 1, 9, 5, 7, 6, 8, 4}};
    return nloc == 4 ? k4[i][c] : k10[i][c];
}
__host__ __device__ inline int canon_diag(int nloc, int i) { return (nloc == 10 && i >= 4) ? 4 : 0; }

// ------------------------------------------------------------------ context
struct anigpu_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    cudaStream_t side_stream = nullptr;  // second stream for concurrent launches inside one call
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    int row_warps = 2;  // row-gather warps (32 rows each) per block; the batch autotuner sets it
    bool asm_pdl = false;  // the gathers being launched follow the per-tet kernel on its stream
    bool chain_enabled = true;  // learned preconditioner: coarse products as one cooperative launch
    std::string err;
    int64_t launches = 0;

    // mesh
    int64_t nv = 0, nt = 0;
    double* xyz = nullptr;    // nv*3
    float2* xyz2 = nullptr;   // nv*3 (hi, lo) float pairs with hi + lo == xyz to ~2^-48 (FP32 geometry)
    int32_t* tets = nullptr;  // nt*4 (oriented)

    // problem
    int space = -1;      // ANIGPU_P1 / ANIGPU_P2 / ANIGPU_VEC3_P2
    int nloc_s = 0;      // scalar local DOFs per tet (4 or 10)
    int ncomp = 1;
    int64_t ne = 0;      // edges
    int64_t nds = 0;     // scalar DOFs
    int64_t ndof = 0;    // DOFs (ncomp * nds)
    int64_t nnz_s = 0;   // scalar template nnz
    int64_t nnz = 0;     // template nnz
    int32_t* tet_edges = nullptr;  // nt*6
    int32_t* edofs = nullptr;      // nt*nloc_s (scalar DOFs)
    int64_t* rowptr_s = nullptr;   // nds+1
    int32_t* col_s = nullptr;      // nnz_s
    int64_t* rowptr = nullptr;     // ndof+1 (== rowptr_s for scalar spaces)
    int32_t* col = nullptr;        // nnz   (== col_s for scalar spaces)
    int64_t* inc_ptr = nullptr;    // nds+1
    ScatterRec* recs = nullptr;    // nt*nloc_s
    // P2 edge rows in ring order (the tets around each edge, consecutive tets sharing a face):
    // per warp of 32 edge rows a header slot, then one 8-byte record per incident tet, lane-interleaved
    uint2* ring = nullptr;
    int64_t* ring_woff = nullptr;  // first slot of each warp (nwarps + 1)
    int64_t ring_ws = 0;           // slots per warp when every warp has the same (else 0)
    bool ring_ok = false;          // every edge row of the mesh has a ring (else the record gather)
    bool ring_enabled = true;      // anigpu_set_gather_layouts: rings and interleaved vertex records
    // vertex rows' scatter records in the same lane-interleaved layout (no header)
    ScatterRec* vrec = nullptr;
    // P2 vertex rows by symmetry: the edge walks store every off-diagonal entry of the vertex rows
    // at its transposed position (tpos: per edge row the positions of (A,E), (B,E), (A,B), (B,A) and
    // the first ring vertex's (P,E), then (N,E) of each incidence), and a pass over the vertex rows'
    // incidences (vrec4: tet | local vertex << 27) adds the diagonal (at vdiag) and the rhs
    int32_t* tpos = nullptr;
    int64_t* tpos_woff = nullptr;
    int64_t tpos_ws = 0;
    uint32_t* vrec4 = nullptr;
    int32_t* vdiag = nullptr;
    bool tr_ok = false;
    int64_t* vrec_woff = nullptr;
    int64_t vrec_ws = 0;
    int max_row_len_s = 0;
    int64_t row_range[3] = {0, 0, 0};  // scalar rows [vertex DOFs | edge DOFs]
    int row_range_cap[2] = {0, 0};     // longest row of each range
    int max_deg = 0;               // max incident tets of a scalar DOF
    uint8_t* dir_mask = nullptr;   // ndof
    double* dir_bc = nullptr;      // ndof
    int64_t* dir_cptr = nullptr;   // nds+1: per non-Dirichlet scalar row, its Dirichlet columns ...
    uint16_t* dir_coff = nullptr;  // ... as offsets within the row (ascending)
    bool bc_nonzero = false;
    bool has_dirichlet = false;
    int order_assembled = -1;

    // scratch
    void* tetdata = nullptr;       // per-tet K blocks (phase 1 output)
    size_t tetdata_bytes = 0;
    int* d_status = nullptr;       // device status word
    double* d_ref_tables = nullptr; // device copy of the T tables etc.
    size_t d_ref_tables_bytes = 0;

    // solver workspace (lazily sized)
    void* solve_ws = nullptr;
    size_t solve_ws_bytes = 0;
    void* learned = nullptr;       // learned preconditioner state
    void* fcg_ws = nullptr;        // flexible-CG workspace and its captured graphs
    void* batch_ws = nullptr;      // batched-instances map, tiles and solver workspace
    void* enum_ws = nullptr;       // renumbering to a non-NATURAL enumeration
    void* gen_ws = nullptr;        // general-path spaces (P0, P3, CR1, B2, B4, ND0, RT0)

    // per-phase timing (anigpu_set_timing)
    bool timing = false;
    cudaEvent_t tev[9] = {};
    int ntev = 0;  // events recorded in the last timed call

    std::vector<void*> extra_allocs;
    // device copies of reference-element tables, keyed by 100*space + order
    std::vector<std::pair<int, double*>> basis_dev;
    // lengths of the cached FP64 reference-tensor term lists (key as in basis_dev)
    std::vector<std::pair<int, int>> reft_len;
};
// device table for (space, order): q*nf values then q*nf*3 gradients, then q weights
int get_basis_dev(anigpu_ctx* h, int space, int order, const double** dev, ScalarBasisTable* host, int face = -1);

// ------------------------------------------------------------------ helpers
// record timing event k (k = 0 starts the call) when timing is enabled
inline void time_mark(anigpu_ctx* h, int k) {
    if (!h->timing || k >= 9) return;
    if (!h->tev[k]) cudaEventCreate(&h->tev[k]);
    cudaEventRecord(h->tev[k], h->stream);
    h->ntev = k + 1;
}
int set_err(anigpu_ctx* h, int code, const std::string& msg);
int cuda_check(anigpu_ctx* h, cudaError_t e, const char* what);
#define ANI_CUDA(h, call)                                      \
    do {                                                       \
        cudaError_t _e = (call);                               \
        if (_e != cudaSuccess) return cuda_check(h, _e, #call); \
    } while (0)
#define ANI_LAUNCHED(h)                                                  \
    do {                                                                 \
        (h)->launches++;                                                 \
        cudaError_t _e = cudaGetLastError();                             \
        if (_e != cudaSuccess) return cuda_check(h, _e, "kernel launch"); \
    } while (0)

template <typename T>
int dev_alloc(anigpu_ctx* h, T** p, size_t count) {
    if (*p) {
        cudaFree(*p);
        *p = nullptr;
    }
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
    if (e != cudaSuccess) return cuda_check(h, e, "cudaMalloc");
    return ANIGPU_OK;
}
inline unsigned grid_for(int64_t n, int block) {
    int64_t g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > 2147483647LL) g = 2147483647LL;
    return (unsigned)g;
}

// ------------------------------------------------------------------ kernel entry points (host side)
// element level (k_element.cu)
int launch_fem3dtet(anigpu_ctx* h, int opA, int opB, int kind, int order, int precision, int64_t nt,
                    const double* XY, const double* D, void* A, int face = -1, int normal = 0);
int launch_fem3dtet_custom(anigpu_ctx* h, int dimA, int nfA, const double* UA, int dimB, int nfB, const double* VB,
                           int kind, int order, int precision, int64_t nt, const double* XY, const double* D, void* A);
int launch_quad_points(anigpu_ctx* h, int order, int64_t nt, const double* XY, double* XYG, int face = -1);
// general-path spaces (k_general.cu)
bool is_general_space(int space);
void free_general(anigpu_ctx* h);
int general_setup(anigpu_ctx* h, int space);
int general_assemble(anigpu_ctx* h, int opA, int opB, int kind, const double* D, int rhs_kind, const double* F,
                     int order, double* vals, double* rhs);
int general_dof_coords(anigpu_ctx* h, double* out);
int general_gather(anigpu_ctx* h, const double* A, const double* F, double* vals, double* rhs);
// the fast path's template (P1, P2, vector P2): scatter of caller-computed element matrices (k_assemble.cu)
int elements_scatter(anigpu_ctx* h, const double* A, const double* F, double* vals, double* rhs);
const int8_t* general_signs(anigpu_ctx* h);
// DOFs per entity (node, edge, face, cell) and the first global DOF of each entity block (off[4] = ndof)
bool general_dof_blocks(anigpu_ctx* h, int per[4], int64_t off[5]);
// enumerations (k_enum.cu)
void free_enum(anigpu_ctx* h);
int enum_setup(anigpu_ctx* h, int type);
int enum_template(anigpu_ctx* h, int64_t* rowptr, int32_t* col, int64_t* perm);
int enum_apply(anigpu_ctx* h, const void* vals_in, int precision, const double* rhs_in, void* vals_out, double* rhs_out);
int enum_to_natural(anigpu_ctx* h, const double* x_in, double* x_out);
int launch_fem3d_apply(anigpu_ctx* h, int op, int64_t nt, const double* XY, int npts, const double* pts, int phys,
                       const double* dofs, const double* x, double* out);
int launch_apply_dir(anigpu_ctx* h, int64_t nt, int n, double* A, double* F, const uint32_t* mask, const double* bc);
// setup (k_setup.cu)
int setup_orient(anigpu_ctx* h);
int setup_problem(anigpu_ctx* h, int space);
int setup_dirichlet_bits(anigpu_ctx* h);
int setup_row_layouts(anigpu_ctx* h);
int setup_dof_coords(anigpu_ctx* h, double* out);
// refresh the (hi, lo) float copy of the coordinates after an upload or update
int setup_coords_split(anigpu_ctx* h);
// exclusive scan of cnt[0..n] (cnt[n] must be 0) into ptr[0..n]; ptr[n] = total
int scan_counts(anigpu_ctx* h, unsigned long long* cnt, int64_t n, int64_t* ptr);
// assembly (k_assemble.cu)
int run_assemble(anigpu_ctx* h, int kind, const double* D, const double* f, double f_const, int order,
                 int precision, void* vals, double* rhs, uint8_t* touched, double drop_val);
int run_compact(anigpu_ctx* h, int64_t* rowptr, int32_t* col, void* vals, int precision, const uint8_t* touched,
                int64_t* nnz_out);
// solve (k_solve.cu)
int run_spmv(anigpu_ctx* h, const void* vals, int precision, const double* x, double* y);
int run_solve_refined(anigpu_ctx* h, int method, const float* vals32, const double* vals64, const double* b, double* x,
                      double rtol, int64_t maxit, anigpu_solve_stats* st);
int run_solve(anigpu_ctx* h, int method, const void* vals, int precision, const double* b, double* x, double rtol,
              int64_t maxit, anigpu_solve_stats* st);
void free_solver(anigpu_ctx* h);
// batched instances (k_batch.cu)
void free_batch(anigpu_ctx* h);
int batch_set_instances(anigpu_ctx* h, int ninst, const int64_t* toff_host, const void* vals_for_tuning);
int batch_info(anigpu_ctx* h, int* ntiles, int* lanes, float* tune_ms, int* device_loop);
int batch_run(anigpu_ctx* h, int kind, const double* D, const double* f, double f_const, int order, double* vals,
              double* rhs_assembled, const double* b, double* x, double rtol, int64_t maxit, anigpu_solve_stats* st);
int batch_run_jobs(int njobs, const anigpu_batch_job* jobs, double rtol, int64_t maxit);
int batch_assembly_tuning(anigpu_ctx* h, int* row_warps, float* ms);
