// The C ABI of anigpu (declared in include/anigpu.h): handles, errors, mesh upload and
// the thin host orchestration around the kernels.  No computation of the path happens
// on the host; every entry point that produces numbers launches device kernels.
#include <cstring>
#include <new>

#include "anigpu_internal.h"
#include "learned.h"
#include "quad_tables.h"
#include "tri_quad_tables.h"

int set_err(anigpu_ctx* h, int code, const std::string& msg) {
    if (h) h->err = msg;
    return code;
}

int cuda_check(anigpu_ctx* h, cudaError_t e, const char* what) {
    return set_err(h, ANIGPU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// entry check; also clears a sticky error left by other code in this thread so that the
// launch checks below report this library's own launches only
#define CHECK_H(h)                   \
    if (!(h)) return ANIGPU_ERR_ARG; \
    (void)cudaGetLastError()

extern "C" {

int anigpu_create(anigpu_handle* out, int device) {
    if (!out) return ANIGPU_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return ANIGPU_ERR_CUDA;
    if (device < 0 || device >= ndev) return ANIGPU_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return ANIGPU_ERR_CUDA;
    anigpu_ctx* h = new (std::nothrow) anigpu_ctx();
    if (!h) return ANIGPU_ERR_ARG;
    h->device = device;
    if (cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete h;
        return ANIGPU_ERR_CUDA;
    }
    h->stream = h->own_stream;
    if (cudaStreamCreateWithFlags(&h->side_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->fork_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->join_ev, cudaEventDisableTiming) != cudaSuccess) {
        cudaStreamDestroy(h->own_stream);
        delete h;
        return ANIGPU_ERR_CUDA;
    }
    if (cudaMalloc((void**)&h->d_status, sizeof(int)) != cudaSuccess ||
        cudaMemset(h->d_status, 0, sizeof(int)) != cudaSuccess) {
        cudaStreamDestroy(h->own_stream);
        delete h;
        return ANIGPU_ERR_CUDA;
    }
    *out = h;
    return ANIGPU_OK;
}

int anigpu_destroy(anigpu_handle h) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->stream);
    free_solver(h);
    free_fcg(h);
    free_learned(h);
    free_batch(h);
    free_enum(h);
    free_general(h);
    void* ptrs[] = {h->xyz, h->xyz2, h->tets, h->tet_edges, h->edofs, h->inc_ptr, h->recs, h->dir_mask, h->dir_bc,
                    h->dir_cptr, h->dir_coff, h->ring, h->ring_woff, h->vrec, h->vrec_woff,
                    h->tpos, h->tpos_woff, h->vrec4, h->vdiag,
                    h->tetdata, h->d_status, h->d_ref_tables};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (h->rowptr && h->rowptr != h->rowptr_s) cudaFree(h->rowptr);
    if (h->col && h->col != h->col_s) cudaFree(h->col);
    if (h->rowptr_s) cudaFree(h->rowptr_s);
    if (h->col_s) cudaFree(h->col_s);
    for (auto& kv : h->basis_dev) cudaFree(kv.second);
    for (void* p : h->extra_allocs) cudaFree(p);
    for (auto& e : h->tev)
        if (e) cudaEventDestroy(e);
    if (h->fork_ev) cudaEventDestroy(h->fork_ev);
    if (h->join_ev) cudaEventDestroy(h->join_ev);
    if (h->side_stream) cudaStreamDestroy(h->side_stream);
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
    delete h;
    return ANIGPU_OK;
}

int anigpu_set_stream(anigpu_handle h, void* stream) {
    CHECK_H(h);
    h->stream = stream ? (cudaStream_t)stream : h->own_stream;
    return ANIGPU_OK;
}

int anigpu_get_stream(anigpu_handle h, void** stream) {
    CHECK_H(h);
    if (!stream) return set_err(h, ANIGPU_ERR_ARG, "NULL");
    *stream = (void*)h->stream;
    return ANIGPU_OK;
}

const char* anigpu_last_error(anigpu_handle h) { return h ? h->err.c_str() : "invalid handle"; }

int64_t anigpu_launch_count(anigpu_handle h) { return h ? h->launches : -1; }

int anigpu_set_timing(anigpu_handle h, int enable) {
    CHECK_H(h);
    h->timing = enable != 0;
    h->ntev = 0;
    return ANIGPU_OK;
}

int anigpu_last_timing(anigpu_handle h, double* ms_host, int cap) {
    CHECK_H(h);
    if (!h->timing || h->ntev < 2) return 0;
    ANI_CUDA(h, cudaEventSynchronize(h->tev[h->ntev - 1]));
    int n = 0;
    for (int k = 1; k < h->ntev && n < cap; ++k, ++n) {
        float ms = 0;
        ANI_CUDA(h, cudaEventElapsedTime(&ms, h->tev[k - 1], h->tev[k]));
        ms_host[n] = ms;
    }
    return n;
}

int anigpu_fem3dtet(anigpu_handle h, int opA, int opB, int tensor_kind, int order, int precision, int64_t nt,
                    const double* XY, const double* D, void* A) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    return launch_fem3dtet(h, opA, opB, tensor_kind, order, precision, nt, XY, D, A);
}

int anigpu_fem3dtet_custom(anigpu_handle h, int dimA, int nfA, const double* UA, int dimB, int nfB, const double* VB,
                           int tensor_kind, int order, int precision, int64_t nt, const double* XY, const double* D,
                           void* A) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    return launch_fem3dtet_custom(h, dimA, nfA, UA, dimB, nfB, VB, tensor_kind, order, precision, nt, XY, D, A);
}

int anigpu_quadrature(int order, double* p_host, double* w_host, int cap) {
    const double *p, *w;
    int np;
    if (!anigpu_quad_rule(order, &p, &w, &np)) return ANIGPU_ERR_UNSUPPORTED;
    if (np > cap) return ANIGPU_ERR_ARG;
    if (p_host) std::memcpy(p_host, p, sizeof(double) * 4 * np);
    if (w_host) std::memcpy(w_host, w, sizeof(double) * np);
    return np;
}

int anigpu_quadrature_points(anigpu_handle h, int order, int64_t nt, const double* XY, double* XYG) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    return launch_quad_points(h, order, nt, XY, XYG);
}

int anigpu_fem3dface(anigpu_handle h, int opA, int opB, int tensor_kind, int order, int precision, int64_t nt,
                     const double* XY, int face, const double* D, void* A) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    if (face < 0 || face > 3) return set_err(h, ANIGPU_ERR_ARG, "face number must be 0..3");
    return launch_fem3dtet(h, opA, opB, tensor_kind, order, precision, nt, XY, D, A, face);
}

int anigpu_fem3dface_n(anigpu_handle h, int opA, int opB, int tensor_kind, int order, int precision, int64_t nt,
                       const double* XY, int face, const double* D, void* A) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    if (face < 0 || face > 3) return set_err(h, ANIGPU_ERR_ARG, "face number must be 0..3");
    return launch_fem3dtet(h, opA, opB, tensor_kind, order, precision, nt, XY, D, A, face, 1);
}

int anigpu_face_quadrature(int order, double* p_host, double* w_host, int cap) {
    const double *p, *w;
    int np;
    if (order < 0 || order > ANIGPU_TRI_MAX_ORDER || !anigpu_tri_rule(order, &p, &w, &np)) return ANIGPU_ERR_UNSUPPORTED;
    if (np > cap) return ANIGPU_ERR_ARG;
    if (p_host) std::memcpy(p_host, p, sizeof(double) * 3 * np);
    if (w_host) std::memcpy(w_host, w, sizeof(double) * np);
    return np;
}

int anigpu_face_quadrature_points(anigpu_handle h, int order, int face, int64_t nt, const double* XY, double* XYG) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    if (face < 0 || face > 3) return set_err(h, ANIGPU_ERR_ARG, "face number must be 0..3");
    return launch_quad_points(h, order, nt, XY, XYG, face);
}

int anigpu_enumeration_setup(anigpu_handle h, int type) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    return enum_setup(h, type);
}

int anigpu_enumeration_template(anigpu_handle h, int64_t* rowptr, int32_t* col, int64_t* perm) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    return enum_template(h, rowptr, col, perm);
}

int anigpu_enumeration_apply(anigpu_handle h, const void* vals_in, int precision, const double* rhs_in, void* vals_out,
                             double* rhs_out) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    return enum_apply(h, vals_in, precision, rhs_in, vals_out, rhs_out);
}

int anigpu_enumeration_to_natural(anigpu_handle h, const double* x_in, double* x_out) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    return enum_to_natural(h, x_in, x_out);
}

int anigpu_fem3d_apply(anigpu_handle h, int op, int64_t nt, const double* XY, int npts, const double* XYL,
                       const double* dofs, double* opU) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    if (!XY) return set_err(h, ANIGPU_ERR_ARG, "NULL coordinates");
    return launch_fem3d_apply(h, op, nt, XY, npts, XYL, 0, dofs, nullptr, opU);
}

int anigpu_fem3d_apply_x(anigpu_handle h, int op, int64_t nt, const double* XY, int npts, const double* X,
                         const double* dofs, double* opU) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    if (!XY) return set_err(h, ANIGPU_ERR_ARG, "NULL coordinates");
    return launch_fem3d_apply(h, op, nt, XY, npts, X, 1, dofs, nullptr, opU);
}

int anigpu_eval_solution(anigpu_handle h, int op, const double* x, int npts, const double* XYL, double* opU) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    if (h->space < 0) return set_err(h, ANIGPU_ERR_STATE, "anigpu_problem_setup not called");
    const bool vecsp = h->space == ANIGPU_ND0 || h->space == ANIGPU_RT0;
    if (op != ANIGPU_IDEN && op != ANIGPU_GRAD && !(vecsp && (op == ANIGPU_DIV || op == ANIGPU_CURL)))
        return set_err(h, ANIGPU_ERR_ARG, "op must be ANIGPU_IDEN or ANIGPU_GRAD (DIV, CURL for ND0 / RT0)");
    return launch_fem3d_apply(h, ANIGPU_OP(h->space, op), h->nt, nullptr, npts, XYL, 0, nullptr, x, opU);
}

int anigpu_apply_dir(anigpu_handle h, int64_t nt, int n, double* A, double* F, const uint32_t* mask,
                     const double* bc) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    return launch_apply_dir(h, nt, n, A, F, mask, bc);
}

int anigpu_mesh_upload(anigpu_handle h, int64_t nv, const double* xyz, int64_t nt, const int32_t* tets) {
    CHECK_H(h);
    if (nv <= 0 || nt <= 0 || !xyz || !tets) return set_err(h, ANIGPU_ERR_ARG, "empty or NULL mesh");
    if (nv >= (int64_t)INT32_MAX || nt >= ((int64_t)1 << 27))
        return set_err(h, ANIGPU_ERR_UNSUPPORTED, "mesh too large for 32-bit vertex / 27-bit tet ids");
    cudaSetDevice(h->device);
    learned_invalidate(h);  // bindings and captured solver graphs refer to the old mesh
    free_batch(h);
    free_enum(h);
    free_general(h);
    int rc = dev_alloc(h, &h->xyz, (size_t)nv * 3);
    if (rc) return rc;
    rc = dev_alloc(h, &h->tets, (size_t)nt * 4);
    if (rc) return rc;
    ANI_CUDA(h, cudaMemcpyAsync(h->xyz, xyz, sizeof(double) * 3 * nv, cudaMemcpyDefault, h->stream));
    ANI_CUDA(h, cudaMemcpyAsync(h->tets, tets, sizeof(int32_t) * 4 * nt, cudaMemcpyDefault, h->stream));
    h->nv = nv;
    h->nt = nt;
    h->space = -1;
    if (h->xyz2) {
        cudaFree(h->xyz2);
        h->xyz2 = nullptr;
    }
    rc = setup_coords_split(h);
    if (rc) return rc;
    return setup_orient(h);
}

int anigpu_mesh_update_coords(anigpu_handle h, const double* xyz) {
    CHECK_H(h);
    if (!h->xyz || !xyz) return set_err(h, ANIGPU_ERR_STATE, "no mesh");
    cudaSetDevice(h->device);
    ANI_CUDA(h, cudaMemcpyAsync(h->xyz, xyz, sizeof(double) * 3 * h->nv, cudaMemcpyDefault, h->stream));
    return setup_coords_split(h);
}

int anigpu_problem_setup(anigpu_handle h, int space) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    learned_invalidate(h);
    free_batch(h);
    free_enum(h);
    if (is_general_space(space)) return general_setup(h, space);
    free_general(h);
    return setup_problem(h, space);
}

int anigpu_problem_info(anigpu_handle h, int64_t* ndof, int64_t* nnz, int64_t* nedges) {
    CHECK_H(h);
    if (h->space < 0) return set_err(h, ANIGPU_ERR_STATE, "anigpu_problem_setup not called");
    if (ndof) *ndof = h->ndof;
    if (nnz) *nnz = h->nnz;
    if (nedges) *nedges = h->ne;
    return ANIGPU_OK;
}

int anigpu_gather_layouts(anigpu_handle h, int* rings, int* enabled) {
    CHECK_H(h);
    if (rings) *rings = h->ring_ok ? 1 : 0;
    if (enabled) *enabled = h->ring_enabled ? 1 : 0;
    return ANIGPU_OK;
}

int anigpu_set_gather_layouts(anigpu_handle h, int enable) {
    CHECK_H(h);
    h->ring_enabled = enable != 0;
    return ANIGPU_OK;
}

int anigpu_csr_template(anigpu_handle h, int64_t* rowptr, int32_t* col) {
    CHECK_H(h);
    if (h->space < 0) return set_err(h, ANIGPU_ERR_STATE, "anigpu_problem_setup not called");
    cudaSetDevice(h->device);
    if (rowptr)
        ANI_CUDA(h, cudaMemcpyAsync(rowptr, h->rowptr, sizeof(int64_t) * (h->ndof + 1), cudaMemcpyDefault, h->stream));
    if (col) ANI_CUDA(h, cudaMemcpyAsync(col, h->col, sizeof(int32_t) * h->nnz, cudaMemcpyDefault, h->stream));
    ANI_CUDA(h, cudaStreamSynchronize(h->stream));
    return ANIGPU_OK;
}

namespace {
__global__ void element_coords_kernel(int64_t nt, const double* __restrict__ xyz, const int32_t* __restrict__ tets,
                                      double* __restrict__ XY) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;  // (tet, vertex, coordinate)
    if (i >= nt * 12) return;
    const int64_t t = i / 12;
    const int r = (int)(i - 12 * t), v = r / 3, c = r - 3 * v;
    XY[i] = xyz[3 * (int64_t)tets[4 * t + v] + c];
}
}  // namespace

int anigpu_element_coords(anigpu_handle h, double* XY) {
    CHECK_H(h);
    if (h->nt <= 0 || !h->tets) return set_err(h, ANIGPU_ERR_STATE, "no mesh uploaded");
    if (!XY) return set_err(h, ANIGPU_ERR_ARG, "NULL");
    cudaSetDevice(h->device);
    element_coords_kernel<<<grid_for(h->nt * 12, 256), 256, 0, h->stream>>>(h->nt, h->xyz, h->tets, XY);
    ANI_LAUNCHED(h);
    ANI_CUDA(h, cudaStreamSynchronize(h->stream));
    return ANIGPU_OK;
}

int anigpu_element_nodes(anigpu_handle h, int32_t* tets) {
    CHECK_H(h);
    if (h->nt <= 0 || !h->tets) return set_err(h, ANIGPU_ERR_STATE, "no mesh uploaded");
    if (!tets) return set_err(h, ANIGPU_ERR_ARG, "NULL");
    cudaSetDevice(h->device);
    ANI_CUDA(h, cudaMemcpyAsync(tets, h->tets, sizeof(int32_t) * 4 * h->nt, cudaMemcpyDefault, h->stream));
    ANI_CUDA(h, cudaStreamSynchronize(h->stream));
    return ANIGPU_OK;
}

int anigpu_element_dofs(anigpu_handle h, int32_t* edofs) {
    CHECK_H(h);
    if (h->space < 0) return set_err(h, ANIGPU_ERR_STATE, "anigpu_problem_setup not called");
    if (!edofs) return set_err(h, ANIGPU_ERR_ARG, "NULL");
    cudaSetDevice(h->device);
    ANI_CUDA(h, cudaMemcpyAsync(edofs, h->edofs, sizeof(int32_t) * h->nt * h->nloc_s, cudaMemcpyDefault, h->stream));
    ANI_CUDA(h, cudaStreamSynchronize(h->stream));
    return ANIGPU_OK;
}

int anigpu_dof_coords(anigpu_handle h, double* xyz) {
    CHECK_H(h);
    if (h->space < 0) return set_err(h, ANIGPU_ERR_STATE, "anigpu_problem_setup not called");
    if (!xyz) return set_err(h, ANIGPU_ERR_ARG, "NULL");
    cudaSetDevice(h->device);
    if (is_general_space(h->space)) return general_dof_coords(h, xyz);
    return setup_dof_coords(h, xyz);
}

int anigpu_set_dirichlet(anigpu_handle h, const uint8_t* mask, const double* bc) {
    CHECK_H(h);
    if (h->space < 0) return set_err(h, ANIGPU_ERR_STATE, "anigpu_problem_setup not called");
    cudaSetDevice(h->device);
    if (mask)
        ANI_CUDA(h, cudaMemcpyAsync(h->dir_mask, mask, h->ndof, cudaMemcpyDefault, h->stream));
    else
        ANI_CUDA(h, cudaMemsetAsync(h->dir_mask, 0, h->ndof, h->stream));
    if (bc)
        ANI_CUDA(h, cudaMemcpyAsync(h->dir_bc, bc, sizeof(double) * h->ndof, cudaMemcpyDefault, h->stream));
    else
        ANI_CUDA(h, cudaMemsetAsync(h->dir_bc, 0, sizeof(double) * h->ndof, h->stream));
    h->has_dirichlet = mask != nullptr;
    h->bc_nonzero = bc != nullptr;
    return setup_dirichlet_bits(h);
}

int anigpu_assemble(anigpu_handle h, int tensor_kind, const double* D, const double* f, double f_const, int order,
                    int precision, void* vals, double* rhs, uint8_t* touched, double drop_val) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    int rc = run_assemble(h, tensor_kind, D, f, f_const, order, precision, vals, rhs, touched, drop_val);
    if (rc) return rc;
    int st = 0;
    ANI_CUDA(h, cudaMemcpyAsync(&st, h->d_status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    ANI_CUDA(h, cudaStreamSynchronize(h->stream));
    if (st) {
        ANI_CUDA(h, cudaMemsetAsync(h->d_status, 0, sizeof(int), h->stream));
        return set_err(h, st, "non-finite value in assembly (AssemblerT status -1)");
    }
    return ANIGPU_OK;
}

int anigpu_assemble_general(anigpu_handle h, int opA, int opB, int tensor_kind, const double* D, int rhs_kind,
                            const double* F, int order, double* vals, double* rhs) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    int rc = general_assemble(h, opA, opB, tensor_kind, D, rhs_kind, F, order, vals, rhs);
    if (rc) return rc;
    int st = 0;
    ANI_CUDA(h, cudaMemcpyAsync(&st, h->d_status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    ANI_CUDA(h, cudaStreamSynchronize(h->stream));
    if (st) {
        ANI_CUDA(h, cudaMemsetAsync(h->d_status, 0, sizeof(int), h->stream));
        return set_err(h, st, "non-finite value in assembly (AssemblerT status -1)");
    }
    return ANIGPU_OK;
}

int anigpu_assemble_elements(anigpu_handle h, const double* Aelem, const double* Felem, double* vals,
                                     double* rhs) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    if (h->space < 0) return set_err(h, ANIGPU_ERR_STATE, "anigpu_problem_setup not called");
    int rc = is_general_space(h->space) ? general_gather(h, Aelem, Felem, vals, rhs)
                                        : elements_scatter(h, Aelem, Felem, vals, rhs);
    if (rc) return rc;
    int st = 0;
    ANI_CUDA(h, cudaMemcpyAsync(&st, h->d_status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    ANI_CUDA(h, cudaStreamSynchronize(h->stream));
    if (st) {
        ANI_CUDA(h, cudaMemsetAsync(h->d_status, 0, sizeof(int), h->stream));
        return set_err(h, st, "non-finite value in assembly (AssemblerT status -1)");
    }
    return ANIGPU_OK;
}

int anigpu_assemble_async(anigpu_handle h, int tensor_kind, const double* D, const double* f, double f_const,
                          int order, int precision, void* vals, double* rhs, uint8_t* touched, double drop_val) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    return run_assemble(h, tensor_kind, D, f, f_const, order, precision, vals, rhs, touched, drop_val);
}

int anigpu_batch_set_instances(anigpu_handle h, int ninst, const int64_t* tet_offsets, const double* vals_for_tuning) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    return batch_set_instances(h, ninst, tet_offsets, vals_for_tuning);
}

int anigpu_batch_info(anigpu_handle h, int* ntiles, int* lanes_per_row, float* tune_ms, int* device_loop) {
    CHECK_H(h);
    return batch_info(h, ntiles, lanes_per_row, tune_ms, device_loop);
}

int anigpu_batch_run_jobs(int njobs, const anigpu_batch_job* jobs, double rtol, int64_t maxit) {
    if (njobs < 1 || !jobs) return ANIGPU_ERR_ARG;
    for (int k = 0; k < njobs; ++k)
        if (!jobs[k].h) return ANIGPU_ERR_ARG;
    cudaSetDevice(jobs[0].h->device);
    return batch_run_jobs(njobs, jobs, rtol, maxit);
}

int anigpu_batch_assembly_tuning(anigpu_handle h, int* row_warps, float* ms) {
    CHECK_H(h);
    return batch_assembly_tuning(h, row_warps, ms);
}

int anigpu_batch_run(anigpu_handle h, int tensor_kind, const double* D, const double* f, double f_const, int order,
                     double* vals, double* rhs_assembled, const double* b, double* x, double rtol, int64_t maxit,
                     anigpu_solve_stats* stats) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    return batch_run(h, tensor_kind, D, f, f_const, order, vals, rhs_assembled, b, x, rtol, maxit, stats);
}

int anigpu_status(anigpu_handle h) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    int st = 0;
    ANI_CUDA(h, cudaMemcpyAsync(&st, h->d_status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    ANI_CUDA(h, cudaStreamSynchronize(h->stream));
    if (st) {
        ANI_CUDA(h, cudaMemsetAsync(h->d_status, 0, sizeof(int), h->stream));
        return set_err(h, st, "non-finite value in assembly (AssemblerT status -1)");
    }
    return ANIGPU_OK;
}

int anigpu_csr_compact(anigpu_handle h, int64_t* rowptr, int32_t* col, void* vals, int precision,
                       const uint8_t* touched, int64_t* nnz_out) {
    CHECK_H(h);
    if (!rowptr || !col || !touched || !nnz_out) return set_err(h, ANIGPU_ERR_ARG, "NULL argument");
    cudaSetDevice(h->device);
    return run_compact(h, rowptr, col, vals, precision, touched, nnz_out);
}

int anigpu_solve(anigpu_handle h, int method, const void* vals, int precision, const double* b, double* x,
                 double rtol, int64_t maxit, anigpu_solve_stats* stats) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    return run_solve(h, method, vals, precision, b, x, rtol, maxit, stats);
}

int anigpu_solve_refined(anigpu_handle h, int method, const float* vals32, const double* vals64, const double* b,
                         double* x, double rtol, int64_t maxit, anigpu_solve_stats* stats) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    return run_solve_refined(h, method, vals32, vals64, b, x, rtol, maxit, stats);
}

int anigpu_spmv(anigpu_handle h, const void* vals, int precision, const double* x, double* y) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    return run_spmv(h, vals, precision, x, y);
}

}  // extern "C"

extern "C" {

int anigpu_gnn_init(anigpu_handle h, int layers, int act_precision, uint64_t seed) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    return gnn_init(h, layers, act_precision, seed);
}
int64_t anigpu_gnn_num_params(anigpu_handle h) { return h ? gnn_num_params(h) : -1; }
int anigpu_gnn_get_params(anigpu_handle h, float* host, int64_t n) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    return gnn_params(h, host, n, 0, 0);
}
int anigpu_gnn_set_params(anigpu_handle h, const float* host, int64_t n) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    return gnn_params(h, const_cast<float*>(host), n, 1, 0);
}
int anigpu_gnn_get_grads(anigpu_handle h, float* host, int64_t n) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    return gnn_params(h, host, n, 0, 1);
}
int anigpu_gnn_zero_grads(anigpu_handle h) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    return gnn_zero_grads(h);
}
int anigpu_gnn_bind(anigpu_handle h, const void* vals, int precision, int tensor_kind, const double* D) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    return gnn_bind(h, vals, precision, tensor_kind, D);
}
int anigpu_gnn_apply(anigpu_handle h, const double* r, double* z) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    int rc = gnn_apply(h, r, z);
    if (rc) return rc;
    ANI_CUDA(h, cudaStreamSynchronize(h->stream));
    return ANIGPU_OK;
}
int anigpu_gnn_apply_f32(anigpu_handle h, const float* r, float* z) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    int rc = gnn_apply_f32(h, r, z);
    if (rc) return rc;
    ANI_CUDA(h, cudaStreamSynchronize(h->stream));
    return ANIGPU_OK;
}
int anigpu_gnn_coarse_chain(anigpu_handle h, int enable, int* active) {
    CHECK_H(h);
    if (enable >= 0) h->chain_enabled = enable != 0;
    if (active) *active = gnn_chain_active(h);
    return ANIGPU_OK;
}
int anigpu_gnn_coefficients(anigpu_handle h, float* coef) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    return gnn_coefficients(h, coef);
}
int anigpu_gnn_loss_grad(anigpu_handle h, const double* r, const double* e, double* loss_host) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    return gnn_loss_grad(h, r, e, loss_host);
}
int anigpu_gnn_adam(anigpu_handle h, float lr, float beta1, float beta2, float eps, int step, float grad_scale) {
    CHECK_H(h);
    cudaSetDevice(h->device);
    return gnn_adam(h, lr, beta1, beta2, eps, step, grad_scale);
}

}  // extern "C"
