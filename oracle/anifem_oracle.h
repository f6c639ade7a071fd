/* The oracle: a plain-C CPU restatement of the reference's hot path, used ONLY as
 * test infrastructure (tests/, the smoke check and bench.py's CPU-baseline leg).
 * It is never linked into, called by or shipped with the anigpu product library.
 *
 * Parity is pinned two ways: tests compare it with the reference's own fem3Dtet
 * (oracle/_ref, compiled from the reference sources where they are present) and with
 * the reference's golden matrices (tests/fem/operations/int_tet_test.cpp:229-243,
 * :333-346, :455), committed as fixtures under tests/golden/.
 */
#ifndef ANIFEM_ORACLE_H
#define ANIFEM_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* operator code = 10*space + op; op 1 IDEN, 2 GRAD; space 0 P0, 1 P1, 2 P2, 3 P3, 4 Vec3P1, 5 Vec3P2 */
/* tensor kinds */
enum { ORC_NULL = 0, ORC_CONST_SCALAR = 1, ORC_TET_SCALAR = 2, ORC_TET_SYM = 3, ORC_TET_GENERAL = 4, ORC_POINT = 5 };

int orc_op_info(int code, int* nf, int* dim);
int orc_quad_rule(int order, double* p /*4*np*/, double* w /*np*/, int cap);
/* physical quadrature points XYG[nt][q][3] (core.inl:249-269) */
int orc_quad_points(int order, long nt, const double* XY, double* XYG);
/* element matrices A[nt][nfA][nfB] (col-major nfB x nfA per tet), int_tet.inl:93-122 */
int orc_fem3dtet(int codeA, int codeB, int kind, int order, long nt, const double* XY, const double* D, double* A);
/* Op(u) at points of each tet: fem3DapplyL (phys 0: shared barycentric points [npts][4]) or
 * fem3DapplyX (phys 1: per-tet physical points [nt][npts][3]); opU[nt][npts][dim] */
int orc_fem3d_apply(int code, long nt, const double* XY, int npts, const double* pts, int phys,
                    const double* dofs, double* opU);
/* face integrals (fem3Dface, int_face.inl:12-44): same layout as orc_fem3dtet, the triangle rule of
 * `order` mapped onto face k = vertices {k, k+1, k+2 mod 4}, measure = the face area */
int orc_fem3dface(int codeA, int codeB, int kind, int order, int face, long nt, const double* XY, const double* D,
                  double* A);
/* fem3DfaceN (int_face.inl:48-78): the tensor has 3*dimB rows, contracted with the outward normal */
int orc_fem3dface_n(int codeA, int codeB, int kind, int order, int face, long nt, const double* XY, const double* D,
                    double* A);
/* the triangle rule of the face integrals (the table the product uses): p[3*np], w[np] */
int orc_tri_rule(int order, double* p, double* w, int cap);
/* physical points of that rule XYG[nt][q][3]; returns q */
int orc_face_quad_points(int order, int face, long nt, const double* XY, double* XYG);
/* Ani::applyDir (dc_on_dof.h:39-45) on one col-major n x n element matrix */
void orc_apply_dir(int n, double* A, double* F, int k, double bc);

/* mesh topology */
void orc_orient(const double* xyz, long nt, int32_t* tets);               /* ordering.inl:9-26 */
long orc_edges(long nv, long nt, const int32_t* tets, int32_t* tet_edges); /* returns #edges */
/* element DOF table: space 1 P1 (4), 2 P2 (10), 5 Vec3P2 (30, component-major blocks) */
long orc_element_dofs(int space, long nv, long ne, long nt, const int32_t* tets, const int32_t* tet_edges,
                      int32_t* edofs);
/* topological sparsity template (assembler.inl:590-693): rows sorted, diagonal forced.
 * Call with col == NULL to get nnz (rowptr filled), then again with col. */
long orc_csr_template(long ndof, long nt, int nloc, const int32_t* edofs, int64_t* rowptr, int32_t* col);
/* global scatter (assembler.inl:386-480) into the template:
 * vals[slot] += A_e(i,j) when |A_e(i,j)| > drop, touched[slot] = 1 for every such add; rhs += F.
 * Returns 0, or -1 when a non-finite element value is met (status -1 of Assemble). */
int orc_scatter(long ndof, const int64_t* rowptr, const int32_t* col, long nt, int nloc, const int32_t* edofs,
                const double* Aelem, const double* Felem, double drop, double* vals, double* rhs, uint8_t* touched);
/* drop-rule pattern: keep touched slots and the diagonal; returns new nnz (in-place compaction) */
long orc_csr_compact(long ndof, int64_t* rowptr, int32_t* col, double* vals, const uint8_t* touched);

/* linear algebra */
void orc_spmv(long n, const int64_t* rowptr, const int32_t* col, const double* vals, const double* x, double* y);
double orc_true_residual(long n, const int64_t* rowptr, const int32_t* col, const double* vals, const double* x,
                         const double* b);
/* FP64 Jacobi-PCG (a restatement: the reference solves through INMOST's Solver).
 * Stops when ||r||_2 <= rtol * ||b||_2 ; returns iterations or -1 if maxit reached. */
long orc_jacobi_pcg(long n, const int64_t* rowptr, const int32_t* col, const double* vals, const double* b,
                    double* x, double rtol, long maxit, double* final_rel);

/* CPU baseline: P2 GRAD.GRAD, per-tet symmetric tensor, over nthreads threads (contiguous chunks);
 * returns seconds */
double orc_time_p2_sym(long nt, const double* XY, const double* D6, int order, int nthreads, double* A);
/* multi-threaded drivers (bitwise equal to the serial functions; threads own tets or rows) */
int orc_fem3dtet_mt(int codeA, int codeB, int kind, int order, long nt, const double* XY, const double* D, double* A,
                    int nthreads);
void orc_apply_dir_elems(long nt, int nloc, double* A, double* F, const int32_t* edofs, const uint8_t* mask,
                         const double* bc, int nthreads);
long orc_csr_template_mt(long ndof, long nt, int nloc, const int32_t* edofs, int64_t* rowptr, int32_t* col,
                         int nthreads);
int orc_scatter_mt(long ndof, const int64_t* rowptr, const int32_t* col, long nt, int nloc, const int32_t* edofs,
                   const double* Aelem, const double* Felem, double drop, double* vals, double* rhs,
                   uint8_t* touched, int nthreads);
double orc_pcg_time_mt(long n, const int64_t* rowptr, const int32_t* col, const double* vals, const double* b,
                       long iters, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
