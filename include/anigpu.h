/* anigpu -- GB300-native element-matrix assembly, CSR scatter and Krylov solve for
 * tetrahedral finite elements.  C ABI: plain pointers and sizes, int status codes,
 * no exceptions across the boundary.  All array arguments are DEVICE pointers unless
 * the parameter name ends in _host.  One CUDA stream per handle; a handle is not
 * thread-safe, distinct handles are.
 *
 * Each entry point names the reference interface it replaces (AniFem++,
 * INMOST-DEV/INMOST-FEM; paths relative to that project).
 */
#ifndef ANIGPU_H
#define ANIGPU_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes.  -1/-2 keep the meaning of AssemblerT::Assemble's status
 * (anifem++/inmost_interface/assembler.inl:306-313). */
#define ANIGPU_OK 0
#define ANIGPU_ERR_NONFINITE (-1)     /* a non-finite element value was produced */
#define ANIGPU_ERR_BAD_ELEMENT (-2)   /* degenerate / broken element */
#define ANIGPU_ERR_ARG (-3)           /* invalid argument or size */
#define ANIGPU_ERR_UNSUPPORTED (-4)   /* operator pair, order or tensor kind not provided */
#define ANIGPU_ERR_CUDA (-5)          /* a CUDA runtime call failed */
#define ANIGPU_ERR_NOT_CONVERGED (-6) /* Krylov solve hit maxit or stagnated */
#define ANIGPU_ERR_STATE (-7)         /* call order violated (e.g. assemble before setup) */
#define ANIGPU_ERR_TIMEOUT (-8)       /* a bounded device-side wait expired */

/* ---- spaces and operators: code = 10*space + op (Ani::FiniteElement / Ani::OperatorType,
 * anifem++/fem/operators.h:25-45; FemVec<3,.> as anifem++/fem/operators.h:63-67,127-155) */
#define ANIGPU_P0 0
#define ANIGPU_P1 1
#define ANIGPU_P2 2
#define ANIGPU_P3 3
#define ANIGPU_VEC3_P1 4
#define ANIGPU_VEC3_P2 5
/* scalar spaces of the element level only (anifem++/fem/operators.h:26-34 and the spaces/ headers):
 * Crouzeix-Raviart (4 face DOFs, 1 - 3 lambda of the opposite vertex), edge bubbles
 * (4 lambda_i lambda_j in edge order), the volume bubble (256 lambda_0 lambda_1 lambda_2 lambda_3) */
#define ANIGPU_CR1 6
#define ANIGPU_B2 7
#define ANIGPU_B4 8
/* vector-valued lowest-order spaces of the element level (spaces/nedelec_0.h, raviant_thomas_0.h):
 * Nedelec ND0 (6 edge DOFs; IDEN dim 3, CURL dim 3, GRAD dim 9 = the skew part curl/2, DIV = 0) and
 * Raviart-Thomas RT0 (4 face DOFs; IDEN dim 3, DIV dim 1, GRAD dim 9, CURL = 0).  Their operator
 * codes use the reference's DIV = 3 and CURL = 4: 10*space + op, e.g. ANIGPU_OP(ANIGPU_RT0, ANIGPU_DIV). */
#define ANIGPU_ND0 9
#define ANIGPU_RT0 10
#define ANIGPU_DIV 3
#define ANIGPU_CURL 4
#define ANIGPU_IDEN 1
#define ANIGPU_GRAD 2
#define ANIGPU_OP(space, op) (10 * (space) + (op))

/* ---- coefficient tensor kinds (Ani::TensorType + DfuncTraits sparsity,
 * anifem++/fem/diff_tensor.h:17-53).  Tensor data layouts:
 *   NULL          no data (identity, or a column of ones when dim(OpA) == 1)
 *   CONST_SCALAR  1 value for all tets
 *   TET_SCALAR    nt values
 *   TET_SYM       6 values per tet: d00 d01 d02 d11 d12 d22 (3x3 operators only)
 *   TET_GENERAL   dimB*dimA per tet, column-major dimB x dimA (the layout the user
 *                 functor writes, int_tet_test.cpp:218)
 *   POINT         dimB*dimA per (tet, quadrature point), column-major, points in the order
 *                 of anigpu_quadrature() (the PerPoint functor evaluated at
 *                 anigpu_quadrature_points(), diff_tensor.h:488-552) */
#define ANIGPU_TENSOR_NULL 0
#define ANIGPU_TENSOR_CONST_SCALAR 1
#define ANIGPU_TENSOR_TET_SCALAR 2
#define ANIGPU_TENSOR_TET_SYM 3
#define ANIGPU_TENSOR_TET_GENERAL 4
#define ANIGPU_TENSOR_POINT 5

/* ---- arithmetic of element matrices / CSR values (BF16: learned-preconditioner activations) */
#define ANIGPU_F64 0
#define ANIGPU_F32 1
#define ANIGPU_BF16 2

/* ---- Krylov methods (replacing INMOST Solver, examples/tutorials/ex1.cpp:161-163) */
#define ANIGPU_SOLVE_JACOBI_PCG 0 /* FP64 Jacobi-preconditioned CG */
#define ANIGPU_SOLVE_IR_CG32 1    /* FP32-SpMV Jacobi-CG inside FP64 iterative refinement */
#define ANIGPU_SOLVE_FCG_LEARNED 2 /* flexible CG, learned preconditioner, Jacobi fallback */

typedef struct anigpu_ctx* anigpu_handle;

typedef struct anigpu_solve_stats {
    int64_t iterations;       /* total inner Krylov iterations */
    int64_t outer_iterations; /* refinement steps (IR / FCG restarts) */
    double rel_residual;      /* final FP64 ||b - A x|| / ||b|| */
    double seconds;           /* wall time of the solve (device events) */
    int64_t fallback_steps;   /* FCG steps that fell back to Jacobi */
} anigpu_solve_stats;

/* ---- lifetime */
int anigpu_create(anigpu_handle* h, int device);
int anigpu_destroy(anigpu_handle h);
/* run the handle's work on an existing stream (cudaStream_t), 0 = the handle's own */
int anigpu_set_stream(anigpu_handle h, void* stream);
/* the stream (cudaStream_t) the handle's work runs on; host code that copies the handle's outputs
 * orders its copies on it (the handle's own stream does not synchronise with the legacy default
 * stream) */
int anigpu_get_stream(anigpu_handle h, void** stream);
const char* anigpu_last_error(anigpu_handle h);
/* kernels launched by this handle since creation (evidence for bench reports) */
int64_t anigpu_launch_count(anigpu_handle h);

/* per-phase device timings (CUDA events on the handle's stream), the counterpart of the
 * reference's OPTIMIZER_TIMERS_FEM3DTET phase timers (anifem++/fem/operations/core.inl:1-9)
 * and WITH_ASSEMBLER_TIMERS (assembler.h:234-247).  When enabled, anigpu_assemble records
 * [tet prepare, row gather] in milliseconds; anigpu_last_timing copies them out. */
int anigpu_set_timing(anigpu_handle h, int enable);
int anigpu_last_timing(anigpu_handle h, double* ms_host, int cap);

/* ---- element level: the fused batch of Ani::fem3Dtet
 * (anifem++/fem/operations/int_tet.h:17-29, int_tet.inl:30-57,93-122; the FUSION batch of
 * TetrasT columns becomes the whole device batch).
 *   XY: nt*12 doubles, per tet X0 X1 X2 X3 (3 each), the TetrasT columns
 *   D : tensor data by kind (see above), doubles
 *   A : nt * nfB * nfA values (F64 or F32 by precision), per tet column-major nfB x nfA,
 *       A(i_test, j_trial), exactly the DenseMatrix A of fem3Dtet
 *   order: quadrature order 0..20 (the rules of tetrahedron_quadrature_formulas; the
 *          memoryless fem3Dtet stops at 6, int_tet.inl:98-99, its PlainMemory overload,
 *          int_tet.inl:30-57, takes them all) */
int anigpu_fem3dtet(anigpu_handle h, int opA, int opB, int tensor_kind, int order, int precision, int64_t nt,
                    const double* XY, const double* D, void* A);

/* the same with user-defined operators, the counterpart of Ani::ApplyOpCustom
 * (anifem++/fem/operators.h:450-471) used through fem3Dtet with runtime operators
 * (int_tet.h:111-147): the functor that fills U at the quadrature points becomes data.
 *   UA: the A operator's values at the points of the rule of `order` (anigpu_quadrature_points
 *       gives their coordinates), per tet and point a dimA x nfA column-major matrix:
 *       UA[((t*q + n)*nfA + i)*dimA + k], doubles on the device
 *   VB: the same for the B operator (dimB x nfB), or NULL when B is A
 * 1 <= dim <= 9; tensor kinds and the identity-tensor rule as anigpu_fem3dtet; A as there. */
int anigpu_fem3dtet_custom(anigpu_handle h, int dimA, int nfA, const double* UA, int dimB, int nfB, const double* VB,
                           int tensor_kind, int order, int precision, int64_t nt, const double* XY, const double* D,
                           void* A);
/* quadrature rule (host arrays): p[4*np] barycentric, w[np] summing to 1; returns np or <0
 * (replaces tetrahedron_quadrature_formulas, anifem++/fem/quadrature_formulas.cpp:526) */
int anigpu_quadrature(int order, double* p_host, double* w_host, int cap);
/* physical quadrature points XYG[nt][q][3] (internalFem3DtetGeomInit_XYG, core.inl:249-269) */
int anigpu_quadrature_points(anigpu_handle h, int order, int64_t nt, const double* XY, double* XYG);

/* ---- face integrals: the fused batch of Ani::fem3Dface (anifem++/fem/operations/int_face.h:13-19,
 * int_face.inl:12-44): A = int over face `face` of (D OpA(u)) . OpB(v), the same element engine as
 * anigpu_fem3dtet with the triangle rule of `order` (0..9; the reference's stack-memory fem3Dface
 * limit is 9, int_face.inl:22-23) mapped onto the face and |face| as the measure.  face k is the
 * face of vertices {k, k+1, k+2 mod 4} of every tet of the batch (face 0 = {X0,X1,X2}, 1 =
 * {X1,X2,X3}, 2 = {X2,X3,X0}, 3 = {X3,X0,X1}).  Tensor kinds and layouts as for anigpu_fem3dtet;
 * POINT data follow the points of anigpu_face_quadrature_points.  Neumann loads are
 * OpA = IDEN P0 (1 DOF) with the load as the tensor (a 3x1 GENERAL tensor for a vector traction
 * on IDEN FemVec<3,.>), Robin terms OpA = OpB = IDEN.  The rules are the reference's triangle
 * family (triangle_quadrature_formulas, quadrature_formulas.cpp:109), recomputed. */
int anigpu_fem3dface(anigpu_handle h, int opA, int opB, int tensor_kind, int order, int precision, int64_t nt,
                     const double* XY, int face, const double* D, void* A);
/* Ani::fem3DfaceN (int_face.h:28-34, int_face.inl:48-78): int over the face of ((D OpA(u)) . N) . OpB(v)
 * with N the outward unit normal of the face (Ani::face_normal, geometry.h:77-93).  The tensor has
 * 3*dimB rows (row l + 3k: normal component l of output row k, DotWithNormalHelper, core.h:175-190):
 * e.g. a pressure p I as a 9x1 GENERAL tensor with OpA = IDEN P0 gives the load p n . v, and
 * OpA = GRAD, OpB = IDEN with the NULL tensor gives the normal derivative term (grad u . n) v. */
int anigpu_fem3dface_n(anigpu_handle h, int opA, int opB, int tensor_kind, int order, int precision, int64_t nt,
                       const double* XY, int face, const double* D, void* A);
/* triangle rule (host arrays): p[3*np] barycentric on the face, w[np] summing to 1; returns np or <0 */
int anigpu_face_quadrature(int order, double* p_host, double* w_host, int cap);
/* physical points of the face rule, XYG[nt][q][3] */
int anigpu_face_quadrature_points(anigpu_handle h, int order, int face, int64_t nt, const double* XY, double* XYG);

/* ---- global enumerations (GlobEnumeration::ASSEMBLING_TYPE, anifem++/inmost_interface/
 * global_enumerator.h:392-404; same values).  anigpu_problem_setup numbers the DOFs NATURAL
 * (VAR DIM ELEM_TYPE ELEM_ID DOF_ID: component-major blocks, nodes before edges); the other types
 * order the same key differently.  For the spaces of this library (one variable, one DOF per node
 * or edge) they give three numberings of DOF (component c, scalar DOF s): NATURAL c*nds + s;
 * ANITYPE and BYELEMTYPE: nodes of component 0, 1, 2, then edges of component 0, 1, 2; MINIBLOCKS,
 * DIMUNION and ETDIMBLOCKS: the components of a node or edge together (ncomp*s + c).  Scalar spaces:
 * all equal NATURAL.  General-path spaces (P0, P3, CR1, B2, B4, ND0, RT0; DOFs of an entity
 * consecutive in NATURAL): all equal NATURAL except ANITYPE where an entity holds several DOFs
 * (P3 edges: DOF 0 of every edge, then DOF 1 of every edge).
 * setup: the permutation, the template in the new numbering and the map of every template slot;
 * template: rowptr[ndof+1] / col[nnz] of that template (rows sorted) and perm[ndof] (new index of
 * each NATURAL DOF), any may be NULL; apply: values (precision F32/F64) and right-hand side of an
 * assembled system into the new numbering (one gather, not in place; either pair may be NULL);
 * to_natural: a vector of the new numbering (e.g. a solution) back to NATURAL. */
#define ANIGPU_ENUM_ANITYPE 0
#define ANIGPU_ENUM_MINIBLOCKS 1
#define ANIGPU_ENUM_NATURAL 2
#define ANIGPU_ENUM_DIMUNION 3
#define ANIGPU_ENUM_BYELEMTYPE 4
#define ANIGPU_ENUM_ETDIMBLOCKS 5
int anigpu_enumeration_setup(anigpu_handle h, int type);
int anigpu_enumeration_template(anigpu_handle h, int64_t* rowptr, int32_t* col, int64_t* perm);
int anigpu_enumeration_apply(anigpu_handle h, const void* vals_in, int precision, const double* rhs_in, void* vals_out,
                             double* rhs_out);
int anigpu_enumeration_to_natural(anigpu_handle h, const double* x_in, double* x_out);

/* ---- evaluation of Op(u) at points of each tet (FP64).
 * anigpu_fem3d_apply is Ani::fem3DapplyL (anifem++/fem/operations/eval.h:13-18,93-111, eval.inl:93-111)
 *   over the whole batch: XYL[npts][4] barycentric points shared by every tet (the reference's
 *   fused XYL), dofs[nt][nf] the element DOF values (the columns of its dofs matrix),
 *   opU[nt][npts][dim] (per tet the vectorised Op(u) at each point, its opU_r column).
 * anigpu_fem3d_apply_x is Ani::fem3DapplyX (eval.h:27-32,112-125, eval.inl:103-151): X[nt][npts][3]
 *   physical points per tet, turned into barycentric coordinates as getBaryCoord does
 *   (core.inl:120-137; points outside the tet extrapolate the tet's polynomial).
 * anigpu_eval_solution: the same for the set-up problem and a global DOF vector x[ndof] (device),
 *   op = ANIGPU_IDEN or ANIGPU_GRAD on the problem's space, points barycentric in the oriented
 *   local vertex order (the order of anigpu_element_dofs); opU[nt][npts][dim].
 * Errors: unknown operator code (ANIGPU_ERR_UNSUPPORTED), npts < 1 or NULL arrays (ANIGPU_ERR_ARG). */
int anigpu_fem3d_apply(anigpu_handle h, int op, int64_t nt, const double* XY, int npts, const double* XYL,
                       const double* dofs, double* opU);
int anigpu_fem3d_apply_x(anigpu_handle h, int op, int64_t nt, const double* XY, int npts, const double* X,
                         const double* dofs, double* opU);
int anigpu_eval_solution(anigpu_handle h, int op, const double* x, int npts, const double* XYL, double* opU);
/* element-level Dirichlet on a batch of element matrices (Ani::applyDir,
 * anifem++/fem/operations/dc_on_dof.h:39-45): for every tet t and local DOF k with bit k of
 * mask[t] set, applies applyDir(A_t, F_t, k, bc[t*n + k]) in ascending k.  A: F64, n x n. */
int anigpu_apply_dir(anigpu_handle h, int64_t nt, int n, double* A, double* F, const uint32_t* mask,
                     const double* bc);

/* ---- mesh and global problem (AssemblerT, anifem++/inmost_interface/assembler.h:316-386)
 * mesh_upload: coordinates xyz[nv*3] (f64) and tets[nt*4] (i32) -- device pointers; the
 * library keeps its own copies, with every tet reoriented like reorderNodesOnTetrahedron
 * (anifem++/inmost_interface/ordering.inl:9-26). */
int anigpu_mesh_upload(anigpu_handle h, int64_t nv, const double* xyz, int64_t nt, const int32_t* tets);
/* replace the coordinates only (moving mesh), same topology */
int anigpu_mesh_update_coords(anigpu_handle h, const double* xyz);
/* space: ANIGPU_P1, ANIGPU_P2 or ANIGPU_VEC3_P2.  Builds the NATURAL DOF numbering
 * (GlobEnumeration default, global_enumerator.h:392-404: vertex DOFs by vertex id, then edge
 * DOFs by edge id, edges ranked by (min vertex, max vertex); FemVec component-major), the
 * topological CSR template (AssembleTemplate, assembler.inl:590-693: sorted rows, diagonal
 * forced) and the row-gather scatter records.  All on the device. */
int anigpu_problem_setup(anigpu_handle h, int space);
int anigpu_problem_info(anigpu_handle h, int64_t* ndof, int64_t* nnz, int64_t* nedges);
/* Row layouts of the Gram-form gathers, built by anigpu_problem_setup: P2 edge rows in ring order
 * (the tets around each edge walked face to face, so each value is written once) and vertex rows
 * from lane-interleaved scatter records (one contiguous load per warp and step).
 * *rings = 1 when every edge of the mesh has a ring; *enabled = whether assemblies use these
 * layouts (default 1).  Calls that need a touched map or non-zero Dirichlet values, meshes without
 * rings (edge rows) and the table form use the record gather.  Both sum the same element
 * contributions (AssemblerT::Assemble, assembler.inl:314-487) in fixed, different orders: results
 * agree to rounding. */
int anigpu_gather_layouts(anigpu_handle h, int* rings, int* enabled);
int anigpu_set_gather_layouts(anigpu_handle h, int enable);
/* copy the template out: rowptr[ndof+1] (i64), col[nnz] (i32) -- device pointers */
int anigpu_csr_template(anigpu_handle h, int64_t* rowptr, int32_t* col);
/* element DOF table edofs[nt*nloc] (i32, device) */
int anigpu_element_dofs(anigpu_handle h, int32_t* edofs);
/* coordinates of every tet's vertices in the library's (reoriented) local order, XY[nt*12] (f64,
 * device): the TetrasT columns a local assembler sees (ElementalAssembler nodes,
 * elemental_assembler.h:221), so that element matrices computed from them by anigpu_fem3dtet fit
 * anigpu_element_dofs and anigpu_assemble_elements */
int anigpu_element_coords(anigpu_handle h, double* XY);
/* vertex ids of every tet in the same reoriented local order, tets[nt*4] (i32, device or host):
 * which mesh node each local node of anigpu_element_coords is (the ElementalAssembler's node
 * list, elemental_assembler.h:221, after reorderNodesOnTetrahedron, ordering.inl:9-26) */
int anigpu_element_nodes(anigpu_handle h, int32_t* tets);
/* coordinates of every DOF's node: xyz[ndof*3] (f64, device).  Vertex DOFs sit at the
 * vertex, P2 edge DOFs at the edge midpoint (DOF_coord<FEM_P2>, anifem++/fem/operators.h:750-767);
 * vector components repeat the scalar coordinates. */
int anigpu_dof_coords(anigpu_handle h, double* xyz);
/* Dirichlet DOFs: mask[ndof] (u8, nonzero = Dirichlet), bc[ndof] (f64) or NULL for zero */
int anigpu_set_dirichlet(anigpu_handle h, const uint8_t* mask, const double* bc);

/* Global assembly (AssemblerT::Assemble, assembler.inl:314-487) of
 *   A = sum_T fem3Dtet<GRAD space, GRAD space>(T, D_T)     (element matrices)
 *   b = sum_T fem3Dtet<IDEN P0, IDEN space>(T, f_T)         (right-hand side)
 * with applyDir on Dirichlet DOFs, into the template: vals[nnz] (F64/F32 by precision),
 * rhs[ndof] (f64).  tensor_kind: NULL, CONST_SCALAR, TET_SCALAR, TET_SYM for scalar spaces;
 * for ANIGPU_VEC3_P2: TET_GENERAL (9x9 per tet) or ANIGPU_TENSOR_LAME (2 per tet: lambda, mu).
 * f: per-tet source (f64[nt]) or NULL for f = f_const.  order: quadrature order of both integrals
 * (0..6, as fem3Dtet's `order`).  touched (u8[nnz], optional) marks
 * every slot that received |a| > drop_val (assembler.inl:416-418); NULL skips it.
 * Deterministic: every CSR value is summed in ascending tet order, no atomics.
 * Returns ANIGPU_ERR_NONFINITE when a value is not finite (assembler.inl:419-423). */
#define ANIGPU_TENSOR_LAME 7
int anigpu_assemble(anigpu_handle h, int tensor_kind, const double* D, const double* f, double f_const, int order,
                    int precision, void* vals, double* rhs, uint8_t* touched, double drop_val);
/* Allocation-free variant of anigpu_assemble (this entry point has no counterpart in the
 * reference).  For callers that cannot allocate device memory when they assemble: code whose
 * device memory is held by another allocator (a framework's caching allocator, for example)
 * and latency-critical loops that cannot afford cudaMalloc's implicit device-wide
 * synchronisation.  Same arguments and results as anigpu_assemble without the touched map.
 * It calls no cudaMalloc, cudaFree or other allocating routine: its scratch (the per-tet
 * blocks and the reference tables) is a fixed device array inside the library (16 MiB of
 * per-tet blocks plus 16 KiB of tables), which every GPU that loads the library holds until the
 * process exits.  Limit: 524,288 tets in F32 (32 bytes a tet), 262,144 in F64 (64 bytes a
 * tet); larger meshes are rejected with ANIGPU_ERR_ARG and a message.  The
 * handle must already be set up (anigpu_problem_setup and anigpu_set_dirichlet allocate).
 * The first call on a device looks up the array's device address (cudaGetSymbolAddress) and
 * should come before any stream capture.  All calls share the one array: calls that overlap
 * on the GPU (other handles, other streams) race and must be serialised by the caller. */
int anigpu_assemble_noalloc(anigpu_handle h, int tensor_kind, const double* D, const double* f, double f_const,
                            int order, int precision, void* vals, double* rhs, double drop_val);

/* anigpu_assemble without the wait: the kernels are enqueued on the handle's stream and the
 * call returns (no counterpart in the reference, whose Assemble is synchronous).  Argument
 * errors are returned at once; a non-finite value is recorded on the device and reported by
 * the next anigpu_status, so that back-to-back assemblies (or a CUDA graph of them) keep
 * the GPU busy.  The caller keeps D, f, vals, rhs and touched alive until the stream passes. */
/* General-path spaces: anigpu_problem_setup also takes ANIGPU_P0, ANIGPU_P3, ANIGPU_CR1, ANIGPU_B2,
 * ANIGPU_B4, ANIGPU_ND0, ANIGPU_RT0.  Their DOFs are numbered NATURAL over nodes, edges, faces and
 * cells (edge ids rank (min, max) vertex pairs, face ids sorted vertex triples), with oriented DOFs
 * as AssemblerT's sign-encoded indices do (assembler.inl:48-54,136-190): the two P3 DOFs of an edge
 * follow the edge's global direction (smaller to larger vertex id), ND0 DOFs carry the sign of
 * their local edge direction against the global one, RT0 DOFs the sign of the tet's outward face
 * normal against the global face normal (sorted vertex triple a < b < c: (X_b-X_a) x (X_c-X_a)).
 * anigpu_assemble_general: A = sum over tets of s_i s_j fem3Dtet<opA, opB>(tensor) (FP64 values in
 * the template, both operators on the problem's space), rhs_i = sum s_i fem3Dtet<IDEN P0, IDEN space>
 * (rhs tensor: a scalar source for scalar spaces, a 3x1 GENERAL or POINT tensor for ND0 / RT0);
 * rhs may be NULL.  Dirichlet DOFs (anigpu_set_dirichlet) as in the other paths.  Setup memory is
 * about 24 nt nloc^2 bytes (sorts of the element-matrix entries); the fast kernels (anigpu_assemble)
 * and batching take P1 / P2 / vector P2 only.
 * anigpu_assemble_elements (P1, P2, vector P2 and the general-path spaces): the scatter of
 * element matrices and right-hand sides that the caller computed, FP64 values in the problem's
 * template, the counterpart of AssemblerT::Assemble with a user local-assembler function
 * (assembler.inl:314-487; ElementalAssembler, elemental_assembler.h:118-219): Aelem [nt][nloc][nloc]
 * (column-major per tet in the local, unsigned basis: fem3Dtet's layout, e.g. sums of
 * anigpu_fem3dtet / anigpu_fem3dtet_custom outputs), Felem [nt][nloc] or NULL, device doubles;
 * nloc = local DOFs of the problem's space.  The library applies the orientation signs and the
 * Dirichlet rows and columns. */
int anigpu_assemble_general(anigpu_handle h, int opA, int opB, int tensor_kind, const double* D, int rhs_kind,
                            const double* F, int order, double* vals, double* rhs);
int anigpu_assemble_elements(anigpu_handle h, const double* Aelem, const double* Felem, double* vals,
                                     double* rhs);
int anigpu_assemble_async(anigpu_handle h, int tensor_kind, const double* D, const double* f, double f_const,
                          int order, int precision, void* vals, double* rhs, uint8_t* touched, double drop_val);
/* waits for the handle's stream; ANIGPU_ERR_NONFINITE (and clears it) when an assembly since
 * the last check met a non-finite value, else ANIGPU_OK */
int anigpu_status(anigpu_handle h);

/* the drop-rule pattern (assembler without template): keep touched slots and the diagonal
 * (set_elements_on_matrix_diagonal, assembler.inl:114-135).  In-place on rowptr/col/vals;
 * returns the new nnz through nnz_out. */
int anigpu_csr_compact(anigpu_handle h, int64_t* rowptr, int32_t* col, void* vals, int precision,
                       const uint8_t* touched, int64_t* nnz_out);

/* ---- Krylov solve on the handle's CSR template with given values.
 * vals: F64 (JACOBI_PCG) or the values in `precision`; b, x: f64[ndof] (x is the initial guess
 * and the result).  Convergence: ||b - A x||_2 <= rtol * ||b||_2 in FP64. */
int anigpu_solve(anigpu_handle h, int method, const void* vals, int precision, const double* b, double* x,
                 double rtol, int64_t maxit, anigpu_solve_stats* stats);
/* The same solve of the FP64-assembled system vals64 (the system the reference solves) with its
 * FP32-assembled counterpart vals32 as the operator of the inner iterations: IR_CG32 (outer residual
 * b - A64 x, inner FP32 CG on vals32) or FCG_LEARNED (FCG on vals32, bound by anigpu_gnn_bind; every
 * residual replacement and the convergence test use b - A64 x in FP64).  Convergence: ||b - A64 x||
 * <= rtol ||b||.  No counterpart in the reference (its solver is INMOST's, ex1.cpp:161-163). */
int anigpu_solve_refined(anigpu_handle h, int method, const float* vals32, const double* vals64, const double* b,
                         double* x, double rtol, int64_t maxit, anigpu_solve_stats* stats);
/* ---- learned preconditioner for ANIGPU_SOLVE_FCG_LEARNED (no counterpart in the reference,
 * whose solves go through INMOST's ILU-Krylov, examples/tutorials/ex1.cpp:161-163).
 *   M r = D^-1 r + P Dc^-1/2 B B^T Dc^-1/2 P^T r,   B = sum_{k<4} diag(a_k) A_hat^k
 *   (symmetric positive definite by construction).  Coarse nodes are the vertex DOFs of every
 *   component (ANIGPU_P2: nv nodes; ANIGPU_VEC3_P2: 3 nv nodes, node c*nv + v = vertex v of
 *   component c).  P interpolates vertex values onto the P2 DOFs of the same component, Dc =
 *   the coarse diagonal, A_hat = -Dc^-1/2 A_cc' Dc^-1/2 over the off-diagonal couplings between
 *   coarse nodes (across components too).  The per-node coefficients a (4 per node) come from a
 *   message-passing network on that coarse graph, run once per bind on static features (log of
 *   the diagonal and the local mean of log(trace D / 3), for ANIGPU_TENSOR_LAME of
 *   log(lambda + 2 mu)).  Hidden width 64, `layers` residual layers, activations
 *   in act_precision (ANIGPU_BF16, or ANIGPU_F32 for gradient checks), FP32 accumulation,
 *   FP32 master parameters.
 * init: random parameters (seeded; the untrained B is the identity); get/set_params: the flat
 *   FP32 parameter vector (checkpoint); bind: the system the preconditioner serves (values of
 *   a P2 or vector P2 problem, and the per-tet tensor for the features), runs the network;
 * apply: z = M r (f64 vectors); apply_f32: z = M r with the fused FP32 kernels the solver
 *   uses (f32[ndof] vectors); coefficients: a as f32[ncomp*nv][4] into a device buffer;
 * loss_grad: L = (M r - e)^T A (M r - e) / (e^T A e) for a pair (r, e = A^-1 r), gradients
 *   accumulated; adam: one Adam step on the accumulated gradients (then zeroed), network re-run. */
int anigpu_gnn_init(anigpu_handle h, int layers, int act_precision, uint64_t seed);
int64_t anigpu_gnn_num_params(anigpu_handle h);
int anigpu_gnn_get_params(anigpu_handle h, float* host, int64_t n);
int anigpu_gnn_set_params(anigpu_handle h, const float* host, int64_t n);
int anigpu_gnn_get_grads(anigpu_handle h, float* host, int64_t n);
int anigpu_gnn_zero_grads(anigpu_handle h);
int anigpu_gnn_bind(anigpu_handle h, const void* vals, int precision, int tensor_kind, const double* D);
int anigpu_gnn_apply(anigpu_handle h, const double* r, double* z);
int anigpu_gnn_apply_f32(anigpu_handle h, const float* r, float* z);
/* The coarse products of the FP32 apply (restriction, Horner, powers, combination) as one
 * cooperative launch with bounded grid barriers (enable = 1, the default) or as separate launches
 * (0); takes effect at the next anigpu_gnn_bind.  *active: whether the current binding uses the
 * single launch (it needs cooperative launches that CUDA graphs can capture). */
int anigpu_gnn_coarse_chain(anigpu_handle h, int enable, int* active);
int anigpu_gnn_coefficients(anigpu_handle h, float* coef);
int anigpu_gnn_loss_grad(anigpu_handle h, const double* r, const double* e, double* loss_host);
int anigpu_gnn_adam(anigpu_handle h, float lr, float beta1, float beta2, float eps, int step, float grad_scale);

/* ---- batched uneven instances (no counterpart in the reference, which assembles and solves one
 * mesh at a time: examples/tutorials/ex1.cpp:120-163).  Upload the disjoint union of the meshes
 * (vertex and tet ids offset per instance) with anigpu_mesh_upload, set it up and its Dirichlet DOFs
 * as one problem, then
 *   set_instances: tet_offsets (host, ninst+1, from 0 to nt) give the tets of each instance; builds the
 *     DOF -> instance map and the row tiles (each within one instance), and autotunes the solver's
 *     lanes per CSR row on vals_for_tuning (F64 values of this template; NULL skips the tuning);
 *   info: number of tiles, chosen lanes per row, the timings of the candidates 2, 4, 8, 16 (ms), and
 *     whether the last run looped on the device (1) or was driven from the host (0);
 *   run: the whole job as one CUDA graph launch where the toolkit has conditional graph nodes:
 *     the F64 assembly into vals (when rhs_assembled is not NULL; tensor kind and data as
 *     anigpu_assemble), then Jacobi-PCG from x = 0 on every instance at once with per-instance
 *     scalars and convergence (||b_i - A_i x_i|| <= rtol ||b_i||, FP64), looping on the device until
 *     every instance has converged or maxit iterations were taken.  b and x are f64[ndof]; stats
 *     (host, ninst) receive per instance: iterations, iterations of the whole batch, FP64 true
 *     relative residual, seconds of the whole job.  Returns ANIGPU_ERR_NOT_CONVERGED when an
 *     instance missed the tolerance. */
int anigpu_batch_set_instances(anigpu_handle h, int ninst, const int64_t* tet_offsets, const double* vals_for_tuning);
int anigpu_batch_info(anigpu_handle h, int* ntiles, int* lanes_per_row, float* tune_ms, int* device_loop);
int anigpu_batch_run(anigpu_handle h, int tensor_kind, const double* D, const double* f, double f_const, int order,
                     double* vals, double* rhs_assembled, const double* b, double* x, double rtol, int64_t maxit,
                     anigpu_solve_stats* stats);
/* Several batched jobs (handles on one device, each set up with its own instances: e.g. the P1
 * instances and the P2 instances of one study) as ONE CUDA graph launch: per job the same
 * assembly, initialisation and device-side solve loop as anigpu_batch_run, the jobs' node chains
 * independent so that they run concurrently.  The launch is on the first job's stream; every job's
 * stream waits for it.  Returns the first error (ANIGPU_ERR_NOT_CONVERGED when an instance of any
 * job missed rtol; stats per job as anigpu_batch_run). */
typedef struct anigpu_batch_job {
    anigpu_handle h;
    int tensor_kind;
    const double* D;
    const double* f;
    double f_const;
    int order;
    double* vals;
    double* rhs_assembled;
    const double* b;
    double* x;
    anigpu_solve_stats* stats;
} anigpu_batch_job;
int anigpu_batch_run_jobs(int njobs, const anigpu_batch_job* jobs, double rtol, int64_t maxit);
/* the assembly's autotuned rows per block of a batched job: warps of 32 rows (1 or 2) and the
 * timings of the two candidates (ms per assembly, ms[2]), measured at the job's first run */
int anigpu_batch_assembly_tuning(anigpu_handle h, int* row_warps, float* ms);

/* y = A x on the handle's template (F64 or F32 values, f64 vectors) */
int anigpu_spmv(anigpu_handle h, const void* vals, int precision, const double* x, double* y);

#ifdef __cplusplus
}
#endif
#endif /* ANIGPU_H */
