"""anigpu: Python host binding of the anigpu C ABI (include/anigpu.h).

The classes mirror the reference's interfaces for the hot path:
  * ``Anigpu.fem3dtet``      -- Ani::fem3Dtet over a batch of tets
                                (anifem++/fem/operations/int_tet.h:17-29)
  * ``Anigpu.mesh_upload`` / ``problem_setup`` / ``assemble``
                             -- AssemblerT::PrepareProblem / Assemble
                                (anifem++/inmost_interface/assembler.h:316-386)
  * ``Anigpu.solve``         -- the Krylov solve that consumes the matrix
All numerics run in libanigpu.so on the GPU.  There is no CPU fallback: importing works
anywhere, but creating a handle raises when the library or a CUDA device is missing.
Device buffers are torch CUDA tensors (plumbing only); the library sees raw pointers.
"""
import ctypes
import os

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "libanigpu.so")

# ---- constants (include/anigpu.h)
OK = 0
ERR_NONFINITE, ERR_BAD_ELEMENT, ERR_ARG, ERR_UNSUPPORTED, ERR_CUDA, ERR_NOT_CONVERGED, ERR_STATE, ERR_TIMEOUT = (
    -1, -2, -3, -4, -5, -6, -7, -8)
P0, P1, P2, P3, VEC3_P1, VEC3_P2 = 0, 1, 2, 3, 4, 5
CR1, B2, B4 = 6, 7, 8  # element level only
ND0, RT0 = 9, 10        # vector-valued, element level only
DIV, CURL = 3, 4
IDEN, GRAD = 1, 2
# GlobEnumeration::ASSEMBLING_TYPE (global_enumerator.h:392-404)
ENUM_ANITYPE, ENUM_MINIBLOCKS, ENUM_NATURAL, ENUM_DIMUNION, ENUM_BYELEMTYPE, ENUM_ETDIMBLOCKS = 0, 1, 2, 3, 4, 5
TENSOR_NULL, TENSOR_CONST_SCALAR, TENSOR_TET_SCALAR, TENSOR_TET_SYM, TENSOR_TET_GENERAL, TENSOR_POINT = range(6)
TENSOR_LAME = 7
F64, F32, BF16 = 0, 1, 2
SOLVE_JACOBI_PCG, SOLVE_IR_CG32, SOLVE_FCG_LEARNED = 0, 1, 2

# every entry point the header declares: name -> (restype, argtypes)
_vp, _i, _i64, _d = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double


class SolveStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int64), ("outer_iterations", ctypes.c_int64),
                ("rel_residual", ctypes.c_double), ("seconds", ctypes.c_double),
                ("fallback_steps", ctypes.c_int64)]


SIGNATURES = {
    "anigpu_create": (_i, [ctypes.POINTER(_vp), _i]),
    "anigpu_destroy": (_i, [_vp]),
    "anigpu_set_stream": (_i, [_vp, _vp]),
    "anigpu_last_error": (ctypes.c_char_p, [_vp]),
    "anigpu_launch_count": (_i64, [_vp]),
    "anigpu_set_timing": (_i, [_vp, _i]),
    "anigpu_last_timing": (_i, [_vp, _vp, _i]),
    "anigpu_fem3dtet": (_i, [_vp, _i, _i, _i, _i, _i, _i64, _vp, _vp, _vp]),
    "anigpu_fem3dtet_custom": (_i, [_vp, _i, _i, _vp, _i, _i, _vp, _i, _i, _i, _i64, _vp, _vp, _vp]),
    "anigpu_quadrature": (_i, [_i, _vp, _vp, _i]),
    "anigpu_quadrature_points": (_i, [_vp, _i, _i64, _vp, _vp]),
    "anigpu_fem3dface": (_i, [_vp, _i, _i, _i, _i, _i, _i64, _vp, _i, _vp, _vp]),
    "anigpu_fem3dface_n": (_i, [_vp, _i, _i, _i, _i, _i, _i64, _vp, _i, _vp, _vp]),
    "anigpu_face_quadrature": (_i, [_i, _vp, _vp, _i]),
    "anigpu_face_quadrature_points": (_i, [_vp, _i, _i, _i64, _vp, _vp]),
    "anigpu_enumeration_setup": (_i, [_vp, _i]),
    "anigpu_enumeration_template": (_i, [_vp, _vp, _vp, _vp]),
    "anigpu_enumeration_apply": (_i, [_vp, _vp, _i, _vp, _vp, _vp]),
    "anigpu_enumeration_to_natural": (_i, [_vp, _vp, _vp]),
    "anigpu_fem3d_apply": (_i, [_vp, _i, _i64, _vp, _i, _vp, _vp, _vp]),
    "anigpu_fem3d_apply_x": (_i, [_vp, _i, _i64, _vp, _i, _vp, _vp, _vp]),
    "anigpu_eval_solution": (_i, [_vp, _i, _vp, _i, _vp, _vp]),
    "anigpu_apply_dir": (_i, [_vp, _i64, _i, _vp, _vp, _vp, _vp]),
    "anigpu_mesh_upload": (_i, [_vp, _i64, _vp, _i64, _vp]),
    "anigpu_mesh_update_coords": (_i, [_vp, _vp]),
    "anigpu_problem_setup": (_i, [_vp, _i]),
    "anigpu_problem_info": (_i, [_vp, ctypes.POINTER(_i64), ctypes.POINTER(_i64), ctypes.POINTER(_i64)]),
    "anigpu_gather_layouts": (_i, [_vp, ctypes.POINTER(_i), ctypes.POINTER(_i)]),
    "anigpu_set_gather_layouts": (_i, [_vp, _i]),
    "anigpu_csr_template": (_i, [_vp, _vp, _vp]),
    "anigpu_element_dofs": (_i, [_vp, _vp]),
    "anigpu_element_coords": (_i, [_vp, _vp]),
    "anigpu_element_nodes": (_i, [_vp, _vp]),
    "anigpu_get_stream": (_i, [_vp, ctypes.POINTER(_vp)]),
    "anigpu_dof_coords": (_i, [_vp, _vp]),
    "anigpu_set_dirichlet": (_i, [_vp, _vp, _vp]),
    "anigpu_assemble": (_i, [_vp, _i, _vp, _vp, _d, _i, _i, _vp, _vp, _vp, _d]),
    "anigpu_assemble_async": (_i, [_vp, _i, _vp, _vp, _d, _i, _i, _vp, _vp, _vp, _d]),
    "anigpu_assemble_general": (_i, [_vp, _i, _i, _i, _vp, _i, _vp, _i, _vp, _vp]),
    "anigpu_assemble_elements": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "anigpu_status": (_i, [_vp]),
    "anigpu_assemble_noalloc": (_i, [_vp, _i, _vp, _vp, _d, _i, _i, _vp, _vp, _d]),
    "anigpu_csr_compact": (_i, [_vp, _vp, _vp, _vp, _i, _vp, ctypes.POINTER(_i64)]),
    "anigpu_solve": (_i, [_vp, _i, _vp, _i, _vp, _vp, _d, _i64, ctypes.POINTER(SolveStats)]),
    "anigpu_solve_refined": (_i, [_vp, _i, _vp, _vp, _vp, _vp, _d, _i64, ctypes.POINTER(SolveStats)]),
    "anigpu_spmv": (_i, [_vp, _vp, _i, _vp, _vp]),
    "anigpu_batch_set_instances": (_i, [_vp, _i, _vp, _vp]),
    "anigpu_batch_info": (_i, [_vp, ctypes.POINTER(_i), ctypes.POINTER(_i), _vp, ctypes.POINTER(_i)]),
    "anigpu_batch_run": (_i, [_vp, _i, _vp, _vp, _d, _i, _vp, _vp, _vp, _vp, _d, _i64, _vp]),
    "anigpu_batch_run_jobs": (_i, [_i, _vp, _d, _i64]),
    "anigpu_batch_assembly_tuning": (_i, [_vp, _vp, _vp]),
    "anigpu_gnn_init": (_i, [_vp, _i, _i, ctypes.c_uint64]),
    "anigpu_gnn_num_params": (_i64, [_vp]),
    "anigpu_gnn_get_params": (_i, [_vp, _vp, _i64]),
    "anigpu_gnn_set_params": (_i, [_vp, _vp, _i64]),
    "anigpu_gnn_get_grads": (_i, [_vp, _vp, _i64]),
    "anigpu_gnn_zero_grads": (_i, [_vp]),
    "anigpu_gnn_bind": (_i, [_vp, _vp, _i, _i, _vp]),
    "anigpu_gnn_apply": (_i, [_vp, _vp, _vp]),
    "anigpu_gnn_apply_f32": (_i, [_vp, _vp, _vp]),
    "anigpu_gnn_coarse_chain": (_i, [_vp, _i, ctypes.POINTER(_i)]),
    "anigpu_gnn_coefficients": (_i, [_vp, _vp]),
    "anigpu_gnn_loss_grad": (_i, [_vp, _vp, _vp, ctypes.POINTER(_d)]),
    "anigpu_gnn_adam": (_i, [_vp, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, _i,
                             ctypes.c_float]),
}

_LIB = None


def load_library(path=None):
    """Load libanigpu.so (raises OSError when it is missing: there is no fallback)."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    lib = ctypes.CDLL(path or LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = lib
    return lib


def build(verbose=False, force=False):
    from . import _build
    return _build.build_library(verbose=verbose, force=force)


class AnigpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"anigpu error {code}: {msg}")
        self.code = code


def op_info(code):
    """(nf, dim) of operator code 10*space + op (Operator<OP, FEM>::Nfa / Dim)."""
    space, op = divmod(code, 10)
    if space in (ND0, RT0):
        return (6 if space == ND0 else 4), {IDEN: 3, GRAD: 9, DIV: 1, CURL: 3}[op]
    nfs = {P0: 1, P1: 4, P2: 10, P3: 20, VEC3_P1: 4, VEC3_P2: 10, CR1: 4, B2: 6, B4: 1}[space]
    nc = 3 if space in (VEC3_P1, VEC3_P2) else 1
    bd = 1 if op == IDEN else 3
    return nfs * nc, bd * nc


def face_quadrature(order):
    """(points[np,3], weights[np]) of the triangle rule of the face integrals."""
    import numpy as np
    lib = load_library()
    p = np.zeros(3 * 256)
    w = np.zeros(256)
    n = lib.anigpu_face_quadrature(order, p.ctypes.data, w.ctypes.data, 256)
    if n <= 0:
        raise AnigpuError(n, "unsupported face quadrature order")
    return p[:3 * n].reshape(n, 3).copy(), w[:n].copy()


def quadrature(order):
    """(points[np,4], weights[np]) -- tetrahedron_quadrature_formulas(order)."""
    import numpy as np
    lib = load_library()
    p = np.zeros(4 * 1024)
    w = np.zeros(1024)
    n = lib.anigpu_quadrature(order, p.ctypes.data, w.ctypes.data, 1024)
    if n < 0:
        raise AnigpuError(n, f"no quadrature rule of order {order}")
    return p[:4 * n].reshape(n, 4).copy(), w[:n].copy()


def _streamed(fn):
    import functools

    @functools.wraps(fn)
    def wrap(self, *a, **k):
        with self.on_stream():
            return fn(self, *a, **k)
    return wrap


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


class Anigpu:
    """One library handle: one device, one stream (the caller's torch stream by default)."""

    def __init__(self, device=0):
        import torch
        if not torch.cuda.is_available():
            raise RuntimeError("anigpu needs a CUDA device (no CPU fallback)")
        self.torch = torch
        self.lib = load_library()
        self.device = device
        h = ctypes.c_void_p()
        self._check(self.lib.anigpu_create(ctypes.byref(h), device), None)
        self.h = h
        # one stream for the torch plumbing and the library kernels of this handle
        self.stream = torch.cuda.Stream(device=device)
        self.set_stream(self.stream.cuda_stream)
        self.space = None

    class _OnStream:
        def __init__(self, outer):
            self.o = outer

        def __enter__(self):
            t = self.o.torch
            self.caller = t.cuda.current_stream(self.o.device)
            self.o.stream.wait_stream(self.caller)
            self.ctx = t.cuda.stream(self.o.stream)
            self.ctx.__enter__()

        def __exit__(self, *a):
            self.ctx.__exit__(*a)
            self.caller.wait_stream(self.o.stream)

    def on_stream(self):
        """Context in which torch work and library calls share the handle's stream."""
        return Anigpu._OnStream(self)

    # -------------------------------------------------------------- plumbing
    def _check(self, rc, h="self"):
        if rc < 0:
            hh = self.h if h == "self" else h
            msg = self.lib.anigpu_last_error(hh).decode() if hh is not None else ""
            raise AnigpuError(rc, msg)
        return rc

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.anigpu_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle):
        self._check(self.lib.anigpu_set_stream(self.h, ctypes.c_void_p(stream_handle)))

    def set_timing(self, enable=True):
        self._check(self.lib.anigpu_set_timing(self.h, 1 if enable else 0))

    def last_timing(self):
        """Per-phase device milliseconds of the last timed call."""
        import numpy as np
        ms = np.zeros(8)
        n = self._check(self.lib.anigpu_last_timing(self.h, ms.ctypes.data, 8))
        return ms[:n].tolist()

    def launch_count(self):
        return int(self.lib.anigpu_launch_count(self.h))

    def _dev(self, a, dtype):
        """numpy array or tensor -> contiguous CUDA tensor of dtype."""
        torch = self.torch
        if a is None:
            return None
        if not isinstance(a, torch.Tensor):
            a = torch.as_tensor(a)
        return a.to(device=f"cuda:{self.device}", dtype=dtype).contiguous()

    # -------------------------------------------------------------- element level
    @_streamed
    def fem3dtet(self, opA, opB, XY, D=None, kind=TENSOR_NULL, order=5, precision=F64, out=None):
        """Element matrices of a batch of tets: A[nt, nfA, nfB] whose per-tet memory is the
        column-major nfB x nfA DenseMatrix of fem3Dtet (so A[t].T is A(i_test, j_trial))."""
        torch = self.torch
        XY = self._dev(XY, torch.float64)
        nt = XY.numel() // 12
        nfA, _ = op_info(opA)
        nfB, _ = op_info(opB)
        dt = torch.float64 if precision == F64 else torch.float32
        if out is None:
            out = torch.empty((nt, nfA, nfB), dtype=dt, device=XY.device)
        Dd = self._dev(D, torch.float64) if D is not None else None
        self._check(self.lib.anigpu_fem3dtet(self.h, opA, opB, kind, order, precision, nt, _ptr(XY), _ptr(Dd),
                                             _ptr(out)))
        return out

    @_streamed
    def fem3dtet_custom(self, UA, XY, VB=None, D=None, kind=TENSOR_NULL, order=5, precision=F64, out=None):
        """Element matrices with user-defined operators (Ani::ApplyOpCustom): UA[nt, q, nfA, dimA]
        holds the A operator's values at the rule's points (quadrature_points gives them), VB the
        B operator's (None: B is A).  A[nt, nfA, nfB] as fem3dtet."""
        torch = self.torch
        XY = self._dev(XY, torch.float64)
        nt = XY.numel() // 12
        UA = self._dev(UA, torch.float64)
        nfA, dimA = int(UA.shape[-2]), int(UA.shape[-1])
        if VB is not None:
            VB = self._dev(VB, torch.float64)
            nfB, dimB = int(VB.shape[-2]), int(VB.shape[-1])
        else:
            nfB, dimB = nfA, dimA
        dt = torch.float64 if precision == F64 else torch.float32
        if out is None:
            out = torch.empty((nt, nfA, nfB), dtype=dt, device=XY.device)
        Dd = self._dev(D, torch.float64) if D is not None else None
        self._check(self.lib.anigpu_fem3dtet_custom(self.h, dimA, nfA, _ptr(UA), dimB, nfB, _ptr(VB), kind, order,
                                                    precision, nt, _ptr(XY), _ptr(Dd), _ptr(out)))
        return out

    @_streamed
    def quadrature_points(self, order, XY):
        torch = self.torch
        XY = self._dev(XY, torch.float64)
        nt = XY.numel() // 12
        q = quadrature(order)[1].size
        out = torch.empty((nt, q, 3), dtype=torch.float64, device=XY.device)
        self._check(self.lib.anigpu_quadrature_points(self.h, order, nt, _ptr(XY), _ptr(out)))
        return out

    @_streamed
    def fem3dface(self, opA, opB, XY, face, D=None, kind=TENSOR_NULL, order=5, precision=F64, out=None,
                  normal=False):
        """Face-integral element matrices (Ani::fem3Dface; Ani::fem3DfaceN with normal=True, the
        tensor then having 3*dimB rows contracted with the outward normal) over face `face` (0..3)
        of every tet: A[nt, nfA, nfB], the same layout as fem3dtet."""
        torch = self.torch
        XY = self._dev(XY, torch.float64)
        nt = XY.numel() // 12
        nfA, _ = op_info(opA)
        nfB, _ = op_info(opB)
        dt = torch.float64 if precision == F64 else torch.float32
        if out is None:
            out = torch.empty((nt, nfA, nfB), dtype=dt, device=XY.device)
        Dd = self._dev(D, torch.float64) if D is not None else None
        call = self.lib.anigpu_fem3dface_n if normal else self.lib.anigpu_fem3dface
        self._check(call(self.h, opA, opB, kind, order, precision, nt, _ptr(XY), face, _ptr(Dd), _ptr(out)))
        return out

    @_streamed
    def face_quadrature_points(self, order, face, XY):
        torch = self.torch
        XY = self._dev(XY, torch.float64)
        nt = XY.numel() // 12
        q = face_quadrature(order)[1].size
        out = torch.empty((nt, q, 3), dtype=torch.float64, device=XY.device)
        self._check(self.lib.anigpu_face_quadrature_points(self.h, order, face, nt, _ptr(XY), _ptr(out)))
        return out

    @_streamed
    def enumeration_setup(self, etype):
        """Renumbering of the set-up problem into enumeration etype (ENUM_*); returns
        (rowptr, col, perm) of the new template (perm: new index of each NATURAL DOF)."""
        torch = self.torch
        self._check(self.lib.anigpu_enumeration_setup(self.h, etype))
        dev = f"cuda:{self.device}"
        rp = torch.empty(self.ndof + 1, dtype=torch.int64, device=dev)
        col = torch.empty(self.nnz, dtype=torch.int32, device=dev)
        perm = torch.empty(self.ndof, dtype=torch.int64, device=dev)
        self._check(self.lib.anigpu_enumeration_template(self.h, _ptr(rp), _ptr(col), _ptr(perm)))
        return rp, col, perm

    @_streamed
    def enumeration_apply(self, vals, precision, rhs=None):
        """Values (and right-hand side) of an assembled NATURAL system in the set-up enumeration."""
        torch = self.torch
        vout = torch.empty_like(vals)
        rout = torch.empty_like(rhs) if rhs is not None else None
        self._check(self.lib.anigpu_enumeration_apply(self.h, _ptr(vals), precision, _ptr(rhs), _ptr(vout),
                                                      _ptr(rout)))
        return vout, rout

    @_streamed
    def enumeration_to_natural(self, x):
        torch = self.torch
        xd = self._dev(x, torch.float64)
        out = torch.empty_like(xd)
        self._check(self.lib.anigpu_enumeration_to_natural(self.h, _ptr(xd), _ptr(out)))
        return out

    @_streamed
    def fem3d_apply(self, op, XY, XYL, dofs):
        """Op(u) at barycentric points XYL[npts, 4] shared by every tet (Ani::fem3DapplyL):
        opU[nt, npts, dim] from the element DOF values dofs[nt, nf]."""
        torch = self.torch
        XY = self._dev(XY, torch.float64)
        nt = XY.numel() // 12
        _, dim = op_info(op)
        P = self._dev(XYL, torch.float64).reshape(-1, 4)
        d = self._dev(dofs, torch.float64)
        out = torch.empty((nt, P.shape[0], dim), dtype=torch.float64, device=XY.device)
        self._check(self.lib.anigpu_fem3d_apply(self.h, op, nt, _ptr(XY), P.shape[0], _ptr(P), _ptr(d), _ptr(out)))
        return out

    @_streamed
    def fem3d_apply_x(self, op, XY, X, dofs):
        """Op(u) at physical points X[nt, npts, 3] of each tet (Ani::fem3DapplyX)."""
        torch = self.torch
        XY = self._dev(XY, torch.float64)
        nt = XY.numel() // 12
        _, dim = op_info(op)
        Xd = self._dev(X, torch.float64).reshape(nt, -1, 3)
        d = self._dev(dofs, torch.float64)
        out = torch.empty((nt, Xd.shape[1], dim), dtype=torch.float64, device=XY.device)
        self._check(self.lib.anigpu_fem3d_apply_x(self.h, op, nt, _ptr(XY), Xd.shape[1], _ptr(Xd), _ptr(d),
                                                  _ptr(out)))
        return out

    @_streamed
    def eval_solution(self, op, x, XYL):
        """IDEN or GRAD of the global solution x of the set-up problem at barycentric points
        XYL[npts, 4] of every tet (oriented local order): opU[nt, npts, dim]."""
        torch = self.torch
        _, dim = op_info(10 * self.space + op)
        P = self._dev(XYL, torch.float64).reshape(-1, 4)
        xd = self._dev(x, torch.float64)
        out = torch.empty((self.nt, P.shape[0], dim), dtype=torch.float64, device=f"cuda:{self.device}")
        self._check(self.lib.anigpu_eval_solution(self.h, op, _ptr(xd), P.shape[0], _ptr(P), _ptr(out)))
        return out

    @_streamed
    def apply_dir(self, A, F, mask, bc=None):
        torch = self.torch
        nt, n = F.shape[0], F.shape[1]
        m = self._dev(mask, torch.int32)
        b = self._dev(bc, torch.float64) if bc is not None else None
        self._check(self.lib.anigpu_apply_dir(self.h, nt, n, _ptr(A), _ptr(F), _ptr(m), _ptr(b)))

    # -------------------------------------------------------------- global problem
    @_streamed
    def mesh_upload(self, xyz, tets):
        torch = self.torch
        self._xyz = self._dev(xyz, torch.float64)
        self._tets = self._dev(tets, torch.int32)
        self.nv = self._xyz.numel() // 3
        self.nt = self._tets.numel() // 4
        self._check(self.lib.anigpu_mesh_upload(self.h, self.nv, _ptr(self._xyz), self.nt, _ptr(self._tets)))

    @_streamed
    def update_coords(self, xyz):
        self._xyz = self._dev(xyz, self.torch.float64)
        self._check(self.lib.anigpu_mesh_update_coords(self.h, _ptr(self._xyz)))

    @_streamed
    def problem_setup(self, space):
        self._check(self.lib.anigpu_problem_setup(self.h, space))
        self.space = space
        nd, nz, ne = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        self._check(self.lib.anigpu_problem_info(self.h, ctypes.byref(nd), ctypes.byref(nz), ctypes.byref(ne)))
        self.ndof, self.nnz, self.nedges = nd.value, nz.value, ne.value
        return self.ndof, self.nnz

    def gather_layouts(self):
        """(rings, enabled): every P2 edge has a ring; the ring / interleaved gathers are used."""
        a, e = ctypes.c_int(), ctypes.c_int()
        self._check(self.lib.anigpu_gather_layouts(self.h, ctypes.byref(a), ctypes.byref(e)))
        return bool(a.value), bool(e.value)

    def set_gather_layouts(self, enable):
        self._check(self.lib.anigpu_set_gather_layouts(self.h, 1 if enable else 0))

    @_streamed
    def csr_template(self):
        torch = self.torch
        rp = torch.empty(self.ndof + 1, dtype=torch.int64, device=f"cuda:{self.device}")
        col = torch.empty(self.nnz, dtype=torch.int32, device=f"cuda:{self.device}")
        self._check(self.lib.anigpu_csr_template(self.h, _ptr(rp), _ptr(col)))
        return rp, col

    @_streamed
    def element_coords(self):
        """XY[nt, 12]: every tet's vertex coordinates in the library's reoriented local order."""
        torch = self.torch
        out = torch.empty((self.nt, 12), dtype=torch.float64, device=f"cuda:{self.device}")
        self._check(self.lib.anigpu_element_coords(self.h, _ptr(out)))
        return out

    @_streamed
    def element_dofs(self):
        torch = self.torch
        nloc = op_info(10 * self.space + IDEN)[0] if self.space not in (VEC3_P1, VEC3_P2) else 10
        e = torch.empty((self.nt, nloc), dtype=torch.int32, device=f"cuda:{self.device}")
        self._check(self.lib.anigpu_element_dofs(self.h, _ptr(e)))
        return e

    @_streamed
    def dof_coords(self):
        torch = self.torch
        c = torch.empty((self.ndof, 3), dtype=torch.float64, device=f"cuda:{self.device}")
        self._check(self.lib.anigpu_dof_coords(self.h, _ptr(c)))
        return c

    @_streamed
    def set_dirichlet(self, mask=None, bc=None):
        torch = self.torch
        self._dmask = self._dev(mask, torch.uint8) if mask is not None else None
        self._dbc = self._dev(bc, torch.float64) if bc is not None else None
        self._check(self.lib.anigpu_set_dirichlet(self.h, _ptr(self._dmask), _ptr(self._dbc)))

    @_streamed
    def assemble_general(self, opA, opB, kind=TENSOR_NULL, D=None, rhs_kind=None, F=None, order=4):
        """General-path spaces (P0, P3, CR1, B2, B4, ND0, RT0): FP64 values in the template and the
        right-hand side (rhs_kind None: no right-hand side)."""
        torch = self.torch
        dev = f"cuda:{self.device}"
        vals = torch.empty(self.nnz, dtype=torch.float64, device=dev)
        rhs = torch.empty(self.ndof, dtype=torch.float64, device=dev) if rhs_kind is not None else None
        Dd = self._dev(D, torch.float64) if D is not None else None
        Fd = self._dev(F, torch.float64) if F is not None else None
        self._check(self.lib.anigpu_assemble_general(self.h, opA, opB, kind, _ptr(Dd),
                                                     rhs_kind if rhs_kind is not None else 0, _ptr(Fd), order,
                                                     _ptr(vals), _ptr(rhs)))
        return vals, rhs

    @_streamed
    def assemble_elements(self, Aelem, Felem=None):
        """P1, P2, vector P2 and the general-path spaces: scatter of caller-computed element matrices
        Aelem[nt, nloc, nloc] (fem3dtet's layout, local unsigned basis, on element_coords()) and
        right-hand sides Felem[nt, nloc] (or None) into the template, FP64, with the orientation
        signs and Dirichlet DOFs applied (the local-assembler contract)."""
        torch = self.torch
        dev = f"cuda:{self.device}"
        A = self._dev(Aelem, torch.float64)
        Fd = self._dev(Felem, torch.float64) if Felem is not None else None
        vals = torch.empty(self.nnz, dtype=torch.float64, device=dev)
        rhs = torch.empty(self.ndof, dtype=torch.float64, device=dev) if Fd is not None else None
        self._check(self.lib.anigpu_assemble_elements(self.h, _ptr(A), _ptr(Fd), _ptr(vals), _ptr(rhs)))
        return vals, rhs

    @_streamed
    def assemble(self, kind=TENSOR_NULL, D=None, f=None, f_const=1.0, order=2, precision=F64, vals=None, rhs=None,
                 touched=False, drop=1e-100, sync=True):
        """AssemblerT::Assemble: returns (vals[nnz], rhs[ndof], touched[nnz] or None).  With
        sync=False the kernels are only enqueued; status() reports a non-finite value later."""
        torch = self.torch
        dev = f"cuda:{self.device}"
        dt = torch.float64 if precision == F64 else torch.float32
        if vals is None:
            vals = torch.empty(self.nnz, dtype=dt, device=dev)
        if rhs is None:
            rhs = torch.empty(self.ndof, dtype=torch.float64, device=dev)
        tch = torch.empty(self.nnz, dtype=torch.uint8, device=dev) if touched else None
        Dd = self._dev(D, torch.float64) if D is not None else None
        fd = self._dev(f, torch.float64) if f is not None else None
        fn = self.lib.anigpu_assemble if sync else self.lib.anigpu_assemble_async
        self._check(fn(self.h, kind, _ptr(Dd), _ptr(fd), float(f_const), order, precision, _ptr(vals), _ptr(rhs),
                       _ptr(tch), float(drop)))
        if not sync:
            self._keep = (Dd, fd)  # inputs stay alive until the enqueued kernels have read them
        return vals, rhs, tch

    # -------------------------------------------------------------- batched instances
    @_streamed
    def batch_set_instances(self, tet_offsets, vals_for_tuning=None):
        """The uploaded mesh is the disjoint union of instances; tet_offsets[i]..tet_offsets[i+1]
        are the tets of instance i.  Builds the instance map and tiles, autotunes on the values."""
        import numpy as np
        toff = np.ascontiguousarray(tet_offsets, dtype=np.int64)
        self.ninst = toff.size - 1
        self._check(self.lib.anigpu_batch_set_instances(self.h, self.ninst, toff.ctypes.data, _ptr(vals_for_tuning)))

    def batch_info(self):
        import numpy as np
        nt, lanes, loop = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        ms = np.zeros(4, dtype=np.float32)
        self._check(self.lib.anigpu_batch_info(self.h, ctypes.byref(nt), ctypes.byref(lanes), ms.ctypes.data,
                                               ctypes.byref(loop)))
        return dict(ntiles=nt.value, lanes_per_row=lanes.value, tune_ms=ms.tolist(), device_loop=loop.value)

    @_streamed
    def batch_run(self, b, kind=TENSOR_NULL, D=None, f=None, f_const=1.0, order=2, vals=None, assemble=True,
                  rtol=1e-8, maxit=100000, check=True):
        """Assemble (FP64, into vals) and solve every instance by Jacobi-PCG in one graph launch.
        Returns (x, vals, stats[ninst])."""
        torch = self.torch
        dev = f"cuda:{self.device}"
        if vals is None:
            vals = torch.empty(self.nnz, dtype=torch.float64, device=dev)
        rhs = torch.empty(self.ndof, dtype=torch.float64, device=dev) if assemble else None
        b = self._dev(b, torch.float64)
        x = torch.empty_like(b)
        Dd = self._dev(D, torch.float64) if D is not None else None
        fd = self._dev(f, torch.float64) if f is not None else None
        st = (SolveStats * self.ninst)()
        rc = self.lib.anigpu_batch_run(self.h, kind, _ptr(Dd), _ptr(fd), float(f_const), order, _ptr(vals), _ptr(rhs),
                                       _ptr(b), _ptr(x), float(rtol), int(maxit), ctypes.cast(st, ctypes.c_void_p))
        if check:
            self._check(rc)
        return x, vals, list(st)

    def batch_assembly_tuning(self):
        """(rows per block in warps of 32, [ms for 1, 2 warps]) of the batch's assembly."""
        import numpy as np
        w = ctypes.c_int()
        ms = np.zeros(2, dtype=np.float32)
        self._check(self.lib.anigpu_batch_assembly_tuning(self.h, ctypes.byref(w), ms.ctypes.data))
        return w.value, ms.tolist()

    def status(self):
        """Waits for the handle's stream; raises AnigpuError on a non-finite value recorded
        by an assembly since the last check."""
        self._check(self.lib.anigpu_status(self.h))

    @_streamed
    def csr_compact(self, rowptr, col, vals, precision, touched):
        n = ctypes.c_int64()
        self._check(self.lib.anigpu_csr_compact(self.h, _ptr(rowptr), _ptr(col), _ptr(vals), precision,
                                                _ptr(touched), ctypes.byref(n)))
        return n.value

    @_streamed
    def spmv(self, vals, x, precision=F64):
        torch = self.torch
        x = self._dev(x, torch.float64)
        y = torch.empty_like(x)
        self._check(self.lib.anigpu_spmv(self.h, _ptr(vals), precision, _ptr(x), _ptr(y)))
        return y

    @_streamed
    def solve(self, vals, b, method=SOLVE_JACOBI_PCG, precision=F64, x0=None, rtol=1e-10, maxit=100000,
              check=True):
        """Returns (x, stats).  stats: SolveStats (iterations, outer_iterations, rel_residual, seconds)."""
        torch = self.torch
        b = self._dev(b, torch.float64)
        x = torch.zeros_like(b) if x0 is None else self._dev(x0, torch.float64).clone()
        st = SolveStats()
        rc = self.lib.anigpu_solve(self.h, method, _ptr(vals), precision, _ptr(b), _ptr(x), float(rtol), int(maxit),
                                   ctypes.byref(st))
        if check:
            self._check(rc)
        return x, st

    def solve_refined(self, vals32, vals64, b, method=SOLVE_FCG_LEARNED, x0=None, rtol=1e-8, maxit=100000,
                      check=True):
        """Solve the FP64-assembled system vals64 with the FP32-assembled vals32 as the inner operator
        (anigpu_solve_refined): every residual replacement and the convergence test use FP64 b - A64 x."""
        torch = self.torch
        b = self._dev(b, torch.float64)
        x = torch.zeros_like(b) if x0 is None else self._dev(x0, torch.float64).clone()
        st = SolveStats()
        rc = self.lib.anigpu_solve_refined(self.h, method, _ptr(vals32), _ptr(vals64), _ptr(b), _ptr(x), float(rtol),
                                           int(maxit), ctypes.byref(st))
        if check:
            self._check(rc)
        return x, st


class BatchJob(ctypes.Structure):
    """anigpu_batch_job (include/anigpu.h)."""
    _fields_ = [("h", ctypes.c_void_p), ("tensor_kind", ctypes.c_int), ("D", ctypes.c_void_p),
                ("f", ctypes.c_void_p), ("f_const", ctypes.c_double), ("order", ctypes.c_int),
                ("vals", ctypes.c_void_p), ("rhs_assembled", ctypes.c_void_p), ("b", ctypes.c_void_p),
                ("x", ctypes.c_void_p), ("stats", ctypes.c_void_p)]


def batch_run_jobs(jobs, rtol=1e-8, maxit=100000, check=True):
    """Several batched jobs as one CUDA graph launch (anigpu_batch_run_jobs).  jobs: list of dicts
    with keys lib (an Anigpu with instances set), b, kind, D, f, f_const, order and optionally vals.
    Returns a list of (x, vals, stats) per job."""
    import torch
    arr = (BatchJob * len(jobs))()
    keep, out = [], []
    addr = lambda t: None if t is None else t.data_ptr()  # noqa: E731
    for k, j in enumerate(jobs):
        lib = j["lib"]
        dev = f"cuda:{lib.device}"
        vals = j.get("vals")
        if vals is None:
            vals = torch.empty(lib.nnz, dtype=torch.float64, device=dev)
        rhs = torch.empty(lib.ndof, dtype=torch.float64, device=dev)
        b = lib._dev(j["b"], torch.float64)
        x = torch.empty_like(b)
        D = lib._dev(j["D"], torch.float64) if j.get("D") is not None else None
        f = lib._dev(j["f"], torch.float64) if j.get("f") is not None else None
        st = (SolveStats * lib.ninst)()
        h = lib.h.value if isinstance(lib.h, ctypes.c_void_p) else lib.h
        arr[k] = BatchJob(h, j.get("kind", TENSOR_NULL), addr(D), addr(f), float(j.get("f_const", 1.0)),
                          j.get("order", 2), addr(vals), addr(rhs), addr(b), addr(x), ctypes.addressof(st))
        keep += [vals, rhs, b, x, D, f, st]
        out.append((x, vals, st))
    lib0 = jobs[0]["lib"]
    torch.cuda.synchronize()
    rc = lib0.lib.anigpu_batch_run_jobs(len(jobs), ctypes.cast(arr, ctypes.c_void_p), float(rtol), int(maxit))
    torch.cuda.synchronize()
    if check:
        lib0._check(rc)
    return [(x, vals, list(st)) for x, vals, st in out]


class LearnedPreconditioner:
    """Training and use of the learned preconditioner of ANIGPU_SOLVE_FCG_LEARNED on a handle.

    Mirrors nothing in the reference (its solves go through INMOST's ILU-Krylov); see
    include/anigpu.h for the network.  Parameters are a flat FP32 vector (checkpoint: save with
    get_params, restore with set_params)."""

    def __init__(self, lib, layers=4, act=BF16, seed=1234):
        self.lib = lib
        lib._check(lib.lib.anigpu_gnn_init(lib.h, layers, act, seed))
        self.nparam = int(lib.lib.anigpu_gnn_num_params(lib.h))
        self.step = 0

    def get_params(self):
        import numpy as np
        w = np.zeros(self.nparam, dtype=np.float32)
        self.lib._check(self.lib.lib.anigpu_gnn_get_params(self.lib.h, w.ctypes.data, self.nparam))
        return w

    def set_params(self, w):
        import numpy as np
        w = np.ascontiguousarray(w, dtype=np.float32)
        self.lib._check(self.lib.lib.anigpu_gnn_set_params(self.lib.h, w.ctypes.data, self.nparam))

    def get_grads(self):
        import numpy as np
        g = np.zeros(self.nparam, dtype=np.float32)
        self.lib._check(self.lib.lib.anigpu_gnn_get_grads(self.lib.h, g.ctypes.data, self.nparam))
        return g

    def zero_grads(self):
        self.lib._check(self.lib.lib.anigpu_gnn_zero_grads(self.lib.h))

    def bind(self, vals, precision, kind, D):
        with self.lib.on_stream():
            Dd = self.lib._dev(D, self.lib.torch.float64) if D is not None else None
            self._D = Dd
            self._vals = vals
            self.lib._check(self.lib.lib.anigpu_gnn_bind(self.lib.h, _ptr(vals), precision, kind, _ptr(Dd)))

    def apply(self, r):
        with self.lib.on_stream():
            r = self.lib._dev(r, self.lib.torch.float64)
            z = self.lib.torch.empty_like(r)
            self.lib._check(self.lib.lib.anigpu_gnn_apply(self.lib.h, _ptr(r), _ptr(z)))
        return z

    def apply_f32(self, r):
        """z = M r with the fused FP32 kernels the FCG solve runs."""
        with self.lib.on_stream():
            r = self.lib._dev(r, self.lib.torch.float32)
            z = self.lib.torch.empty_like(r)
            self.lib._check(self.lib.lib.anigpu_gnn_apply_f32(self.lib.h, _ptr(r), _ptr(z)))
        return z

    def coarse_chain(self, enable=None):
        """Whether the bound preconditioner runs its coarse products as one cooperative launch;
        enable=True/False selects it for the next bind."""
        a = ctypes.c_int()
        self.lib._check(self.lib.lib.anigpu_gnn_coarse_chain(self.lib.h, -1 if enable is None else int(bool(enable)),
                                                             ctypes.byref(a)))
        return bool(a.value)

    def coefficients(self):
        """The network output a, float32 [ncomp * nv, 4] (row c * nv + v: vertex v, component c)."""
        torch = self.lib.torch
        ncomp = 3 if self.lib.space in (VEC3_P1, VEC3_P2) else 1
        with self.lib.on_stream():
            a = torch.empty((ncomp * self.lib.nv, 4), dtype=torch.float32, device=f"cuda:{self.lib.device}")
            self.lib._check(self.lib.lib.anigpu_gnn_coefficients(self.lib.h, _ptr(a)))
        return a

    def loss_grad(self, r, e):
        loss = ctypes.c_double()
        with self.lib.on_stream():
            r = self.lib._dev(r, self.lib.torch.float64)
            e = self.lib._dev(e, self.lib.torch.float64)
            self.lib._check(self.lib.lib.anigpu_gnn_loss_grad(self.lib.h, _ptr(r), _ptr(e), ctypes.byref(loss)))
        return loss.value

    def adam(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8, grad_scale=1.0):
        self.step += 1
        with self.lib.on_stream():
            self.lib._check(self.lib.lib.anigpu_gnn_adam(self.lib.h, lr, b1, b2, eps, self.step, grad_scale))
