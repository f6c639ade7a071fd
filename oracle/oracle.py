"""ctypes binding of the oracle (test infrastructure only).

    Restated  -- oracle/_build/libanifem_oracle.so: the plain-C restatement (anifem_oracle.c)
    Reference -- oracle/_ref/libanifem_ref.so: the reference's own fem3Dtet compiled from its
                 sources (only where the reference sources exist; absent on GPU machines)

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
RESTATE_PATH = os.path.join(HERE, "_build", "libanifem_oracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libanifem_ref.so")

NULL, CONST_SCALAR, TET_SCALAR, TET_SYM, TET_GENERAL, POINT = range(6)

_vp, _i, _l, _d = ctypes.c_void_p, ctypes.c_int, ctypes.c_long, ctypes.c_double


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _apply(fn, nf_dim, code, XY, pts, dofs, phys):
    nf, dim = nf_dim
    XY = np.ascontiguousarray(XY, dtype=np.float64)
    nt = XY.size // 12
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    npts = pts.shape[-2] if phys else pts.shape[0]
    dofs = np.ascontiguousarray(dofs, dtype=np.float64).reshape(nt, nf)
    out = np.zeros((nt, npts, dim))
    rc = fn(code, nt, _p(XY), npts, _p(pts), 1 if phys else 0, _p(dofs), _p(out))
    assert rc == 0, rc
    return out


def build_restated():
    if not os.path.exists(RESTATE_PATH):
        subprocess.run(["make", "-C", HERE, "restate"], check=True, capture_output=True)


class Restated:
    def __init__(self):
        build_restated()
        L = ctypes.CDLL(RESTATE_PATH)
        L.orc_op_info.argtypes = [_i, ctypes.POINTER(_i), ctypes.POINTER(_i)]
        L.orc_quad_rule.argtypes = [_i, _vp, _vp, _i]
        L.orc_quad_points.argtypes = [_i, _l, _vp, _vp]
        L.orc_fem3dtet.argtypes = [_i, _i, _i, _i, _l, _vp, _vp, _vp]
        L.orc_apply_dir.argtypes = [_i, _vp, _vp, _i, _d]
        L.orc_fem3d_apply.argtypes = [_i, _l, _vp, _i, _vp, _i, _vp, _vp]
        L.orc_fem3dface.argtypes = [_i, _i, _i, _i, _i, _l, _vp, _vp, _vp]
        L.orc_face_quad_points.argtypes = [_i, _i, _l, _vp, _vp]
        L.orc_tri_rule.argtypes = [_i, _vp, _vp, _i]
        L.orc_fem3dface_n.argtypes = [_i, _i, _i, _i, _i, _l, _vp, _vp, _vp]
        L.orc_orient.argtypes = [_vp, _l, _vp]
        L.orc_edges.argtypes = [_l, _l, _vp, _vp]
        L.orc_edges.restype = _l
        L.orc_element_dofs.argtypes = [_i, _l, _l, _l, _vp, _vp, _vp]
        L.orc_element_dofs.restype = _l
        L.orc_csr_template.argtypes = [_l, _l, _i, _vp, _vp, _vp]
        L.orc_csr_template.restype = _l
        L.orc_scatter.argtypes = [_l, _vp, _vp, _l, _i, _vp, _vp, _vp, _d, _vp, _vp, _vp]
        L.orc_csr_compact.argtypes = [_l, _vp, _vp, _vp, _vp]
        L.orc_csr_compact.restype = _l
        L.orc_spmv.argtypes = [_l, _vp, _vp, _vp, _vp, _vp]
        L.orc_true_residual.argtypes = [_l, _vp, _vp, _vp, _vp, _vp]
        L.orc_true_residual.restype = _d
        L.orc_jacobi_pcg.argtypes = [_l, _vp, _vp, _vp, _vp, _vp, _d, _l, ctypes.POINTER(_d)]
        L.orc_jacobi_pcg.restype = _l
        L.orc_time_p2_sym.argtypes = [_l, _vp, _vp, _i, _i, _vp]
        L.orc_time_p2_sym.restype = _d
        L.orc_fem3dtet_mt.argtypes = [_i, _i, _i, _i, _l, _vp, _vp, _vp, _i]
        L.orc_apply_dir_elems.argtypes = [_l, _i, _vp, _vp, _vp, _vp, _vp, _i]
        L.orc_csr_template_mt.argtypes = [_l, _l, _i, _vp, _vp, _vp, _i]
        L.orc_csr_template_mt.restype = _l
        L.orc_scatter_mt.argtypes = [_l, _vp, _vp, _l, _i, _vp, _vp, _vp, _d, _vp, _vp, _vp, _i]
        L.orc_pcg_time_mt.argtypes = [_l, _vp, _vp, _vp, _vp, _l, _i]
        L.orc_pcg_time_mt.restype = _d
        self.L = L
        self.threads = os.cpu_count() or 1

    def op_info(self, code):
        nf, dim = _i(), _i()
        assert self.L.orc_op_info(code, ctypes.byref(nf), ctypes.byref(dim)) == 0
        return nf.value, dim.value

    def quadrature(self, order):
        p = np.zeros(4 * 1024)
        w = np.zeros(1024)
        n = self.L.orc_quad_rule(order, _p(p), _p(w), 1024)
        assert n > 0
        return p[:4 * n].reshape(n, 4).copy(), w[:n].copy()

    def quad_points(self, order, XY):
        XY = np.ascontiguousarray(XY, dtype=np.float64)
        nt = XY.size // 12
        q = self.quadrature(order)[1].size
        out = np.zeros((nt, q, 3))
        self.L.orc_quad_points(order, nt, _p(XY), _p(out))
        return out

    def fem3dtet(self, codeA, codeB, kind, order, XY, D=None):
        """A[nt, nfA, nfB] with the memory of the column-major nfB x nfA matrix per tet."""
        XY = np.ascontiguousarray(XY, dtype=np.float64)
        nt = XY.size // 12
        nfA, _ = self.op_info(codeA)
        nfB, _ = self.op_info(codeB)
        A = np.zeros((nt, nfA, nfB))
        Dd = None if D is None else np.ascontiguousarray(D, dtype=np.float64)
        rc = self.L.orc_fem3dtet(codeA, codeB, kind, order, nt, _p(XY), _p(Dd), _p(A))
        assert rc == 0, rc
        return A

    def apply_dir(self, A, F, k, bc):
        n = F.shape[0]
        self.L.orc_apply_dir(n, _p(A), _p(F), k, bc)

    def fem3dface(self, codeA, codeB, kind, order, face, XY, D=None, normal=False):
        """Face-integral element matrices (fem3Dface; fem3DfaceN with normal), same layout as fem3dtet."""
        XY = np.ascontiguousarray(XY, dtype=np.float64)
        nt = XY.size // 12
        nfA, _ = self.op_info(codeA)
        nfB, _ = self.op_info(codeB)
        A = np.zeros((nt, nfA, nfB))
        Dd = None if D is None else np.ascontiguousarray(D, dtype=np.float64)
        fn = self.L.orc_fem3dface_n if normal else self.L.orc_fem3dface
        rc = fn(codeA, codeB, kind, order, face, nt, _p(XY), _p(Dd), _p(A))
        assert rc == 0, rc
        return A

    def tri_rule(self, order):
        p = np.zeros(3 * 1024)
        w = np.zeros(1024)
        n = self.L.orc_tri_rule(order, _p(p), _p(w), 1024)
        assert n > 0
        return p[:3 * n].reshape(n, 3).copy(), w[:n].copy()

    def face_quad_points(self, order, face, XY):
        XY = np.ascontiguousarray(XY, dtype=np.float64)
        nt = XY.size // 12
        out = np.zeros(nt * 1024 * 3)
        q = self.L.orc_face_quad_points(order, face, nt, _p(XY), _p(out))
        assert q > 0
        return out[:nt * q * 3].reshape(nt, q, 3).copy()

    def fem3d_apply(self, code, XY, pts, dofs, phys=False):
        """Op(u) at points of each tet, opU[nt, npts, dim]: fem3DapplyL (pts [npts, 4] barycentric,
        shared) or fem3DapplyX (phys: pts [nt, npts, 3] physical)."""
        return _apply(self.L.orc_fem3d_apply, self.op_info(code), code, XY, pts, dofs, phys)

    def orient(self, xyz, tets):
        t = np.ascontiguousarray(tets, dtype=np.int32).copy()
        self.L.orc_orient(_p(np.ascontiguousarray(xyz, dtype=np.float64)), t.shape[0], _p(t))
        return t

    def edges(self, nv, tets):
        tets = np.ascontiguousarray(tets, dtype=np.int32)
        te = np.zeros((tets.shape[0], 6), dtype=np.int32)
        ne = self.L.orc_edges(nv, tets.shape[0], _p(tets), _p(te))
        return ne, te

    def element_dofs(self, space, nv, ne, tets, tet_edges):
        tets = np.ascontiguousarray(tets, dtype=np.int32)
        nloc = {1: 4, 2: 10, 5: 30}[space]
        e = np.zeros((tets.shape[0], nloc), dtype=np.int32)
        if space != 1 and tet_edges is None:
            raise ValueError("element_dofs: spaces with edge DOFs need the tet edge table")
        te = np.ascontiguousarray(tet_edges, dtype=np.int32) if tet_edges is not None else np.zeros((1, 6), np.int32)
        nd = self.L.orc_element_dofs(space, nv, ne, tets.shape[0], _p(tets), _p(te), _p(e))
        return nd, e

    def csr_template(self, ndof, edofs):
        edofs = np.ascontiguousarray(edofs, dtype=np.int32)
        nt, nloc = edofs.shape
        rp = np.zeros(ndof + 1, dtype=np.int64)
        nnz = self.L.orc_csr_template(ndof, nt, nloc, _p(edofs), _p(rp), None)
        col = np.zeros(nnz, dtype=np.int32)
        self.L.orc_csr_template(ndof, nt, nloc, _p(edofs), _p(rp), _p(col))
        return rp, col

    def scatter(self, rowptr, col, edofs, Aelem, Felem=None, drop=1e-100):
        edofs = np.ascontiguousarray(edofs, dtype=np.int32)
        nt, nloc = edofs.shape
        n = rowptr.size - 1
        vals = np.zeros(col.size)
        rhs = np.zeros(n)
        touched = np.zeros(col.size, dtype=np.uint8)
        Ae = np.ascontiguousarray(Aelem, dtype=np.float64)
        Fe = None if Felem is None else np.ascontiguousarray(Felem, dtype=np.float64)
        rc = self.L.orc_scatter(n, _p(rowptr), _p(col), nt, nloc, _p(edofs), _p(Ae), _p(Fe), drop, _p(vals), _p(rhs),
                                _p(touched))
        return rc, vals, rhs, touched

    def csr_compact(self, rowptr, col, vals, touched):
        rp, c, v = rowptr.copy(), col.copy(), vals.copy()
        nnz = self.L.orc_csr_compact(rp.size - 1, _p(rp), _p(c), _p(v), _p(np.ascontiguousarray(touched)))
        return rp, c[:nnz], v[:nnz]

    def spmv(self, rowptr, col, vals, x):
        y = np.zeros(rowptr.size - 1)
        self.L.orc_spmv(y.size, _p(rowptr), _p(col), _p(np.ascontiguousarray(vals, dtype=np.float64)),
                        _p(np.ascontiguousarray(x, dtype=np.float64)), _p(y))
        return y

    def true_residual(self, rowptr, col, vals, x, b):
        return self.L.orc_true_residual(rowptr.size - 1, _p(rowptr), _p(col),
                                        _p(np.ascontiguousarray(vals, dtype=np.float64)),
                                        _p(np.ascontiguousarray(x, dtype=np.float64)),
                                        _p(np.ascontiguousarray(b, dtype=np.float64)))

    def jacobi_pcg(self, rowptr, col, vals, b, rtol, maxit):
        x = np.zeros(rowptr.size - 1)
        rel = _d()
        it = self.L.orc_jacobi_pcg(x.size, _p(rowptr), _p(col), _p(np.ascontiguousarray(vals, dtype=np.float64)),
                                   _p(np.ascontiguousarray(b, dtype=np.float64)), _p(x), rtol, maxit,
                                   ctypes.byref(rel))
        return x, it, rel.value

    def time_p2_sym(self, XY, D6, order, nthreads):
        XY = np.ascontiguousarray(XY, dtype=np.float64)
        D6 = np.ascontiguousarray(D6, dtype=np.float64)
        nt = XY.size // 12
        A = np.zeros((nt, 100))
        sec = self.L.orc_time_p2_sym(nt, _p(XY), _p(D6), order, nthreads, _p(A))
        return sec, A

    # ---- the whole restated assembler for a scalar problem (P1 or P2)
    def assemble_problem(self, xyz, tets, space, kind, D, f_const, order, dirichlet=None, f=None):
        """orient -> numbering -> template -> element matrices + rhs -> applyDir -> scatter.
        Returns dict(rowptr, col, vals, rhs, touched, edofs, ndof)."""
        nv = xyz.shape[0]
        t = self.orient(xyz, tets)
        ne, te = self.edges(nv, t) if space in (2, 5) else (0, None)
        ndof, ed = self.element_dofs(space, nv, ne, t, te)
        rp, col = self.csr_template(ndof, ed)
        XY = np.ascontiguousarray(xyz[t].reshape(-1, 12))
        code = 10 * space + 2
        A = self.fem3dtet(code, code, kind, order, XY, D)  # [nt, nf, nf] (col-major per tet)
        rhs_code = 10 * space + 1
        if f is None:
            F = self.fem3dtet(1, rhs_code, CONST_SCALAR, order, XY, np.array([f_const]))[:, 0, :]
        else:
            F = self.fem3dtet(1, rhs_code, TET_SCALAR, order, XY, np.asarray(f, dtype=np.float64))[:, 0, :]
        F = np.ascontiguousarray(F)
        if dirichlet is not None:
            mask, bc = dirichlet
            for tt in range(ed.shape[0]):
                for k in range(ed.shape[1]):
                    d = ed[tt, k]
                    if mask[d]:
                        self.apply_dir(A[tt], F[tt], k, float(bc[d]) if bc is not None else 0.0)
        rc, vals, rhs, touched = self.scatter(rp, col, ed, A, F)
        assert rc == 0, rc
        return dict(rowptr=rp, col=col, vals=vals, rhs=rhs, touched=touched, edofs=ed, ndof=ndof, oriented=t,
                    nedges=ne)


    # ---- multi-threaded drivers (bitwise equal to the serial ones), for full-size checks
    def fem3dtet_mt(self, codeA, codeB, kind, order, XY, D=None, threads=None):
        XY = np.ascontiguousarray(XY, dtype=np.float64)
        nt = XY.size // 12
        nfA, _ = self.op_info(codeA)
        nfB, _ = self.op_info(codeB)
        A = np.zeros((nt, nfA, nfB))
        Dd = None if D is None else np.ascontiguousarray(D, dtype=np.float64)
        rc = self.L.orc_fem3dtet_mt(codeA, codeB, kind, order, nt, _p(XY), _p(Dd), _p(A), threads or self.threads)
        assert rc == 0, rc
        return A

    def assemble_problem_mt(self, xyz, tets, space, kind, D, f_const, order, dirichlet=None, threads=None):
        """assemble_problem on all host threads: the same numbers (element loop and scatter split
        over tets and rows), for meshes of millions of tets."""
        import time
        th = threads or self.threads
        sec = {}
        t0 = time.perf_counter()
        nv = xyz.shape[0]
        t = self.orient(xyz, tets)
        ne, te = self.edges(nv, t) if space in (2, 5) else (0, None)
        ndof, ed = self.element_dofs(space, nv, ne, t, te)
        nloc = ed.shape[1]
        rp = np.zeros(ndof + 1, dtype=np.int64)
        nnz = self.L.orc_csr_template_mt(ndof, ed.shape[0], nloc, _p(ed), _p(rp), None, th)
        col = np.zeros(nnz, dtype=np.int32)
        self.L.orc_csr_template_mt(ndof, ed.shape[0], nloc, _p(ed), _p(rp), _p(col), th)
        XY = np.ascontiguousarray(xyz[t].reshape(-1, 12))
        t1 = time.perf_counter()
        sec["setup"] = t1 - t0
        code = 10 * space + 2
        A = self.fem3dtet_mt(code, code, kind, order, XY, D, th)
        F = np.ascontiguousarray(self.fem3dtet_mt(1, 10 * space + 1, CONST_SCALAR, order, XY, np.array([f_const]),
                                                  th)[:, 0, :])
        t2 = time.perf_counter()
        sec["elements"] = t2 - t1
        if dirichlet is not None:
            mask, bc = dirichlet
            mask = np.ascontiguousarray(mask, dtype=np.uint8)
            bcv = None if bc is None else np.ascontiguousarray(bc, dtype=np.float64)
            self.L.orc_apply_dir_elems(ed.shape[0], nloc, _p(A), _p(F), _p(ed), _p(mask), _p(bcv), th)
        t3 = time.perf_counter()
        sec["dirichlet"] = t3 - t2
        vals = np.zeros(nnz)
        rhs = np.zeros(ndof)
        rc = self.L.orc_scatter_mt(ndof, _p(rp), _p(col), ed.shape[0], nloc, _p(ed), _p(A), _p(F), 1e-100, _p(vals),
                                   _p(rhs), None, th)
        sec["scatter"] = time.perf_counter() - t3
        assert rc == 0, rc
        return dict(rowptr=rp, col=col, vals=vals, rhs=rhs, edofs=ed, ndof=ndof, oriented=t, nedges=ne, seconds=sec,
                    threads=th)

    def pcg_seconds_per_iteration(self, rowptr, col, vals, b, iters=20, threads=None):
        """Wall seconds per FP64 Jacobi-PCG iteration on all host threads (the CPU baseline of the
        solve; a restatement: the reference solves through INMOST)."""
        sec = self.L.orc_pcg_time_mt(rowptr.size - 1, _p(rowptr), _p(col),
                                     _p(np.ascontiguousarray(vals, dtype=np.float64)),
                                     _p(np.ascontiguousarray(b, dtype=np.float64)), iters, threads or self.threads)
        return sec / iters


class Reference:
    """The reference's own fem3Dtet (only where oracle/_ref/libanifem_ref.so was built)."""

    @staticmethod
    def available():
        return os.path.exists(REF_PATH)

    def __init__(self):
        L = ctypes.CDLL(REF_PATH)
        L.ref_fem3dtet.argtypes = [_i, _i, _i, _i, _l, _vp, _vp, _i, _vp]
        L.ref_quadrature.argtypes = [_i, _vp, _vp, _i]
        L.ref_applyDir.argtypes = [_vp, _vp, _i, _i, _d]
        L.ref_time_p2_sym.argtypes = [_l, _vp, _vp, _i, _i, _vp]
        L.ref_time_p2_sym.restype = _d
        L.ref_fem3d_apply.argtypes = [_i, _l, _vp, _i, _vp, _i, _vp, _vp]
        L.ref_fem3dface.argtypes = [_i, _i, _i, _i, _i, _l, _vp, _vp, _i, _vp]
        L.ref_fem3dface_n.argtypes = [_i, _i, _i, _i, _i, _l, _vp, _vp, _i, _vp]
        L.ref_tri_quadrature.argtypes = [_i, _vp, _vp, _i, _vp]
        self.L = L

    def fem3dtet(self, codeA, codeB, kind, order, XY, D=None, fn=0, nfA=None, nfB=None):
        XY = np.ascontiguousarray(XY, dtype=np.float64)
        nt = XY.size // 12
        A = np.zeros((nt, nfA, nfB))
        Dd = None if D is None else np.ascontiguousarray(D, dtype=np.float64)
        rc = self.L.ref_fem3dtet(codeA, codeB, kind, order, nt, _p(XY), _p(Dd), fn, _p(A))
        assert rc == 0, rc
        return A

    def fem3dface(self, codeA, codeB, kind, order, face, XY, D=None, fn=0, nfA=None, nfB=None, normal=False):
        XY = np.ascontiguousarray(XY, dtype=np.float64)
        nt = XY.size // 12
        A = np.zeros((nt, nfA, nfB))
        Dd = None if D is None else np.ascontiguousarray(D, dtype=np.float64)
        call = self.L.ref_fem3dface_n if normal else self.L.ref_fem3dface
        rc = call(codeA, codeB, kind, order, face, nt, _p(XY), _p(Dd), fn, _p(A))
        assert rc == 0, rc
        return A

    def tri_quadrature(self, order):
        p = np.zeros(3 * 1024)
        w = np.zeros(1024)
        sym = np.zeros(3, dtype=np.int32)
        n = self.L.ref_tri_quadrature(order, _p(p), _p(w), 1024, _p(sym))
        assert n > 0
        return p[:3 * n].reshape(n, 3).copy(), w[:n].copy()

    def fem3d_apply(self, code, XY, pts, dofs, nf, dim, phys=False):
        return _apply(self.L.ref_fem3d_apply, (nf, dim), code, XY, pts, dofs, phys)

    def quadrature(self, order):
        p = np.zeros(4 * 1024)
        w = np.zeros(1024)
        n = self.L.ref_quadrature(order, _p(p), _p(w), 1024)
        return p[:4 * n].reshape(n, 4).copy(), w[:n].copy()

    def time_p2_sym(self, XY, D6, order, nthreads):
        XY = np.ascontiguousarray(XY, dtype=np.float64)
        D6 = np.ascontiguousarray(D6, dtype=np.float64)
        nt = XY.size // 12
        A = np.zeros((nt, 100))
        sec = self.L.ref_time_p2_sym(nt, _p(XY), _p(D6), order, nthreads, _p(A))
        return sec, A


# GlobEnumeration::ASSEMBLING_TYPE key orders (anifem++/inmost_interface/global_enumerator.h:392-404):
# the DOFs are sorted lexicographically by these fields of their natural index
_ENUM_KEYS = {
    0: ("ELEM_TYPE", "VAR", "DIM", "DOF_ID", "ELEM_ID"),   # ANITYPE
    1: ("ELEM_TYPE", "ELEM_ID", "VAR", "DIM", "DOF_ID"),   # MINIBLOCKS
    2: ("VAR", "DIM", "ELEM_TYPE", "ELEM_ID", "DOF_ID"),   # NATURAL
    3: ("VAR", "ELEM_TYPE", "ELEM_ID", "DOF_ID", "DIM"),   # DIMUNION
    4: ("ELEM_TYPE", "VAR", "DIM", "ELEM_ID", "DOF_ID"),   # BYELEMTYPE
    5: ("ELEM_TYPE", "VAR", "ELEM_ID", "DOF_ID", "DIM"),   # ETDIMBLOCKS
}


def enumeration_perm(nv, nds, ncomp, etype):
    """New index of every NATURAL DOF (component c, scalar DOF s: a node for s < nv, else edge
    s - nv) under enumeration etype: the rank of its natural index (VAR 0, DIM c, ELEM_TYPE node 0 /
    edge 1, ELEM_ID, DOF_ID 0) in the lexicographic order of that type's key."""
    n = nds * ncomp
    R = np.arange(n)
    c, s = R // nds, R % nds
    fields = {"VAR": np.zeros(n, dtype=np.int64), "DIM": c, "ELEM_TYPE": (s >= nv).astype(np.int64),
              "ELEM_ID": np.where(s < nv, s, s - nv), "DOF_ID": np.zeros(n, dtype=np.int64)}
    keys = [fields[k] for k in _ENUM_KEYS[etype]]
    order = np.lexsort(keys[::-1])  # the first field is the most significant
    perm = np.empty(n, dtype=np.int64)
    perm[order] = np.arange(n)
    return perm


def permute_csr(rowptr, col, vals, perm):
    """P A P^T of a CSR matrix (rows and columns renumbered by perm), rows sorted by column."""
    n = rowptr.size - 1
    rows = np.repeat(np.arange(n), np.diff(rowptr))
    nr, nc = perm[rows], perm[col]
    order = np.lexsort((nc, nr))
    rp = np.zeros(n + 1, dtype=np.int64)
    np.add.at(rp, nr + 1, 1)
    return np.cumsum(rp), nc[order].astype(np.int32), np.asarray(vals)[order]


# ---------------------------------------------------------------- general-path spaces
# DOFs per (node, edge, face, cell) and local DOFs per tet of the general-path spaces
_GEN_LAYOUT = {0: ((0, 0, 0, 1), 1), 3: ((1, 2, 1, 0), 20), 6: ((0, 0, 1, 0), 4), 7: ((0, 1, 0, 0), 6),
               8: ((0, 0, 0, 1), 1), 9: ((0, 1, 0, 0), 6), 10: ((0, 0, 1, 0), 4)}
_EI, _EJ = [0, 0, 0, 1, 1, 2], [1, 2, 3, 2, 3, 3]
_FV = [(0, 1, 2), (1, 2, 3), (0, 2, 3), (0, 1, 3)]
_FOPP = [3, 0, 1, 2]


def _local_dofs(space):
    """(entity type 0 node / 1 edge / 2 face / 3 cell, local entity, DOF within the entity) per local DOF"""
    if space == 3:
        return [(0, v, 0) for v in range(4)] + [(1, e, k) for e in range(6) for k in range(2)] + \
               [(2, f, 0) for f in range(4)]
    if space in (6, 10):
        return [(2, f, 0) for f in range(4)]
    if space in (7, 9):
        return [(1, e, 0) for e in range(6)]
    return [(3, 0, 0)]


def general_numbering(xyz, t, space):
    """Global DOF and orientation sign of every (tet, local DOF) of a general-path space on the
    oriented tets t (NATURAL: nodes, edges ranked by (min, max), faces ranked by sorted triples,
    cells; P3 edge pairs in the global edge direction; ND0 / RT0 signs; see the library's
    k_general.cu for the convention)."""
    nv, nt = xyz.shape[0], t.shape[0]
    per, nloc = _GEN_LAYOUT[space]
    ek = np.stack([np.minimum(t[:, _EI], t[:, _EJ]), np.maximum(t[:, _EI], t[:, _EJ])], axis=-1).astype(np.int64)
    ekey = ek[..., 0] * nv + ek[..., 1]
    ue, eid = np.unique(ekey.reshape(-1), return_inverse=True)
    eid = eid.reshape(nt, 6)
    ft = np.sort(np.stack([t[:, list(f)] for f in _FV], axis=1), axis=-1).astype(np.int64)
    fkey = (ft[..., 0] * nv + ft[..., 1]) * nv + ft[..., 2]
    uf, fid = np.unique(fkey.reshape(-1), return_inverse=True)
    fid = fid.reshape(nt, 4)
    ne, nf = ue.size, uf.size
    off = [0, nv * per[0], nv * per[0] + ne * per[1], nv * per[0] + ne * per[1] + nf * per[2]]
    ndof = off[3] + nt * per[3]
    gd = np.zeros((nt, nloc), dtype=np.int64)
    sg = np.ones((nt, nloc), dtype=np.int64)
    for i, (typ, ent, k) in enumerate(_local_dofs(space)):
        if typ == 0:
            gd[:, i] = off[0] + t[:, ent] * per[0] + k
        elif typ == 1:
            I, J = t[:, _EI[ent]], t[:, _EJ[ent]]
            kk = np.where((per[1] == 2) & (I > J), 1 - k, k)
            gd[:, i] = off[1] + eid[:, ent] * per[1] + kk
            if space == 9:
                sg[:, i] = np.where(I < J, 1, -1)
        elif typ == 2:
            gd[:, i] = off[2] + fid[:, ent] * per[2] + k
            if space == 10:
                a, b, c = ft[:, ent, 0], ft[:, ent, 1], ft[:, ent, 2]
                n = np.cross(xyz[b] - xyz[a], xyz[c] - xyz[a])
                d = np.einsum("ij,ij->i", n, xyz[t[:, _FV[ent][0]]] - xyz[t[:, _FOPP[ent]]])
                sg[:, i] = np.where(d > 0, 1, -1)
        else:
            gd[:, i] = off[3] + np.arange(nt) * per[3] + k
    return gd, sg, ndof


def general_blocks(xyz, t, space):
    """DOFs per entity (node, edge, face, cell) of a general-path space and the first NATURAL DOF of
    each entity block, off[4] = ndof."""
    nv, nt = xyz.shape[0], t.shape[0]
    per, _ = _GEN_LAYOUT[space]
    ek = np.stack([np.minimum(t[:, _EI], t[:, _EJ]), np.maximum(t[:, _EI], t[:, _EJ])], axis=-1).astype(np.int64)
    ne = np.unique((ek[..., 0] * nv + ek[..., 1]).reshape(-1)).size
    ft = np.sort(np.stack([t[:, list(f)] for f in _FV], axis=1), axis=-1).astype(np.int64)
    nf = np.unique(((ft[..., 0] * nv + ft[..., 1]) * nv + ft[..., 2]).reshape(-1)).size
    counts = [nv, ne, nf, nt]
    off = [0]
    for T in range(4):
        off.append(off[-1] + counts[T] * per[T])
    return list(per), off


def general_enumeration_perm(per, off, etype):
    """New index of every NATURAL DOF of a general-path space (one scalar variable) under
    enumeration etype: the rank of (VAR 0, DIM 0, ELEM_TYPE, ELEM_ID, DOF_ID) in the lexicographic
    order of that type's key (global_enumerator.h:392-404)."""
    n = off[4]
    s = np.arange(n)
    T = np.zeros(n, dtype=np.int64)
    for q in range(1, 4):
        T = np.where(s >= off[q], q, T)
    p = np.maximum(np.asarray(per)[T], 1)
    r = s - np.asarray(off)[T]
    fields = {"VAR": np.zeros(n, dtype=np.int64), "DIM": np.zeros(n, dtype=np.int64), "ELEM_TYPE": T,
              "ELEM_ID": r // p, "DOF_ID": r % p}
    keys = [fields[k] for k in _ENUM_KEYS[etype]]
    order = np.lexsort(keys[::-1])
    perm = np.empty(n, dtype=np.int64)
    perm[order] = np.arange(n)
    return perm


def general_assemble(restated, xyz, tets, space, codeA, codeB, kind, D, order, rhs_kind=None, F=None,
                     dirichlet=None):
    """Restatement of the general-path global assembly: signed sum of fem3Dtet element matrices
    (and fem3Dtet<IDEN P0, IDEN space> right-hand sides) into the template of all element pairs,
    Dirichlet rows / columns as the library's paths do.  Returns dict(rowptr, col, vals, rhs, gdof,
    sign, ndof, oriented)."""
    t = restated.orient(xyz, tets)
    gd, sg, ndof = general_numbering(xyz, t, space)
    nt, nloc = gd.shape
    XY = np.ascontiguousarray(xyz[t].reshape(-1, 12))
    A = restated.fem3dtet(codeA, codeB, kind, order, XY, D)            # A[t, j, i] = A_t(i, j)
    rows = np.repeat(gd, nloc, axis=1).reshape(-1)                      # (t, i, j) -> g_i
    cols = np.tile(gd, (1, nloc)).reshape(-1)                           # (t, i, j) -> g_j
    w = (sg[:, :, None] * sg[:, None, :]).reshape(-1) * np.transpose(A, (0, 2, 1)).reshape(-1)
    key = rows * ndof + cols
    uk, inv = np.unique(key, return_inverse=True)
    vals = np.zeros(uk.size)
    np.add.at(vals, inv, w)
    r, c = uk // ndof, uk % ndof
    rowptr = np.zeros(ndof + 1, dtype=np.int64)
    np.add.at(rowptr, r + 1, 1)
    rowptr = np.cumsum(rowptr)
    col = c.astype(np.int32)
    rhs = np.zeros(ndof)
    if rhs_kind is not None:
        Fe = restated.fem3dtet(1, 10 * space + 1, rhs_kind, order, XY, F)[:, 0, :]
        np.add.at(rhs, gd.reshape(-1), (sg * Fe).reshape(-1))
    if dirichlet is not None:
        mask, bc = dirichlet
        bc = np.zeros(ndof) if bc is None else np.asarray(bc, dtype=np.float64)
        cnt = np.bincount(gd.reshape(-1), minlength=ndof)
        for row in range(ndof):
            sl = slice(rowptr[row], rowptr[row + 1])
            if mask[row]:
                vals[sl] = 0.0
                vals[sl][col[sl] == row] = cnt[row]
                rhs[row] = cnt[row] * bc[row]
            else:
                m = mask[col[sl]].astype(bool)
                rhs[row] -= np.sum(vals[sl][m] * bc[col[sl][m]])
                v = vals[sl]
                v[m] = 0.0
    return dict(rowptr=rowptr, col=col, vals=vals, rhs=rhs, gdof=gd, sign=sg, ndof=ndof, oriented=t)
