"""CPU tests: pin the oracle (the plain-C restatement) to the reference.

The restatement is checked against (a) the golden matrices of the reference's own unit
tests (tests/fem/operations/int_tet_test.cpp), (b) outputs of the reference's fem3Dtet
compiled from its sources, committed as fixtures (tests/golden/golden.npz, made by
tests/golden/gen_golden.py), and (c) the reference's quadrature tables.
"""
import itertools
import math

import numpy as np
import pytest

from helpers import KIND_CODE, op_nf_dim, parse_case, point_tensor, ref_tol, rel_err_per_tet


def test_golden_onepoint_tensor(restated, golden):
    # Operations_IntTet_OnePointTensor (int_tet_test.cpp:191-300): GRAD P3 x GRAD FemVec<3,P1>,
    # point-dependent general tensor, expected = integers / 720
    XY = golden["int_tet_test_tet_onepoint"].reshape(1, 12)
    exp = golden["int_tet_test_onepoint_12x20"] / golden["int_tet_test_onepoint_coef"]
    for order in (5, 6):
        q = restated.quad_points(order, XY)
        D = point_tensor(0, q, 9, 3)  # Ddims = (dim OpB, dim OpA) = (9, 3)
        A = restated.fem3dtet(32, 42, 5, order, XY, D)[0].T  # 12 x 20, A(i_test, j_trial)
        assert np.linalg.norm(A - exp) <= ref_tol(A), order


@pytest.mark.parametrize("kind", ["null", "cscalar", "tsym", "tgeneral"])
def test_golden_vecp1_identity(restated, golden, kind):
    # second golden matrix of the same test (int_tet_test.cpp:327-389): 12x12 / 1440, identity tensor
    XY = golden["int_tet_test_tet_onepoint"].reshape(1, 12)
    exp = golden["int_tet_test_vecp1_12x12"] / golden["int_tet_test_vecp1_coef"]
    D = {"null": None, "cscalar": np.array([1.0]), "tsym": None, "tgeneral": np.eye(9).reshape(1, 81)}[kind]
    code = KIND_CODE[kind]
    if kind == "tsym":
        pytest.skip("TET_SYM is 3x3; the 9x9 identity is covered by tgeneral")
    A = restated.fem3dtet(42, 42, code, 5, XY, D)[0].T
    assert np.linalg.norm(A - exp) <= ref_tol(A)


def test_golden_rhs_eval(restated, golden):
    # RhsEval (int_tet_test.cpp:448-500): int (mu k) phi_i = k * Bp with mu = 40
    XY = golden["int_tet_test_tet_rhs"].reshape(1, 12)
    Bp = golden["int_tet_test_rhs_Bp"]
    for k in (1, 3):
        A = restated.fem3dtet(1, 51, 1, 2, XY, np.array([40.0 * k]))[0, 0]
        assert np.linalg.norm(A - k * Bp) <= ref_tol(A)
    A = restated.fem3dtet(1, 51, 0, 2, XY)[0, 0]
    assert np.linalg.norm(A - Bp / 40) <= ref_tol(A)


def test_oracle_matches_reference_fem3dtet(restated, golden):
    """Every fixture case: the restatement equals the reference's fem3Dtet within 1e-12."""
    XY = golden["tets_XY"]
    worst = 0.0
    for name in golden["case_names"]:
        name = str(name)
        ca, cb, kind, order = parse_case(name)
        nfA, dA = op_nf_dim(ca)
        nfB, dB = op_nf_dim(cb)
        Aref = golden[f"case_{name}_A"]
        if kind.startswith("point"):
            fn = int(kind[5:])
            q = restated.quad_points(order, XY)
            D = point_tensor(fn, q, dB, dA)
            A = restated.fem3dtet(ca, cb, 5, order, XY, D)
        else:
            D = golden[f"case_{name}_D"] if f"case_{name}_D" in golden.files else None
            A = restated.fem3dtet(ca, cb, KIND_CODE[kind], order, XY, D)
        err = rel_err_per_tet(A, Aref)
        assert err <= 1e-12, (name, err)
    assert worst <= 1e-12


@pytest.mark.parametrize("order", range(21))
def test_quadrature_matches_reference(restated, golden, order):
    """Every tet rule (orders 0-20, the 8-point order-3 rule included) equals the reference's
    (tetrahedron_quadrature_formulas, quadrature_formulas.cpp:526-1502) as a set of (point,
    weight), to a unit in the last place."""
    p, w = restated.quadrature(order)
    pr, wr = golden[f"quad_{order}_p"], golden[f"quad_{order}_w"]
    a = np.c_[p, w]
    b = np.c_[pr, wr]
    assert a.shape == b.shape
    a = a[np.lexsort(a.T[::-1])]
    b = b[np.lexsort(b.T[::-1])]
    assert np.abs(a - b).max() <= 4e-16


def _monomial_check(p, w, deg, tol):
    # quadrature_formulas_test.cpp:7-45: exact for every monomial up to the rule's degree
    for a, b, c in itertools.product(range(deg + 1), repeat=3):
        if a + b + c > deg:
            continue
        exact = 6.0 * math.factorial(a) * math.factorial(b) * math.factorial(c) / math.factorial(a + b + c + 3)
        num = np.sum(w * p[:, 1] ** a * p[:, 2] ** b * p[:, 3] ** c)
        assert abs(num - exact) <= tol * max(1.0, exact), (a, b, c)


@pytest.mark.parametrize("order", range(21))
def test_quadrature_exactness(restated, order):
    p, w = restated.quadrature(order)
    deg = {0: 1, 4: 5}.get(order, order)
    assert np.all(w > 0) and p.min() >= 0 and abs(w.sum() - 1) <= 1e-14
    _monomial_check(p, w, deg, 1e-14 if order <= 6 else 1e-13)


def test_apply_dir(restated):
    # dc_on_dof_test.cpp semantics: F -= A(:,k) bc; F(k) = bc; zero row/column k; A(k,k) = 1
    rng = np.random.default_rng(0)
    A = rng.standard_normal((5, 5))
    F = rng.standard_normal(5)
    A0, F0 = A.copy(), F.copy()
    Ac = np.asfortranarray(A)  # column-major storage
    buf = np.ascontiguousarray(Ac.T)  # memory = column-major of A
    restated.apply_dir(buf, F, 2, 0.7)
    An = buf.T
    Fe = F0 - A0[:, 2] * 0.7
    Fe[2] = 0.7
    Ae = A0.copy()
    Ae[:, 2] = 0
    Ae[2, :] = 0
    Ae[2, 2] = 1
    assert np.allclose(An, Ae, atol=0, rtol=0)
    assert np.allclose(F, Fe, atol=1e-15)


def test_mesh_and_numbering(restated):
    from anigpu import meshgen
    n = 3
    xyz, tets = meshgen.kuhn_cube(n)
    t = restated.orient(xyz, tets)
    vol = np.linalg.det(np.stack([xyz[t[:, k]] - xyz[t[:, 3]] for k in range(3)], axis=1))
    assert np.all(vol > 0)
    ne, te = restated.edges(xyz.shape[0], t)
    # Euler characteristic of a ball: V - E + F - T = 1 ; faces from tets: F = (4T + boundary faces)/2
    nb = 2 * 6 * n * n
    F = (4 * t.shape[0] + nb) // 2
    assert xyz.shape[0] - ne + F - t.shape[0] == 1
    nd, ed = restated.element_dofs(2, xyz.shape[0], ne, t, te)
    assert nd == xyz.shape[0] + ne
    rp, col = restated.csr_template(nd, ed)
    # sorted rows, diagonal present, symmetric pattern
    for r in range(nd):
        row = col[rp[r]:rp[r + 1]]
        assert np.all(np.diff(row) > 0) and r in row
    pairs = set(zip(np.repeat(np.arange(nd), np.diff(rp)).tolist(), col.tolist()))
    assert all((c, r) in pairs for r, c in pairs)


def test_config1_counts(restated):
    from anigpu import meshgen
    xyz, tets = meshgen.kuhn_cube(16)
    assert xyz.shape[0] == 4913 and tets.shape[0] == 24576
    t = restated.orient(xyz, tets)
    nd, ed = restated.element_dofs(1, xyz.shape[0], 0, t, None)
    rp, col = restated.csr_template(nd, ed)
    assert col.size == 66961  # topological nnz of the 16^3 Kuhn P1 template


def test_oracle_pcg_solves_poisson(restated):
    from anigpu import meshgen
    xyz, tets = meshgen.kuhn_cube(6)
    prob = restated.assemble_problem(xyz, tets, 1, 0, None, 1.0, 2)
    mask = meshgen.boundary_mask(xyz)
    prob = restated.assemble_problem(xyz, tets, 1, 0, None, 1.0, 2, dirichlet=(mask, None))
    x, it, rel = restated.jacobi_pcg(prob["rowptr"], prob["col"], prob["vals"], prob["rhs"], 1e-10, 10000)
    assert it > 0 and rel <= 1e-10
    assert restated.true_residual(prob["rowptr"], prob["col"], prob["vals"], x, prob["rhs"]) <= 1e-9
    assert np.all(x[mask == 1] == 0)


def test_oracle_apply_matches_reference(restated, golden):
    """fem3DapplyL (shared barycentric points) and fem3DapplyX (physical points, some outside the
    tet) of the restatement against the reference's own (eval.inl:93-151), every operator code."""
    XY = golden["tets_XY"]
    for code in golden["apply_codes"]:
        code = int(code)
        dofs = golden[f"apply_{code}_dofs"]
        for key, pts, phys in (("L", golden["apply_XYL"], False), ("X", golden["apply_X"], True)):
            ref = golden[f"apply_{code}_{key}"]
            got = restated.fem3d_apply(code, XY, pts, dofs, phys=phys)
            assert got.shape == ref.shape
            scale = max(np.abs(ref).max(), 1e-300)
            assert np.abs(got - ref).max() <= 1e-13 * scale, (code, key)


@pytest.mark.parametrize("order", range(21))
def test_triangle_rules_match_reference(restated, golden, order):
    """The recomputed triangle rules of the face integrals equal the reference's
    (triangle_quadrature_formulas, quadrature_formulas.cpp:109) as sets of (point, weight)."""
    p, w = restated.tri_rule(order)
    pr, wr = golden[f"tri_{order}_p"], golden[f"tri_{order}_w"]
    assert p.shape == pr.shape
    for pt, wt in zip(pr, wr):
        d = np.abs(p - pt).max(axis=1)
        k = int(np.argmin(d))
        assert d[k] <= 1e-15 and abs(w[k] - wt) <= 1e-15
    assert abs(w.sum() - 1) <= 1e-15


def test_oracle_matches_reference_on_slivers(restated, golden):
    """Badly shaped tets (slivers, caps, needles, wedges down to |det|/(|e1||e2||e3|) ~ 1e-6): the
    restatement equals the reference's fem3Dtet within 1e-12 per tet."""
    XY = golden["sliver_XY"]
    for name in golden["sliver_case_names"]:
        name = str(name)
        ca, cb, kind, order = parse_case(name)
        D = golden[f"sliver_{name}_D"] if f"sliver_{name}_D" in golden.files else None
        A = restated.fem3dtet(ca, cb, KIND_CODE[kind], order, XY, D)
        err = rel_err_per_tet(A, golden[f"sliver_{name}_A"])
        assert err <= 1e-12, (name, err)


def _face_case(name):
    """'<codeA>_<codeB>_<kind>_o<order>_f<face>' -> its parts"""
    ca, cb, kname, o, f = name.split("_")
    return int(ca), int(cb), kname, int(o[1:]), int(f[1:])


def test_oracle_fem3dface_matches_reference(restated, golden):
    """fem3Dface of the restatement against the reference's own (int_face.inl:12-44): every face,
    orders 1-9, constant, per-tet and per-point tensors."""
    XY = golden["tets_XY"]
    for name in golden["face_case_names"]:
        ca, cb, kname, order, face = _face_case(str(name))
        if kname.startswith("point"):
            nfA, dA = op_nf_dim(ca)
            nfB, dB = op_nf_dim(cb)
            D = point_tensor(int(kname[5:]), restated.face_quad_points(order, face, XY), dB, dA)
            A = restated.fem3dface(ca, cb, 5, order, face, XY, D)
        else:
            D = golden[f"face_{name}_D"] if f"face_{name}_D" in golden.files else None
            A = restated.fem3dface(ca, cb, KIND_CODE[kname], order, face, XY, D)
        ref = golden[f"face_{name}_A"]
        err = rel_err_per_tet(A, ref)
        assert err <= 1e-12, (name, err)


def test_oracle_fem3dface_n_matches_reference(restated, golden):
    """fem3DfaceN (the tensor's 3*dimB rows contracted with the outward normal) of the restatement
    against the reference's own (int_face.inl:48-78): traction from a general tensor, normal
    derivative (NULL), flux (D grad u).n (SYM)."""
    XY = golden["tets_XY"]
    for name in golden["facen_case_names"]:
        ca, cb, kname, order, face = _face_case(str(name))
        D = golden[f"facen_{name}_D"] if f"facen_{name}_D" in golden.files else None
        A = restated.fem3dface(ca, cb, KIND_CODE[kname], order, face, XY, D, normal=True)
        err = rel_err_per_tet(A, golden[f"facen_{name}_A"])
        assert err <= 1e-12, (name, err)


def test_general_enumeration_perm_closed_form():
    """The oracle's lexicographic general-space enumerations: ANITYPE on P3 sends DOF k of edge e to
    nv + k*ne + e and leaves nodes and faces in place; every other type, and every other
    general-path space, is NATURAL."""
    from anigpu import meshgen
    from oracle.oracle import general_blocks, general_enumeration_perm
    xyz, t = meshgen.kuhn_cube(3, perturb=0.2, seed=12)
    per, off = general_blocks(xyz, t, 3)
    s = np.arange(off[4])
    nv, ne = off[1], (off[2] - off[1]) // 2
    exp = s.copy()
    m = (s >= nv) & (s < off[2])
    exp[m] = nv + ((s[m] - nv) % 2) * ne + (s[m] - nv) // 2
    assert np.array_equal(general_enumeration_perm(per, off, 0), exp)
    for etype in range(1, 6):
        assert np.array_equal(general_enumeration_perm(per, off, etype), s)
    for space in (0, 6, 7, 8, 9, 10):
        per, off = general_blocks(xyz, t, space)
        for etype in range(6):
            assert np.array_equal(general_enumeration_perm(per, off, etype), np.arange(off[4]))


@pytest.mark.parametrize("n,perturb", [(3, 0.0), (4, 0.2)])
def test_p2_edge_row_length_matches_its_ring(restated, n, perturb):
    """The invariant the GPU's ring walk relies on to skip clearing its row buffer: in the
    topological P2 template an edge row (A, B) holds exactly A, B, the edge itself, three columns
    per ring vertex (the vertex and its edges to A and B) and one per incident tet (the opposite
    edge) -- 3 + 3 V + n entries for V ring vertices and n tets."""
    from anigpu import meshgen
    xyz, tets = meshgen.kuhn_cube(n, perturb=perturb, seed=9)
    t = restated.orient(xyz, tets)
    nv = xyz.shape[0]
    ne, te = restated.edges(nv, t)
    ndof, edofs = restated.element_dofs(2, nv, ne, t, te)
    rp, col = restated.csr_template(ndof, edofs)
    EI, EJ = (0, 0, 0, 1, 1, 2), (1, 2, 3, 2, 3, 3)
    tets_of, ring = {}, {}
    for k in range(t.shape[0]):
        for le in range(6):
            e = int(te[k, le])
            a, b = t[k, EI[le]], t[k, EJ[le]]
            others = [int(v) for v in t[k] if v != a and v != b]
            tets_of[e] = tets_of.get(e, 0) + 1
            ring.setdefault(e, set()).update(others)
    for e, ntet in tets_of.items():
        r = nv + e
        assert rp[r + 1] - rp[r] == 3 + 3 * len(ring[e]) + ntet, e
