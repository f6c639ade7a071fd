"""GPU checks of the general-path global assembly (P0, P3, CR1, B2, B4, ND0, RT0 with oriented
DOFs): the template, values and right-hand side against the oracle's restatement, and exactness
checks that exercise the orientation rules without the oracle (a P3 solution reproduces a
quadratic field, CR1 a linear one, ND0 and RT0 a constant vector field)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (space, opA, opB, tensor kind) of the parity cases
CASES = [(3, 32, 32, 0), (3, 31, 31, 2), (6, 62, 62, 0), (7, 72, 72, 3), (8, 81, 81, 0), (0, 1, 1, 2),
         (9, 94, 94, 0), (9, 91, 91, 3), (10, 103, 103, 0), (10, 101, 101, 3)]


def _mesh(n, seed=3):
    from anigpu import meshgen
    return meshgen.kuhn_cube(n, perturb=0.2, seed=seed)


@pytest.mark.parametrize("space,opA,opB,kind", CASES)
@pytest.mark.parametrize("with_dir", [False, True])
def test_general_assembly_matches_oracle(lib, restated, space, opA, opB, kind, with_dir):
    from anigpu import meshgen
    from oracle.oracle import general_assemble
    xyz, tets = _mesh(3)
    nt = tets.shape[0]
    D = None
    if kind == 2:
        D = np.exp(meshgen.normal(17, nt))
    elif kind == 3:
        D = meshgen.aniso_tensors(nt, 1.0, 18)
    lib.mesh_upload(xyz, tets)
    ndof, nnz = lib.problem_setup(space)
    dirichlet = None
    if with_dir:
        coords = lib.dof_coords().cpu().numpy()
        mask = meshgen.boundary_mask(coords)
        bc = (0.3 + coords[:, 0] - 0.5 * coords[:, 2]) * mask
        lib.set_dirichlet(mask, bc)
        dirichlet = (mask, bc)
    rhs_kind, F = (4, np.tile([0.5, -1.0, 2.0], (nt, 1))) if space in (9, 10) else (1, np.array([1.5]))
    vals, rhs = lib.assemble_general(opA, opB, kind, D, rhs_kind, F, 4)
    ref = general_assemble(restated, xyz, tets, space, opA, opB, kind, D, 4, rhs_kind, F, dirichlet)
    rp, col = lib.csr_template()
    assert ndof == ref["ndof"] and nnz == ref["rowptr"][-1]
    assert np.array_equal(rp.cpu().numpy(), ref["rowptr"]) and np.array_equal(col.cpu().numpy(), ref["col"])
    assert np.array_equal(lib.element_dofs().cpu().numpy(), ref["gdof"])
    v, r = vals.cpu().numpy(), rhs.cpu().numpy()
    assert np.abs(v - ref["vals"]).max() <= 1e-12 * np.abs(ref["vals"]).max()
    assert np.abs(r - ref["rhs"]).max() <= 1e-12 * max(np.abs(ref["rhs"]).max(), 1e-300)


def test_p3_reproduces_quadratic_solution(lib):
    """-lap u = -2 with u = x^2 + yz - z/2 on the boundary: the P3 solution equals u at every DOF
    (the two DOFs of every edge included, so their order follows the edge direction)."""
    import anigpu
    from anigpu import meshgen
    xyz, tets = _mesh(3, seed=9)
    lib.mesh_upload(xyz, tets)
    lib.problem_setup(anigpu.P3)
    c = lib.dof_coords().cpu().numpy()
    u = c[:, 0] ** 2 + c[:, 1] * c[:, 2] - 0.5 * c[:, 2]
    mask = meshgen.boundary_mask(c)
    lib.set_dirichlet(mask, u * mask)
    vals, rhs = lib.assemble_general(32, 32, anigpu.TENSOR_NULL, None, anigpu.TENSOR_CONST_SCALAR, np.array([-2.0]), 4)
    x, st = lib.solve(vals, rhs, anigpu.SOLVE_JACOBI_PCG, anigpu.F64, rtol=1e-13, maxit=100000)
    assert np.abs(x.cpu().numpy() - u).max() <= 1e-9
    # gradient of the solution at quadrature points: exact
    p4 = anigpu.quadrature(4)[0]
    g = lib.eval_solution(anigpu.GRAD, x, p4).cpu().numpy()
    XG = np.einsum("qv,tvd->tqd", p4, xyz[lib.element_dofs().cpu().numpy()[:, :4]])
    gx = np.stack([2 * XG[..., 0], XG[..., 2], XG[..., 1] - 0.5], axis=-1)
    assert np.abs(g - gx).max() <= 1e-8


def test_cr1_reproduces_linear_solution(lib):
    import anigpu
    from anigpu import meshgen
    xyz, tets = _mesh(3, seed=10)
    lib.mesh_upload(xyz, tets)
    lib.problem_setup(anigpu.CR1)
    c = lib.dof_coords().cpu().numpy()
    u = 1.0 + 2.0 * c[:, 0] - c[:, 1] + 0.5 * c[:, 2]
    mask = meshgen.boundary_mask(c)
    lib.set_dirichlet(mask, u * mask)
    vals, rhs = lib.assemble_general(62, 62, anigpu.TENSOR_NULL, None, anigpu.TENSOR_CONST_SCALAR, np.array([0.0]), 4)
    x, _ = lib.solve(vals, rhs, anigpu.SOLVE_JACOBI_PCG, anigpu.F64, rtol=1e-13, maxit=100000)
    assert np.abs(x.cpu().numpy() - u).max() <= 1e-9


@pytest.mark.parametrize("space,opK", [(9, 94), (10, 103)])
def test_nd0_rt0_reproduce_constant_field(lib, space, opK):
    """(K + M) x = int u0 . v with K the curl-curl (ND0) or div-div (RT0) form and u0 a constant
    vector: u0 lies in the space and K u0 = 0, so the solution evaluated anywhere is u0 -- only with
    consistent orientation signs across the tets."""
    import anigpu
    xyz, tets = _mesh(3, seed=11)
    nt = tets.shape[0]
    lib.mesh_upload(xyz, tets)
    lib.problem_setup(space)
    u0 = np.array([0.7, -1.2, 0.4])
    K, rhs = lib.assemble_general(opK, opK, anigpu.TENSOR_NULL, None, anigpu.TENSOR_TET_GENERAL, np.tile(u0, (nt, 1)), 4)
    M, _ = lib.assemble_general(10 * space + 1, 10 * space + 1, anigpu.TENSOR_NULL, None, None, None, 4)
    A = K + M
    x, st = lib.solve(A, rhs, anigpu.SOLVE_JACOBI_PCG, anigpu.F64, rtol=1e-13, maxit=100000)
    p4 = anigpu.quadrature(4)[0]
    val = lib.eval_solution(anigpu.IDEN, x, p4).cpu().numpy()
    assert np.abs(val - u0).max() <= 1e-8


@pytest.mark.parametrize("space,op", [(3, 32), (9, 94), (6, 62)])
def test_general_enumerations_match_oracle(lib, space, op):
    """Every GlobEnumeration type on a general-path system: permutation, renumbered template and
    renumbered values / right-hand side equal the oracle's lexicographic ordering (ANITYPE splits
    the two DOFs of every P3 edge; the rest is NATURAL), bit for bit."""
    import anigpu
    from oracle.oracle import general_blocks, general_enumeration_perm, permute_csr
    xyz, tets = _mesh(3, seed=12)
    lib.mesh_upload(xyz, tets)
    ndof, nnz = lib.problem_setup(space)
    nt = tets.shape[0]
    rhs_kind, F = (4, np.tile([0.5, -1.0, 2.0], (nt, 1))) if space in (9, 10) else (1, np.array([1.5]))
    vals, rhs = lib.assemble_general(op, op, anigpu.TENSOR_NULL, None, rhs_kind, F, 4)
    rp, col = lib.csr_template()
    rp, col, v, b = rp.cpu().numpy(), col.cpu().numpy(), vals.cpu().numpy(), rhs.cpu().numpy()
    per, off = general_blocks(xyz, tets, space)
    assert off[4] == ndof
    for etype in range(6):
        perm = general_enumeration_perm(per, off, etype)
        if space != 3:
            assert np.array_equal(perm, np.arange(ndof))
        rp_o, col_o, v_o = permute_csr(rp, col, v, perm)
        grp, gcol, gperm = lib.enumeration_setup(etype)
        assert np.array_equal(gperm.cpu().numpy(), perm), etype
        assert np.array_equal(grp.cpu().numpy(), rp_o) and np.array_equal(gcol.cpu().numpy(), col_o), etype
        gv, gb = lib.enumeration_apply(vals, anigpu.F64, rhs)
        assert np.array_equal(gv.cpu().numpy(), v_o), etype
        b_o = np.empty_like(b)
        b_o[perm] = b
        assert np.array_equal(gb.cpu().numpy(), b_o), etype
        assert np.array_equal(lib.enumeration_to_natural(gb).cpu().numpy(), b), etype


@pytest.mark.parametrize("space,opK,opM", [(9, 94, 91), (3, 32, 31), (10, 103, 101)])
def test_general_assembly_from_element_matrices(lib, space, opK, opM):
    """The local-assembler contract: element matrices the caller sums itself (K + M per tet, from
    two fem3Dtet calls on the library's oriented tets) scatter to the sum of the two assembled
    matrices up to one rounding per entry; the right-hand side likewise; Dirichlet rows are the
    unit rows scaled by their number of tets, as in every path."""
    import anigpu
    from anigpu import meshgen
    xyz, tets = _mesh(3, seed=13)
    nt = tets.shape[0]
    lib.mesh_upload(xyz, tets)
    lib.problem_setup(space)
    coords = lib.dof_coords().cpu().numpy()
    lib.set_dirichlet(meshgen.boundary_mask(coords))
    rhs_kind, F = (4, np.tile([0.5, -1.0, 2.0], (nt, 1))) if space in (9, 10) else (1, np.array([1.5]))
    K, rhs = lib.assemble_general(opK, opK, anigpu.TENSOR_NULL, None, rhs_kind, F, 4)
    M, _ = lib.assemble_general(opM, opM, anigpu.TENSOR_NULL, None, None, None, 4)
    # the same element matrices computed by the caller, on the oriented tets the library uses
    XY = lib.element_coords()
    Ak = lib.fem3dtet(opK, opK, XY, None, anigpu.TENSOR_NULL, 4)
    Am = lib.fem3dtet(opM, opM, XY, None, anigpu.TENSOR_NULL, 4)
    Fe = lib.fem3dtet(1, 10 * space + 1, XY, F if rhs_kind == 4 else np.full(nt, F[0]),
                      anigpu.TENSOR_TET_GENERAL if rhs_kind == 4 else anigpu.TENSOR_TET_SCALAR, 4)
    v, r = lib.assemble_elements(Ak + Am, Fe.reshape(nt, -1))
    ref = (K + M).cpu().numpy()
    # a Dirichlet row is the unit row scaled by its number of tets, whatever the matrices were
    rp = lib.csr_template()[0].cpu().numpy()
    dmask = meshgen.boundary_mask(coords).astype(bool)
    on_dir = dmask[np.repeat(np.arange(rp.size - 1), np.diff(rp))]
    ref[on_dir] = K.cpu().numpy()[on_dir]
    assert np.abs(v.cpu().numpy() - ref).max() <= 1e-13 * np.abs(ref).max()
    assert np.abs(r.cpu().numpy() - rhs.cpu().numpy()).max() <= 1e-13 * np.abs(rhs.cpu().numpy()).max()
