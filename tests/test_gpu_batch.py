"""GPU test of the batched uneven instances (one graph launch assembles and solves every instance):
each instance's solution equals the single-instance Jacobi-PCG solution of the same mesh."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _instances(ns, seed):
    from anigpu import meshgen
    meshes = [meshgen.kuhn_cube(n, perturb=0.15, seed=seed + i) for i, n in enumerate(ns)]
    coefs = [np.exp(meshgen.normal(seed + 100 + i, m[1].shape[0])) for i, m in enumerate(meshes)]
    return meshes, coefs


@pytest.mark.parametrize("space,order", [(1, 2), (2, 4)])
def test_batched_instances_match_single_solves(lib, space, order):
    import anigpu
    from anigpu import meshgen
    ns = [3, 5, 4, 6, 2]
    meshes, coefs = _instances(ns, 40 + space)
    xyz, tets, toff = meshgen.union(meshes)
    coef = np.concatenate(coefs)
    lib.mesh_upload(xyz, tets)
    lib.problem_setup(space)
    mask = meshgen.boundary_mask(lib.dof_coords().cpu().numpy())
    lib.set_dirichlet(mask)
    vals0, _, _ = lib.assemble(anigpu.TENSOR_TET_SCALAR, coef, None, 1.0, order, anigpu.F64)
    vals0 = vals0.clone()
    lib.batch_set_instances(toff, vals0)
    info = lib.batch_info()
    assert info["lanes_per_row"] in (2, 4, 8, 16) and info["ntiles"] > 0
    b = meshgen.normal(7, lib.ndof) * (1 - mask)
    x, vals, st = lib.batch_run(b, anigpu.TENSOR_TET_SCALAR, coef, None, 1.0, order, rtol=1e-10, maxit=20000)
    print("batch info", lib.batch_info(), [s.iterations for s in st])
    assert bool((vals == vals0).all())  # the graph's assembly is the plain assembly
    assert all(s.rel_residual <= 1e-10 for s in st)
    xb, bu = x.cpu().numpy(), b
    nv_tot = xyz.shape[0]
    voff = np.concatenate([[0], np.cumsum([m[0].shape[0] for m in meshes])])
    eoff = 0
    for i, (m, c) in enumerate(zip(meshes, coefs)):
        lib.mesh_upload(*m)
        nd, _ = lib.problem_setup(space)
        ne = lib.nedges if space == 2 else 0
        nvi = m[0].shape[0]
        idx = np.concatenate([voff[i] + np.arange(nvi), nv_tot + eoff + np.arange(nd - nvi)]).astype(np.int64)
        eoff += ne
        lib.set_dirichlet(mask[idx])
        vi, _, _ = lib.assemble(anigpu.TENSOR_TET_SCALAR, c, None, 1.0, order, anigpu.F64)
        xi, si = lib.solve(vi, bu[idx], anigpu.SOLVE_JACOBI_PCG, anigpu.F64, rtol=1e-10, maxit=20000)
        assert abs(si.iterations - st[i].iterations) <= 1, (i, si.iterations, st[i].iterations)
        xr = xi.cpu().numpy()
        assert np.abs(xb[idx] - xr).max() <= 1e-8 * max(np.abs(xr).max(), 1e-300)
