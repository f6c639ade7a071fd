"""Seeded synthetic inputs: Kuhn (Freudenthal) cube meshes, vertex perturbation and the
anisotropic per-tet diffusion tensors of the P2 benchmark workload.

No dataset is involved anywhere: the reference ships its meshes as Git-LFS pointers
only, and its own GenerateCube uses a different 6-tet split
(anifem++/utils/mesh_utils.cpp:20-49).  "Kuhn" here is the Freudenthal split: every
cube is cut into the 6 tets that share its main diagonal (0,0,0)-(1,1,1).

Random numbers come from splitmix64 so that the streams are identical on every machine
and every numpy version (uniforms from the top 53 bits, normals by Box-Muller).
"""
import itertools

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(seed, n):
    """n consecutive splitmix64 outputs of state `seed` (uint64 array)."""
    with np.errstate(over="ignore"):
        idx = np.arange(1, n + 1, dtype=np.uint64)
        z = np.uint64(seed) + idx * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def uniform(seed, n):
    """U[0,1) doubles."""
    return (splitmix64(seed, n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def normal(seed, n):
    """N(0,1) by Box-Muller over 2*ceil(n/2) uniforms."""
    m = (n + 1) // 2
    u = uniform(seed, 2 * m)
    u1 = np.maximum(u[:m], 1e-300)
    u2 = u[m:]
    r = np.sqrt(-2.0 * np.log(u1))
    z = np.concatenate([r * np.cos(2 * np.pi * u2), r * np.sin(2 * np.pi * u2)])
    return z[:n]


def kuhn_cube(n, perturb=0.0, seed=0, lengths=(1.0, 1.0, 1.0)):
    """Unit cube split into n^3 cubes x 6 Kuhn tets.

    Vertex (i,j,k) has id i + (n+1)*(j + (n+1)*k).  Interior vertices are moved by
    U(-perturb*h, perturb*h) per coordinate (h = 1/n).  Returns (xyz[nv,3] f64,
    tets[nt,4] i32); tets are listed cube by cube, 6 per cube."""
    n1 = n + 1
    g = np.arange(n1, dtype=np.float64) / n
    k, j, i = np.meshgrid(np.arange(n1), np.arange(n1), np.arange(n1), indexing="ij")
    xyz = np.stack([g[i.ravel()] * lengths[0], g[j.ravel()] * lengths[1], g[k.ravel()] * lengths[2]], axis=1)
    if perturb > 0:
        interior = ((i > 0) & (i < n) & (j > 0) & (j < n) & (k > 0) & (k < n)).ravel()
        d = (uniform(seed, 3 * xyz.shape[0]).reshape(-1, 3) * 2.0 - 1.0) * (perturb / n)
        d[:, 0] *= lengths[0]
        d[:, 1] *= lengths[1]
        d[:, 2] *= lengths[2]
        xyz = xyz + d * interior[:, None]
    ci, cj, ck = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    base = (ck.ravel() * n1 + cj.ravel()) * n1 + ci.ravel()
    # cube ordering: x fastest
    order = np.lexsort((ci.ravel(), cj.ravel(), ck.ravel()))
    base = base[order]
    step = np.array([1, n1, n1 * n1], dtype=np.int64)
    tets = []
    for perm in itertools.permutations(range(3)):
        a = step[perm[0]]
        b = a + step[perm[1]]
        tets.append(np.stack([base, base + a, base + b, base + step.sum()], axis=1))
    tets = np.stack(tets, axis=1).reshape(-1, 4).astype(np.int32)
    return xyz, tets


def aniso_tensors(nt, sigma=1.5, seed=1):
    """Per-tet SPD tensors D = R diag(exp(g)) R^T, g ~ N(0, sigma^2), R a uniform random
    rotation (normalised Gaussian quaternion).  Returns sym6 [nt,6]: d00 d01 d02 d11 d12 d22."""
    g = normal(seed, 3 * nt).reshape(nt, 3) * sigma
    qv = normal(seed + 0x5151, 4 * nt).reshape(nt, 4)
    qv /= np.linalg.norm(qv, axis=1, keepdims=True)
    w, x, y, z = qv.T
    R = np.empty((nt, 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z)
    R[:, 0, 1] = 2 * (x * y - z * w)
    R[:, 0, 2] = 2 * (x * z + y * w)
    R[:, 1, 0] = 2 * (x * y + z * w)
    R[:, 1, 1] = 1 - 2 * (x * x + z * z)
    R[:, 1, 2] = 2 * (y * z - x * w)
    R[:, 2, 0] = 2 * (x * z - y * w)
    R[:, 2, 1] = 2 * (y * z + x * w)
    R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    lam = np.exp(g)
    D = np.einsum("tab,tb,tcb->tac", R, lam, R)
    return np.stack([D[:, 0, 0], D[:, 0, 1], D[:, 0, 2], D[:, 1, 1], D[:, 1, 2], D[:, 2, 2]], axis=1)


def sym6_to_full(d6):
    d6 = np.asarray(d6)
    return np.stack([d6[..., 0], d6[..., 1], d6[..., 2], d6[..., 1], d6[..., 3], d6[..., 4],
                     d6[..., 2], d6[..., 4], d6[..., 5]], axis=-1).reshape(d6.shape[:-1] + (3, 3))


def tet_coords(xyz, tets):
    """XY[nt, 12]: per tet X0 X1 X2 X3 (the TetrasT columns of fem3Dtet)."""
    return np.ascontiguousarray(xyz[tets].reshape(-1, 12))


def boundary_mask(coords, tol=1e-12, lengths=(1.0, 1.0, 1.0)):
    """DOFs on the boundary of the box [0,L]^3 (ex1.cpp:49-58 labels nodes the same way)."""
    c = np.asarray(coords)
    L = np.asarray(lengths)
    return (np.any(np.abs(c) < tol, axis=1) | np.any(np.abs(c - L) < tol, axis=1)).astype(np.uint8)


def random_tets(nt, seed=3, scale=1.0):
    """Independent random (non-degenerate) tets for element-level parity, XY[nt,12]."""
    base = uniform(seed, 3 * nt).reshape(nt, 1, 3) * 4.0
    off = (uniform(seed + 1, 12 * nt).reshape(nt, 4, 3) - 0.5) * scale
    off[:, 1, 0] += 0.6 * scale
    off[:, 2, 1] += 0.6 * scale
    off[:, 3, 2] += 0.6 * scale
    return np.ascontiguousarray((base + off).reshape(nt, 12))


def union(meshes):
    """Disjoint union of meshes [(xyz, tets), ...]: concatenated coordinates, tets with vertex ids
    offset per mesh, and the tet offsets of the meshes (len(meshes) + 1)."""
    xs, ts, toff, voff = [], [], [0], 0
    for xyz, tets in meshes:
        xs.append(np.asarray(xyz, dtype=np.float64))
        ts.append(np.asarray(tets, dtype=np.int32) + voff)
        voff += xyz.shape[0]
        toff.append(toff[-1] + tets.shape[0])
    return np.concatenate(xs), np.concatenate(ts), np.asarray(toff, dtype=np.int64)


def p2_aniso_workload(n, seed=2024):
    """The P2 anisotropic-diffusion workload: n^3 x 6 Kuhn tets, interior vertices perturbed by
    U(-0.2h, 0.2h), per-tet tensors D = R diag(exp g) R^T with g ~ N(0, 1.5^2).
    Returns (xyz, tets, D sym6)."""
    xyz, tets = kuhn_cube(n, perturb=0.2, seed=seed)
    return xyz, tets, aniso_tensors(tets.shape[0], 1.5, seed + 1)


def elasticity_workload(n, seed=48):
    """The vector-P2 elasticity workload: n^3 x 6 perturbed Kuhn tets, per-tet Lame parameters from
    E ~ lognormal(0, 0.5^2), nu ~ U[0.2, 0.45].  Returns (xyz, tets, LM [nt, 2] = (lambda, mu))."""
    xyz, tets = kuhn_cube(n, perturb=0.2, seed=seed)
    nt = tets.shape[0]
    E = np.exp(0.5 * normal(seed * 100 + 1, nt))
    nu = 0.2 + 0.25 * uniform(seed * 100 + 2, nt)
    return xyz, tets, np.stack([E * nu / ((1 + nu) * (1 - 2 * nu)), E / (2 * (1 + nu))], axis=1)


def lame9(lam, mu):
    """The Lame tensor as the 9x9 GENERAL tensor of Operator<GRAD, FemVec<3,P2>> (index j + 3c for
    derivative j of component c), [nt, 81]; symmetric, so column- and row-major agree."""
    lam, mu = np.asarray(lam), np.asarray(mu)
    D = np.zeros((lam.size, 9, 9))
    for c1 in range(3):
        for j1 in range(3):
            for c2 in range(3):
                for j2 in range(3):
                    D[:, j1 + 3 * c1, j2 + 3 * c2] = (lam * (j1 == c1) * (j2 == c2)
                                                      + mu * ((c1 == c2) * (j1 == j2) + (c1 == j2) * (j1 == c2)))
    return D.reshape(lam.size, 81)


def fp64_redo_count(xyz, tets):
    """Tets that the FP32 kernels redo in FP64 geometry: |det| <= 0.05 |e1| |e2| |e3| for the
    edges e_k = X_k - X_0."""
    X = xyz[tets]
    e = X[:, 1:] - X[:, :1]
    det = np.abs(np.einsum("ti,ti->t", e[:, 0], np.cross(e[:, 1], e[:, 2])))
    return int((det <= 0.05 * np.prod(np.linalg.norm(e, axis=2), axis=1)).sum())
