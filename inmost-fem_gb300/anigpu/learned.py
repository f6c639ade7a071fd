"""Training of the learned preconditioner of ANIGPU_SOLVE_FCG_LEARNED on the GPU.

Everything runs through the library: the network forward pass (at bind), the hand-written
backward kernels (loss_grad) and Adam.  A training example is a pair (r, e = A^-1 r); the
residuals are those of the early iterates of a Jacobi-CG solve, where a preconditioner has to
act on smooth, slowly converging error, plus the right-hand side itself.
"""
import os

import numpy as np

import anigpu

WEIGHTS_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights")
DEFAULT_WEIGHTS = os.path.join(WEIGHTS_DIR, "p2_aniso_l4.npy")
ELASTIC_WEIGHTS = os.path.join(WEIGHTS_DIR, "p2_elastic_l4.npy")


def training_pairs(lib, vals, b, ks=(0, 1, 2, 4, 8, 16, 32, 64, 128, 256), rtol=1e-10):
    """Pairs (r_k, x* - x_k) for Jacobi-PCG iterates x_k of A x = b (FP32 values)."""
    torch = lib.torch
    b = lib._dev(b, torch.float64)
    xs, _ = lib.solve(vals, b, anigpu.SOLVE_IR_CG32, anigpu.F32, rtol=rtol, maxit=1_000_000)
    pairs = []
    for k in ks:
        if k == 0:
            xk = torch.zeros_like(b)
        else:
            xk, _ = lib.solve(vals, b, anigpu.SOLVE_JACOBI_PCG, anigpu.F32, rtol=1e-30, maxit=k, check=False)
        rk = b - lib.spmv(vals, xk, anigpu.F32)
        pairs.append((rk.clone(), (xs - xk).clone()))
    return pairs


def train(prec, systems, steps, lr=2e-3, lr_final=5e-4, batch=4, seed=0, log_every=0, log=print):
    """Adam on the relative energy-norm error.  systems: list of (vals, kind, D, pairs).
    Returns the per-step mean losses."""
    rng = np.random.default_rng(seed)
    hist = []
    for step in range(steps):
        vals, kind, D, pairs = systems[step % len(systems)]
        prec.bind(vals, anigpu.F32, kind, D)
        prec.zero_grads()
        idx = rng.choice(len(pairs), min(batch, len(pairs)), replace=False)
        loss = sum(prec.loss_grad(*pairs[i]) for i in idx) / len(idx)
        prec.adam(lr=lr if step < 0.7 * steps else lr_final, grad_scale=1.0 / len(idx))
        hist.append(loss)
        if log_every and (step % log_every == 0 or step == steps - 1):
            log(f"step {step} loss {np.mean(hist[-log_every:]):.4f}")
    return hist


def mean_loss(prec, systems):
    """Mean loss over every pair of every system (no gradient step)."""
    tot, cnt = 0.0, 0
    for vals, kind, D, pairs in systems:
        prec.bind(vals, anigpu.F32, kind, D)
        for r, e in pairs:
            prec.zero_grads()
            tot += prec.loss_grad(r, e)
            cnt += 1
    prec.zero_grads()
    return tot / max(cnt, 1)


def load_default(prec, problem="aniso"):
    """Set committed trained parameters: "aniso" (scalar P2, anisotropic tensors) or "elastic"
    (vector P2 elasticity, per-tet Lame parameters); 4 layers."""
    w = np.load(DEFAULT_WEIGHTS if problem == "aniso" else ELASTIC_WEIGHTS)
    prec.set_params(w)
    return w


def lame_params(nt, seed):
    """Per-tet (lambda, mu) from E ~ lognormal(0, 0.5^2), nu ~ U[0.2, 0.45]."""
    from anigpu import meshgen
    E = np.exp(0.5 * meshgen.normal(seed, nt))
    nu = 0.2 + 0.25 * meshgen.uniform(seed + 1, nt)
    return np.stack([E * nu / ((1 + nu) * (1 - 2 * nu)), E / (2 * (1 + nu))], axis=1)


def make_systems(lib, problem, n, count, seed0=0):
    """Seeded synthetic training systems on a perturbed Kuhn cube of n^3 x 6 tets.
    aniso: scalar P2, anisotropic per-tet tensors (log-normal eigenvalues), Dirichlet boundary.
    elastic: vector P2, per-tet Lame parameters, clamped face x = 0."""
    from anigpu import meshgen
    xyz, tets = meshgen.kuhn_cube(n, perturb=0.2, seed=7)
    nt = tets.shape[0]
    lib.mesh_upload(xyz, tets)
    if problem == "aniso":
        lib.problem_setup(anigpu.P2)
        mask = meshgen.boundary_mask(lib.dof_coords().cpu().numpy())
        kind = anigpu.TENSOR_TET_SYM
    else:
        lib.problem_setup(anigpu.VEC3_P2)
        mask = (np.abs(lib.dof_coords().cpu().numpy()[:, 0]) < 1e-12).astype(np.uint8)
        kind = anigpu.TENSOR_LAME
    lib.set_dirichlet(mask)
    systems = []
    for sd in range(seed0, seed0 + count):
        D = meshgen.aniso_tensors(nt, 1.5, 100 + sd) if problem == "aniso" else lame_params(nt, 2 * sd + 300)
        v, _, _ = lib.assemble(kind, D, None, 1.0, 4, anigpu.F32)
        v = v.clone()
        b = meshgen.normal(500 + sd, lib.ndof) * (1 - mask)
        systems.append((v, kind, D, training_pairs(lib, v, b)))
    return systems


def evaluate(lib, weights, sizes, seed=2024):
    """FCG iterations to 1e-8 on the benchmark family (P2, anisotropic per-tet tensors on a
    perturbed n^3 x 6 Kuhn cube, seed 2024: not a training system) for each parameter file in
    weights (None: the untrained net) and each n in sizes, with FP32 Jacobi-PCG for reference.
    Returns {n: {name: iterations}}."""
    import torch
    from anigpu import meshgen
    out = {}
    for n in sizes:
        xyz, tets = meshgen.kuhn_cube(n, perturb=0.2, seed=seed)
        D = meshgen.aniso_tensors(tets.shape[0], 1.5, seed + 1)
        lib.mesh_upload(xyz, tets)
        lib.problem_setup(anigpu.P2)
        lib.set_dirichlet(meshgen.boundary_mask(lib.dof_coords().cpu().numpy()))
        Dd = torch.tensor(D, device=f"cuda:{lib.device}")
        v, b, _ = lib.assemble(anigpu.TENSOR_TET_SYM, Dd, None, 1.0, 4, anigpu.F32)
        v, b = v.clone(), b.clone()
        _, st = lib.solve(v, b, anigpu.SOLVE_JACOBI_PCG, anigpu.F32, rtol=1e-8, maxit=1_000_000, check=False)
        row = {"jacobi_pcg": st.iterations}
        for name, wf in weights.items():
            prec = anigpu.LearnedPreconditioner(lib, layers=4, act=anigpu.BF16, seed=1)
            if wf is not None:
                prec.set_params(np.load(wf))
            prec.bind(v, anigpu.F32, anigpu.TENSOR_TET_SYM, Dd)
            _, st = lib.solve(v, b, anigpu.SOLVE_FCG_LEARNED, anigpu.F32, rtol=1e-8, maxit=1_000_000, check=True)
            row[name] = st.iterations
        out[n] = row
    return out


def main(argv=None):
    """Train parameters on seeded synthetic problems and save them:
        python -m anigpu.learned --problem aniso --n 12 --systems 200 --steps 2000
        python -m anigpu.learned --problem elastic --n 8 --systems 200 --steps 3000
    (each system gives 10 Jacobi-PCG iterates = 10 residual/correction pairs), or compare parameter
    files on the benchmark family:
        python -m anigpu.learned --evaluate 16,32,64 --weights other.npy"""
    import argparse
    import time

    ap = argparse.ArgumentParser()
    ap.add_argument("--problem", choices=("aniso", "elastic"), default="aniso")
    ap.add_argument("--n", type=int, default=None)
    ap.add_argument("--systems", type=int, default=None)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--layers", type=int, default=4)
    ap.add_argument("--out", default=None)
    ap.add_argument("--evaluate", default=None,
                    help="instead of training: FCG iterations on the benchmark family at these sizes, e.g. 16,32,64, "
                         "for the committed parameters, the untrained net and the files given with --weights")
    ap.add_argument("--weights", default="", help="comma-separated parameter files for --evaluate")
    a = ap.parse_args(argv)
    if a.evaluate:
        import json
        lib = anigpu.Anigpu(0)
        weights = {"committed": DEFAULT_WEIGHTS, "untrained": None}
        for wf in filter(None, a.weights.split(",")):
            weights[os.path.basename(wf)] = wf
        print(json.dumps(evaluate(lib, weights, [int(x) for x in a.evaluate.split(",")])))
        return
    elastic = a.problem == "elastic"
    n = a.n or (8 if elastic else 12)
    count = a.systems or 200
    steps = a.steps or (3000 if elastic else 2000)
    out = a.out or (ELASTIC_WEIGHTS if elastic else DEFAULT_WEIGHTS)
    lib = anigpu.Anigpu(0)
    t0 = time.time()
    systems = make_systems(lib, a.problem, n, count)
    print(f"{count} systems ({lib.ndof} DOFs) in {time.time() - t0:.1f} s")
    prec = anigpu.LearnedPreconditioner(lib, layers=a.layers, act=anigpu.BF16, seed=a.seed)
    t0 = time.time()
    train(prec, systems, steps, lr=a.lr, lr_final=a.lr / 3, log_every=max(1, steps // 10))
    print(f"trained {steps} steps in {time.time() - t0:.1f} s; mean loss {mean_loss(prec, systems[:4]):.4f}")
    os.makedirs(os.path.dirname(os.path.abspath(out)), exist_ok=True)
    np.save(out, prec.get_params())
    print("saved", out)


if __name__ == "__main__":
    main()
