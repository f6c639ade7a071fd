"""CPU oracle of the learned preconditioner (test infrastructure only): the same network,
transfers, polynomial and loss as inmost-fem_gb300/csrc/k_learned.cu, written with torch
autograd in FP64, used to check the GPU forward pass and the hand-written backward kernels.

    M r = D^-1 r + P Dc^-1/2 B B^T Dc^-1/2 P^T r,   B = sum_{k<K} diag(a_k) A_hat^k
    a   = GNN(static vertex features)                (once per system)
    L   = (M r - e)^T A (M r - e) / (e^T A e)
"""
import numpy as np
import torch

C = 64
K = 4
NF = 2


def layout(L):
    off = {}
    p = 0
    off["W0"] = (p, (NF, C)); p += NF * C
    off["b0"] = (p, (C,)); p += C
    for l in range(L):
        off[f"W{l + 1}"] = (p, (C, C)); p += C * C
        off[f"b{l + 1}"] = (p, (C,)); p += C
    off["wout"] = (p, (C, K)); p += C * K
    off["bout"] = (p, (K,)); p += K
    return off, p


def _sp(r, c, v, shape):
    return torch.sparse_coo_tensor(np.vstack([r, c]), torch.tensor(np.asarray(v, dtype=np.float64)),
                                   shape).coalesce()


class GnnOracle:
    """Built from the P2 (or vector P2) system (CSR of the matrix the GPU used), the oriented
    tets, the scalar element DOF table and the per-tet tensors: symmetric (d00 d01 d02 d11 d12
    d22) or, with lame=True, (lambda, mu).  With ncomp components the fine DOF c*nds + s is
    scalar DOF s of component c and the coarse node c*nv + v is vertex v of component c."""

    def __init__(self, rowptr, col, vals, tets, edofs, D, nv, layers=4, ncomp=1, lame=False):
        self.L = layers
        n = rowptr.size - 1
        nds = n // ncomp
        nc = ncomp * nv
        self.n, self.nv, self.nc = n, nv, nc
        rows = np.repeat(np.arange(n), np.diff(rowptr))
        vals = np.asarray(vals, dtype=np.float64)
        self.A = _sp(rows, col, vals, (n, n))
        diag = np.zeros(n)
        m = rows == col
        diag[rows[m]] = vals[m]
        self.diag_f = torch.tensor(diag)
        # fine DOF -> coarse node (-1 for edge DOFs) and back
        fine = np.arange(n)
        comp, s = fine // nds, fine % nds
        coarse_of = np.where(s < nv, comp * nv + s, -1)
        cid = np.arange(nc)
        fine_of = (cid // nv) * nds + cid % nv
        dc = diag[fine_of]
        self.isd = torch.tensor(1.0 / np.sqrt(dc))
        # coarse graph: off-diagonal entries between vertex DOFs, A_hat = -a / sqrt(d_v d_w)
        cr, cc = coarse_of[rows], coarse_of[col]
        sel = (cr >= 0) & (cc >= 0) & (rows != col)
        r, c, a = cr[sel], cc[sel], vals[sel]
        self.Ahat = _sp(r, c, -a / np.sqrt(dc[r] * dc[c]), (nc, nc))
        # prolongation per component: vertex DOF -> its vertex; edge DOF -> mean of its two vertices
        I = [0, 0, 0, 1, 1, 2]
        J = [1, 2, 3, 2, 3, 3]
        ends = {}
        for t in range(tets.shape[0]):
            for e in range(6):
                ends[int(edofs[t, 4 + e])] = (int(tets[t, I[e]]), int(tets[t, J[e]]))
        pr, pc, pv = [], [], []
        for k in range(ncomp):
            pr += list(k * nds + np.arange(nv))
            pc += list(k * nv + np.arange(nv))
            pv += [1.0] * nv
            for d, (a0, b0) in ends.items():
                pr += [k * nds + d, k * nds + d]
                pc += [k * nv + a0, k * nv + b0]
                pv += [0.5, 0.5]
        self.P = _sp(pr, pc, pv, (n, nc))
        self.PT = self.P.t().coalesce()
        # static features: log A_vv and the mean over the incident tets of log(trace D / 3)
        # (Lame: of lambda + 2 mu), the second shared by the components of a vertex
        f1 = np.log(dc)
        D = np.asarray(D, dtype=np.float64)
        tr = D[:, 0] + 2.0 * D[:, 1] if lame else (D[:, 0] + D[:, 3] + D[:, 5]) / 3.0
        acc = np.zeros(nv)
        cnt = np.zeros(nv)
        for k in range(4):
            np.add.at(acc, tets[:, k], np.log(tr))
            np.add.at(cnt, tets[:, k], 1.0)
        f2 = np.tile(acc / np.maximum(cnt, 1), ncomp)
        self.fs = torch.tensor(np.stack([f1 - f1.mean(), f2 - f2.mean()], axis=1))

    def params(self, w):
        off, _ = layout(self.L)
        w = torch.tensor(np.asarray(w, dtype=np.float64), requires_grad=True)
        return w, {k: w[o:o + int(np.prod(s))].reshape(s) for k, (o, s) in off.items()}

    def coefficients(self, P):
        h = torch.relu(self.fs @ P["W0"] + P["b0"])
        for l in range(1, self.L + 1):
            g = torch.sparse.mm(self.Ahat, h)
            h = h + torch.relu(g @ P[f"W{l}"] + P[f"b{l}"])
        return h @ P["wout"] + P["bout"]          # (nc, K)

    def _mv(self, x):
        return torch.sparse.mm(self.Ahat, x[:, None])[:, 0]

    def apply(self, w, r, return_parts=False):
        wt, P = self.params(w)
        a = self.coefficients(P)
        r = torch.as_tensor(np.asarray(r, dtype=np.float64))
        u = self.isd * torch.sparse.mm(self.PT, r[:, None])[:, 0]
        # w = B^T u = sum_k A_hat^k (a_k * u)
        wv = a[:, K - 1] * u
        for k in range(K - 2, -1, -1):
            wv = self._mv(wv) + a[:, k] * u
        # c = Dc^-1/2 B w = Dc^-1/2 sum_k a_k * A_hat^k w
        pk = wv
        cp = a[:, 0] * pk
        for k in range(1, K):
            pk = self._mv(pk)
            cp = cp + a[:, k] * pk
        c = self.isd * cp
        z = r / self.diag_f + torch.sparse.mm(self.P, c[:, None])[:, 0]
        return (z, wt, a) if return_parts else z

    def coefficients_np(self, w):
        _, P = self.params(w)
        return self.coefficients(P).detach().numpy()

    def loss_and_grad(self, w, r, e):
        z, wt, _ = self.apply(w, r, return_parts=True)
        e = torch.as_tensor(np.asarray(e, dtype=np.float64))
        d = z - e
        Ad = torch.sparse.mm(self.A, d[:, None])[:, 0]
        Ae = torch.sparse.mm(self.A, e[:, None])[:, 0]
        loss = (d @ Ad) / (e @ Ae)
        loss.backward()
        return float(loss.detach()), wt.grad.numpy().copy()
