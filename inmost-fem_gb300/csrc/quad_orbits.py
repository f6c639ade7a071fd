"""Symmetric quadrature rules as orbits of barycentric coordinates, checked and completed
against the moment equations in multiprecision (used by gen_quadrature.py and
gen_tri_quadrature.py).

Some rules of the published family (Jaskowiec & Sukumar 2021 for tetrahedra, the
Dunavant/Gatermann/Xiao-Gimbutas family for triangles) cannot be recovered from their orbit
structure alone:
  * the moment system is underdetermined (the 8-point degree-3 tet rule: two S4 orbits,
    4 unknowns, 3 invariant moments; a one-parameter family of exact rules), or
  * the system is too large for a random-start search (tet degrees 7-20 with up to 115
    unknowns, triangle degrees 10-20).
For those orders the tabulated values, as the reference build prints them in double
precision (tests/golden/golden.npz: quad_<order>_p/w and tri_<order>_p/w, written by
tests/golden/gen_golden.py), serve as the starting point and pin the member of the family.
This module then

  1. splits the points into orbits of the symmetric group acting on the barycentric
     coordinates and checks that every orbit is complete with one weight;
  2. takes the distinct coordinate values of each orbit (one value follows from the sum
     being 1) and the orbit weights as unknowns;
  3. solves the invariant moment equations
         sum_orbits w_o |o| p(rep_o) = E[p]     for every invariant p of degree <= deg
     (p = e2^i e3^j [e4^k], e_r the elementary symmetric polynomials of the barycentric
     coordinates; E[.] the exact mean over the simplex) by Gauss-Newton with minimum-norm
     steps at 60 digits, starting from the tabulated doubles;
  4. checks the residual (< 1e-40), the weights (> 0), the points (inside the closed
     simplex) and the distance to the starting values (< 1e-13), and returns the points
     in the tabulated order, correctly rounded to double from the exact solution.

The rule that comes out is an exact solution of the moment equations; for a determined
system it is the tabulated rule itself, for the underdetermined degree-3 tet system it is
the member of the family nearest to the tabulated one.
"""
import itertools
import math

import mpmath as mp

mp.mp.dps = 60


def _esym(l):
    """Elementary symmetric polynomials e2, e3 (and e4 for 4 coordinates)."""
    d = len(l)
    e2 = sum(l[p] * l[q] for p, q in itertools.combinations(range(d), 2))
    e3 = sum(l[p] * l[q] * l[r] for p, q, r in itertools.combinations(range(d), 3))
    e4 = l[0] * l[1] * l[2] * l[3] if d == 4 else None
    return e2, e3, e4


def invariants(d, deg):
    if d == 4:
        return [(i, j, k) for i in range(deg // 2 + 1) for j in range(deg // 3 + 1) for k in range(deg // 4 + 1)
                if 2 * i + 3 * j + 4 * k <= deg]
    return [(i, j, 0) for i in range(deg // 2 + 1) for j in range(deg // 3 + 1) if 2 * i + 3 * j <= deg]


def _poly_mul(a, b):
    out = {}
    for ma, ca in a.items():
        for mb, cb in b.items():
            m = tuple(x + y for x, y in zip(ma, mb))
            out[m] = out.get(m, 0) + ca * cb
    return out


def exact_moment(d, ijk):
    """E[e2^i e3^j e4^k] over the simplex with d barycentric coordinates, as an mpf:
    E[l0^a0 ... l_{d-1}^a_{d-1}] = (d-1)! prod a_r! / (sum a_r + d - 1)!."""
    from fractions import Fraction

    def esym_poly(r):
        out = {}
        for c in itertools.combinations(range(d), r):
            m = tuple(1 if t in c else 0 for t in range(d))
            out[m] = out.get(m, 0) + 1
        return out

    one = {tuple([0] * d): 1}
    poly = one
    for r, e in zip((2, 3, 4), ijk):
        for _ in range(e):
            poly = _poly_mul(poly, esym_poly(r))
    tot = Fraction(0)
    for mon, coef in poly.items():
        num = math.factorial(d - 1)
        for a in mon:
            num *= math.factorial(a)
        tot += Fraction(coef * num, math.factorial(sum(mon) + d - 1))
    return mp.mpf(tot.numerator) / mp.mpf(tot.denominator)


def _inv_value(ijk, l):
    e2, e3, e4 = _esym(l)
    v = e2 ** ijk[0] * e3 ** ijk[1]
    if ijk[2]:
        v *= e4 ** ijk[2]
    return v


class Orbit:
    """One orbit: distinct values (all but the last are unknowns), multiplicities, weight."""

    def __init__(self, values, mults):
        self.mults = mults           # multiplicity of each distinct value
        self.values = values         # float starting values, same order
        self.size = math.factorial(sum(mults)) // math.prod(math.factorial(m) for m in mults)

    def npar(self):
        return len(self.mults) - 1

    def full(self, par):
        """All distinct values from the free ones (the last value closes the sum to 1)."""
        vals = list(par)
        rest = mp.mpf(1) - sum(m * v for m, v in zip(self.mults[:-1], vals))
        vals.append(rest / self.mults[-1])
        return vals

    def rep(self, par):
        pt = []
        for m, v in zip(self.mults, self.full(par)):
            pt += [v] * m
        return pt


def split_orbits(P, W, tol=1e-9):
    """Group tabulated points (n x d barycentric) into orbits.  Returns the orbits and, per
    point, (orbit index, per-coordinate index into that orbit's distinct values)."""
    n, d = len(P), len(P[0])
    keys, orbits, owner = [], [], []
    for t in range(n):
        srt = sorted(P[t])
        vals, mults = [], []
        for v in srt:
            if vals and abs(v - vals[-1]) < tol:
                mults[-1] += 1
            else:
                vals.append(v)
                mults.append(1)
        # canonical order: multiplicity descending, then value ascending; the last value is
        # the dependent one
        order = sorted(range(len(vals)), key=lambda k: (-mults[k], vals[k]))
        vals = [vals[k] for k in order]
        mults = [mults[k] for k in order]
        key = None
        for o, (kv, km) in enumerate(keys):
            if km == mults and all(abs(a - b) < tol for a, b in zip(kv, vals)) and abs(W[t] - orbits[o][1]) < tol:
                key = o
                break
        if key is None:
            keys.append((vals, mults))
            orbits.append((Orbit(vals, mults), W[t], []))
            key = len(orbits) - 1
        orb = orbits[key][0]
        slots = []
        for v in P[t]:
            k = min(range(len(orb.values)), key=lambda k: abs(orb.values[k] - v))
            assert abs(orb.values[k] - v) < tol
            slots.append(k)
        assert sorted(slots) == sorted(sum(([k] * m for k, m in enumerate(orb.mults)), [])), "not an orbit point"
        orbits[key][2].append(t)
        owner.append((key, slots))
    for orb, w, members in orbits:
        assert len(members) == orb.size, f"incomplete orbit: {len(members)} of {orb.size} points"
    return [(o, w) for o, w, _ in orbits], owner


def _unpack(orbits, x):
    pars, p = [], 0
    for orb, _ in orbits:
        pars.append(x[p:p + orb.npar()])
        p += orb.npar()
    ws = x[p:p + len(orbits)]
    return pars, ws


def _residual(d, orbits, invs, moments, x):
    pars, ws = _unpack(orbits, x)
    reps = [orb.rep(par) for (orb, _), par in zip(orbits, pars)]
    out = []
    for ijk, m in zip(invs, moments):
        s = mp.mpf(0)
        for (orb, _), rep, w in zip(orbits, reps, ws):
            s += w * orb.size * _inv_value(ijk, rep)
        out.append(s - m)
    return out


def polish(P, W, deg, max_iter=12):
    """Exact rule of degree `deg` nearest to the tabulated one.  Returns (points, weights) as
    lists of mpf in the tabulated order, and a report dict."""
    d = len(P[0])
    orbits, owner = split_orbits(P, W)
    invs = invariants(d, deg)
    moments = [exact_moment(d, t) for t in invs]
    x = []
    for orb, _ in orbits:
        x += [mp.mpf(v) for v in orb.values[:-1]]
    x += [mp.mpf(w) for _, w in orbits]
    x0 = list(x)
    nun, neq = len(x), len(invs)
    h = mp.mpf(10) ** (-30)
    r = _residual(d, orbits, invs, moments, x)
    r_start = max(abs(v) for v in r)
    for _ in range(max_iter):
        if max(abs(v) for v in r) < mp.mpf(10) ** (-55):
            break
        J = mp.matrix(neq, nun)
        for c in range(nun):
            xp = list(x)
            xp[c] += h
            rp = _residual(d, orbits, invs, moments, xp)
            for e in range(neq):
                J[e, c] = (rp[e] - r[e]) / h
        rv = mp.matrix(r)
        mu = mp.mpf(10) ** (-80)
        if nun > neq:   # minimum-norm step: dx = -J^T (J J^T)^-1 r
            JJt = J * J.T
            for k in range(neq):
                JJt[k, k] += mu
            dx = -(J.T * mp.lu_solve(JJt, rv))
        else:           # least-squares step: dx = -(J^T J)^-1 J^T r
            JtJ = J.T * J
            for k in range(nun):
                JtJ[k, k] += mu
            dx = -mp.lu_solve(JtJ, J.T * rv)
        x = [x[k] + dx[k] for k in range(nun)]
        r = _residual(d, orbits, invs, moments, x)
    res = max(abs(v) for v in r)
    pars, ws = _unpack(orbits, x)
    fulls = [orb.full(par) for (orb, _), par in zip(orbits, pars)]
    pts = [[fulls[o][k] for k in slots] for o, slots in owner]
    wts = [ws[o] for o, _ in owner]
    depth = min(min(p) for p in pts)
    moved = max(abs(a - b) for a, b in zip(x, x0))
    rep = {"orbits": [(orb.mults, orb.size) for orb, _ in orbits], "unknowns": nun, "equations": neq,
           "residual_start": float(r_start), "residual": float(res), "min_weight": float(min(ws)),
           "depth": float(depth), "moved": float(moved)}
    assert res < mp.mpf(10) ** (-40), rep
    assert min(ws) > 0 and depth > -mp.mpf(10) ** (-40), rep
    assert moved < 1e-13, rep
    return pts, wts, rep


def orbit_signature(orbits):
    """Orbit counts by size, e.g. {1: 0, 4: 2, 6: 1, 12: 0, 24: 0} for a tet rule."""
    out = {}
    for mults, size in orbits:
        out[size] = out.get(size, 0) + 1
    return out
