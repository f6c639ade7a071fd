#!/usr/bin/env python3
"""Generate the fully symmetric triangle quadrature rules of the face integrals (fem3Dface).

The rules belong to the published family the reference library tabulates for its face
integrals (anifem++/fem/quadrature_formulas.cpp:109, triangle_quadrature_formulas: centroid,
Strang-Fix, Dunavant and Gatermann rules as collected by quadpy).  Nothing is copied: each
rule is recomputed from its orbit structure by solving the moment equations.

Orbits of the symmetric group S3 acting on barycentric coordinates (l0, l1, l2):
    C       (1/3, 1/3, 1/3)                  1 point
    T3(a)   (a, a, 1-2a)                     3 points
    T6(a,b) (a, b, 1-a-b)                    6 points
One weight per orbit, weights summing to 1 (the reference integrates as
|f| * sum_n w_n g(x_n)).  A rule is exact to degree p iff it integrates every S3-invariant
polynomial of degree <= p, spanned by e2^i e3^j (2i + 3j <= p) with e2, e3 the elementary
symmetric polynomials of the barycentric coordinates.  For the structures below the
number of unknowns equals the number of invariants; the square system is solved by a
float64 multi-start least-squares search and a multiprecision Newton polish.  Exact
moments: E[l0^a l1^b l2^c] = 2! a! b! c! / (a+b+c+2)!.  Among several valid solutions
(points in the closed triangle, positive weights) the one with the largest smallest weight
is kept, ties broken by the points lying deepest inside (degree 2: the interior Strang-Fix
points, not the edge midpoints; degrees 6 and 7: the rules with weights >= 0.05).
Degrees 8 and 9 need ~2000 random starts (about half an hour in all).

Output: tri_quad_tables.h (plain C: points as 3 barycentric coordinates, weights).
"""
import itertools
import sys

import mpmath as mp
import sympy as sp

mp.mp.dps = 60

# orbit structure per degree (degree = the order a caller asks for)
STRUCTURES = {
    1: ["C"],
    2: ["T3"],
    3: ["T6"],
    4: ["T3", "T3"],
    5: ["C", "T3", "T3"],
    6: ["T3", "T3", "T6"],
    7: ["T3", "T6", "T6"],
    8: ["C", "T3", "T3", "T3", "T6"],
    9: ["C", "T3", "T3", "T3", "T3", "T6"],
}
NPAR = {"C": 0, "T3": 1, "T6": 2}
NPTS = {"C": 1, "T3": 3, "T6": 6}


def orbit_points(kind, par):
    one = mp.mpf(1)
    if kind == "C":
        return [(one / 3,) * 3]
    if kind == "T3":
        a = par[0]
        c = one - 2 * a
        return [(a, a, c), (a, c, a), (c, a, a)]
    a, b = par
    c = one - a - b
    return [(a, b, c), (b, c, a), (c, a, b), (a, c, b), (c, b, a), (b, a, c)]


def orbit_rep_f(kind, par):
    if kind == "C":
        return (1 / 3,) * 3
    if kind == "T3":
        return (par[0], par[0], 1 - 2 * par[0])
    return (par[0], par[1], 1 - par[0] - par[1])


def invariants(deg):
    return [(i, j) for i in range(deg // 2 + 1) for j in range(deg // 3 + 1) if 2 * i + 3 * j <= deg]


_L = sp.symbols("l0:3")


def exact_moment(ij):
    i, j = ij
    l0, l1, l2 = _L
    e2 = l0 * l1 + l0 * l2 + l1 * l2
    e3 = l0 * l1 * l2
    poly = sp.Poly(sp.expand(e2 ** i * e3 ** j), *_L)
    tot = sp.Rational(0)
    for mon, coef in poly.terms():
        num = sp.Integer(2)
        for m in mon:
            num *= sp.factorial(m)
        tot += coef * num / sp.factorial(sum(mon) + 2)
    return tot


def eval_inv(ij, l):
    i, j = ij
    e2 = l[0] * l[1] + l[0] * l[2] + l[1] * l[2]
    e3 = l[0] * l[1] * l[2]
    return e2 ** i * e3 ** j


def unpack(structure, x):
    pars, ws, p = [], [], 0
    for kind in structure:
        pars.append(x[p:p + NPAR[kind]])
        p += NPAR[kind]
    for _ in structure:
        ws.append(x[p])
        p += 1
    return pars, ws


def residual(structure, invs, moments, x):
    pars, ws = unpack(structure, x)
    out = []
    for ij, m in zip(invs, moments):
        s = mp.mpf(0)
        for kind, par, w in zip(structure, pars, ws):
            s += w * NPTS[kind] * eval_inv(ij, orbit_points(kind, par)[0])
        out.append(s - m)
    return out


def depth(structure, x):
    """Smallest barycentric coordinate over all points (negative: outside)."""
    pars, _ = unpack(structure, x)
    return min(min(pt) for kind, par in zip(structure, pars) for pt in orbit_points(kind, par))


def valid(structure, x, tol=mp.mpf("1e-40")):
    _, ws = unpack(structure, x)
    return all(w > 0 for w in ws) and depth(structure, x) >= -tol


def solve_degree(deg, tries=None, seed=4321):
    import numpy as np
    from scipy.optimize import least_squares
    structure = STRUCTURES[deg]
    if tries is None:
        tries = 60 if deg < 8 else 2000
    invs = invariants(deg)
    moments = []
    for t in invs:
        r = sp.Rational(exact_moment(t))
        moments.append(mp.mpf(r.p) / mp.mpf(r.q))
    mf = [float(m) for m in moments]
    nun = sum(NPAR[k] for k in structure) + len(structure)
    assert nun == len(invs), (deg, nun, len(invs))
    if nun == 1:  # centroid rule
        return structure, [[mp.mpf(1)]]

    def res_f(x):
        pars, ws = unpack(structure, list(x))
        reps = [orbit_rep_f(k, p) for k, p in zip(structure, pars)]
        return [sum(w * NPTS[k] * eval_inv(ij, rep) for k, rep, w in zip(structure, reps, ws)) - m
                for ij, m in zip(invs, mf)]

    rng = np.random.default_rng(seed)
    cands, keys = [], []
    for _ in range(tries):
        x0 = []
        for kind in structure:
            if kind == "T3":
                x0.append(rng.uniform(0.0, 0.5))
            elif kind == "T6":
                a = rng.uniform(0.0, 1.0)
                x0.extend([a, rng.uniform(0.0, 1.0 - a)])
        x0 += [rng.uniform(0.01, 1.0) / len(structure) for _ in structure]
        sol = least_squares(res_f, x0, xtol=1e-15, ftol=1e-15, gtol=1e-15, max_nfev=600, method="lm")
        if np.max(np.abs(sol.fun)) > 1e-12:
            continue
        x = [mp.mpf(float(v)) for v in sol.x]
        if not valid(structure, x, tol=mp.mpf("1e-9")):
            continue
        pars, ws = unpack(structure, x)
        key = tuple(sorted((k, tuple(sorted(round(float(v), 8) for v in orbit_points(k, p)[0])), round(float(w), 8))
                           for k, p, w in zip(structure, pars, ws)))
        if key in keys:
            continue
        keys.append(key)
        cands.append(x)
    sols = []
    for x0 in cands:
        try:
            x = mp.findroot(lambda *v: residual(structure, invs, moments, list(v)), x0, tol=mp.mpf("1e-50"),
                            maxsteps=40)
        except (ZeroDivisionError, ValueError):
            continue
        x = [x[i] for i in range(nun)]
        if max(abs(v) for v in residual(structure, invs, moments, x)) > mp.mpf("1e-45") or not valid(structure, x):
            continue
        sols.append(x)
    return structure, sols


# degrees 10-20 (up to 44 unknowns, beyond the random-start search) are completed by
# quad_orbits.polish from the tabulated rules as the reference build prints them
# (tests/golden/golden.npz, tri_<order>_p/w): the tabulated doubles start a multiprecision
# Gauss-Newton solve of the same moment equations, whose exact solution is written out
PINNED = list(range(10, 21))
KIND_OF_SIZE = {1: "C", 3: "T3", 6: "T6"}


def pinned_rule(deg, fixtures):
    import numpy as np
    import quad_orbits
    g = np.load(fixtures)
    P, W = g[f"tri_{deg}_p"], g[f"tri_{deg}_w"]
    pts, wts, rep = quad_orbits.polish(P.tolist(), W.tolist(), deg)
    structure = [KIND_OF_SIZE[size] for _, size in rep["orbits"]]
    print(f"triangle degree {deg}: {len(pts)} points from the tabulated rule, {rep['unknowns']} unknowns, "
          f"{rep['equations']} moments, residual {rep['residual']:.1e}, moved {rep['moved']:.1e}", file=sys.stderr)
    return structure, pts, wts


def main():
    import os
    fixtures = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "..", "tests", "golden", "golden.npz")
    rules = {}
    for deg in sorted(set(STRUCTURES) | set(PINNED)):
        if deg in PINNED:
            rules[deg] = pinned_rule(deg, fixtures)
            continue
        structure, sols = solve_degree(deg)
        if not sols:
            raise SystemExit(f"no valid triangle rule for degree {deg}")
        best = max(sols, key=lambda x: (round(float(min(unpack(structure, x)[1])), 12), depth(structure, x)))
        pars, ws = unpack(structure, best)
        pts, wts = [], []
        for kind, par, w in zip(structure, pars, ws):
            for pt in orbit_points(kind, par):
                pts.append(pt)
                wts.append(w)
        rules[deg] = (structure, pts, wts)
        print(f"triangle degree {deg}: {len(pts)} points, {len(sols)} valid solution(s)", file=sys.stderr)
    L = ["/* Generated by gen_tri_quadrature.py -- do not edit.",
         " * Fully symmetric triangle rules (centroid, Strang-Fix, Dunavant, Gatermann family), recomputed",
         " * from their orbit structure by Newton's method on the S3-invariant moment equations;",
         " * degrees 10-20 solved from the tabulated rules (quad_orbits.py).",
         " * Points: 3 barycentric coordinates each; weights sum to 1.  Plain C. */",
         "#ifndef ANIGPU_TRI_QUAD_TABLES_H",
         "#define ANIGPU_TRI_QUAD_TABLES_H"]
    for deg, (structure, pts, wts) in rules.items():
        L.append(f"/* degree {deg}: orbits {'+'.join(structure)}, {len(pts)} points */")
        L.append(f"static const int anigpu_tri_np{deg} = {len(pts)};")
        L.append(f"static const double anigpu_tri_pts{deg}[{3 * len(pts)}] = {{")
        for pt in pts:
            L.append("    " + ", ".join(mp.nstr(v, 20, min_fixed=-5, max_fixed=5) for v in pt) + ",")
        L.append("};")
        L.append(f"static const double anigpu_tri_wts{deg}[{len(pts)}] = {{")
        for w in wts:
            L.append("    " + mp.nstr(w, 20, min_fixed=-5, max_fixed=5) + ",")
        L.append("};")
    maxo = max(rules)
    L.append(f"#define ANIGPU_TRI_MAX_ORDER {maxo}")
    L.append(f"#define ANIGPU_TRI_MAX_POINTS {max(len(r[1]) for r in rules.values())}")
    L.append("/* order 0 is served by the centroid rule, orders 1..max by the rule of that degree */")
    L.append("static inline int anigpu_tri_rule(int order, const double** p, const double** w, int* np) {")
    L.append("  switch (order < 1 ? 1 : order) {")
    for deg in rules:
        L.append(f"    case {deg}: *p = anigpu_tri_pts{deg}; *w = anigpu_tri_wts{deg}; *np = anigpu_tri_np{deg}; return 1;")
    L.append("  }")
    L.append("  return 0;")
    L.append("}")
    L.append("#endif")
    path = sys.argv[1] if len(sys.argv) > 1 else "tri_quad_tables.h"
    with open(path, "w") as fh:
        fh.write("\n".join(L) + "\n")


if __name__ == "__main__":
    main()
