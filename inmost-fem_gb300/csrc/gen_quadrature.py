#!/usr/bin/env python3
"""Generate the fully symmetric tetrahedron quadrature rules used by anigpu.

The rules are the symmetric cubatures of Jaskowiec & Sukumar (2021), "High-order
symmetric cubature rules for tetrahedra and pyramids", IJNME 122(1):148-171, the
family the reference library tabulates (anifem++/fem/quadrature_formulas.cpp:526-1502).
Nothing is copied from that table: every rule is recomputed here from its orbit
structure by solving the moment equations.

Method.  A rule is a set of orbits of the symmetric group S4 acting on barycentric
coordinates:
    S1        (1/4, 1/4, 1/4, 1/4)                     1 point
    S4(a)     (a, a, a, 1-3a)                          4 points
    S6(a)     (a, a, 1/2-a, 1/2-a)                     6 points
    S12(a,b)  (a, a, b, 1-2a-b)                       12 points
Each orbit carries one weight; weights sum to 1 (the reference integrates as
|T| * sum_n w_n f(x_n)).  A rule is exact to degree p iff it integrates every
S4-invariant polynomial of degree <= p exactly; those are spanned by
e2^i e3^j e4^k (elementary symmetric polynomials of the barycentric coordinates,
2i+3j+4k <= p).  For the orbit structures below the number of unknowns equals the
number of invariants, so the square system is solved by Newton's method in
multiprecision (mpmath) from many random starts; solutions with all points inside
the tetrahedron and positive weights are kept.  The exact moments use the Dirichlet
integral  E[l0^a l1^b l2^c l3^d] = 3! a! b! c! d! / (a+b+c+d+3)!.

Order 3 (two S4 orbits, 4 unknowns, 3 invariants: a one-parameter family of exact
8-point rules) and orders 7-20 (up to 115 unknowns, beyond a random-start search) are
completed by quad_orbits.polish from the tabulated rules as the reference build prints them
(tests/golden/golden.npz, quad_<order>_p/w): the tabulated doubles pin the member of the
family and start a multiprecision Gauss-Newton solve of the same moment equations, whose
exact solution is written out (within 1e-16 of the tabulated values).

Output: quad_tables.h (C header; points as 4 barycentric coordinates per point,
weights summing to 1) and, with --json, the same data as JSON.
"""
import itertools
import json
import math
import os
import random
import sys

import mpmath as mp
import sympy as sp

mp.mp.dps = 60

# orbit structure per generated degree: list of orbit kinds
STRUCTURES = {
    1: ["S1"],
    2: ["S4"],
    5: ["S4", "S4", "S6"],
    6: ["S4", "S4", "S4", "S12"],
}
# degrees completed from the tabulated rules (quad_orbits.polish)
PINNED = [3] + list(range(7, 21))
# order requested by a caller -> degree of the rule that serves it (quadrature_formulas.cpp:1492-1495:
# orders 0 and 1 share the centroid rule, orders 4 and 5 the degree-5 rule)
ORDER_TO_DEGREE = {0: 1, 1: 1, 2: 2, 3: 3, 4: 5, 5: 5, 6: 6, **{o: o for o in range(7, 21)}}
NPAR = {"S1": 0, "S4": 1, "S6": 1, "S12": 2}
NPTS = {"S1": 1, "S4": 4, "S6": 6, "S12": 12}


def orbit_points(kind, par):
    one = mp.mpf(1)
    if kind == "S1":
        return [(one / 4,) * 4]
    if kind == "S4":
        a = par[0]
        c = one - 3 * a
        return [tuple(c if i == k else a for i in range(4)) for k in range(4)]
    if kind == "S6":
        a = par[0]
        b = one / 2 - a
        pts = []
        for pair in itertools.combinations(range(4), 2):
            pts.append(tuple(a if i in pair else b for i in range(4)))
        return pts
    if kind == "S12":
        a, b = par
        c = one - 2 * a - b
        pts = []
        for ib in range(4):
            for ic in range(4):
                if ic == ib:
                    continue
                pts.append(tuple(b if i == ib else (c if i == ic else a) for i in range(4)))
        return pts
    raise ValueError(kind)


def invariants(deg):
    out = []
    for i in range(deg // 2 + 1):
        for j in range(deg // 3 + 1):
            for k in range(deg // 4 + 1):
                if 2 * i + 3 * j + 4 * k <= deg:
                    out.append((i, j, k))
    return out


_L = sp.symbols("l0:4")


def exact_moment(ijk):
    i, j, k = ijk
    l0, l1, l2, l3 = _L
    e2 = sum(_L[p] * _L[q] for p, q in itertools.combinations(range(4), 2))
    e3 = sum(_L[p] * _L[q] * _L[r] for p, q, r in itertools.combinations(range(4), 3))
    e4 = l0 * l1 * l2 * l3
    poly = sp.Poly(sp.expand(e2 ** i * e3 ** j * e4 ** k), *_L)
    tot = sp.Rational(0)
    for mon, coef in poly.terms():
        num = sp.Integer(6)
        for m in mon:
            num *= sp.factorial(m)
        tot += coef * num / sp.factorial(sum(mon) + 3)
    return tot


def eval_inv(ijk, pt):
    i, j, k = ijk
    l = pt
    e2 = sum(l[p] * l[q] for p, q in itertools.combinations(range(4), 2))
    e3 = sum(l[p] * l[q] * l[r] for p, q, r in itertools.combinations(range(4), 3))
    e4 = l[0] * l[1] * l[2] * l[3]
    return e2 ** i * e3 ** j * e4 ** k


def unpack(structure, x):
    pars, ws, p = [], [], 0
    for kind in structure:
        n = NPAR[kind]
        pars.append(x[p:p + n])
        p += n
    for kind in structure:
        ws.append(x[p])
        p += 1
    return pars, ws


def residual(structure, invs, moments, x):
    pars, ws = unpack(structure, x)
    res = []
    for ijk, m in zip(invs, moments):
        s = mp.mpf(0)
        for kind, par, w in zip(structure, pars, ws):
            # invariant polynomial is constant on an orbit
            s += w * NPTS[kind] * eval_inv(ijk, orbit_points(kind, par)[0])
        res.append(s - m)
    return res


def valid(structure, x, tol=mp.mpf("1e-40")):
    pars, ws = unpack(structure, x)
    for w in ws:
        if w <= 0:
            return False
    for kind, par in zip(structure, pars):
        for pt in orbit_points(kind, par):
            if min(pt) < -tol:
                return False
    return True


def canonical(structure, x):
    """Orbit parameters in a canonical form so that equal rules compare equal."""
    pars, ws = unpack(structure, x)
    items = []
    for kind, par, w in zip(structure, pars, ws):
        pts = sorted(tuple(float(v) for v in pt) for pt in orbit_points(kind, par))
        items.append((kind, tuple(pts[0]), float(w)))
    return tuple(sorted(items))


def _resid_f64(structure, invs, moments_f, x):
    pars, ws = unpack(structure, list(x))
    res = []
    reps = [orbit_points_f(kind, par)[0] for kind, par in zip(structure, pars)]
    for ijk, m in zip(invs, moments_f):
        s = 0.0
        for kind, rep, w in zip(structure, reps, ws):
            s += w * NPTS[kind] * eval_inv(ijk, rep)
        res.append(s - m)
    return res


def orbit_points_f(kind, par):
    if kind == "S1":
        return [(0.25,) * 4]
    if kind == "S4":
        a = par[0]
        return [(a, a, a, 1 - 3 * a)]
    if kind == "S6":
        a = par[0]
        return [(a, a, 0.5 - a, 0.5 - a)]
    a, b = par
    return [(a, a, b, 1 - 2 * a - b)]


def solve_degree(deg, tries=30, seed=12345):
    """Float64 multi-start search (scipy least squares), then a multiprecision Newton polish."""
    import numpy as np
    from scipy.optimize import least_squares
    structure = STRUCTURES[deg]
    invs = invariants(deg)
    moments = []
    for t in invs:
        r = sp.Rational(exact_moment(t))
        moments.append(mp.mpf(r.p) / mp.mpf(r.q))
    moments_f = [float(m) for m in moments]
    nun = sum(NPAR[k] for k in structure) + len(structure)
    assert nun == len(invs), (deg, nun, len(invs))
    rng = np.random.default_rng(seed)
    cands = []
    for _ in range(tries):
        x0 = []
        for kind in structure:
            if kind == "S4":
                x0.append(rng.uniform(0.0, 1.0 / 3.0))
            elif kind == "S6":
                x0.append(rng.uniform(0.0, 0.5))
            elif kind == "S12":
                a = rng.uniform(0.0, 0.5)
                x0.extend([a, rng.uniform(0.0, 1.0 - 2 * a)])
        for kind in structure:
            x0.append(rng.uniform(0.01, 1.0) / len(structure))
        sol = least_squares(lambda x: _resid_f64(structure, invs, moments_f, x), x0,
                            xtol=1e-15, ftol=1e-15, gtol=1e-15, max_nfev=400, method="lm")
        if np.max(np.abs(sol.fun)) > 1e-12:
            continue
        x = [mp.mpf(float(v)) for v in sol.x]
        if not valid(structure, x, tol=mp.mpf("1e-9")):
            continue
        key = canonical(structure, x)
        key = tuple((k, tuple(round(v, 8) for v in p), round(w, 8)) for k, p, w in key)
        if key in [c[0] for c in cands]:
            continue
        cands.append((key, x))
    sols = []
    for key, x0 in cands:
        f = lambda *x: residual(structure, invs, moments, list(x))
        try:
            x = mp.findroot(f, x0, tol=mp.mpf("1e-50"), maxsteps=30)
        except (ZeroDivisionError, ValueError):
            continue
        x = [x[i] for i in range(nun)]
        r = residual(structure, invs, moments, x)
        if max(abs(v) for v in r) > mp.mpf("1e-45") or not valid(structure, x):
            continue
        sols.append(x)
    return structure, sols


def expand(structure, x):
    pars, ws = unpack(structure, x)
    pts, wts = [], []
    for kind, par, w in zip(structure, pars, ws):
        for pt in orbit_points(kind, par):
            pts.append(pt)
            wts.append(w)
    return pts, wts


KIND_OF_SIZE = {1: "S1", 4: "S4", 6: "S6", 12: "S12", 24: "S24"}


def pinned_rule(deg, fixtures):
    import numpy as np
    import quad_orbits
    g = np.load(fixtures)
    P, W = g[f"quad_{deg}_p"], g[f"quad_{deg}_w"]
    pts, wts, rep = quad_orbits.polish(P.tolist(), W.tolist(), deg)
    structure = [KIND_OF_SIZE[size] for _, size in rep["orbits"]]
    print(f"degree {deg}: {len(pts)} points from the tabulated rule, {rep['unknowns']} unknowns, "
          f"{rep['equations']} moments, residual {rep['residual']:.1e}, moved {rep['moved']:.1e}", file=sys.stderr)
    return structure, pts, wts


def main():
    here = os.path.dirname(os.path.abspath(__file__))
    fixtures = os.path.join(here, "..", "..", "tests", "golden", "golden.npz")
    rules = {}
    for deg in sorted(set(STRUCTURES) | set(PINNED)):
        if deg in PINNED:
            structure, pts, wts = pinned_rule(deg, fixtures)
            rules[deg] = (structure, pts, wts, 1)
            continue
        structure, sols = solve_degree(deg)
        if not sols:
            raise SystemExit(f"no valid rule found for degree {deg}")
        # several valid solutions: keep the one whose smallest weight is largest
        best = max(sols, key=lambda x: min(unpack(structure, x)[1]))
        pts, wts = expand(structure, best)
        rules[deg] = (structure, pts, wts, len(sols))
        print(f"degree {deg}: {len(pts)} points, {len(sols)} valid solution(s)", file=sys.stderr)

    lines = []
    lines.append("/* Generated by gen_quadrature.py -- do not edit.")
    lines.append(" * Fully symmetric tetrahedron rules (Jaskowiec & Sukumar 2021 family), recomputed")
    lines.append(" * from their orbit structure by Newton's method on the S4-invariant moment equations;")
    lines.append(" * degrees " + ", ".join(str(d) for d in PINNED) + " solved from the tabulated rules")
    lines.append(" * (quad_orbits.py), which pin the member of an underdetermined family (degree 3).")
    lines.append(" * Points: 4 barycentric coordinates each (lambda_0 belongs to vertex 0); weights sum to 1.")
    lines.append(" * Plain C so that both the CUDA library and the C oracle can include it. */")
    lines.append("#ifndef ANIGPU_QUAD_TABLES_H")
    lines.append("#define ANIGPU_QUAD_TABLES_H")
    for deg, (structure, pts, wts, nsol) in rules.items():
        lines.append(f"/* degree {deg}: orbits {'+'.join(structure)}, {len(pts)} points */")
        lines.append(f"static const int anigpu_quad_np{deg} = {len(pts)};")
        lines.append(f"static const double anigpu_quad_pts{deg}[{4 * len(pts)}] = {{")
        for pt in pts:
            lines.append("    " + ", ".join(mp.nstr(v, 20, min_fixed=-5, max_fixed=5) for v in pt) + ",")
        lines.append("};")
        lines.append(f"static const double anigpu_quad_wts{deg}[{len(pts)}] = {{")
        for w in wts:
            lines.append("    " + mp.nstr(w, 20, min_fixed=-5, max_fixed=5) + ",")
        lines.append("};")
    maxo = max(ORDER_TO_DEGREE)
    lines.append(f"#define ANIGPU_QUAD_MAX_ORDER {maxo}")
    lines.append(f"#define ANIGPU_QUAD_MAX_POINTS {max(len(r[1]) for r in rules.values())}")
    lines.append("/* quadrature order requested by a caller -> degree of the rule that serves it */")
    lines.append("static const int anigpu_quad_order_to_degree[ANIGPU_QUAD_MAX_ORDER + 1] = {"
                 + ", ".join(str(ORDER_TO_DEGREE[o]) for o in range(maxo + 1)) + "};")
    lines.append("static inline int anigpu_quad_rule(int order, const double** p, const double** w, int* np) {")
    lines.append("  if (order < 0 || order > ANIGPU_QUAD_MAX_ORDER) return 0;")
    lines.append("  switch (anigpu_quad_order_to_degree[order]) {")
    for deg in rules:
        lines.append(f"    case {deg}: *p = anigpu_quad_pts{deg}; *w = anigpu_quad_wts{deg}; *np = anigpu_quad_np{deg}; return 1;")
    lines.append("  }")
    lines.append("  return 0;")
    lines.append("}")
    lines.append("#endif")
    out = "\n".join(lines) + "\n"
    path = sys.argv[1] if len(sys.argv) > 1 else "quad_tables.h"
    with open(path, "w") as fh:
        fh.write(out)


if __name__ == "__main__":
    main()
