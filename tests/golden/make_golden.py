"""Generate the golden fixtures in this folder.

The reference ships no golden vectors (its drivers only print totals), and it
cannot be built here (CGAL, Eigen and GMP are absent).  These fixtures therefore
come from an exact restatement of the quantities ``MA::kantorovich`` and
``MA::first_moment`` / ``MA::second_moment`` define, computed in rational
arithmetic (``fractions.Fraction``) for tiny inputs:

* every Laguerre piece (power cell of site i) ∩ (triangle f) is obtained by exact
  clipping of f by the closed half-planes  |x-x_i|^2 - w_i <= |x-x_j|^2 - w_j,
  against every other site j (no neighbour search, no predicates to trust);
* mass, value and moments are exact rationals: a degree-3 quadrature rule that is
  exact for cubics is evaluated in rational arithmetic and checked against the
  simplex monomial integrals below;
* the Hessian entries -int_{edge} rho / (2 |x_i - x_j|) contain square roots and
  are evaluated with mpmath at 60 significant digits.

The results are rounded to doubles once, at the end.  Run from the repo root:
``python tests/golden/make_golden.py`` (takes a few seconds).
"""
from __future__ import annotations

import json
import os
from fractions import Fraction as Fr

import mpmath
import numpy as np

mpmath.mp.dps = 60
HERE = os.path.dirname(os.path.abspath(__file__))

# degree-3 rule on a triangle: weight 1/20 at each vertex, 2/15 at each edge
# midpoint, 9/20 at the centroid (exact for every polynomial of degree <= 3)
RULE_V, RULE_M, RULE_C = Fr(1, 20), Fr(2, 15), Fr(9, 20)


def tri_integral(p0, p1, p2, f):
    area = ((p1[0] - p0[0]) * (p2[1] - p0[1]) - (p2[0] - p0[0]) * (p1[1] - p0[1])) / 2
    mid = lambda a, b: ((a[0] + b[0]) / 2, (a[1] + b[1]) / 2)
    cen = ((p0[0] + p1[0] + p2[0]) / 3, (p0[1] + p1[1] + p2[1]) / 3)
    s = RULE_V * (f(p0) + f(p1) + f(p2)) + RULE_M * (f(mid(p0, p1)) + f(mid(p1, p2)) + f(mid(p2, p0)))
    s += RULE_C * f(cen)
    return area * s


def _check_rule():
    # on the unit simplex, int s^i t^j = i! j! / (i + j + 2)!
    from math import factorial
    z, a, b = (Fr(0), Fr(0)), (Fr(1), Fr(0)), (Fr(0), Fr(1))
    for i in range(4):
        for j in range(4 - i):
            got = tri_integral(z, a, b, lambda p: p[0] ** i * p[1] ** j)
            want = Fr(factorial(i) * factorial(j), factorial(i + j + 2))
            assert got == want, (i, j, got, want)


def pi_(site_i, site_j, p):
    """|p - x_i|^2 - w_i - (|p - x_j|^2 - w_j)"""
    (xi, yi, wi), (xj, yj, wj) = site_i, site_j
    return ((p[0] - xi) ** 2 + (p[1] - yi) ** 2 - wi) - ((p[0] - xj) ** 2 + (p[1] - yj) ** 2 - wj)


def clip(poly, labels, si, sj, j):
    """Keep {pi_(si, sj, .) <= 0}.  labels[k] tags the edge poly[k] -> poly[k+1]:
    -1 for a mesh edge, the site index for a bisector."""
    n = len(poly)
    if n == 0:
        return [], []
    val = [pi_(si, sj, p) for p in poly]
    out, lab = [], []
    for k in range(n):
        k1 = (k + 1) % n
        a, b = val[k], val[k1]
        if a <= 0:
            out.append(poly[k])
            lab.append(labels[k])
            if b > 0:
                t = a / (a - b)
                q = (poly[k][0] + t * (poly[k1][0] - poly[k][0]), poly[k][1] + t * (poly[k1][1] - poly[k][1]))
                if q != poly[k]:
                    out.append(q)
                    lab.append(j)
                else:
                    lab[-1] = j
        elif b <= 0:
            t = a / (a - b)
            q = (poly[k][0] + t * (poly[k1][0] - poly[k][0]), poly[k][1] + t * (poly[k1][1] - poly[k][1]))
            if q != poly[k1]:
                out.append(q)
                lab.append(labels[k])
    # drop zero-length edges
    m = len(out)
    keep_p, keep_l = [], []
    for k in range(m):
        if out[k] != out[(k + 1) % m]:
            keep_p.append(out[k])
            keep_l.append(lab[k])
    return keep_p, keep_l


def poly_area(poly):
    s = Fr(0)
    for k in range(len(poly)):
        a, b = poly[k], poly[(k + 1) % len(poly)]
        s += a[0] * b[1] - b[0] * a[1]
    return s / 2


def linear_fn(p, q, r, fp, fq, fr):
    """rho = a x + b y + c through the three vertex values (exact)."""
    M = [[p[0], p[1], Fr(1)], [q[0], q[1], Fr(1)], [r[0], r[1], Fr(1)]]
    rhs = [fp, fq, fr]
    det = lambda A: (A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) - A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0])
                     + A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]))
    D = det(M)
    sol = []
    for c in range(3):
        A = [row[:] for row in M]
        for k in range(3):
            A[k][c] = rhs[k]
        sol.append(det(A) / D)
    return sol


def compute(mesh, x, y, w):
    V = [(Fr(a), Fr(b)) for a, b in zip(mesh["vx"], mesh["vy"])]
    vals = [Fr(v) for v in mesh["values"]]
    S = [(Fr(a), Fr(b), Fr(c)) for a, b, c in zip(x, y, w)]
    n = len(S)
    g = [Fr(0)] * n
    second = [Fr(0)] * n
    mom = [[Fr(0)] * 6 for _ in range(n)]
    H = {}
    pieces = []
    for f, t in enumerate(mesh["tri"]):
        a, b, c = linear_fn(V[t[0]], V[t[1]], V[t[2]], vals[t[0]], vals[t[1]], vals[t[2]])
        rho = lambda p: a * p[0] + b * p[1] + c
        for i in range(n):
            poly = [V[t[0]], V[t[1]], V[t[2]]]
            lab = [-1, -1, -1]
            for j in range(n):
                if j == i:
                    continue
                poly, lab = clip(poly, lab, S[i], S[j], j)
                if not poly:
                    break
            if len(poly) < 3 or poly_area(poly) == 0:
                continue
            xi, yi = S[i][0], S[i][1]
            pieces.append((f, i, len(poly)))
            for k in range(1, len(poly) - 1):
                p0, p1, p2 = poly[0], poly[k], poly[k + 1]
                g[i] += tri_integral(p0, p1, p2, rho)
                second[i] += tri_integral(p0, p1, p2, lambda p: rho(p) * ((p[0] - xi) ** 2 + (p[1] - yi) ** 2))
                fs = (lambda p: rho(p), lambda p: rho(p) * p[0], lambda p: rho(p) * p[1],
                      lambda p: rho(p) * p[0] ** 2, lambda p: rho(p) * p[1] ** 2, lambda p: rho(p) * p[0] * p[1])
                for q in range(6):
                    mom[i][q] += tri_integral(p0, p1, p2, fs[q])
            for k, j in enumerate(lab):
                if j < 0:
                    continue
                p, q = poly[k], poly[(k + 1) % len(poly)]
                L = mpmath.sqrt(mpmath.mpf(Fr((q[0] - p[0]) ** 2 + (q[1] - p[1]) ** 2).numerator)
                                / mpmath.mpf(Fr((q[0] - p[0]) ** 2 + (q[1] - p[1]) ** 2).denominator))
                mid = ((p[0] + q[0]) / 2, (p[1] + q[1]) / 2)
                rm = rho(mid)
                r = L * mpmath.mpf(rm.numerator) / mpmath.mpf(rm.denominator)
                d2 = (S[i][0] - S[j][0]) ** 2 + (S[i][1] - S[j][1]) ** 2
                d = 2 * mpmath.sqrt(mpmath.mpf(d2.numerator) / mpmath.mpf(d2.denominator))
                H[(i, j)] = H.get((i, j), mpmath.mpf(0)) - r / d
                H[(i, i)] = H.get((i, i), mpmath.mpf(0)) + r / d
    value = sum((S[i][2] * g[i] - second[i] for i in range(n)), Fr(0))
    hess = sorted([[i, j, float(v)] for (i, j), v in H.items()])
    return {
        "value": float(value),
        "g": [float(v) for v in g],
        "moments": [[float(v) for v in row] for row in mom],
        "hessian": hess,
        "pieces": sorted([list(p) for p in pieces]),
    }


def grid_mesh(gx, gy, values):
    nx, ny = len(gx), len(gy)
    vx, vy, tri = [], [], []
    for j in range(ny):
        for i in range(nx):
            vx.append(float(gx[i]))
            vy.append(float(gy[j]))
    for j in range(ny - 1):
        for i in range(nx - 1):
            k = j * nx + i
            tri.append([k, k + 1, k + nx + 1])
            tri.append([k, k + nx + 1, k + nx])
    return {"kind": "grid", "gx": [float(v) for v in gx], "gy": [float(v) for v in gy],
            "values": [float(v) for v in np.ravel(values)], "vx": vx, "vy": vy, "tri": tri}


def cases():
    rng = np.random.Generator(np.random.PCG64(20240611))
    out = []
    g2 = np.linspace(0.0, 1.0, 2)
    out.append(("one_site", grid_mesh(g2, g2, [1.0, 2.0, 3.0, 4.0]), [0.3], [0.6], [0.0]))
    out.append(("two_sites", grid_mesh(g2, g2, rng.uniform(0.5, 1.5, 4)), [0.2, 0.7], [0.3, 0.6], [0.0, 0.05]))
    g3 = np.linspace(0.0, 1.0, 3)
    p = rng.uniform(0, 1, (5, 2))
    out.append(("five_sites_grid3", grid_mesh(g3, g3, rng.uniform(0.5, 1.5, 9)), p[:, 0], p[:, 1],
                rng.uniform(-0.02, 0.02, 5)))
    g4 = np.linspace(0.0, 1.0, 4)
    p = rng.uniform(0, 1, (8, 2))
    out.append(("eight_sites_grid4", grid_mesh(g4, g4, rng.uniform(0.5, 1.5, 16)), p[:, 0], p[:, 1],
                rng.uniform(-0.01, 0.01, 8)))
    # a hidden site (its weight is so low that its power cell is empty)
    p = rng.uniform(0.1, 0.9, (4, 2))
    out.append(("hidden_site", grid_mesh(g3, g3, rng.uniform(0.5, 1.5, 9)),
                list(p[:, 0]) + [0.5], list(p[:, 1]) + [0.5], [0.0, 0.0, 0.0, 0.0, -1.0]))
    # sites outside the mesh whose cells still reach into it
    p = rng.uniform(0, 1, (5, 2))
    out.append(("outside_sites", grid_mesh(g3, g3, rng.uniform(0.5, 1.5, 9)),
                list(p[:, 0]) + [1.3, -0.2], list(p[:, 1]) + [0.5, 0.8], [0.0] * 5 + [0.1, 0.05]))
    # non-uniform grid spacing
    gxn = np.array([0.0, 0.15, 0.5, 1.0])
    gyn = np.array([0.0, 0.6, 1.0])
    p = rng.uniform(0, 1, (6, 2))
    out.append(("nonuniform_grid", grid_mesh(gxn, gyn, rng.uniform(0.5, 1.5, 12)), p[:, 0], p[:, 1],
                rng.uniform(-0.01, 0.01, 6)))
    # an explicit, non-grid triangulation: a hexagon fan around an off-centre vertex
    ang = np.arange(6) * np.pi / 3 + 0.1
    vx = [0.52] + list(0.5 + 0.45 * np.cos(ang))
    vy = [0.47] + list(0.5 + 0.45 * np.sin(ang))
    tri = [[0, 1 + k, 1 + (k + 1) % 6] for k in range(6)]
    mesh = {"kind": "tri", "vx": [float(v) for v in vx], "vy": [float(v) for v in vy],
            "values": [float(v) for v in rng.uniform(0.5, 1.5, 7)], "tri": tri}
    p = rng.uniform(0.2, 0.8, (6, 2))
    out.append(("hexagon_mesh", mesh, p[:, 0], p[:, 1], rng.uniform(-0.01, 0.01, 6)))
    # a non-convex (L-shaped) domain: adjacency is restricted to the mesh
    vx = [0, 1, 2, 0, 1, 2, 0, 1]
    vy = [0, 0, 0, 1, 1, 1, 2, 2]
    tri = [[0, 1, 4], [0, 4, 3], [1, 2, 5], [1, 5, 4], [3, 4, 7], [3, 7, 6]]
    mesh = {"kind": "tri", "vx": [float(v) / 2 for v in vx], "vy": [float(v) / 2 for v in vy],
            "values": [float(v) for v in rng.uniform(0.5, 1.5, 8)], "tri": tri}
    p = rng.uniform(0.05, 0.95, (7, 2))
    out.append(("l_shape_mesh", mesh, p[:, 0], p[:, 1], rng.uniform(-0.01, 0.01, 7)))
    return out


def main():
    _check_rule()
    for name, mesh, x, y, w in cases():
        res = compute(mesh, list(map(float, x)), list(map(float, y)), list(map(float, w)))
        doc = {"name": name, "mesh": mesh, "x": [float(v) for v in x], "y": [float(v) for v in y],
               "w": [float(v) for v in w], **res}
        with open(os.path.join(HERE, name + ".json"), "w") as fh:
            json.dump(doc, fh, indent=1)
        print(name, len(res["pieces"]), "pieces", len(res["hessian"]), "nnz")


if __name__ == "__main__":
    main()
