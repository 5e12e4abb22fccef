#!/usr/bin/env python3
"""Generate ``quad_rules.h``: the quadrature rules of the collocation BEM path.

Two families are produced, both to full double precision:

* Gauss-Legendre rules on [-1, 1] with n = 1..21 nodes.  Nodes are the roots of
  the Legendre polynomial P_n found by Newton iteration in 40-digit arithmetic;
  weights are 2 / ((1 - x^2) P_n'(x)^2).  These are the same rules the
  reference obtains from the Golub-Welsch eigenproblem
  (nihu/core/gaussian_quadrature.hpp:64-88); n = degree/2 + 1 per direction
  (:136-151 line, :186-202 quad tensor product).

* Dunavant (1985) symmetric rules on the reference triangle (0,0),(1,0),(0,1)
  for polynomial degrees 0..9 and 14 (nihu/core/gaussian_quadrature.hpp:209-513
  uses the same published rules; point counts 1,1,3,4,6,7,12,13,16,19 and 42).  Each
  rule is described by its orbit structure (centroid S3, S21 orbits
  (a, a, 1-2a), S111 orbits (a, b, 1-a-b)).  The orbit parameters are seeded
  with 4-6 significant digits of the published 1985 values and refined by
  Gauss-Newton iteration on the moment equations (all monomials up to the
  rule's degree) in 40-digit arithmetic, then rounded to double.  Weights are
  scaled to sum to 1/2 (the reference triangle's area).

Run ``python gen_quad_rules.py`` to rewrite ``quad_rules.h`` beside it.
"""
import itertools
import os
import sys

import mpmath as mp

mp.mp.dps = 40

# ---------------------------------------------------------------- Gauss-Legendre


def legendre_and_derivative(n, x):
    p0, p1 = mp.mpf(1), x
    if n == 0:
        return p0, mp.mpf(0)
    for k in range(2, n + 1):
        p0, p1 = p1, ((2 * k - 1) * x * p1 - (k - 1) * p0) / k
    dp = n * (x * p1 - p0) / (x * x - 1)
    return p1, dp


def gauss_legendre(n):
    nodes, weights = [], []
    for i in range(1, n + 1):
        x = mp.cos(mp.pi * (i - mp.mpf(1) / 4) / (n + mp.mpf(1) / 2))
        for _ in range(100):
            p, dp = legendre_and_derivative(n, x)
            dx = p / dp
            x -= dx
            if abs(dx) < mp.mpf(10) ** (-38):
                break
        p, dp = legendre_and_derivative(n, x)
        nodes.append(x)
        weights.append(2 / ((1 - x * x) * dp * dp))
    order = sorted(range(n), key=lambda k: nodes[k])
    return [nodes[k] for k in order], [weights[k] for k in order]


# ---------------------------------------------------------------- Dunavant

# orbit seeds: ('S3', w) | ('S21', a, w) | ('S111', a, b, w); weights sum to 1
DUNAVANT_SEEDS = {
    0: [("S3", 1.0)],
    1: [("S3", 1.0)],
    2: [("S21", 1.0 / 6.0, 1.0 / 3.0)],
    3: [("S3", -0.5625), ("S21", 0.2, 0.520833)],
    4: [("S21", 0.445948, 0.223382), ("S21", 0.091576, 0.109952)],
    5: [("S3", 0.225), ("S21", 0.470142, 0.132394), ("S21", 0.101287, 0.125939)],
    6: [("S21", 0.249287, 0.116786), ("S21", 0.063089, 0.050845),
        ("S111", 0.053145, 0.310352, 0.082851)],
    7: [("S3", -0.149570), ("S21", 0.260346, 0.175615), ("S21", 0.065130, 0.053347),
        ("S111", 0.048690, 0.312865, 0.077114)],
    8: [("S3", 0.144316), ("S21", 0.459293, 0.0950916), ("S21", 0.170569, 0.103217),
        ("S21", 0.0505472, 0.0324585), ("S111", 0.00839478, 0.263113, 0.0272303)],
    9: [("S3", 0.0971358), ("S21", 0.489682, 0.0313347), ("S21", 0.437090, 0.0778275),
        ("S21", 0.188204, 0.0796477), ("S21", 0.0447295, 0.0255777), ("S111", 0.0368384, 0.221963, 0.0432835)],
    14: [("S21", 0.488964, 0.0218836), ("S21", 0.417645, 0.0327884),
         ("S21", 0.273478, 0.0517741), ("S21", 0.177206, 0.0421626),
         ("S21", 0.0617999, 0.0144337), ("S21", 0.0193910, 0.00492340),
         ("S111", 0.0571248, 0.172267, 0.0246658), ("S111", 0.0929162, 0.336861, 0.0385715),
         ("S111", 0.0146470, 0.298373, 0.0144363), ("S111", 0.00126833, 0.118974, 0.00501023)],
}


def unpack(orbits):
    """Split seeds into a parameter vector and a structure list."""
    params, struct = [], []
    for o in orbits:
        struct.append(o[0])
        params.extend(mp.mpf(v) for v in o[1:])
    return params, struct


def expand(params, struct):
    """Return [(xi, eta, w)] for the orbit parameters (barycentric -> (xi, eta))."""
    pts, k = [], 0
    for kind in struct:
        if kind == "S3":
            w = params[k]; k += 1
            pts.append((mp.mpf(1) / 3, mp.mpf(1) / 3, w))
        elif kind == "S21":
            a, w = params[k], params[k + 1]; k += 2
            b = 1 - 2 * a
            for l1, l2, l3 in ((a, a, b), (a, b, a), (b, a, a)):
                pts.append((l2, l3, w / 3))
        else:
            a, b, w = params[k], params[k + 1], params[k + 2]; k += 3
            c = 1 - a - b
            for l1, l2, l3 in sorted(set(itertools.permutations((a, b, c)))):
                pts.append((l2, l3, w / 6))
    return pts


def exact_moment(p, q):
    # integral of xi^p eta^q over the reference triangle divided by its area 1/2
    return 2 * mp.factorial(p) * mp.factorial(q) / mp.factorial(p + q + 2)


def residual(params, struct, degree):
    pts = expand(params, struct)
    res = []
    for tot in range(degree + 1):
        for p in range(tot + 1):
            q = tot - p
            s = mp.fsum(w * x ** p * y ** q for x, y, w in pts)
            res.append(s - exact_moment(p, q))
    return res


def refine(degree):
    params, struct = unpack(DUNAVANT_SEEDS[degree])
    for _ in range(60):
        r = residual(params, struct, degree)
        if max(abs(v) for v in r) < mp.mpf(10) ** (-36):
            break
        h = mp.mpf(10) ** (-20)
        J = mp.matrix(len(r), len(params))
        for j in range(len(params)):
            pp = list(params)
            pp[j] += h
            rp = residual(pp, struct, degree)
            for i in range(len(r)):
                J[i, j] = (rp[i] - r[i]) / h
        # least-squares Gauss-Newton step
        JT = J.T
        step = mp.lu_solve(JT * J, JT * mp.matrix(r))
        params = [params[j] - step[j] for j in range(len(params))]
    r = residual(params, struct, degree)
    err = max(abs(v) for v in r)
    if err > mp.mpf(10) ** (-30):
        raise RuntimeError(f"Dunavant degree {degree} did not converge: {err}")
    pts = expand(params, struct)
    for x, y, w in pts:
        if not (x > 0 and y > 0 and x + y < 1):
            raise RuntimeError(f"Dunavant degree {degree}: point outside the triangle")
    return [(x, y, w / 2) for x, y, w in pts]


# ---------------------------------------------------------------- output


def fmt(v):
    return repr(float(v))


def main(out_path):
    lines = [
        "/* Quadrature rules of the collocation BEM path.",
        " * GENERATED by gen_quad_rules.py -- do not edit by hand.",
        " * Gauss-Legendre: roots of P_n by Newton iteration (40 digits).",
        " * Dunavant (1985) triangle rules: orbit parameters refined by",
        " * Gauss-Newton on the moment equations (40 digits); weights sum to 1/2.",
        " * Plain C; included by host and device code. */",
        "#ifndef NIHU_GB300_QUAD_RULES_H",
        "#define NIHU_GB300_QUAD_RULES_H",
        "",
        "#define NIHU_GAUSS_MAX_N 21",
    ]
    offs, data = [], []
    for n in range(1, 22):
        x, w = gauss_legendre(n)
        offs.append(len(data) // 2)
        for xi, wi in zip(x, w):
            data.extend([xi, wi])
    lines.append("/* offset (in points) of the n-point rule, n = 1..21, index n-1 */")
    lines.append("#define NIHU_GAUSS_OFFSETS { " + ", ".join(str(o) for o in offs) + " }")
    lines.append("/* (node, weight) pairs on [-1, 1] */")
    lines.append("#define NIHU_GAUSS_DATA { \\")
    for i in range(0, len(data), 4):
        lines.append("  " + ", ".join(fmt(v) for v in data[i:i + 4]) + ", \\")
    lines.append("}")
    lines.append("#define NIHU_GAUSS_DATA_LEN %d" % len(data))
    lines.append("")

    degrees = list(range(15))
    tri_offs, tri_npts, tri = [], [], []
    for d in degrees:
        if d in DUNAVANT_SEEDS:
            pts = refine(d)
            tri_offs.append(len(tri) // 3)
            tri_npts.append(len(pts))
            for x, y, w in pts:
                tri.extend([x, y, w])
        else:
            tri_offs.append(0)
            tri_npts.append(0)
    lines.append("#define NIHU_TRI_MAX_DEGREE 14")
    lines.append("/* number of points of the Dunavant rule of degree 0..14 (0: not provided) */")
    lines.append("#define NIHU_TRI_NPTS { " + ", ".join(str(v) for v in tri_npts) + " }")
    lines.append("#define NIHU_TRI_OFFSETS { " + ", ".join(str(v) for v in tri_offs) + " }")
    lines.append("/* (xi, eta, w) triples on the reference triangle */")
    lines.append("#define NIHU_TRI_DATA { \\")
    for i in range(0, len(tri), 3):
        lines.append("  " + ", ".join(fmt(v) for v in tri[i:i + 3]) + ", \\")
    lines.append("}")
    lines.append("#define NIHU_TRI_DATA_LEN %d" % len(tri))
    lines.append("")
    lines.append("#endif")
    with open(out_path, "w") as f:
        f.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    here = os.path.dirname(os.path.abspath(__file__))
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(here, "quad_rules.h"))
