"""Quadrature tables: exactness of every generated rule (CPU)."""
import math
import os
import re

import numpy as np
import pytest

HDR = os.path.join(os.path.dirname(__file__), "..", "nihu_gb300", "csrc", "quad_rules.h")


def _macro(name):
    txt = open(HDR).read()
    m = re.search(r"#define %s \{(.*?)\}" % name, txt, re.S)
    return [float(v) for v in m.group(1).replace("\\", " ").split(",") if v.strip()]


def gauss(n):
    offs = [int(v) for v in _macro("NIHU_GAUSS_OFFSETS")]
    data = np.array(_macro("NIHU_GAUSS_DATA")).reshape(-1, 2)
    return data[offs[n - 1]:offs[n - 1] + n]


def tri(degree):
    npts = [int(v) for v in _macro("NIHU_TRI_NPTS")]
    offs = [int(v) for v in _macro("NIHU_TRI_OFFSETS")]
    data = np.array(_macro("NIHU_TRI_DATA")).reshape(-1, 3)
    return data[offs[degree]:offs[degree] + npts[degree]]


@pytest.mark.parametrize("n", range(1, 22))
def test_gauss_legendre_exact(n):
    r = gauss(n)
    assert np.all(np.diff(r[:, 0]) > 0)
    for p in range(2 * n):
        exact = 0.0 if p % 2 else 2.0 / (p + 1)
        assert abs(np.sum(r[:, 1] * r[:, 0] ** p) - exact) < 1e-14


@pytest.mark.parametrize("degree,npts", [(0, 1), (1, 1), (2, 3), (3, 4), (4, 6), (5, 7), (6, 12), (7, 13), (8, 16), (9, 19), (14, 42)])
def test_dunavant_exact(degree, npts):
    r = tri(degree)
    assert len(r) == npts
    assert abs(r[:, 2].sum() - 0.5) < 1e-15
    # points strictly inside the reference triangle (0,0),(1,0),(0,1)
    assert np.all(r[:, 0] > 0) and np.all(r[:, 1] > 0) and np.all(r[:, 0] + r[:, 1] < 1)
    for p in range(degree + 1):
        for q in range(degree + 1 - p):
            exact = math.factorial(p) * math.factorial(q) / math.factorial(p + q + 2)
            got = np.sum(r[:, 2] * r[:, 0] ** p * r[:, 1] ** q)
            assert abs(got - exact) < 1e-15, (p, q)


def test_dunavant_seed_degree14_matches_published_structure():
    # 6 orbits (a, a, 1-2a) and 4 orbits (a, b, 1-a-b): 6*3 + 4*6 = 42 points
    r = tri(14)
    bary = np.column_stack([1 - r[:, 0] - r[:, 1], r[:, 0], r[:, 1]])
    s21 = sum(1 for b in bary if np.isclose(b[0], b[1]) or np.isclose(b[1], b[2]) or np.isclose(b[0], b[2]))
    assert s21 == 18
