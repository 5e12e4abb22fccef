"""Entry-by-entry comparison of assembled matrices against the oracle, shared
by the GPU parity tests and the CPU tests that check the comparison itself.

The bar: every entry of the FP32 mode within PER_ENTRY of its own magnitude.
A DLP entry of two coplanar flat elements (the diagonal, a cylinder column, a
cap) is exactly zero (r.n = 0 at every point) and the oracle's value is FP64
rounding, so those entries are bounded absolutely: within FLAT_ZERO of the
largest entry of the matrix.
"""
import numpy as np

import nihu_gb300 as g
from nihu_gb300 import meshes

PER_ENTRY = 1e-5  # every entry of the FP32 mode, relative to its own magnitude
FLAT_ZERO = 1e-6  # DLP entries of coplanar flat pairs, relative to the largest entry


def rel_norm(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def rel_entry(a, b):
    return (np.abs(a - b) / np.abs(b)).max()


def coplanar_pairs(mesh, tol=1e-9):
    """Boolean (n, n): the centre of element i lies in the plane of element j
    and the two normals are parallel (flat elements; the diagonal included)."""
    cen, nrm = meshes.centroids_and_normals(*mesh)
    parallel = np.abs(nrm @ nrm.T) > 1.0 - tol
    offset = np.abs(cen @ nrm.T - np.einsum("ij,ij->i", cen, nrm)[None, :])
    return parallel & (offset < tol)


def entry_check(got, ref, op, mesh):
    """(worst relative error over the checked entries, worst coplanar DLP
    error relative to the largest entry); SLP: every entry; DLP: coplanar
    pairs apart."""
    got = np.asarray(got, np.complex128)
    d = np.abs(got - ref)
    if op == g.DLP:
        cop = coplanar_pairs(mesh)
        flat = float(d[cop].max() / np.abs(ref).max()) if cop.any() else 0.0
        rest = ~cop
        return float((d[rest] / np.abs(ref[rest])).max()), flat
    assert np.abs(ref).min() > 0.0
    return float((d / np.abs(ref)).max()), 0.0


def assert_entries(got, ref, op, mesh, tol=PER_ENTRY, flat_tol=FLAT_ZERO):
    worst, flat = entry_check(got, ref, op, mesh)
    assert worst < tol, (op, worst)
    assert flat < flat_tol, (op, flat)
