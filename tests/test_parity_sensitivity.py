"""The per-entry comparison of the GPU parity tests catches a wrong
quadrature level.

The FP32 kernel's warp-uniform paths pick a pair's quadrature level without
the per-lane classification, so the parity tests must fail when a pair gets
the wrong rule.  Here a wrong level is planted in the oracle's matrix on the
CPU -- one pair's entry recomputed with the rule of the next lower degree --
and the comparison the GPU tests use (parity.entry_check at PER_ENTRY) must
flag it.  Mesh and wave number are those of the 5120-triangle per-entry test.
"""
import numpy as np
import pytest

import nihu_gb300 as g
from nihu_gb300 import meshes
from parity import PER_ENTRY, entry_check


@pytest.fixture(scope="module")
def setup(oracle):
    mesh = meshes.icosphere(4)
    corners = meshes.element_corners(*mesh)[:, :3]
    cen, _ = meshes.centroids_and_normals(*mesh)
    rows = (0, 256)  # a block of rows keeps the CPU work small
    return mesh, corners, cen, rows


def wrong_level_changes(oracle, mesh, corners, cen, rows, op, k, deg_from, deg_to):
    """Relative change of every regular entry of degree deg_from in the row
    block when its rule is replaced by degree deg_to."""
    deg = oracle.degree(mesh, mesh, op, rows=rows)
    ii, jj = np.nonzero(deg == deg_from)
    out = []
    for i, j in zip(ii + rows[0], jj):
        good = oracle.elem_integral(corners[j], cen[i], oracle.HELMHOLTZ, op, k, 0, deg_from)
        bad = oracle.elem_integral(corners[j], cen[i], oracle.HELMHOLTZ, op, k, 0, deg_to)
        out.append((abs(bad - good) / abs(good), i, j, bad))
    return out


@pytest.mark.parametrize("op,deg_from,deg_to,floor", [(g.SLP, 4, 2, 3e-5), (g.SLP, 2, 0, 1e-3),
                                                     (g.DLP, 2, 0, 1e-3)])
def test_planted_wrong_level_fails_entry_check(oracle, setup, op, deg_from, deg_to, floor):
    """Every such pair's entry moves by more than PER_ENTRY (the smallest
    move is above `floor`), and an oracle matrix with one entry recomputed at
    the lower degree fails the GPU tests' per-entry comparison."""
    mesh, corners, cen, rows = setup
    k = 5.0
    ch = wrong_level_changes(oracle, mesh, corners, cen, rows, op, k, deg_from, deg_to)
    assert len(ch) > 10
    smallest = min(c[0] for c in ch)
    assert smallest > floor > PER_ENTRY, smallest
    ref = oracle.assemble(mesh, mesh, oracle.HELMHOLTZ, op, k, rows=rows, threads=8)
    n = len(mesh[1])
    full_ref = np.zeros((n, n), np.complex128)
    full_ref[rows[0]:rows[1]] = ref
    full_ref[rows[1]:] = 1.0  # rows outside the block: identical in both
    _, i, j, bad = min(ch)  # the pair at the class boundary: the smallest move
    planted = full_ref.copy()
    planted[i, j] = bad
    worst_ok, _ = entry_check(full_ref, full_ref, op, mesh)
    worst_bad, _ = entry_check(planted, full_ref, op, mesh)
    assert worst_ok == 0.0
    assert worst_bad > PER_ENTRY


def test_dlp_degree_four_to_two_at_the_class_boundary(oracle, setup):
    """Degree 2 in place of degree 4 moves a DLP entry least at the class
    boundary (d/D -> 2.8): there the two rules agree to about 1e-6, below
    PER_ENTRY and below what an FP32 entry resolves, so a wrong level there
    changes the entry by less than the bar.  The FP32 kernel takes the FP64
    decision for every pair within 1e-5 of a threshold (classify.cuh), so no
    such pair gets a wrong level; this records the size of the move."""
    mesh, corners, cen, rows = setup
    ch = wrong_level_changes(oracle, mesh, corners, cen, rows, g.DLP, 5.0, 4, 2)
    smallest = min(c[0] for c in ch)
    largest = max(c[0] for c in ch)
    assert 0.0 < smallest < PER_ENTRY, smallest
    assert largest > PER_ENTRY, largest
