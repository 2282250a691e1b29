"""The host-side coarse-space factors (sfem_coarse_factors, C++) against the coarse-space oracle:
the same aggregates and offsets, and bases that are orthonormal and span the same rigid motions
(the eigenvectors may differ in sign and order, so the checks are on projections).  No device
work: these run without a GPU."""
import numpy as np
import pytest

from oracle import coarse_oracle as co
from oracle.oracle import Oracle
from solidfem_gb300 import _native as nat
from solidfem_gb300.coarse import coarse_factors
from solidfem_gb300.mesh import box_lattice


def same_span(P1, P2, seed=0):
    v = np.random.default_rng(seed).normal(size=(P1.shape[0], 4))
    return np.abs(P1 @ (P1.T @ v) - P2 @ (P2.T @ v)).max() / np.abs(v).max()


@pytest.mark.parametrize("cell", [4 / 64, 16 / 64])
def test_factors_match_the_oracle_on_a_slab(cell):
    m = box_lattice(32, 8, 8, extent=(0.5, 0.125, 0.125), jitter=0.2, seed=0)
    o = Oracle(m.nodes, m.tets, m.face_nodes(2, 0), 1e5, 0.49)
    X = o.free_positions().reshape(-1, 3)
    aid, d, R = coarse_factors(X, cell)
    aid_o = co.aggregate_cells(X, cell)
    d_o, R_o = co.rigid_body_factors(X, aid_o)
    np.testing.assert_array_equal(aid, aid_o)
    np.testing.assert_allclose(d, d_o, rtol=0, atol=1e-15)
    P = co.basis_from_factors(aid, d, R)
    P_o = co.basis_from_factors(aid_o, d_o, R_o)
    assert P.shape == P_o.shape
    np.testing.assert_allclose((P.T @ P).toarray(), np.eye(P.shape[1]), atol=1e-12)
    assert same_span(P, P_o) < 1e-12


@pytest.mark.parametrize("cell,modes", [(4 / 64, 12), (16 / 64, 12), (4 / 64, 30), (16 / 64, 30)])
def test_polynomial_factors_span_the_oracles_modes(cell, modes):
    m = box_lattice(32, 8, 8, extent=(0.5, 0.125, 0.125), jitter=0.2, seed=0)
    o = Oracle(m.nodes, m.tets, m.face_nodes(2, 0), 1e5, 0.49)
    X = o.free_positions().reshape(-1, 3)
    aid, d, R = coarse_factors(X, cell, modes=modes)
    np.testing.assert_array_equal(aid, co.aggregate_cells(X, cell))
    P = co.basis_from_factors(aid, d, R)
    P_o = co.poly_basis(X, aid, 1 if modes == 12 else 2)
    assert P.shape == P_o.shape
    np.testing.assert_allclose((P.T @ P).toarray(), np.eye(P.shape[1]), atol=1e-10)
    assert same_span(P, P_o) < 1e-10


@pytest.mark.parametrize("modes,full,line", [(12, 12, 6), (30, 30, 9)])
def test_degenerate_aggregates_drop_polynomial_modes(modes, full, line):
    rng = np.random.default_rng(4)
    X = np.vstack([
        rng.uniform(0.0, 1.0, size=(40, 3)),              # a full aggregate: every mode
        [[2.5, 0.5, 0.5]],                                 # one point: translations only
        [[4.2, 0.5, 0.5], [4.5, 0.5, 0.5], [4.8, 0.5, 0.5]],  # collinear: 1, x (and x^2) per component
    ])
    aid, d, R = coarse_factors(X, 1.0, modes=modes)
    kept = (np.abs(R).sum(axis=1) > 0).sum(axis=1)
    np.testing.assert_array_equal(kept[aid[[0, 40, 41]]], [full, 3, line])
    P = co.basis_from_factors(aid, d, R)
    np.testing.assert_allclose((P.T @ P).toarray(), np.eye(P.shape[1]), atol=1e-10)
    assert same_span(P, co.poly_basis(X, co.aggregate_cells(X, 1.0), 1 if modes == 12 else 2)) < 1e-10


def test_degenerate_aggregates_drop_rotations():
    rng = np.random.default_rng(4)
    X = np.vstack([
        rng.uniform(0.0, 1.0, size=(20, 3)),              # a full aggregate: 6 modes
        [[2.5, 0.5, 0.5]],                                 # one point: translations only
        [[4.2, 0.5, 0.5], [4.5, 0.5, 0.5], [4.8, 0.5, 0.5]],  # collinear: no rotation about the line
    ])
    aid, d, R = coarse_factors(X, 1.0)
    kept = (np.abs(R).sum(axis=1) > 0).sum(axis=1)
    np.testing.assert_array_equal(kept[aid[[0, 20, 21]]], [6, 3, 5])
    P = co.basis_from_factors(aid, d, R)
    np.testing.assert_allclose((P.T @ P).toarray(), np.eye(P.shape[1]), atol=1e-12)
    assert same_span(P, co.rigid_body_basis(X, co.aggregate_cells(X, 1.0))) < 1e-12


def test_invalid_arguments():
    X = np.zeros((4, 3))
    with pytest.raises(nat.SfemError):
        coarse_factors(X, 0.0)
    with pytest.raises(nat.SfemError):
        coarse_factors(np.full((2, 3), np.nan), 1.0)
    with pytest.raises(nat.SfemError):
        coarse_factors(X, 0.0, modes=30)
    with pytest.raises(ValueError):
        coarse_factors(X, 1.0, modes=9)
    # the C entry point checks the degree itself
    import ctypes as C
    lib = nat.load()
    aid = np.empty(4, dtype=np.int32)
    d = np.empty((4, 3))
    na = C.c_int64()
    st = lib.sfem_coarse_factors_poly(np.ascontiguousarray(X).ctypes.data_as(nat._dp), 4, 1.0, 1e-8, 3,
                                      aid.ctypes.data_as(nat._ip), d.ctypes.data_as(nat._dp), None, C.byref(na))
    assert st != 0
