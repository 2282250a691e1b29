import numpy as np

from solidfem_gb300.mesh import box_lattice, lumped_face_load, random_top_traction


def vols(m):
    x = m.nodes[m.tets]
    return np.linalg.det(np.stack([x[:, 1] - x[:, 0], x[:, 2] - x[:, 0], x[:, 3] - x[:, 0]], axis=2)) / 6


def test_counts_and_orientation():
    m = box_lattice(16, 4, 4, extent=(4, 1, 1))
    assert m.n_nodes == 425 and m.n_tets == 1536
    v = vols(m)
    assert (v > 0).all()
    np.testing.assert_allclose(v.sum(), 4.0, rtol=1e-12)


def test_conforming_faces():
    # every interior triangle is shared by exactly two tets
    m = box_lattice(4, 3, 2, jitter=0.2, seed=3)
    f = np.sort(m.tets[:, [[1, 2, 3], [0, 2, 3], [0, 1, 3], [0, 1, 2]]].reshape(-1, 3), axis=1)
    _, c = np.unique(f, axis=0, return_counts=True)
    assert set(np.unique(c)) <= {1, 2}
    nb = (c == 1).sum()
    assert nb == 2 * (4 * 3 + 3 * 2 + 4 * 2) * 2
    assert (vols(m) > 0).all()


def test_lumped_load_total():
    m = box_lattice(8, 2, 2, extent=(8, 2, 2))
    f = lumped_face_load(m, 0, 1, (0, 0, -500.0))
    np.testing.assert_allclose(f.sum(axis=0), [0, 0, -500.0 * 4], rtol=1e-12)
    assert set(np.nonzero(f[:, 2])[0]) == set(m.face_nodes(0, 1))


def test_random_traction_stats():
    m = box_lattice(32, 8, 8, extent=(4, 1, 1))
    f = random_top_traction(m, seed=10000)
    top = m.face_nodes(2, 1)
    assert np.abs(f[np.setdiff1d(np.arange(m.n_nodes), top)]).max() == 0
    assert np.abs(f[:, :2]).max() == 0
    f2 = random_top_traction(m, seed=10000)
    np.testing.assert_array_equal(f, f2)
