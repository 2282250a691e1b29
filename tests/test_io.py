"""Mesh / scene formats (Source/FemIO.cpp): tet1 and vol readers, XML scenes, VTK export.
CPU only; the reference's own model file is read when the reference tree is present."""
import os

import numpy as np
import pytest

from oracle.oracle import REF_TREE
from solidfem_gb300 import io
from solidfem_gb300.mesh import box_lattice

HERE = os.path.dirname(os.path.abspath(__file__))
REF_MODELS = os.path.join(REF_TREE, "Models")


def test_tet1_roundtrip_swaps_y_and_z(tmp_path):
    m = box_lattice(3, 2, 2, extent=(1.0, 0.5, 0.25), jitter=0.1, seed=1)
    p = tmp_path / "m.tet"
    io.save_tet1(str(p), m.nodes, m.tets)
    txt = p.read_text().splitlines()
    x, y, z = (float(w) for w in txt[1].split()[1:])
    np.testing.assert_allclose([x, z, y], m.nodes[1])  # the file stores (x, z, y)
    nodes, tets = io.load_tet1(str(p))
    np.testing.assert_array_equal(nodes, m.nodes)
    np.testing.assert_array_equal(tets, m.tets)
    nodes2, _ = io.load_tet1(str(p), scale=2.0, offset=(1.0, 0.0, 0.0))
    np.testing.assert_allclose(nodes2, 2.0 * m.nodes + [1.0, 0.0, 0.0])


@pytest.mark.skipif(not os.path.isdir(REF_MODELS), reason="reference models not present")
def test_tet1_reads_reference_box2_like_the_reference():
    g = np.load(os.path.join(HERE, "golden", "box2_nh.npz"))
    nodes, tets = io.load_tet1(os.path.join(REF_MODELS, "box2.tet"))
    np.testing.assert_array_equal(nodes, g["nodes"])
    np.testing.assert_array_equal(tets, g["tets"])


def test_vol_reader(tmp_path):
    p = tmp_path / "m.vol"
    p.write_text("mesh3d\nvolumeelements\n2\n1 4 1 2 3 4\n1 4 2 3 4 5\n\npoints\n5\n"
                 "0 0 0\n1 0 0\n0 1 0\n0 0 1\n1 1 1\n")
    nodes, tets = io.load_vol(str(p), scale=0.5)
    np.testing.assert_array_equal(tets, [[0, 1, 2, 3], [1, 2, 3, 4]])
    np.testing.assert_allclose(nodes[4], [0.5, 0.5, 0.5])


def test_xml_scene(tmp_path):
    m = box_lattice(4, 1, 1, extent=(4.0, 1.0, 1.0))
    io.save_tet1(str(tmp_path / "box.tet"), m.nodes, m.tets)
    (tmp_path / "scene.xml").write_text(
        '<solidfem>\n <model path="box.tet" type="tet1" scale="2" swap="xy">\n'
        '  <dirichlet>0, 1 2 3</dirichlet>\n </model>\n'
        ' <material name="neo-hookean" young="66000" poisson="0.45" density="1070"/>\n'
        ' <simulation type="quasi-static" steps="4" method="nonlinear" gravity="-9.8">\n'
        '  <pressure p="250"/>\n </simulation>\n'
        ' <solver method="newton" iterations="100" tolerance="0.1"/>\n</solidfem>\n')
    s = io.load_xml(str(tmp_path / "scene.xml"))
    np.testing.assert_allclose(s.nodes, 2.0 * m.nodes[:, [1, 0, 2]])
    np.testing.assert_array_equal(s.fixed, [0, 1, 2, 3])
    assert s.config == {"material": 3, "young": 66000.0, "poisson": 0.45, "density": 1070.0, "gravity": -9.8,
                        "maxiter": 100, "tol": 0.1, "solver": "newton"}
    assert s.sim_type == io.SIM_QUASI_STATIC and s.steps == 4 and s.pressure == 250.0


def test_vtk_export(tmp_path):
    m = box_lattice(2, 1, 1)
    u = np.random.default_rng(0).normal(size=m.nodes.shape) * 1e-3
    P = np.random.default_rng(1).normal(size=(m.n_tets, 3, 3))
    p = tmp_path / "out.vtk"
    io.export_vtk(str(p), m.nodes + u, m.tets, u, P)
    lines = p.read_text().splitlines()
    assert lines[0] == "# vtk DataFile Version 2.0" and lines[3] == "DATASET UNSTRUCTURED_GRID"
    i = lines.index(f"POINTS {m.n_nodes} double")
    np.testing.assert_allclose(np.loadtxt(lines[i + 1:i + 1 + m.n_nodes]), m.nodes + u, atol=1e-6)
    i = lines.index(f"CELLS {m.n_tets} {5 * m.n_tets}")
    np.testing.assert_array_equal(np.loadtxt(lines[i + 1:i + 1 + m.n_tets], dtype=int)[:, 1:], m.tets)
    i = lines.index("TENSORS stress float")
    np.testing.assert_allclose(np.loadtxt(lines[i + 1:i + 4]), P[0], rtol=1e-8)
