"""Mesh and scene formats of SolidFEM: the 'tet1' text mesh, the Netgen 'vol' mesh, the
XML scene description and the legacy-VTK heat-map export.

* ``load_tet1``  follows ``IO::LoadFromTet1File`` (Source/FemIO.cpp:506-570): lines
  ``v x y z`` and ``t i j k l``; the reader swaps y and z of every node, then applies
  ``scale * pos + offset``.
* ``load_vol``   follows ``IO::LoadFromVolFile`` (Source/FemIO.cpp:401-504): the
  ``volumeelements`` block (``matnr np i1 i2 i3 i4``, 1-based) and the ``points`` block,
  positions scaled.
* ``load_xml``   follows ``IO::LoadFromXmlFile`` (Source/FemIO.cpp:572-848): ``<model path type
  scale swap>`` with ``<dirichlet>`` node ids, ``<material name young poisson density>``,
  ``<simulation type method steps gravity>`` with ``<pressure p>``, ``<solver method iterations
  tolerance>``.  The result carries the keys of ``pysolidfem.NonlinearFEM``'s config dict.
* ``export_vtk`` writes what ``IO::ExportToVTKHeatMap`` writes (Source/FemIO.cpp:317-399):
  deformed points, tetra cells, point displacements and cell PK1 stress tensors.
"""
from __future__ import annotations

import os
import xml.etree.ElementTree as ET
from dataclasses import dataclass, field

import numpy as np

# FemDataStructures.h: MaterialModelType / SimulationType / MethodType ordinals
MATERIAL_IDS = {"linear": 0, "stvk": 1, "corotational": 2, "neo-hookean": 3}
SIM_STATIC, SIM_QUASI_STATIC, SIM_EXPLICIT = 0, 1, 2


def load_tet1(path: str, scale: float = 1.0, offset=(0.0, 0.0, 0.0)):
    """Nodes (N, 3) and tets (E, 4) of a 'tet1' file, with the reference reader's y<->z swap."""
    nodes, tets = [], []
    with open(path) as f:
        for line in f:
            if line.startswith("v"):
                x, y, z = (float(w) for w in line[2:].split()[:3])
                nodes.append((x, z, y))
            elif line.startswith("t"):
                tets.append([int(w) for w in line[2:].split()[:4]])
    x = np.asarray(nodes, dtype=np.float64).reshape(-1, 3) * scale + np.asarray(offset, dtype=np.float64)
    return x, np.asarray(tets, dtype=np.int32).reshape(-1, 4)


def save_tet1(path: str, nodes, tets) -> None:
    """Write a 'tet1' file that ``load_tet1`` (and the reference reader) reads back as ``nodes``."""
    nodes = np.asarray(nodes, dtype=np.float64)
    with open(path, "w") as f:
        for x, y, z in nodes.tolist():
            f.write(f"v {x!r} {z!r} {y!r}\n")
        for t in np.asarray(tets, dtype=np.int64):
            f.write("t {} {} {} {}\n".format(*t))


def load_vol(path: str, scale: float = 1.0):
    """Nodes and tets of a Netgen 'vol' file (1-based element indices become 0-based)."""
    nodes, tets = [], []
    with open(path) as f:
        lines = [ln.strip() for ln in f]
    i = 0
    while i < len(lines):
        key = lines[i]
        if key == "volumeelements":
            n = int(lines[i + 1].split()[0])
            for ln in lines[i + 2:i + 2 + n]:
                w = ln.split()
                tets.append([int(v) - 1 for v in w[2:6]])
            i += 2 + n
        elif key == "points":
            n = int(lines[i + 1].split()[0])
            for ln in lines[i + 2:i + 2 + n]:
                nodes.append([float(v) for v in ln.split()[:3]])
            i += 2 + n
        else:
            i += 1
    return np.asarray(nodes, dtype=np.float64).reshape(-1, 3) * scale, np.asarray(tets, dtype=np.int32).reshape(-1, 4)


@dataclass
class Scene:
    nodes: np.ndarray
    tets: np.ndarray
    fixed: np.ndarray
    config: dict = field(default_factory=dict)   # NonlinearFEM config keys
    sim_type: int = SIM_STATIC
    steps: int = 1
    pressure: float | None = None
    visual: str | None = None


def _ints(text: str):
    return [int(v) for v in text.replace(",", " ").split()] if text else []


def load_xml(path: str) -> Scene:
    """A SolidFEM XML scene: mesh, Dirichlet nodes, material, simulation and solver settings."""
    root = ET.parse(path).getroot()
    if root.tag != "solidfem":
        raise ValueError(f"{path}: root element is <{root.tag}>, expected <solidfem>")
    base = os.path.dirname(os.path.abspath(path))
    model = root.find("model")
    if model is None or "path" not in model.attrib:
        raise ValueError(f"{path}: no <model path=...>")
    scale = float(model.get("scale", "1"))
    mpath = os.path.join(base, model.get("path"))
    kind = model.get("type", "tet1")
    if kind == "tet1":
        nodes, tets = load_tet1(mpath, scale)
    elif kind == "vol":
        nodes, tets = load_vol(mpath, scale)
    else:
        raise ValueError(f"{path}: model type {kind!r} is not supported (tet1, vol)")
    swap = model.get("swap")
    if swap in ("xy", "xz", "yz"):
        a, b = {"xy": (0, 1), "xz": (0, 2), "yz": (1, 2)}[swap]
        nodes[:, [a, b]] = nodes[:, [b, a]]
    d = model.find("dirichlet")
    fixed = np.asarray(_ints(d.text if d is not None else ""), dtype=np.int32)
    cfg: dict = {}
    mat = root.find("material")
    if mat is not None:
        name = mat.get("name")
        if name in MATERIAL_IDS:
            cfg["material"] = MATERIAL_IDS[name]
        for key in ("young", "poisson", "density"):
            if mat.get(key) is not None:
                cfg[key] = float(mat.get(key))
    scene = Scene(nodes=nodes, tets=tets, fixed=fixed, config=cfg,
                  visual=os.path.join(base, model.get("visual")) if model.get("visual") else None)
    sim = root.find("simulation")
    if sim is not None:
        t = sim.get("type")
        scene.sim_type = {"quasi-static": SIM_QUASI_STATIC, "explicit": SIM_EXPLICIT}.get(t, SIM_STATIC)
        if sim.get("steps"):
            scene.steps = int(sim.get("steps"))
        if sim.get("gravity"):
            cfg["gravity"] = float(sim.get("gravity"))
        pr = sim.find("pressure")
        if pr is not None and pr.get("p"):
            scene.pressure = float(pr.get("p"))
    sol = root.find("solver")
    if sol is not None:
        if sol.get("iterations"):
            cfg["maxiter"] = int(sol.get("iterations"))
        if sol.get("tolerance"):
            cfg["tol"] = float(sol.get("tolerance"))
        if sol.get("method"):
            cfg["solver"] = sol.get("method")
    return scene


def export_vtk(path: str, positions, tets, displacement=None, stress=None) -> None:
    """Legacy ASCII VTK unstructured grid: deformed positions, tetra cells, optional point
    displacements (N, 3) and cell stress tensors (E, 3, 3)."""
    x = np.asarray(positions, dtype=np.float64)
    t = np.asarray(tets, dtype=np.int64)
    with open(path, "w") as f:
        f.write("# vtk DataFile Version 2.0\nUnstructured Grid\nASCII\nDATASET UNSTRUCTURED_GRID\n")
        f.write(f"POINTS {len(x)} double\n")
        np.savetxt(f, x, fmt="%.6f")
        f.write(f"\nCELLS {len(t)} {5 * len(t)}\n")
        np.savetxt(f, np.column_stack([np.full(len(t), 4), t]), fmt="%d")
        f.write(f"\nCELL_TYPES {len(t)}\n")
        np.savetxt(f, np.full(len(t), 10), fmt="%d")
        if displacement is not None:
            f.write(f"\nPOINT_DATA {len(x)}\nVECTORS displacement float\n")
            np.savetxt(f, np.asarray(displacement, dtype=np.float64).reshape(-1, 3), fmt="%.6f")
        if stress is not None:
            s = np.asarray(stress, dtype=np.float64).reshape(-1, 3, 3)
            f.write(f"\nCELL_DATA {len(s)}\nTENSORS stress float\n")
            for m in s:
                np.savetxt(f, m, fmt="%.9g")
                f.write("\n")


def export_physics_vtk(path: str, phys) -> None:
    """``ExportToVTKHeatMap`` for a ``FemPhysicsMatrixFree``: current positions, displacement
    from the rest configuration, per-element PK1 stress (caller's node and element order)."""
    x = phys.get_positions()
    export_vtk(path, x, phys.tets_original, x - phys.rest_positions, phys.element_stress())
