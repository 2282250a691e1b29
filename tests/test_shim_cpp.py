"""The C++ drop-in (include/sfem_femphysics.hpp) compiled against the reference's own headers:
the reference's solver templates SolveConjugateGradientMF<real, Vector3R, FemPhysicsMatrixFreeGpu>
(Math/IterativeSolvers.h:115-195) and NonlinearConjugateGradientMinimizer<FemPhysicsMatrixFreeGpu,
std::vector<Vector3R>> (Include/NonlinearCG.h:38-114) are instantiated on it and linked with
libsfem_gb300.so.  Where no GPU is present the program runs and the constructor reports
SFEM_ERR_NO_DEVICE through the shim's exception; with a GPU it runs both solvers.

Needs the reference tree (development container only; SFEM_REF_TREE overrides its location)."""
import os
import shutil
import subprocess

import pytest

from oracle.oracle import REF_TREE

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <stdio.h>
#include <math.h>
#include "Engine/Utils.h"
#include "FemDataStructures.h"
#include "IterativeSolvers.h"
#include "NonlinearCG.h"
#include "sfem_femphysics.hpp"

using namespace FEM_SYSTEM;

int main() {
  // one hexahedron of a unit box split into 6 tets, the x = 0 face clamped
  std::vector<Node> nodes(8);
  for (int k = 0; k < 8; k++) {
    nodes[k].pos = Vector3R(k & 1, (k >> 1) & 1, (k >> 2) & 1);
    nodes[k].pos0 = nodes[k].pos;
    if ((k & 1) == 0) nodes[k].invMass = 0;
  }
  const int t6[6][4] = {{0, 1, 3, 7}, {0, 1, 7, 5}, {0, 5, 7, 4}, {0, 3, 2, 7}, {0, 2, 6, 7}, {0, 6, 4, 7}};
  std::vector<Tet> tets(6);
  for (int e = 0; e < 6; e++)
    for (int j = 0; j < 4; j++) tets[e].idx[j] = (uint32)t6[e][j];
  FemConfig cfg;
  cfg.mYoungsModulus = 1e5;
  cfg.mPoissonRatio = 0.45;
  cfg.mDensity = 1070;
  cfg.mGravity = -9.81;
  cfg.mZUpAxis = true;
  cfg.mMaterial = MMT_NEO_HOOKEAN;
  try {
    FemPhysicsMatrixFreeGpu phys(tets, nodes, cfg);
    const uint32 nf = phys.GetNumFreeNodes();
    std::vector<Vector3R> b(nf), x(nf);
    phys.ComputeGradients(b);
    const int its = SolveConjugateGradientMF<real, Vector3R, FemPhysicsMatrixFreeGpu>(phys, b, x, 100, 1e-6f);
    std::vector<Vector3R> kx(nf);
    phys.MatrixVectorMultiply(x, kx);
    const double res = sqrt(phys.DotProduct(kx - b, kx - b) / phys.DotProduct(b, b));
    std::vector<Vector3R> free_pos(nf);
    NonlinearConjugateGradientMinimizer<FemPhysicsMatrixFreeGpu, std::vector<Vector3R>> nlcg;
    nlcg.mOuterIterations = 5;
    std::vector<double> fp(3 * nf);
    sfem_get_free_positions(phys.handle(), fp.data());
    for (uint32 i = 0; i < nf; i++) free_pos[i] = Vector3R(fp[3 * i], fp[3 * i + 1], fp[3 * i + 2]);
    nlcg.Solve(phys, nf, free_pos);
    printf("GPU cg_iters=%d rel_res=%.3e inverted=%d\n", its, res, (int)phys.CheckForInversion());
    return res < 1e-5 ? 0 : 3;
  } catch (const sfem_gpu_error& e) {
    printf("sfem_gpu_error %d: %s\n", e.code(), e.what());
    return e.code() == SFEM_ERR_NO_DEVICE ? 0 : 2;
  }
}
"""


@pytest.mark.skipif(not os.path.isdir(REF_TREE), reason="the reference tree is present in the development container only")
@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_cpp_shim_runs_reference_solver_templates(tmp_path):
    from solidfem_gb300 import build

    lib = build.build()
    shim = tmp_path / "shim" / "Math"
    shim.mkdir(parents=True)
    # FemDataStructures.h includes Math/Vector3.h and Math/Matrix3.h with capital letters
    os.symlink(os.path.join(REF_TREE, "Math", "vector3.h"), shim / "Vector3.h")
    os.symlink(os.path.join(REF_TREE, "Math", "matrix3.h"), shim / "Matrix3.h")
    src = tmp_path / "shim_main.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "shim_main"
    libdir = os.path.dirname(lib)
    cmd = ["g++", "-std=c++17", "-O1", "-DLINUX", "-DNDEBUG", "-w", "-include", "memory",
           "-I", str(tmp_path / "shim"), "-I", os.path.join(ROOT, "include"), "-I", REF_TREE,
           "-I", os.path.join(REF_TREE, "Include"), "-I", os.path.join(REF_TREE, "Math"),
           str(src), "-o", str(exe), "-L", libdir, "-lsfem_gb300", f"-Wl,-rpath,{libdir}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    print(out.stdout)
    assert out.returncode == 0, out.stdout + out.stderr
    import torch

    if not torch.cuda.is_available():
        assert "sfem_gpu_error -7" in out.stdout
    else:
        assert "GPU cg_iters=" in out.stdout
