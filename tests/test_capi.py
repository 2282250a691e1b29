"""The C-ABI library builds for sm_103a, loads, and exports every entry point that
include/sfem.h declares (no compute calls here)."""
import ctypes
import os
import re

from tests.conftest import ROOT


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "sfem.h")).read()
    return sorted(set(re.findall(r"\b(sfem_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from solidfem_gb300 import _native

    lib = _native.load()
    syms = declared_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    # the Python binding wraps exactly the declared ABI
    assert set(_native.SIGNATURES) == set(syms)


def test_no_device_is_reported_not_faked():
    """Without a GPU the library reports SFEM_ERR_NO_DEVICE instead of computing on the CPU."""
    import numpy as np
    import pytest
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from solidfem_gb300 import SfemError, FemPhysicsMatrixFree
    from solidfem_gb300.mesh import box_lattice

    m = box_lattice(2, 1, 1)
    with pytest.raises(SfemError) as ei:
        FemPhysicsMatrixFree(m.tets, m.nodes, np.array([0]))
    assert ei.value.code == -7


def test_invalid_arguments_are_rejected_before_any_device_work():
    import numpy as np
    import pytest

    from solidfem_gb300 import FemPhysicsMatrixFree, SfemError
    from solidfem_gb300.mesh import box_lattice

    m = box_lattice(2, 1, 1)
    bad = m.tets.copy()
    bad[0, 0] = m.n_nodes + 5
    with pytest.raises(SfemError) as ei:
        FemPhysicsMatrixFree(bad, m.nodes, np.array([0]))
    assert ei.value.code == -1 and "out of range" in str(ei.value)
    with pytest.raises(SfemError) as ei:
        FemPhysicsMatrixFree(m.tets, m.nodes, np.array([0]), poisson=0.5)
    assert ei.value.code == -1
