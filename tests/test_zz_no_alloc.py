"""The allocation-free dot product (sfem_dot_noalloc_dev) against the library's
regular dot product (sfem_dot), through the C ABI.

That entry point exists for callers that cannot call cudaMalloc where they need a
reduction -- inside a CUDA stream capture, in loops that forbid allocation after
start-up, or in hosts that plan all device memory themselves -- so its scratch is a
fixed static device array shared by all calls.  Two calls in a row check that the
array's leftover contents from one call do not leak into the next.  This file is
collected last so that a stop-at-first-failure run has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the relative tolerance of the FP64 parity tests


def test_noalloc_dot_matches_sfem_dot_on_two_calls_in_a_row():
    import torch

    from solidfem_gb300 import FemPhysicsMatrixFree
    from solidfem_gb300 import _native as nat
    from solidfem_gb300.mesh import box_lattice

    m = box_lattice(64, 16, 16)
    p = FemPhysicsMatrixFree(m.tets, m.nodes, m.face_nodes(0, 0), young=1e5, poisson=0.45)
    lib = nat.load()
    n = 3 * p.n_free
    rng = np.random.default_rng(11)
    stream = torch.cuda.current_stream()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    for call in range(2):
        a = rng.normal(size=n)
        b = rng.normal(size=n) * (10.0 ** call)
        expected = p.DotProduct(a, b)  # the existing entry point (sfem_dot)
        ad = torch.from_numpy(a).cuda()
        bd = torch.from_numpy(b).cuda()
        out.fill_(float("nan"))
        rc = lib.sfem_dot_noalloc_dev(C.c_void_p(ad.data_ptr()), C.c_void_p(bd.data_ptr()), n,
                                      C.c_void_p(out.data_ptr()), C.c_void_p(stream.cuda_stream))
        assert rc == 0, lib.sfem_last_error()
        stream.synchronize()
        got = out.item()
        scale = float(np.abs(a) @ np.abs(b))
        assert abs(got - expected) <= TOL * scale, (call, got, expected)
        # and against the FP64 dot product on the host
        assert abs(got - float(a @ b)) <= TOL * scale, (call, got, float(a @ b))


def test_noalloc_dot_rejects_sizes_beyond_its_maximum():
    import torch

    from solidfem_gb300 import _native as nat

    lib = nat.load()
    buf = torch.zeros(4, dtype=torch.float64, device="cuda")
    ptr = C.c_void_p(buf.data_ptr())
    rc = lib.sfem_dot_noalloc_dev(ptr, ptr, 134217728 + 1, ptr, C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == nat.SFEM_ERR_INVALID
    assert b"maximum" in lib.sfem_last_error()
