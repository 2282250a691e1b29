"""The two-term FP32 arithmetic of the FP32 handles' neo-Hookean residual (solidfem_gb300/csrc/sfem_df32.cuh),
compiled as plain C++ and checked against quad precision (tests/df32_check.cpp): the exact FP64 split, log1p,
and the element forces and energy of ElasticEnergy.cpp:170-186 / :80-86 over strains from 1e-6 to 0.3 at
nu = 0.49.  The GPU kernel (k_element_nh_df) runs the same header; its residuals are compared with the FP64
pass's in tests/test_gpu_c3.py."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def measured(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    exe = str(tmp_path_factory.mktemp("df32") / "df32_check")
    cmd = [gxx, "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "solidfem_gb300", "csrc"),
           os.path.join(ROOT, "tests", "df32_check.cpp"), "-o", exe]
    if os.uname().machine == "x86_64":
        cmd.append("-lquadmath")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("df32_check did not compile here: " + r.stderr[-300:])
    out = subprocess.run([exe], capture_output=True, text=True, check=True, timeout=120).stdout
    return {k: float(v) for k, v in (line.split() for line in out.splitlines())}


def test_split_is_exact_to_48_bits(measured):
    assert measured["split_rel"] <= 2.0 ** -47


def test_log1p(measured):
    assert measured["log1p_rel"] <= 1e-13


def test_forces_fp64_accurate(measured):
    # relative to each element's largest force; the FP64 formula loses the digits of |H| at small strains
    assert measured["force_rel_two_term"] <= 1e-12
    assert measured["force_rel_two_term"] <= measured["force_rel_fp64"]


def test_energy(measured):
    # the H form keeps psi = O(|H|^2) relative; the FP64 form's I1 - 3 does not
    assert measured["energy_rel_two_term"] <= 1e-7
    assert measured["energy_rel_two_term"] <= measured["energy_rel_fp64"]


def test_node_sums(measured):
    # the gather's accurate two-term addition over 24 cancelling contributions: about 3u^2 (u = 2^-24) per
    # addition relative to the partial sums, so ~25x FP64 recursive summation's error, far below the
    # element forces' own
    assert measured["node_sum_rel_two_term"] <= 1e-13


def test_inverted_element(measured):
    assert measured["inverted_flag"] == 1
    assert measured["forces_nan"] == 1
    assert measured["valid_not_flagged"] == 1
