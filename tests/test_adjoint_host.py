"""The differentiable form's hand-derived reverse passes (sgx_adjoint.cuh) on
the host, no GPU: against central differences of the forward functions, and
the separated right-hand side against the reference grouping of the oracle
(kerr_hamilton.h:97-155 restated in oracle/geodesic_oracle.hpp).  The header
is host-and-device code; tests/adjoint_fd_check.cpp exercises it in double."""

from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_reverse_passes_match_central_differences(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    exe = tmp_path / "adjoint_fd_check"
    subprocess.run([cxx, "-std=c++20", "-O2", "-fno-fast-math", "-o", str(exe),
                    str(ROOT / "tests" / "adjoint_fd_check.cpp"),
                    "-I", str(ROOT / "singularity_gb300" / "csrc"), "-I", str(ROOT / "oracle"),
                    "-I", str(ROOT / "include")], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    w_rhs, w_state, w_const, w_same = (float(x) for x in out)
    print(f"rhs_vjp7 {w_rhs:.1e}, step_vjp state {w_state:.1e} constants {w_const:.1e}, "
          f"separated vs reference grouping {w_same:.1e}")
    # central differences with step 1e-6 carry ~1e-9 truncation and rounding;
    # near the poles (damping active) the right-hand side's derivatives reach
    # 1e4 and the differences lose digits to ~1e-5
    assert w_rhs <= 1e-5 and w_state <= 1e-6 and w_const <= 1e-6
    assert w_same <= 1e-10
