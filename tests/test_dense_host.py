"""The host-side dense algebra of the FGMRES-DR restart (chroma_gb300/csrc/dense.cc), compiled with
the system C++ compiler and checked on the CPU: complex Schur form (A = Q T Q^H, T triangular, Q
unitary) and its reordering (the k smallest |eigenvalues| first), LU solves with A and A^H, thin QR,
and Morgan's harmonic-Ritz property (every harmonic Ritz residual of an Arnoldi Hessenberg is
parallel to the least-squares residual direction), which the deflated restart's Arnoldi relation
rests on."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_dense_algebra(tmp_path):
    cxx = os.environ.get("CXX") or shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "dense_check")
    subprocess.run([cxx, "-O2", "-std=c++17", os.path.join(ROOT, "tests", "host", "dense_check.cc"),
                    os.path.join(ROOT, "chroma_gb300", "csrc", "dense.cc"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    print(r.stdout)
    assert r.returncode == 0, r.stdout
