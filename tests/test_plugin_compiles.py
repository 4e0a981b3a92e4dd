"""The Chroma adapter (chroma_plugin/) compiles: g++ -fsyntax-only against the C ABI header and the
compile-only stand-ins of tests/plugin_mock/ for the QDP++ and Chroma declarations it uses.  This
checks the adapter's calls into include/gbclover.h (struct fields, argument lists, constants) and
its own C++ without a Chroma build; whether it links into Chroma is left to a build with QDP++."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CXX = os.environ.get("CXX") or shutil.which("g++")
FLAGS = ["-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only",
         "-I", os.path.join(ROOT, "tests", "plugin_mock"), "-I", os.path.join(ROOT, "include"), "-I", ROOT]

pytestmark = pytest.mark.skipif(CXX is None, reason="no C++ compiler")


@pytest.mark.parametrize("src", ["syssolver_gb300_clover_params.cc", "syssolver_linop_clover_gb300_w.cc",
                                 "quarkprop4_gb300_w.cc"])
def test_adapter_compiles(src):
    r = subprocess.run([CXX, *FLAGS, os.path.join(ROOT, "chroma_plugin", src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_check_catches_an_abi_mismatch(tmp_path):
    # the same command rejects a call with the wrong argument list
    bad = tmp_path / "bad.cc"
    bad.write_text('#include "gbclover.h"\nint f(gbc_ctx* c, double* p) { return gbc_solve(c, nullptr, 1, p, p); }\n')
    r = subprocess.run([CXX, *FLAGS, str(bad)], capture_output=True, text=True)
    assert r.returncode != 0 and "gbc_solve" in r.stderr


def test_abi_header_is_plain_c99(tmp_path):
    # callers in C (or any FFI that parses C) include the header without a C++ compiler
    cc = os.environ.get("CC") or shutil.which("gcc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "caller.c"
    src.write_text('#include "gbclover.h"\n'
                   'int main(void) {\n'
                   '  gbc_ctx* c = 0; gbc_solve_params p = {0}; gbc_result r; double x = 0;\n'
                   '  return gbc_solve(c, &p, 1, &x, &x, &r) + gbc_get_logdet(c, &x, 0);\n'
                   '}\n')
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-fsyntax-only",
                        "-I", os.path.join(ROOT, "include"), str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
