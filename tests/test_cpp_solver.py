"""The C++ mirror of the reference's solver interface (include/gwgb_solver.hpp)
compiles against gwgb.h, links against libgwgb.so, and turns a rejected call
into std::runtime_error as the reference does -- without touching a GPU (the
parameters are rejected before any CUDA call)."""
import os
import shutil
import subprocess

import pytest

from mbsymmetry_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r'''
#include <cstdio>
#include <cstring>
#include "gwgb_solver.hpp"

int main() {
  std::printf("%s\n", gwgb_version());
  gwgb_params p{};
  p.ns = 3;  // rejected: ns must be 1 or 2
  p.nts = 62; p.nw = 60; p.nw_b = 59; p.beta = 50.0;
  gwgb_layout L{};
  std::vector<gwgb::gb300_gw_solver::dcomplex> G(10), S(10);
  try {
    gwgb::gb300_gw_solver s(p, L, G.data(), S.data(), nullptr, 0, 1, 1);
    std::printf("no exception\n");
    return 1;
  } catch (const std::runtime_error &e) {
    std::printf("runtime_error: %s\n", e.what());
    return std::strstr(e.what(), "ns must be 1 or 2") ? 0 : 2;
  }
}
'''


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_cpp_solver_compiles_links_and_throws(tmp_path):
    _abi.load()  # the library is built
    src = tmp_path / "use_solver.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "use_solver"
    libdir = os.path.join(ROOT, "mbsymmetry_gb300", "csrc")
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
                    "-L", libdir, "-lgwgb", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "sm_103a" in out.stdout and "runtime_error" in out.stdout
