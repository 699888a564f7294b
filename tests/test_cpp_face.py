"""The header-only C++ face (include/m3d_gb300_forward_solver.hpp) compiles
against the C ABI, links against the in-tree library, and turns a failing
C call into m3d::SolverError carrying the M3D_ERR_* code."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

PROGRAM = r"""
#include <cstdio>
#include "m3d_gb300_forward_solver.hpp"
int main() {
    try {
        m3d::GpuForwardSolverFV s(0);
        std::printf("DEVICE\n");
    } catch (const m3d::SolverError& e) {
        std::printf("ERROR %d %s\n", e.code, e.what());
    }
    return 0;
}
"""


def test_cpp_face_compiles_links_and_reports_errors(lib, tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    from maple3dmt_gb300 import _loader
    src = tmp_path / "face.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "face"
    libdir = os.path.dirname(_loader.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
                    "-L", libdir, "-lm3d_gb300", "-Wl,-rpath," + libdir, "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.strip()
    if out == "DEVICE":
        pytest.skip("a CUDA device is present; the error path is covered on CPU-only hosts")
    assert out.startswith("ERROR 5 "), out   # M3D_ERR_NO_DEVICE
