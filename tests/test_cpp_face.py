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


SOLVE_PROGRAM = r"""
#include <cstdio>
#include <vector>
#include "m3d_gb300_forward_solver.hpp"
// input (doubles unless noted): n_cells (int), domain[6], min_level, max_level (int), level[n] (int),
// cx[n], cy[n], cz[n], cell_type[n] (int), sigma[n], n_st (int), xyz[n_st][3], freq, sigma_bg
template <class T> std::vector<T> rd(FILE* f, size_t n) { std::vector<T> v(n); fread(v.data(), sizeof(T), n, f); return v; }
int main(int argc, char** argv) {
    FILE* f = std::fopen(argv[1], "rb");
    int n, lmin, lmax, ns;
    double dom[6], freq, sbg;
    fread(&n, sizeof(int), 1, f); fread(dom, sizeof(double), 6, f);
    fread(&lmin, sizeof(int), 1, f); fread(&lmax, sizeof(int), 1, f);
    auto level = rd<int>(f, n); auto cx = rd<double>(f, n); auto cy = rd<double>(f, n); auto cz = rd<double>(f, n);
    auto ct = rd<int>(f, n); auto sigma = rd<double>(f, n);
    fread(&ns, sizeof(int), 1, f);
    auto xyz = rd<double>(f, 3 * (size_t)ns);
    fread(&freq, sizeof(double), 1, f); fread(&sbg, sizeof(double), 1, f);
    std::fclose(f);
    try {
        m3d::GpuForwardSolverFV s(0);
        m3d_leaves lv{};
        for (int i = 0; i < 6; ++i) lv.domain[i] = dom[i];
        lv.min_level = lmin; lv.max_level = lmax; lv.n_cells = n;
        lv.level = level.data(); lv.cx = cx.data(); lv.cy = cy.data(); lv.cz = cz.data(); lv.cell_type = ct.data();
        m3d_params p; m3d_params_default(&p);
        p.bicgstab_tol = 1e-10; p.bicgstab_maxiter = 5000; p.sigma_bg = sbg; p.precision = 1;
        s.setup(lv, p);
        s.set_sigma(sigma);
        std::vector<std::array<double, 3>> st(ns);
        for (int i = 0; i < ns; ++i) st[i] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
        s.set_stations(st);
        auto Z = s.compute_single_frequency(freq);
        for (auto& z : Z)
            for (int k = 0; k < 4; ++k) std::printf("%.17g %.17g\n", z[k].real(), z[k].imag());
        // one residual source per station (unit weight on Zxy at that station): per-station gradients
        std::vector<std::vector<std::array<m3d::Complex, 4>>> wr(ns, std::vector<std::array<m3d::Complex, 4>>(ns));
        for (int j = 0; j < ns; ++j) wr[j][j][1] = m3d::Complex(1.0, -0.5);
        auto g = s.station_gradients(wr);
        for (int j = 0; j < ns; ++j) {
            double sum = 0.0;
            for (double v : g[j]) sum += v;
            std::printf("G %d %.17g\n", j, sum);
        }
    } catch (const m3d::SolverError& e) {
        std::printf("ERROR %d %s\n", e.code, e.what());
        return 1;
    }
    return 0;
}
"""


@pytest.mark.gpu
def test_cpp_face_solves_on_device(lib, tmp_path):
    """The C++ face a maintainer drops under InversionFV: set-up from a leaf
    list, conductivity, stations and one forward solve on the GPU give the
    reference's impedances (tests/golden/small_block.npz) to 1e-6, and its
    per-station gradients equal the Python face's."""
    import numpy as np
    from conftest import load_golden, rel
    from maple3dmt_gb300 import _loader
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    g = load_golden("small_block")
    src = tmp_path / "solve.cpp"
    src.write_text(SOLVE_PROGRAM)
    exe = tmp_path / "solve"
    libdir = os.path.dirname(_loader.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), str(src), "-L", libdir,
                    "-lm3d_gb300", "-Wl,-rpath," + libdir, "-o", str(exe)], check=True)
    n = g["level"].shape[0]
    st = np.asarray(g["stations"], np.float64).reshape(-1, 3)
    freq = float(g["freqs"][0])
    with open(tmp_path / "in.bin", "wb") as f:
        f.write(np.int32(n).tobytes()); f.write(np.asarray(g["domain"], np.float64).tobytes())
        f.write(np.int32(g["min_level"]).tobytes()); f.write(np.int32(g["max_level"]).tobytes())
        f.write(np.asarray(g["level"], np.int32).tobytes())
        for k in ("cx", "cy", "cz"):
            f.write(np.asarray(g[k], np.float64).tobytes())
        f.write(np.asarray(g["cell_type"], np.int32).tobytes())
        f.write(np.asarray(g["sigma"], np.float64).tobytes())
        f.write(np.int32(st.shape[0]).tobytes()); f.write(st.tobytes())
        f.write(np.float64(freq).tobytes()); f.write(np.float64(g["sigma_bg"]).tobytes())
    out = subprocess.run([str(exe), str(tmp_path / "in.bin")], check=True, capture_output=True, text=True).stdout
    lines = out.strip().splitlines()
    v = np.array([[float(a) for a in line.split()] for line in lines if not line.startswith("G ")])
    Z = (v[:, 0] + 1j * v[:, 1]).reshape(-1, 4)
    ns, nf = st.shape[0], g["freqs"].shape[0]
    assert rel(Z, g["ref_Z"].reshape(nf, ns, 4)[0]) < 1e-6
    # per-station gradients through the C++ face equal the Python face's on the same handle settings
    gs = np.array([float(line.split()[2]) for line in lines if line.startswith("G ")])
    from maple3dmt_gb300.solver import ForwardSolverFV
    from conftest import leaves_from_golden
    py = ForwardSolverFV(0)
    py.setup(leaves_from_golden(g), bicgstab_tol=1e-10, bicgstab_maxiter=5000, sigma_bg=float(g["sigma_bg"]),
             precision=1)
    py.set_sigma(g["sigma"])
    py.set_stations(g["stations"])
    py.compute_single_frequency(freq)
    wr = np.zeros((ns, ns, 4), np.complex128)
    for j in range(ns):
        wr[j, j, 1] = 1.0 - 0.5j
    gp = py.station_gradients(wr).sum(axis=1)
    assert gs.shape == (ns,) and np.abs(gp).max() > 0
    assert rel(gs, gp) < 1e-9
