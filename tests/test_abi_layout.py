"""The ctypes mirrors of the C-ABI structs (maple3dmt_gb300/_abi_solver.py)
match include/m3d_gb300.h field by field, and the parameter defaults are the
documented ones.  CPU only: a probe compiled with gcc prints sizeof and
offsetof of every field."""
import ctypes as C
import os
import subprocess

import pytest

from conftest import ROOT

STRUCTS = ("m3d_params", "m3d_stats", "m3d_kernel_times", "m3d_reg_params", "m3d_tune_entry")


def _probe(tmp_path):
    from maple3dmt_gb300._abi_solver import KernelTimes, Params, RegParams, Stats, TuneEntry
    mirrors = {"m3d_params": Params, "m3d_stats": Stats, "m3d_kernel_times": KernelTimes, "m3d_reg_params": RegParams,
               "m3d_tune_entry": TuneEntry}
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "m3d_gb300.h"', "int main(void) {"]
    for name in STRUCTS:
        lines.append(f'    printf("{name} sizeof %zu\\n", sizeof({name}));')
        for field, _ in mirrors[name]._fields_:
            lines.append(f'    printf("{name} {field} %zu\\n", offsetof({name}, {field}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "probe"
    subprocess.check_call(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    out = subprocess.check_output([str(exe)], text=True)
    got = {}
    for line in out.splitlines():
        s, f, v = line.split()
        got[(s, f)] = int(v)
    return mirrors, got


def test_struct_mirrors_match_header(tmp_path):
    mirrors, got = _probe(tmp_path)
    for name in STRUCTS:
        m = mirrors[name]
        assert C.sizeof(m) == got[(name, "sizeof")], name
        for field, _ in m._fields_:
            assert getattr(m, field).offset == got[(name, field)], (name, field)


def test_param_defaults(lib):
    from maple3dmt_gb300.solver import default_params
    p = default_params()
    assert p.bicgstab_tol == pytest.approx(1e-7)
    assert p.div_correction == 1 and p.divcorr_iter_per_dc == 500
    assert p.row_kernels == 1 and p.divcorr_precond == 1 and p.ssor_form == 1
    assert p.gradcorr == 1 and p.gradcorr_presmooth == 0 and p.gradcorr_fmax > 1e20
    assert p.divcorr_mixed == 1 and p.gradcorr_overlap == 1
    assert p.inner_tol_floor == pytest.approx(3e-5)
    assert p.residual_replacement == 0
