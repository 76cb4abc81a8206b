"""The C-ABI library builds, loads and exports every symbol include/gba.h
declares; pure host helpers agree with the oracle's sizes.  No GPU needed."""
import ctypes as C
import os
import re

import pytest

from hs_sfm_gb300 import abi, synthetic
from hs_sfm_gb300 import build as gba_build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "gba.h")).read()
    return sorted(set(re.findall(r"^GBA_API [^(]*?\b(gba_\w+)\(", text, flags=re.M)))


@pytest.fixture(scope="module")
def libgba():
    path = gba_build.build()
    return C.CDLL(path)


def test_every_declared_symbol_is_exported(libgba):
    syms = declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(libgba, s)]
    assert not missing, missing


def test_host_helpers(libgba):
    from hs_sfm_gb300 import gba
    L = gba.lib()
    s = synthetic.config(0)
    cp = abi.CProblem(s)
    assert L.gba_x_size(cp.ref) == abi.x_size(s) == 3 * 1000 + 6 * 10
    assert L.gba_y_size(cp.ref) == abi.y_size(s) == 2 * 5000
    full = synthetic.full_model_scene(seed=3)
    cpf = abi.CProblem(full)
    assert L.gba_x_size(cpf.ref) == abi.x_size(full)
    assert L.gba_y_size(cpf.ref) == abi.y_size(full)
    assert L.gba_params_per_camera(7) == 10
    assert L.gba_status_string(-6) == b"reduced system not positive definite"
    opt = abi.Options()
    L.gba_default_options(C.byref(opt))
    assert (opt.max_iterations, opt.tau, opt.eps1, opt.eps2) == (50, 1e-3, 1e-8, 1e-8)


def _c_layout(tmp_path):
    """sizeof / offsetof of the ABI structs as the C compiler lays them out."""
    src = tmp_path / "layout.c"
    fields = {
        "gba_problem": [f for f, _ in abi.Problem._fields_],
        "gba_options": [f for f, _ in abi.Options._fields_],
        "gba_report": [f for f, _ in abi.Report._fields_],
        "gba_triangulation": [f for f, _ in abi.Triangulation._fields_],
        "gba_tuning": [f for f, _ in abi.Tuning._fields_],
        "gba_plan_structure_info": [f for f, _ in abi.PlanStructure._fields_],
    }
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{ROOT}/include/gba.h"',
             'int main(void) {']
    for st, fs in fields.items():
        lines.append(f'printf("{st} %zu\\n", sizeof({st}));')
        for f in fs:
            lines.append(f'printf("{st}.{f} %zu\\n", offsetof({st}, {f}));')
    lines.append('return 0; }')
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    import subprocess
    subprocess.run(["gcc", "-o", str(exe), str(src)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return dict(line.split() for line in out.strip().splitlines())


def test_struct_layouts_match_header(tmp_path):
    lay = _c_layout(tmp_path)
    for name, cls in (("gba_problem", abi.Problem), ("gba_options", abi.Options),
                      ("gba_report", abi.Report), ("gba_triangulation", abi.Triangulation),
                      ("gba_tuning", abi.Tuning),
                      ("gba_plan_structure_info", abi.PlanStructure)):
        assert int(lay[name]) == C.sizeof(cls), name
        for f, _ in cls._fields_:
            assert int(lay[f"{name}.{f}"]) == getattr(cls, f).offset, (name, f)
