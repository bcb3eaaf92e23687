"""CPU checks of the C ABI library: it loads, exports every function that
include/*.h declares, and its host-only helpers agree with the oracle (and
hence with the reference's cpml_coe and fwi_init arithmetic)."""
import ctypes as C
import glob
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        for m in re.finditer(r"\b(fwi_[A-Za-z0-9_]+)\s*\(", txt):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol(engine_lib):
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(engine_lib, n)]
    assert not missing, missing


def test_cpml_profile_matches_reference_arithmetic(engine_lib, oracles):
    import fwigpu
    _, o32, _ = oracles
    for npml, d, dt, f, v, r in [(20, 10.0, 0.001, 15.0, 6000.0, 0.001), (12, 12.5, 0.0008, 10.0, 4500.0, 1e-4),
                                 (7, 5.0, 0.0005, 25.0, 6000.0, 0.01)]:
        a, b = fwigpu.cpml_profile(npml, d, dt, f, v, r)
        a0, b0 = o32.cpml_coe(npml, d, dt, f, v, r)
        assert np.array_equal(a, a0) and np.array_equal(b, b0)


def test_fd_coefficients_and_cells(engine_lib, oracles):
    import fwigpu
    _, o32, _ = oracles
    for dx, dz in [(10.0, 10.0), (12.5, 10.0), (5.0, 7.5)]:
        assert np.array_equal(fwigpu.fd_coefficients(dx, dz), o32.fd_coeffs(dx, dz))
    # fwi_2d.c:363-364: ix = round(x/dx), iz = round(z/dz - 0.5)
    assert fwigpu.cell_of(0.0, 2.0, 10.0, 10.0) == (0, 0)
    assert fwigpu.cell_of(104.9, 10.0, 10.0, 10.0) == (10, 1)
    assert fwigpu.cell_of(105.0, 25.0, 10.0, 10.0) == (11, 2)


def test_check_config_rejects_bad_input(engine_lib):
    import fwigpu
    good = fwigpu.make_config(64, 48, 10.0, 10.0, 0.001, 100)
    assert fwigpu.check_config(good) == 0
    for field, val in [("nx", 4), ("npml", 0), ("dt", 0.0), ("jump", 0), ("free_surface", 2),
                       ("pml_coef_r", 1.5), ("nt_max", 0), ("store", 3), ("store", -1), ("snapshots", -2),
                       ("snap_precision", 3), ("hbm_budget_mb", -1), ("fd_order", 6), ("fd_order", 2)]:
        cfg = fwigpu.make_config(64, 48, 10.0, 10.0, 0.001, 100)
        setattr(cfg, field, val)
        assert fwigpu.check_config(cfg) == -1, field
    cfg = fwigpu.make_config(64, 48, 10.0, 10.0, 0.001, 100)
    cfg.reserved[0] = 1
    assert fwigpu.check_config(cfg) == -1
    for store, prec, order in [(2, 0, 4), (2, 1, 8), (2, 2, 0), (1, 0, 8), (0, 2, 4)]:
        assert fwigpu.check_config(fwigpu.make_config(64, 48, 10.0, 10.0, 0.001, 100, store=store,
                                                      snap_precision=prec, fd_order=order)) == 0


def test_create_without_device_reports_nodevice(engine_lib):
    import fwigpu
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a device is present")
    with pytest.raises(fwigpu.FwiError) as e:
        fwigpu.Engine(fwigpu.make_config(64, 48, 10.0, 10.0, 0.001, 100))
    assert e.value.status == -8


def test_status_strings(engine_lib):
    engine_lib.fwi_status_string.restype = C.c_char_p
    for s in range(0, -9, -1):
        assert engine_lib.fwi_status_string(s)
    assert engine_lib.fwi_version() >= 1


def test_ctypes_structs_match_the_header(tmp_path):
    """The ctypes mirrors in fwigpu.py have the header's field names, offsets
    and sizes: a C program built against include/fwi_gb300.h prints them.  A
    field renamed in one place fails to compile; one moved or resized fails
    the comparison."""
    import shutil
    import subprocess
    import fwigpu
    cc = shutil.which(os.environ.get("CC", "gcc"))
    if not cc:
        pytest.skip("no C compiler")
    structs = {"fwi_config": fwigpu.FwiConfig, "fwi_shot": fwigpu.FwiShot, "fwi_stats": fwigpu.FwiStats,
               "fwi_misfit": fwigpu.FwiMisfit, "fwi_tuning": fwigpu.FwiTuning,
               "fwi_lbfgs_param": fwigpu.FwiLbfgsParam}
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "fwi_gb300.h"', "int main(void) {"]
    want = []
    for cname, py in structs.items():
        lines.append(f'printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        want.append(f"{cname} sizeof {C.sizeof(py)}")
        for name, _ in py._fields_:
            lines.append(f'printf("{cname} {name} %zu\\n", offsetof({cname}, {name}));')
            want.append(f"{cname} {name} {getattr(py, name).offset}")
    lines += ["return 0;", "}"]
    src, exe = tmp_path / "layout.c", tmp_path / "layout"
    src.write_text("\n".join(lines) + "\n")
    r = subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    assert [g for g in got if g] == want
