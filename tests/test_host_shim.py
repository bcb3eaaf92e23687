"""The C drop-in for the reference's missing grad4_1shot (header.h:283)
compiles against the reference's own header and links with the reference's
own sources (fwi_2d.c, grad_prec.c, triangle_smooth.c, min_max.c, alloc.c,
read_write.c) and libfwigpu.so.  Runs where the reference checkout exists."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("FWI_REFERENCE_DIR", "/root/reference")
SHIM = os.path.join(ROOT, "oracle", "ref_shim")

pytestmark = pytest.mark.skipif(not os.path.isfile(os.path.join(REF, "header.h")),
                                reason="reference checkout not present")


def test_shim_links_with_reference_sources(engine_lib, tmp_path):
    pkg = os.path.join(ROOT, "fwi2dacoustic-mpi-lbfgs_gb300")
    # triangle_smooth.c includes a header the reference does not ship (triangle_smooth.c:3)
    (tmp_path / "triangle_smooth.h").write_text("#include <stdlib.h>\n")
    exe = tmp_path / "shim_link"
    srcs = [os.path.join(pkg, "host", "grad4_1shot_gpu.c"), os.path.join(ROOT, "tests", "c", "shim_link_main.c")]
    srcs += [os.path.join(REF, f) for f in ("fwi_2d.c", "grad_prec.c", "triangle_smooth.c", "min_max.c",
                                            "alloc.c", "read_write.c")]
    cmd = ["gcc", "-std=gnu99", "-O1", "-fopenmp", "-w", f"-I{tmp_path}", f"-I{SHIM}", f"-I{REF}",
           f"-I{os.path.join(ROOT, 'include')}", "-include", os.path.join(SHIM, "ref_config.h"), "-o", str(exe)]
    cmd += srcs + [f"-L{pkg}", "-lfwigpu", f"-Wl,-rpath,{pkg}", "-lm"]
    subprocess.run(cmd, check=True)
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if not has_gpu:
        r = subprocess.run([str(exe)], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "no usable sm_103 device" in r.stderr
