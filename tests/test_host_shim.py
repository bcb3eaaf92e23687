"""The C drop-in for the reference's missing grad4_1shot (header.h:283).

host/grad4_1shot_gpu.c compiles against the reference's own header.h and
links with the reference's own sources (fwi_2d.c, grad_prec.c,
triangle_smooth.c, min_max.c, alloc.c, read_write.c) and libfwigpu.so, as
MBotOpt.c would link it.  The sources come from the reference checkout or its
staged copy (oracle/_ref/src); the tests skip where neither exists.

* Without a GPU the shim must report a failed trial (NaN misfit) instead of
  exiting.
* On a GPU, two real plans go through fwi_plans_gradient: plan->grad->body
  must equal the FP64 oracle's gradient after the reference's own
  grad_precond_new5 (relative L2 error <= 1e-4, the gradient bound of the
  parity tests) and msf->val[1] the oracle's misfit (relative 1e-5).
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import ricker

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "fwi2dacoustic-mpi-lbfgs_gb300")
SHIM = os.path.join(ROOT, "oracle", "ref_shim")


def _ref_dir():
    import oracle as O
    O.build()
    return O.reference_sources()


def _link(tmp_path, main_c, exe_name):
    ref = _ref_dir()
    if ref is None:
        pytest.skip("the reference's sources are not present")
    # triangle_smooth.c includes a header the reference does not ship (triangle_smooth.c:3)
    (tmp_path / "triangle_smooth.h").write_text("#include <stdlib.h>\n")
    exe = tmp_path / exe_name
    srcs = [os.path.join(PKG, "host", "grad4_1shot_gpu.c"), os.path.join(ROOT, "tests", "c", main_c)]
    srcs += [os.path.join(ref, f) for f in ("fwi_2d.c", "grad_prec.c", "triangle_smooth.c", "min_max.c",
                                            "alloc.c", "read_write.c")]
    cmd = ["gcc", "-std=gnu99", "-O1", "-fopenmp", "-w", f"-I{tmp_path}", f"-I{SHIM}", f"-I{ref}",
           f"-I{os.path.join(ROOT, 'include')}", "-include", os.path.join(SHIM, "ref_config.h"), "-o", str(exe)]
    cmd += srcs + [f"-L{PKG}", "-lfwigpu", f"-Wl,-rpath,{PKG}", "-lm"]
    subprocess.run(cmd, check=True)
    return exe


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_shim_links_with_reference_sources(engine_lib, tmp_path):
    exe = _link(tmp_path, "shim_link_main.c", "shim_link")
    if not _has_gpu():
        r = subprocess.run([str(exe)], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "no usable sm_103 device" in r.stderr


@pytest.mark.gpu
def test_shim_gradient_on_real_plans(engine_lib, oracles, tmp_path):
    O, _, o64 = oracles
    exe = _link(tmp_path, "shim_gpu_main.c", "shim_gpu")
    nx, nz, nt, jump, npml, dx, dt = 120, 80, 401, 2, 12, 10.0, 0.001
    perc, rectx1, repeat1, rectx2, repeat2, alpha = 0.95, 3, 1, 2, 1, 0.5
    rng = np.random.default_rng(21)
    vel = (np.linspace(1600.0, 2900.0, nz)[:, None] + rng.uniform(-60, 60, (nz, nx))).astype(np.float32)
    vtrue = vel.copy()
    vtrue[20:28, 30:90] += 220.0
    ibtry = np.full(nx, 3, np.int32)
    ibtry[nx // 2:] = 5
    ocfg = O.make_config(nx=nx, nz=nz, npml=npml, nt=nt, dx=dx, dz=dx, dt=dt, free_surface=1, jump=jump)
    d = tmp_path / "case"
    d.mkdir()
    (d / "params.txt").write_text(f"{nx} {nz} {nt} {jump} {npml} {dx} {dt} 2 {perc} {rectx1} {repeat1} "
                                  f"{rectx2} {repeat2} {alpha}\n")
    vel.tofile(d / "model.bin")
    ibtry.tofile(d / "ibtry.bin")
    oshots, obs = [], []
    for s, (sx, f0) in enumerate([(31, 14.0), (88, 11.0)]):
        irx = np.arange(1, nx - 1, 3)
        xyz = np.concatenate([[sx * dx + 1.0, 14.0], np.stack([irx * dx + 1.0, np.full(irx.size, 2.0)], 1).ravel()])
        wav = ricker(nt, dt, f0)
        isx, isz = o64.cell_of(float(xyz[0]), float(xyz[1]), dx, dx)
        sh = O.Shot(isx, isz, irx, np.zeros_like(irx), wav)
        ob = o64.forward(ocfg, vtrue, sh).astype(np.float32)
        np.asarray(xyz, np.float32).tofile(d / f"xyz_{s}.bin")
        wav.tofile(d / f"wav_{s}.bin")
        ob.tofile(d / f"obs_{s}.bin")
        oshots.append(sh)
        obs.append(ob)
    r = subprocess.run([str(exe), str(d)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    got = np.fromfile(d / "grad.bin", np.float32).reshape(nz, nx)
    val = [float(v) for v in (d / "val.txt").read_text().split()]
    J64, g64, _ = o64.gradient(ocfg, vel, oshots, obs)
    want = O.AuxOracle().grad_precond(g64.astype(np.float32), perc, rectx1, repeat1, rectx2, repeat2, alpha, ibtry)
    err = np.linalg.norm(got.astype(np.float64) - want) / np.linalg.norm(want)
    assert err <= 1e-4, err
    assert val[0] == val[1] and abs(val[1] - J64) <= 1e-5 * J64, (val, J64)
