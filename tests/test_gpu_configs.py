"""GPU parity at the benchmark configurations' sizes and shapes.

* The 8th-order inversion workload at full size: 201 x 401 grid, dx 10 m, dt 1 ms, nt 2000, CPML 20,
  8 surface shots, 10 Hz Ricker, 200 receivers at 2 m depth, the layered
  model with 3 Gaussian anomalies and its triangle-smoothed start model.
  Seismograms of every shot against the FP32 oracle (relative L2 <= 2e-5),
  the whole 8-shot gradient against the FP64 oracle (<= 1e-4) and the misfit
  (<= 1e-5).
* The uneven 256-shot batch (600 x 2000) at a quarter of its size: 150 x 500 grid, 64 shots with uneven records
  (750-1500 steps, sorted into the active-prefix launches, several shots
  ending mid-loop) and uneven off-end spreads.  Gradient against the FP64
  oracle (<= 1e-4), and the batched gradient against the plain per-shot path
  (the same kernels shot by shot: bit-identical).
The workloads are the seeded synthetic ones of workloads.py; the shots'
cells come from the oracle's restatement of fwi_2d.c:363-364.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SYN_TOL = 2e-5
GRAD_TOL = 1e-4
MISFIT_TOL = 1e-5


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _oracle_case(O, o, cfgkw, shots):
    """Per-shot oracle configs (records may differ in length) and shots."""
    out = []
    for sh in shots:
        isx, isz = o.cell_of(sh.src_x, sh.src_z, cfgkw["dx"], cfgkw["dz"])
        cells = [o.cell_of(float(x), float(z), cfgkw["dx"], cfgkw["dz"]) for x, z in sh.rec_xz]
        irx = np.array([c[0] for c in cells], np.int32)
        irz = np.array([c[1] for c in cells], np.int32)
        ocfg = O.make_config(nx=cfgkw["nx"], nz=cfgkw["nz"], npml=cfgkw["npml"], nt=sh.nt, dx=cfgkw["dx"],
                             dz=cfgkw["dz"], dt=cfgkw["dt"], free_surface=1, jump=cfgkw["jump"])
        out.append((ocfg, O.Shot(isx, isz, irx, irz, sh.wavelet)))
    return out


def _fp64_gradient(o64, cases, vel, obs):
    J, g = 0.0, None
    for (ocfg, sh), ob in zip(cases, obs):
        j, gg, _ = o64.gradient(ocfg, vel, [sh], [ob])
        J += j
        g = gg if g is None else g + gg
    return J, g


def test_c1_full_size(engine_lib, oracles):
    import fwigpu
    import workloads
    O, o32, o64 = oracles
    cfgkw, vtrue, vstart, shots = workloads.build("c1")
    assert (cfgkw["nz"], cfgkw["nx"], len(shots), shots[0].nt, shots[0].nr) == (201, 401, 8, 2000, 200)
    cases = _oracle_case(O, o64, cfgkw, shots)
    obs = [o64.forward(c, vtrue, sh).astype(np.float32) for c, sh in cases]
    with fwigpu.Engine(fwigpu.make_config(**cfgkw)) as e:
        e.set_shots(shots)
        e.set_model(vstart)
        syn = e.split(e.forward())
        for (c, sh), got in zip(cases, syn):
            want = o32.forward(c, vstart, sh)
            assert rel(got, want) <= SYN_TOL, rel(got, want)
        e.set_observed(np.concatenate([o.ravel() for o in obs]))
        J, g = e.gradient()
    J64, g64 = _fp64_gradient(o64, cases, vstart, obs)
    assert abs(J - J64) <= MISFIT_TOL * J64, (J, J64)
    assert rel(g, g64) <= GRAD_TOL, rel(g, g64)


def test_c3_uneven_batch_quarter_size(engine_lib, oracles):
    import fwigpu
    import workloads
    O, _, o64 = oracles
    cfgkw, vtrue, vstart, shots = workloads.build("c3", scale=0.25)
    nts = [s.nt for s in shots]
    nrs = [s.nr for s in shots]
    assert len(shots) == 64 and min(nts) < 0.6 * max(nts) and max(nrs) > 3 * min(nrs)
    cases = _oracle_case(O, o64, cfgkw, shots)
    obs = [o64.forward(c, vtrue, sh).astype(np.float32) for c, sh in cases]
    flat = np.concatenate([o.ravel() for o in obs])
    out = []
    for plain in (0, 1):
        with fwigpu.Engine(fwigpu.make_config(**cfgkw, use_graph=1 - plain, plain_per_shot=plain)) as e:
            e.set_shots(shots)
            e.set_model(vstart)
            e.set_observed(flat)
            out.append(e.gradient())
    (J, g), (Jp, gp) = out
    assert J == Jp and np.array_equal(g, gp)                 # batched == plain, bit for bit
    J64, g64 = _fp64_gradient(o64, cases, vstart, obs)
    assert abs(J - J64) <= MISFIT_TOL * J64, (J, J64)
    assert rel(g, g64) <= GRAD_TOL, rel(g, g64)
