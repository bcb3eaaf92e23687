"""GPU parity at the benchmark configurations' sizes and shapes.

* The 8th-order inversion workload at full size: 201 x 401 grid, dx 10 m, dt 1 ms, nt 2000, CPML 20,
  8 surface shots, 10 Hz Ricker, 200 receivers at 2 m depth, the layered
  model with 3 Gaussian anomalies and its triangle-smoothed start model.
  Seismograms of every shot against the FP32 oracle (relative L2 <= 2e-5),
  the whole 8-shot gradient against the FP64 oracle (<= 1e-4) and the misfit
  (<= 1e-5).
* The headline workload's full grid (560 x 1700, dx 10 m, dt 0.8 ms, CPML 20) with
  three shots of 1201 steps: one of its own surface shots with its 1700
  receivers, one at the surface 100 m from the left edge with the same
  receivers, and one at 5.3 km depth near the bottom-right corner, recorded
  by a line of receivers 50 m above the bottom CPML and a column 50 m inside
  the right one (with a weaker source, so that its misfit is near the other
  shots').  Every tile class (x-general, z-general above and below,
  corners, interior) carries field and adjoint field, and every shot carries
  misfit.  The gradient is taken at a start model 5% slower than the smoothed
  one, so that the residuals are of the order of the data: with the nearly
  equal early arrivals of the smoothed model the residuals are 4e-4 of the
  traces and FP32 rounding of the modelling (about 1e-6, the FP32 oracle's
  as well) would dominate them.  Seismograms against the FP32 oracle,
  gradient and misfit against the FP64 oracle, and two properties that hold
  at any size: the batched gradient equals the plain per-shot one bit for
  bit, and doubling the wavelet and the observed traces multiplies the misfit
  and the gradient by 4.  The latter is exact in IEEE arithmetic except where
  an intermediate is subnormal; the precursor ahead of each wavefront is, and
  from there the two runs round differently, so it holds to FP32 accuracy.
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


def test_c2_full_grid(engine_lib, oracles):
    import fwigpu
    import workloads
    O, o32, o64 = oracles
    cfgkw, vtrue, vstart, shots = workloads.build("c2", nshots=1, nt=1201)
    assert (cfgkw["nz"], cfgkw["nx"], cfgkw["npml"], shots[0].nr) == (560, 1700, 20, 1700)
    v0 = (0.95 * vstart).astype(np.float32)
    rec, wav = shots[0].rec_xz, shots[0].wavelet
    dx = cfgkw["dx"]
    length, depth = cfgkw["nx"] * dx, cfgkw["nz"] * dx
    xs = np.arange(0.0, length - dx, 2 * dx)
    zs = np.arange(2.0, depth - dx, 10 * dx)
    deep = np.concatenate([np.stack([xs, np.full_like(xs, depth - 5 * dx)], 1),
                           np.stack([np.full_like(zs, length - 5 * dx), zs], 1)])
    # the deep shot's receivers sit close to it: a weaker source keeps its misfit near the others'
    shots += [fwigpu.ShotSpec(100.0, 10.0, rec, wav), fwigpu.ShotSpec(length - 200.0, depth - 300.0, deep, 0.02 * wav)]
    cases = _oracle_case(O, o64, cfgkw, shots)
    obs = [o64.forward(c, vtrue, sh).astype(np.float32) for c, sh in cases]
    flat = np.concatenate([o.ravel() for o in obs])
    out = []
    for plain in (0, 1):
        with fwigpu.Engine(fwigpu.make_config(**cfgkw, use_graph=1 - plain, plain_per_shot=plain)) as e:
            e.set_shots(shots)
            e.set_model(v0)
            if not plain:
                syn = e.split(e.forward())
                for (c, sh), got in zip(cases, syn):
                    want = o32.forward(c, v0, sh)
                    assert rel(got, want) <= SYN_TOL, rel(got, want)
            e.set_observed(flat)
            out.append(e.gradient())
            if not plain:                       # twice the source, twice the data: 4x misfit and gradient
                e.set_shots([fwigpu.ShotSpec(s.src_x, s.src_z, s.rec_xz, 2.0 * s.wavelet) for s in shots])
                e.set_model(v0)
                e.set_observed(2.0 * flat)
                J2, g2 = e.gradient()
    (J, g), (Jp, gp) = out
    assert J == Jp and np.array_equal(g, gp)                 # batched == plain, bit for bit
    assert abs(J2 / (4.0 * J) - 1.0) <= MISFIT_TOL and rel(g2, 4.0 * g) <= GRAD_TOL, (J2 / J, rel(g2, 4.0 * g))
    per = [o64.gradient(c, v0, [sh], [ob]) for (c, sh), ob in zip(cases, obs)]
    J64, g64 = sum(p[0] for p in per), sum(p[1] for p in per)
    assert min(p[0] for p in per) > 0.05 * J64, [p[0] for p in per]     # every shot carries misfit
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
