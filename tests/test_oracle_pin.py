"""Pins the oracle restatement to the reference's own kernels.

* against ``tests/golden/ref_kernels.npz``, produced from the reference's
  fwi_2d.c by ``tests/golden/make_golden.py`` (runs everywhere);
* against the live reference kernels in ``oracle/_ref`` when they were built
  here (skipped where the reference checkout is absent).

The FP32 twin is compiled with -ffp-contract=off, so on the machine that made
the fixtures the match is bit for bit; across machines libm's exp/log may
differ in the last place, hence the 1e-6 relative allowance on the fixtures.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden as MG  # noqa: E402

GOLD = os.path.join(HERE, "golden", "ref_kernels.npz")


def close(a, b, rtol=1e-6):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = max(np.abs(b).max(), 1e-30)
    return np.abs(a - b).max() <= rtol * scale


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD))


@pytest.fixture(scope="module")
def case(oracles):
    O, o32, _ = oracles
    cfg, vel, shot, p_fs, p_nofs, p_int, model, steps = MG.case_inputs()
    return dict(O=O, o32=o32, c1=O.make_config(free_surface=1, **cfg), c0=O.make_config(free_surface=0, **cfg),
                vel=vel, shot=O.Shot(**shot), p_fs=p_fs, p_nofs=p_nofs, p_int=p_int, model=model, steps=steps)


def test_cpml_coefficients(gold, case):
    o32 = case["o32"]
    for npml, d, dt in [(8, 10.0, 0.001), (20, 12.5, 0.0008)]:
        a, b = o32.cpml_coe(npml, d, dt)
        assert close(a, gold[f"cpml_a_{npml}"]) and close(b, gold[f"cpml_b_{npml}"])


def test_model_extension(gold, case):
    o32, m = case["o32"], case["model"]
    assert np.array_equal(o32.model_ext(m, 56, 38, 1), gold["ext_fs1"])
    assert np.array_equal(o32.model_ext(m, 56, 46, 0), gold["ext_fs0"])


def test_cpml_operator_one_step(gold, case):
    o32 = case["o32"]
    w, psi = o32.apply_op(case["c1"], case["p_fs"], gold["op_psi_in"])
    assert close(w, gold["op_w"]) and close(psi, gold["op_psi_out"])


def test_interior_operator(gold, case):
    ux, vz = case["o32"].apply_int(case["c1"], case["p_int"])
    assert close(ux, gold["int_ux"]) and close(vz, gold["int_vz"])


def test_boundary_strips(gold, case):
    o32 = case["o32"]
    ud, lr = o32.strips_write(case["c1"], case["p_fs"])
    assert np.array_equal(ud, gold["strips_ud_fs1"]) and np.array_equal(lr, gold["strips_lr_fs1"])
    ud, lr = o32.strips_write(case["c0"], case["p_nofs"])
    assert np.array_equal(ud, gold["strips_ud_fs0"]) and np.array_equal(lr, gold["strips_lr_fs0"])


def test_forward_and_rebuild(gold, case):
    o32, c1 = case["o32"], case["c1"]
    syn, pf, pp = o32.forward(c1, case["vel"], case["shot"], finals=True)
    assert close(syn, gold["fwd_syn"]) and close(pf, gold["fwd_pfin"]) and close(pp, gold["fwd_pprev"])
    fs, rs = o32.probe(c1, case["vel"], case["shot"], gold["steps"])
    assert close(fs, gold["fwd_snaps"]) and close(rs, gold["reb_snaps"])


@pytest.mark.skipif(not os.path.isfile(os.path.join(os.path.dirname(HERE), "oracle", "_ref", "libfwiref.so")),
                    reason="reference kernels not built here (no reference checkout)")
def test_bit_exact_against_live_reference(case):
    O, o32, c1 = case["O"], case["o32"], case["c1"]
    ref = O.RefKernels()
    rng = np.random.default_rng(5)
    for npml, d, dt in [(8, 10.0, 0.001), (13, 7.5, 0.0006)]:
        a1, b1 = o32.cpml_coe(npml, d, dt)
        a2, b2 = ref.cpml_coe(npml, d, dt)
        assert np.array_equal(a1, a2) and np.array_equal(b1, b2)
    p = rng.standard_normal(case["p_fs"].shape).astype(np.float32)
    psi = rng.standard_normal(o32.psi_len(c1)).astype(np.float32)
    w1, s1 = o32.apply_op(c1, p, psi)
    w2, s2 = ref.apply_op(c1, p, psi)
    assert np.array_equal(w1, w2) and np.array_equal(s1, s2)
    # forward + chunked strip file rebuild (nt_mem < nt exercises fseek/fread of read_bdr)
    cfg = O.make_config(nx=40, nz=36, npml=6, nt=240, dx=12.5, dz=10.0, dt=0.001, free_surface=1, jump=1)
    vel = rng.uniform(1500, 3500, (36, 40)).astype(np.float32)
    sh = O.Shot(11, 4, np.arange(0, 40, 3), np.zeros(14, np.int32), rng.standard_normal(240).astype(np.float32))
    steps = [1, 2, 5, 100, 237, 238]
    syn1, pf1, pp1 = o32.forward(cfg, vel, sh, finals=True)
    syn2, pf2, pp2, fs2, rs2 = ref.forward(cfg, vel, sh, nt_mem=40, steps=steps)
    fs1, rs1 = o32.probe(cfg, vel, sh, steps)
    assert np.array_equal(syn1, syn2) and np.array_equal(pf1, pf2) and np.array_equal(pp1, pp2)
    assert np.array_equal(fs1, fs2) and np.array_equal(rs1, rs2)
