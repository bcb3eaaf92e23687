"""Pins the aux oracle (oracle/fwi_oracle_aux.c) to the reference.

* grad_precond_new5 + triangle2 (grad_prec.c:5-52, triangle_smooth.c:5-110)
  and sfbandpass (butterworth_filter.c:127-200): bit for bit.
* XCORR1D (xcorr_msf.c:4-181): misfit to 1e-5 and residual to 1e-4
  relative; the reference evaluates its two correlations with
  single-precision FFTs, the oracle with exact sums.

Each comparison runs against the committed fixtures (tests/golden/ref_aux.npz,
made by tests/golden/make_golden.py --aux from the reference itself) and,
where the reference sources are present, against the reference routines
compiled live by `make -C oracle ref`.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden as G  # noqa: E402

XCORR_MISFIT_RTOL = 1e-5
XCORR_RES_RTOL = 1e-4


@pytest.fixture(scope="module")
def aux(oracles):
    O = oracles[0]
    return O.AuxOracle()


@pytest.fixture(scope="module")
def golden():
    return np.load(os.path.join(HERE, "golden", "ref_aux.npz"))


@pytest.fixture(scope="module")
def ref(oracles):
    O = oracles[0]
    if not O.RefAux.available():
        pytest.skip("reference sources not available")
    return O.RefAux()


def _rel(a, b):
    return np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(np.asarray(b, np.float64)), 1e-300)


@pytest.mark.parametrize("k", range(len(G.PRECOND_CASES)))
def test_precond_bit_exact_to_fixture(aux, golden, k):
    grad, bottom, *_ = G.aux_inputs()
    got = aux.grad_precond(grad, *G.PRECOND_CASES[k], bottom)
    assert np.array_equal(got, golden[f"precond_{k}"])


@pytest.mark.parametrize("k", range(len(G.BANDPASS_CASES)))
def test_bandpass_bit_exact_to_fixture(aux, golden, k):
    _, _, traces, *_ = G.aux_inputs()
    got = aux.bandpass(traces, *G.BANDPASS_CASES[k])
    assert np.array_equal(got, golden[f"bandpass_{k}"])


@pytest.mark.parametrize("k", range(len(G.XCORR_CASES)))
def test_xcorr_matches_fixture(aux, golden, k):
    mode, omin, omax, kind = G.XCORR_CASES[k]
    obs, syn, sr = G.xcorr_traces(kind)
    mis, res = aux.xcorr1d(obs, syn, sr, omin, omax, mode)
    want_mis, want_res = golden[f"xcorr_mis_{k}"], golden[f"xcorr_res_{k}"]
    assert np.allclose(mis, want_mis, rtol=XCORR_MISFIT_RTOL, atol=0), (mis, want_mis)
    assert _rel(res, want_res) <= XCORR_RES_RTOL, _rel(res, want_res)
    # skipped traces (energy ratio, offsets outside the window) have res == 0 in both
    assert np.array_equal(np.all(res == 0, axis=1), np.all(want_res == 0, axis=1))


def test_xcorr_skips_and_lag_weights(aux):
    """The energy-ratio and offset tests exclude traces, and a syn equal to
    obs shifted by zero lag gives alpha = sum T^2 x^2 / sum x^2 at its
    minimum over shifts."""
    *_, obs, syn, sr = G.aux_inputs()
    mis, res = aux.xcorr1d(obs, syn, sr, 50.0, 550.0, 0)
    skipped = np.all(res == 0, axis=1)
    assert skipped[0] and skipped[6] and skipped[5]          # offsets 0 and 600 m; 25x weaker trace
    assert not skipped[1:5].any()
    nt = obs.shape[1]
    t = np.arange(nt)
    base = (np.exp(-((t - 60) / 6.0) ** 2) * np.cos(0.3 * (t - 60))).astype(np.float32)[None]
    sr1 = np.array([0, 0, 100.0, 2.0], np.float32)
    alphas = [aux.xcorr1d(base, np.roll(base, s, axis=1), sr1, 0.0, 1e9, 0)[0][1] for s in (-6, -3, 0, 3, 6)]
    assert np.argmin(alphas) == 2


def test_precond_bit_exact_live(aux, ref):
    grad, bottom, *_ = G.aux_inputs()
    rng = np.random.default_rng(11)
    g2 = rng.standard_normal((64, 91)).astype(np.float32) * 1e-3
    b2 = rng.integers(0, 9, 91).astype(np.int32)
    for g, b in ((grad, bottom), (g2, b2)):
        for c in G.PRECOND_CASES + [(0.95, 20, 3, 15, 2, 1.0)]:
            assert np.array_equal(aux.grad_precond(g, *c, b), ref.grad_precond(g, *c, b))


def test_bandpass_bit_exact_live(aux, ref):
    rng = np.random.default_rng(12)
    tr = rng.standard_normal((5, 777)).astype(np.float32)
    for c in G.BANDPASS_CASES + [(0.0005, 0, 8, 8, 25.0, 2.0), (0.001, 1, 7, 9, 100.0, 8.0)]:
        assert np.array_equal(aux.bandpass(tr, *c), ref.bandpass(tr, *c))


def test_xcorr_live(aux, ref):
    for nt in (121, 120):                                     # odd and even trace lengths
        for mode, omin, omax, kind in G.XCORR_CASES:
            obs, syn, sr = G.xcorr_traces(kind)
            m1, r1 = aux.xcorr1d(obs[:, :nt], syn[:, :nt], sr, omin, omax, mode)
            m2, r2 = ref.xcorr1d(obs[:, :nt], syn[:, :nt], sr, omin, omax, mode, npad=3)
            assert np.allclose(m1, m2, rtol=XCORR_MISFIT_RTOL, atol=0), (m1, m2)
            assert _rel(r1, r2) <= XCORR_RES_RTOL
