"""Synthetic workloads: shapes, value ranges, stability limit, seeding."""
import numpy as np

import workloads as W


def test_configs_shapes_and_cfl():
    for name in ("c1", "c2", "c3", "c4", "c5"):
        cfg, true, start, shots = W.build(name, scale=0.05)
        c = W.CONFIGS[name]
        assert true.shape == (cfg["nz"], cfg["nx"]) == start.shape
        assert true.min() >= c["vmin"] - 1e-3 and true.max() <= c["vmax"] + 1e-3
        cfl = true.max() * cfg["dt"] * 1.17205612 * np.sqrt(2.0) / cfg["dx"]
        assert cfl < 1.0
        for s in shots:
            assert (s.nt - 1) % cfg["jump"] == 0 and s.nt <= cfg["nt_max"]
            assert (s.rec_xz[:, 0] >= 0).all() and (s.rec_xz[:, 0] < cfg["nx"] * cfg["dx"]).all()


def test_full_size_c2_matches_the_benchmark_configuration():
    cfg, true, start, shots = W.build("c2")
    assert (cfg["nz"], cfg["nx"], cfg["dx"], cfg["dt"], cfg["npml"]) == (560, 1700, 10.0, 0.0008, 20)
    assert len(shots) == 64 and all(s.nt == 4000 or s.nt == 3999 + 1 for s in shots)
    assert all(s.nr == 1700 for s in shots)
    assert 1500.0 <= true.min() and true.max() <= 5500.0


def test_uneven_batch_c3():
    cfg, true, start, shots = W.build("c3", scale=0.1)
    nts = {s.nt for s in shots}
    nrs = {s.nr for s in shots}
    assert len(nts) > 1 and len(nrs) > 1


def test_seeded():
    a = W.build("c1", scale=0.1)
    b = W.build("c1", scale=0.1)
    assert np.array_equal(a[1], b[1]) and np.array_equal(a[3][0].wavelet, b[3][0].wavelet)


def test_ricker_peak():
    w = W.ricker(400, 0.001, 10.0)
    assert abs(int(np.argmax(w)) - 120) <= 1 and abs(w.max() - 1.0) < 1e-3
