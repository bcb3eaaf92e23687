"""The autotuner's sweep without a GPU, on a fake engine whose step time is a
known function of the tuning: it takes a candidate only when it is faster by
more than the margin, goes back to the best tuning after a candidate the
engine rejects, sets the shots and the model again after a tile-grid change
(the engine discards them), applies a cached choice without timing anything,
and sweeps only the serial and priority knobs for the 8th-order kernels."""
import fwigpu
import tuning

SHOTS = [fwigpu.ShotSpec(100.0, 10.0, [[5.0, 2.0]], [0.0] * 100)]
BASE = dict(x_first=28, z_first=8, fwd_gen_blocks=4, bwd_gen_blocks=3, fwd_int_blocks=6, bwd_int_blocks=4,
            class_order=1, serial=2, priority=1, gen_grid=1, bwd_zgen_blocks=4)


class FakeEngine:
    def __init__(self, fd_order=4, cost=None, bad=()):
        self.cfg = fwigpu.make_config(400, 200, 10.0, 10.0, 0.001, 100, fd_order=fd_order)
        self.t = dict(BASE)
        self.cost = cost or {}              # (knob, value) -> change of the step time, relative
        self.bad = set(bad)                 # (knob, value) pairs that fwi_set_tuning rejects
        self.shots = None
        self.model = None
        self.timed = 0

    def tuning(self):
        return dict(self.t)

    def set_tuning(self, t):
        if any((k, v) in self.bad for k, v in t.items()):
            raise fwigpu.FwiError(-1, "fwi_set_tuning")
        relayout = any(t.get(k, self.t[k]) != self.t[k] for k in ("x_first", "z_first"))
        self.t.update(t)
        if relayout:                        # a new tile grid discards the shots and the model
            self.shots = self.model = None

    def set_shots(self, shots):
        self.shots = shots
        self.model = None

    def set_model(self, vel):
        self.model = vel

    def time_steps(self, steps):
        assert self.shots is not None and self.model is not None
        self.timed += 1
        ms = 1.0 + sum(self.cost.get((k, v), 0.0) for k, v in self.t.items())
        return 0.3 * ms, 0.7 * ms


def test_sweep_takes_gains_above_the_margin_and_recovers_from_rejections(tmp_path):
    cost = {("z_first", 16): -0.01, ("bwd_zgen_blocks", 3): -0.02,
            ("class_order", 2): -0.003}                                  # below the 0.5% margin
    eng = FakeEngine(cost=cost, bad={("x_first", 60)})
    out = tuning.autotune(eng, SHOTS, "vel", cache=str(tmp_path / "c.json"))
    want = dict(BASE, z_first=16, bwd_zgen_blocks=3)
    assert out["tuning"] == want and eng.tuning() == want and not out["cached"]
    assert abs(out["ms_step"] - 0.97) < 1e-12 and out["default_ms_step"] == 1.0
    assert [t for t in out["trials"] if "error" in t][0]["tuning"]["x_first"] == 60
    assert eng.shots is SHOTS and eng.model == "vel"                # set again after the grid moved
    tried = [t["tuning"] for t in out["trials"]]
    assert any(t["class_order"] == 2 for t in tried)                   # tried, not taken


def test_cached_choice_is_applied_without_timing(tmp_path):
    path = str(tmp_path / "c.json")
    first = FakeEngine(cost={("bwd_int_blocks", 3): -0.05})
    tuning.autotune(first, SHOTS, "vel", cache=path)
    again = FakeEngine(cost={("bwd_int_blocks", 3): -0.05})
    out = tuning.autotune(again, SHOTS, "vel", cache=path)
    assert out["cached"] and again.timed == 0
    assert again.tuning() == dict(BASE, bwd_int_blocks=3)


def test_eighth_order_sweeps_only_serial_and_priority(tmp_path):
    eng = FakeEngine(fd_order=8, cost={("serial", 1): -0.1, ("x_first", 36): -0.5})
    out = tuning.autotune(eng, SHOTS, "vel", cache=str(tmp_path / "c.json"))
    changed = {k for t in out["trials"] for k, v in t["tuning"].items() if v != BASE[k]}
    assert changed == {"serial", "priority"}
    assert out["tuning"] == dict(BASE, serial=1)
