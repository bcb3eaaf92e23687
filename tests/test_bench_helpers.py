"""bench.py's host helpers without a GPU: the summary of the nvidia-smi clock
samples taken during the timed region (median SM clock, the active throttle
reasons that decide whether a run is kept) and the DRAM traffic figure read
from profiles/traffic.txt."""
import importlib.util
import os
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_clock_samples_are_summarised():
    b = _bench()
    c = b.Clocks.__new__(b.Clocks)              # the sampler without starting nvidia-smi
    c.p = None
    c.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
    # clocks.sm, clocks.max.sm, power.draw, hw_slowdown, hw_thermal_slowdown, sw_thermal_slowdown, sw_power_cap
    c.f.write("2070, 2070, 900.5, Not Active, Not Active, Not Active, Active\n"
              "1965, 2070, 1301.2, Not Active, Active, Not Active, Not Active\n"
              "2070, 2070, 955.0, Not Active, Not Active, Not Active, Not Active\n"
              "[N/A], 2070, 950.0, Not Active, Not Active, Not Active, Not Active\n"
              "2070, 2070\n")
    name = c.f.name
    r = c.stop()
    assert r == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "samples": 3,
                 "reasons": ["hw_thermal_slowdown", "sw_power_cap"]}
    assert not os.path.exists(name)


def test_traffic_figure_is_read_from_the_profiles():
    b = _bench()
    with open(os.path.join(ROOT, "profiles", "traffic.txt")) as f:
        line = [ln for ln in f if ln.startswith("k_backward ")][0]
    assert b.traffic_per_cell_step("k_backward") == float(line.split()[1])
    assert 20.0 < b.traffic_per_cell_step("k_backward") < 36.0      # at most the algorithmic 36 B
    assert b.traffic_per_cell_step("no_such_kernel") is None
