"""Launch autotuner of the engine, with a JSON cache.

The reference has nothing to tune: its grid is a compile-time macro set
(Mpar.h) and its kernels are OpenMP loops.  Here the tile is 64 x 32 cells at
compile time, and ``fwi_set_tuning`` exposes what the kernels allow to be
chosen at run time (include/fwi_gb300.h, ``fwi_tuning``):

* where the tile grid starts (``x_first``, ``z_first``): this moves the tile
  boundaries and so decides how many tiles fall in the general (edge, CPML,
  strip) classes and how wide the partial tiles at the far ends are;
* the occupancy each heavy kernel's register budget is compiled for
  (``fwd_gen_blocks``, ``bwd_gen_blocks``, ``fwd_int_blocks``,
  ``bwd_int_blocks``, and ``bwd_zgen_blocks`` for the z-general backward
  class, whose best setting differs from that of the other general classes);
* the launch order of the general classes, whether they run concurrently
  with the interior tiles and at which stream priority (``class_order``,
  ``serial``, ``priority``).

``gen_grid`` (general classes on a fixed grid of blocks that loop over their
tiles) is not swept: on the 560 x 1700, 64-shot workload every setting was
7-57% slower per step than one
block per tile, with and without the largest shared-memory carveout.

``autotune`` times a few forward and backward steps of the actual shot batch
(``fwi_time_steps``, which replays them as CUDA graphs, as the gradient does)
for each candidate, first the tile grid (coordinate by coordinate), then the
kernel variants (one knob at a time), and stores the winner under a key of the
grid and batch shape, so the next engine with that shape picks it up without a
sweep.  A candidate replaces the current best only when it is faster by more
than ``MARGIN``: a launch order or stream priority that only ties on the device
can still cost time around the copies of a whole gradient.
"""
from __future__ import annotations

import json
import os

PKG = os.path.dirname(os.path.abspath(__file__))
DEFAULT_CACHE = os.path.join(PKG, "tuning_cache.json")

KNOBS = (("fwd_gen_blocks", (4, 3)), ("bwd_gen_blocks", (4, 3)), ("fwd_int_blocks", (6, 4)),
         ("bwd_int_blocks", (4, 3)), ("class_order", (1, 2)), ("serial", (2, 1)), ("priority", (1, 2)),
         ("bwd_zgen_blocks", (4, 3)))
MARGIN = 0.005                      # relative gain a candidate needs to replace the current best


def cache_key(cfg, shots) -> str:
    nts = [s.nt for s in shots]
    return (f"{cfg.nx}x{cfg.nz}:npml{cfg.npml}:fs{cfg.free_surface}:fd{cfg.fd_order or 4}:store{cfg.store}:"
            f"shots{len(shots)}:nt{max(nts)}:steps{sum(nts)}")


def load_cache(path: str) -> dict:
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _score(eng, steps: int) -> float:
    eng.time_steps(2)                          # loads the variant's module, warms the caches
    best = None
    for _ in range(2):
        f, b = eng.time_steps(steps)
        best = f + b if best is None else min(best, f + b)
    return best


def _apply(eng, tuning: dict, shots, vel):
    before = eng.tuning()
    eng.set_tuning(tuning)
    if eng.tuning()["x_first"] != before["x_first"] or eng.tuning()["z_first"] != before["z_first"]:
        eng.set_shots(shots)
        eng.set_model(vel)


def autotune(eng, shots, vel, steps: int = 12, cache: str | None = DEFAULT_CACHE, force: bool = False) -> dict:
    """Tunes `eng` (an fwigpu.Engine) for `shots` on model `vel` and returns
    {"tuning", "ms_step", "default_ms_step", "trials", "cached"}.  The engine
    ends with the best tuning, the shots set and the model set (observed
    traces must be set afterwards: a new tile grid discards them)."""
    cfg = eng.cfg
    key = cache_key(cfg, shots)
    db = load_cache(cache) if cache else {}
    if not eng.shots:
        eng.set_shots(shots)
    eng.set_model(vel)
    if key in db and not force:
        _apply(eng, db[key]["tuning"], shots, vel)
        return dict(db[key], cached=True)
    base = eng.tuning()
    best_t, best = dict(base), _score(eng, steps)
    default_ms = best
    trials = [{"tuning": dict(base), "ms_step": best}]

    def trial(t):
        nonlocal best_t, best
        try:
            _apply(eng, t, shots, vel)
        except Exception as e:                      # a candidate the grid cannot take
            trials.append({"tuning": dict(t), "error": str(e)})
            _apply(eng, best_t, shots, vel)
            return
        ms = _score(eng, steps)
        trials.append({"tuning": dict(t), "ms_step": ms})
        if ms < best * (1.0 - MARGIN):
            best_t, best = dict(t), ms
        else:
            _apply(eng, best_t, shots, vel)

    eighth = (cfg.fd_order or 4) == 8
    if not eighth:
        for shift in (8, 16, 32):                   # tile grid: x, then z
            trial(dict(best_t, x_first=base["x_first"] + shift))
        for shift in (4, 8, 16):
            trial(dict(best_t, z_first=base["z_first"] + shift))
    for knob, values in KNOBS:
        if eighth and knob not in ("serial", "priority"):
            continue                                # the 8th-order passes have one variant each
        for v in values:
            if v != best_t[knob]:
                trial(dict(best_t, **{knob: v}))
    _apply(eng, best_t, shots, vel)
    out = {"tuning": best_t, "ms_step": best, "default_ms_step": default_ms, "trials": trials}
    if cache:
        db = load_cache(cache)
        db[key] = out
        tmp = cache + ".tmp"
        with open(tmp, "w") as f:
            json.dump(db, f, indent=1, sort_keys=True)
        os.replace(tmp, cache)
    return dict(out, cached=False)
