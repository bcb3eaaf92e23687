"""The autotuner's cache handling without a GPU: the key follows the grid and
batch shape, and a missing or corrupt cache file reads as empty."""
import fwigpu
import tuning


def test_cache_key_and_files(tmp_path):
    cfg = fwigpu.make_config(400, 200, 10.0, 10.0, 0.001, 2000, fd_order=8)
    shots = [fwigpu.ShotSpec(100.0, 10.0, [[5.0, 2.0]], [0.0] * n) for n in (2000, 1500)]
    k = tuning.cache_key(cfg, shots)
    assert k == "400x200:npml20:fs1:fd8:store0:shots2:nt2000:steps3500"
    assert k != tuning.cache_key(cfg, shots[:1])
    assert tuning.load_cache(str(tmp_path / "missing.json")) == {}
    bad = tmp_path / "bad.json"
    bad.write_text("{not json")
    assert tuning.load_cache(str(bad)) == {}
    # every run-time knob but the tile grid (swept separately) and gen_grid (not swept)
    assert [k for k, _ in tuning.KNOBS] == [k for k in fwigpu.FwiTuning.KEYS[2:] if k != "gen_grid"]
