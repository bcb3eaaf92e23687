"""The reference's on-disk formats (fwi_2d.c:320-352, read_write.c): raw
float32 files with exact element counts, the file-name patterns of
fwi_files_path.h, and a round trip into the engine's ShotSpec."""
import numpy as np
import pytest


def test_shot_round_trip_and_layout(tmp_path):
    import formats
    import fwigpu
    common = str(tmp_path) + "/"
    rng = np.random.default_rng(1)
    nr, nt_trace, nt = 5, 51, 101
    rec = np.stack([np.arange(nr) * 10.0 + 3.0, np.full(nr, 2.0)], 1)
    spec = fwigpu.ShotSpec(205.0, 12.0, rec, rng.standard_normal(nt).astype(np.float32))
    obs = rng.standard_normal((nr, nt_trace)).astype(np.float32)
    fbt = rng.uniform(0, 1, nr).astype(np.float32)
    formats.save_shot(common, 7, spec, obs, step=4, fbt=fbt)
    # the reference's names: shots 4..7 share wavelet_4_7.bin
    assert (tmp_path / "input" / "shot2ms_7.bin").stat().st_size == 4 * nr * nt_trace
    assert (tmp_path / "input" / "sr_location_7.bin").stat().st_size == 4 * 2 * (nr + 1)
    assert (tmp_path / "wavelet_4_7.bin").is_file()
    # raw little-endian float32, source first then receiver pairs
    raw = np.fromfile(tmp_path / "input" / "sr_location_7.bin", "<f4")
    assert raw[0] == 205.0 and raw[1] == 12.0 and np.array_equal(raw[2:].reshape(nr, 2), rec.astype(np.float32))
    spec2, obs2, fbt2 = formats.load_shot(common, 7, nr, nt_trace, nt, step=4, wav_scale=2.0)
    assert np.array_equal(obs2, obs) and np.array_equal(fbt2, fbt)
    assert spec2.src_x == 205.0 and np.array_equal(spec2.rec_xz, rec.astype(np.float32))
    assert np.array_equal(spec2.wavelet, spec.wavelet * np.float32(2.0))


def test_exact_sizes_are_enforced(tmp_path):
    import formats
    common = str(tmp_path) + "/"
    (tmp_path / "input").mkdir()
    formats.write_f32(str(tmp_path / "input" / "initial_model.bin"), np.ones((4, 6)))
    assert formats.load_model(common, 4, 6).shape == (4, 6)
    with pytest.raises(formats.FormatError):
        formats.load_model(common, 4, 5)          # elements left over
    with pytest.raises(formats.FormatError):
        formats.load_model(common, 5, 6)          # short file
    with pytest.raises(formats.FormatError):
        formats.load_bottom(common, 6)            # missing file
