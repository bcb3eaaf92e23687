"""The reference's on-disk inputs, for real-data runs (fwi_2d.c:320-352,
fwi_files_path.h, read_write.c).

Every file is raw native-endian float32 (little-endian on x86-64 and
aarch64) without a header, read with an exact element count (read_write.c's
``check == 1``: a short file or a file with elements left over is an error):

* ``<common>input/shot2ms_<ishot>.bin``: observed traces [nr][nt];
* ``<common>input/sr_location_<ishot>.bin``: source x, z then receiver x, z
  pairs, metres ((nr + 1) * 2 values);
* ``<common>input/fbt_<ishot>.bin``: first-break times [nr] (optional);
* ``<common>input/initial_model.bin``: velocity [nz][nx];
* ``<common>input/bottom.bin``: bottom (water) depth per column [nx];
* ``<common>wavelet_<first>_<last>.bin``: source wavelet [nt], shared by the
  shots first..last of a group of ``step`` shots.

``load_shot`` turns a shot's files into the engine's ``ShotSpec`` and its
observed traces.
"""
from __future__ import annotations

import os

import numpy as np

SHOTS = "{common}input/shot2ms_{ishot}.bin"
XYZ_SR = "{common}input/sr_location_{ishot}.bin"
FBT = "{common}input/fbt_{ishot}.bin"
INIT_MDL = "{common}input/initial_model.bin"
BTRY = "{common}input/bottom.bin"
WAVELET = "{common}wavelet_{first}_{last}.bin"


class FormatError(ValueError):
    """A file is missing or does not hold exactly the expected number of values."""


def read_f32(path: str, n: int) -> np.ndarray:
    """Exactly n float32 values from path (read_from_file with check == 1)."""
    if not os.path.isfile(path):
        raise FormatError(f"error opening {path}")
    size = os.path.getsize(path)
    if size != 4 * n:
        raise FormatError(f"{path}: {size} bytes, expected {4 * n} ({n} float32 values)")
    return np.fromfile(path, dtype="<f4", count=n).astype(np.float32)


def write_f32(path: str, a) -> None:
    """write_to_file: the values of a as raw little-endian float32."""
    np.ascontiguousarray(a, dtype="<f4").tofile(path)


def wavelet_path(common: str, ishot: int, step: int = 1) -> str:
    first = (ishot // step) * step
    return WAVELET.format(common=common, first=first, last=first + step - 1)


def load_model(common: str, nz: int, nx: int) -> np.ndarray:
    return read_f32(INIT_MDL.format(common=common), nz * nx).reshape(nz, nx)


def load_bottom(common: str, nx: int) -> np.ndarray:
    return read_f32(BTRY.format(common=common), nx)


def load_shot(common: str, ishot: int, nr: int, nt_trace: int, nt: int, step: int = 1, wav_scale: float = 1.0):
    """(ShotSpec, obs [nr][nt_trace], fbt [nr] or None) of shot ishot.
    nt_trace is the number of samples per recorded trace, nt the number of
    wavelet samples (time steps); the wavelet is scaled by wav_scale
    (WAV_SCALE, fwi_2d.c:352)."""
    from fwigpu import ShotSpec
    obs = read_f32(SHOTS.format(common=common, ishot=ishot), nr * nt_trace).reshape(nr, nt_trace)
    xyz = read_f32(XYZ_SR.format(common=common, ishot=ishot), 2 * (nr + 1))
    wav = read_f32(wavelet_path(common, ishot, step), nt) * np.float32(wav_scale)
    fbt_path = FBT.format(common=common, ishot=ishot)
    fbt = read_f32(fbt_path, nr) if os.path.isfile(fbt_path) else None
    spec = ShotSpec(xyz[0], xyz[1], xyz[2:].reshape(nr, 2), wav)
    return spec, obs, fbt


def save_shot(common: str, ishot: int, spec, obs, step: int = 1, fbt=None) -> None:
    """Writes a shot in the reference's layout (the inverse of load_shot)."""
    os.makedirs(os.path.join(common, "input"), exist_ok=True)
    write_f32(SHOTS.format(common=common, ishot=ishot), obs)
    write_f32(XYZ_SR.format(common=common, ishot=ishot),
              np.concatenate([[spec.src_x, spec.src_z], np.asarray(spec.rec_xz, np.float32).ravel()]))
    write_f32(wavelet_path(common, ishot, step), spec.wavelet)
    if fbt is not None:
        write_f32(FBT.format(common=common, ishot=ishot), fbt)
