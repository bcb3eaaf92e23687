"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this module.  It loads

* ``_build/libfwioracle_f32.so`` / ``_build/libfwioracle_f64.so`` -- the C
  restatement of the reference's propagator kernels (fwi_2d.c) and of the
  missing gradient driver ``grad4_1shot`` (header.h:283), FP32 and FP64 twins;
* ``_ref/libfwiref.so`` (optional) -- the reference's own fwi_2d.c kernels
  compiled by ``make ref`` from the reference checkout or from its staged,
  git-ignored copy in ``_ref/src``; present only where those sources are.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REFDIR = os.path.join(HERE, "_ref")


class OrcConfig(C.Structure):
    _fields_ = [("nx", C.c_int), ("nz", C.c_int), ("npml", C.c_int),
                ("free_surface", C.c_int), ("nt", C.c_int), ("jump", C.c_int),
                ("dx", C.c_float), ("dz", C.c_float), ("dt", C.c_float),
                ("pml_max_f", C.c_float), ("pml_max_v", C.c_float),
                ("pml_coef_r", C.c_float), ("nthreads", C.c_int), ("fd_order", C.c_int)]


class OrcShot(C.Structure):
    _fields_ = [("isx", C.c_int), ("isz", C.c_int), ("nr", C.c_int),
                ("irx", C.POINTER(C.c_int)), ("irz", C.POINTER(C.c_int)),
                ("wav", C.POINTER(C.c_float))]


STAGED = os.path.join(REFDIR, "src")


def reference_sources() -> str | None:
    """Directory with the reference's C sources and headers: the git-ignored
    copy that ``make stage`` leaves in ``_ref/src`` (taken from the reference
    checkout where it exists), or None where neither was ever present."""
    return STAGED if os.path.isfile(os.path.join(STAGED, "fwi_2d.c")) else None


def build(quiet: bool = True) -> None:
    """Compile the oracle twins, and the reference's own kernels when their
    sources are at hand (the checkout, or the staged copy of it)."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True, stdout=out)
    subprocess.run(["make", "-s", "-C", HERE, "stage"], check=True, stdout=out)
    if reference_sources():
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True, stdout=out)


def _ptr(a, ctype):
    return a.ctypes.data_as(C.POINTER(ctype)) if a is not None else None


def make_config(nx, nz, npml, nt, dx, dz, dt, free_surface=1, jump=1,
                pml_max_f=15.0, pml_max_v=6000.0, pml_coef_r=0.001, nthreads=0, fd_order=4) -> OrcConfig:
    """Defaults of the CPML constants are fwi_sys.h:2-4 (MAX_F, MAX_V, COEF_R);
    fd_order 4 is the reference's (fwi_sys.h:7), 8 the 8th-order extension."""
    return OrcConfig(nx, nz, npml, int(free_surface), nt, jump, dx, dz, dt,
                     pml_max_f, pml_max_v, pml_coef_r, nthreads, fd_order)


class Shot:
    """Keeps the numpy buffers of one orc_shot alive."""

    def __init__(self, isx, isz, irx, irz, wav):
        self.irx = np.ascontiguousarray(irx, dtype=np.int32)
        self.irz = np.ascontiguousarray(irz, dtype=np.int32)
        self.wav = np.ascontiguousarray(wav, dtype=np.float32)
        self.c = OrcShot(int(isx), int(isz), len(self.irx), _ptr(self.irx, C.c_int),
                         _ptr(self.irz, C.c_int), _ptr(self.wav, C.c_float))

    @property
    def nr(self):
        return len(self.irx)


class Oracle:
    """One twin of the restatement (``twin`` = 'f32' or 'f64')."""

    def __init__(self, twin: str = "f32"):
        path = os.path.join(BUILD, f"libfwioracle_{twin}.so")
        if not os.path.isfile(path):
            build()
        self.lib = C.CDLL(path)
        self.real = np.float32 if self.lib.orc_real_bytes() == 4 else np.float64
        self.creal = C.c_float if self.real == np.float32 else C.c_double
        self.twin = twin

    # -- geometry -----------------------------------------------------------------
    def grid(self, cfg):
        out = (C.c_int * 4)()
        self.lib.orc_grid(C.byref(cfg), out)
        return tuple(out)  # pnx, pnz, x0, z0

    def nt0(self, cfg):
        return (cfg.nt - 1) // cfg.jump + 1

    def cell_of(self, x, z, dx, dz):
        """Cell of a position in metres, fwi_2d.c:363-364."""
        ix, iz = C.c_int(), C.c_int()
        self.lib.orc_cell_of(C.c_float(x), C.c_float(z), C.c_float(dx), C.c_float(dz), C.byref(ix), C.byref(iz))
        return ix.value, iz.value

    # -- single pieces ------------------------------------------------------------
    def cpml_coe(self, npml, d, dt, max_f=15.0, max_v=6000.0, coef_r=0.001):
        a = np.zeros(2 * npml + 1, np.float32)
        b = np.zeros(2 * npml + 1, np.float32)
        self.lib.orc_cpml_coe(_ptr(a, C.c_float), _ptr(b, C.c_float), C.c_int(npml), C.c_float(d),
                              C.c_float(dt), C.c_float(max_f), C.c_float(max_v), C.c_float(coef_r))
        return a, b

    def model_ext(self, model, en1, en2, fs):
        model = np.ascontiguousarray(model, np.float32)
        n2, n1 = model.shape
        out = np.zeros((en2, en1), np.float32)
        self.lib.orc_model_ext(_ptr(model, C.c_float), n1, n2, _ptr(out, C.c_float), en1, en2, int(fs))
        return out

    def fd_coeffs(self, dx, dz):
        out = np.zeros(8, np.float32)
        self.lib.orc_fd_coeffs(C.c_float(dx), C.c_float(dz), _ptr(out, C.c_float))
        return out

    def ekp(self, cfg, vel):
        pnx, pnz, _, _ = self.grid(cfg)
        vel = np.ascontiguousarray(vel, np.float32)
        out = np.zeros((pnz, pnx), np.float32)
        self.lib.orc_ekp(C.byref(cfg), _ptr(vel, C.c_float), _ptr(out, C.c_float))
        return out

    def psi_len(self, cfg):
        return self.lib.orc_psi_len(C.byref(cfg))

    def apply_op(self, cfg, p, psi):
        pnx, pnz, _, _ = self.grid(cfg)
        p = np.ascontiguousarray(p, self.real)
        psi = np.ascontiguousarray(psi, self.real).copy()
        w = np.zeros((pnz, pnx), self.real)
        st = self.lib.orc_apply_op(C.byref(cfg), _ptr(p, self.creal), _ptr(psi, self.creal), _ptr(w, self.creal))
        assert st == 0, st
        return w, psi

    def apply_op_t(self, cfg, q, psib):
        pnx, pnz, _, _ = self.grid(cfg)
        q = np.ascontiguousarray(q, self.real)
        psib = np.ascontiguousarray(psib, self.real).copy()
        pbar = np.zeros((pnz, pnx), self.real)
        st = self.lib.orc_apply_op_t(C.byref(cfg), _ptr(q, self.creal), _ptr(psib, self.creal),
                                     _ptr(pbar, self.creal))
        assert st == 0, st
        return pbar, psib

    def apply_int(self, cfg, p):
        p = np.ascontiguousarray(p, self.real)
        ux = np.zeros_like(p)
        vz = np.zeros_like(p)
        assert self.lib.orc_apply_int(C.byref(cfg), _ptr(p, self.creal), _ptr(ux, self.creal),
                                      _ptr(vz, self.creal)) == 0
        return ux, vz

    def strips_write(self, cfg, p_pad):
        S = 7 if cfg.fd_order == 8 else 3
        p_pad = np.ascontiguousarray(p_pad, self.real)
        ud = np.zeros((2 * S, cfg.nx), self.real)
        lr = np.zeros((cfg.nz, 2 * S), self.real)
        self.lib.orc_strips_write(C.byref(cfg), _ptr(p_pad, self.creal), _ptr(ud, self.creal),
                                  _ptr(lr, self.creal))
        return ud, lr

    # -- drivers ------------------------------------------------------------------
    def forward(self, cfg, vel, shot: Shot, finals=False):
        pnx, pnz, _, _ = self.grid(cfg)
        vel = np.ascontiguousarray(vel, np.float32)
        syn = np.zeros((shot.nr, self.nt0(cfg)), self.real)
        pf = np.zeros((pnz, pnx), self.real) if finals else None
        pp = np.zeros((pnz, pnx), self.real) if finals else None
        st = self.lib.orc_forward(C.byref(cfg), _ptr(vel, C.c_float), C.byref(shot.c), _ptr(syn, self.creal),
                                  _ptr(pf, self.creal), _ptr(pp, self.creal))
        if st:
            raise ValueError(f"orc_forward failed: {st}")
        return (syn, pf, pp) if finals else syn

    def gradient(self, cfg, vel, shots, obs_list):
        vel = np.ascontiguousarray(vel, np.float32)
        arr = (OrcShot * len(shots))(*[s.c for s in shots])
        obs = np.ascontiguousarray(np.concatenate([np.asarray(o, np.float32).ravel() for o in obs_list]))
        syn = np.zeros(obs.size, self.real)
        grad = np.zeros((cfg.nz, cfg.nx), np.float64)
        mis = np.zeros(1, np.float64)
        st = self.lib.orc_gradient(C.byref(cfg), _ptr(vel, C.c_float), len(shots), arr, _ptr(obs, C.c_float),
                                   _ptr(mis, C.c_double), _ptr(grad, C.c_double), _ptr(syn, self.creal))
        if st:
            raise ValueError(f"orc_gradient failed: {st}")
        return float(mis[0]), grad, syn

    def backward(self, cfg, vel, shot, res):
        vel = np.ascontiguousarray(vel, np.float32)
        res = np.ascontiguousarray(res, self.real)
        grad = np.zeros((cfg.nz, cfg.nx), np.float64)
        st = self.lib.orc_backward(C.byref(cfg), _ptr(vel, C.c_float), C.byref(shot.c), _ptr(res, self.creal),
                                   _ptr(grad, C.c_double))
        if st:
            raise ValueError(f"orc_backward failed: {st}")
        return grad

    def adjoint_wavelet(self, cfg, vel, shot, res):
        vel = np.ascontiguousarray(vel, np.float32)
        res = np.ascontiguousarray(res, self.real)
        wbar = np.zeros(cfg.nt, self.real)
        st = self.lib.orc_adjoint_wavelet(C.byref(cfg), _ptr(vel, C.c_float), C.byref(shot.c),
                                          _ptr(res, self.creal), _ptr(wbar, self.creal))
        if st:
            raise ValueError(f"orc_adjoint_wavelet failed: {st}")
        return wbar

    def probe(self, cfg, vel, shot, steps, fwd=True, reb=True):
        pnx, pnz, _, _ = self.grid(cfg)
        vel = np.ascontiguousarray(vel, np.float32)
        steps = np.ascontiguousarray(steps, np.int32)
        fs = np.zeros((len(steps), pnz, pnx), self.real) if fwd else None
        rs = np.zeros((len(steps), cfg.nz, cfg.nx), self.real) if reb else None
        st = self.lib.orc_probe(C.byref(cfg), _ptr(vel, C.c_float), C.byref(shot.c), len(steps),
                                _ptr(steps, C.c_int), _ptr(fs, self.creal), _ptr(rs, self.creal))
        if st:
            raise ValueError(f"orc_probe failed: {st}")
        return fs, rs


class RefKernels:
    """The reference's own kernels (oracle/_ref/libfwiref.so), FP32."""

    path = os.path.join(REFDIR, "libfwiref.so")

    @classmethod
    def available(cls) -> bool:
        return os.path.isfile(cls.path)

    def __init__(self):
        self.lib = C.CDLL(self.path)

    def cpml_coe(self, npml, d, dt, max_f=15.0, max_v=6000.0, coef_r=0.001):
        a = np.zeros(2 * npml + 1, np.float32)
        b = np.zeros(2 * npml + 1, np.float32)
        self.lib.ref_cpml_coe(_ptr(a, C.c_float), _ptr(b, C.c_float), C.c_int(npml), C.c_float(d),
                              C.c_float(dt), C.c_float(max_f), C.c_float(max_v), C.c_float(coef_r))
        return a, b

    def model_ext(self, model, en1, en2, fs):
        model = np.ascontiguousarray(model, np.float32)
        n2, n1 = model.shape
        out = np.zeros((en2, en1), np.float32)
        self.lib.ref_model_ext(_ptr(model, C.c_float), n1, n2, _ptr(out, C.c_float), en1, en2, int(fs))
        return out

    def apply_op(self, cfg, p, psi):
        p = np.ascontiguousarray(p, np.float32)
        psi = np.ascontiguousarray(psi, np.float32).copy()
        w = np.zeros_like(p)
        assert self.lib.ref_apply_op(C.byref(cfg), _ptr(p, C.c_float), _ptr(psi, C.c_float), _ptr(w, C.c_float)) == 0
        return w, psi

    def apply_int(self, cfg, p):
        p = np.ascontiguousarray(p, np.float32)
        ux = np.zeros_like(p)
        vz = np.zeros_like(p)
        assert self.lib.ref_apply_int(C.byref(cfg), _ptr(p, C.c_float), _ptr(ux, C.c_float), _ptr(vz, C.c_float)) == 0
        return ux, vz

    def strips_write(self, cfg, p_pad):
        p_pad = np.ascontiguousarray(p_pad, np.float32)
        ud = np.zeros((6, cfg.nx), np.float32)
        lr = np.zeros((cfg.nz, 6), np.float32)
        self.lib.ref_strips_write(C.byref(cfg), _ptr(p_pad, C.c_float), _ptr(ud, C.c_float), _ptr(lr, C.c_float))
        return ud, lr

    def forward(self, cfg, vel, shot: Shot, nt_mem, steps=()):
        pnx = cfg.nx + 2 * cfg.npml
        pnz = cfg.nz + (1 if cfg.free_surface else 2) * cfg.npml
        nt0 = (cfg.nt - 1) // cfg.jump + 1
        vel = np.ascontiguousarray(vel, np.float32)
        syn = np.zeros((shot.nr, nt0), np.float32)
        pf = np.zeros((pnz, pnx), np.float32)
        pp = np.zeros((pnz, pnx), np.float32)
        steps = np.ascontiguousarray(steps, np.int32)
        fs = np.zeros((len(steps), pnz, pnx), np.float32)
        rs = np.zeros((len(steps), cfg.nz, cfg.nx), np.float32)
        st = self.lib.ref_forward(C.byref(cfg), _ptr(vel, C.c_float), C.byref(shot.c), int(nt_mem),
                                  _ptr(syn, C.c_float), _ptr(pf, C.c_float), _ptr(pp, C.c_float),
                                  len(steps), _ptr(steps, C.c_int), _ptr(fs, C.c_float), _ptr(rs, C.c_float))
        if st:
            raise ValueError(f"ref_forward failed: {st}")
        return syn, pf, pp, fs, rs

    def gradient(self, cfg, vel, shots, obs_list, nt_mem=None):
        """L2 gradient of the shots on the reference's own kernels
        (ref_gradient in ref_driver.c: the timing path of the reference
        arm).  nt_mem: steps per strip chunk written to the temp file; by
        default the largest divisor of nt up to 200."""
        if nt_mem is None:
            nt_mem = max(d for d in range(1, min(cfg.nt, 200) + 1) if cfg.nt % d == 0)
        vel = np.ascontiguousarray(vel, np.float32)
        arr = (OrcShot * len(shots))(*[s.c for s in shots])
        obs = np.ascontiguousarray(np.concatenate([np.asarray(o, np.float32).ravel() for o in obs_list]))
        grad = np.zeros((cfg.nz, cfg.nx), np.float64)
        mis = np.zeros(1, np.float64)
        st = self.lib.ref_gradient(C.byref(cfg), _ptr(vel, C.c_float), len(shots), arr, _ptr(obs, C.c_float),
                                   int(nt_mem), _ptr(mis, C.c_double), _ptr(grad, C.c_double))
        if st:
            raise ValueError(f"ref_gradient failed: {st}")
        return float(mis[0]), grad


# ---------------------------------------------------------------------------
# Routines around the gradient: preconditioning, band-pass, XCORR misfit
# ---------------------------------------------------------------------------
def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class _AuxCalls:
    """Shared ctypes calls of the aux oracle and the reference's own routines;
    `pre` is the symbol prefix ("orc_" or "ref_")."""

    def _setup(self, lib, pre):
        self.lib, self.pre = lib, pre
        f = getattr(lib, pre + "grad_precond")
        f.argtypes = [C.POINTER(C.c_float), C.c_int, C.c_int, C.c_float, C.c_int, C.c_int, C.c_int, C.c_int,
                      C.c_float, C.POINTER(C.c_int)]
        f.restype = C.c_int
        f = getattr(lib, pre + "triangle2")
        f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        f.restype = C.c_int
        f = getattr(lib, pre + "xcorr1d")
        if pre == "ref_":
            f.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int, C.c_int, C.POINTER(C.c_float),
                          C.c_float, C.c_float, C.c_int, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        else:
            f.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int, C.c_int, C.POINTER(C.c_float),
                          C.c_float, C.c_float, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        f.restype = C.c_int

    def grad_precond(self, body, perc, rectx1, repeat1, rectx2, repeat2, alpha_grad, bottom):
        """grad_precond_new5 (grad_prec.c:5-52) of body[mnz][mnx]; returns a new array."""
        out = _f32(body).copy()
        mnz, mnx = out.shape
        bot = np.ascontiguousarray(bottom, dtype=np.int32)
        assert bot.shape == (mnx,)
        st = getattr(self.lib, self.pre + "grad_precond")(_ptr(out, C.c_float), mnx, mnz, perc, rectx1, repeat1,
                                                          rectx2, repeat2, alpha_grad, _ptr(bot, C.c_int))
        assert st == 0
        return out

    def triangle2(self, rect1, rect2, nt, uu):
        uu = _f32(uu)
        n2, n1 = uu.shape
        vv = np.zeros_like(uu)
        assert getattr(self.lib, self.pre + "triangle2")(rect1, rect2, nt, n1, n2, _ptr(uu, C.c_float),
                                                         _ptr(vv, C.c_float)) == 0
        return vv

    def xcorr1d(self, obs, syn, sr_xyz, omin, omax, mode, npad=0):
        """XCORR1D (xcorr_msf.c:4-181) of traces [nr][nt]; mode 0 middle, 1 leading.
        Returns (misfit[2] float32, res [nr][nt])."""
        obs, syn, sr = _f32(obs), _f32(syn), _f32(sr_xyz)
        nr, nt = obs.shape
        mis = np.zeros(2, np.float32)
        res = np.zeros_like(obs)
        f = getattr(self.lib, self.pre + "xcorr1d")
        if self.pre == "ref_":
            st = f(_ptr(obs, C.c_float), _ptr(syn, C.c_float), nr, nt, _ptr(sr, C.c_float), omin, omax, npad, mode,
                   _ptr(mis, C.c_float), _ptr(res, C.c_float))
        else:
            st = f(_ptr(obs, C.c_float), _ptr(syn, C.c_float), nr, nt, _ptr(sr, C.c_float), omin, omax, mode,
                   _ptr(mis, C.c_float), _ptr(res, C.c_float))
        assert st == 0
        return mis, res


class AuxOracle(_AuxCalls):
    """The CPU restatement (fwi_oracle_aux.c) of grad_precond_new5, triangle2,
    sfbandpass and XCORR1D."""

    def __init__(self):
        lib = C.CDLL(os.path.join(BUILD, "libfwioracle_aux.so"))
        self._setup(lib, "orc_")
        lib.orc_bandpass.argtypes = [C.POINTER(C.c_float), C.c_int, C.c_int, C.c_float, C.c_int, C.c_int, C.c_int,
                                     C.c_float, C.c_float, C.POINTER(C.c_float)]
        lib.orc_bandpass.restype = C.c_int
        lib.orc_butter_init.argtypes = [C.c_int, C.c_float, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        lib.orc_butter_init.restype = None

    def bandpass(self, traces, dt, phase, nphi, nplo, fhi, flo):
        """sfbandpass (butterworth_filter.c:127-200) of traces [nr][nt]."""
        x = _f32(traces)
        nr, nt = x.shape
        out = np.zeros_like(x)
        st = self.lib.orc_bandpass(_ptr(x, C.c_float), nt, nr, dt, int(phase), nphi, nplo, fhi, flo,
                                   _ptr(out, C.c_float))
        assert st == 0, st
        return out

    def butter_init(self, low, cutoff, nn):
        den = np.zeros(2 * ((nn + 1) // 2) + 2, np.float32)
        mid = C.c_float()
        self.lib.orc_butter_init(int(low), cutoff, nn, _ptr(den, C.c_float), C.byref(mid))
        return den[:2 * ((nn + 1) // 2)], mid.value


class RefAux(_AuxCalls):
    """The reference's own grad_precond_new5 / triangle2 / sfbandpass / XCORR1D
    from ``make ref`` (only where the reference sources are available)."""

    @classmethod
    def available(cls) -> bool:
        return os.path.isfile(os.path.join(REFDIR, "libfwiref.so"))

    def __init__(self):
        lib = C.CDLL(os.path.join(REFDIR, "libfwiref.so"))
        self._setup(lib, "ref_")
        lib.sfbandpass.argtypes = [C.POINTER(C.c_float), C.c_int, C.c_int, C.c_float, C.c_bool, C.c_int, C.c_int,
                                   C.c_float, C.c_float, C.POINTER(C.c_float)]
        lib.sfbandpass.restype = None

    def bandpass(self, traces, dt, phase, nphi, nplo, fhi, flo):
        x = _f32(traces).copy()
        nr, nt = x.shape
        out = np.zeros_like(x)
        self.lib.sfbandpass(_ptr(x, C.c_float), nt, nr, dt, bool(phase), nphi, nplo, fhi, flo, _ptr(out, C.c_float))
        return out


# ---------------------------------------------------------------------------
# L-BFGS driver of MBotOpt.c (fwi_oracle_lbfgs.c) and the reference run
# ---------------------------------------------------------------------------
LBFGS_DEFAULTS = dict(m=12, epsilon=1e-9, max_iterations=8, max_linesearch=6, ftol=1e-7, wolfe=0.98)  # lbfgs.h:77-79
MBOTOPT_N = 601 * 3921           # NZ * NX of the reference's Mpar.h, the size MBotOpt.c optimises


class LbfgsOracle:
    """orc_lbfgs_run: MBotOpt.c's L-BFGS on the objective of lbfgs_objective.h;
    twin "f32" reproduces the reference's float arithmetic, "f64" is the FP64
    oracle of the device optimizer."""

    def __init__(self, twin="f64"):
        self.twin = twin
        self.lib = lib = C.CDLL(os.path.join(BUILD, f"libfwioracle_lbfgs_{twin}.so"))
        lib.orc_lbfgs_run.argtypes = [C.c_long, C.c_int, C.c_double, C.c_int, C.c_int, C.c_double, C.c_double,
                                      C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_int)]
        lib.orc_lbfgs_run.restype = C.c_int
        real = C.c_float if twin == "f32" else C.c_double
        self._np = np.float32 if twin == "f32" else np.float64
        lib.orc_lbfgs_objective.argtypes = [C.c_long, C.POINTER(real), C.POINTER(real)]
        lib.orc_lbfgs_objective.restype = C.c_double
        self._real = real
        lib.orc_lbfgs_x0.argtypes = [C.c_long, C.POINTER(C.c_double)]

    def run(self, n, max_evals=200, **param):
        p = dict(LBFGS_DEFAULTS, **param)
        ft = np.zeros(max_evals)
        x = np.zeros(n)
        ne = C.c_int()
        ret = self.lib.orc_lbfgs_run(n, p["m"], p["epsilon"], p["max_iterations"], p["max_linesearch"], p["ftol"],
                                     p["wolfe"], max_evals, _ptr(ft, C.c_double), _ptr(x, C.c_double), C.byref(ne))
        return ret, ft[:min(ne.value, max_evals)], x

    def objective(self, x):
        x = np.ascontiguousarray(x, dtype=self._np)
        g = np.zeros_like(x)
        f = self.lib.orc_lbfgs_objective(len(x), _ptr(x, self._real), _ptr(g, self._real))
        return f, g

    def x0(self, n):
        x = np.zeros(n)
        self.lib.orc_lbfgs_x0(n, _ptr(x, C.c_double))
        return x


def run_reference_mbotopt(workdir):
    """Runs the reference's own MBotOpt.c (oracle/_ref/mbotopt, single rank,
    objective of lbfgs_objective.h) in workdir; returns (f trace, final x)."""
    exe = os.path.join(REFDIR, "mbotopt")
    trace = os.path.join(workdir, "trace.txt")
    env = dict(os.environ, ORC_LBFGS_TRACE=trace)
    subprocess.run([exe, "x"], cwd=workdir, env=env, check=True, stdout=subprocess.DEVNULL)
    return np.loadtxt(trace, ndmin=1), np.fromfile(trace + ".x", np.float32)
