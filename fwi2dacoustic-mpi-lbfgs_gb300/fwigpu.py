"""Python binding of the C ABI in ``include/fwi_gb300.h`` (ctypes).

This is the host-side mirror used by the tests and the benchmark; C callers
link ``libfwigpu.so`` directly.  Every method maps onto one ``fwi_*`` entry
point and raises :class:`FwiError` with the library's status and message
when the call fails.  Nothing here computes: if the library is missing or no
sm_103 device is present the constructor raises instead of falling back.

The call sequence mirrors one L-BFGS gradient evaluation of the reference
(MBotOpt.c:98-99): broadcast the model, then every shot's ``grad4_1shot``
(header.h:283) -- here one batched call over all shots.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
# FWI_LIB selects another build of the same ABI (the CPU emulation build used
# by the memory-safety tests); by default the sm_103a library is loaded.
LIB_PATH = os.environ.get("FWI_LIB", os.path.join(PKG, "libfwigpu.so"))

FWI_OK = 0
STATUS = {0: "FWI_OK", -1: "FWI_ERR_ARG", -2: "FWI_ERR_GEOMETRY", -3: "FWI_ERR_NOMEM", -4: "FWI_ERR_CUDA",
          -5: "FWI_ERR_STATE", -6: "FWI_ERR_CFL", -7: "FWI_ERR_NONFINITE", -8: "FWI_ERR_NODEVICE"}


class FwiConfig(C.Structure):
    _fields_ = [("nx", C.c_int), ("nz", C.c_int), ("dx", C.c_float), ("dz", C.c_float), ("dt", C.c_float),
                ("nt_max", C.c_int), ("npml", C.c_int), ("free_surface", C.c_int), ("jump", C.c_int),
                ("pml_max_f", C.c_float), ("pml_max_v", C.c_float), ("pml_coef_r", C.c_float),
                ("device", C.c_int), ("use_graph", C.c_int), ("plain_per_shot", C.c_int),
                ("store", C.c_int), ("snapshots", C.c_int), ("snap_precision", C.c_int),
                ("hbm_budget_mb", C.c_int), ("fd_order", C.c_int), ("reserved", C.c_int * 1)]


class FwiShot(C.Structure):
    _fields_ = [("nt", C.c_int), ("nr", C.c_int), ("src_x", C.c_float), ("src_z", C.c_float),
                ("rec_xz", C.POINTER(C.c_float)), ("wavelet", C.POINTER(C.c_float))]


class FwiStats(C.Structure):
    _fields_ = [("ms_forward", C.c_double), ("ms_backward", C.c_double), ("ms_misfit", C.c_double),
                ("ms_total", C.c_double), ("cell_steps", C.c_double), ("launches", C.c_longlong),
                ("device_bytes", C.c_longlong), ("store", C.c_int), ("segments", C.c_int),
                ("store_bytes", C.c_longlong)]


class FwiError(RuntimeError):
    def __init__(self, status: int, what: str):
        self.status = status
        super().__init__(f"{what}: {STATUS.get(status, status)}")


_LIB = None


def load_library(path: str = LIB_PATH) -> C.CDLL:
    """Load ``libfwigpu.so``; raises if it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.isfile(path):
        raise FileNotFoundError(f"{path} is missing: run fwi2dacoustic-mpi-lbfgs_gb300/build.py "
                                "(the engine has no CPU fallback)")
    lib = C.CDLL(path)
    P, I, F, D = C.c_void_p, C.c_int, C.c_float, C.c_double
    lib.fwi_create.restype = P
    lib.fwi_create.argtypes = [C.POINTER(FwiConfig), C.POINTER(I)]
    lib.fwi_destroy.argtypes = [P]
    lib.fwi_destroy.restype = None
    lib.fwi_set_model.argtypes = [P, C.POINTER(F)]
    lib.fwi_set_shots.argtypes = [P, I, C.POINTER(FwiShot)]
    lib.fwi_set_observed.argtypes = [P, C.POINTER(F)]
    lib.fwi_forward.argtypes = [P, C.POINTER(F)]
    lib.fwi_backward.argtypes = [P, C.POINTER(F), C.POINTER(D)]
    lib.fwi_gradient.argtypes = [P, C.POINTER(D), C.POINTER(D)]
    lib.fwi_gradient_obs.argtypes = [P, C.POINTER(F), C.POINTER(D), C.POINTER(D)]
    lib.fwi_gradient_f32.argtypes = [P, C.POINTER(D), C.POINTER(F)]
    lib.fwi_grad_device.argtypes = [P]
    lib.fwi_grad_device.restype = P
    lib.fwi_get_stats.argtypes = [P, C.POINTER(FwiStats)]
    lib.fwi_set_stream.argtypes = [P, P]
    lib.fwi_status_string.argtypes = [I]
    lib.fwi_status_string.restype = C.c_char_p
    lib.fwi_last_error.argtypes = [P]
    lib.fwi_last_error.restype = C.c_char_p
    lib.fwi_check_config.argtypes = [C.POINTER(FwiConfig)]
    lib.fwi_cpml_profile.argtypes = [I, F, F, F, F, F, C.POINTER(F), C.POINTER(F)]
    lib.fwi_fd_coefficients.argtypes = [F, F, C.POINTER(F)]
    lib.fwi_cell_of.argtypes = [F, F, F, F, C.POINTER(I), C.POINTER(I)]
    lib.fwi_set_misfit.argtypes = [P, C.POINTER(FwiMisfit)]
    lib.fwi_grad_precond.argtypes = [C.POINTER(F), I, I, F, I, I, I, I, F, C.POINTER(I)]
    lib.fwi_bandpass.argtypes = [C.POINTER(F), I, I, F, I, I, I, F, F, C.POINTER(F)]
    lib.fwi_xcorr1d.argtypes = [C.POINTER(F), C.POINTER(F), I, I, C.POINTER(F), F, F, I, C.POINTER(F), C.POINTER(F)]
    lib.fwi_lbfgs_create.argtypes = [C.c_longlong, C.POINTER(FwiLbfgsParam), C.POINTER(I)]
    lib.fwi_lbfgs_create.restype = P
    lib.fwi_lbfgs_destroy.argtypes = [P]
    lib.fwi_lbfgs_destroy.restype = None
    lib.fwi_lbfgs_begin.argtypes = [P, C.POINTER(D), D, P, I, C.POINTER(I)]
    lib.fwi_lbfgs_next.argtypes = [P, C.POINTER(D), D, P, I, C.POINTER(I)]
    lib.fwi_lbfgs_info.argtypes = [P, C.POINTER(I), C.POINTER(D), C.POINTER(I)]
    lib.fwi_set_tuning.argtypes = [P, C.POINTER(FwiTuning)]
    lib.fwi_get_tuning.argtypes = [P, C.POINTER(FwiTuning)]
    lib.fwi_time_steps.argtypes = [P, I, C.POINTER(D), C.POINTER(D)]
    _LIB = lib
    return lib


class FwiMisfit(C.Structure):
    """fwi_misfit (include/fwi_gb300.h)."""
    _fields_ = [("kind", C.c_int), ("slice", C.c_int), ("offset_min", C.c_float), ("offset_max", C.c_float),
                ("reserved", C.c_int * 4)]


class FwiTuning(C.Structure):
    """fwi_tuning (include/fwi_gb300.h): run-time launch choices, 0 = default."""
    _fields_ = [("x_first", C.c_int), ("z_first", C.c_int), ("fwd_gen_blocks", C.c_int), ("bwd_gen_blocks", C.c_int),
                ("fwd_int_blocks", C.c_int), ("bwd_int_blocks", C.c_int), ("class_order", C.c_int),
                ("serial", C.c_int), ("priority", C.c_int), ("gen_grid", C.c_int),
                ("bwd_zgen_blocks", C.c_int), ("reserved", C.c_int * 5)]
    KEYS = ("x_first", "z_first", "fwd_gen_blocks", "bwd_gen_blocks", "fwd_int_blocks", "bwd_int_blocks",
            "class_order", "serial", "priority", "gen_grid", "bwd_zgen_blocks")


class FwiLbfgsParam(C.Structure):
    """fwi_lbfgs_param (include/fwi_gb300.h); defaults of lbfgs.h:77-79."""
    _fields_ = [("m", C.c_int), ("epsilon", C.c_double), ("max_iterations", C.c_int), ("max_linesearch", C.c_int),
                ("ftol", C.c_double), ("wolfe", C.c_double)]


LBFGS_SUCCESS, LBFGS_MAXLINESEARCH, LBFGS_MAXITERATION, LBFGS_EVALUATE = 0, 1, 2, 3
MISFIT_L2, MISFIT_XCORR = 0, 1
XCORR_MIDDLE, XCORR_LEADING = 0, 1


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float)) if a is not None else None


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


STORE_AUTO, STORE_STRIPS, STORE_SNAPSHOTS = 0, 1, 2
SNAP_F32, SNAP_F16, SNAP_BF16 = 0, 1, 2
SNAP_PRECISION = {"f32": SNAP_F32, "f16": SNAP_F16, "bf16": SNAP_BF16}


def make_config(nx, nz, dx, dz, dt, nt_max, npml=20, free_surface=1, jump=1, pml_max_f=15.0,
                pml_max_v=6000.0, pml_coef_r=0.001, device=0, use_graph=0, plain_per_shot=0,
                store=STORE_AUTO, snapshots=0, snap_precision=SNAP_F32, hbm_budget_mb=0,
                fd_order=4) -> FwiConfig:
    """CPML defaults are MAX_F, MAX_V, COEF_R of fwi_sys.h:2-4.  ``store``:
    STORE_AUTO / STORE_STRIPS / STORE_SNAPSHOTS; ``snapshots``: segments of
    the checkpointed backward (0 = ceil(sqrt(nt))); ``snap_precision``:
    SNAP_F32 / SNAP_F16 / SNAP_BF16 (or "f32", "f16", "bf16"); ``fd_order``:
    4 (the reference's) or 8."""
    cfg = FwiConfig()
    cfg.nx, cfg.nz, cfg.dx, cfg.dz, cfg.dt = nx, nz, dx, dz, dt
    cfg.nt_max, cfg.npml, cfg.free_surface, cfg.jump = nt_max, npml, int(free_surface), jump
    cfg.pml_max_f, cfg.pml_max_v, cfg.pml_coef_r = pml_max_f, pml_max_v, pml_coef_r
    cfg.device, cfg.use_graph, cfg.plain_per_shot = device, use_graph, plain_per_shot
    cfg.store, cfg.snapshots, cfg.hbm_budget_mb = store, snapshots, hbm_budget_mb
    cfg.snap_precision = SNAP_PRECISION.get(snap_precision, snap_precision)
    cfg.fd_order = fd_order
    return cfg


class ShotSpec:
    """One shot in metres, as fwi_init reads it (sr_location file + wavelet)."""

    def __init__(self, src_x, src_z, rec_xz, wavelet):
        self.src_x, self.src_z = float(src_x), float(src_z)
        self.rec_xz = np.ascontiguousarray(rec_xz, np.float32).reshape(-1, 2)
        self.wavelet = np.ascontiguousarray(wavelet, np.float32)

    @property
    def nt(self):
        return len(self.wavelet)

    @property
    def nr(self):
        return len(self.rec_xz)

    def nt0(self, jump):
        return (self.nt - 1) // jump + 1


class Engine:
    """Owns one ``fwi_ctx``."""

    def __init__(self, cfg: FwiConfig):
        self.lib = load_library()
        st = C.c_int(0)
        self.cfg = cfg
        self.ctx = self.lib.fwi_create(C.byref(cfg), C.byref(st))
        if not self.ctx:
            raise FwiError(st.value, "fwi_create")
        self.shots: list[ShotSpec] = []
        self._keep = None

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.fwi_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st, what):
        if st != FWI_OK:
            msg = self.lib.fwi_last_error(self.ctx)
            raise FwiError(st, f"{what} ({msg.decode() if msg else ''})")

    @property
    def nsamples(self):
        return sum(s.nr * s.nt0(self.cfg.jump) for s in self.shots)

    def set_model(self, vel):
        vel = np.ascontiguousarray(vel, np.float32)
        assert vel.shape == (self.cfg.nz, self.cfg.nx), vel.shape
        self._check(self.lib.fwi_set_model(self.ctx, _fp(vel)), "fwi_set_model")

    def set_shots(self, shots):
        self.shots = list(shots)
        arr = (FwiShot * len(self.shots))()
        for a, s in zip(arr, self.shots):
            a.nt, a.nr, a.src_x, a.src_z = s.nt, s.nr, s.src_x, s.src_z
            a.rec_xz, a.wavelet = _fp(s.rec_xz), _fp(s.wavelet)
        self._check(self.lib.fwi_set_shots(self.ctx, len(self.shots), arr), "fwi_set_shots")

    def set_observed(self, obs):
        obs = np.ascontiguousarray(obs, np.float32).ravel()
        assert obs.size == self.nsamples, (obs.size, self.nsamples)
        self._check(self.lib.fwi_set_observed(self.ctx, _fp(obs)), "fwi_set_observed")

    def forward(self):
        syn = np.zeros(self.nsamples, np.float32)
        self._check(self.lib.fwi_forward(self.ctx, _fp(syn)), "fwi_forward")
        return syn

    def backward(self, residual):
        res = np.ascontiguousarray(residual, np.float32).ravel()
        grad = np.zeros((self.cfg.nz, self.cfg.nx), np.float64)
        self._check(self.lib.fwi_backward(self.ctx, _fp(res), _dp(grad)), "fwi_backward")
        return grad

    def gradient(self, keep_on_device=False, out=None, observed=None):
        """Misfit and dJ/dv.  ``out`` (float64 [nz][nx], e.g. pinned memory)
        receives the gradient; ``keep_on_device`` leaves it on the device.
        ``observed`` (the traces of set_observed, best in pinned memory) sets
        the observed traces in the same call, uploaded beside the forward
        phase (fwi_gradient_obs)."""
        mis = np.zeros(2, np.float64)
        grad = None
        if not keep_on_device:
            grad = out if out is not None else np.zeros((self.cfg.nz, self.cfg.nx), np.float64)
            assert grad.dtype == np.float64 and grad.size == self.cfg.nz * self.cfg.nx and grad.flags.c_contiguous
        if observed is None:
            self._check(self.lib.fwi_gradient(self.ctx, _dp(mis), _dp(grad)), "fwi_gradient")
        else:
            obs = np.ascontiguousarray(observed, np.float32).ravel()
            assert obs.size == self.nsamples, (obs.size, self.nsamples)
            self._check(self.lib.fwi_gradient_obs(self.ctx, _fp(obs), _dp(mis), _dp(grad)), "fwi_gradient_obs")
        return float(mis[1]), grad

    def grad_device_ptr(self) -> int:
        return int(self.lib.fwi_grad_device(self.ctx) or 0)

    def gradient_f32(self):
        mis = np.zeros(2, np.float64)
        grad = np.zeros((self.cfg.nz, self.cfg.nx), np.float32)
        self._check(self.lib.fwi_gradient_f32(self.ctx, _dp(mis), _fp(grad)), "fwi_gradient_f32")
        return float(mis[1]), grad

    def set_misfit(self, kind=MISFIT_L2, slice=XCORR_MIDDLE, offset_min=0.0, offset_max=1.0e30):
        """Misfit of gradient(): MISFIT_L2 (default) or MISFIT_XCORR (XCORR1D,
        slice XCORR_MIDDLE / XCORR_LEADING, traces outside [offset_min,
        offset_max] metres skipped)."""
        m = FwiMisfit(kind, slice, offset_min, offset_max)
        self._check(self.lib.fwi_set_misfit(self.ctx, C.byref(m)), "fwi_set_misfit")

    def set_stream(self, stream_ptr):
        """Run on the caller's cudaStream_t (an int handle, e.g. torch's
        ``torch.cuda.current_stream().cuda_stream``); None restores the own stream."""
        self._check(self.lib.fwi_set_stream(self.ctx, C.c_void_p(stream_ptr) if stream_ptr else None),
                    "fwi_set_stream")

    def set_tuning(self, tuning: dict):
        """fwi_set_tuning from a dict of FwiTuning fields (missing or 0 = default).
        Changing x_first / z_first discards the shots and the model."""
        t = FwiTuning()
        for k, v in tuning.items():
            setattr(t, k, int(v))
        relayout = any(tuning.get(k, 0) and tuning.get(k) != self.tuning()[k] for k in ("x_first", "z_first"))
        self._check(self.lib.fwi_set_tuning(self.ctx, C.byref(t)), "fwi_set_tuning")
        if relayout:
            self.shots = []

    def tuning(self) -> dict:
        t = FwiTuning()
        self._check(self.lib.fwi_get_tuning(self.ctx, C.byref(t)), "fwi_get_tuning")
        return {k: getattr(t, k) for k in FwiTuning.KEYS}

    def time_steps(self, steps: int):
        """(ms per forward step, ms per backward step) of the current batch."""
        f, b = C.c_double(), C.c_double()
        self._check(self.lib.fwi_time_steps(self.ctx, int(steps), C.byref(f), C.byref(b)), "fwi_time_steps")
        return f.value, b.value

    def stats(self) -> dict:
        s = FwiStats()
        self._check(self.lib.fwi_get_stats(self.ctx, C.byref(s)), "fwi_get_stats")
        return {k: getattr(s, k) for k, _ in FwiStats._fields_}

    def split(self, flat):
        """Split a flat trace vector into per-shot [nr][nt0] arrays."""
        out, o = [], 0
        for s in self.shots:
            n = s.nr * s.nt0(self.cfg.jump)
            out.append(np.asarray(flat[o:o + n]).reshape(s.nr, s.nt0(self.cfg.jump)))
            o += n
        return out


# ---- routines around the gradient (standalone, on the current device) ---------

def _check_status(st, what):
    if st != FWI_OK:
        raise FwiError(st, what)


def grad_precond(body, perc, rectx1, repeat1, rectx2, repeat2, alpha_grad, bottom):
    """grad_precond_new5 (grad_prec.c:5-52) of a float32 gradient [mnz][mnx];
    returns a new array."""
    lib = load_library()
    out = np.ascontiguousarray(body, dtype=np.float32).copy()
    mnz, mnx = out.shape
    bot = np.ascontiguousarray(bottom, dtype=np.int32)
    if bot.shape != (mnx,):
        raise ValueError("bottom must have one entry per column")
    _check_status(lib.fwi_grad_precond(_fp(out), mnx, mnz, perc, rectx1, repeat1, rectx2, repeat2, alpha_grad,
                                       bot.ctypes.data_as(C.POINTER(C.c_int))), "fwi_grad_precond")
    return out


def bandpass(traces, dt, phase, nphi, nplo, fhi, flo):
    """sfbandpass (butterworth_filter.c:127-200) of float32 traces [nr][nt]."""
    lib = load_library()
    x = np.ascontiguousarray(traces, dtype=np.float32)
    nr, nt = x.shape
    out = np.zeros_like(x)
    _check_status(lib.fwi_bandpass(_fp(x), nt, nr, dt, int(phase), nphi, nplo, fhi, flo, _fp(out)), "fwi_bandpass")
    return out


def xcorr1d(obs, syn, sr_xyz, offset_min, offset_max, slice=XCORR_MIDDLE):
    """XCORR1D (xcorr_msf.c:4-181) of float32 traces [nr][nt]; returns
    (misfit[2], res[nr][nt])."""
    lib = load_library()
    o = np.ascontiguousarray(obs, dtype=np.float32)
    sy = np.ascontiguousarray(syn, dtype=np.float32)
    sr = np.ascontiguousarray(sr_xyz, dtype=np.float32)
    nr, nt = o.shape
    mis = np.zeros(2, np.float32)
    res = np.zeros_like(o)
    _check_status(lib.fwi_xcorr1d(_fp(o), _fp(sy), nr, nt, _fp(sr), offset_min, offset_max, slice, _fp(mis),
                                  _fp(res)), "fwi_xcorr1d")
    return mis, res


class Lbfgs:
    """The device L-BFGS optimizer (MBotOpt.c:55-214, FP64) with reverse
    communication::

        opt = Lbfgs(n)
        x = x0.copy(); f, g = evaluate(x)
        state = opt.begin(x, f, g)            # x now holds the first trial point
        while state == LBFGS_EVALUATE:
            f, g = evaluate(x)
            state = opt.next(x, f, g)         # next trial point, or the final point

    g is a float64 host array, or an int device pointer (e.g.
    Engine.grad_device_ptr()) of n float64 values."""

    def __init__(self, n, m=12, epsilon=1e-9, max_iterations=8, max_linesearch=6, ftol=1e-7, wolfe=0.98):
        self.lib = load_library()
        self.n = int(n)
        p = FwiLbfgsParam(m, epsilon, max_iterations, max_linesearch, ftol, wolfe)
        st = C.c_int(0)
        self.h = self.lib.fwi_lbfgs_create(self.n, C.byref(p), C.byref(st))
        if not self.h:
            raise FwiError(st.value, "fwi_lbfgs_create")

    def close(self):
        if self.h:
            self.lib.fwi_lbfgs_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _call(self, fn, x, f, g):
        if x.dtype != np.float64 or not x.flags.c_contiguous or x.size != self.n:
            raise ValueError("x must be a contiguous float64 array of n values")
        if isinstance(g, int):
            gp, dev = C.c_void_p(g), 1
        else:
            g = np.ascontiguousarray(g, dtype=np.float64)
            gp, dev = C.c_void_p(g.ctypes.data), 0
        state = C.c_int(-1)
        _check_status(fn(self.h, _dp(x), float(f), gp, dev, C.byref(state)), fn.__name__)
        return state.value

    def begin(self, x, f, g):
        return self._call(self.lib.fwi_lbfgs_begin, x, f, g)

    def next(self, x, f, g):
        return self._call(self.lib.fwi_lbfgs_next, x, f, g)

    def info(self):
        k, ne, step = C.c_int(), C.c_int(), C.c_double()
        _check_status(self.lib.fwi_lbfgs_info(self.h, C.byref(k), C.byref(step), C.byref(ne)), "fwi_lbfgs_info")
        return {"iteration": k.value, "step": step.value, "evaluations": ne.value}


# ---- host-only helpers (no device needed) ----------------------------------------

def cpml_profile(npml, d, dt, max_f=15.0, max_v=6000.0, coef_r=0.001):
    lib = load_library()
    a = np.zeros(2 * npml + 1, np.float32)
    b = np.zeros(2 * npml + 1, np.float32)
    st = lib.fwi_cpml_profile(npml, d, dt, max_f, max_v, coef_r, _fp(a), _fp(b))
    if st:
        raise FwiError(st, "fwi_cpml_profile")
    return a, b


def fd_coefficients(dx, dz):
    lib = load_library()
    out = np.zeros(8, np.float32)
    st = lib.fwi_fd_coefficients(dx, dz, _fp(out))
    if st:
        raise FwiError(st, "fwi_fd_coefficients")
    return out


def cell_of(x, z, dx, dz):
    lib = load_library()
    ix, iz = C.c_int(), C.c_int()
    st = lib.fwi_cell_of(x, z, dx, dz, C.byref(ix), C.byref(iz))
    if st:
        raise FwiError(st, "fwi_cell_of")
    return ix.value, iz.value


def check_config(cfg: FwiConfig) -> int:
    return load_library().fwi_check_config(C.byref(cfg))
