"""Python binding of the GB300 MEMD engine's C ABI (ctypes over libmemd_gb300.so).

The library is the product; this module only marshals arguments: device
buffers are torch CUDA tensors (or raw device pointers), host buffers numpy
arrays.  There is no CPU fallback: if the shared library is missing the import
fails, and running without a GPU raises the CUDA error the library reports.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "lib", "libmemd_gb300.so")
# the bounds-checked build of the same library (index checks report
# FLAG_CHECK_FAILED instead of touching memory out of bounds; for tests)
LIB_CHECKED_PATH = os.path.join(PKG, "lib", "libmemd_gb300_checked.so")

MEMD_OK = 0
MEMD_ERR_INVALID = 1
MEMD_ERR_CUDA = 2
MEMD_ERR_NOMEM = 3
MEMD_ERR_COORD = 4
MEMD_ERR_PRECISION = 5
MEMD_ERR_UNSUPPORTED = 6

PREC_F64, PREC_F32, PREC_MIXED = 0, 1, 2
STOP_FIXED, STOP_CRITERION = 0, 1
SPLINE_NATURAL, SPLINE_NOT_A_KNOT = 0, 1
BOUNDARY_REFERENCE, BOUNDARY_MIRROR = 0, 1
FLAG_NO_QUALIFIED_DIRECTION = 1
FLAG_KNOT_OVERFLOW = 2
FLAG_DEVICE_TIMEOUT = 4
FLAG_CHECK_FAILED = 8
PROJ_AUTO, PROJ_CUDA_CORES = 0, 1

TRACE_DTYPE = np.dtype([("count", "<i4"), ("flags", "<i4"), ("hash", "<u8")])

# every symbol include/memd_gb300.h and include/memd_synth.h declare
EXPORTS = [
    "memd_default_config", "memd_plan_create", "memd_plan_create_tuned", "memd_plan_get_tuning",
    "memd_plan_destroy", "memd_plan_workspace_bytes",
    "memd_plan_set_trace", "memd_run_f64", "memd_run_f32", "memd_run_batched_f64",
    "memd_run_batched_f32", "memd_batched_counts", "memd_profile_f64", "memd_profile_f32", "memd_profile_batched_f64",
    "memd_profile_batched_f32", "memd_directions_f64", "memd_directions_f32", "memd_directions_noalloc_f64", "memd_diag_fma_rate", "memd_diag_wait_timeout", "memd_last_error",
    "memd_version", "memd_synth_tones", "memd_synth_eeg", "memd_write_bin", "memd_bin_count",
    "memd_read_bin",
]


class MemdError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"memd status {status}: {msg}")
        self.status = status


class Config(ctypes.Structure):
    _fields_ = [
        ("channels", ctypes.c_int64),
        ("length", ctypes.c_int64),
        ("directions", ctypes.c_int64),
        ("num_imfs", ctypes.c_int64),
        ("max_iter", ctypes.c_int64),
        ("precision", ctypes.c_int32),
        ("stop_mode", ctypes.c_int32),
        ("stop_sd", ctypes.c_double),
        ("stop_sd2", ctypes.c_double),
        ("stop_tol", ctypes.c_double),
        ("ref_window", ctypes.c_int32),
        ("dir_chunk", ctypes.c_int32),
        ("solve_window", ctypes.c_int32),
        ("max_epochs", ctypes.c_int32),
        ("mean_eval", ctypes.c_int32),
        ("spline_end", ctypes.c_int32),
        ("boundary", ctypes.c_int32),
        ("projection", ctypes.c_int32),
        ("reserved", ctypes.c_int64 * 2),
    ]


class Tuning(ctypes.Structure):
    """Launch shapes of a plan (memd_tuning); 0 = the default."""
    _fields_ = [
        ("solve_segment", ctypes.c_int32),
        ("solve_min_segment", ctypes.c_int32),
        ("factor_segment", ctypes.c_int32),
        ("solve_queue", ctypes.c_int32),
        ("mean_ctas", ctypes.c_int32),
        ("proj_tile_n", ctypes.c_int32),
        ("solve_layout", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 9),
    ]
    KEYS = ("solve_segment", "solve_min_segment", "factor_segment", "solve_queue", "mean_ctas", "proj_tile_n",
            "solve_layout")

    def as_dict(self):
        return {k: int(getattr(self, k)) for k in self.KEYS}

    @classmethod
    def from_dict(cls, d):
        t = cls()
        for k, v in (d or {}).items():
            if k in cls.KEYS:
                setattr(t, k, int(v))
        return t


class Stats(ctypes.Structure):
    _fields_ = [
        ("n_imfs", ctypes.c_int32),
        ("flags", ctypes.c_int32),
        ("elapsed_ms", ctypes.c_double),
        ("launches", ctypes.c_int64),
        ("sifts", ctypes.c_int32 * 64),
        ("refined", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


STAGES = ("project", "compact", "factor", "solve", "eval", "other")


class Profile(ctypes.Structure):
    _fields_ = [("ms", ctypes.c_double * 8), ("launches", ctypes.c_int64 * 8)]

    def as_dict(self):
        return {name: {"ms": self.ms[i], "launches": int(self.launches[i])} for i, name in enumerate(STAGES)}


_lib = None
_lib_checked = None


def lib():
    global _lib
    if _lib is None:
        _lib = _load(LIB_PATH)
    return _lib


def checked_lib():
    """The bounds-checked build, bound like lib() (its own plans and state)."""
    global _lib_checked
    if _lib_checked is None:
        _lib_checked = _load(LIB_CHECKED_PATH)
    return _lib_checked


def _load(path):
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: run __graft_entry__.build() (nvcc, sm_103a)")
    L = ctypes.CDLL(path)
    vp, i64, i32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32
    L.memd_default_config.argtypes = [ctypes.POINTER(Config)]
    L.memd_default_config.restype = None
    L.memd_plan_create.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(vp)]
    L.memd_plan_create.restype = ctypes.c_int
    L.memd_plan_create_tuned.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(Tuning), ctypes.POINTER(vp)]
    L.memd_plan_create_tuned.restype = ctypes.c_int
    L.memd_plan_get_tuning.argtypes = [vp, ctypes.POINTER(Tuning)]
    L.memd_plan_get_tuning.restype = ctypes.c_int
    L.memd_plan_destroy.argtypes = [vp]
    L.memd_plan_destroy.restype = ctypes.c_int
    L.memd_plan_workspace_bytes.argtypes = [vp]
    L.memd_plan_workspace_bytes.restype = ctypes.c_size_t
    L.memd_plan_set_trace.argtypes = [vp, vp]
    L.memd_plan_set_trace.restype = ctypes.c_int
    for name in ("memd_run_f64", "memd_run_f32"):
        f = getattr(L, name)
        f.argtypes = [vp, vp, vp, vp, vp, vp, ctypes.POINTER(Stats)]
        f.restype = ctypes.c_int
    for name in ("memd_run_batched_f64", "memd_run_batched_f32"):
        f = getattr(L, name)
        f.argtypes = [vp, i32, vp, vp, vp, vp, vp, vp, ctypes.POINTER(Stats)]
        f.restype = ctypes.c_int
    L.memd_batched_counts.argtypes = [vp, i32, vp, vp]
    L.memd_batched_counts.restype = ctypes.c_int
    for name in ("memd_profile_f64", "memd_profile_f32"):
        f = getattr(L, name)
        f.argtypes = [vp, vp, vp, vp, vp, ctypes.POINTER(Profile)]
        f.restype = ctypes.c_int
    for name in ("memd_profile_batched_f64", "memd_profile_batched_f32"):
        f = getattr(L, name)
        f.argtypes = [vp, i32, vp, vp, vp, vp, vp, vp, ctypes.POINTER(Profile)]
        f.restype = ctypes.c_int
    for name in ("memd_directions_f64", "memd_directions_f32", "memd_directions_noalloc_f64"):
        f = getattr(L, name)
        f.argtypes = [i64, i64, vp, vp, vp]
        f.restype = ctypes.c_int
    L.memd_diag_fma_rate.argtypes = [i32, ctypes.POINTER(ctypes.c_double)]
    L.memd_diag_fma_rate.restype = ctypes.c_int
    L.memd_diag_wait_timeout.argtypes = [i64, ctypes.POINTER(ctypes.c_int32)]
    L.memd_diag_wait_timeout.restype = ctypes.c_int
    L.memd_last_error.argtypes = []
    L.memd_last_error.restype = ctypes.c_char_p
    L.memd_version.argtypes = []
    L.memd_version.restype = ctypes.c_char_p
    for name in ("memd_synth_tones", "memd_synth_eeg"):
        f = getattr(L, name)
        f.argtypes = [i64, i64, ctypes.c_double, ctypes.c_uint64, vp]
        f.restype = ctypes.c_int
    L.memd_write_bin.argtypes = [ctypes.c_char_p, vp, i64, i32]
    L.memd_write_bin.restype = ctypes.c_int
    L.memd_bin_count.argtypes = [ctypes.c_char_p, i32]
    L.memd_bin_count.restype = i64
    L.memd_read_bin.argtypes = [ctypes.c_char_p, vp, i64, i32]
    L.memd_read_bin.restype = ctypes.c_int
    return L


def _check(status: int, L=None):
    if status != MEMD_OK:
        raise MemdError(status, (L or lib()).memd_last_error().decode())


def last_error() -> str:
    return lib().memd_last_error().decode()


def default_config(**kw) -> Config:
    c = Config()
    lib().memd_default_config(ctypes.byref(c))
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def _dptr(t) -> int | None:
    """Device pointer of a torch tensor (or an int address, or None)."""
    if t is None:
        return None
    if isinstance(t, int):
        return t
    return t.data_ptr()


def _stream_ptr(stream) -> int | None:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


class Plan:
    """Owns a memd_plan: all device buffers of one decomposition shape."""

    def __init__(self, channels: int, length: int, directions: int, num_imfs: int = 9,
                 max_iter: int = 10, precision: int = PREC_F64, tuning=None, library=None, **kw):
        """tuning: None (defaults), a dict / Tuning of launch shapes, or "auto"
        (the autotuner's stored choice for this shape, if there is one).
        library: the bound library (lib() by default; checked_lib() for the
        bounds-checked build)."""
        self._L = library or lib()
        self._chk = lambda status: _check(status, self._L)
        self.cfg = default_config(channels=channels, length=length, directions=directions,
                                  num_imfs=num_imfs, max_iter=max_iter, precision=precision, **kw)
        if isinstance(tuning, str):
            if tuning != "auto":
                raise ValueError("tuning must be None, a dict, a Tuning or 'auto'")
            import memd_autotune

            tuning = memd_autotune.lookup(self.cfg)
        t = tuning if isinstance(tuning, Tuning) else Tuning.from_dict(tuning)
        h = ctypes.c_void_p()
        self._chk(self._L.memd_plan_create_tuned(ctypes.byref(self.cfg), ctypes.byref(t), ctypes.byref(h)))
        self.handle = h
        self._trace = None

    def tuning(self) -> dict:
        """The launch shapes the plan uses (defaults filled in)."""
        t = Tuning()
        self._chk(self._L.memd_plan_get_tuning(self.handle, ctypes.byref(t)))
        return t.as_dict()

    @property
    def workspace_bytes(self) -> int:
        return int(self._L.memd_plan_workspace_bytes(self.handle))

    def set_trace(self, enable: bool = True):
        if enable:
            n = self.cfg.num_imfs * (self.cfg.max_iter + 1) * self.cfg.directions * 2
            self._trace = np.zeros(n, dtype=TRACE_DTYPE)
            self._chk(self._L.memd_plan_set_trace(self.handle, self._trace.ctypes.data_as(ctypes.c_void_p)))
        else:
            self._trace = None
            self._chk(self._L.memd_plan_set_trace(self.handle, None))

    def trace(self):
        if self._trace is None:
            return None
        return self._trace.reshape(self.cfg.num_imfs, self.cfg.max_iter + 1, self.cfg.directions, 2)

    def run(self, y, dirs, imfs, x=None, stream=None, stats: bool = True):
        """y: (C, L) device tensor, dirs: (K, C), imfs: (num_imfs, C, L); same dtype."""
        st = Stats()
        fn = self._L.memd_run_f64 if self.cfg.precision == PREC_F64 else self._L.memd_run_f32
        self._chk(fn(self.handle, _dptr(x), _dptr(y), _dptr(dirs), _dptr(imfs), _stream_ptr(stream),
                  ctypes.byref(st) if stats else None))
        return st if stats else None

    def run_batched(self, y, lengths, offsets, dirs, imfs, stream=None, stats: bool = True):
        """Batched plan (max_epochs > 0): epoch e is y[offsets[e] : offsets[e] + C*lengths[e]]
        (C x lengths[e], channel-major) of the 1-D device tensor y; its IMFs go to
        imfs[num_imfs*offsets[e] : ...] (num_imfs x C x lengths[e])."""
        n = len(lengths)
        la = (ctypes.c_int64 * n)(*[int(v) for v in lengths])
        oa = (ctypes.c_int64 * n)(*[int(v) for v in offsets])
        st = Stats()
        fn = self._L.memd_run_batched_f64 if self.cfg.precision == PREC_F64 else self._L.memd_run_batched_f32
        self._chk(fn(self.handle, n, ctypes.cast(la, ctypes.c_void_p), ctypes.cast(oa, ctypes.c_void_p), _dptr(y),
                  _dptr(dirs), _dptr(imfs), _stream_ptr(stream),
                  ctypes.byref(st) if stats else None))
        return st if stats else None

    def batched_counts(self, n_epochs: int):
        """Stop mode, batched: (IMFs per epoch, sifts per IMF and epoch [n, 64])
        of the last run_batched (call after its stream is synchronised)."""
        import numpy as np

        ni = np.zeros(n_epochs, dtype=np.int32)
        sf = np.zeros((n_epochs, 64), dtype=np.int32)
        self._chk(self._L.memd_batched_counts(self.handle, int(n_epochs), ni.ctypes.data_as(ctypes.c_void_p),
                                              sf.ctypes.data_as(ctypes.c_void_p)))
        return ni, sf

    def profile_batched(self, y, lengths, offsets, dirs, imfs, stream=None) -> Profile:
        """Batched run with every kernel timed by CUDA events (per-stage ms)."""
        n = len(lengths)
        la = (ctypes.c_int64 * n)(*[int(v) for v in lengths])
        oa = (ctypes.c_int64 * n)(*[int(v) for v in offsets])
        pr = Profile()
        fn = self._L.memd_profile_batched_f64 if self.cfg.precision == PREC_F64 else self._L.memd_profile_batched_f32
        self._chk(fn(self.handle, n, ctypes.cast(la, ctypes.c_void_p), ctypes.cast(oa, ctypes.c_void_p), _dptr(y),
                  _dptr(dirs), _dptr(imfs), _stream_ptr(stream), ctypes.byref(pr)))
        return pr

    def profile(self, y, dirs, imfs, stream=None) -> Profile:
        """Eager run with every kernel timed by CUDA events (per-stage ms)."""
        pr = Profile()
        fn = self._L.memd_profile_f64 if self.cfg.precision == PREC_F64 else self._L.memd_profile_f32
        self._chk(fn(self.handle, _dptr(y), _dptr(dirs), _dptr(imfs), _stream_ptr(stream), ctypes.byref(pr)))
        return pr

    def close(self):
        if getattr(self, "handle", None):
            self._L.memd_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def directions(C: int, K: int, primes=None, dtype: str = "f64", out=None, stream=None):
    """Direction set (K, C) on the GPU.  out: preallocated torch CUDA tensor."""
    import torch

    tdt = torch.float64 if dtype == "f64" else torch.float32
    if out is None:
        out = torch.empty((K, C), dtype=tdt, device="cuda")
    pr = None
    if primes is not None:
        pr = np.ascontiguousarray(primes, dtype=np.int32)
    fn = lib().memd_directions_f64 if dtype == "f64" else lib().memd_directions_f32
    _check(fn(C, K, None if pr is None else pr.ctypes.data_as(ctypes.c_void_p), _dptr(out), _stream_ptr(stream)))
    return out


def fma_rate(precision: int) -> float:
    """Measured fma throughput of the current GPU in flop/s (fma = 2 flops)."""
    v = ctypes.c_double()
    _check(lib().memd_diag_fma_rate(precision, ctypes.byref(v)))
    return v.value


def wait_timeout_flags(max_clocks: int) -> int:
    """Run the bounded-wait diagnostic (a wait nothing completes); returns the
    run-state flags it set."""
    v = ctypes.c_int32()
    _check(lib().memd_diag_wait_timeout(int(max_clocks), ctypes.byref(v)))
    return int(v.value)


def synth_eeg(C: int, L: int, fs: float = 256.0, seed: int = 0) -> np.ndarray:
    out = np.zeros((C, L), dtype=np.float64)
    rc = lib().memd_synth_eeg(C, L, fs, seed, out.ctypes.data_as(ctypes.c_void_p))
    if rc != 0:
        raise ValueError(f"memd_synth_eeg rc={rc}")
    return out


def synth_tones(C: int, L: int, fs: float = 1000.0, seed: int = 0) -> np.ndarray:
    out = np.zeros((C, L), dtype=np.float64)
    rc = lib().memd_synth_tones(C, L, fs, seed, out.ctypes.data_as(ctypes.c_void_p))
    if rc != 0:
        raise ValueError(f"memd_synth_tones rc={rc}")
    return out
