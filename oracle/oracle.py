"""ctypes front end of the CPU oracle (oracle/memd_oracle.c).

TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and the
cpu_baseline leg of bench.py as the checker / CPU baseline.  The product path
(the CUDA library and its C ABI) never imports this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

TRACE_DTYPE = np.dtype([("count", "<i4"), ("flags", "<i4"), ("hash", "<u8")])


class OracleOpts(ctypes.Structure):
    _fields_ = [
        ("ref_window", ctypes.c_int32),
        ("stop_mode", ctypes.c_int32),
        ("sd", ctypes.c_double),
        ("sd2", ctypes.c_double),
        ("tol", ctypes.c_double),
        ("nthreads", ctypes.c_int32),
        ("spline_end", ctypes.c_int32),
        ("boundary", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


def build(force: bool = False) -> str:
    """Compile liboracle.so next to its source (gcc, OpenMP, no fp contraction)."""
    src = os.path.join(HERE, "memd_oracle.c")
    hdr = os.path.join(HERE, "memd_oracle_impl.h")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB_PATH
    cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", LIB_PATH, src, "-lm"]
    subprocess.check_call(cmd)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        i64, i32p = ctypes.c_int64, ctypes.POINTER(ctypes.c_int32)
        vp = ctypes.c_void_p
        for sfx in ("f64", "f32"):
            f = getattr(L, "oracle_memd_" + sfx)
            f.argtypes = [i64, i64, i64, i64, i64, vp, vp, vp, ctypes.POINTER(OracleOpts), vp, vp, vp]
            f.restype = ctypes.c_int
            g = getattr(L, "oracle_directions_" + sfx)
            g.argtypes = [i64, i64, vp, vp]
            g.restype = ctypes.c_int
        L.oracle_envelope_f64.argtypes = [vp, vp, i64, i64, vp, ctypes.c_int32]
        L.oracle_envelope_f64.restype = ctypes.c_int
        L.oracle_mirror_f64.argtypes = [vp, i64, vp, i64, vp, i64, vp]
        L.oracle_mirror_f64.restype = ctypes.c_int
        L.oracle_window_cover.argtypes = [i64]
        L.oracle_window_cover.restype = i64
        L.oracle_radical_inverse.argtypes = [ctypes.c_int32, ctypes.c_uint32]
        L.oracle_radical_inverse.restype = ctypes.c_float
        L.oracle_prime_table.argtypes = [i64, i64, i32p]
        L.oracle_prime_table.restype = None
        L.oracle_max_threads.argtypes = []
        L.oracle_max_threads.restype = ctypes.c_int
        L.oracle_knot_hash.argtypes = [vp, i64]
        L.oracle_knot_hash.restype = ctypes.c_uint64
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def window_cover(L: int) -> int:
    return int(lib().oracle_window_cover(L))


def knot_hash(pos) -> int:
    p = np.ascontiguousarray(pos, dtype=np.int32)
    return int(lib().oracle_knot_hash(_ptr(p), p.size))


def directions(C: int, K: int, primes=None, dtype=np.float64) -> np.ndarray:
    """K x C direction vectors; primes=None -> standalone convention."""
    out = np.zeros((K, C), dtype=dtype)
    pr = None if primes is None else np.ascontiguousarray(primes, dtype=np.int32)
    fn = lib().oracle_directions_f64 if dtype == np.float64 else lib().oracle_directions_f32
    rc = fn(C, K, None if pr is None else _ptr(pr), _ptr(out))
    if rc != 0:
        raise RuntimeError(f"oracle_directions failed rc={rc}")
    return out


def envelope(pos, val, L: int, nak: bool = False) -> np.ndarray:
    """Spline through (pos, val) evaluated at 0..L-1; nak: not-a-knot ends."""
    p = np.ascontiguousarray(pos, dtype=np.int32)
    v = np.ascontiguousarray(val, dtype=np.float64)
    out = np.zeros(L, dtype=np.float64)
    rc = lib().oracle_envelope_f64(_ptr(p), _ptr(v), p.size, L, _ptr(out), int(nak))
    if rc != 0:
        raise RuntimeError(f"oracle_envelope failed rc={rc}")
    return out


def mirror(P, imax, imin) -> dict:
    """Mirrored end knots of one projection P with interior extrema imax, imin.
    Returns lsym, rsym and per envelope (0 = maxima) the left / right source
    samples in ascending order of mirrored position."""
    P = np.ascontiguousarray(P, dtype=np.float64)
    a = np.ascontiguousarray(imax, dtype=np.int32)
    b = np.ascontiguousarray(imin, dtype=np.int32)
    out = np.zeros(22, dtype=np.int32)
    rc = lib().oracle_mirror_f64(_ptr(P), P.size, _ptr(a), a.size, _ptr(b), b.size, _ptr(out))
    if rc != 0:
        raise RuntimeError(f"oracle_mirror failed rc={rc}")
    nl, nr = out[2:4], out[4:6]
    return {"lsym": int(out[0]), "rsym": int(out[1]),
            "left": [list(out[6 + 4 * e: 6 + 4 * e + nl[e]]) for e in range(2)],
            "right": [list(out[14 + 4 * e: 14 + 4 * e + nr[e]]) for e in range(2)]}


def memd(y: np.ndarray, dirs: np.ndarray, num_imfs: int, max_iter: int, *,
         ref_window: bool = True, stop_mode: bool = False, sd=0.075, sd2=0.75, tol=0.075,
         nthreads: int | None = None, trace: bool = False, spline_end: int = 0, boundary: int = 0):
    """Run the oracle.  y: C x L (channel-major), dirs: K x C.  Returns
    (imfs[num_imfs, C, L], info dict with sifts / n_imfs / trace)."""
    dtype = y.dtype
    if dtype not in (np.float64, np.float32):
        raise TypeError("y must be float64 or float32")
    y = np.ascontiguousarray(y)
    dirs = np.ascontiguousarray(dirs, dtype=dtype)
    C, L = y.shape
    K = dirs.shape[0]
    assert dirs.shape == (K, C)
    imfs = np.zeros((num_imfs, C, L), dtype=dtype)
    o = OracleOpts(int(ref_window), int(stop_mode), sd, sd2, tol,
                   nthreads if nthreads else max_threads(), int(spline_end), int(boundary), 0)
    tr = np.zeros(num_imfs * (max_iter + 1) * K * 2, dtype=TRACE_DTYPE) if trace else None
    sifts = np.zeros(num_imfs, dtype=np.int32)
    nimf = np.zeros(1, dtype=np.int32)
    fn = lib().oracle_memd_f64 if dtype == np.float64 else lib().oracle_memd_f32
    rc = fn(C, L, K, num_imfs, max_iter, _ptr(y), _ptr(dirs), _ptr(imfs), ctypes.byref(o),
            None if tr is None else _ptr(tr), _ptr(sifts), _ptr(nimf))
    if rc != 0:
        raise RuntimeError(f"oracle_memd failed rc={rc}")
    info = {"sifts": sifts, "n_imfs": int(nimf[0])}
    if trace:
        info["trace"] = tr.reshape(num_imfs, max_iter + 1, K, 2)
    return imfs, info
