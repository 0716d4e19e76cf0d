"""Drop-in entry points above the C ABI: the reference's template functions
(include/memd_reference.hpp, exercised by the sample_synthetic_signal driver),
the .bin command-line tool, and the MATLAB MEX entry (run through a stub of the
mex/mxGPU API with the reference MEX's eight inputs)."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import memd_gb300 as mg
import oracle

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(REPO, "memd-gpu_gb300", "bin")
STUB = os.path.join(REPO, "memd-gpu_gb300", "lib", "libmemd_mex_stub.so")


def test_tools_built_and_cli_usage():
    for name in ("sample_synthetic_signal", "memd_cli", "memd_sweep"):
        assert os.access(os.path.join(BIN, name), os.X_OK), name
    r = subprocess.run([os.path.join(BIN, "memd_cli"), "--help"], capture_output=True, text=True)
    assert r.returncode == 0 and "--channels" in r.stderr
    r = subprocess.run([os.path.join(BIN, "memd_cli"), "--channels", "2"], capture_output=True, text=True)
    assert r.returncode == 2


def test_mex_stub_library_exports():
    L = ctypes.CDLL(STUB)
    for name in ("mexFunction", "mex_stub_call", "mex_stub_last_error"):
        assert hasattr(L, name)


def _stub():
    L = ctypes.CDLL(STUB)
    vp = ctypes.c_void_p
    L.mex_stub_call.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, ctypes.c_long, vp, vp, vp]
    L.mex_stub_call.restype = ctypes.c_int
    L.mex_stub_last_error.restype = ctypes.c_char_p
    return L


@pytest.mark.gpu
def test_sample_synthetic_signal_matches_c_abi(tmp_path):
    torch = pytest.importorskip("torch")
    out = str(tmp_path / "mode_matrix.bin")
    r = subprocess.run([os.path.join(BIN, "sample_synthetic_signal"), out, "f64"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(out, dtype=np.float64).reshape(9, 8, 2000)
    y = mg.synth_tones(8, 2000, 1000.0, seed=0)
    d = mg.directions(8, 64, dtype="f64")
    plan = mg.Plan(8, 2000, 64, 9, 10)
    o = torch.empty((9, 8, 2000), dtype=torch.float64, device="cuda")
    plan.run(torch.as_tensor(y, device="cuda"), d, o)
    assert np.array_equal(got, o.cpu().numpy())
    assert np.abs(got.sum(axis=0) - y).max() < 1e-10


@pytest.mark.gpu
def test_cli_matches_c_abi_and_oracle(tmp_path):
    torch = pytest.importorskip("torch")
    y = mg.synth_eeg(4, 3000, 256.0, seed=7)
    inp = str(tmp_path / "x.bin")
    y.tofile(inp)
    out = str(tmp_path / "imfs.bin")
    r = subprocess.run([os.path.join(BIN, "memd_cli"), "--in", inp, "--channels", "4", "--f64", "--directions", "16",
                        "--imfs", "4", "--iter", "5", "--out", out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(out, dtype=np.float64).reshape(4, 4, 3000)
    d = oracle.directions(4, 16)
    ref, _ = oracle.memd(y, d, 4, 5)
    for i in range(4):
        assert np.linalg.norm(got[i] - ref[i]) / np.linalg.norm(ref[i]) < 1e-10


@pytest.mark.gpu
def test_cli_options_match_oracle(tmp_path):
    y = mg.synth_eeg(3, 2000, 256.0, seed=8)
    inp = str(tmp_path / "x.bin")
    y.tofile(inp)
    out = str(tmp_path / "imfs.bin")
    r = subprocess.run([os.path.join(BIN, "memd_cli"), "--in", inp, "--channels", "3", "--f64", "--directions", "12",
                        "--imfs", "4", "--iter", "4", "--spline", "nak", "--boundary", "mirror", "--out", out],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(out, dtype=np.float64).reshape(4, 3, 2000)
    ref, _ = oracle.memd(y, oracle.directions(3, 12), 4, 4, spline_end=1, boundary=1)
    for i in range(4):
        assert np.linalg.norm(got[i] - ref[i]) / np.linalg.norm(ref[i]) < 1e-10


@pytest.mark.gpu
def test_mex_entry_matches_c_abi_with_mex_primes():
    torch = pytest.importorskip("torch")
    C, L, K, nimf, it = 6, 2500, 24, 5, 6
    y = mg.synth_eeg(C, L, 256.0, seed=3).astype(np.float32)
    primes = np.array([2, 3, 5, 7, 11, 13], dtype=np.int32)  # primes(2000)(1:C), assistMatlabCuda.m:12-13
    dy = torch.as_tensor(y, device="cuda")
    dx = torch.arange(L, dtype=torch.int32, device="cuda")
    dp = torch.as_tensor(primes, device="cuda")
    out = torch.zeros((nimf, C, L), dtype=torch.float32, device="cuda")
    S = _stub()
    rc = S.mex_stub_call(C, K, nimf, it, dy.data_ptr(), L, dx.data_ptr(), dp.data_ptr(), out.data_ptr())
    assert rc == 0, S.mex_stub_last_error()
    d = mg.directions(C, K, primes=primes, dtype="f32")
    plan = mg.Plan(C, L, K, nimf, it, precision=mg.PREC_F32)
    ref = torch.empty_like(out)
    plan.run(dy, d, ref)
    assert torch.equal(out, ref)
    # argument errors come back as MATLAB errors before any device access
    rc = S.mex_stub_call(C, K, 0, it, dy.data_ptr(), L, dx.data_ptr(), dp.data_ptr(), out.data_ptr())
    assert rc == 1 and b"memd:args" in S.mex_stub_last_error()


def test_sweep_usage():
    r = subprocess.run([os.path.join(BIN, "memd_sweep"), "--help"], capture_output=True, text=True)
    assert r.returncode == 0 and "--lengths" in r.stderr
    r = subprocess.run([os.path.join(BIN, "memd_sweep"), "--precision", "f16"], capture_output=True, text=True)
    assert r.returncode == 2


@pytest.mark.gpu
def test_sweep_prints_the_reference_table():
    """The runBenchmark equivalent prints one "Channel, Length, DirVec, Time"
    row per (channels, directions, length) point."""
    r = subprocess.run([os.path.join(BIN, "memd_sweep"), "--channels", "4,8", "--directions", "8",
                        "--lengths", "500:1500:500", "--imfs", "3", "--iter", "2", "--precision", "mixed"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    assert lines[0] == "Channel, Length, DirVec, Time"
    rows = [tuple(x.strip() for x in l.split(",")) for l in lines[1:]]
    assert [(int(a), int(b), int(c)) for a, b, c, _ in rows] == [(C, L, 8) for C in (4, 8) for L in (500, 1000, 1500)]
    assert all(float(t) > 0 for *_, t in rows)


def test_profile_case_usage():
    import sys
    r = subprocess.run([sys.executable, os.path.join(os.path.dirname(BIN), "examples", "profile_case.py"), "--help"],
                       capture_output=True, text=True)
    assert r.returncode == 0 and "eeg32" in r.stdout and "batched" in r.stdout
