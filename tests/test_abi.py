"""The C-ABI library: loads, exports what include/*.h declares, validates
arguments on the host (no GPU needed for any of this)."""
import ctypes
import os
import re

import numpy as np
import pytest

import memd_gb300

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in ("memd_gb300.h", "memd_synth.h"):
        text = open(os.path.join(REPO, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names.update(re.findall(r"\b(memd_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(memd_gb300.EXPORTS)


def test_version_and_default_config(lib):
    assert b"sm_103a" in lib.memd_version()
    c = memd_gb300.default_config()
    assert c.num_imfs == 9 and c.max_iter == 10
    assert c.ref_window == 1 and c.precision == memd_gb300.PREC_F64
    assert abs(c.stop_sd - 0.075) < 1e-15 and abs(c.stop_sd2 - 0.75) < 1e-15


@pytest.mark.parametrize("kw", [
    dict(channels=0, length=100, directions=4),
    dict(channels=2, length=3, directions=4),
    dict(channels=2, length=100, directions=0),
    dict(channels=2, length=100, directions=4, num_imfs=0),
    dict(channels=2, length=100, directions=4, max_iter=-1),
    dict(channels=2, length=100, directions=4, precision=7),
    dict(channels=2, length=100, directions=4, mean_eval=3),
])
def test_plan_rejects_bad_config_on_host(kw):
    with pytest.raises(memd_gb300.MemdError) as ei:
        memd_gb300.Plan(**kw)
    assert ei.value.status == memd_gb300.MEMD_ERR_INVALID


@pytest.mark.parametrize("kw", [
    dict(precision=memd_gb300.PREC_F64, mean_eval=2),
    dict(precision=memd_gb300.PREC_F32, mean_eval=2),
    dict(precision=memd_gb300.PREC_MIXED, mean_eval=2, stop_mode=memd_gb300.STOP_CRITERION),
])
def test_impulse_mean_only_for_mixed_fixed_mode(kw):
    with pytest.raises(memd_gb300.MemdError) as ei:
        memd_gb300.Plan(2, 100, 4, **kw)
    assert ei.value.status == memd_gb300.MEMD_ERR_UNSUPPORTED


def test_null_plan_arguments(lib):
    assert lib.memd_plan_create(None, None) == memd_gb300.MEMD_ERR_INVALID
    assert lib.memd_run_f64(None, None, None, None, None, None, None) == memd_gb300.MEMD_ERR_INVALID
    assert lib.memd_plan_destroy(None) == memd_gb300.MEMD_OK


def test_synth_is_deterministic_and_shaped():
    a = memd_gb300.synth_eeg(4, 3000, 256.0, seed=3)
    b = memd_gb300.synth_eeg(4, 3000, 256.0, seed=3)
    c = memd_gb300.synth_eeg(4, 3000, 256.0, seed=4)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert 5 < a.std() < 200
    t = memd_gb300.synth_tones(8, 2000, 1000.0, seed=0)
    # three unit-ish tones + small noise: per-channel RMS ~ sqrt(3/2 * E[A^2])
    assert np.all((t.std(axis=1) > 0.6) & (t.std(axis=1) < 2.0))


def test_pink_spectrum_slope():
    x = memd_gb300.synth_eeg(1, 1 << 15, 256.0, seed=9)[0]
    # the EEG generator without bursts/drift dominates mid-band: check the
    # power falls with frequency between 2 and 60 Hz
    f = np.fft.rfftfreq(x.size, 1 / 256.0)
    p = np.abs(np.fft.rfft(x)) ** 2
    lo = p[(f > 2) & (f < 6)].mean()
    hi = p[(f > 30) & (f < 60)].mean()
    assert lo > 4 * hi


def test_bin_roundtrip(tmp_path, lib):
    a = np.arange(12, dtype=np.float32)
    path = str(tmp_path / "x.bin").encode()
    assert lib.memd_write_bin(path, a.ctypes.data_as(ctypes.c_void_p), a.size, 4) == 0
    assert lib.memd_bin_count(path, 4) == 12
    b = np.zeros(12, dtype=np.float32)
    assert lib.memd_read_bin(path, b.ctypes.data_as(ctypes.c_void_p), 12, 4) == 0
    assert np.array_equal(a, b)
    assert lib.memd_read_bin(b"/nonexistent/x.bin", b.ctypes.data_as(ctypes.c_void_p), 1, 4) != 0
