"""Device-side failure detection without a GPU fault: every wait a kernel of
this library makes is bounded (iterations and clock) and reports through the
run-state flags instead of hanging.  The diagnostic kernel waits on an
mbarrier that nothing completes; it must give up within its limit, report
MEMD_FLAG_DEVICE_TIMEOUT, and leave the context usable for a decomposition."""
import ctypes

import numpy as np
import pytest

import memd_gb300 as mg
import oracle


@pytest.mark.gpu
def test_bounded_wait_gives_up_and_context_stays_usable():
    torch = pytest.importorskip("torch")
    flags = mg.wait_timeout_flags(2_000_000)  # about a millisecond of clocks
    assert flags & mg.FLAG_DEVICE_TIMEOUT
    # the same process still decomposes correctly
    y = mg.synth_tones(3, 600, 1000.0, seed=4)
    d = oracle.directions(3, 8)
    plan = mg.Plan(3, 600, 8, 3, 4)
    out = torch.empty((3, 3, 600), dtype=torch.float64, device="cuda")
    st = plan.run(torch.as_tensor(y, device="cuda"), torch.as_tensor(d, device="cuda"), out)
    plan.close()
    ref, _ = oracle.memd(y, d, 3, 4)
    assert st.flags == 0
    assert np.linalg.norm(out.cpu().numpy() - ref) <= 1e-10 * np.linalg.norm(ref)


def test_wait_timeout_diagnostic_rejects_bad_limits():
    v = ctypes.c_int32()
    assert mg.lib().memd_diag_wait_timeout(0, ctypes.byref(v)) == mg.MEMD_ERR_INVALID
    assert mg.lib().memd_diag_wait_timeout(1 << 40, ctypes.byref(v)) == mg.MEMD_ERR_INVALID
