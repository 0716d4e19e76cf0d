"""The bounds-checked build (libmemd_gb300_checked.so, compiled with
-DMEMD_CHECKED): index checks in the substitution sweeps, the impulse-
accumulation mean and the tensor-core projection record a failure in the run
flags (FLAG_CHECK_FAILED) and skip the access instead of touching memory out
of bounds.  On valid runs no check may fail, and the checked build computes
exactly what the normal build does."""
import numpy as np
import pytest

import memd_gb300 as mg
import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,kw", [(mg.PREC_MIXED, {}), (mg.PREC_F64, {}),
                                          (mg.PREC_MIXED, {"dir_chunk": 16}), (mg.PREC_F64, {"solve_window": -1})])
def test_checked_build_passes_its_checks_and_matches(precision, kw):
    y = mg.synth_eeg(12, 4000, 256.0, seed=41)
    d = oracle.directions(12, 40)
    tdt = torch.float64 if precision == mg.PREC_F64 else torch.float32
    outs, flags = [], []
    for L in (mg.lib(), mg.checked_lib()):
        plan = mg.Plan(12, 4000, 40, 4, 5, precision=precision, library=L, **kw)
        o = torch.empty((4, 12, 4000), dtype=tdt, device="cuda")
        st = plan.run(torch.as_tensor(y, dtype=tdt, device="cuda"), torch.as_tensor(d, dtype=tdt, device="cuda"), o)
        plan.close()
        outs.append(o.cpu().numpy())
        flags.append(int(st.flags))
    assert b"bounds-checked" in mg.checked_lib().memd_version()
    assert flags == [0, 0]
    assert np.array_equal(outs[0], outs[1])
