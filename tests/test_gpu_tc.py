"""The tensor-core projection of the mixed form (k_project_tc: TMA-staged tf32
tiles of the signal's first differences, 3xTF32 tcgen05.mma into TMEM,
certified signs of the projected differences) against
the CUDA-core projection (k_project_mx) and the FP64 path: identical extrema
index sets at every sift, so identical decompositions.

Shapes cover one and several 32-channel blocks (C = 5, 32, 40, 128), one
and several direction tiles (K = 17, 128, 300), direction chunks, short
records (L < 128) and batched epochs."""
import numpy as np
import pytest

import memd_gb300 as mg
import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def run(y, d, nimf, it, precision, **kw):
    C, L = y.shape
    K = d.shape[0]
    tdt = torch.float64 if precision == mg.PREC_F64 else torch.float32
    plan = mg.Plan(C, L, K, nimf, it, precision=precision, **kw)
    plan.set_trace(True)
    out = torch.empty((nimf, C, L), dtype=tdt, device="cuda")
    st = plan.run(torch.as_tensor(y, dtype=tdt, device="cuda"), torch.as_tensor(d, dtype=tdt, device="cuda"), out)
    tr = plan.trace()[: nimf - 1, :it].copy()
    plan.close()
    return out.cpu().numpy().astype(np.float64), st, tr


@pytest.mark.parametrize("C,L,K,chunk", [(32, 4096, 128, 0), (5, 3000, 17, 0), (40, 2500, 24, 0),
                                         (32, 2000, 300, 0), (12, 3000, 40, 16), (3, 100, 8, 0),
                                         (128, 3000, 64, 0)])
def test_tensor_core_projection_equals_cuda_core_and_fp64(C, L, K, chunk):
    y = mg.synth_eeg(C, L, 256.0, seed=C + K).astype(np.float32)
    d = oracle.directions(C, K).astype(np.float32)
    nimf, it = 4, 5
    a, sa, ta = run(y, d, nimf, it, mg.PREC_MIXED, dir_chunk=chunk, projection=mg.PROJ_AUTO)
    b, sb, tb = run(y, d, nimf, it, mg.PREC_MIXED, dir_chunk=chunk, projection=mg.PROJ_CUDA_CORES)
    c, sc, tc = run(y.astype(np.float64), d.astype(np.float64), nimf, it, mg.PREC_F64, dir_chunk=chunk)
    assert sa.flags == 0 and sb.flags == 0, (sa.flags, sb.flags)
    assert np.array_equal(ta["count"], tb["count"]) and np.array_equal(ta["hash"], tb["hash"])
    assert np.array_equal(ta["count"], tc["count"]) and np.array_equal(ta["hash"], tc["hash"])
    assert np.array_equal(a, b)


def test_tensor_core_projection_in_batched_runs():
    C, K, nimf, it = 8, 24, 4, 4
    lengths = [3000, 1500, 4100, 64, 900]
    recs = [mg.synth_eeg(C, L, 256.0, seed=80 + e).astype(np.float32) for e, L in enumerate(lengths)]
    offs = np.concatenate([[0], np.cumsum([C * L for L in lengths])[:-1]]).astype(np.int64)
    d = torch.as_tensor(oracle.directions(C, K).astype(np.float32), device="cuda")
    y = torch.as_tensor(np.concatenate([r.ravel() for r in recs]), device="cuda")
    outs = []
    for proj in (mg.PROJ_AUTO, mg.PROJ_CUDA_CORES):
        plan = mg.Plan(C, max(lengths), K, nimf, it, precision=mg.PREC_MIXED, max_epochs=len(lengths), projection=proj)
        o = torch.full((nimf * y.numel(),), float("nan"), dtype=torch.float32, device="cuda")
        st = plan.run_batched(y, lengths, offs, d, o)
        assert st.flags == 0
        plan.close()
        outs.append(o.cpu().numpy())
    assert np.array_equal(outs[0], outs[1])


def test_projection_option_is_checked():
    with pytest.raises(mg.MemdError) as ei:
        mg.Plan(4, 100, 8, 2, 1, precision=mg.PREC_MIXED, projection=2)
    assert ei.value.status == mg.MEMD_ERR_INVALID
