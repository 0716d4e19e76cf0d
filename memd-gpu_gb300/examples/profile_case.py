"""One decomposition of a named workload, for profiler captures (ncu -k ... -s ... -c ...).

    python memd-gpu_gb300/examples/profile_case.py eeg32 [--precision mixed|f64|f32] [--runs R]
    python memd-gpu_gb300/examples/profile_case.py batched --epochs 8 [--precision mixed|f64]
    ... --stages   (after the runs: one eager run with every kernel timed by CUDA events,
                    printed as ms and launches per stage; no profiler needed)

eeg32:   32 channels x 30,504 samples (EEG-shaped, seed 0), 128 directions, 9 slots x 10 sifts.
batched: N epochs of 32 channels, lengths uniform in [1024, 8192] (seed 1000), 64 directions,
         8 slots x 10 sifts, one batched call.
Each run launches the decomposition graph once; the kernel order within a run is
project (mixed form: tf32 split, then the tensor-core projection), compact, factor,
solve (forward, backward), mean, per sift.
"""
import argparse
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "py"))

import numpy as np  # noqa: E402
import torch  # noqa: E402

import memd_gb300 as mg  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["eeg32", "batched"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "f64", "f32"])
    ap.add_argument("--epochs", type=int, default=8)
    ap.add_argument("--runs", type=int, default=1)
    ap.add_argument("--projection", default="auto", choices=["auto", "cuda-cores"],
                    help="mixed form: tensor-core (auto) or CUDA-core projection")
    ap.add_argument("--stages", action="store_true",
                    help="also print the per-stage times of one eager run (CUDA events per kernel)")
    a = ap.parse_args()
    if a.runs < 1:
        ap.error("--runs must be at least 1")
    prec = {"mixed": mg.PREC_MIXED, "f64": mg.PREC_F64, "f32": mg.PREC_F32}[a.precision]
    proj = mg.PROJ_AUTO if a.projection == "auto" else mg.PROJ_CUDA_CORES
    tdt = torch.float64 if prec == mg.PREC_F64 else torch.float32
    if a.case == "eeg32":
        C, L, K = 32, 30504, 128
        y = torch.as_tensor(mg.synth_eeg(C, L, 256.0, seed=0).astype(np.float32), dtype=tdt, device="cuda")
        d = mg.directions(C, K, dtype="f32").to(tdt)
        plan = mg.Plan(C, L, K, 9, 10, precision=prec, projection=proj)
        out = torch.empty((9, C, L), dtype=tdt, device="cuda")
        for _ in range(a.runs):
            st = plan.run(y, d, out)
        prof = plan.profile(y, d, out) if a.stages else None
    else:
        C, K, NI, IT, E = 32, 64, 8, 10, a.epochs
        rng = np.random.default_rng(1000)
        lengths = rng.integers(1024, 8193, size=E).astype(np.int64)
        recs = [mg.synth_eeg(C, int(L), 256.0, seed=10_000 + e).astype(np.float32) for e, L in enumerate(lengths)]
        offs = np.concatenate([[0], np.cumsum(C * lengths)[:-1]]).astype(np.int64)
        y = torch.as_tensor(np.concatenate([r.ravel() for r in recs]), dtype=tdt, device="cuda")
        d = mg.directions(C, K, dtype="f32").to(tdt)
        plan = mg.Plan(C, 8192, K, NI, IT, precision=prec, max_epochs=E, projection=proj)
        out = torch.empty(NI * y.numel(), dtype=tdt, device="cuda")
        for _ in range(a.runs):
            st = plan.run_batched(y, lengths, offs, d, out)
        prof = plan.profile_batched(y, lengths, offs, d, out) if a.stages else None
    print(f"{a.case} {a.precision}: {st.elapsed_ms:.3f} ms, {st.launches} launches, flags {st.flags}, "
          f"tests re-decided in double-float {st.refined}")
    if prof is not None:
        stages = prof.as_dict()
        total = sum(v["ms"] for v in stages.values())
        print("| stage | ms | launches | share |")
        print("|---|---|---|---|")
        for name, v in stages.items():
            print(f"| {name} | {v['ms']:.3f} | {v['launches']} | {100.0 * v['ms'] / total:.1f}% |")
        print(f"| total (eager) | {total:.3f} | {sum(v['launches'] for v in stages.values())} | |")
    plan.close()


if __name__ == "__main__":
    main()
