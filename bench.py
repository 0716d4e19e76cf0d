#!/usr/bin/env python
"""Benchmark of the GB300 MEMD engine on the 32-channel EEG-shaped workload.

Workload (one "step" = one full decomposition): 32 channels x 30,504 samples
(fs = 256 Hz, seeded EEG-shaped synthetic record), 128 Hammersley directions,
9 output slots = 8 IMFs x 10 sifts + residual (the reference's fixed mode,
memReducedEpochs_dev.cu:1473-1476), i.e. 80 sifts per step.

Metric: channel-samples/s = C*L / (device time of one decomposition), for
the precision form that meets <= 1e-4 relative L2 per IMF against the FP64
path (FP32 form when it meets the gate, else FP64); sift iterations/s beside
it.  Inputs resident in HBM for `value`; `e2e` adds the pinned host->device
copy of the record and the device->host copy of all IMFs through the C ABI.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank decomposes its own record (a replica with
its own seed, no exchange): weak scaling, max time over ranks.
--impl reference times the reference algorithm's CPU transcription (the FP64
OpenMP oracle, all host cores): every step is the full decomposition of the
same record (all 80 sifts), with nothing scaled.  That arm loads no part of
the CUDA library: both arms draw the record from memd_signals (numpy).
"""
from __future__ import annotations

import argparse
import csv
import io
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "memd-gpu_gb300", "py"))

import memd_signals  # noqa: E402  (numpy only)

METRIC = "channel-samples/sec at ≤1e-4 rel-L2 per IMF vs FP64 (1 GB300); sift iters/sec"
WL = dict(workload="eeg32_30504_k128_fixed", C=32, L=30504, K=128, num_imfs=9, max_iter=10, fs=256.0)
SIFTS = (WL["num_imfs"] - 1) * WL["max_iter"]
GATE = 1e-4
# precision forms timed by our arm; "mixed" builds the mean envelope by impulse
# accumulation, "mixed_direct" evaluates every envelope at every sample
NAMES = ("fp64", "mixed", "mixed_direct", "fp32")
GATED = ("mixed", "mixed_direct", "fp32")


def bench_record(seed: int) -> np.ndarray:
    """The benchmark record, rounded to float32 once so that every precision
    form (and the CPU arm) decomposes exactly the same numbers."""
    return memd_signals.as_float32_record(memd_signals.eeg(WL["C"], WL["L"], WL["fs"], seed))


def bench_config(ws: int) -> dict:
    """The workload description both arms print (same keys, same values)."""
    return {"workload": WL["workload"], "C": WL["C"], "L": WL["L"], "K": WL["K"], "num_imfs": WL["num_imfs"],
            "max_iter": WL["max_iter"], "sifts_per_step": SIFTS, "mode": "fixed (reference)",
            "l2": "flushed between steps", "parallelism": "replicas" if ws > 1 else "single"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-reference-gpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-epochs measurement")
    ap.add_argument("--no-long", action="store_true", help="skip the long-record measurement")
    ap.add_argument("--no-wide", action="store_true", help="skip the 128-channel record measurement")
    ap.add_argument("--no-stop", action="store_true", help="skip the stop-criterion (8 x 2000 tones) measurement")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _reduce_over_ranks(x: float, device, op_name: str) -> float:
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=getattr(dist.ReduceOp, op_name))
    return float(t.item())


def max_over_ranks(x: float, device="cuda") -> float:
    """Largest x over the ranks of the process group (x itself on one rank):
    the timed region of a replicated run ends when its slowest rank does."""
    return _reduce_over_ranks(x, device, "MAX")


def sum_over_ranks(x: float, device="cuda") -> float:
    """Sum of x over the ranks (x itself on one rank): the units of work that
    all replicas processed."""
    return _reduce_over_ranks(x, device, "SUM")


def barrier():
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()


class WallSteps:
    """Step timer on the host clock (CPU work)."""

    def __init__(self):
        self.ms = []

    def start(self):
        self._t0 = time.perf_counter()

    def stop(self):
        self.ms.append((time.perf_counter() - self._t0) * 1e3)

    def total_ms(self) -> float:
        return float(sum(self.ms))


class CudaSteps:
    """Step timer from CUDA events recorded on the launching stream."""

    def __init__(self, stream):
        self.stream = stream
        self.ev = []

    def start(self):
        import torch

        self.ev.append([torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)])
        self.ev[-1][0].record(self.stream)

    def stop(self):
        self.ev[-1][1].record(self.stream)

    def total_ms(self) -> float:
        import torch

        torch.cuda.synchronize()
        return float(sum(a.elapsed_time(b) for a, b in self.ev))


def measure_replicated(step, units: float, steps: int, warmup: int, timer, device="cuda", sync=lambda: None,
                       between=lambda: None) -> dict:
    """Times `steps` calls of step() after `warmup` untimed ones, each call
    bracketed by the timer (`between` runs outside the timed region, before
    every timed step: the L2 flush), with a barrier and a synchronisation on
    both sides.  Every rank is a replica working on its own data: the step
    time is the slowest rank's, the units are summed over the ranks, and the
    whole-job rate is units / step time."""
    for _ in range(warmup):
        step()
    sync()
    barrier()
    sync()
    t0 = time.perf_counter()
    for _ in range(steps):
        between()
        timer.start()
        step()
        timer.stop()
    local = timer.total_ms() / steps
    sync()
    wall = time.perf_counter() - t0
    barrier()
    ms = max_over_ranks(local, device)
    tot = sum_over_ranks(units, device)
    return {"ms_per_step": ms, "units": tot, "value": tot / (ms / 1e3), "wall_s": wall, "local_ms_per_step": local}


# ----------------------------------------------------------------------------
# clocks sampling (nvidia-smi during the timed region)
# ----------------------------------------------------------------------------
SMI_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


class Clocks:
    def __init__(self, gpu_index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), f"--query-gpu={SMI_FIELDS}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        time.sleep(0.25)
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r for r in csv.reader(io.StringIO(self.f.read())) if len(r) >= 9]
        os.unlink(self.f.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if "Active" in r[5 + i] and "Not" not in r[5 + i]})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ----------------------------------------------------------------------------
# algorithmic work per stage (flops, bytes) from the knot counts of a traced run
# ----------------------------------------------------------------------------
def stage_work(C, L, K, sifts, sum_E, rb, cum=False):
    """sum_E: total knots over all sifts, directions and both envelopes.
    cum: the mean envelope is built by impulse accumulation (per knot and
    channel: d_j and its jump, 3 flops; per 32-sample word, envelope and
    channel: the anchor piece's coefficients and Taylor shift, 20 flops; reads
    each knot's value and solution once and the working signal once)."""
    KCL = float(K) * C * L * sifts
    CE = float(C) * sum_E
    W = (L + 31) // 32
    if cum:
        ev = {"flops": 3.0 * CE + 20.0 * W * 2 * K * C * sifts, "bytes": 2.0 * rb * CE + sifts * 2.0 * C * L * rb}
    else:
        # per sample, channel, direction: 2 envelopes x 3 fma + 2 adds;
        # per knot and channel: 9 flops of coefficients
        ev = {"flops": 14.0 * KCL + 9.0 * CE, "bytes": 2.0 * rb * CE + sifts * 2.0 * C * L * rb}
    return {
        # P = dir . X: one fma per (direction, channel, sample)
        "project": {"flops": 2.0 * KCL, "bytes": sifts * (C * L * rb + 2.0 * K * L / 8.0)},
        "compact": {"flops": 0.0, "bytes": sifts * 2.0 * K * L / 8.0 + 4.0 * sum_E},
        "factor": {"flops": 8.0 * sum_E, "bytes": sum_E * (4.0 + 4 * rb)},
        # slope, rhs, forward (2), backward (1) per knot and channel
        "solve": {"flops": 7.0 * CE, "bytes": CE * (rb + 3 * 2 * rb) + sum_E * 4 * rb},
        "eval": ev,
    }


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def load_profile_traffic():
    """DRAM bytes per launch of the kernels, from the committed ncu capture
    summary profiles/dram_traffic_eeg32_30504_k128.json (keys "<form>:<stage>",
    each with bytes_per_launch averaged over every launch of one whole
    decomposition and the capture command as "source"); empty if absent.  The
    bench itself runs without a profiler, so this figure is a committed
    measurement of the same workload, labelled as such in the line."""
    p = os.path.join(REPO, "profiles", "dram_traffic_eeg32_30504_k128.json")
    if os.path.exists(p):
        try:
            return json.load(open(p))
        except Exception:
            return {}
    return {}


# ----------------------------------------------------------------------------
# our arm
# ----------------------------------------------------------------------------
def run_ours(args):
    import torch
    import torch.distributed as dist

    import memd_gb300 as mg

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        dist.init_process_group("nccl")
    C, L, K, NI, IT = WL["C"], WL["L"], WL["K"], WL["num_imfs"], WL["max_iter"]
    # the record is rounded to float32 once, so that every precision form
    # decomposes exactly the same input (the FP32 forms take float32 input)
    y = bench_record(rank)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    results = {}
    outs = {}
    plans = {}
    # one direction set for all forms: float32 Hammersley directions, widened
    # exactly to float64 for the FP64 path
    d32 = mg.directions(C, K, dtype="f32")
    FORMS = (("fp64", mg.PREC_F64, torch.float64, {}),
             ("mixed", mg.PREC_MIXED, torch.float32, {"mean_eval": 2}),
             ("mixed_direct", mg.PREC_MIXED, torch.float32, {"mean_eval": 1}),
             ("fp32", mg.PREC_F32, torch.float32, {}))
    import memd_autotune

    tuned = {}
    for name, prec, tdt, kw in FORMS:
        plan = mg.Plan(C, L, K, NI, IT, precision=prec, tuning="auto", **kw)
        plans[name] = plan
        key = memd_autotune.config_key(plan.cfg)
        tuned[name] = {"key": key, "choice": plan.tuning(),
                       "source": ("autotuner (memd-gpu_gb300/tuning/gb300.json)"
                                  if memd_autotune.lookup(plan.cfg) else "defaults (no stored choice)")}
        d = d32.to(tdt)
        dy = torch.as_tensor(y, dtype=tdt, device="cuda")
        out = torch.empty((NI, C, L), dtype=tdt, device="cuda")
        clocks = Clocks(local) if rank == 0 else None
        m = measure_replicated(lambda: plan.run(dy, d, out, stream=stream, stats=False), float(C * L), args.steps,
                               args.warmup, CudaSteps(stream), sync=torch.cuda.synchronize,
                               between=flush.zero_)  # L2 flush between timed steps (256 MB > 129 MB L2)
        ck = clocks.stop() if clocks else None
        st = plan.run(dy, d, out, stats=True)
        results[name] = {"ms_per_step": m["ms_per_step"], "wall_s": m["wall_s"], "clocks": ck,
                         "launches_per_step": int(st.launches), "flags": int(st.flags), "refined": int(st.refined),
                         "workspace_gb": plan.workspace_bytes / 1e9}
        outs[name] = (out, d, dy)

    # precision gate: each FP32-arithmetic form against the FP64 path, per IMF
    ref = outs["fp64"][0].cpu().numpy()
    gates = {}
    for name in GATED:
        o = outs[name][0].cpu().numpy()
        rl = [rel_l2(o[i], ref[i]) for i in range(NI)]
        gates[name] = {"rel_l2_per_imf_vs_fp64": rl, "max": max(rl), "passed": all(r <= GATE for r in rl)}
    passing = [n for n in GATED if gates[n]["passed"]]
    head = min(passing, key=lambda n: results[n]["ms_per_step"]) if passing else "fp64"

    # e2e through the C ABI with host buffers (pinned), headline precision
    plan = plans[head]
    tdt = torch.float64 if head == "fp64" else torch.float32
    hy = torch.as_tensor(y, dtype=tdt).pin_memory()
    hout = torch.empty((NI, C, L), dtype=tdt).pin_memory()
    dy = torch.empty((C, L), dtype=tdt, device="cuda")
    dout = torch.empty((NI, C, L), dtype=tdt, device="cuda")
    d = outs[head][1]

    def e2e_step():
        dy.copy_(hy, non_blocking=True)
        plan.run(dy, d, dout, stream=stream, stats=False)
        hout.copy_(dout, non_blocking=True)

    e2e_ms = measure_replicated(e2e_step, float(C * L), args.steps, max(args.warmup, 2), CudaSteps(stream),
                                sync=torch.cuda.synchronize, between=flush.zero_)["ms_per_step"]
    elem = 8 if head == "fp64" else 4

    # per-stage timing (eager, every kernel bracketed by CUDA events) and knot
    # counts (traced run) for the roofline of the dominant kernel
    stage = {}
    for name in NAMES:
        p = plans[name]
        out, dd, yy = outs[name]
        prof = p.profile(yy, dd, out).as_dict()
        p.set_trace(True)
        p.run(yy, dd, out)
        tr = p.trace()
        p.set_trace(False)
        sum_E = float(tr["count"][: NI - 1, :IT].astype(np.int64).sum())
        rb = 4 if name == "fp32" else 8  # double, float or double-float
        work = stage_work(C, L, K, SIFTS, sum_E, rb, cum=(name == "mixed"))
        stage[name] = {"profile": prof, "sum_knots": sum_E, "work": work}

    meas = {}
    peaks_path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        meas = json.load(open(peaks_path))
    hbm_peak = meas.get("hbm_gbs", 6800.0)
    traffic = load_profile_traffic()

    fma = {"f64": mg.fma_rate(mg.PREC_F64) / 1e12, "f32": mg.fma_rate(mg.PREC_F32) / 1e12}

    def roofline(name):
        """Dominant stage of the form's eager per-stage profile against the
        algorithmic work of one sift: projection 2*K*C*L flops, the two
        envelope evaluations with the mean 16*K*C*L, spline setup and solve
        15*C*sum(E) (sum over directions and envelopes of the knot counts); the
        signal read and written once, 2*C*L*s bytes.  The bound is the CUDA-core
        FMA pipe of the form's arithmetic (FP32 for the mixed and FP32 forms,
        FP64 for the FP64 path), measured live on this GPU; the HBM fraction of
        the algorithmic bytes is reported beside it."""
        prof = stage[name]["profile"]
        work = stage[name]["work"]
        dom = max(("project", "compact", "factor", "solve", "eval"), key=lambda s: prof[s]["ms"])
        ms = prof[dom]["ms"]
        n = max(prof[dom]["launches"], 1)
        per_launch_s = ms / 1e3 / n
        sums = stage[name]["sum_knots"] / SIFTS  # knots per sift, all directions and envelopes
        kcl = float(K) * C * L
        alg = {"project": 2.0 * kcl, "eval": 16.0 * kcl, "solve": 15.0 * C * sums, "factor": 0.0, "compact": 0.0}
        per_sift_launches = n / SIFTS
        f = alg[dom] / per_sift_launches
        s_bytes = 4 if name == "fp32" else 8
        b_alg = 2.0 * C * L * s_bytes / per_sift_launches
        pipe = "f64" if name == "fp64" else "f32"
        achieved = f / per_launch_s / 1e12
        tr = traffic.get(f"{name}:{dom}")
        kern = {"project": "k_split_tf32 + k_project_tc" if name.startswith("mixed") else "k_project_extrema",
                "eval": {"mixed": "k_mean_cum", "mixed_direct": "k_eval_w", "fp32": "k_eval_w", "fp64": "k_eval"}[name],
                "solve": "k_solve_fwd + k_solve_bwd", "factor": "k_factor", "compact": "k_compact"}[dom]
        step_s = results[name]["ms_per_step"] / 1e3
        return {"kernel": kern, "stage": dom, "bound": f"{pipe} fma pipe (CUDA cores)", "achieved": achieved,
                "peak": fma[pipe], "unit": "TFLOP/s", "frac": achieved / fma[pipe],
                "peak_source": f"memd_diag_fma_rate({pipe}), measured live on this GPU (MEASURED_PEAKS.json has no "
                               f"CUDA-core rate)",
                "alg_flops_per_launch": f, "avg_launch_ms": ms / n, "launches": n,
                "hbm": {"alg_bytes_per_launch": b_alg, "achieved_gbs": b_alg / per_launch_s / 1e9, "peak_gbs": hbm_peak,
                        "frac": b_alg / per_launch_s / 1e9 / hbm_peak,
                        "peak_source": "MEASURED_PEAKS.json hbm_gbs" if meas else "fallback 6.8 TB/s"},
                "design_bytes_per_launch": work[dom]["bytes"] / n,
                "traffic": tr.get("bytes_per_launch") if tr else None,
                "traffic_source": tr.get("source") if tr else None,
                "step": {"alg_flops": 18.0 * kcl * SIFTS, "achieved_tflops": 18.0 * kcl * SIFTS / step_s / 1e12,
                         "frac": 18.0 * kcl * SIFTS / step_s / 1e12 / fma[pipe]},
                "stage_ms": {st: round(prof[st]["ms"], 3) for st in prof}}

    line = None
    if rank == 0:
        hv = results[head]
        value = ws * C * L / (hv["ms_per_step"] / 1e3)
        line = {
            "metric": METRIC,
            "value": value,
            "unit": "channel-samples/s",
            "n_gpus": ws,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": hv["ms_per_step"],
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": {"fp64": "f64", "fp32": "f32", "mixed": "f32 (double-float working signal)",
                      "mixed_direct": "f32 (double-float working signal)"}[head],
            "form": head,
            "data": "synthetic EEG-shaped (seeded 1/f mixture + alpha bursts + drift), generated on the host",
            "config": bench_config(ws),
            "sift_iters_per_s": ws * SIFTS / (hv["ms_per_step"] / 1e3),
            "precision_gate": gates,
            "fp64": {"ms_per_step": results["fp64"]["ms_per_step"],
                     "channel_samples_per_s": ws * C * L / (results["fp64"]["ms_per_step"] / 1e3),
                     "workspace_gb": results["fp64"]["workspace_gb"], "flags": results["fp64"]["flags"]},
            "fp32": {"ms_per_step": results["fp32"]["ms_per_step"],
                     "channel_samples_per_s": ws * C * L / (results["fp32"]["ms_per_step"] / 1e3),
                     "workspace_gb": results["fp32"]["workspace_gb"], "flags": results["fp32"]["flags"]},
            "mixed": {"ms_per_step": results["mixed"]["ms_per_step"],
                      "channel_samples_per_s": ws * C * L / (results["mixed"]["ms_per_step"] / 1e3),
                      "workspace_gb": results["mixed"]["workspace_gb"], "flags": results["mixed"]["flags"],
                      "refined_tests": results["mixed"]["refined"],
                      "mean": "impulse accumulation"},
            "mixed_direct": {"ms_per_step": results["mixed_direct"]["ms_per_step"],
                             "channel_samples_per_s": ws * C * L / (results["mixed_direct"]["ms_per_step"] / 1e3),
                             "flags": results["mixed_direct"]["flags"], "mean": "direct evaluation"},
            "e2e": {"value": ws * C * L / (e2e_ms / 1e3), "unit": "channel-samples/s",
                    "h2d_bytes_per_step": C * L * elem, "d2h_bytes_per_step": NI * C * L * elem,
                    "ms_per_step": e2e_ms, "api": "memd_run_f32/f64 (C ABI) via ctypes"},
            "gpu_launches": results[head]["launches_per_step"] * args.steps,
            "tuning": tuned,
            "roofline": roofline(head),
            "roofline_by_form": {n: roofline(n) for n in NAMES},
            "fma_rate_tflops": fma,
            "clocks": results[head]["clocks"],
        }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(y, outs["fp64"][1].cpu().numpy())
    if rank == 0 and not args.no_reference_gpu:
        line["reference_gpu"] = reference_gpu(y)
    if not args.no_batched:
        for p in plans.values():
            p.close()
        plans = {}
        bres = batched_epochs(rank)
        if rank == 0:
            line["batched_epochs"] = bres
    if not args.no_stop:
        for p in plans.values():
            p.close()
        plans = {}
        sres = stop_criterion(rank, args)
        if rank == 0:
            line["stop_criterion"] = sres
    if not args.no_wide:
        for p in plans.values():
            p.close()
        plans = {}
        wres = single_record(rank, WIDE)
        if rank == 0:
            line["wide_record"] = wres
    if not args.no_long:
        for p in plans.values():
            p.close()
        plans = {}
        lres = single_record(rank, LONG)
        if rank == 0:
            line["long_record"] = lres
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()
    for p in plans.values():
        p.close()
    if rank == 0:
        print(json.dumps(line))


# ----------------------------------------------------------------------------
# CPU baseline: the FP64 OpenMP oracle (a transcription of the reference
# algorithm) on a bounded sample: all 8 IMF stages with one sift each, scaled
# to the 80 sifts of the full decomposition.
# ----------------------------------------------------------------------------
# batched epochs: 512 epochs of 32 channels, lengths uniform in [1024, 8192]
# (seeded), 64 directions, 8 IMF slots x 10 sifts (fixed mode)
BATCH = dict(workload="epochs512_c32_L1024-8192_k64_fixed", epochs=512, C=32, Lmin=1024, Lmax=8192, K=64,
             num_imfs=8, max_iter=10, fs=256.0, warmup=1, steps=2)


def batched_epochs(rank):
    """Channel-samples/s of the batched mixed and FP64 paths on the epoch set,
    with the per-IMF precision gate of the mixed form against FP64."""
    import torch

    import memd_gb300 as mg

    B = BATCH
    rng = np.random.default_rng(1000 + rank)
    lengths = rng.integers(B["Lmin"], B["Lmax"] + 1, size=B["epochs"]).astype(np.int64)
    C, K, NI, IT = B["C"], B["K"], B["num_imfs"], B["max_iter"]
    recs = [mg.synth_eeg(C, int(L), B["fs"], seed=10_000 * (rank + 1) + e).astype(np.float32)
            for e, L in enumerate(lengths)]
    offs = np.concatenate([[0], np.cumsum(C * lengths)[:-1]]).astype(np.int64)
    flat = np.concatenate([r.ravel() for r in recs])
    d32 = mg.directions(C, K, dtype="f32")
    out = {"workload": B["workload"], "epochs": int(B["epochs"]), "total_samples": int(lengths.sum()),
           "channel_samples": int(C * lengths.sum())}
    outs = {}
    stream = torch.cuda.current_stream()
    for name, prec, tdt in (("mixed", mg.PREC_MIXED, torch.float32), ("fp64", mg.PREC_F64, torch.float64)):
        plan = mg.Plan(C, B["Lmax"], K, NI, IT, precision=prec, max_epochs=B["epochs"], tuning="auto")
        y = torch.as_tensor(flat, dtype=tdt, device="cuda")
        o = torch.empty(NI * y.numel(), dtype=tdt, device="cuda")
        d = d32.to(tdt)
        # every replica decomposes its own epoch set
        m = measure_replicated(lambda: plan.run_batched(y, lengths, offs, d, o, stream=stream, stats=False),
                               C * float(lengths.sum()), B["steps"], B["warmup"], CudaSteps(stream),
                               sync=torch.cuda.synchronize)
        ms = m["ms_per_step"]
        st = plan.run_batched(y, lengths, offs, d, o)
        out[name] = {"ms_per_step": ms, "channel_samples_per_s": m["value"],
                     "workspace_gb": plan.workspace_bytes / 1e9, "flags": int(st.flags), "tuning": plan.tuning()}
        outs[name] = o.cpu().numpy().astype(np.float64)
        plan.close()
        del y, o
        torch.cuda.empty_cache()
    worst = 0.0
    for off, L in zip(offs, lengths):
        a = outs["mixed"][NI * off: NI * off + NI * C * L].reshape(NI, C, L)
        b = outs["fp64"][NI * off: NI * off + NI * C * L].reshape(NI, C, L)
        for i in range(NI):
            worst = max(worst, rel_l2(a[i], b[i]))
    out["precision_gate"] = {"max_rel_l2_per_imf_vs_fp64": worst, "passed": worst <= GATE}
    out["mixed_over_fp64"] = out["fp64"]["ms_per_step"] / out["mixed"]["ms_per_step"]
    return out


# stop criterion: 8 channels x 2,000 samples (fs 1 kHz) of tones at 5, 20 and
# 60 Hz with noise (seed 0), 64 directions, thresholds (0.075, 0.75, 0.075),
# up to 10 IMFs plus the residual, at most 200 sifts per IMF
STOP = dict(workload="tones8_2000_k64_stop", C=8, L=2000, K=64, num_imfs=11, max_iter=200, fs=1000.0,
            sd=0.075, sd2=0.75, tol=0.075)


def stop_criterion(rank, args):
    """Decomposition time of the FP64 and mixed forms in stop mode (nested
    conditional graph loops, no host round trip), their IMF and sift counts,
    and the mixed form's per-IMF error against FP64."""
    import torch

    import memd_gb300 as mg

    S = STOP
    C, L, K, NI, IT = S["C"], S["L"], S["K"], S["num_imfs"], S["max_iter"]
    y = memd_signals.as_float32_record(memd_signals.tones(C, L, S["fs"], seed=rank))
    d32 = mg.directions(C, K, dtype="f32")
    stream = torch.cuda.current_stream()
    out = {"workload": S["workload"], "C": C, "L": L, "K": K, "max_imfs": NI - 1, "max_iter": IT,
           "thresholds": [S["sd"], S["sd2"], S["tol"]]}
    res = {}
    for name, prec, tdt in (("fp64", mg.PREC_F64, torch.float64), ("mixed", mg.PREC_MIXED, torch.float32)):
        plan = mg.Plan(C, L, K, NI, IT, precision=prec, stop_mode=mg.STOP_CRITERION, stop_sd=S["sd"],
                       stop_sd2=S["sd2"], stop_tol=S["tol"])
        dy = torch.as_tensor(y, dtype=tdt, device="cuda")
        o = torch.empty((NI, C, L), dtype=tdt, device="cuda")
        d = d32.to(tdt)
        m = measure_replicated(lambda: plan.run(dy, d, o, stream=stream, stats=False), float(C * L),
                               max(args.steps, 5), max(args.warmup, 3), CudaSteps(stream), sync=torch.cuda.synchronize)
        st = plan.run(dy, d, o)
        sifts = [int(v) for v in st.sifts[: st.n_imfs]]
        out[name] = {"ms_per_step": m["ms_per_step"], "channel_samples_per_s": m["value"], "n_imfs": int(st.n_imfs),
                     "sifts": sifts, "sift_iters_per_s": sum(sifts) / (m["ms_per_step"] / 1e3),
                     "flags": int(st.flags)}
        res[name] = o.cpu().numpy().astype(np.float64)
        plan.close()
    rl = [rel_l2(res["mixed"][i], res["fp64"][i]) for i in range(NI) if np.linalg.norm(res["fp64"][i]) > 0]
    out["precision_gate"] = {"rel_l2_per_imf_vs_fp64": rl, "max": max(rl), "passed": max(rl) <= GATE,
                             "same_imf_and_sift_counts": out["mixed"]["sifts"] == out["fp64"]["sifts"]}
    out["mixed_over_fp64"] = out["fp64"]["ms_per_step"] / out["mixed"]["ms_per_step"]
    return out


# long record: 64 channels x 262,144 samples (fs 512 Hz), 256 directions,
# 12 IMF slots x 10 sifts (fixed mode); beyond the reference's int32 indexing
LONG = dict(workload="long64_262144_k256_fixed", C=64, L=262144, K=256, num_imfs=12, max_iter=10, fs=512.0,
            warmup=1, steps=1, seed=500)
# wide record: 128 channels x 10,000 samples (fs 256 Hz), 256 directions,
# 9 IMF slots x 10 sifts (fixed mode)
WIDE = dict(workload="wide128_10000_k256_fixed", C=128, L=10000, K=256, num_imfs=9, max_iter=10, fs=256.0,
            warmup=1, steps=2, seed=700)


def single_record(rank, Lr):
    """Mixed-form channel-samples/s on one record (the long or the wide one),
    the per-IMF gate against the FP64 path, and the mean HBM rate of the
    decomposition's algorithmic traffic (knot arrays and signal, from a traced
    run's knot counts)."""
    import torch

    import memd_gb300 as mg

    C, L, K, NI, IT = Lr["C"], Lr["L"], Lr["K"], Lr["num_imfs"], Lr["max_iter"]
    y = mg.synth_eeg(C, L, Lr["fs"], seed=Lr["seed"] + rank).astype(np.float32)
    d32 = mg.directions(C, K, dtype="f32")
    stream = torch.cuda.current_stream()
    out = {"workload": Lr["workload"], "C": C, "L": L, "K": K, "num_imfs": NI, "max_iter": IT}
    res = {}
    for name, prec, tdt in (("mixed", mg.PREC_MIXED, torch.float32), ("fp64", mg.PREC_F64, torch.float64)):
        plan = mg.Plan(C, L, K, NI, IT, precision=prec, tuning="auto")
        dy = torch.as_tensor(y, dtype=tdt, device="cuda")
        o = torch.empty((NI, C, L), dtype=tdt, device="cuda")
        d = d32.to(tdt)
        m = measure_replicated(lambda: plan.run(dy, d, o, stream=stream, stats=False), float(C * L), Lr["steps"],
                               Lr["warmup"], CudaSteps(stream), sync=torch.cuda.synchronize)
        ms = m["ms_per_step"]
        st = plan.run(dy, d, o)
        entry = {"ms_per_step": ms, "channel_samples_per_s": m["value"],
                 "workspace_gb": plan.workspace_bytes / 1e9, "flags": int(st.flags)}
        if name == "mixed":
            plan.set_trace(True)
            plan.run(dy, d, o)
            sum_E = float(plan.trace()["count"][: NI - 1, :IT].astype(np.int64).sum())
            plan.set_trace(False)
            work = stage_work(C, L, K, (NI - 1) * IT, sum_E, 8, cum=True)
            tot_bytes = sum(w["bytes"] for w in work.values())
            meas = {}
            pp = os.path.join(REPO, "MEASURED_PEAKS.json")
            if os.path.exists(pp):
                meas = json.load(open(pp))
            peak = meas.get("hbm_gbs", 6800.0)
            entry["alg_hbm_gbs"] = tot_bytes / (ms / 1e3) / 1e9
            entry["alg_hbm_frac_of_measured_peak"] = entry["alg_hbm_gbs"] / peak
        out[name] = entry
        res[name] = o.cpu().numpy().astype(np.float64)
        plan.close()
        del dy, o
        torch.cuda.empty_cache()
    rl = [rel_l2(res["mixed"][i], res["fp64"][i]) for i in range(NI)]
    out["precision_gate"] = {"rel_l2_per_imf_vs_fp64": rl, "max": max(rl), "passed": max(rl) <= GATE}
    out["mixed_over_fp64"] = out["fp64"]["ms_per_step"] / out["mixed"]["ms_per_step"]
    return out


def cpu_baseline(y, dirs, reps: int = 1):
    """The FP64 OpenMP oracle (a transcription of the reference algorithm) on
    the machine's host cores: the full decomposition of the benchmark record, all
    80 sifts, nothing scaled."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle

    C, L = y.shape
    best = None
    for _ in range(reps):
        t0 = time.perf_counter()
        oracle.memd(y, dirs, WL["num_imfs"], WL["max_iter"])
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    return {"value": C * L / best, "unit": "channel-samples/s", "cores": oracle.max_threads(),
            "kind": "port", "sample": f"one full decomposition of the benchmark record ({SIFTS} sifts), {best:.2f} s",
            "nproc": os.cpu_count()}


# ----------------------------------------------------------------------------
# the reference's own CUDA build (oracle/_ref, FP32 as shipped) on this GPU
# ----------------------------------------------------------------------------
def reference_gpu(y, repeats: int = 3):
    exe = os.path.join(REPO, "oracle", "_ref", "memd_ref_f32")
    if not os.path.exists(exe):
        return {"unavailable": "reference build not present (oracle/_ref)"}
    C, L = y.shape
    with tempfile.TemporaryDirectory() as td:
        inp = os.path.join(td, "in.bin")
        y.astype(np.float32).tofile(inp)
        cmd = [exe, inp, str(C), str(WL["K"]), str(WL["num_imfs"]), str(WL["max_iter"]),
               os.path.join(td, "out.bin"), "-", str(repeats)]
        p = subprocess.run(cmd, capture_output=True, text=True, timeout=1200)
    try:
        r = json.loads(p.stdout.strip().splitlines()[-1])
    except Exception:
        return {"unavailable": f"reference run failed rc={p.returncode}: {p.stderr[-300:]}"}
    if "unavailable" in r:
        return r
    return {"precision": "f32 (as shipped)", "best_call_ms": r["best_call_ms"], "best_loop_s": r["best_loop_s"],
            "channel_samples_per_s_call": C * L / (r["best_call_ms"] / 1e3),
            "channel_samples_per_s_loop": C * L / r["best_loop_s"], "repeats": repeats,
            "note": "call = cudaEvents around memd() incl. its workspace allocation; loop = its own omp_get_wtime"}


# ----------------------------------------------------------------------------
# reference arm: the CPU transcription of the reference algorithm
# ----------------------------------------------------------------------------
def run_reference(args):
    """CPU arm: the FP64 OpenMP oracle (oracle/, a restatement of the
    reference algorithm, which the reference itself implements only in CUDA),
    every step one full decomposition of the benchmark record on all host
    threads.  Only rank 0 works; it loads oracle/liboracle.so and nothing of
    the CUDA library."""
    ws, rank, local = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle

    C, L, K, NI, IT = WL["C"], WL["L"], WL["K"], WL["num_imfs"], WL["max_iter"]
    y = bench_record(0)
    # the GPU arm's direction set: float32 Hammersley directions widened to float64
    dirs = oracle.directions(C, K, dtype=np.float32).astype(np.float64)
    for _ in range(args.warmup):
        oracle.memd(y, dirs, NI, IT)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.memd(y, dirs, NI, IT)
        times.append(time.perf_counter() - t0)
    per_step = float(np.mean(times))
    value = C * L / per_step
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": "channel-samples/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": per_step * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic EEG-shaped (seeded numpy generator, rounded to float32), the GPU arm's record",
        "config": bench_config(ws),
        "sift_iters_per_s": SIFTS / per_step,
        "cpu_baseline": {"value": value, "unit": "channel-samples/s", "cores": oracle.max_threads(),
                         "kind": "port",
                         "sample": f"each step: one full decomposition ({SIFTS} sifts) of the benchmark record, "
                                   f"mean of {args.steps} steps"},
        "e2e": {"value": value, "unit": "channel-samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference implements this path only as CUDA (no CPU code); its CPU arm is the FP64 OpenMP "
                "transcription (oracle/), timed on all host threads; the reference's own CUDA build on the GPU is "
                "the reference_gpu entry of the GPU arm's line",
    }
    print(json.dumps(line))


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)
