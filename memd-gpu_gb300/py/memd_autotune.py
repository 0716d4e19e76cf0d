"""Autotuner of a plan's launch shapes (memd_tuning), persisted to JSON.

The knobs are the ones the C ABI exposes through memd_plan_create_tuned:
the longest and shortest substitution segments, the factorisation rows per
thread, the substitution's work distribution (device work queue pulled by a
persistent grid, or one warp per possible segment), the number of CTAs the
impulse-accumulation mean splits its spans over, and the directions per tile
of the tensor-core projection.  None of them changes what a decomposition
computes beyond rounding; a candidate is accepted only if its extrema index
sets equal the default plan's at every sift and its IMFs agree to 1e-10
(FP64) / 1e-6 (mixed and FP32 forms).

The search is one pass of coordinate descent from the defaults: each knob in
turn takes the value with the lowest median decomposition time (CUDA events,
after a warm-up), the others held at their best so far.

Choices are stored under a key (C, K, L rounded up to a power of two,
precision, single record or batched epochs, fixed or stop mode) in
memd-gpu_gb300/tuning/gb300.json, or the file $MEMD_TUNING_FILE names;
Plan(..., tuning="auto") reads them back.

    python memd-gpu_gb300/py/memd_autotune.py eeg32     # 32 x 30,504, K = 128, mixed and FP64
    python memd-gpu_gb300/py/memd_autotune.py batched   # 64 epochs of 32 channels, L in [1024, 8192], K = 64
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
DEFAULT_FILE = os.path.join(PKG, "tuning", "gb300.json")

PREC_NAMES = {0: "f64", 1: "f32", 2: "mixed"}


def tuning_file() -> str:
    return os.environ.get("MEMD_TUNING_FILE") or DEFAULT_FILE


def shape_key(C: int, K: int, L: int, precision: int, batched: bool, stop: bool) -> str:
    lb = 1
    while lb < L:
        lb <<= 1
    return f"C{C}-K{K}-L{lb}-{PREC_NAMES[int(precision)]}-{'batched' if batched else 'single'}-" \
           f"{'stop' if stop else 'fixed'}"


def config_key(cfg) -> str:
    return shape_key(int(cfg.channels), int(cfg.directions), int(cfg.length), int(cfg.precision),
                     int(cfg.max_epochs) > 0, int(cfg.stop_mode) != 0)


def load(path: str | None = None) -> dict:
    path = path or tuning_file()
    if not os.path.exists(path):
        return {}
    with open(path) as f:
        return json.load(f)


def lookup(cfg, path: str | None = None):
    """The stored launch shapes for a memd_config, or None."""
    e = load(path).get(config_key(cfg))
    return e["choice"] if e else None


def store(key: str, choice: dict, meta: dict, path: str | None = None) -> None:
    path = path or tuning_file()
    data = load(path)
    data[key] = {"choice": choice, **meta}
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def search_space(precision: int, cum: bool) -> dict:
    """Values tried per knob (0 = the default)."""
    f64 = int(precision) == 0
    space = {
        "solve_segment": [0, 128, 512],
        "solve_min_segment": [0, 32, 128],
        "factor_segment": [0, 32, 128] if f64 else [0, 8, 32],
        "solve_queue": [0, 1],
    }
    if cum:
        space["mean_ctas"] = [0, 1024, 4096]
    if int(precision) == 2:
        space["proj_tile_n"] = [0, 32, 128]
    return space


def coordinate_descent(measure, space: dict, valid) -> tuple[dict, float, list]:
    """measure(choice) -> (ms, result); valid(base result, result) -> bool.
    Returns the best choice, its time and the log of every trial."""
    best = {k: 0 for k in space}
    best_ms, base = measure(dict(best))
    log = [{"choice": dict(best), "ms": best_ms, "valid": True}]
    for knob, values in space.items():
        for v in values:
            if v == best[knob]:
                continue
            cand = dict(best)
            cand[knob] = v
            ms, res = measure(cand)
            ok = valid(base, res)
            log.append({"choice": dict(cand), "ms": ms, "valid": ok})
            if ok and ms < best_ms:
                best, best_ms = cand, ms
    return best, best_ms, log


def _equal_runs(tol: float):
    def valid(a, b):
        ta, oa = a
        tb, ob = b
        if not (np.array_equal(ta["count"], tb["count"]) and np.array_equal(ta["hash"], tb["hash"])):
            return False
        for i in range(oa.shape[0]):
            n = np.linalg.norm(oa[i])
            if n > 0 and np.linalg.norm(ob[i] - oa[i]) > tol * n:
                return False
        return True

    return valid


def tune_record(y: np.ndarray, dirs: np.ndarray, num_imfs: int, max_iter: int, precision: int, reps: int = 3,
                persist: bool = True, **cfg):
    """Tune a single-record plan on the record y (C x L) and directions
    (K x C); returns (key, choice, ms, default ms, log)."""
    import torch

    import memd_gb300 as mg

    C, L = y.shape
    K = dirs.shape[0]
    tdt = torch.float64 if precision == mg.PREC_F64 else torch.float32
    dy = torch.as_tensor(y, dtype=tdt, device="cuda")
    dd = torch.as_tensor(dirs, dtype=tdt, device="cuda")
    out = torch.empty((num_imfs, C, L), dtype=tdt, device="cuda")
    cum = precision == mg.PREC_MIXED and cfg.get("stop_mode", 0) == 0 and cfg.get("mean_eval", 0) != 1

    def measure(choice):
        plan = mg.Plan(C, L, K, num_imfs, max_iter, precision=precision, tuning=choice, **cfg)
        plan.set_trace(True)
        plan.run(dy, dd, out)
        tr = plan.trace().copy()
        res = (tr, out.cpu().numpy().astype(np.float64))
        plan.set_trace(False)
        plan.run(dy, dd, out)  # warm-up of the untraced graph
        ts = [plan.run(dy, dd, out).elapsed_ms for _ in range(reps)]
        plan.close()
        return float(np.median(ts)), res

    tol = 1e-10 if precision == mg.PREC_F64 else 1e-6
    best, ms, log = coordinate_descent(measure, search_space(precision, cum), _equal_runs(tol))
    key = shape_key(C, K, L, precision, False, bool(cfg.get("stop_mode", 0)))
    full = mg.Plan(C, L, K, num_imfs, max_iter, precision=precision, tuning=best, **cfg)
    chosen = full.tuning()
    full.close()
    if persist:
        store(key, chosen, {"ms": ms, "default_ms": log[0]["ms"], "workload": f"C{C} L{L} K{K}",
                            "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime()),
                            "device": torch.cuda.get_device_name(0)})
    return key, chosen, ms, log[0]["ms"], log


def tune_batched(recs, dirs: np.ndarray, num_imfs: int, max_iter: int, precision: int, reps: int = 2,
                 persist: bool = True):
    """Tune a batched plan on a list of records (C x L_e each)."""
    import torch

    import memd_gb300 as mg

    C = recs[0].shape[0]
    K = dirs.shape[0]
    lengths = np.array([r.shape[1] for r in recs], dtype=np.int64)
    offs = np.concatenate([[0], np.cumsum(C * lengths)[:-1]]).astype(np.int64)
    tdt = torch.float64 if precision == mg.PREC_F64 else torch.float32
    y = torch.as_tensor(np.concatenate([r.ravel() for r in recs]), dtype=tdt, device="cuda")
    dd = torch.as_tensor(dirs, dtype=tdt, device="cuda")
    out = torch.empty(num_imfs * y.numel(), dtype=tdt, device="cuda")
    Lmax = int(lengths.max())

    def measure(choice):
        plan = mg.Plan(C, Lmax, K, num_imfs, max_iter, precision=precision, max_epochs=len(recs), tuning=choice)
        plan.run_batched(y, lengths, offs, dd, out)
        res = ({"count": np.zeros(1), "hash": np.zeros(1)}, out.cpu().numpy().astype(np.float64)[None, :])
        ts = [plan.run_batched(y, lengths, offs, dd, out).elapsed_ms for _ in range(reps)]
        plan.close()
        return float(np.median(ts)), res

    tol = 1e-10 if precision == mg.PREC_F64 else 1e-6
    best, ms, log = coordinate_descent(measure, search_space(precision, precision == mg.PREC_MIXED),
                                       _equal_runs(tol))
    key = shape_key(C, K, Lmax, precision, True, False)
    full = mg.Plan(C, Lmax, K, num_imfs, max_iter, precision=precision, max_epochs=len(recs), tuning=best)
    chosen = full.tuning()
    full.close()
    if persist:
        store(key, chosen, {"ms": ms, "default_ms": log[0]["ms"], "workload": f"{len(recs)} epochs C{C} K{K}",
                            "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime()),
                            "device": torch.cuda.get_device_name(0)})
    return key, chosen, ms, log[0]["ms"], log


def main(argv):
    sys.path.insert(0, HERE)
    import memd_gb300 as mg
    import memd_signals

    what = argv[1] if len(argv) > 1 else "eeg32"
    if what == "eeg32":
        C, L, K = 32, 30504, 128
        y = memd_signals.as_float32_record(memd_signals.eeg(C, L, 256.0, 0))
        d = mg.directions(C, K, dtype="f32").double().cpu().numpy()
        for prec in (mg.PREC_MIXED, mg.PREC_F64):
            key, choice, ms, ms0, _ = tune_record(y, d, 9, 10, prec)
            print(json.dumps({"key": key, "choice": choice, "ms": ms, "default_ms": ms0}))
    elif what == "batched":
        rng = np.random.default_rng(1000)
        lengths = rng.integers(1024, 8193, size=64)
        C, K = 32, 64
        recs = [memd_signals.as_float32_record(memd_signals.eeg(C, int(L), 256.0, 10_000 + e))
                for e, L in enumerate(lengths)]
        d = mg.directions(C, K, dtype="f32").double().cpu().numpy()
        for prec in (mg.PREC_MIXED, mg.PREC_F64):
            key, choice, ms, ms0, _ = tune_batched(recs, d, 8, 10, prec)
            print(json.dumps({"key": key, "choice": choice, "ms": ms, "default_ms": ms0}))
    else:
        print(__doc__)
        return 2
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
