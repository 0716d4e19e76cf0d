"""Golden vectors from the reference MEMD build.

Step 1 (on a GPU host, needs oracle/_ref built by oracle/ref_recipe.py):
    python tests/golden/make_golden.py run OUTDIR
  writes, per small case, the seeded input (raw float64 / float32, C x L
  channel-major) and the reference's outputs: IMFs (num_imfs x C x L) and the
  direction set the reference generated itself (K x C), for the FP64-patched
  and the as-shipped FP32 build.
    python tests/golden/make_golden.py run-scale OUTDIR
  runs the FP64-patched reference on the full-size cases (SCALE_CASES: the
  reference's own fixture EEGsample_32CH_30504.bin with its main()'s C = 32,
  K = 64, 9 slots x 10 sifts, and the 32 x 30,504 x 128 benchmark record) with
  its extrema dump hook on, and keeps: the reference's knot count and index-set
  hash for every (IMF, sift, direction, envelope), its directions, the IMF
  values at 4096 seeded (channel, sample) positions, and per-IMF per-channel
  norms (the full IMFs are 70 MB a case; the GPU tests compare the full IMFs
  with the CPU oracle instead).
Step 2 (anywhere):
    python tests/golden/make_golden.py collect OUTDIR
    python tests/golden/make_golden.py collect-scale OUTDIR
  copies those files into tests/golden/ and writes manifest.json /
  manifest_scale.json (shapes and sha256 of every file).  The committed
  fixtures are what the tests read; the reference itself is never needed at
  test time (the fixture-based case reads the copy of the reference's input
  that oracle/ref_recipe.py leaves in oracle/_ref/).
"""
from __future__ import annotations

import hashlib
import json
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
for _sub in ("memd-gpu_gb300/py", "oracle"):
    _p = os.path.join(REPO, _sub)
    if _p not in sys.path:
        sys.path.insert(0, _p)

# Small cases: each runs in well under a second on the CPU oracle.
CASES = [
    # sinusoid mixture (the 8-channel tone workload's signal family), reduced size
    dict(name="tones_c4_l1000_k8", C=4, L=1000, K=8, nimf=5, max_iter=10, kind="tones", seed=1),
    # the tone workload's shape (8 ch x 2000, 64 directions), reference fixed mode, 4 IMFs
    dict(name="tones_c8_l2000_k64", C=8, L=2000, K=64, nimf=4, max_iter=10, kind="tones", seed=0),
    # L = 4096: the reference extrema launch skips 14 interior samples
    dict(name="pink_c2_l4096_k16", C=2, L=4096, K=16, nimf=5, max_iter=6, kind="pink", seed=2),
    # C = 1 (single channel, one coordinate per direction) and odd L
    dict(name="pink_c1_l777_k4", C=1, L=777, K=4, nimf=4, max_iter=8, kind="pink", seed=3),
]


def make_input(case) -> np.ndarray:
    rng = np.random.default_rng(case["seed"])
    C, L = case["C"], case["L"]
    if case["kind"] == "tones":
        t = np.arange(L) / 1000.0
        y = np.zeros((C, L))
        for c in range(C):
            for f in (5.0, 20.0, 60.0):
                y[c] += rng.uniform(0.5, 1.5) * np.sin(2 * np.pi * f * t + rng.uniform(0, 2 * np.pi))
            y[c] += 0.1 * rng.standard_normal(L)
    else:
        # 1/f noise by spectral shaping of white noise
        w = rng.standard_normal((C, L))
        F = np.fft.rfft(w, axis=1)
        f = np.arange(F.shape[1], dtype=np.float64)
        f[0] = 1.0
        y = np.fft.irfft(F / np.sqrt(f), n=L, axis=1)
        y /= y.std(axis=1, keepdims=True)
    return np.ascontiguousarray(y, dtype=np.float64)


def run(outdir: str) -> int:
    os.makedirs(outdir, exist_ok=True)
    log = []
    rc_all = 0
    for case in CASES:
        y = make_input(case)
        base = os.path.join(outdir, case["name"])
        y.tofile(base + ".in_f64.bin")
        y.astype(np.float32).tofile(base + ".in_f32.bin")
        for prec in ("f64", "f32"):
            exe = os.path.join(REPO, "oracle", "_ref", f"memd_ref_{prec}")
            cmd = [exe, f"{base}.in_{prec}.bin", str(case["C"]), str(case["K"]), str(case["nimf"]),
                   str(case["max_iter"]), f"{base}.ref_{prec}.bin", "-", "1"]
            p = subprocess.run(cmd, capture_output=True, text=True)
            log.append({"case": case["name"], "prec": prec, "rc": p.returncode,
                        "stdout": p.stdout.strip(), "stderr": p.stderr.strip()[-2000:]})
            rc_all |= p.returncode
    with open(os.path.join(outdir, "run_log.json"), "w") as f:
        json.dump(log, f, indent=1)
    print(json.dumps(log, indent=1))
    return rc_all


def _sha(path: str) -> str:
    h = hashlib.sha256()
    with open(path, "rb") as f:
        h.update(f.read())
    return h.hexdigest()


def collect(outdir: str) -> None:
    manifest = {"generator": "tests/golden/make_golden.py", "cases": []}
    for case in CASES:
        entry = dict(case)
        entry["files"] = {}
        for suffix in ("in_f64.bin", "in_f32.bin", "ref_f64.bin", "ref_f64.bin.dirs",
                       "ref_f32.bin", "ref_f32.bin.dirs"):
            src = os.path.join(outdir, f"{case['name']}.{suffix}")
            dst = os.path.join(HERE, f"{case['name']}.{suffix}")
            shutil.copyfile(src, dst)
            entry["files"][suffix] = {"sha256": _sha(dst), "bytes": os.path.getsize(dst)}
        manifest["cases"].append(entry)
    log_path = os.path.join(outdir, "run_log.json")
    if os.path.exists(log_path):
        with open(log_path) as f:
            manifest["reference_run_log"] = json.load(f)
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)


def load_case(name: str) -> dict:
    """Read a committed case: input, reference IMFs and directions."""
    with open(os.path.join(HERE, "manifest.json")) as f:
        man = json.load(f)
    case = next(c for c in man["cases"] if c["name"] == name)
    C, L, K, nimf = case["C"], case["L"], case["K"], case["nimf"]
    out = dict(case)
    for prec, dt in (("f64", np.float64), ("f32", np.float32)):
        p = lambda s: os.path.join(HERE, f"{name}.{s}")
        out[f"in_{prec}"] = np.fromfile(p(f"in_{prec}.bin"), dtype=dt).reshape(C, L)
        out[f"ref_{prec}"] = np.fromfile(p(f"ref_{prec}.bin"), dtype=dt).reshape(nimf, C, L)
        out[f"dirs_{prec}"] = np.fromfile(p(f"ref_{prec}.bin.dirs"), dtype=dt).reshape(K, C)
    return out


# Full-size cases, FP64 reference build only.
SCALE_CASES = [
    # the reference's own main(): its fixture, C = 32, K = 64, 9 slots x 10 sifts
    # (memReducedEpochs_dev.cu:1473-1476, 1484)
    dict(name="eegfixture_c32_l30504_k64", C=32, L=30504, K=64, nimf=9, max_iter=10, kind="fixture"),
    # the benchmark record: 32 x 30,504 EEG-shaped (seed 0, rounded to float32), K = 128
    dict(name="eegsynth_c32_l30504_k128", C=32, L=30504, K=128, nimf=9, max_iter=10, kind="synth", seed=0,
         fs=256.0),
]
NSUB = 4096
SUB_SEED = 2024


def scale_input(case) -> np.ndarray | None:
    """The case's C x L float64 input, or None when the reference fixture copy
    (oracle/_ref) is absent."""
    if case["kind"] == "fixture":
        import ref_recipe

        path = ref_recipe.fixture_path()
        if not os.path.exists(path):
            return None
        y = np.fromfile(path, dtype=np.float32)
        return y.reshape(case["C"], case["L"]).astype(np.float64)
    import memd_signals

    return memd_signals.as_float32_record(memd_signals.eeg(case["C"], case["L"], case["fs"], case["seed"]))


def sub_positions(case) -> np.ndarray:
    """Seeded flat (channel * L + sample) positions where IMF values are kept."""
    rng = np.random.default_rng(SUB_SEED)
    return np.sort(rng.choice(case["C"] * case["L"], size=NSUB, replace=False)).astype(np.int64)


def input_sha(y: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(y, dtype=np.float64).tobytes()).hexdigest()


def run_scale(outdir: str) -> int:
    os.makedirs(outdir, exist_ok=True)
    log = []
    rc_all = 0
    exe = os.path.join(REPO, "oracle", "_ref", "memd_ref_f64")
    for case in SCALE_CASES:
        y = scale_input(case)
        if y is None:
            log.append({"case": case["name"], "skipped": "reference fixture copy absent"})
            continue
        base = os.path.join(outdir, case["name"])
        inp = base + ".in_f64.bin"
        y.tofile(inp)
        out = base + ".ref_f64.bin"
        env = dict(os.environ, MEMD_REF_TRACE=base + ".ref_f64.trace")
        cmd = [exe, inp, str(case["C"]), str(case["K"]), str(case["nimf"]), str(case["max_iter"]), out, "-", "1"]
        p = subprocess.run(cmd, capture_output=True, text=True, env=env)
        log.append({"case": case["name"], "prec": "f64", "rc": p.returncode, "stdout": p.stdout.strip(),
                    "stderr": p.stderr.strip()[-2000:], "input_sha256": input_sha(y)})
        rc_all |= p.returncode
        if p.returncode == 0:
            C, L, nimf = case["C"], case["L"], case["nimf"]
            imfs = np.fromfile(out, dtype=np.float64).reshape(nimf, C * L)
            np.ascontiguousarray(imfs[:, sub_positions(case)]).tofile(base + ".ref_f64.sub")
            np.linalg.norm(imfs.reshape(nimf, C, L), axis=2).tofile(base + ".ref_f64.norms")
        os.remove(inp)
        if os.path.exists(out):
            os.remove(out)
    with open(os.path.join(outdir, "run_scale_log.json"), "w") as f:
        json.dump(log, f, indent=1)
    print(json.dumps(log, indent=1))
    return rc_all


def collect_scale(outdir: str) -> None:
    with open(os.path.join(outdir, "run_scale_log.json")) as f:
        log = json.load(f)
    manifest = {"generator": "tests/golden/make_golden.py run-scale", "nsub": NSUB, "sub_seed": SUB_SEED,
                "trace_record": "int32 count, int32 0, uint64 sum of splitmix64(n); order [imf][sift][env][k]",
                "cases": []}
    for case in SCALE_CASES:
        entry = dict(case)
        run = next((r for r in log if r["case"] == case["name"]), None)
        if run is None or run.get("rc") != 0:
            continue
        entry["input_sha256"] = run["input_sha256"]
        entry["reference_run"] = {k: run[k] for k in ("stdout", "stderr")}
        entry["files"] = {}
        for suffix in ("ref_f64.trace", "ref_f64.sub", "ref_f64.norms", "ref_f64.bin.dirs"):
            src = os.path.join(outdir, f"{case['name']}.{suffix}")
            dst = os.path.join(HERE, f"{case['name']}.{suffix}")
            shutil.copyfile(src, dst)
            entry["files"][suffix] = {"sha256": _sha(dst), "bytes": os.path.getsize(dst)}
        manifest["cases"].append(entry)
    with open(os.path.join(HERE, "manifest_scale.json"), "w") as f:
        json.dump(manifest, f, indent=1)


TRACE_REC = np.dtype([("count", "<i4"), ("flags", "<i4"), ("hash", "<u8")])


def load_scale_case(name: str) -> dict:
    """A committed full-size case: the reference's trace as [imf][sift][k][env]
    (the layout of the library's trace), IMF values at the seeded positions,
    per-IMF per-channel norms and the reference's directions."""
    with open(os.path.join(HERE, "manifest_scale.json")) as f:
        man = json.load(f)
    case = dict(next(c for c in man["cases"] if c["name"] == name))
    C, L, K, nimf, it = case["C"], case["L"], case["K"], case["nimf"], case["max_iter"]
    p = lambda s: os.path.join(HERE, f"{name}.{s}")
    tr = np.fromfile(p("ref_f64.trace"), dtype=TRACE_REC).reshape(nimf - 1, it, 2, K)
    case["trace"] = np.ascontiguousarray(tr.transpose(0, 1, 3, 2))
    case["sub"] = np.fromfile(p("ref_f64.sub"), dtype=np.float64).reshape(nimf, NSUB)
    case["norms"] = np.fromfile(p("ref_f64.norms"), dtype=np.float64).reshape(nimf, C)
    case["dirs"] = np.fromfile(p("ref_f64.bin.dirs"), dtype=np.float64).reshape(K, C)
    case["positions"] = sub_positions(case)
    return case


if __name__ == "__main__":
    if len(sys.argv) != 3 or sys.argv[1] not in ("run", "collect", "run-scale", "collect-scale"):
        print(__doc__)
        sys.exit(2)
    if sys.argv[1] == "run":
        sys.exit(run(sys.argv[2]))
    if sys.argv[1] == "run-scale":
        sys.exit(run_scale(sys.argv[2]))
    if sys.argv[1] == "collect-scale":
        collect_scale(sys.argv[2])
    else:
        collect(sys.argv[2])
