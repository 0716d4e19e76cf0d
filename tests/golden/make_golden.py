"""Golden vectors from the reference MEMD build.

Step 1 (on a GPU host, needs oracle/_ref built by oracle/ref_recipe.py):
    python tests/golden/make_golden.py run OUTDIR
  writes, per case, the seeded input (raw float64 / float32, C x L channel-major)
  and the reference's outputs: IMFs (num_imfs x C x L) and the direction set the
  reference generated itself (K x C), for the FP64-patched and the as-shipped
  FP32 build.
Step 2 (anywhere):
    python tests/golden/make_golden.py collect OUTDIR
  copies those files into tests/golden/ and writes manifest.json (shapes and
  sha256 of every file).  The committed fixtures are what the tests read; the
  reference itself is never needed at test time.
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

# Small cases: each runs in well under a second on the CPU oracle.
CASES = [
    # sinusoid mixture, the configs[0] signal family at reduced size
    dict(name="tones_c4_l1000_k8", C=4, L=1000, K=8, nimf=5, max_iter=10, kind="tones", seed=1),
    # configs[0] shape (8 ch x 2000, 64 directions), reference fixed mode, 4 IMFs
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


if __name__ == "__main__":
    if len(sys.argv) != 3 or sys.argv[1] not in ("run", "collect"):
        print(__doc__)
        sys.exit(2)
    if sys.argv[1] == "run":
        sys.exit(run(sys.argv[2]))
    collect(sys.argv[2])
