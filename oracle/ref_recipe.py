"""Recipe that builds the reference MEMD implementation as a checker.

TEST INFRASTRUCTURE ONLY.  Two steps:

generate()  -- run where the reference checkout is present (its directory is
               the argument, else $MEMD_REFERENCE_DIR, else the checkout this
               build was set up with): reads memReducedEpochs_dev.cu from it
               and writes two patched copies into oracle/_ref/ (git-ignored,
               never committed), plus a copy of the reference's input fixture
               EEGsample_32CH_30504.bin (data, used as a parity input):
                 * memd_ref_f32.cu: the reference as shipped, with
                   - line 1472 ("configuration for the input signal", a stray
                     text line that stops nvcc) turned into a comment,
                   - its main() renamed so ref_driver.cu can supply one,
                   - two test hooks that change no arithmetic: after each
                     D2H copy of the knot counts (:1228 maxima, :1285 minima)
                     REF_TRACE_HOOK records every direction's knot count and
                     index-set hash (ref_driver.cu, when asked), and the
                     fixed 4 MiB gtsv2 buffer (:1144) is allocated with
                     REF_GTSV_BUFFER_BYTES (the larger of 4 MiB and the
                     library's own size query for the longest possible knot
                     list), while REF_GTSV_CHECK compares every per-direction
                     size query (:1237, :1295) with what was allocated;
                 * memd_ref_f64.cu: the same plus the FP64 switch of the
                   library calls the reference hard-wires to FP32
                   (cublasSgemm -> cublasDgemm at :1182,
                    cusparseSgtsv2_nopivot[_bufferSizeExt] -> D at :1237-1239,
                    :1295-1297, float alpha/beta -> real_t at :1089-1090),
                   with the float-only runBenchmark()/main() (:1370-1529)
                   compiled out.
build()     -- run anywhere with nvcc (here and on the GPU host, where the
               generated sources travel with the repository copy): compiles
               ref_driver.cu against each copy into oracle/_ref/memd_ref_<p>.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
DEFAULT_REF = os.environ.get("MEMD_REFERENCE_DIR") or "/root/reference"
FIXTURE = "EEGsample_32CH_30504.bin"
SRC_NAME = "memReducedEpochs_dev.cu"

_SIZE_QUERY = ("cusparseSgtsv2_nopivot_bufferSizeExt(handle_sparse, h_num_extrema[k], SignalDim, currentLowerDia, "
               "currentMiddleDia, currentUpperDia, currentRightDia, h_num_extrema[k], buffer_size);")
_COUNTS_MAX = "cudaMemcpy(h_num_extrema, d_num_extrema_max, NumDirVector * sizeof(coord_t), cudaMemcpyDeviceToHost);"
_COUNTS_MIN = "cudaMemcpy(h_num_extrema, d_num_extrema_min, NumDirVector * sizeof(coord_t), cudaMemcpyDeviceToHost);"
COMMON_PATCHES = [
    ("\n    configuration for the input signal\n", "\n    // configuration for the input signal\n"),
    ("\nint main()\n", "\nint memd_reference_original_main()\n"),
    ("cudaMalloc(&buffer, 1024 * 1024 * sizeof(real_t));",
     "cudaMalloc(&buffer, REF_GTSV_BUFFER_BYTES(1024 * 1024 * sizeof(real_t)));"),
    (_SIZE_QUERY, _SIZE_QUERY + " REF_GTSV_CHECK(*buffer_size);"),
    (_COUNTS_MAX, _COUNTS_MAX + " REF_TRACE_HOOK(0, h_num_extrema, d_compactIndex, SignalLength, SignalDim, NumDirVector);"),
    (_COUNTS_MIN, _COUNTS_MIN + " REF_TRACE_HOOK(1, h_num_extrema, d_compactIndex, SignalLength, SignalDim, NumDirVector);"),
]
F64_PATCHES = [
    ("cublasSgemm(", "cublasDgemm("),
    ("cusparseSgtsv2_nopivot_bufferSizeExt(", "cusparseDgtsv2_nopivot_bufferSizeExt("),
    ("cusparseSgtsv2_nopivot(", "cusparseDgtsv2_nopivot("),
    ("    float alpha = 1;\n", "    real_t alpha = 1;\n"),
    ("    float beta = 0;\n", "    real_t beta = 0;\n"),
    # runBenchmark() and main() call memd<int, float>, which no longer compiles
    # once the library calls are FP64; the driver supplies its own main().
    ("\nvoid runBenchmark()\n", "\n#if 0 /* float-only drivers */\nvoid runBenchmark()\n"),
]
EXPECTED_COUNTS = {
    _SIZE_QUERY: 2,
    "cublasSgemm(": 1,
    "cusparseSgtsv2_nopivot_bufferSizeExt(": 2,
    "cusparseSgtsv2_nopivot(": 2,
}


def _apply(text: str, patches) -> str:
    for old, new in patches:
        n = text.count(old)
        want = EXPECTED_COUNTS.get(old, 1)
        if n != want:
            raise RuntimeError(f"patch anchor {old!r} found {n} times, expected {want}")
        text = text.replace(old, new)
    return text


def generate(ref_dir: str = DEFAULT_REF) -> bool:
    src = os.path.join(ref_dir, SRC_NAME)
    if not os.path.exists(src):
        return False
    with open(src, "r", encoding="utf-8-sig", newline="") as f:
        text = f.read().replace("\r\n", "\n")
    os.makedirs(OUT, exist_ok=True)
    f32 = _apply(text, COMMON_PATCHES)
    f64 = _apply(f32, F64_PATCHES).rstrip("\n") + "\n#endif /* float-only drivers */\n"
    for name, body in (("memd_ref_f32.cu", f32), ("memd_ref_f64.cu", f64)):
        path = os.path.join(OUT, name)
        old = None
        if os.path.exists(path):
            with open(path) as f:
                old = f.read()
        if old != body:
            with open(path, "w") as f:
                f.write(body)
    fx = os.path.join(ref_dir, FIXTURE)
    if os.path.exists(fx):
        dst = fixture_path()
        if not os.path.exists(dst) or os.path.getsize(dst) != os.path.getsize(fx):
            shutil.copyfile(fx, dst)
    return True


def fixture_path() -> str:
    """Where generate() leaves the reference's input fixture (32 x 30,504
    float32, channel-major); absent where the reference was never present."""
    return os.path.join(OUT, FIXTURE)


def binary(prec: str) -> str:
    return os.path.join(OUT, f"memd_ref_{prec}")


def _compile(prec: str) -> str:
    src = os.path.join(OUT, f"memd_ref_{prec}.cu")
    out = binary(prec)
    drv = os.path.join(HERE, "ref_driver.cu")
    if os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(src), os.path.getmtime(drv)):
        return out
    real = "float" if prec == "f32" else "double"
    cmd = ["nvcc", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17",
           "-w", "-Xcompiler", "-fopenmp", f"-I{OUT}",
           f"-DREF_SOURCE=\"memd_ref_{prec}.cu\"", f"-DREF_REAL={real}",
           f"-DREF_F64={1 if prec == 'f64' else 0}",
           "-o", out, drv, "-lcublas", "-lcusparse", "-lgomp"]
    subprocess.check_call(cmd)
    return out


def build() -> list[str]:
    """Compile whatever generated copies are present.  Returns built paths."""
    if shutil.which("nvcc") is None:
        return []
    precs = [p for p in ("f32", "f64") if os.path.exists(os.path.join(OUT, f"memd_ref_{p}.cu"))]
    if not precs:
        return []
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        return list(ex.map(_compile, precs))


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else DEFAULT_REF
    print("generated:", generate(ref))
    print("built:", build())
