"""In-tree build of the native libraries.

- `_build/libwflow_gb300.so`: the CUDA step library (sm_103a only) with its C ABI.
- `_build/libwflow_synth.so`: host-only synthetic catchment generator.
Both are compiled with explicit nvcc / g++ command lines (no CMake, no setuptools), in
parallel, into the package's `_build/` folder.
"""

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

from .abi import BUILD_DIR, LIB_PATH, PKG_ROOT, REPO_ROOT, SYNTH_LIB_PATH

CSRC = PKG_ROOT / "csrc"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Translation units of the step library and their floating-point contraction policy:
# FP64 plain-form kernels are compiled without implicit FMA contraction so that every
# operation rounds like the reference's scalar Float64 code; the split form contracts freely and
# divides in FP32 with the full-range approximate division (2 ulp; its FP32 rates carry 1e-7
# relative error anyway, and every balance quantity is an exact double-FP32 partition). The
# adaptive sub-step selection serves both forms and follows the FP64 policy.
CUDA_UNITS = [
    ("wf_api.cu", []),
    ("wf_plan.cpp", None),
    ("wf_netcdf.cpp", None),
    ("kernels_fp64.cu", ["--fmad=false"]),
    ("kernels_split.cu", ["-prec-div=false"]),
    ("kernels_adaptive.cu", ["--fmad=false"]),
    ("kernels_li.cu", ["--fmad=false"]),
    ("kernels_snow.cu", ["--fmad=false"]),
]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _newer(out, srcs):
    if not out.exists():
        return False
    t = out.stat().st_mtime
    return all(Path(s).stat().st_mtime <= t for s in srcs)


def build_synth(force=False):
    BUILD_DIR.mkdir(exist_ok=True)
    src = CSRC / "synth.cpp"
    if not force and _newer(SYNTH_LIB_PATH, [src]):
        return SYNTH_LIB_PATH
    _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-o", str(SYNTH_LIB_PATH), str(src)])
    return SYNTH_LIB_PATH


def _headers():
    return list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((REPO_ROOT / "include").glob("wflow_gb300*.h"))


def build_cuda(force=False, verbose=False):
    BUILD_DIR.mkdir(exist_ok=True)
    srcs = [CSRC / u for u, _ in CUDA_UNITS]
    if not force and _newer(LIB_PATH, srcs + _headers()):
        return LIB_PATH
    nvcc = _nvcc()
    inc = ["-I", str(REPO_ROOT / "include"), "-I", str(CSRC)]
    objs = []
    cmds = []
    for unit, extra in CUDA_UNITS:
        src = CSRC / unit
        obj = BUILD_DIR / (src.stem + ".o")
        objs.append(obj)
        if unit.endswith(".cpp"):
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-c", "-ffp-contract=off", *inc,
                   "-I", "/usr/local/cuda/include", "-o", str(obj), str(src)]
        else:
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                   "-Xptxas", "-v" if verbose else "-O3", *extra, *inc, "-c", "-o", str(obj), str(src)]
        cmds.append(cmd)
    with ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        logs = list(ex.map(_run, cmds))
    if verbose:
        for l in logs:
            print(l)
    _run([nvcc, *ARCH, "-shared", "--cudart", "static", "-o", str(LIB_PATH), *[str(o) for o in objs]])
    return LIB_PATH


def build_oracle(force=False):
    """Build the CPU oracle (test infrastructure) with its own Makefile."""
    oracle = REPO_ROOT / "oracle"
    cmd = ["make", "-C", str(oracle)]
    if force:
        _run(["make", "-C", str(oracle), "clean"])
    _run(cmd)
    return oracle / "_build" / "liboracle.so"


def build_all(force=False, verbose=False):
    build_synth(force)
    build_cuda(force, verbose)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB_PATH)
