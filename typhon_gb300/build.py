"""Build libtyphon_gpu.so in-tree for sm_103a (GB300).

Host sources are compiled with g++ and -ffp-contract=off (no fused multiply-add in the
set-up arithmetic, on x86-64 and on aarch64 alike); the kernels with nvcc, once per
arithmetic mode: kernels_exact.cu with -fmad=false, kernels_fast.cu with fused
multiply-add.  Output: typhon_gb300/_lib/libtyphon_gpu.so.
"""
import os
import pathlib
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parent
SRC = HERE / "csrc"
OUT_DIR = HERE / "_lib"
OBJ_DIR = HERE / "_build"
LIB = OUT_DIR / "libtyphon_gpu.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and (pathlib.Path(c) / "bin" / "nvcc").exists():
            return pathlib.Path(c)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return pathlib.Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(map(str, cmd)) + "\n" + r.stdout + r.stderr)
    return r.stderr


def sources():
    return sorted(SRC.glob("*.cpp")) + sorted(SRC.glob("*.cu")) + sorted(SRC.glob("*.cuh")) + \
        sorted(SRC.glob("*.hpp")) + [ROOT / "include" / "typhon_gpu.h"]


def up_to_date():
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in sources())


def build_fp64_probe():
    """The FP64/FP32 throughput probe that bench.py runs (fp64_peak.cu at the repository
    root, bench support, not part of the library) -> _build/fp64_peak."""
    out = ROOT / "_build" / "fp64_peak"
    src = ROOT / "fp64_peak.cu"
    if out.exists() and out.stat().st_mtime >= src.stat().st_mtime:
        return out
    out.parent.mkdir(exist_ok=True)
    _run([str(cuda_home() / "bin" / "nvcc"), "-O3", ARCH, "-o", str(out), str(src)])
    return out


def build(force=False, verbose=False):
    """Compile and link; returns the path of the shared library."""
    if not force and up_to_date():
        return LIB
    cuda = cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    OUT_DIR.mkdir(exist_ok=True)
    OBJ_DIR.mkdir(exist_ok=True)
    inc = ["-I", str(ROOT / "include"), "-I", str(cuda / "include")]
    jobs = []
    for cpp in sorted(SRC.glob("*.cpp")):
        obj = OBJ_DIR / (cpp.stem + ".o")
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall",
                     *inc, "-c", str(cpp), "-o", str(obj)])
    nvflags = ["-O3", "-std=c++17", ARCH, "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
               "--expt-relaxed-constexpr", "-Xptxas", "-v"]
    for cu, extra in (("kernels_exact.cu", ["-fmad=false"]), ("kernels_fast.cu", ["-fmad=true"]),
                      ("timestep_static.cu", ["-fmad=false"])):
        obj = OBJ_DIR / (pathlib.Path(cu).stem + ".o")
        jobs.append([nvcc, *nvflags, *extra, *inc, "-c", str(SRC / cu), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        logs = list(ex.map(_run, jobs))
    if verbose:
        for lg in logs:
            sys.stderr.write(lg)
    objs = [str(p) for p in sorted(OBJ_DIR.glob("*.o"))]
    tmp = LIB.with_suffix(".so.tmp")
    _run([nvcc, "-shared", ARCH, "-o", str(tmp), *objs, "-lcudart_static", "-lrt", "-lpthread", "-ldl"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
