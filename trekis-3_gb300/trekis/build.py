"""In-tree build of the CUDA library (sm_103a) and of the test oracle.

Each CUDA translation unit is compiled in parallel with one ``-gencode``
(arch=compute_103a, code=sm_103a) and linked into
``trekis-3_gb300/_build/libtrekis_gb300.so``.  No cmake, no pip install:
the same recipe runs on the x86_64 development host (cross-compiling) and on
the aarch64 GPU host.
"""
import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess

PKG = pathlib.Path(__file__).resolve().parent.parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libtrekis_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
# The track-loop kernels: single-precision division and square root to about
# one ulp and FP32 denormals flushed.  These flags touch only FP32 arithmetic,
# so FP64 runs keep IEEE division and square root (and their oracle parity).
_FAST32 = ["--prec-div=false", "--prec-sqrt=false", "--ftz=true"]
PER_FILE_FLAGS = {"mc_f32": _FAST32, "mc_f64": _FAST32, "mc_tally": _FAST32,
                  # host-only output code: no fused multiply-add, so sums print the same on every host
                  "output": ["-Xcompiler", "-ffp-contract=off"]}


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and pathlib.Path(c).exists():
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build_library(verbose=False, extra=()):
    OUT.mkdir(exist_ok=True)
    srcs = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))   # .cpp: host-only units
    deps = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + [ROOT / "include" / "trekis_gb300.h"]
    newest_dep = max(p.stat().st_mtime for p in deps)
    objs = []
    jobs = []
    for s in srcs:
        o = OUT / (s.stem + ".o")
        objs.append(o)
        if not o.exists() or o.stat().st_mtime < max(s.stat().st_mtime, newest_dep):
            jobs.append([nvcc(), *ARCH, *NVCC_FLAGS, *PER_FILE_FLAGS.get(s.stem, []), *extra, "-c", str(s), "-o",
                         str(o)])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    if jobs or not LIB.exists():
        _run([nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"])
    return LIB


def build_oracle():
    """Compile the FP64 oracle (test infrastructure) with its Makefile."""
    _run(["make", "-s", "-C", str(ROOT / "oracle")])
    return ROOT / "oracle" / "_build" / "liboracle.so"
