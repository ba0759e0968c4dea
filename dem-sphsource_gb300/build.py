"""Builds the in-tree libraries.

* ``dem-sphsource_gb300/libdemsph_gb300.so`` - the product: CUDA kernels for
  sm_103a (csrc/*.cu, nvcc) and the host API (host/*.cpp, g++), linked into one
  shared library exporting the C ABI of include/demsph_gb300.h.
* ``oracle/liboracle_demsph.so`` - the FP64 CPU oracle (test infrastructure).
* ``oracle/_ref/libref_demsph.so`` - the reference compiled for the CPU, only
  where the reference sources exist (test infrastructure, golden fixtures).

Objects go to ``_build/`` (git-ignored).  Sources compile in parallel and only
when they or a header changed.  No cmake.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libdemsph_gb300.so")
ORACLE_SRC = os.path.join(ROOT, "oracle", "demsph_oracle.cpp")
ORACLE_LIB = os.path.join(ROOT, "oracle", "liboracle_demsph.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nv = shutil.which("nvcc")
    if nv:
        return os.path.dirname(os.path.dirname(os.path.realpath(nv)))
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _headers():
    hs = glob.glob(os.path.join(PKG, "csrc", "*.cuh")) + glob.glob(os.path.join(PKG, "csrc", "*.h"))
    hs += glob.glob(os.path.join(PKG, "host", "*.h")) + glob.glob(os.path.join(ROOT, "include", "*.h"))
    return hs


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


# Per-file flags.  The fluid pair loops (sph.cu, sph_tiles.cu) divide and take square roots
# several times per pair; their approximate forms (a few ulp, far inside the
# stated tolerance against the FP64 oracle) replace the IEEE-rounded ones.
# The double-float helpers call the correctly rounded intrinsics explicitly
# and are unaffected.
#
# The DEM kernels (dem.cu) run the same arithmetic (a pair's contact law, a
# solid's force sum and integration) inside several kernels whose results must
# agree bit for bit (one-launch and two-launch contact forces, the per-solid
# sums with and without the integration pass, staged calls and graphs); no
# product is contracted into an FMA there (-fmad=false), so every kernel rounds
# each operation as the source writes it, whatever code surrounds it.
FILE_FLAGS = {"sph.cu": ["-prec-div=false", "-prec-sqrt=false"],
              "sph_tiles.cu": ["-prec-div=false", "-prec-sqrt=false"],
              "dem.cu": ["-fmad=false"]}


def nvcc_flags(cuda):
    return ["-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
            f"-I{os.path.join(ROOT, 'include')}", f"-I{os.path.join(PKG, 'host')}", "--expt-relaxed-constexpr"]


def cxx_flags(cuda):
    # no FMA contraction: the host code (scene builder, point generators)
    # rounds the same on x86 and Arm, and as the reference's host code does
    return ["-std=c++17", "-O2", "-fPIC", "-fvisibility=hidden", "-ffp-contract=off",
            f"-I{os.path.join(cuda, 'include')}",
            f"-I{os.path.join(ROOT, 'include')}", f"-I{os.path.join(PKG, 'host')}"]


def build_library(verbose=False, ptxas_verbose=False, jobs=None):
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    hdrs = _headers()
    units = []
    for src in sorted(glob.glob(os.path.join(PKG, "csrc", "*.cu"))):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        flags = nvcc_flags(cuda) + FILE_FLAGS.get(os.path.basename(src), []) + (["-Xptxas", "-v"] if ptxas_verbose else [])
        units.append((src, obj, [nvcc, *flags, "-c", src, "-o", obj]))
    for src in sorted(glob.glob(os.path.join(PKG, "host", "*.cpp"))):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        units.append((src, obj, ["g++", *cxx_flags(cuda), "-c", src, "-o", obj]))
    todo = [u for u in units if ptxas_verbose or _stale(u[1], [u[0], *hdrs])]
    logs = {}
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        futs = {ex.submit(_run, cmd, verbose): src for src, _, cmd in todo}
        for f in cf.as_completed(futs):
            logs[futs[f]] = f.result()
    objs = [u[1] for u in units]
    if todo or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        _run([nvcc, "-shared", *ARCH, "-o", tmp, *objs, "-lcudart"], verbose)
        os.replace(tmp, LIB)
    return logs


def build_oracle(verbose=False):
    """The FP64 oracle: plain C++ with OpenMP; no FMA contraction, so x86 and
    Arm builds round identically."""
    if _stale(ORACLE_LIB, [ORACLE_SRC, os.path.join(ROOT, "include", "demsph_gb300.h")]):
        tmp = ORACLE_LIB + ".tmp"
        _run(["g++", "-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
              f"-I{os.path.join(ROOT, 'include')}", ORACLE_SRC, "-o", tmp], verbose)
        os.replace(tmp, ORACLE_LIB)


def build_reference(verbose=False):
    """The reference compiled for the CPU (oracle/build_ref.sh), where its
    sources are: $REF, else a ``reference`` directory beside the repository."""
    ref = os.environ.get("REF") or os.path.join(os.path.dirname(ROOT), "reference")
    if not os.path.isdir(os.path.join(ref, "core")):
        return False
    out = os.path.join(ROOT, "oracle", "_ref", "libref_demsph.so")
    srcs = glob.glob(os.path.join(ref, "core", "*")) + glob.glob(os.path.join(ROOT, "oracle", "refshim", "**", "*.h"),
                                                                   recursive=True)
    srcs.append(os.path.join(ROOT, "oracle", "ref_harness.cpp"))
    if _stale(out, srcs):
        _run(["env", f"REF={ref}", "sh", os.path.join(ROOT, "oracle", "build_ref.sh")], verbose)
    return True


def build_all(verbose=False):
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        f_lib = ex.submit(build_library, verbose)
        f_orc = ex.submit(build_oracle, verbose)
        f_ref = ex.submit(build_reference, verbose)
        f_lib.result()
        f_orc.result()
        f_ref.result()


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
    print("built", LIB)
