"""In-tree build of the native library and of the CPU oracle.

``build()`` compiles

* ``forkerrenderer_gb300/_build/libforkerrenderer.so``: the host C++ (scene ingest,
  C ABI) with ``g++ -ffp-contract=off`` and the CUDA kernels with
  ``nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo --fmad=false``;
* ``oracle/_build/liboracle.so``: the CPU oracle (test infrastructure).

Translation units compile in parallel; a unit is rebuilt only when it or a
header of its directory changed. No cmake, no torch extension machinery.
"""

from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")
ORACLE = os.path.join(ROOT, "oracle")
ORACLE_BUILD = os.path.join(ORACLE, "_build")

ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build_native(verbose: bool = False) -> str:
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    jobs = []
    objs = []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cpp")) + glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if not _stale(obj, [src] + headers):
            continue
        if src.endswith(".cpp"):
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
                   f"-I{INCLUDE}", f"-I{CSRC}", f"-I{os.path.join(cuda, 'include')}",
                   "-c", src, "-o", obj]
        else:
            cmd = [nvcc, ARCH, "-O3", "-lineinfo", "--fmad=false", "-std=c++17",
                   "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr",
                   f"-I{INCLUDE}", f"-I{CSRC}", "-c", src, "-o", obj]
        jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    lib = os.path.join(BUILD, "libforkerrenderer.so")
    if jobs or not os.path.exists(lib):
        _run([nvcc, ARCH, "-shared", "-o", lib] + objs + ["-lcudart", "-lpthread"])
    if verbose:
        print("built", lib)
    return lib


def build_oracle(verbose: bool = False) -> str:
    os.makedirs(ORACLE_BUILD, exist_ok=True)
    srcs = [os.path.join(ORACLE, "fr_oracle.cpp"), os.path.join(ORACLE, "fr_oracle_tga.cpp")]
    out = os.path.join(ORACLE_BUILD, "liboracle.so")
    deps = srcs + [os.path.join(ORACLE, "fr_oracle.h"),
                   os.path.join(INCLUDE, "fr_sample_tables.h"), os.path.join(INCLUDE, "forkerrenderer.h"), os.path.join(INCLUDE, "fr_batch.h")]
    if _stale(out, deps):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-pthread",
              f"-I{INCLUDE}"] + srcs + ["-o", out])
    if verbose:
        print("built", out)
    return out


def reference_dir() -> str | None:
    """The reference checkout to build the test harness from: FR_REFERENCE_DIR, or
    a sibling directory named `reference` of this repository; None if neither
    holds the reference's src/."""
    for cand in (os.environ.get("FR_REFERENCE_DIR"), os.path.join(os.path.dirname(ROOT), "reference")):
        if cand and os.path.isdir(os.path.join(cand, "src")):
            return cand
    return None


def build_reference(verbose: bool = False) -> str | None:
    """Compiles the reference sources into oracle/_ref when a reference checkout
    is available (reference_dir()); GPU hosts have none."""
    ref = reference_dir()
    if ref is None:
        return None
    _run(["make", "-s", "-C", ROOT, "-f", "oracle/Makefile.ref", f"REF={ref}",
          f"-j{os.cpu_count() or 4}"])
    out = os.path.join(ORACLE, "_ref")
    if verbose:
        print("built", out)
    return out


def build(verbose: bool = False) -> None:
    build_native(verbose)
    build_oracle(verbose)
    build_reference(verbose)


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
