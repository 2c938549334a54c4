"""Builds the native libraries in-tree.

* ``gundam_gb300/_lib/libgw.so``           -- the engine (C ABI in include/gw.h),
  CUDA kernels compiled for sm_103a only.
* ``gundam_gb300/_lib/libgw_workload.so``  -- the synthetic workload generator.
* ``oracle/_build/liboracle.so``           -- the CPU oracle (test infrastructure).
* ``oracle/_ref/libref_dials.so``          -- the reference's own dial headers,
  built only when the environment variable GUNDAM_REFERENCE names the
  reference source tree (see oracle/ref/).

The translation units compile in parallel; a full build takes well under a
minute.  Nothing here links against torch.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "gundam_gb300"
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
INCLUDE = ROOT / "include"
ORACLE = ROOT / "oracle"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgw")


def _cuda_lib_dir(nvcc: str) -> str:
    base = Path(nvcc).resolve().parent.parent
    for sub in ("lib64", "lib", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib"):
        if (base / sub / "libcudart.so").exists() or list((base / sub).glob("libcudart.so*")):
            return str(base / sub)
    return str(base / "lib64")


def _run_all(jobs: list[tuple[str, list[str]]], verbose: bool) -> None:
    procs = []
    for name, cmd in jobs:
        if verbose:
            print("[build]", " ".join(cmd), flush=True)
        procs.append((name, cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for name, cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((name, cmd, out.decode(errors="replace")))
        elif verbose and out:
            sys.stdout.write(out.decode(errors="replace"))
    if failed:
        msg = "\n".join(f"--- {n} failed:\n{' '.join(c)}\n{o}" for n, c, o in failed)
        raise RuntimeError("native build failed\n" + msg)


def build(verbose: bool = False) -> dict[str, Path]:
    """Compiles every native library; returns their paths."""
    nvcc = _nvcc()
    cudalib = _cuda_lib_dir(nvcc)
    LIBDIR.mkdir(exist_ok=True)
    objdir = PKG / "_build"
    objdir.mkdir(exist_ok=True)
    (ORACLE / "_build").mkdir(exist_ok=True)
    cxx = os.environ.get("CXX", "g++")

    common_nv = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", str(INCLUDE), "-I", str(CSRC)]
    units = ["gw_kernels.cu", "gw_lanes.cu", "gw_multi.cu", "gw_ws.cu", "gw_noalloc.cu", "gw_mlp.cu", "gw_engine.cpp"]
    objs = [objdir / (Path(u).stem + ".o") for u in units]
    jobs = [(u, [nvcc, *common_nv, "-c", str(CSRC / u), "-o", str(o)]) for u, o in zip(units, objs)]
    jobs += [
        (
            "gw_workload",
            [cxx, "-std=c++17", "-O2", "-fPIC", "-shared", "-pthread", "-I", str(INCLUDE),
             str(CSRC / "gw_workload.cpp"), "-o", str(LIBDIR / "libgw_workload.so")],
        ),
        (
            "oracle",
            [cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
             str(ORACLE / "oracle.cpp"), "-o", str(ORACLE / "_build" / "liboracle.so")],
        ),
    ]
    # the reference's own sources, compiled into oracle/_ref/ as parity
    # sources for the tests, only when GUNDAM_REFERENCE names their tree
    ref_script = ORACLE / "ref" / "build_ref.py"
    reference = os.environ.get("GUNDAM_REFERENCE", "")
    if reference and ref_script.exists() and (Path(reference) / "src" / "Utils" / "include").is_dir():
        jobs.append(("ref_dials", [sys.executable, str(ref_script), reference]))
    _run_all(jobs, verbose)
    link = [
        nvcc, *ARCH, "-shared", "-cudart", "shared", *[str(o) for o in objs], "-o", str(LIBDIR / "libgw.so"),
        "-Xlinker", f"-rpath,{cudalib}", "-L", cudalib, "-lcudart",
    ]
    _run_all([("link libgw", link)], verbose)
    out = {
        "libgw": LIBDIR / "libgw.so",
        "libgw_workload": LIBDIR / "libgw_workload.so",
        "liboracle": ORACLE / "_build" / "liboracle.so",
    }
    ref = ORACLE / "_ref" / "libref_dials.so"
    if ref.exists():
        out["libref_dials"] = ref
    return out


if __name__ == "__main__":
    for k, v in build(verbose="-v" in sys.argv).items():
        print(k, v)
