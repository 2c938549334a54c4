"""Builds, from the reference's own sources where they lie, three host
libraries into oracle/_ref/ (never committed; test infrastructure):

* libref_dials.so: the per-dial response functions (src/Utils/include/
  Calculate*.h, header-only) behind oracle/ref/ref_dials.cpp;
* libref_cache.so: GUNDAM's Cache::Manager calculators compiled for the host
  (src/CacheManager/src/{CacheParameters, CacheWeights, WeightBase,
  WeightNormalization, Weight*Spline, WeightGraph, WeightBilinear,
  CacheRecursiveSums, CacheAtomicCAS}.cpp with HEMI_CUDA_DISABLE and the
  stand-in headers of oracle/ref/stubs/) behind oracle/ref/ref_cache.cpp;
* libref_llh.so: GUNDAM's per-bin likelihood classes (src/StatisticalInference/
  JointProbability/include/{PoissonLogLikelihood, BarlowBeestonBanff2022}.h,
  header-only, with the stand-ins of oracle/ref/stubs/) behind
  oracle/ref/ref_llh.cpp.

Usage: python oracle/ref/build_ref.py <path of the GUNDAM source tree>
"""
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE.parent / "_ref"


def main(reference: str) -> None:
    inc = Path(reference) / "src" / "Utils" / "include"
    if not inc.is_dir():
        raise SystemExit(f"no reference headers under {inc}")
    OUT.mkdir(exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-w",
           "-I", str(inc), str(HERE / "ref_dials.cpp"), "-o", str(OUT / "libref_dials.so")]
    subprocess.run(cmd, check=True)
    cm = Path(reference) / "src" / "CacheManager"
    units = ["CacheParameters", "CacheWeights", "WeightBase", "WeightNormalization", "WeightMonotonicSpline",
             "WeightUniformSpline", "WeightGeneralSpline", "WeightCompactSpline", "WeightGraph", "WeightBilinear",
             "CacheRecursiveSums", "CacheAtomicCAS"]
    srcs = [str(cm / "src" / f"{u}.cpp") for u in units]
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-w", "-DHEMI_CUDA_DISABLE",
           "-I", str(HERE / "stubs"), "-I", str(cm / "include"), "-I", str(inc),
           str(HERE / "ref_cache.cpp"), *srcs, "-o", str(OUT / "libref_cache.so")]
    subprocess.run(cmd, check=True)
    jp = Path(reference) / "src" / "StatisticalInference" / "JointProbability" / "include"
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-w",
           "-I", str(HERE / "stubs"), "-I", str(jp), str(HERE / "ref_llh.cpp"), "-o", str(OUT / "libref_llh.so")]
    subprocess.run(cmd, check=True)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: python oracle/ref/build_ref.py <path of the GUNDAM source tree>")
    main(sys.argv[1])
