"""Builds oracle/_ref/libref_dials.so from the reference's own dial headers.

Usage: python oracle/ref/build_ref.py <path of the GUNDAM source tree>

Only the header directory src/Utils/include of that tree is read (with -I);
the output goes to oracle/_ref/ and is never committed.
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


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
