"""Build the CPU oracle (test infrastructure) into oracle/_build/.

gcc only, one translation unit, OpenMP over scenarios.  The product library
never links this file.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libgp_oracle.so")


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "gp_oracle.c")
    hdr = os.path.join(os.path.dirname(HERE), "include", "gradpower_gb300.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-std=c11", "-fno-fast-math",
           "-ffp-contract=off", "-o", LIB + ".tmp", src, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
