"""Build recipe for the CPU oracle (test infrastructure, not the product).

Compiles oracle/dem_oracle.c into oracle/_build/liborc.so with gcc.  The flags
matter: -ffp-contract=off keeps every float expression rounded as written
(gcc on aarch64 would otherwise fuse a*b+c), -fno-strict-aliasing because the
reference's contact/bond records are viewed both as int32 words and as structs.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = [os.path.join(HERE, "dem_oracle.c")]
DEPS = SRC + [os.path.join(HERE, "dem_oracle.h"), os.path.join(HERE, "dem_oracle_step.inc")]
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liborc.so")
CFLAGS = ["-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
          "-fno-strict-aliasing", "-fno-fast-math", "-Wall", "-Wno-unused-function"]


def build(force=False, verbose=False):
    """Compile liborc.so if it is missing or older than its sources; return its path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in DEPS):
            return LIB
    cmd = ["gcc"] + CFLAGS + SRC + ["-o", LIB + ".tmp", "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
