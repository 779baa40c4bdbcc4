"""Build recipe for the oracle (test infrastructure): compiles smob_oracle.cpp into oracle/_build/liboracle.so."""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SRC = os.path.join(HERE, "smob_oracle.cpp")


def build(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "smob_oracle.h"))):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    # -ffp-contract=off: every product and sum rounded as written, on x86 and on Arm alike (GCC fuses
    # them into FMAs by default where the target has FMA), so boundary decisions such as the near-pair
    # rule are the IEEE evaluation of the expression
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-fno-math-errno", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", tmp, SRC]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
