"""Build recipe for the C oracle (test infrastructure only).

Compiles oracle/ernn_oracle.c (the ERNN cell and its adjoint) and
oracle/fem_oracle.c (the FEM data generator's time loop) into
oracle/_build/liboracle.so with gcc.  The
product library never links this file; tests, the smoke check and bench.py's
CPU-baseline leg load it through oracle/oracle.py.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "ernn_oracle.c")
IMPL = os.path.join(HERE, "ernn_oracle_impl.h")
FEM_SRC = os.path.join(HERE, "fem_oracle.c")
FEM_IMPL = os.path.join(HERE, "fem_oracle_impl.h")
OUT_DIR = os.path.join(HERE, "_build")
OUT = os.path.join(OUT_DIR, "liboracle.so")


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile the oracle if the shared object is missing or stale; return its path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(OUT):
        newest = max(os.path.getmtime(f) for f in (SRC, IMPL, FEM_SRC, FEM_IMPL, __file__))
        if os.path.getmtime(OUT) >= newest:
            return OUT
    tmp = OUT + f".tmp{os.getpid()}"
    # -ffp-contract=off keeps a*b+c as two roundings, as the reference's
    # elementwise torch ops round them.
    cmd = ["gcc", "-O2", "-std=c99", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-o", tmp, SRC, FEM_SRC, "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
