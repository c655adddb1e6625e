"""Build recipe for the oracle (test infrastructure only).

Compiles oracle/pf_oracle.c twice -- REAL=double (symbols *_d) and REAL=float
(symbols *_f) -- into oracle/libpf_oracle.so with gcc, OpenMP and
-ffp-contract=off (no fused multiply-add, so x86-64 and aarch64 give the same
bits).  The reference itself is Fortran and no Fortran compiler exists in the
build container, so there is no oracle/_ref build of it.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "pf_oracle.c")
LIB = os.path.join(HERE, "libpf_oracle.so")
CFLAGS = ["-O3", "-fPIC", "-fopenmp", "-ffp-contract=off", "-std=c11", "-Wall", "-Wno-unknown-pragmas"]


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    objs = []
    for real, sfx in (("double", "_d"), ("float", "_f")):
        obj = os.path.join(HERE, f"pf_oracle{sfx}.o")
        cmd = ["gcc", *CFLAGS, f"-DREAL={real}", f"-DSFX={sfx}", "-c", SRC, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        subprocess.check_call(cmd)
        objs.append(obj)
    tmp = LIB + ".tmp"
    cmd = ["gcc", "-shared", "-fopenmp", *objs, "-o", tmp, "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    for o in objs:
        os.remove(o)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
