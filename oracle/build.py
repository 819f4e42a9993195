"""Build recipe for the CPU oracle (test infrastructure, not product code).

Compiles ``ifx_oracle.c`` -- the FP64 C restatement of ImageFiltering.jl's FIR
and rank-filter loops -- into ``oracle/_build/libifx_oracle.so`` with gcc.
``-ffp-contract=off`` keeps every ``tmp += a*k`` as a separate multiply and
add, as the reference loops are written (src/imfilter.jl:660-666, 730-735), on
x86-64 and on aarch64 alike.

The reference itself (Julia) cannot be compiled here: there is no Julia
toolchain, so there is no ``oracle/_ref`` build.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "ifx_oracle.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libifx_oracle.so")


def build(force: bool = False) -> str:
    """Compile the oracle if the library is missing or older than its source."""
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
           "-o", tmp, SRC, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
