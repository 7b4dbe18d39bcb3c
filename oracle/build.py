"""Build recipe for the CPU oracle (test infrastructure, not the product).

Compiles ``nbody_oracle.c`` with gcc into ``libnbody_oracle.so`` next to this
file.  ``-ffp-contract=off`` keeps a*b+c as two rounded operations, as Julia
evaluates it; ``-fno-fast-math`` keeps IEEE semantics.  Portable flags only
(the same recipe runs on x86_64 and aarch64).
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "nbody_oracle.c")
LIB = os.path.join(HERE, "libnbody_oracle.so")


def build_oracle(force: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = [
        "gcc", "-O2", "-fno-fast-math", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
        "-std=c11", "-o", LIB + ".tmp", SRC, "-lm",
    ]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build_oracle(force=True))
