"""Build recipe for the oracle's C restatement (test infrastructure only).

Produces oracle/liboracle.so from oracle/oracle.c with plain gcc.  The flags
pin IEEE behaviour on both x86-64 and aarch64 hosts: no FMA contraction, no
fast-math, so the double-double checkers stay exact and results agree across
machines.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "oracle.c")
    hdr = os.path.join(HERE, "oracle.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-std=c11",
                           "-ffp-contract=off", "-fno-fast-math", "-Wall",
                           "-o", tmp, src, "-lm"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build_oracle(force=True))
