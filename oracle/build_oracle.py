"""Builds the oracle (test infrastructure) into oracle/_build/liboracle.so.

gcc, -O2, -ffp-contract=off (the reference never fuses a*b+c), no -march
flags so the same source builds on x86_64 and aarch64 hosts.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liboracle.so")


def build(force: bool = False) -> str:
    src = [os.path.join(HERE, "oracle.c")]
    deps = src + [os.path.join(HERE, "oracle.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    os.makedirs(OUT, exist_ok=True)
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-Wall", "-Wno-unused-function", "-pthread", "-o", tmp, *src, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
