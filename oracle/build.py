"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/oracle.c with gcc into oracle/_build/liboracle.so.  Plain C,
no architecture-specific flags, so the same source builds on x86_64 and
aarch64 hosts.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SRC = [os.path.join(HERE, "oracle.c")]


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    newest_src = max(os.path.getmtime(s) for s in SRC + [os.path.join(HERE, "oracle.h")])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest_src:
        return LIB
    tmp = LIB + ".tmp"
    cmd = ["gcc", "-O3", "-std=gnu11", "-shared", "-fPIC", "-pthread", "-o", tmp] + SRC + ["-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
