"""Builds the oracle's C restatement: oracle/libjmg_oracle.so (gcc, OpenMP).

-ffp-contract=off keeps every multiply and add separately rounded, as in the
reference's XLA CPU arithmetic; no -march flags, so the same source builds on x86-64
and aarch64 hosts.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "jmg_oracle.c")
LIB = os.path.join(HERE, "libjmg_oracle.so")


def build(force=False):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["gcc", "-O3", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", SRC, "-o", LIB, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle C build failed:\n" + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
