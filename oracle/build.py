"""Build recipe for the oracle (test infrastructure, not the product).

Compiles oracle/vlm_oracle.c into oracle/_build/libvlm_oracle.so with gcc.
``-ffp-contract=off`` keeps float expressions unfused on every host (gcc
contracts to FMA by default on aarch64), so the oracle rounds the same way
on x86-64 and on Arm.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libvlm_oracle.so")
SOURCES = [os.path.join(HERE, "vlm_oracle.c")]
DEPS = SOURCES + [os.path.join(HERE, "vlm_oracle_impl.h")]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in DEPS)


def build(force=False):
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", "-o", tmp] + SOURCES + ["-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
