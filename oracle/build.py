"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``nr_oracle.cpp`` into ``oracle/_build/libnr_oracle.so`` with g++.
``-ffp-contract=off`` keeps every product and sum rounded separately, as the
reference's Rust f64 arithmetic is; no host-specific flags are used so the
same recipe builds on x86_64 and aarch64.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "nr_oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libnr_oracle.so")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-pthread",
           "-ffp-contract=off", "-fno-fast-math", SRC, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
