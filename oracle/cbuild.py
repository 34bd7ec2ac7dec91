"""Build the oracle's C restatement (oracle/c/*.c -> oracle/_build/libcpu_march.so).

Test infrastructure: the C time loop is the timed CPU baseline ("port") and a
second checker; it is never linked into the product library.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "c", "cpu_march.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libcpu_march.so")


def build(force=False):
    """Compile the C restatement of the v6 loop (OpenMP) into a shared library
    beside it, unless it is newer than its source; returns the library path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-o", LIB, SRC]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle C build failed:\n" + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
