"""Build recipe of the oracle (test infrastructure): compiles nunatak_oracle.cpp with g++ into
oracle/_build/libnunatak_oracle.so.  -ffp-contract=off keeps every multiply and add separately
rounded, so the oracle gives the same bits on x86-64 and aarch64."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "nunatak_oracle.cpp")
HEADER = os.path.join(HERE, "..", "include", "nunatak_gb300.h")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libnunatak_oracle.so")


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    newest = max(os.path.getmtime(SRC), os.path.getmtime(HEADER), os.path.getmtime(__file__))
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
           "-Wall", "-Wno-unused-function", "-o", LIB + ".tmp", SRC]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
