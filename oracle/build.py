"""ORACLE — TEST INFRASTRUCTURE ONLY. Builds oracle/_build/liboracle.so from oracle.cpp.

Host-only C++ (g++), OpenMP when the compiler has it, -ffp-contract=off so that results match
bit for bit between x86-64 and aarch64 hosts.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def build(force: bool = False, verbose: bool = False) -> str:
    src = os.path.join(HERE, "oracle.cpp")
    hdr = os.path.join(HERE, "oracle.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    base = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
            src, "-o", tmp]
    for extra in (["-fopenmp"], []):
        r = subprocess.run(base + extra, capture_output=True, text=True)
        if r.returncode == 0:
            break
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stderr)
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
