"""Build recipe for the oracle (test infrastructure only).

Compiles the C++ restatement of the reference's CPU backend, ring and BFV layers into
``oracle/_build/liboracle.so``. It is single-threaded and optimised like the reference's release
profile (``-O3``, no CPU-specific tuning, as a Cargo release build sets no target CPU), so it
doubles as the timed CPU baseline; the same flags build it on x86-64 and on aarch64.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "liboracle.so")
SOURCES = ["capi.cpp"]
HEADERS = ["arith.hpp", "ntt.hpp", "cpu_backend.hpp", "field.hpp", "ring.hpp", "bfv.hpp"]


def build(force=False):
    os.makedirs(BUILD_DIR, exist_ok=True)
    deps = [os.path.join(HERE, f) for f in SOURCES + HEADERS]
    if not force and os.path.exists(LIB):
        lib_mtime = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= lib_mtime for d in deps):
            return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O3", "-std=c++17", "-shared", "-fPIC", "-o", tmp] + [
        os.path.join(HERE, s) for s in SOURCES
    ]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
