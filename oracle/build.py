"""Build recipe for the oracle (test infrastructure only).

Compiles the C++ restatement of the reference's CPU backend, ring and BFV layers into
``oracle/_build/liboracle.so``. It is single-threaded like the reference and doubles as the timed
CPU baseline. The reference's release profile (Cargo.toml:26-31) builds with ``-Ctarget-cpu=native``;
this recipe builds with ``-O3`` and no CPU-specific tuning (``FLAGS``), because the same host code
must build and behave identically on the x86-64 development machine and the aarch64 GPU host. On
the Grace host a ``-mcpu=native`` build of the oracle ran the field_36864 ct-mult 1-3 % faster
(2.03-2.05 against 2.00 ct-mults/s on one core), so the portable baseline is that much slower
than a natively tuned one; the benchmark's CPU lines name these flags.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "liboracle.so")
SOURCES = ["capi.cpp"]
HEADERS = ["arith.hpp", "ntt.hpp", "cpu_backend.hpp", "field.hpp", "ring.hpp", "bfv.hpp", "dbfv.hpp"]
FLAGS = ["-O3", "-std=c++17"]


def build(force=False):
    os.makedirs(BUILD_DIR, exist_ok=True)
    deps = [os.path.join(HERE, f) for f in SOURCES + HEADERS]
    if not force and os.path.exists(LIB):
        lib_mtime = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= lib_mtime for d in deps):
            return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++"] + FLAGS + ["-shared", "-fPIC", "-o", tmp] + [
        os.path.join(HERE, s) for s in SOURCES
    ]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
