"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/pir_oracle.cc into oracle/_build/libpir_oracle.so with g++.
No target-specific flags: the same source must round identically on the
x86_64 development host and on the aarch64 GPU host, so FP contraction is
disabled and no -march/-mcpu is given.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libpir_oracle.so")
SOURCES = [os.path.join(HERE, "pir_oracle.cc")]

CXXFLAGS = ["-O3", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
            "-fno-fast-math", "-Wall", "-Wno-sign-compare", "-pthread"]


def _stale():
    if not os.path.exists(LIB_PATH):
        return True
    built = os.path.getmtime(LIB_PATH)
    deps = SOURCES + [os.path.join(HERE, "pir_oracle.h"), __file__]
    return any(os.path.getmtime(p) > built for p in deps)


def build(force=False, verbose=False):
    """Compile the oracle library if it is missing or older than its sources."""
    if not force and not _stale():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB_PATH + ".tmp.%d" % os.getpid()
    cmd = ["g++"] + CXXFLAGS + SOURCES + ["-o", tmp]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
