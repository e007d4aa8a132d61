"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/pir_oracle.cc twice with g++:

* oracle/_build/libpir_oracle.so, the checker: no target-specific flags, so
  the same source rounds identically on the x86_64 development host and on
  the aarch64 GPU host (FP contraction disabled, no -march/-mcpu);
* oracle/_build/libpir_oracle_timing.so, the timed CPU baseline: the same
  source and the same FP rules, compiled for the host core it times (on a
  Neoverse V2 / Grace host `-mcpu=neoverse-v2`, which turns on SVE2 for the
  64-bit multiply-adds of the condensed DB product). Its outputs equal the
  checker's (integer products are exact, and contraction stays off).
"""
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libpir_oracle.so")
TIMING_LIB_PATH = os.path.join(BUILD_DIR, "libpir_oracle_timing.so")
SOURCES = [os.path.join(HERE, "pir_oracle.cc")]

CXXFLAGS = ["-O3", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
            "-fno-fast-math", "-Wall", "-Wno-sign-compare", "-pthread"]

# Arm "CPU part" numbers of cores with a matching -mcpu name.
_ARM_PARTS = {"0xd4f": "neoverse-v2", "0xd40": "neoverse-v1",
              "0xd0c": "neoverse-n1", "0xd49": "neoverse-n2"}
# Optional extensions of those cores (gcc name, /proc/cpuinfo flag): the
# ones the kernel does not report are switched off, since a host (or a
# virtual machine) may hide some, and code using them would trap.
_ARM_EXTS = [("sve", "sve"), ("sve2", "sve2"), ("i8mm", "i8mm"),
             ("bf16", "bf16"), ("dotprod", "asimddp"), ("fp16", "asimdhp"),
             ("rng", "rng"), ("memtag", "mte"), ("sb", "sb"),
             ("ssbs", "ssbs"), ("pauth", "paca"), ("crypto", "aes"),
             ("lse", "atomics"), ("rcpc", "lrcpc"), ("flagm", "flagm")]


def _cpuinfo():
    part, feats = None, set()
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                key = line.split(":")[0].strip().lower()
                if key == "cpu part" and part is None:
                    part = line.split(":")[1].strip().lower()
                elif key == "features" and not feats:
                    feats = set(line.split(":")[1].split())
    except OSError:
        pass
    return part, feats


def timing_target_flags():
    """Target flags of the timing build for this host: an -mcpu named for
    the host's Arm core when it is a known one, minus the extensions the
    host does not report; else none."""
    if platform.machine() not in ("aarch64", "arm64"):
        return []
    part, feats = _cpuinfo()
    if part not in _ARM_PARTS or not feats:
        return []
    off = "".join("+no" + ext for ext, flag in _ARM_EXTS if flag not in feats)
    return ["-mcpu=" + _ARM_PARTS[part] + off]


def _stale(path):
    if not os.path.exists(path):
        return True
    built = os.path.getmtime(path)
    deps = SOURCES + [os.path.join(HERE, "pir_oracle.h"), __file__]
    return any(os.path.getmtime(p) > built for p in deps)


def _compile(path, flags, force, verbose):
    if not force and not _stale(path):
        return path
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = path + ".tmp.%d" % os.getpid()
    cmd = ["g++"] + flags + SOURCES + ["-o", tmp]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(tmp, path)
    return path


def build(force=False, verbose=False):
    """Compile the checker library if it is missing or older than its
    sources."""
    return _compile(LIB_PATH, CXXFLAGS, force, verbose)


def build_timing(force=False, verbose=False):
    """Compile the timing flavour (same source, host-tuned target flags;
    without them if the compiler refuses the flags)."""
    try:
        return _compile(TIMING_LIB_PATH, CXXFLAGS + timing_target_flags(),
                        force, verbose)
    except subprocess.CalledProcessError:
        return _compile(TIMING_LIB_PATH, CXXFLAGS, True, verbose)


def timing_build_string():
    return "g++ " + " ".join(["-O3", "-ffp-contract=off"] +
                             (timing_target_flags() or ["(no target flags)"]))


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
    print(build_timing(force="--force" in sys.argv, verbose=True))
