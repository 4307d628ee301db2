"""Oracle build recipe (test infrastructure).

Builds, with g++ only:
  * oracle/_build/liboracle.so - the CPU restatement (pt_*.hpp + oracle_capi.cpp);
  * oracle/_ref/libaliasmap_ref.so - the reference's own AliasMap.cpp, compiled in place from the
    reference tree with oracle/ref_shim standing in for its precompiled header, when that tree is
    present (it is not on the GPU host; the tests that need it skip there).

FP contraction is disabled so the oracle gives the same bits on x86-64 and aarch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference checkout this recipe compiles from (read-only; absent on machines that only run the
# built files).  AURORA_REFERENCE_ROOT overrides the default location.
REFERENCE_ROOT = os.environ.get("AURORA_REFERENCE_ROOT", "/root/reference")
REFERENCE_SOURCE = os.path.join(REFERENCE_ROOT, "Libraries", "Aurora", "Source")

CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-pthread",
            "-fvisibility=hidden"]


def _needs(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(verbose=False):
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    target = os.path.join(out_dir, "liboracle.so")
    sources = [os.path.join(HERE, f) for f in os.listdir(HERE)
               if f.endswith((".hpp", ".cpp"))]
    if _needs(target, sources):
        cmd = ["g++", *CXXFLAGS, os.path.join(HERE, "oracle_capi.cpp"), "-o", target + ".tmp"]
        if verbose:
            print(" ".join(cmd))
        subprocess.check_call(cmd)
        os.replace(target + ".tmp", target)
    return target


def build_reference_alias(verbose=False):
    """Compiles the reference's AliasMap.cpp where it lies; returns the .so path or None."""
    src = os.path.join(REFERENCE_SOURCE, "AliasMap.cpp")
    if not os.path.exists(src):
        return None
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    target = os.path.join(out_dir, "libaliasmap_ref.so")
    shim = os.path.join(HERE, "ref_shim")
    wrapper = os.path.join(shim, "alias_ref_capi.cpp")
    if _needs(target, [src, wrapper, os.path.join(shim, "pch.h")]):
        # "-I-" stops quote includes from searching the including file's own directory first, so the
        # reference's `#include "pch.h"` resolves to the shim while AliasMap.h still comes from the
        # reference tree.
        cmd = ["g++", *CXXFLAGS, "-I" + shim, "-I-", "-I" + REFERENCE_SOURCE, src, wrapper,
               "-o", target + ".tmp"]
        if verbose:
            print(" ".join(cmd))
        subprocess.check_call(cmd, stderr=subprocess.DEVNULL if not verbose else None)
        os.replace(target + ".tmp", target)
    return target


if __name__ == "__main__":
    print(build_oracle(verbose=True))
    print(build_reference_alias(verbose=True))
    sys.exit(0)
