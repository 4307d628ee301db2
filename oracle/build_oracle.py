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


# The reference's shader files the pin compiles, in include order.
REFERENCE_SHADERS = ["Globals", "Colors", "Random", "Sampling", "BSDFCommon", "Material",
                     "StandardSurfaceBSDF", "Environment"]


def rewrite_slang(text):
    """Mechanical rewrite of a reference .slang file into C++ over oracle/ref_shim/hlsl.h:
    comments dropped; includes of other shader files point at their generated copies (and
    GlobalPipelineState.slang, whose resource bindings have no host meaning, at
    ref_shim/pipeline_state.h); `out T x` / `inout T x` / `in out T x` parameters become `T& x`;
    scalar swizzles (`s.xx`, `s.xxx`) become vector constructors and vector swizzles (`.xy`, `.zw`,
    `.xyz`, `.rgb`) accessor calls; unsuffixed floating literals get an `f` (HLSL types them as
    float); the HLSL spelling of infinity is dropped (the C library's INFINITY stands in)."""
    import re
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    text = re.sub(r'#include\s+"GlobalPipelineState\.slang"', '#include "pipeline_state.h"', text)
    text = re.sub(r'#include\s+"(\w+)\.slang"', r'#include "\1.slang.h"', text)
    text = re.sub(r"#define\s+INFINITY\s+\+1\.#INF", "", text)
    text = re.sub(r"\b(?:in\s+out|inout|out)\s+(\w+)\s+(\w+)", r"\1& \2", text)
    text = re.sub(r"\bin\s+(\w+\s+\w+\s*[,)])", r"\1", text)
    text = re.sub(r"(\d+\.\d*f?|\b\w+)\.xxx\b", r"float3(\1)", text)
    text = re.sub(r"(\d+\.\d*f?|\b\w+)\.xx\b", r"float2(\1)", text)
    text = re.sub(r"\.(xyz|rgb|xy|zw)\b(?!\s*\()", r".\1()", text)
    text = re.sub(r"(?<![\w.])(\d+\.\d*|\.\d+)([eE][+-]?\d+)?(?![fFhH\w.])", r"\1\2f", text)
    text = re.sub(r"(?<![\w.])(\d+[eE][+-]?\d+)(?![fF\w.])", r"\1f", text)
    return text


def build_reference_shaders(verbose=False):
    """Compiles the reference's own shader functions (Standard Surface BSDF, sampling, random
    numbers, environment) as host C++ where the reference tree lies: the unmodified .slang files
    are rewritten by rewrite_slang into oracle/_ref/gen/ and compiled with oracle/ref_shim in FP32
    (ref32_*) and FP64 (ref64_*) into oracle/_ref/libshaders_ref.so.  Returns its path, or None
    when the reference tree is absent."""
    shader_dir = os.path.join(REFERENCE_SOURCE, "Shaders")
    sources = [os.path.join(shader_dir, n + ".slang") for n in REFERENCE_SHADERS]
    if not all(os.path.exists(p) for p in sources):
        return None
    out_dir = os.path.join(HERE, "_ref")
    gen = os.path.join(out_dir, "gen")
    os.makedirs(gen, exist_ok=True)
    shim = os.path.join(HERE, "ref_shim")
    wrapper = os.path.join(shim, "shaders_ref_capi.cpp")
    target = os.path.join(out_dir, "libshaders_ref.so")
    deps = sources + [wrapper, os.path.join(shim, "hlsl.h"), os.path.join(shim, "pipeline_state.h"),
                      os.path.abspath(__file__)]
    if not _needs(target, deps):
        return target
    for n, src in zip(REFERENCE_SHADERS, sources):
        with open(src) as f:
            text = rewrite_slang(f.read())
        with open(os.path.join(gen, n + ".slang.h"), "w") as f:
            f.write(text)
    objs = []
    for prec in (32, 64):
        obj = os.path.join(out_dir, f"shaders_ref{prec}.o")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fvisibility=hidden",
               "-w", f"-DREF_PREC={prec}", "-I" + shim, "-I" + gen, "-c", wrapper, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        subprocess.check_call(cmd)
        objs.append(obj)
    subprocess.check_call(["g++", "-shared", "-o", target + ".tmp", *objs])
    os.replace(target + ".tmp", target)
    return target


if __name__ == "__main__":
    print(build_oracle(verbose=True))
    print(build_reference_alias(verbose=True))
    print(build_reference_shaders(verbose=True))
    sys.exit(0)
