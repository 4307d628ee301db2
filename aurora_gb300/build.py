"""Builds libagb_cuda.so (the CUDA kernels + C ABI) in-tree for sm_103a with nvcc.

Every translation unit is compiled with -fmad=false: the shading arithmetic must follow the
reference's operation order (multiply-add contraction would change FP32 results), and the kernels
that want fused multiply-adds (BVH slab tests) call fmaf() explicitly.  Host code is compiled with
-ffp-contract=off so transforms computed on the host give the same bits on x86-64 and aarch64.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libagb_cuda.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

SOURCES = ["agb_pt.cu", "agb_env_build.cu", "agb_env_noalloc.cu", "agb_temporal.cu", "agb_denoise.cu", "agb_conv.cu",
           "agb_unet.cu", "agb_unit.cu",
           "agb_capi.cu", "agb_serve.cpp", "agb_aurora.cpp", "agb_aurora_api.cpp", "agb_obj.cpp", "agb_gltf.cpp", "agb_mtlx.cpp", "agb_image_io.cpp", "agb_bvh_build.cpp",
           "agb_bvh_gpu.cu"]
CLI_SRC = os.path.join(HERE, "cli", "agb_render.cpp")
CLI = os.path.join(BUILD, "agb_render")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-prec-div=true",
              "-prec-sqrt=true", "-Xcompiler",
              "-fPIC,-O2,-ffp-contract=off,-fvisibility=hidden", "-I" + INCLUDE,
              "-I" + os.path.join(INCLUDE, "glm_shim"), "-I" + CSRC]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return path


def _headers():
    out = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    for d, _, files in os.walk(INCLUDE):
        out += [os.path.join(d, f) for f in files if f.endswith((".h", ".hpp"))]
    return out


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, verbose):
    obj = os.path.join(BUILD, src + ".o")
    deps = [os.path.join(CSRC, src)] + _headers()
    if not _stale(obj, deps):
        return obj
    lang = ["-x", "cu"]  # host-only .cpp units include the device layout headers too
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *lang, "-c", os.path.join(CSRC, src), "-o", obj + ".tmp"]
    if src.endswith(".cu"):
        cmd += ["-Xptxas", "-v"] if verbose else []
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        print(r.stderr, flush=True)
    os.replace(obj + ".tmp", obj)
    return obj


def build_cli(verbose=False):
    """The headless renderer (cli/agb_render.cpp) linked against libagb_cuda.so."""
    deps = [CLI_SRC, LIB, os.path.join(INCLUDE, "aurora_gb300.hpp"), os.path.join(INCLUDE, "aurora_gb300_loaders.hpp")]
    if _stale(CLI, deps):
        gxx = shutil.which("g++") or "g++"
        cmd = [gxx, "-std=c++17", "-O2", "-I" + INCLUDE, CLI_SRC, "-L" + BUILD, "-lagb_cuda",
               "-Wl,-rpath," + BUILD, "-o", CLI + ".tmp"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)
        os.replace(CLI + ".tmp", CLI)
    return CLI


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lcudart"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)
        os.replace(LIB + ".tmp", LIB)
    build_cli(verbose)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
