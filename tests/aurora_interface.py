"""Helpers for the Aurora interface tests (tests/test_aurora_dropin.py) and the fixture script
(tests/golden/make_golden.py): compile tests/cpp/aurora_abi_probe.cpp against an Aurora header
tree and run it; read the reference's Names values (Libraries/Aurora/Source/AuroraNames.cpp); print
the values this library defines; read and write tests/golden/aurora_interface.txt."""
import os
import re
import shutil
import subprocess
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PROBE = os.path.join(ROOT, "tests", "cpp", "aurora_abi_probe.cpp")
CLIENT = os.path.join(ROOT, "tests", "cpp", "aurora_dropin_render.cpp")
FIXTURE = os.path.join(ROOT, "tests", "golden", "aurora_interface.txt")
GLM = os.path.join(ROOT, "include", "glm_shim")
MIRROR = [os.path.join(ROOT, "include"), GLM]


def reference_includes(ref_root):
    """The reference's public header directories (Aurora.h includes <Aurora/Foundation/Log.h>),
    with the GLM stand-in: GLM itself is not in this image."""
    return [os.path.join(ref_root, "Libraries", "Aurora", "API"),
            os.path.join(ref_root, "Libraries", "Foundation", "API"), GLM]


def gxx():
    return shutil.which("g++") or "g++"


def compile_cpp(src, includes, out, libs=()):
    cmd = [gxx(), "-std=c++17", "-O1", "-w"] + ["-I" + d for d in includes] + [src, "-o", out] + list(libs)
    subprocess.check_call(cmd)
    return out


def probe_layout(includes):
    """The probe's output (vtable slots, layouts, enumerator values) for a header tree."""
    with tempfile.TemporaryDirectory() as tmp:
        exe = compile_cpp(PROBE, includes, os.path.join(tmp, "probe"))
        return subprocess.check_output([exe], text=True)


def reference_names(ref_root):
    """(qualified name, value) for every Aurora::Names string the reference defines."""
    path = os.path.join(ref_root, "Libraries", "Aurora", "Source", "AuroraNames.cpp")
    out = []
    for line in open(path):
        m = re.match(r'\s*const (?:std::)?string Names::(\w+)::(\w+)\s*(?:\(\s*|=\s*)"([^"]*)"', line)
        if m:
            out.append((f"{m.group(1)}::{m.group(2)}", m.group(3)))
    return sorted(out)


def library_names(names, lib_dir):
    """The values libagb_cuda.so defines for `names`, through a program compiled against this
    library's copy of the Aurora headers (linking proves each symbol is exported)."""
    with tempfile.TemporaryDirectory() as tmp:
        src = os.path.join(tmp, "names.cpp")
        with open(src, "w") as f:
            f.write("#include <Aurora/Aurora.h>\n#include <cstdio>\nint main()\n{\n")
            for q, _ in names:
                f.write(f'    std::printf("%s %s\\n", "{q}", Aurora::Names::{q}.c_str());\n')
            f.write("    return 0;\n}\n")
        exe = compile_cpp(src, MIRROR, os.path.join(tmp, "names"),
                          ["-L" + lib_dir, "-lagb_cuda", "-Wl,-rpath," + lib_dir])
        lines = subprocess.check_output([exe], text=True).splitlines()
    return sorted(tuple(line.split(" ", 1)) if " " in line else (line, "") for line in lines)


def write_fixture(ref_root):
    layout = probe_layout(reference_includes(ref_root))
    names = reference_names(ref_root)
    with open(FIXTURE, "w") as f:
        f.write("[layout]\n" + layout + "[names]\n")
        f.writelines(f"{q} {v}\n" for q, v in names)


def read_fixture():
    text = open(FIXTURE).read()
    layout, names = text.split("[names]\n")
    assert layout.startswith("[layout]\n")
    pairs = [tuple(line.split(" ", 1)) if " " in line else (line, "") for line in names.splitlines()]
    return layout[len("[layout]\n"):], sorted(pairs)
