"""Compiles the C and C++ caller programs under tests/programs against the
public headers (include/) and links them with libgbcompute.so."""
import os
import shutil
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(ROOT, "opencl-sdk_gb300")
PROGRAMS = os.path.join(ROOT, "tests", "programs")


def compile_program(name: str, out_dir: str) -> str:
    """name: 'capi_hotpath.c' (C99) or 'cxx_algorithms.cpp' (C++14). Returns the executable."""
    src = os.path.join(PROGRAMS, name)
    exe = os.path.join(out_dir, os.path.splitext(name)[0])
    link = ["-L" + LIBDIR, "-lgbcompute", "-Wl,-rpath," + LIBDIR]
    if name.endswith(".c"):
        cc = shutil.which("cc") or shutil.which("gcc")
        cmd = [cc, "-std=c99", "-pedantic", "-Wall", "-Wextra", "-Werror", "-O1", "-I" + INCLUDE, src, "-o", exe] + link + ["-lm"]
    else:
        cxx = shutil.which("c++") or shutil.which("g++")
        cmd = [cxx, "-std=c++14", "-Wall", "-Wextra", "-Werror", "-O1", "-I" + INCLUDE, src, "-o", exe] + link
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(" ".join(cmd) + "\n" + r.stdout + r.stderr)
    return exe
