"""The stream-ordered slab arena (slab sharing, best fit, merging of freed
neighbours, retain limit, statistics, one retry after idle slabs are handed
back on out of memory) built natively against a fake upstream and run on the
host."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_stream_arena(tmp_path):
    exe = tmp_path / "arena_test"
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "opencl-sdk_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "arena_test.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
