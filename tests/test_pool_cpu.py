"""Memory-resource logic (size classes, reuse, statistics, release-and-retry on
out of memory) built natively against a fake upstream and run on the host."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_pool_resource(tmp_path):
    exe = tmp_path / "pool_test"
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "opencl-sdk_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "pool_test.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
