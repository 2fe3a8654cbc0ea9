"""Programs written against the public headers, run on the GPU: a C99 caller
of the C interface doing what the reference's capi.c checks for the hot path
(lib/test/Compute/capi.c:52-157), and a C++ caller of the cl::compute facade
running the algorithm, static_map and compression cases of the reference's
main.cpp:184-451 with its own
host checks. Each exits with its number of failed checks."""
import subprocess

import pytest

from programs_build import compile_program

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["capi_hotpath.c", "cxx_algorithms.cpp"])
def test_program_runs_clean(tmp_path, name):
    exe = compile_program(name, str(tmp_path))
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("0 of "), r.stdout
