"""The public headers compile as C99 (compute_c.h) and C++14
(gbcompute/compute.hpp) with warnings as errors, and programs written against
them link with libgbcompute.so (they run in test_programs_gpu.py)."""
import pytest

from programs_build import compile_program


@pytest.mark.parametrize("name", ["capi_hotpath.c", "cxx_algorithms.cpp"])
def test_program_compiles_and_links(tmp_path, name):
    compile_program(name, str(tmp_path))
