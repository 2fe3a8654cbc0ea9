"""Python binding of libgbcompute.so (ctypes over the C ABI in include/compute_c.h).

It mirrors the reference C++ API of the OpenCL Compute library
(lib/include/CL/Compute/Algorithm.hpp:119-250): a ``Context`` plays
``compute_context``, ``DeviceBuffer`` plays ``device_buffer<T>``,
``binary_op``/``ops`` are the operator descriptions, and ``sort``,
``sort_by_key``, ``reduce``, ``inclusive_scan``, ``exclusive_scan``,
``histogram_even``, ``fill`` and ``sequence`` keep the reference's argument
meaning and exceptions (``ValueError`` where the reference throws
``std::invalid_argument``/``length_error``, ``MemoryError`` for out of memory).

There is no fallback: importing this module fails loudly when the shared
library has not been built.
"""
from __future__ import annotations

import ctypes as C
import os
from collections import namedtuple

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIBRARY_PATH = os.path.join(os.path.dirname(_HERE), "libgbcompute.so")

if not os.path.exists(LIBRARY_PATH):
    raise ImportError(
        f"gbcompute: {LIBRARY_PATH} is missing; build it with "
        "`python opencl-sdk_gb300/build.py` (needs nvcc)"
    )
lib = C.CDLL(LIBRARY_PATH)

# ---- enums (include/compute_c.h) --------------------------------------------

SUCCESS = 0
ERROR_OPENCL = 1
ERROR_INVALID_ARGUMENT = 2
ERROR_BUILD = 3
ERROR_NO_DEVICE = 4
ERROR_OUT_OF_MEMORY = 5
ERROR_UNSUPPORTED = 6
ERROR_INTERNAL = 7
ERROR_IO = 8

TYPE_I8, TYPE_U8, TYPE_I16, TYPE_U16, TYPE_I32, TYPE_U32, TYPE_I64, TYPE_U64, TYPE_F32, TYPE_F64 = range(10)
DEFAULT_DEVICE = C.c_size_t(-1).value

_NP_TO_CLC = {
    np.dtype(np.int8): TYPE_I8,
    np.dtype(np.uint8): TYPE_U8,
    np.dtype(np.int16): TYPE_I16,
    np.dtype(np.uint16): TYPE_U16,
    np.dtype(np.int32): TYPE_I32,
    np.dtype(np.uint32): TYPE_U32,
    np.dtype(np.int64): TYPE_I64,
    np.dtype(np.uint64): TYPE_U64,
    np.dtype(np.float32): TYPE_F32,
    np.dtype(np.float64): TYPE_F64,
}


def clc_type(dtype) -> int:
    try:
        return _NP_TO_CLC[np.dtype(dtype)]
    except KeyError:
        raise ValueError(f"gbcompute: unsupported element type {dtype}") from None


class ClcError(RuntimeError):
    """A non-success clc_status; ``status`` and ``native`` (cudaError_t) attached."""

    def __init__(self, status: int, message: str, native: int = 0):
        super().__init__(f"[{status}] {message}")
        self.status = status
        self.native = native


class UnsupportedError(ClcError, NotImplementedError):
    pass


class NoDeviceError(ClcError):
    pass


class InvalidArgumentError(ClcError, ValueError):
    pass


class OutOfMemoryError(ClcError, MemoryError):
    pass


class BuildError(ClcError):
    """A malformed expression (the reference's build_error); the message holds a build log."""


def _raise_for(status: int) -> None:
    if status == SUCCESS:
        return
    msg = lib.clc_last_error().decode(errors="replace")
    native = lib.clc_last_cl_error()
    cls = {
        ERROR_INVALID_ARGUMENT: InvalidArgumentError,
        ERROR_UNSUPPORTED: UnsupportedError,
        ERROR_NO_DEVICE: NoDeviceError,
        ERROR_OUT_OF_MEMORY: OutOfMemoryError,
        ERROR_BUILD: BuildError,
    }.get(status, ClcError)
    raise cls(status, msg, native)


# ---- prototypes ---------------------------------------------------------------

class DeviceInfo(C.Structure):
    _fields_ = [
        ("name", C.c_char * 256),
        ("platform", C.c_char * 256),
        ("is_gpu", C.c_int),
        ("has_fp64", C.c_int),
        ("global_memory", C.c_ulonglong),
        ("max_work_group_size", C.c_size_t),
    ]


class MemoryStats(C.Structure):
    _fields_ = [
        ("current_bytes", C.c_size_t),
        ("peak_bytes", C.c_size_t),
        ("total_bytes", C.c_size_t),
        ("current_allocations", C.c_size_t),
        ("total_allocations", C.c_size_t),
        ("cached_bytes", C.c_size_t),
    ]


_vp, _sz, _i, _cp = C.c_void_p, C.c_size_t, C.c_int, C.c_char_p
_PROTOS = {
    "clc_last_error": (_cp, []),
    "clc_last_cl_error": (_i, []),
    "clc_device_count": (_i, [C.POINTER(_sz)]),
    "clc_device_get_info": (_i, [_sz, C.POINTER(DeviceInfo)]),
    "clc_context_create": (_i, [_sz, C.POINTER(_vp)]),
    "clc_context_create_with_cache": (_i, [_sz, _cp, C.POINTER(_vp)]),
    "clc_context_release": (None, [_vp]),
    "clc_context_get_info": (_i, [_vp, C.POINTER(DeviceInfo)]),
    "clc_finish": (_i, [_vp]),
    "clc_buffer_alloc": (_i, [_vp, _sz, C.POINTER(_vp)]),
    "clc_buffer_release": (None, [_vp]),
    "clc_buffer_size": (_sz, [_vp]),
    "clc_buffer_write": (_i, [_vp, _vp, _sz, _sz, _vp]),
    "clc_buffer_read": (_i, [_vp, _vp, _sz, _sz, _vp]),
    "clc_buffer_copy": (_i, [_vp, _vp, _sz, _vp, _sz, _sz]),
    "clc_file_size": (_i, [_cp, C.POINTER(_sz)]),
    "clc_file_read": (_i, [_vp, _cp, _sz, _vp, _sz, _sz, C.POINTER(_sz)]),
    "clc_file_write": (_i, [_vp, _cp, _i, _sz, _vp, _sz, _sz, C.POINTER(_sz)]),
    "clc_fill": (_i, [_vp, _vp, _sz, _i, _vp]),
    "clc_sequence": (_i, [_vp, _vp, _sz, _i, _vp, _vp]),
    "clc_transform": (_i, [_vp, _vp, _i, _vp, _i, _sz, _cp]),
    "clc_transform2": (_i, [_vp, _vp, _i, _vp, _i, _vp, _i, _sz, _cp]),
    "clc_reduce": (_i, [_vp, _vp, _sz, _i, _cp, _cp, _vp, _vp]),
    "clc_scan": (_i, [_vp, _vp, _vp, _sz, _i, _cp, _cp, _i]),
    "clc_sort": (_i, [_vp, _vp, _i, _vp, _sz, _i]),
    "clc_copy_if": (_i, [_vp, _vp, _vp, _sz, _i, _cp, C.POINTER(_sz)]),
    "clc_transform_compile": (_i, [_cp, _i, _i, _i, _i, _cp, _sz]),
    "clc_add_header": (_i, [_vp, _cp, _cp]),
    "clc_kernel_create": (_i, [_vp, _cp, _cp, _cp, _vp, _vp, _sz, C.POINTER(_vp)]),
    "clc_kernel_release": (None, [_vp]),
    "clc_kernel_set_buffer": (_i, [_vp, C.c_uint, _vp]),
    "clc_kernel_set_value": (_i, [_vp, C.c_uint, _sz, _vp]),
    "clc_kernel_set_local": (_i, [_vp, C.c_uint, _sz]),
    "clc_kernel_work_group_size": (_i, [_vp, _vp, _sz, C.POINTER(_sz)]),
    "clc_kernel_launch": (_i, [_vp, _vp, _sz, _sz]),
    "clc_histogram_even": (_i, [_vp, _vp, _sz, _i, _vp, _sz, C.c_double, C.c_double]),
    "clc_scan_ex": (_i, [_vp, _vp, _vp, _sz, _i, _cp, _cp, _i, _vp]),
    "clc_sort_ex": (_i, [_vp, _vp, _i, _vp, _sz, _i]),
    "clc_segmented_sort": (_i, [_vp, _vp, _i, _vp, _sz, _vp, _sz, _i]),
    "clc_segmented_sort_raw": (_i, [_vp, _vp, _vp, _i, _vp, _vp, _sz, _vp, _sz, _i]),
    "clc_segmented_scan": (_i, [_vp, _vp, _vp, _sz, _i, _cp, _cp, _i, _vp, _sz]),
    "clc_segmented_scan_raw": (_i, [_vp, _vp, _vp, _sz, _i, _cp, _cp, _i, _vp, _sz]),
    "clc_reduce_by_key_raw": (_i, [_vp, _vp, _i, _vp, _sz, _vp, _vp, _vp, _vp, C.POINTER(_sz)]),
    "clc_learned_default_options": (None, [_vp]),
    "clc_sort_learned": (_i, [_vp, _vp, _vp, _i, _sz, _vp, _vp]),
    "clc_sort_learned_pairs": (_i, [_vp, _vp, _vp, _i, _vp, _vp, _sz, _vp, _vp]),
    "clc_learned_param_count": (_i, []),
    "clc_autotune_sort": (_i, [_vp, _vp, _vp, _i, _vp, _vp, _sz, _i, _vp, _vp]),
    "clc_autotune_segmented_sort": (_i, [_vp, _vp, _vp, _i, _vp, _vp, _sz, _vp, _sz, _i, _vp, _vp]),
    "clc_learned_mlp_gradients": (_i, [_vp, _vp, _vp, C.c_float, _vp, _vp, _sz, _vp, _vp]),
    "clc_graph_begin": (_i, [_vp]),
    "clc_graph_end": (_i, [_vp, C.POINTER(_vp)]),
    "clc_graph_launch": (_i, [_vp, _vp]),
    "clc_graph_release": (None, [_vp]),
    "clc_buffer_device_pointer": (_vp, [_vp]),
    "clc_buffer_wrap": (_i, [_vp, _vp, _sz, C.POINTER(_vp)]),
    "clc_context_stream": (_vp, [_vp]),
    "clc_context_memory_stats": (_i, [_vp, C.POINTER(MemoryStats)]),
    "clc_context_release_cache": (_i, [_vp]),
    "clc_context_arena_info": (_i, [_vp, C.POINTER(_sz), C.POINTER(_sz), C.POINTER(_sz), C.POINTER(_sz)]),
    "clc_sort_keys_raw": (_i, [_vp, _vp, _vp, _i, _vp, _vp, _sz, _i]),
    "clc_scan_raw": (_i, [_vp, _vp, _vp, _sz, _i, _cp, _cp, _i, _vp]),
    "clc_histogram_even_raw": (_i, [_vp, _vp, _sz, _i, _vp, _sz, C.c_double, C.c_double]),
    "clc_reduce_raw": (_i, [_vp, _vp, _sz, _i, _cp, _cp, _vp, _vp]),
    "clc_bitpack_words_bound": (_sz, [_sz, _sz]),
    "clc_bitpack_compress": (_i, [_vp, _vp, _sz, _sz, _i, C.POINTER(_vp), C.POINTER(_sz)]),
    "clc_bitpack_decompress": (_i, [_vp, _vp, _sz, _sz, _i, _vp]),
    "clc_bitpack_compress_raw": (_i, [_vp, _vp, _sz, _sz, _i, _vp, _sz, C.POINTER(_sz)]),
    "clc_bitpack_decompress_raw": (_i, [_vp, _vp, _sz, _sz, _sz, _i, _vp]),
    "clc_bitpack_serialize": (_i, [_vp, _vp, _sz, _sz, _i, _vp, _sz, C.POINTER(_sz)]),
    "clc_bitpack_deserialize": (_i, [_vp, _vp, _sz, C.POINTER(_vp), C.POINTER(_sz), C.POINTER(_sz),
                                     C.POINTER(_i)]),
    "clc_map_create": (_i, [_vp, _sz, C.c_uint32, C.c_uint32, C.POINTER(_vp)]),
    "clc_map_release": (None, [_vp]),
    "clc_map_info": (_i, [_vp, C.POINTER(_sz), C.POINTER(_sz), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    "clc_map_clear": (_i, [_vp, _vp]),
    "clc_map_insert": (_i, [_vp, _vp, _vp, _vp, _sz, C.POINTER(_sz)]),
    "clc_map_find": (_i, [_vp, _vp, _vp, _sz, _vp]),
    "clc_map_contains": (_i, [_vp, _vp, _vp, _sz, _vp]),
    "clc_map_slots": (_i, [_vp, _vp, _vp, _vp]),
    "clc_map_insert_raw": (_i, [_vp, _vp, _vp, _vp, _sz, C.POINTER(_sz)]),
    "clc_map_find_raw": (_i, [_vp, _vp, _vp, _sz, _vp]),
    "clc_map_contains_raw": (_i, [_vp, _vp, _vp, _sz, _vp]),
    "clc_scan_i32_noalloc": (_i, [_vp, _vp, _sz, _i, _vp]),
    "clc_scan_i32_noalloc_status": (_i, [_vp]),
    "clc_selftest_noalloc_timeout": (_i, [_vp, _sz, _vp]),
    "clc_selftest_lookback_timeout": (_i, [_vp]),
    "clc_profile_enable": (_i, [_vp, _i]),
    "clc_profile_reset": (_i, [_vp]),
    "clc_profile_count": (_i, [_vp, C.POINTER(_sz)]),
    "clc_profile_entry": (_i, [_vp, _sz, _cp, _sz, C.POINTER(C.c_ulonglong), C.POINTER(C.c_double)]),
    "clc_tuning_sort_variants": (_i, [_i, _i]),
    "clc_tuning_sort_key": (_i, [_i, _i, _sz, _cp, _sz]),
    "clc_tuning_set": (_i, [_vp, _cp, _i]),
    "clc_tuning_get": (_i, [_vp, _cp, C.POINTER(_i)]),
    "clc_tuning_save": (_i, [_vp, _cp]),
}
for _name, (_res, _args) in _PROTOS.items():
    _f = getattr(lib, _name)
    _f.restype = _res
    _f.argtypes = _args

EXPORTED_SYMBOLS = tuple(_PROTOS)


# ---- devices and contexts ---------------------------------------------------

def device_count() -> int:
    n = C.c_size_t(0)
    _raise_for(lib.clc_device_count(C.byref(n)))
    return n.value


def device_info(index: int) -> DeviceInfo:
    info = DeviceInfo()
    _raise_for(lib.clc_device_get_info(index, C.byref(info)))
    return info


class Context:
    """One device, one CUDA stream, a pooled stream-ordered memory resource and
    the tuning table (the reference's compute_context)."""

    def __init__(self, device: int = DEFAULT_DEVICE, cache_dir: str | None = None):
        h = C.c_void_p()
        if cache_dir is None:
            _raise_for(lib.clc_context_create(device, C.byref(h)))
        else:
            _raise_for(lib.clc_context_create_with_cache(device, cache_dir.encode(), C.byref(h)))
        self.handle = h

    def close(self) -> None:
        if self.handle:
            lib.clc_context_release(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self) -> DeviceInfo:
        info = DeviceInfo()
        _raise_for(lib.clc_context_get_info(self.handle, C.byref(info)))
        return info

    def finish(self) -> None:
        _raise_for(lib.clc_finish(self.handle))

    @property
    def stream(self) -> int:
        return lib.clc_context_stream(self.handle) or 0

    def memory_stats(self) -> MemoryStats:
        s = MemoryStats()
        _raise_for(lib.clc_context_memory_stats(self.handle, C.byref(s)))
        return s

    def arena_info(self) -> dict:
        """held_bytes, slabs, slab_allocations, slab_releases of the context's arena."""
        v = [C.c_size_t() for _ in range(4)]
        _raise_for(lib.clc_context_arena_info(self.handle, *[C.byref(x) for x in v]))
        return dict(zip(("held_bytes", "slabs", "slab_allocations", "slab_releases"), (x.value for x in v)))

    def release_cache(self) -> None:
        _raise_for(lib.clc_context_release_cache(self.handle))

    # profiler
    def profile_enable(self, on: bool = True) -> None:
        _raise_for(lib.clc_profile_enable(self.handle, int(on)))

    def profile_reset(self) -> None:
        _raise_for(lib.clc_profile_reset(self.handle))

    def profile(self) -> dict:
        """{kernel family: (launches, total milliseconds)}; synchronises."""
        n = C.c_size_t(0)
        _raise_for(lib.clc_profile_count(self.handle, C.byref(n)))
        out = {}
        name = C.create_string_buffer(128)
        launches, ms = C.c_ulonglong(0), C.c_double(0)
        for i in range(n.value):
            _raise_for(lib.clc_profile_entry(self.handle, i, name, 128, C.byref(launches), C.byref(ms)))
            out[name.value.decode()] = (launches.value, ms.value)
        return out

    # tuning table
    def tuning_set(self, key: str, variant: int) -> None:
        _raise_for(lib.clc_tuning_set(self.handle, key.encode(), variant))

    def tuning_get(self, key: str) -> int:
        v = C.c_int(-1)
        _raise_for(lib.clc_tuning_get(self.handle, key.encode(), C.byref(v)))
        return v.value

    def tuning_save(self, path: str | None = None) -> None:
        _raise_for(lib.clc_tuning_save(self.handle, path.encode() if path else None))


class DeviceBuffer:
    """Typed device allocation (device_buffer<T>): ``size`` elements of ``dtype``."""

    def __init__(self, ctx: Context, size: int, dtype, _handle=None):
        self.ctx = ctx
        self.dtype = np.dtype(dtype)
        self.size = int(size)
        if _handle is None:
            h = C.c_void_p()
            _raise_for(lib.clc_buffer_alloc(ctx.handle, self.size * self.dtype.itemsize, C.byref(h)))
            self.handle = h
        else:
            self.handle = _handle

    @classmethod
    def from_host(cls, ctx: Context, host) -> "DeviceBuffer":
        host = np.ascontiguousarray(host)
        b = cls(ctx, host.size, host.dtype)
        b.write(host)
        return b

    @classmethod
    def wrap(cls, ctx: Context, device_pointer: int, size: int, dtype) -> "DeviceBuffer":
        """A non-owning view of existing device memory (e.g. a torch tensor)."""
        dtype = np.dtype(dtype)
        h = C.c_void_p()
        _raise_for(lib.clc_buffer_wrap(ctx.handle, C.c_void_p(device_pointer), size * dtype.itemsize, C.byref(h)))
        return cls(ctx, size, dtype, _handle=h)

    @property
    def nbytes(self) -> int:
        return self.size * self.dtype.itemsize

    @property
    def device_pointer(self) -> int:
        return lib.clc_buffer_device_pointer(self.handle) or 0

    def write(self, host, offset: int = 0) -> None:
        host = np.ascontiguousarray(host, dtype=self.dtype)
        _raise_for(lib.clc_buffer_write(self.ctx.handle, self.handle, offset * self.dtype.itemsize,
                                        host.nbytes, host.ctypes.data_as(C.c_void_p)))

    def to_host(self, count: int | None = None) -> np.ndarray:
        count = self.size if count is None else count
        out = np.empty(count, dtype=self.dtype)
        _raise_for(lib.clc_buffer_read(self.ctx.handle, self.handle, 0, out.nbytes,
                                       out.ctypes.data_as(C.c_void_p)))
        return out

    def release(self) -> None:
        if self.handle:
            lib.clc_buffer_release(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


# ---- operators (Algorithm.hpp:25-66) ------------------------------------------

binary_op = namedtuple("binary_op", ["expression", "identity"])

_LIMITS = {
    np.dtype(np.int8): ("CHAR_MIN", "CHAR_MAX"),
    np.dtype(np.uint8): ("0", "UCHAR_MAX"),
    np.dtype(np.int16): ("SHRT_MIN", "SHRT_MAX"),
    np.dtype(np.uint16): ("0", "USHRT_MAX"),
    np.dtype(np.int32): ("INT_MIN", "INT_MAX"),
    np.dtype(np.uint32): ("0", "UINT_MAX"),
    np.dtype(np.int64): ("LONG_MIN", "LONG_MAX"),
    np.dtype(np.uint64): ("0", "ULONG_MAX"),
    np.dtype(np.float32): ("(-INFINITY)", "INFINITY"),
    np.dtype(np.float64): ("(-INFINITY)", "INFINITY"),
}


class ops:
    @staticmethod
    def plus():
        return binary_op("(a + b)", "0")

    @staticmethod
    def multiplies():
        return binary_op("(a * b)", "1")

    @staticmethod
    def bit_and():
        return binary_op("(a & b)", "(~0)")

    @staticmethod
    def bit_or():
        return binary_op("(a | b)", "0")

    @staticmethod
    def bit_xor():
        return binary_op("(a ^ b)", "0")

    @staticmethod
    def minimum(dtype):
        return binary_op("((b < a) ? b : a)", _LIMITS[np.dtype(dtype)][1])

    @staticmethod
    def maximum(dtype):
        return binary_op("((a < b) ? b : a)", _LIMITS[np.dtype(dtype)][0])


# ---- algorithms ----------------------------------------------------------------

def _scalar(dtype, value):
    return np.array([value], dtype=dtype)


def fill(ctx: Context, out: DeviceBuffer, value) -> None:
    v = _scalar(out.dtype, value)
    _raise_for(lib.clc_fill(ctx.handle, out.handle, out.size, clc_type(out.dtype), v.ctypes.data_as(C.c_void_p)))


def sequence(ctx: Context, out: DeviceBuffer, start=0, step=1) -> None:
    s, d = _scalar(out.dtype, start), _scalar(out.dtype, step)
    _raise_for(lib.clc_sequence(ctx.handle, out.handle, out.size, clc_type(out.dtype),
                                s.ctypes.data_as(C.c_void_p), d.ctypes.data_as(C.c_void_p)))


def transform(ctx: Context, a: DeviceBuffer, b: DeviceBuffer, c, d: str | None = None) -> None:
    """Element-wise transform (reference Algorithm.hpp:135-157), both overloads:
    ``transform(ctx, inp, out, expression)`` computes out[i] = expression(x =
    inp[i]); ``transform(ctx, in1, in2, out, expression)`` computes out[i] =
    expression(x = in1[i], y = in2[i]), and out may alias an input. The
    expression is OpenCL C from the subset the library compiles (operators,
    casts, literals, min/max/clamp/abs/fabs/as_T/convert_T); a malformed one
    raises BuildError, one outside the subset UnsupportedError."""
    if d is None:
        inp, out, expression = a, b, c
        if out.size < inp.size:
            raise ValueError("transform: output too small")
        _raise_for(lib.clc_transform(ctx.handle, inp.handle, clc_type(inp.dtype), out.handle, clc_type(out.dtype),
                                     inp.size, expression.encode()))
        return
    in1, in2, out, expression = a, b, c, d
    if in2.size < in1.size or out.size < in1.size:
        raise ValueError("transform: size mismatch")
    _raise_for(lib.clc_transform2(ctx.handle, in1.handle, clc_type(in1.dtype), in2.handle, clc_type(in2.dtype),
                                  out.handle, clc_type(out.dtype), in1.size, expression.encode()))


def transform_compile(expression: str, in_dtype, out_dtype, in2_dtype=None) -> str:
    """Compiles a transform expression without a device; returns the program
    listing (one operation per line). Raises BuildError / UnsupportedError as
    transform does."""
    buf = C.create_string_buffer(8192)
    has2 = in2_dtype is not None
    _raise_for(lib.clc_transform_compile(expression.encode(), clc_type(in_dtype), int(has2),
                                         clc_type(in2_dtype if has2 else in_dtype), clc_type(out_dtype),
                                         buf, len(buf)))
    return buf.value.decode()


def reduce(ctx: Context, inp: DeviceBuffer, op: binary_op | None = None, init=0):
    op = op or ops.plus()
    i = _scalar(inp.dtype, init)
    r = np.zeros(1, dtype=inp.dtype)
    _raise_for(lib.clc_reduce(ctx.handle, inp.handle, inp.size, clc_type(inp.dtype), op.expression.encode(),
                              op.identity.encode(), i.ctypes.data_as(C.c_void_p), r.ctypes.data_as(C.c_void_p)))
    return r[0]


def copy_if(ctx: Context, inp: DeviceBuffer, out: DeviceBuffer, predicate: str) -> int:
    """Stable compaction (reference Algorithm.hpp:229-237): out[0:count] = the
    elements x of inp for which the predicate, an OpenCL C expression over x
    from the subset transform compiles, is nonzero; returns count. A
    malformed predicate raises BuildError, one outside the subset
    UnsupportedError."""
    if out.size < inp.size:
        raise ValueError("copy_if: output too small")
    count = C.c_size_t(0)
    _raise_for(lib.clc_copy_if(ctx.handle, inp.handle, out.handle, inp.size, clc_type(inp.dtype),
                               predicate.encode(), C.byref(count)))
    return count.value


def _scan(ctx, inp, out, op, exclusive, want_total):
    if out.size < inp.size:
        raise ValueError(("exclusive" if exclusive else "inclusive") + "_scan: output too small")
    op = op or ops.plus()
    if not want_total:
        _raise_for(lib.clc_scan(ctx.handle, inp.handle, out.handle, inp.size, clc_type(inp.dtype),
                                op.expression.encode(), op.identity.encode(), int(exclusive)))
        return None
    total = np.zeros(1, dtype=np.float64 if inp.dtype.kind == "f" else
                     (np.int64 if inp.dtype.kind == "i" else np.uint64))
    _raise_for(lib.clc_scan_ex(ctx.handle, inp.handle, out.handle, inp.size, clc_type(inp.dtype),
                               op.expression.encode(), op.identity.encode(), int(exclusive),
                               total.ctypes.data_as(C.c_void_p)))
    return total[0]


def inclusive_scan(ctx, inp, out, op=None, total=False):
    return _scan(ctx, inp, out, op, False, total)


def exclusive_scan(ctx, inp, out, op=None, total=False):
    return _scan(ctx, inp, out, op, True, total)


def sort(ctx: Context, keys: DeviceBuffer, descending: bool = False) -> None:
    """Stable radix sort of 32-bit keys in place (cl::compute::sort)."""
    if keys.dtype.itemsize != 4:
        raise TypeError("sort: keys must be 32-bit")
    _raise_for(lib.clc_sort(ctx.handle, keys.handle, clc_type(keys.dtype), None, keys.size, int(descending)))


def sort_by_key(ctx: Context, keys: DeviceBuffer, values: DeviceBuffer, descending: bool = False) -> None:
    """Sorts keys and permutes 32-bit values alongside (cl::compute::sort_by_key)."""
    if keys.dtype.itemsize != 4 or values.dtype.itemsize != 4:
        raise TypeError("sort_by_key: keys and values must be 32-bit")
    if values.size < keys.size:
        raise ValueError("sort_by_key: too few values")
    _raise_for(lib.clc_sort(ctx.handle, keys.handle, clc_type(keys.dtype), values.handle, keys.size,
                            int(descending)))


def sort_ex(ctx: Context, keys: DeviceBuffer, values: DeviceBuffer | None = None, descending: bool = False) -> None:
    """Extension: 32- or 64-bit keys with optional 32-bit values."""
    if values is not None and values.size < keys.size:
        raise ValueError("sort_ex: too few values")
    _raise_for(lib.clc_sort_ex(ctx.handle, keys.handle, clc_type(keys.dtype),
                               values.handle if values is not None else None, keys.size, int(descending)))


def sort_raw(ctx: Context, keys_in: int, keys_out: int, key_dtype, n: int, vals_in: int = 0, vals_out: int = 0,
             descending: bool = False) -> None:
    """Extension: sort on raw device pointers (asynchronous)."""
    _raise_for(lib.clc_sort_keys_raw(ctx.handle, C.c_void_p(keys_in), C.c_void_p(keys_out), clc_type(key_dtype),
                                     C.c_void_p(vals_in or None), C.c_void_p(vals_out or None), n, int(descending)))


def scan_raw(ctx: Context, inp: int, out: int, n: int, dtype, op: binary_op | None = None, exclusive: bool = False,
             total_device: int = 0) -> None:
    op = op or ops.plus()
    _raise_for(lib.clc_scan_raw(ctx.handle, C.c_void_p(inp), C.c_void_p(out), n, clc_type(dtype),
                                op.expression.encode(), op.identity.encode(), int(exclusive),
                                C.c_void_p(total_device or None)))


def histogram_even(ctx: Context, inp: DeviceBuffer, hist: DeviceBuffer, lower: float, upper: float) -> None:
    """Counts into hist.size equal-width bins over [lower, upper) (cl::compute::histogram_even)."""
    if hist.dtype != np.dtype(np.uint32):
        raise TypeError("histogram_even: histogram must be uint32")
    _raise_for(lib.clc_histogram_even(ctx.handle, inp.handle, inp.size, clc_type(inp.dtype), hist.handle,
                                      hist.size, float(lower), float(upper)))


def histogram_even_raw(ctx: Context, inp: int, n: int, dtype, hist: int, bins: int, lower: float,
                       upper: float) -> None:
    _raise_for(lib.clc_histogram_even_raw(ctx.handle, C.c_void_p(inp), n, clc_type(dtype), C.c_void_p(hist), bins,
                                          float(lower), float(upper)))


def tuning_sort_variants(key_bytes: int, has_values: bool) -> int:
    return lib.clc_tuning_sort_variants(key_bytes, int(has_values))


def tuning_sort_key(key_bytes: int, has_values: bool, n: int) -> str:
    buf = C.create_string_buffer(128)
    _raise_for(lib.clc_tuning_sort_key(key_bytes, int(has_values), n, buf, 128))
    return buf.value.decode()


# ---- batched (segmented) forms and CUDA graphs ----------------------------------

def segmented_sort(ctx: Context, keys: DeviceBuffer, offsets: DeviceBuffer, values: DeviceBuffer | None = None,
                   descending: bool = False) -> None:
    """Sorts every segment [offsets[i], offsets[i+1]) of keys (and values) in place."""
    if offsets.dtype != np.dtype(np.uint32):
        raise TypeError("segmented_sort: offsets must be uint32")
    _raise_for(lib.clc_segmented_sort(ctx.handle, keys.handle, clc_type(keys.dtype),
                                      values.handle if values is not None else None, keys.size, offsets.handle,
                                      max(offsets.size - 1, 0), int(descending)))


def segmented_sort_raw(ctx: Context, keys_in: int, keys_out: int, key_dtype, n: int, offsets: int,
                       num_segments: int, vals_in: int = 0, vals_out: int = 0, descending: bool = False) -> None:
    _raise_for(lib.clc_segmented_sort_raw(ctx.handle, C.c_void_p(keys_in), C.c_void_p(keys_out), clc_type(key_dtype),
                                          C.c_void_p(vals_in or None), C.c_void_p(vals_out or None), n,
                                          C.c_void_p(offsets), num_segments, int(descending)))


def segmented_scan(ctx: Context, inp: DeviceBuffer, out: DeviceBuffer, offsets: DeviceBuffer,
                   op: binary_op | None = None, exclusive: bool = False) -> None:
    op = op or ops.plus()
    _raise_for(lib.clc_segmented_scan(ctx.handle, inp.handle, out.handle, inp.size, clc_type(inp.dtype),
                                      op.expression.encode(), op.identity.encode(), int(exclusive), offsets.handle,
                                      max(offsets.size - 1, 0)))


def segmented_scan_raw(ctx: Context, inp: int, out: int, n: int, dtype, offsets: int, num_segments: int,
                       op: binary_op | None = None, exclusive: bool = False) -> None:
    op = op or ops.plus()
    _raise_for(lib.clc_segmented_scan_raw(ctx.handle, C.c_void_p(inp), C.c_void_p(out), n, clc_type(dtype),
                                          op.expression.encode(), op.identity.encode(), int(exclusive),
                                          C.c_void_p(offsets), num_segments))


class Graph:
    """A CUDA graph of calls captured on a context's stream (clc_graph_*)."""

    def __init__(self, ctx: Context, handle):
        self.ctx = ctx
        self.handle = handle

    def launch(self) -> None:
        _raise_for(lib.clc_graph_launch(self.ctx.handle, self.handle))

    def release(self) -> None:
        if self.handle:
            lib.clc_graph_release(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


def capture(ctx: Context, fn) -> Graph:
    """Captures the library calls made by fn() into a graph (they do not run)."""
    _raise_for(lib.clc_graph_begin(ctx.handle))
    try:
        fn()
    finally:
        h = C.c_void_p()
        status = lib.clc_graph_end(ctx.handle, C.byref(h))
    _raise_for(status)
    return Graph(ctx, h)


# ---- learned-CDF sort ---------------------------------------------------------

class LearnedOptions(C.Structure):
    _fields_ = [("sample", C.c_int), ("points", C.c_int), ("buckets", C.c_int), ("steps", C.c_int),
                ("lr", C.c_float), ("use_model", C.c_int), ("params_in", C.c_void_p), ("params_out", C.c_void_p),
                ("splitters_in", C.c_void_p), ("refine", C.c_int)]


class LearnedStats(C.Structure):
    _fields_ = [("buckets", C.c_uint), ("nonempty_buckets", C.c_uint), ("largest_bucket", C.c_uint),
                ("oversized_buckets", C.c_uint), ("oversized_keys", C.c_uint), ("constant_keys", C.c_uint),
                ("estimated_oversized_keys", C.c_uint), ("violation", C.c_uint), ("fallback", C.c_uint),
                ("first_loss", C.c_float), ("last_loss", C.c_float), ("refined_splitters", C.c_uint)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


def learned_options(**kw) -> LearnedOptions:
    o = LearnedOptions()
    lib.clc_learned_default_options(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def sort_learned(ctx: Context, keys_in: int, keys_out: int, key_dtype, n: int,
                 options: LearnedOptions | None = None) -> LearnedStats:
    """Learned-CDF sort of 32-bit keys, out of place; returns its statistics."""
    st = LearnedStats()
    _raise_for(lib.clc_sort_learned(ctx.handle, C.c_void_p(keys_in), C.c_void_p(keys_out), clc_type(key_dtype), n,
                                    C.byref(options) if options is not None else None, C.byref(st)))
    return st


def sort_learned_pairs(ctx: Context, keys_in: int, keys_out: int, key_dtype, vals_in: int, vals_out: int, n: int,
                       options: LearnedOptions | None = None) -> LearnedStats:
    """Learned-CDF sort of key-value pairs (32- or 64-bit keys, 32-bit values),
    stable, out of place, on device pointers; returns its statistics."""
    st = LearnedStats()
    _raise_for(lib.clc_sort_learned_pairs(ctx.handle, C.c_void_p(keys_in), C.c_void_p(keys_out), clc_type(key_dtype),
                                          C.c_void_p(vals_in), C.c_void_p(vals_out), n,
                                          C.byref(options) if options is not None else None, C.byref(st)))
    return st


def autotune_sort(ctx: Context, keys_in: int, keys_out: int, key_dtype, n: int, vals_in: int = 0, vals_out: int = 0,
                  repetitions: int = 3):
    """Times every compiled sort variant on the given device data, stores the
    fastest in the context's tuning table; returns (variant, ms per call)."""
    best, ms = C.c_int(-1), C.c_double(0)
    _raise_for(lib.clc_autotune_sort(ctx.handle, C.c_void_p(keys_in), C.c_void_p(keys_out), clc_type(key_dtype),
                                     C.c_void_p(vals_in or None), C.c_void_p(vals_out or None), n, repetitions,
                                     C.byref(best), C.byref(ms)))
    return best.value, ms.value


def autotune_segmented_sort(ctx: Context, keys_in: int, keys_out: int, key_dtype, n: int, offsets: int,
                            num_segments: int, vals_in: int = 0, vals_out: int = 0, repetitions: int = 3):
    """Times the segmented sort's one-CTA capacities on the given device data,
    stores the fastest; returns (capacity, ms per call)."""
    best, ms = C.c_int(-1), C.c_double(0)
    _raise_for(lib.clc_autotune_segmented_sort(ctx.handle, C.c_void_p(keys_in), C.c_void_p(keys_out),
                                               clc_type(key_dtype), C.c_void_p(vals_in or None),
                                               C.c_void_p(vals_out or None), n, C.c_void_p(offsets), num_segments,
                                               repetitions, C.byref(best), C.byref(ms)))
    return best.value, ms.value


def learned_param_count() -> int:
    return lib.clc_learned_param_count()


def learned_mlp_gradients(ctx: Context, params: np.ndarray, centres: np.ndarray, inv_span: float, keys: np.ndarray,
                          ys: np.ndarray):
    """Gradient (raw parameters) and loss of the network's mean squared error
    over the points (keys in the order-preserving u32 domain, targets ys)."""
    p = np.ascontiguousarray(params, dtype=np.float32)
    c = np.ascontiguousarray(centres, dtype=np.uint32)
    k = np.ascontiguousarray(keys, dtype=np.uint32)
    y = np.ascontiguousarray(ys, dtype=np.float32)
    g = np.zeros_like(p)
    loss = np.zeros(1, dtype=np.float32)
    _raise_for(lib.clc_learned_mlp_gradients(ctx.handle, p.ctypes.data, c.ctypes.data, C.c_float(inv_span),
                                             k.ctypes.data, y.ctypes.data, k.size, g.ctypes.data, loss.ctypes.data))
    return g, float(loss[0])


def reduce_by_key_raw(ctx: Context, keys: int, key_dtype, values: int, n: int, keys_out: int, sums_out: int,
                      counts_out: int = 0, hist16: int = 0, want_count: bool = True):
    """Runs of equal adjacent keys: key, uint64 sum of values, length; returns the run count (blocking) or None."""
    runs = C.c_size_t(0)
    _raise_for(lib.clc_reduce_by_key_raw(ctx.handle, C.c_void_p(keys), clc_type(key_dtype), C.c_void_p(values), n,
                                         C.c_void_p(keys_out), C.c_void_p(sums_out), C.c_void_p(counts_out or None),
                                         C.c_void_p(hist16 or None), C.byref(runs) if want_count else None))
    return runs.value if want_count else None


# ---- bitpack compression (Compression.hpp) ----------------------------------

class CompressedBuffer:
    """compressed_buffer: the device words of the reference's chunk format
    (3 header words per chunk, then the packed words) and how to read them."""

    def __init__(self, data: DeviceBuffer, num_elements: int, chunk_size: int, delta: bool):
        self.data = data
        self.num_elements = int(num_elements)
        self.chunk_size = int(chunk_size)
        self.delta = bool(delta)

    def num_chunks(self) -> int:
        return 0 if self.chunk_size == 0 else (self.num_elements + self.chunk_size - 1) // self.chunk_size

    def compressed_bytes(self) -> int:
        return self.data.nbytes

    def uncompressed_bytes(self) -> int:
        return 4 * self.num_elements

    def serialize(self) -> bytes:
        needed = C.c_size_t(0)
        _raise_for(lib.clc_bitpack_serialize(self.data.ctx.handle, self.data.handle, self.num_elements,
                                             self.chunk_size, int(self.delta), None, 0, C.byref(needed)))
        blob = (C.c_ubyte * needed.value)()
        _raise_for(lib.clc_bitpack_serialize(self.data.ctx.handle, self.data.handle, self.num_elements,
                                             self.chunk_size, int(self.delta), blob, needed.value, C.byref(needed)))
        return bytes(blob)

    @classmethod
    def deserialize(cls, ctx: Context, blob: bytes) -> "CompressedBuffer":
        h, n, chunk, delta = C.c_void_p(), C.c_size_t(), C.c_size_t(), C.c_int()
        buf = (C.c_ubyte * len(blob)).from_buffer_copy(blob) if blob else (C.c_ubyte * 1)()
        _raise_for(lib.clc_bitpack_deserialize(ctx.handle, buf, len(blob), C.byref(h), C.byref(n), C.byref(chunk),
                                               C.byref(delta)))
        words = lib.clc_buffer_size(h) // 4
        return cls(DeviceBuffer(ctx, words, np.uint32, _handle=h), n.value, chunk.value, bool(delta.value))


def compress_bitpack(ctx: Context, inp: DeviceBuffer, delta: bool = False, chunk_size: int = 2048) -> CompressedBuffer:
    h, words = C.c_void_p(), C.c_size_t()
    _raise_for(lib.clc_bitpack_compress(ctx.handle, inp.handle, inp.size, chunk_size, int(delta), C.byref(h),
                                        C.byref(words)))
    return CompressedBuffer(DeviceBuffer(ctx, words.value, np.uint32, _handle=h), inp.size, chunk_size, delta)


def decompress_bitpack(ctx: Context, comp: CompressedBuffer, out: DeviceBuffer) -> None:
    if out.size < comp.num_elements:
        raise InvalidArgumentError(ERROR_INVALID_ARGUMENT, "decompress_bitpack: output too small", 0)
    _raise_for(lib.clc_bitpack_decompress(ctx.handle, comp.data.handle, comp.num_elements, comp.chunk_size,
                                          int(comp.delta), out.handle))


def bitpack_words_bound(n: int, chunk_size: int = 2048) -> int:
    return lib.clc_bitpack_words_bound(n, chunk_size)


def compress_bitpack_raw(ctx: Context, inp: int, n: int, out: int, capacity_words: int, delta: bool = False,
                         chunk_size: int = 2048) -> int:
    words = C.c_size_t()
    _raise_for(lib.clc_bitpack_compress_raw(ctx.handle, C.c_void_p(inp), n, chunk_size, int(delta), C.c_void_p(out),
                                            capacity_words, C.byref(words)))
    return words.value


def decompress_bitpack_raw(ctx: Context, data: int, words: int, n: int, out: int, delta: bool = False,
                           chunk_size: int = 2048) -> None:
    _raise_for(lib.clc_bitpack_decompress_raw(ctx.handle, C.c_void_p(data), words, n, chunk_size, int(delta),
                                              C.c_void_p(out)))


# ---- static_map (HashMap.hpp) ----------------------------------------------

class StaticMap:
    """static_map: fixed-capacity uint32 -> uint32 hash map (linear probing,
    MurmurHash3 finalizer); insert keeps a key's first value and raises
    OutOfMemoryError ("table is full") when keys cannot be placed."""

    def __init__(self, ctx: Context, capacity: int, empty_key: int = 0xFFFFFFFF, empty_value: int = 0xFFFFFFFF):
        self.ctx = ctx
        h = C.c_void_p()
        _raise_for(lib.clc_map_create(ctx.handle, capacity, empty_key, empty_value, C.byref(h)))
        self.handle = h

    def _info(self):
        size, cap, ek, ev = C.c_size_t(), C.c_size_t(), C.c_uint32(), C.c_uint32()
        _raise_for(lib.clc_map_info(self.handle, C.byref(size), C.byref(cap), C.byref(ek), C.byref(ev)))
        return size.value, cap.value, ek.value, ev.value

    def size(self) -> int:
        return self._info()[0]

    def capacity(self) -> int:
        return self._info()[1]

    def empty_key(self) -> int:
        return self._info()[2]

    def empty_value(self) -> int:
        return self._info()[3]

    def load_factor(self) -> float:
        s, c, _, _ = self._info()
        return s / c

    def insert(self, keys: DeviceBuffer, values: DeviceBuffer, n: int | None = None) -> int:
        n = keys.size if n is None else n
        added = C.c_size_t()
        _raise_for(lib.clc_map_insert(self.ctx.handle, self.handle, keys.handle, values.handle, n, C.byref(added)))
        return added.value

    def find(self, keys: DeviceBuffer, values: DeviceBuffer) -> None:
        _raise_for(lib.clc_map_find(self.ctx.handle, self.handle, keys.handle, keys.size, values.handle))

    def contains(self, keys: DeviceBuffer, found: DeviceBuffer) -> None:
        _raise_for(lib.clc_map_contains(self.ctx.handle, self.handle, keys.handle, keys.size, found.handle))

    def clear(self) -> None:
        _raise_for(lib.clc_map_clear(self.ctx.handle, self.handle))

    def slots(self):
        """(slot keys, slot values) as host arrays."""
        cap = self.capacity()
        k, v = DeviceBuffer(self.ctx, cap, np.uint32), DeviceBuffer(self.ctx, cap, np.uint32)
        _raise_for(lib.clc_map_slots(self.ctx.handle, self.handle, k.handle, v.handle))
        return k.to_host(), v.to_host()

    def insert_raw(self, keys: int, values: int, n: int) -> int:
        added = C.c_size_t()
        _raise_for(lib.clc_map_insert_raw(self.ctx.handle, self.handle, C.c_void_p(keys), C.c_void_p(values), n,
                                          C.byref(added)))
        return added.value

    def find_raw(self, keys: int, n: int, values: int) -> None:
        _raise_for(lib.clc_map_find_raw(self.ctx.handle, self.handle, C.c_void_p(keys), n, C.c_void_p(values)))

    def contains_raw(self, keys: int, n: int, found: int) -> None:
        _raise_for(lib.clc_map_contains_raw(self.ctx.handle, self.handle, C.c_void_p(keys), n, C.c_void_p(found)))

    def release(self) -> None:
        if self.handle:
            lib.clc_map_release(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass
