import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

TESTS = os.path.dirname(os.path.abspath(__file__))
CPU_PIPE_SRC = os.path.join(TESTS, "cpu_pipeline.cc")
CPU_PIPE_LIB = os.path.join(TESTS, "_build", "libcpu_pipeline.so")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def _cuda_include():
    for d in ("/usr/local/cuda/include", "/usr/local/cuda/targets/sbsa-linux/include",
              "/usr/local/cuda/targets/x86_64-linux/include"):
        if os.path.exists(os.path.join(d, "vector_types.h")):
            return d
    return "/usr/local/cuda/include"


@pytest.fixture(scope="session")
def cpu_pipeline():
    """The kernels' per-thread bodies compiled for the CPU (tests/cpu_pipeline.cc)."""
    import ctypes
    os.makedirs(os.path.dirname(CPU_PIPE_LIB), exist_ok=True)
    csrc = os.path.join(ROOT, "skity_gb300", "csrc")
    deps = [CPU_PIPE_SRC] + [os.path.join(csrc, f) for f in os.listdir(csrc)]
    if not os.path.exists(CPU_PIPE_LIB) or any(
            os.path.getmtime(d) > os.path.getmtime(CPU_PIPE_LIB) for d in deps):
        r = subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                            "-I" + _cuda_include(), CPU_PIPE_SRC, "-o", CPU_PIPE_LIB],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
    lib = ctypes.CDLL(CPU_PIPE_LIB)
    lib.skc_cpu_render.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_void_p,
                                   ctypes.POINTER(ctypes.c_uint64)]
    lib.skc_cpu_render_mode.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_void_p,
                                        ctypes.POINTER(ctypes.c_uint64), ctypes.c_int,
                                        ctypes.c_uint64]
    lib.skc_cpu_introsort.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    lib.skc_std_sort.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    lib.skc_cpu_fixed_div_check.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]
    lib.skc_cpu_fixed_div_check.restype = ctypes.c_int64
    return lib


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu_ctx():
    """A context on cuda:0 over the freshly built library (fails loudly if
    the library or the GPU is missing)."""
    from skity_gb300 import build
    build.build()
    from skity_gb300.canvas import Context
    ctx = Context(0)
    yield ctx
    ctx.close()
