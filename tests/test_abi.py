"""The C ABI without a GPU: libpfgpu.so builds, loads and exports every
function include/pfgpu.h declares; argument validation that happens on the
host returns its status codes; host-side helpers agree with the oracle."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "pfgpu.h"


@pytest.fixture(scope="module")
def lib():
    from platelet_fiber_gpu_gb300 import build, gpu
    build.build()
    return gpu.lib()


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"typedef struct[^;]*?\{.*?\}\s*\w+\s*;", "", text, flags=re.S)
    names = set()
    for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\(", text, flags=re.M):
        name = m.group(1)
        if name in ("sizeof", "typedef", "return"):
            continue
        names.add(name)
    return sorted(names)


def test_header_declares_the_reference_entry_points():
    names = declared_functions()
    for ref in ("fluid_allocGPUKernel", "fluid_initGPUKernel", "fluid_invokeGPUKernel", "fluid_releaseGPUKernel",
                "sem_allocGPUKernel", "sem_initGPUKernel", "sem_invokeGPUKernel_Force", "sem_copyGPUKernel",
                "sem_releaseGPUKernel", "fiber_allocGPUKernel", "fiber_init_GPUKernel", "fiber_copy_GPUKernel",
                "fiber_release_GPUKernel"):
        assert ref in names


def test_library_exports_every_declared_function(lib):
    names = declared_functions()
    assert len(names) > 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_host_validation_without_gpu(lib):
    h = C.c_void_p()
    lib.pfgpu_job_create.argtypes = [C.c_void_p, C.c_int, C.c_double, C.POINTER(C.c_void_p)]
    assert lib.pfgpu_job_create(None, 1, 0.0, C.byref(h)) == 1
    assert b"NULL" in lib.pfgpu_last_error()
    from platelet_fiber_gpu_gb300 import workloads as W
    sc = W.mixed_small()
    c = sc.to_c()
    assert lib.pfgpu_job_create(C.byref(c), 7, 0.0, C.byref(h)) == 1  # bad precision
    bad = W.mixed_small()
    bad.rec_tri = bad.rec_tri.copy()
    bad.rec_tri[0, 0] = 10 ** 6
    cb = bad.to_c()
    assert lib.pfgpu_job_create(C.byref(cb), 1, 0.0, C.byref(h)) == 1
    assert b"receptor triangle" in lib.pfgpu_last_error()
    lib.fluid_allocGPUKernel.restype = C.c_void_p
    lib.fluid_allocGPUKernel.argtypes = [C.c_void_p, C.c_float, C.c_float, C.c_int, C.c_int, C.c_int]
    assert lib.fluid_allocGPUKernel(None, 1e-8, 0.2, 0, 4, 4) is None
    lib.pfgpu_membrane_forces_noalloc.argtypes = [C.c_void_p, C.c_void_p]
    assert lib.pfgpu_membrane_forces_noalloc(None, None) == 1
    # membrane force bits outside PF_MEM_ALL | PF_MEM_FEMBEND
    odd = W.mixed_small()
    odd.membrane_forces = 64
    co = odd.to_c()
    assert lib.pfgpu_job_create(C.byref(co), 1, 0.0, C.byref(h)) == 1
    assert b"membrane force bits" in lib.pfgpu_last_error()
    # the no-allocation entry point has no scratch for the FEM bending chain
    args = (C.c_int * 7)(1, 8, 4, 4, 6, 0, 15 | 16)
    assert lib.pfgpu_membrane_forces_noalloc(C.cast(args, C.c_void_p), None) == 1
    assert b"FEM" in lib.pfgpu_last_error()


def test_receptor_uniforms_match_oracle(lib):
    from oracle import binding as ob
    out = np.zeros(2)
    lib.pfgpu_receptor_uniforms.argtypes = [C.c_uint64, C.c_int64, C.c_int64, C.POINTER(C.c_double)]
    lib.pfgpu_detach_uniform.restype = C.c_double
    lib.pfgpu_detach_uniform.argtypes = [C.c_uint64, C.c_int64]
    for seed, step, rid in ((1, 0, 0), (7, 39, 11), (2 ** 40 + 3, 123456789, 99999)):
        lib.pfgpu_receptor_uniforms(seed, step, rid, out.ctypes.data_as(C.POINTER(C.c_double)))
        np.testing.assert_array_equal(out, ob.receptor_uniforms(seed, step, rid))
        assert lib.pfgpu_detach_uniform(seed, step) == ob.detach_uniform(seed, step)


def test_scene_device_bytes_is_host_arithmetic(lib):
    from platelet_fiber_gpu_gb300 import gpu, workloads as W
    sc = W.plain_small()
    b32 = gpu.scene_device_bytes(sc, 1)
    b16 = gpu.scene_device_bytes(sc, 2)
    b64 = gpu.scene_device_bytes(sc, 0)
    assert b16 < b32 < b64
    assert b32 > 2 * 19 * sc.n_nodes * 4


def test_batch_shape_validation_without_gpu(lib):
    """Forcing the fused batch step's shapes is checked on the host: the
    row count and CTAs per SM in 1..64, marker threads a multiple of 32 up to
    256; zero hands the shapes back to the autotuner."""
    h = C.c_void_p()
    lib.pfgpu_batch_create.argtypes = [C.c_size_t, C.POINTER(C.c_void_p)]
    lib.pfgpu_batch_set_shape.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int]
    lib.pfgpu_batch_destroy.argtypes = [C.c_void_p]
    assert lib.pfgpu_batch_create(1 << 20, C.byref(h)) == 0
    try:
        assert lib.pfgpu_batch_set_shape(h, 4, 8, 128) == 0
        assert lib.pfgpu_batch_set_shape(h, 0, 0, 0) == 0
        for bad in ((4, 8, 100), (4, 8, 512), (0 - 1, 8, 128), (4, 0, 128), (65, 8, 128)):
            assert lib.pfgpu_batch_set_shape(h, *bad) == 1, bad
        assert lib.pfgpu_batch_set_shape(None, 4, 8, 128) == 1
        lib.pfgpu_batch_set_stop.argtypes = [C.c_void_p, C.c_int, C.c_int64]
        assert lib.pfgpu_batch_set_stop(h, 0, 5) == 1  # no job in the slot
        lib.pfgpu_job_set_stop.argtypes = [C.c_void_p, C.c_int64]
        assert lib.pfgpu_job_set_stop(None, 5) == 1
    finally:
        lib.pfgpu_batch_destroy(h)
