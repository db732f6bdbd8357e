"""Builds and loads libplume_gpu.so (the sm_103a CUDA library of csrc/).

The library is built in-tree next to this file.  Loading fails loudly when it
is missing or was built for another machine: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

from .abi import PlumeAtmosphere, PlumeDuct, PlumeGrid, PlumeInlet, PlumeOptions, PlumeSoA, PlumeStepLog

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
CSRC = os.path.join(PKG, "csrc")
LIBPATH = os.path.join(HERE, "libplume_gpu.so")
NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
              "--extended-lambda", "-Xcompiler", "-fPIC", "-shared"]
_lock = threading.Lock()
_LIB = None


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith((".cu", ".cuh")))


def build(force: bool = False, verbose: bool = False) -> str:
    """nvcc the library for sm_103a (cross-compiles without a GPU)."""
    newest = max(os.path.getmtime(s) for s in sources() + [os.path.join(PKG, "..", "include", "plume_gpu.h")])
    if not force and os.path.exists(LIBPATH) and os.path.getmtime(LIBPATH) >= newest:
        return LIBPATH
    nvcc = os.environ.get("NVCC", "nvcc")
    if not os.path.exists(nvcc) and os.path.exists("/usr/local/cuda/bin/nvcc"):
        nvcc = "/usr/local/cuda/bin/nvcc"
    tmp = LIBPATH + ".tmp"
    cmd = [nvcc] + NVCC_FLAGS + ["-o", tmp, os.path.join(CSRC, "plume_gpu.cu"),
                                 os.path.join(CSRC, "timestep_noalloc.cu"),
                                 os.path.join(CSRC, "grid_generate.cu")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed:\n" + r.stderr[-4000:])
    if verbose:
        print(r.stderr[-2000:])
    os.replace(tmp, LIBPATH)
    return LIBPATH


def lib():
    """The loaded CUDA library (ctypes)."""
    global _LIB
    with _lock:
        if _LIB is not None:
            return _LIB
        if not os.path.exists(LIBPATH):
            raise RuntimeError(f"{LIBPATH} is missing: run plume_gpu.build() (nvcc for sm_103a)")
        L = C.CDLL(LIBPATH)
        P = C.POINTER
        L.plume_create.argtypes = [P(PlumeOptions), P(PlumeGrid), P(C.c_void_p)]
        L.plume_destroy.argtypes = [C.c_void_p]
        L.plume_upload.argtypes = [C.c_void_p, P(PlumeSoA), C.c_size_t]
        L.plume_upload_device.argtypes = [C.c_void_p, P(PlumeSoA), C.c_size_t]
        L.plume_append.argtypes = [C.c_void_p, P(PlumeSoA), C.c_size_t]
        L.plume_set_ghost_state.argtypes = [C.c_void_p, P(C.c_uint64), P(C.c_double),
                                            P(C.c_double), C.c_size_t]
        L.plume_step.argtypes = [C.c_void_p, P(C.c_double)]
        L.plume_steps.argtypes = [C.c_void_p, C.c_int, P(PlumeStepLog)]
        L.plume_adapt_sml.argtypes = [C.c_void_p]
        L.plume_count.argtypes = [C.c_void_p, P(C.c_size_t), P(C.c_size_t)]
        L.plume_download.argtypes = [C.c_void_p, P(PlumeSoA), C.c_size_t, P(C.c_size_t)]
        L.plume_get_time.argtypes = [C.c_void_p, P(C.c_double), P(C.c_int), P(C.c_int)]
        L.plume_set_time.argtypes = [C.c_void_p, C.c_double, C.c_int, C.c_int, C.c_double]
        L.plume_neighbor_pairs.argtypes = [C.c_void_p, C.c_int, P(C.c_uint64), P(C.c_uint64),
                                           C.c_size_t, P(C.c_size_t)]
        L.plume_neighbor_pairs_of.argtypes = [C.c_void_p, C.c_int, P(C.c_uint64), C.c_size_t, P(C.c_uint64),
                                              P(C.c_uint64), C.c_size_t, P(C.c_size_t)]
        L.plume_phase_times.argtypes = [C.c_void_p, P(C.c_float), C.c_int]
        L.plume_launch_count.argtypes = [C.c_void_p, P(C.c_uint64)]
        L.plume_last_error.argtypes = [C.c_void_p, C.c_char_p, C.c_size_t]
        L.plume_version.restype = C.c_char_p
        L.plume_timestep_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t,
                                             C.c_double, C.c_void_p, C.c_void_p]
        L.plume_batch_create.argtypes = [P(PlumeOptions), P(PlumeGrid), C.c_int, P(C.c_void_p)]
        L.plume_batch_upload.argtypes = [C.c_void_p, P(PlumeSoA), P(C.c_uint16), C.c_size_t]
        L.plume_batch_append.argtypes = [C.c_void_p, P(PlumeSoA), P(C.c_uint16), C.c_size_t]
        L.plume_batch_download.argtypes = [C.c_void_p, P(PlumeSoA), P(C.c_uint16), C.c_size_t,
                                           P(C.c_size_t)]
        L.plume_batch_time.argtypes = [C.c_void_p, P(C.c_double), P(C.c_int), P(C.c_int), P(C.c_int)]
        L.plume_batch_run.argtypes = [C.c_void_p, C.c_int, C.c_int, P(C.c_int)]
        L.plume_adjoint_record.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.plume_set_wall_images.argtypes = [C.c_void_p, P(C.c_uint64), P(C.c_double), C.c_size_t]
        L.plume_apply_bcond.argtypes = [C.c_void_p]
        L.plume_gsph_gradients.argtypes = [C.c_void_p, P(C.c_uint64), P(C.c_double), C.c_size_t,
                                           P(C.c_size_t)]
        L.plume_set_bucket_involvement.argtypes = [C.c_void_p, P(C.c_uint8), C.c_size_t]
        L.plume_get_bucket_involvement.argtypes = [C.c_void_p, P(C.c_uint8), C.c_size_t]
        L.plume_scan_outside_layer.argtypes = [C.c_void_p, P(C.c_int)]
        L.plume_adapt_domain.argtypes = [C.c_void_p]
        L.plume_snapshot_begin.argtypes = [C.c_void_p, P(PlumeSoA), C.c_size_t]
        L.plume_grid_generate.argtypes = [P(C.c_double), P(C.c_double), C.c_double, C.c_int, P(PlumeGrid),
                                          P(C.c_uint8), P(C.c_int8), C.c_size_t, P(C.c_size_t)]
        L.plume_add_pressure_ghost.argtypes = [C.c_void_p, P(PlumeAtmosphere), C.c_uint64, P(C.c_size_t)]
        L.plume_add_wall_ghost.argtypes = [C.c_void_p, P(PlumeAtmosphere), C.c_uint64, P(C.c_size_t)]
        L.plume_add_air.argtypes = [C.c_void_p, P(PlumeAtmosphere), C.c_uint64, P(C.c_size_t)]
        L.plume_setup_erupt.argtypes = [C.c_void_p, P(PlumeDuct), C.c_uint64, P(C.c_size_t), P(C.c_size_t),
                                        P(C.c_double), P(C.c_double)]
        L.plume_search_bnd_images.argtypes = [C.c_void_p, P(C.c_size_t)]
        L.plume_adapt_step.argtypes = [C.c_void_p, P(PlumeAtmosphere), C.c_uint64, P(C.c_int), P(C.c_size_t)]
        L.plume_snapshot_end.argtypes = [C.c_void_p, P(C.c_size_t), P(C.c_double), P(C.c_int)]
        L.plume_set_inlet.argtypes = [C.c_void_p, P(PlumeInlet), C.c_int]
        L.plume_adjoint_backward.argtypes = [C.c_void_p, P(PlumeSoA), C.c_size_t, P(PlumeSoA), C.c_size_t,
                                             P(C.c_size_t), P(C.c_double)]
        _LIB = L
        return L
