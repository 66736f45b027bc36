"""Loader and ctypes signatures of the in-tree ``libdecomp_gb300.so``.

The library is the product: the reference's C API (reshape.h, split_fft.h
and the decomposition headers under ``include/``) backed by sm_103a kernels.
It must be built first (``__graft_entry__.build()`` or
``python decomp_mpi_gb300/build.py``); loading fails loudly otherwise, and
there is no fallback path.
"""
from __future__ import annotations

import ctypes
import os

from .build import LIB_PATH

_vp = ctypes.c_void_p
_i = ctypes.c_int
_ll = ctypes.c_longlong
_ip = ctypes.POINTER(ctypes.c_int)
_cp = ctypes.c_char_p

# name: (restype, argtypes)
SIGNATURES = {
    # virtual communicator and errors
    "dmg_comm_create": (_vp, [_i]),
    "dmg_comm_free": (None, [_vp]),
    "dmg_comm_set_rank": (_i, [_vp, _i]),
    "dmg_last_error": (_cp, []),
    "dmg_last_error_code": (_i, []),
    "dmg_clear_error": (None, []),
    "dmg_set_error_printing": (_i, [_i]),
    "dmg_set_stream": (None, [_vp]),
    "dmg_get_stream": (_vp, []),
    "dmg_device_synchronize": (_i, []),
    # index sets
    "makeIndex": (_vp, []),
    "freeIndex": (None, [_vp]),
    "addIndex": (None, [_vp, _i]),
    "sizeIndex": (_i, [_vp]),
    # DimDecomp plugins
    "makeBlockDecomp": (_vp, [_i, _i]),
    "makeBlockDecompWithFactor": (_vp, [_i, _i, _i]),
    "makeLocalDecomp": (_vp, [_i]),
    "makeSingleDecomp": (_vp, [_i, _i, _i]),
    "makeRotatedDecomp": (_vp, [_i, _vp]),
    "makeInterleaveDecomp": (_vp, [_vp, _i]),
    "makeFactorReverseDecomp": (_vp, [_i, _i, _vp]),
    "freeDimDecomp": (None, [_vp]),
    "cloneDimDecomp": (_vp, [_vp]),
    "sizeDimDecomp": (_i, [_vp]),
    # axis / N-D decompositions
    "makeAxisDecomp": (_vp, [_vp, _vp, _i, _i]),
    "freeAxisDecomp": (None, [_vp]),
    "isLocal": (_i, [_vp, _i]),
    "makeDecomp": (_vp, [_i, ctypes.POINTER(_vp)]),
    "makePackedDecomp": (_vp, [_vp, _i, ctypes.POINTER(_vp)]),
    "makeFactorReverseAxisDecomp": (_vp, [_i, _i, _vp]),
    "freeDecomp": (None, [_vp]),
    "extent": (_i, [_vp]),
    "extent64": (_ll, [_vp]),
    "rankExtent64": (_ll, [_vp, _i]),
    "compatible": (_i, [_vp, _vp]),
    "myRank": (_i, [_vp]),
    "isCoordLocal": (_i, [_vp, _i, _i]),
    "areCoordsLocal": (_i, [_vp, _ip]),
    "getOffset": (_i, [_vp, _ip]),
    "ownerRank": (_i, [_vp, _ip]),
    "globalOffset64": (_ll, [_vp, _ip, _ll]),
    # reshape plans
    "makeReshapePlan": (_vp, [_vp, _i, _vp, _vp]),
    "freeReshapePlan": (None, [_vp]),
    "runReshapePlan": (None, [_vp, _vp, _vp, _vp]),
    "checkReshapePlanBounds": (_i, [_vp, _i, _i, _i]),
    "dmg_reshape_run": (_i, [_vp, _vp, _vp, _vp]),
    "dmg_reshape_run_group": (_i, [_i, _vp, _vp, _vp, _vp]),
    "dmg_reshape_set_pitch": (_i, [_vp, _ll, _ll]),
    "dmg_reshape_pitch": (_ll, [_vp, _i]),
    "dmg_reshape_bytes": (_ll, [_vp]),
    "dmg_reshape_elements": (_ll, [_vp]),
    "dmg_reshape_describe": (_cp, [_vp]),
    "dmg_reshape_launches": (_i, [_vp]),
    # split FFT
    "makeProcessorGrid": (_ip, [_vp, _i, _ip]),
    "makeInterleavedDecomp": (_vp, [_i, _vp, _ip, _ip, _ip]),
    "makeBlockedDecomp": (_vp, [_i, _vp, _ip, _ip, _ip]),
    "gcd": (ctypes.c_uint, [ctypes.c_uint, ctypes.c_uint]),
    "makeSplitPlan": (_vp, [_i, _vp, _vp, _i, _vp]),
    "makeParallelPlan": (_vp, [_vp, _ip, _vp, _i, _vp]),
    "proposeParallelPlan": (_vp, [_i, _vp, _ip, _vp, _i, _vp]),
    "buildParallelPlan": (_vp, [_i, _i, _i, _vp, _i, _ip, _ip, _ip, _ip, _ip, _vp, _i, _vp]),
    "autotuneParallelPlan": (_vp, [_vp, _vp, _i, _vp]),
    "dmg_autotuneParallelPlanTyped": (_vp, [_vp, _vp, _ll, _vp, _i, _i]),
    "dmg_autotune_cache_clear": (None, []),
    "dmg_autotune_cache_entries": (_i, []),
    "dmg_autotune_last_timed": (_i, []),
    "dmg_split_set_tile": (_i, [_vp, _i]),
    "dmg_split_get_tile": (_i, [_vp]),
    "dmg_split_set_radix": (_i, [_vp, _i]),
    "dmg_split_get_radix": (_i, [_vp]),
    "dmg_makeSplitPlanTyped": (_vp, [_i, _vp, _vp, _ll, _vp, _i]),
    "dmg_makeParallelPlanTyped": (_vp, [_vp, _ip, _vp, _ll, _vp, _i]),
    "runSplitPlan": (None, [_vp, _i]),
    "dmg_split_run": (_i, [_vp, _i, _vp]),
    "freeSplitPlan": (None, [_vp]),
    "getTransformed": (_vp, [_vp]),
    "getTransformedExact": (_vp, [_vp]),
    "dmg_split_set_buffers": (_i, [_vp, _vp, _vp]),
    "dmg_split_set_dat_pitch": (_i, [_vp, _ll]),
    "dmg_split_launches": (_i, [_vp, _i]),
    "dmg_split_flops": (ctypes.c_double, [_vp]),
    "dmg_split_describe": (_cp, [_vp]),
    "dmg_split_set_timing": (_i, [_vp, _i]),
    "dmg_split_collect_times": (_i, [_vp]),
    "dmg_split_pass_times": (_i, [_vp, _i, ctypes.POINTER(ctypes.c_float), _i]),
    "dmg_split_run_noalloc": (_i, [_vp, _i, _vp]),
    "dmg_split_set_arith": (_i, [_vp, _i]),
    "dmg_split_get_arith": (_i, [_vp]),
    "dmg_split_device_status": (_i, [_vp]),
    "dmg_split_set_schedule": (_i, [_vp, _i]),
    "dmg_split_run_batch": (_i, [_vp, _i, _vp, _i, _vp, _vp, _vp]),
    "dmg_split_batch_launches": (_i, [_vp, _i, _i]),
    "dmg_split_run_group": (_i, [_i, _vp, _i, _vp]),
    "dmg_split_run_group_batch": (_i, [_i, _vp, _vp, _vp, _vp, _vp, _i, _vp]),
    "dmg_split_group_launches": (_i, [_i, _vp, _i]),
    "dmg_split_extent64": (_ll, [_vp]),
    "dmg_decomp_scale": (_i, [_vp, _i, _vp, ctypes.POINTER(_vp), _i, _vp]),
    "dmg_visit_fill_index": (_i, [_vp, _i, _vp, _vp]),
    "dmg_server_create": (_vp, [_i, _ll, _i, _i]),
    "dmg_server_set_arith": (_i, [_vp, _i, _i]),
    "dmg_server_set_mixing": (_i, [_vp, _i]),
    "dmg_server_job_sizes": (_i, [_vp, _i, _i, ctypes.POINTER(_ll), ctypes.POINTER(_ll), ctypes.POINTER(_ll)]),
    "dmg_server_submit": (_ll, [_vp, _vp]),
    "dmg_server_poll": (_i, [_vp, _vp, _i]),
    "dmg_server_drain": (_i, [_vp]),
    "dmg_server_status": (_i, [_vp, ctypes.POINTER(_i), ctypes.POINTER(_i), ctypes.POINTER(_ll)]),
    "dmg_server_destroy": (None, [_vp]),
    "dmg_makeGlobalDecomp": (_vp, [_vp, _i, _ip]),
    "dmg_io_gather": (_i, [_vp, _i, _vp, _vp, _vp]),
    "dmg_io_scatter": (_i, [_vp, _i, _vp, _vp, _vp]),
    "dmg_io_write_file": (_i, [_cp, _vp, _i, _vp, _vp]),
    "dmg_io_read_file": (_i, [_cp, _vp, _i, _vp, _vp]),
    "dmg_io_view": (_ll, [_vp, _i, ctypes.POINTER(_ll), ctypes.POINTER(_ll), _ll]),
    "dmg_split_get_schedule": (_i, [_vp]),
    "dmg_noalloc_scratch_bytes": (ctypes.c_size_t, []),
}

_lib = None


def load():
    """Load the library (once) and attach signatures; raises if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                "libdecomp_gb300.so is not built (%s); run __graft_entry__.build() first" % LIB_PATH)
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def last_error() -> str:
    return load().dmg_last_error().decode(errors="replace")


class DecompError(RuntimeError):
    """An entry point of the library reported an error."""


def check(status: int, what: str) -> None:
    if status != 0:
        raise DecompError("%s failed (%d): %s" % (what, status, last_error()))
