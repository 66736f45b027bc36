"""A caller-defined DimDecomp plugin through the whole path.

The reference documents its DimDecomp vtable as the application's extension point (reshape.h:37-44).
tests/plugin/block_cyclic.c is such a plugin, written against the plugin struct only: a block-cyclic
distribution.  The same source is compiled against this library's headers here and against the
reference's for the golden fixture (tests/golden/make_plugin_golden.py runs the reference's own reshape
and split FFT with it).  The reshape into the block-cyclic decomposition must match the reference bit for
bit and the split FFT on it within 1e-12; the inverse returns N times the input.
"""
import ctypes
import json
import os
import subprocess

import numpy as np
import pytest

from decomp_mpi_gb300 import api
from decomp_mpi_gb300._lib import load
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PLUGIN_SRC = os.path.join(ROOT, "tests", "plugin", "block_cyclic.c")
PLUGIN_LIB = os.path.join(ROOT, "tests", "plugin", "_build", "libblock_cyclic.so")


def _plugin():
    if not os.path.exists(PLUGIN_LIB) or os.path.getmtime(PLUGIN_LIB) < os.path.getmtime(PLUGIN_SRC):
        os.makedirs(os.path.dirname(PLUGIN_LIB), exist_ok=True)
        subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-std=gnu11", "-I" + os.path.join(ROOT, "include"),
                        PLUGIN_SRC, "-o", PLUGIN_LIB], check=True)
    lib = ctypes.CDLL(PLUGIN_LIB)
    lib.make_block_cyclic.restype = ctypes.c_void_p
    lib.make_block_cyclic.argtypes = [ctypes.c_int] * 3
    return lib


def _golden():
    z = np.load(os.path.join(ROOT, "tests", "golden", "plugin_block_cyclic.npz"))
    return json.loads(str(z["meta"])), z


def _decomps(m):
    """(comm, src, dest): block | block | local and block_cyclic | block | local on the g0 x g1 grid."""
    comm = api.Comm(m["g0"] * m["g1"])
    src = api.decomp_from_spec(comm, "packed:block(%d,%d)|block(%d,%d)|local(%d)" % (
        m["L0"], m["g0"], m["L1"], m["g1"], m["L2"]))
    bc = _plugin().make_block_cyclic(m["L0"], m["b"], m["g0"])
    assert bc
    dims = (ctypes.c_void_p * 3)(bc, api._dim("block", m["L1"], m["g1"]), api._dim("local", m["L2"]))
    h = load().makePackedDecomp(comm.h, 3, dims)
    assert h, api.last_error()
    return comm, src, api.Decomp(comm, h)


def test_plugin_layout_matches_reference():
    """Host side only: the block-cyclic decomposition built from the plugin has the reference's extent, and
    every coordinate's address is where the reference's reshape put that coordinate's value."""
    m, z = _golden()
    comm, src, dst = _decomps(m)
    assert dst.extent() == m["dst_pitch"] and src.extent() == m["src_pitch"]
    P = m["g0"] * m["g1"]
    shape = (m["L0"], m["L1"], m["L2"])
    spec = "packed:block(%d,%d)|block(%d,%d)|local(%d)" % (m["L0"], m["g0"], m["L1"], m["g1"], m["L2"])
    glob = O.gather_global(P, spec, z["src"], m["src_pitch"], shape)
    for c in [(0, 0, 0), (5, 7, 3), (23, 11, 9), (13, 2, 8), (17, 10, 0)]:
        assert z["reshaped"][dst.global_offset(c)] == glob[c]


@pytest.mark.gpu
def test_plugin_reshape_and_split_fft_match_reference(cuda):
    import torch
    m, z = _golden()
    comm, src, dst = _decomps(m)
    P = m["g0"] * m["g1"]
    st = torch.cuda.current_stream(cuda).cuda_stream
    plan = api.ReshapePlan(comm, 16, src, dst)
    assert plan.src_pitch == m["src_pitch"] and plan.dest_pitch == m["dst_pitch"]
    a = torch.from_numpy(z["src"]).to(cuda)
    b = torch.zeros(P * m["dst_pitch"], dtype=torch.complex128, device=cuda)
    plan.run(a.data_ptr(), b.data_ptr(), st)
    torch.cuda.synchronize()
    assert np.array_equal(b.cpu().numpy(), z["reshaped"])

    wl = m["work_len"]
    work = torch.zeros(P * wl, dtype=torch.complex128, device=cuda)
    keep = b.clone()
    sp = api.SplitPlan(dst, b.data_ptr(), wl, work.data_ptr())
    assert sp.extent == m["split_extent"]
    held = z["slot"] >= 0
    want = z["work"][held]
    for arith in (api.ARITH_DF, api.ARITH_FP64):
        sp.set_arith(arith)
        b.copy_(keep)
        work.zero_()
        sp.run(api.FFTW_FORWARD, st)
        torch.cuda.synchronize()
        got = work.cpu().numpy()[held]
        assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-12, arith
        sp.run(api.FFTW_BACKWARD, st)
        torch.cuda.synchronize()
        back = b / (m["L0"] * m["L1"] * m["L2"])
        assert float((torch.linalg.vector_norm(back - keep) / torch.linalg.vector_norm(keep)).item()) < 1e-12
