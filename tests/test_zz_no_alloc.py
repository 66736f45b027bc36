"""The no-allocation split-FFT entry point against the regular one.

dmg_split_run_noalloc is for callers that cannot allocate device memory at
the moment they run a transform: a real-time loop that must not wait on the
allocator, or an application that hands all of HBM to its own pool up front
so that a library's cudaMalloc would fail.  It keeps the intermediate
passes in the library's fixed 64 MiB device array instead of the upper half
of the caller's workspace.  It runs the same kernels on the same values as
runSplitPlan, so its results must be the same bits, call after call, since
every call reuses the same array; it must leave the workspace's upper half
alone and change no device memory in use.

This file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

from decomp_mpi_gb300 import api
from decomp_mpi_gb300._lib import load
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SENTINEL = 12345.0 - 6789.0j


def _setup(cuda, P, spec, shape, seed, dtype):
    import torch
    comm = api.Comm(P)
    start = api.decomp_from_spec(comm, spec)
    dp = start.extent()
    wl = 2 * int(np.prod(shape))
    rng = np.random.default_rng(seed)
    glob = rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)
    host = O.scatter_global(P, spec, glob, dp)
    tdt = torch.complex128 if dtype == api.C128 else torch.complex64
    host = torch.from_numpy(host).to(tdt)
    dat = host.to(cuda)
    work = torch.zeros(P * wl, dtype=tdt, device=cuda)
    plan = api.SplitPlan(start, dat.data_ptr(), wl, work.data_ptr(), dtype=dtype)
    return comm, start, plan, dat, work, host, wl


def _noalloc(plan, direction, stream):
    st = load().dmg_split_run_noalloc(ctypes.c_void_p(plan.h), direction, ctypes.c_void_p(stream))
    assert st == 0, api.last_error()


def _bits(t):
    return t.cpu().numpy().view(np.uint8)


CASES = [
    # (ranks, start decomposition, shape, element type, arithmetic, schedule)
    (4, "packed:block(32,2)|block(24,2)|local(20)", (32, 24, 20), api.C128, api.ARITH_DF, api.SCHEDULE_LINES),
    (16, "packed:block(48,4)|rotate(5,block(48,4))|local(40)", (48, 48, 40), api.C128, api.ARITH_DF,
     api.SCHEDULE_SPLIT),
    (4, "packed:block(32,2)|block(24,2)|local(20)", (32, 24, 20), api.C128, api.ARITH_FP64, api.SCHEDULE_LINES),
    (16, "packed:block(48,4)|rotate(5,block(48,4))|local(40)", (48, 48, 40), api.C128, api.ARITH_FP64,
     api.SCHEDULE_SPLIT),
    (4, "packed:block(64,2)|block(32,2)|local(16)", (64, 32, 16), api.C64, api.ARITH_FP32, api.SCHEDULE_LINES),
    (16, "packed:block(48,4)|rotate(5,block(48,4))|local(40)", (48, 48, 40), api.C64, api.ARITH_FP32,
     api.SCHEDULE_SPLIT),
    # 1024-point lines in the tensor-core form, and 256-point strided lines in FP32's wide tiles
    (4, "packed:block(8,2)|block(8,2)|local(1024)", (8, 8, 1024), api.C64, api.ARITH_TC16, api.SCHEDULE_LINES),
    (4, "packed:local(256)|block(16,2)|block(8,2)", (256, 16, 8), api.C64, api.ARITH_FP32, api.SCHEDULE_LINES),
]


@pytest.mark.parametrize("P,spec,shape,dtype,arith,sched", CASES)
def test_noalloc_matches_regular_run(P, spec, shape, dtype, arith, sched, cuda):
    import torch
    stream = torch.cuda.current_stream(cuda).cuda_stream
    comm, start, plan, dat, work, host, wl = _setup(cuda, P, spec, shape, 11, dtype)
    plan.set_arith(arith)
    plan.set_schedule(sched)
    ext = plan.extent64
    # the regular entry point's results (its first run uploads the plan's tables)
    plan.run(api.FFTW_FORWARD, stream)
    torch.cuda.synchronize()
    want_fwd = work.view(P, wl)[:, :ext].clone()
    plan.run(api.FFTW_BACKWARD, stream)
    torch.cuda.synchronize()
    want_inv = dat.clone()
    for call in range(2):  # two calls in a row, each against the regular entry point
        dat.copy_(host)
        work.zero_()
        # the upper half of each rank's workspace is where the regular run keeps its intermediates: the
        # no-allocation run must not touch it
        work.view(P, wl)[:, ext:] = SENTINEL
        upper = work.view(P, wl)[:, ext:].clone()
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info(cuda)[0]
        _noalloc(plan, api.FFTW_FORWARD, stream)
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info(cuda)[0]
        assert free1 == free0, "device memory in use changed by %d bytes" % (free0 - free1)
        assert np.array_equal(_bits(work.view(P, wl)[:, :ext]), _bits(want_fwd)), call
        _noalloc(plan, api.FFTW_BACKWARD, stream)
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info(cuda)[0] == free0
        assert np.array_equal(_bits(dat), _bits(want_inv)), call
        assert torch.equal(work.view(P, wl)[:, ext:], upper), "the workspace's upper half changed"


def test_noalloc_rejects_plans_beyond_the_array(cuda):
    """A 192^3 complex128 transform on 4 ranks needs about 113 MB of scratch, more than the 64 MiB array."""
    comm = api.Comm(4)
    start = api.decomp_from_spec(comm, "packed:block(192,2)|block(192,2)|local(192)")
    plan = api.SplitPlan(start, 1 << 20, 2 * 192 ** 3, 1 << 21)
    assert load().dmg_noalloc_scratch_bytes() == 64 << 20
    st = load().dmg_split_run_noalloc(ctypes.c_void_p(plan.h), api.FFTW_FORWARD, None)
    assert st == 5  # DMG_ERR_BOUNDS, before any device work
    assert "scratch" in api.last_error()


def test_noalloc_needs_uploaded_tables(cuda):
    import torch
    comm, start, plan, dat, work, host, wl = _setup(cuda, 4, "packed:block(16,2)|block(16,2)|local(16)",
                                                    (16, 16, 16), 3, api.C128)
    st = load().dmg_split_run_noalloc(ctypes.c_void_p(plan.h), api.FFTW_FORWARD,
                                      ctypes.c_void_p(torch.cuda.current_stream(cuda).cuda_stream))
    assert st == 1  # DMG_ERR_ARG: run the plan once first
