"""The no-allocation split-FFT entry point against the regular one.

dmg_split_run_noalloc exists for callers that cannot allocate device memory
when they run a transform (inside a CUDA graph capture, a real-time loop, an
application that owns all of HBM through its own pool): it keeps the
intermediate passes in the library's fixed 64 MiB device array instead of
the upper half of the caller's workspace.  Its results must equal those of
runSplitPlan, call after call, since every call reuses the same array.

This file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

from decomp_mpi_gb300 import api
from decomp_mpi_gb300._lib import load
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative L2, the FP64 bar of the other FFT tests


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _setup(cuda, P, spec, shape, seed):
    import torch
    comm = api.Comm(P)
    start = api.decomp_from_spec(comm, spec)
    dp = start.extent()
    wl = 2 * int(np.prod(shape))
    rng = np.random.default_rng(seed)
    glob = rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)
    host = O.scatter_global(P, spec, glob, dp)
    dat = torch.from_numpy(host).to(cuda)
    work = torch.zeros(P * wl, dtype=torch.complex128, device=cuda)
    plan = api.SplitPlan(start, dat.data_ptr(), wl, work.data_ptr())
    return comm, start, plan, dat, work, host


def _noalloc(plan, direction, stream):
    st = load().dmg_split_run_noalloc(ctypes.c_void_p(plan.h), direction, ctypes.c_void_p(stream))
    assert st == 0, api.last_error()


@pytest.mark.parametrize("P,spec,shape", [
    (4, "packed:block(32,2)|block(24,2)|local(20)", (32, 24, 20)),
    (16, "packed:block(48,4)|rotate(5,block(48,4))|local(40)", (48, 48, 40)),
])
def test_noalloc_matches_regular_run(P, spec, shape, cuda):
    import torch
    stream = torch.cuda.current_stream(cuda).cuda_stream
    comm, start, plan, dat, work, host = _setup(cuda, P, spec, shape, seed=11)
    # reference results from the regular entry point (this also uploads the plan's tables)
    plan.run(api.FFTW_FORWARD, stream)
    torch.cuda.synchronize()
    want_fwd = work.cpu().numpy().copy()
    plan.run(api.FFTW_BACKWARD, stream)
    torch.cuda.synchronize()
    want_inv = dat.cpu().numpy().copy()
    _, mask = O.split_expected_output(P, spec, np.zeros(shape), 2 * int(np.prod(shape)))
    held = O.global_offsets(P, spec, start.extent(), shape).ravel()
    for call in range(2):  # two calls in a row, each against the regular entry point
        dat.copy_(torch.from_numpy(host))
        work.zero_()
        _noalloc(plan, api.FFTW_FORWARD, stream)
        torch.cuda.synchronize()
        got_fwd = work.cpu().numpy()
        assert _rel(got_fwd[mask], want_fwd[mask]) < TOL, call
        _noalloc(plan, api.FFTW_BACKWARD, stream)
        torch.cuda.synchronize()
        got_inv = dat.cpu().numpy()
        assert _rel(got_inv[held], want_inv[held]) < TOL, call


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
    comm, start, plan, dat, work, host = _setup(cuda, 4, "packed:block(16,2)|block(16,2)|local(16)", (16, 16, 16),
                                                seed=3)
    st = load().dmg_split_run_noalloc(ctypes.c_void_p(plan.h), api.FFTW_FORWARD,
                                      ctypes.c_void_p(torch.cuda.current_stream(cuda).cuda_stream))
    assert st == 1  # DMG_ERR_ARG: run the plan once first
