"""Grouped split FFTs: the k-th passes of several plans of different sizes in one launch.

A service that transforms many small arrays of different shapes pays a
kernel launch per pass per array when it runs them one by one;
dmg_split_run_group runs up to 16 plans with one launch per pass index.
Each plan's passes run the runtime-length stages of its radix schedule, the
same kernels on the same values as runSplitPlan with that schedule, so the
grouped results must be the same bits as the plans' own runs, forward and
backward, in every arithmetic.
"""
import ctypes

import numpy as np
import pytest

from decomp_mpi_gb300 import api
from decomp_mpi_gb300._lib import load
from oracle import oracle as O

# (ranks, start decomposition, shape, schedule): cubes, a slab, 2D and long lines, two pass schedules
GROUP = [
    (4, "packed:block(32,2)|block(24,2)|local(20)", (32, 24, 20), api.SCHEDULE_LINES),
    (16, "packed:block(48,4)|rotate(5,block(64,4))|local(32)", (48, 64, 32), api.SCHEDULE_SPLIT),
    (4, "packed:block(12,2)|block(18,2)", (12, 18), None),
    (8, "packed:block(14,2)|block(21,4)|local(11)", (14, 21, 11), api.SCHEDULE_SPLIT),
    (16, "packed:block(64,4)|block(16,4)|local(1024)", (64, 16, 1024), api.SCHEDULE_LINES),
    (6, "packed:block(12,3)|block(10,2)|local(6)", (12, 10, 6), None),
]


def _fake_plan(P, spec, shape, dtype=api.C128, radix=api.RADIX_PLAN8, arith=None):
    comm = api.Comm(P)
    S = api.decomp_from_spec(comm, spec)
    wl = 2 * int(np.prod(shape))
    sp = api.SplitPlan(S, 0x100000, wl, 0x200000, dtype=dtype, arith=arith)
    sp.set_radix(radix)
    sp._keep = (comm, S)
    return sp


def _run_group(plans, direction):
    n = len(plans)
    arr = (ctypes.c_void_p * max(n, 1))(*[p.h for p in plans])
    return load().dmg_split_run_group(n, arr, int(direction), None)


def test_group_launch_count_is_the_longest_plans_passes():
    plans = [_fake_plan(P, spec, shape) for P, spec, shape, _ in GROUP[:4]]
    for d in (api.FFTW_FORWARD, api.FFTW_BACKWARD):
        # double-float plans (the complex128 default) add their exponent pre-pass each
        most = max(p.launches(d) - 1 for p in plans)
        assert api.split_group_launches(plans, d) == most + len(plans)
    fp64 = [_fake_plan(P, spec, shape, arith=api.ARITH_FP64) for P, spec, shape, _ in GROUP[:3]]
    assert api.split_group_launches(fp64, api.FFTW_FORWARD) == max(p.launches() for p in fp64)


def test_group_rejects_before_device_work():
    a = _fake_plan(*GROUP[0][:3])
    b = _fake_plan(*GROUP[2][:3])
    assert _run_group([], api.FFTW_FORWARD) == 1
    assert _run_group([a, b], 7) == 1
    assert _run_group([a, a], api.FFTW_FORWARD) == 1
    assert "twice" in api.last_error()
    fixed = _fake_plan(*GROUP[2][:3], radix=api.RADIX_FIXED)
    assert _run_group([a, fixed], api.FFTW_FORWARD) == 1
    assert "radix" in api.last_error()
    fp64 = _fake_plan(*GROUP[2][:3], arith=api.ARITH_FP64)
    assert _run_group([a, fp64], api.FFTW_FORWARD) == 1
    assert "arithmetic" in api.last_error()
    c64 = _fake_plan(*GROUP[2][:3], dtype=api.C64)
    assert _run_group([a, c64], api.FFTW_FORWARD) == 1
    many = [_fake_plan(4, "packed:block(8,2)|block(8,2)", (8, 8)) for _ in range(17)]
    assert _run_group(many, api.FFTW_FORWARD) == 1
    assert api.split_group_launches(many, api.FFTW_FORWARD) == 0
    assert api.split_group_launches(many[:16], api.FFTW_FORWARD) == many[0].launches() - 1 + 16


def _bits(t):
    return t.cpu().numpy().view(np.uint8)


class _Job:
    def __init__(self, P, spec, shape, schedule, dtype, arith, radix, seed, cuda):
        import torch
        self.P, self.spec, self.shape = P, spec, shape
        self.comm = api.Comm(P)
        self.S = api.decomp_from_spec(self.comm, spec)
        self.dp = self.S.extent()
        self.wl = 2 * int(np.prod(shape))
        rng = np.random.default_rng(seed)
        self.glob = rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)
        tdt = torch.complex128 if dtype == api.C128 else torch.complex64
        npdt = np.complex128 if dtype == api.C128 else np.complex64
        self.host = torch.from_numpy(O.scatter_global(P, spec, self.glob, self.dp).astype(npdt))
        self.dat = self.host.to(cuda)
        self.work = torch.zeros(P * self.wl, dtype=tdt, device=cuda)
        self.plan = api.SplitPlan(self.S, self.dat.data_ptr(), self.wl, self.work.data_ptr(), dtype=dtype,
                                  arith=arith, schedule=schedule)
        self.plan.set_radix(radix)

    def reset(self):
        self.dat.copy_(self.host)
        self.work.zero_()


@pytest.mark.gpu
@pytest.mark.parametrize("dtype,arith", [(api.C128, api.ARITH_FP64), (api.C128, api.ARITH_DF),
                                         (api.C64, api.ARITH_FP32), (api.C64, api.ARITH_TC16)],
                         ids=["fp64", "df", "fp32", "tc16"])
def test_group_matches_each_plans_own_run(dtype, arith, cuda):
    import torch
    stream = torch.cuda.current_stream(cuda).cuda_stream
    jobs = [_Job(P, spec, shape, sch, dtype, arith, api.RADIX_PLAN8 if i % 2 == 0 else api.RADIX_PLAN4, 20 + i, cuda)
            for i, (P, spec, shape, sch) in enumerate(GROUP)]
    want_f, want_b = [], []
    for j in jobs:
        j.plan.run(api.FFTW_FORWARD, stream)
        torch.cuda.synchronize()
        want_f.append(j.work.clone())
        j.plan.run(api.FFTW_BACKWARD, stream)
        torch.cuda.synchronize()
        want_b.append(j.dat.clone())
    tol = 1e-12 if dtype == api.C128 else 2e-6
    for call in range(2):
        for j in jobs:
            j.reset()
        torch.cuda.synchronize()
        api.split_run_group([j.plan for j in jobs], api.FFTW_FORWARD, stream)
        torch.cuda.synchronize()
        for i, j in enumerate(jobs):
            assert np.array_equal(_bits(j.work), _bits(want_f[i])), (call, i)
            if call == 0:
                exp, mask = O.split_expected_output(j.P, j.spec, j.glob, j.wl)
                got = j.work.cpu().numpy().astype(np.complex128)[mask]
                assert np.linalg.norm(got - exp[mask]) / np.linalg.norm(exp[mask]) < tol, i
        api.split_run_group([j.plan for j in jobs], api.FFTW_BACKWARD, stream)
        torch.cuda.synchronize()
        for i, j in enumerate(jobs):
            assert np.array_equal(_bits(j.dat), _bits(want_b[i])), (call, i)


@pytest.mark.gpu
def test_group_of_one_and_of_sixteen(cuda):
    """The smallest and the largest groups: one plan, and sixteen plans of eight shapes in double-float."""
    import torch
    stream = torch.cuda.current_stream(cuda).cuda_stream
    shapes = [(4, "packed:block(%d,2)|block(%d,2)|local(%d)" % (a, b, c), (a, b, c))
              for a, b, c in ((8, 8, 8), (16, 8, 12), (10, 12, 14), (32, 16, 8), (24, 24, 24), (20, 6, 18),
                              (64, 8, 4), (12, 36, 10))]
    for sel in ([0], list(range(16))):
        jobs = [_Job(*shapes[i % 8], None, api.C128, api.ARITH_DF, api.RADIX_PLAN8, 40 + i, cuda) for i in sel]
        want = []
        for j in jobs:
            j.plan.run(api.FFTW_FORWARD, stream)
            torch.cuda.synchronize()
            want.append(j.work.clone())
            j.reset()
        torch.cuda.synchronize()
        api.split_run_group([j.plan for j in jobs], api.FFTW_FORWARD, stream)
        torch.cuda.synchronize()
        for i, j in enumerate(jobs):
            assert np.array_equal(_bits(j.work), _bits(want[i])), (len(sel), i)


@pytest.mark.gpu
def test_group_batch_job_table(cuda):
    """dmg_split_run_group_batch: two plans of different shapes with two and one arrays each give the bits of
    each array's own run (double-float, with an exponent word per array)."""
    import torch
    stream = torch.cuda.current_stream(cuda).cuda_stream
    specs = [GROUP[0], GROUP[2]]
    jobs = [[_Job(P, spec, shape, sch, api.C128, api.ARITH_DF, api.RADIX_PLAN8, 60 + 10 * i + k, cuda)
             for k in range(2 - i)] for i, (P, spec, shape, sch) in enumerate(specs)]
    want = []
    for arrs in jobs:
        for j in arrs:
            j.plan.run(api.FFTW_FORWARD, stream)
            torch.cuda.synchronize()
            want.append(j.work.clone())
            j.reset()
    torch.cuda.synchronize()
    flat = [j for arrs in jobs for j in arrs]
    scales = torch.zeros(64 * len(flat), dtype=torch.int32, device=cuda)
    api.split_run_group_batch([arrs[0].plan for arrs in jobs], [len(a) for a in jobs],
                              [j.dat.data_ptr() for j in flat], [j.work.data_ptr() for j in flat],
                              [scales.data_ptr() + 256 * i for i in range(len(flat))], api.FFTW_FORWARD, stream)
    torch.cuda.synchronize()
    for i, j in enumerate(flat):
        assert np.array_equal(_bits(j.work), _bits(want[i])), i
