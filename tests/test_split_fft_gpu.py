"""GPU split 3D FFT through the C-ABI against the reference's fixtures and the FP64 oracle."""
import numpy as np
import pytest

from decomp_mpi_gb300 import api
from oracle import oracle as O
from tests.golden_cases import split_case, split_names

pytestmark = pytest.mark.gpu

TOL_C128 = 1e-12  # relative L2, FP64
TOL_C64 = 2e-6    # relative L2, FP32


def _rel(a, b):
    # scaled by the largest magnitude first, so that values near the ends of
    # the FP64 range neither overflow nor underflow the norms
    m = float(np.max(np.abs(b)))
    if m == 0.0:
        return float(np.max(np.abs(a)))
    return float(np.linalg.norm((a - b) / m) / np.linalg.norm(b / m))


class Run:
    """One split plan on the GPU with its buffers."""

    def __init__(self, P, spec, shape, cuda, mode=0, B=None, dtype=api.C128, work_len=None, seed=0, arith=None,
                 scale=1.0, schedule=None):
        import torch
        self.torch = torch
        self.P, self.spec, self.shape = P, spec, tuple(shape)
        self.comm = api.Comm(P)
        self.S = api.decomp_from_spec(self.comm, spec)
        self.dp = self.S.extent()
        self.wl = work_len or 2 * int(np.prod(shape))
        rng = np.random.default_rng(seed)
        self.glob = (rng.uniform(-1, 1, self.shape) + 1j * rng.uniform(-1, 1, self.shape)) * scale
        tdt = torch.complex128 if dtype == api.C128 else torch.complex64
        self.npdt = np.complex128 if dtype == api.C128 else np.complex64
        host = O.scatter_global(P, spec, self.glob, self.dp).astype(self.npdt)
        self.dat = torch.from_numpy(host).to(cuda)
        self.work = torch.zeros(P * self.wl, dtype=tdt, device=cuda)
        self.plan = api.SplitPlan(self.S, self.dat.data_ptr(), self.wl, self.work.data_ptr(),
                                  slab=mode if mode < 2 else 0, B=B if mode == 2 else None, dtype=dtype,
                                  arith=arith, schedule=schedule)
        self.mode, self.B = mode, B
        self.stream = torch.cuda.current_stream(cuda).cuda_stream

    def forward(self):
        self.plan.run(api.FFTW_FORWARD, self.stream)
        self.torch.cuda.synchronize()
        return self.work.cpu().numpy()

    def inverse(self):
        self.plan.run(api.FFTW_BACKWARD, self.stream)
        self.torch.cuda.synchronize()
        return self.dat.cpu().numpy()


@pytest.mark.parametrize("name", split_names())
def test_golden_forward(name, cuda):
    """Storage-order parity with the reference's work buffer (FFTW replaced by the FP64 oracle FFT)."""
    import torch
    m, z = split_case(name)
    P, wl = m["P"], m["work_len"]
    comm = api.Comm(P)
    S = api.decomp_from_spec(comm, m["spec"])
    assert S.extent() == m["dat_pitch"]
    dat = torch.from_numpy(z["dat"].copy()).to(cuda)
    work = torch.zeros(P * wl, dtype=torch.complex128, device=cuda)
    plan = api.SplitPlan(S, dat.data_ptr(), wl, work.data_ptr(), slab=m["mode"] if m["mode"] < 2 else 0,
                         B=m["B"] if m["mode"] == 2 else None)
    plan.run(api.FFTW_FORWARD, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got = work.cpu().numpy()
    held = z["slot"] >= 0
    assert _rel(got[held], z["work"][held]) < TOL_C128


CASES = [
    # (P, start spec, shape, mode, B)
    (4, "packed:block(64,2)|block(64,2)|local(64)", (64, 64, 64), 0, None),  # config: 64^3 on 2x2
    (4, "packed:local(8)|block(12,2)|block(16,2)", (8, 12, 16), 0, None),
    (16, "packed:block(48,4)|rotate(5,block(48,4))|local(48)", (48, 48, 48), 0, None),
    (16, "packed:block(120,4)|block(120,4)|local(120)", (120, 120, 120), 0, None),
    (8, "packed:block(14,2)|block(21,4)|local(11)", (14, 21, 11), 0, None),  # primes 7, 11, 3
    (4, "packed:local(8)|block(12,2)|block(16,2)", (8, 12, 16), 1, None),     # slab
    (4, "packed:local(8)|block(12,2)|block(16,2)", (8, 12, 16), 2, [8, 12, 16]),  # every A = 1
    (4, "packed:local(8)|block(12,2)|block(16,2)", (8, 12, 16), 2, [1, 12, 16]),
    (4, "packed:block(30,4)", (30,), 0, None),                                 # 1D
    (4, "packed:block(12,2)|block(18,2)", (12, 18), 0, None),                  # 2D
    (64, "packed:frev(16,8,block(128,8))|rotate(3,block(64,8))|local(32)", (128, 64, 32), 0, None),
    (4, "packed:block(5,4)|local(6)|local(4)", (5, 6, 4), 0, None),          # rank 3 holds nothing
    (4, "packed:block(6,4)|block(9,1)|local(8)", (6, 9, 8), 0, None),        # uneven blocks 2, 2, 2, 0
]


@pytest.mark.parametrize("schedule", [api.SCHEDULE_LINES, api.SCHEDULE_SPLIT], ids=["lines", "split"])
@pytest.mark.parametrize("P,spec,shape,mode,B", CASES, ids=[str(c[2]) + "m%d" % c[3] for c in CASES])
def test_forward_and_inverse_fp64(P, spec, shape, mode, B, schedule, cuda):
    """Double-float arithmetic (the complex128 default) in both pass schedules."""
    r = Run(P, spec, shape, cuda, mode, B, schedule=schedule)
    assert r.plan.schedule == schedule
    got = r.forward()
    exp, mask = O.split_expected_output(P, spec, r.glob, r.wl, mode, B)
    assert _rel(got[mask], exp[mask]) < TOL_C128
    back = r.inverse()
    g = O.gather_global(P, spec, back, r.dp, r.shape) / np.prod(r.shape)
    assert _rel(g, r.glob) < TOL_C128


@pytest.mark.parametrize("schedule", [api.SCHEDULE_LINES, api.SCHEDULE_SPLIT], ids=["lines", "split"])
@pytest.mark.parametrize("P,spec,shape", [
    (4, "packed:block(64,2)|block(64,2)|local(64)", (64, 64, 64)),
    (16, "packed:block(120,4)|block(120,4)|local(120)", (120, 120, 120)),
    (64, "packed:frev(16,8,block(128,8))|rotate(3,block(64,8))|local(32)", (128, 64, 32)),
])
def test_forward_and_inverse_fp32(P, spec, shape, schedule, cuda):
    r = Run(P, spec, shape, cuda, dtype=api.C64, schedule=schedule)
    got = r.forward()
    exp, mask = O.split_expected_output(P, spec, r.glob, r.wl)
    assert _rel(got[mask].astype(np.complex128), exp[mask]) < TOL_C64
    back = r.inverse()
    g = O.gather_global(P, spec, back.astype(np.complex128), r.dp, r.shape) / np.prod(r.shape)
    assert _rel(g, r.glob) < TOL_C64


@pytest.mark.parametrize("dtype", [api.C128, api.C64], ids=["c128", "c64"])
@pytest.mark.parametrize("P,spec,shape", [
    # long contiguous lines (256 and 512 points, each thread keeping its line coordinates) and
    # passes whose walks run along the first vector axis
    (16, "packed:block(16,4)|block(32,4)|local(256)", (16, 32, 256)),
    (4, "packed:block(8,2)|frev(4,2,block(8,2))|local(512)", (8, 8, 512)),
    (16, "packed:frev(16,16,block(256,4))|block(8,4)|local(64)", (256, 8, 64)),
    # 1024- and 2048-point lines (twiddles read through L1 for the 16-byte types)
    (4, "packed:block(8,2)|block(4,2)|local(1024)", (8, 4, 1024)),
    (4, "packed:block(4,2)|block(4,2)|local(2048)", (4, 4, 2048)),
], ids=["16x32x256", "8x8x512", "256x8x64", "8x4x1024", "4x4x2048"])
def test_long_lines(P, spec, shape, dtype, cuda):
    r = Run(P, spec, shape, cuda, dtype=dtype, schedule=api.SCHEDULE_LINES)
    tol = TOL_C128 if dtype == api.C128 else TOL_C64
    got = r.forward().astype(np.complex128)
    exp, mask = O.split_expected_output(P, spec, r.glob, r.wl)
    assert _rel(got[mask], exp[mask]) < tol
    back = r.inverse().astype(np.complex128)
    g = O.gather_global(P, spec, back, r.dp, r.shape) / np.prod(r.shape)
    assert _rel(g, r.glob) < tol


def test_delta_input_known_answer(cuda):
    """fftw_bench.c's delta at the origin: the forward transform is all ones (fftw_bench.c:118-124)."""
    import torch
    P, spec, shape = 4, "packed:block(16,2)|block(16,2)|local(16)", (16, 16, 16)
    r = Run(P, spec, shape, cuda)
    off = O.global_offsets(P, spec, r.dp, shape)
    host = np.zeros(P * r.dp, np.complex128)
    host[off[0, 0, 0]] = 1.0
    r.dat.copy_(torch.from_numpy(host))
    got = r.forward()
    _, mask = O.split_expected_output(P, spec, np.zeros(shape), r.wl)
    assert np.array_equal(got[mask], np.ones(mask.sum(), np.complex128))


@pytest.mark.parametrize("schedule", [api.SCHEDULE_LINES, api.SCHEDULE_SPLIT], ids=["lines", "split"])
def test_point_input_phase_ramp(schedule, cuda):
    """fftw_test.c:93-98's POINT input, a delta at (0, 0, 1): the forward transform is the analytic phase ramp
    exp(-2 pi i k2 / L2), placed in the B layout's slots (slot s holds frequency s / A + B * (s % A))."""
    import torch
    P, spec, shape = 4, "packed:block(16,2)|block(12,2)|local(20)", (16, 12, 20)
    r = Run(P, spec, shape, cuda, schedule=schedule)
    off = O.global_offsets(P, spec, r.dp, shape)
    host = np.zeros(P * r.dp, np.complex128)
    host[off[0, 0, 1]] = 1.0
    r.dat.copy_(torch.from_numpy(host))
    got = r.forward()
    A, B, _, _, a_spec, b_spec = O.split_factors(P, spec)
    out_spec = a_spec if all(a == 1 for a in A) else b_spec
    s2 = np.arange(shape[2])
    k2 = s2 // A[2] + B[2] * (s2 % A[2])
    ramp = np.broadcast_to(np.exp(-2j * np.pi * k2 / shape[2]), shape)
    want = np.zeros(P * r.wl, np.complex128)
    want[O.global_offsets(P, out_spec, r.wl, shape).ravel()] = ramp.ravel()
    _, mask = O.split_expected_output(P, spec, np.zeros(shape), r.wl)
    assert np.max(np.abs(got[mask] - want[mask])) < 1e-13


def test_linear_index_pattern_roundtrip(cuda):
    """split_plan_test.c's pattern value = i + L*(j + L*k), forward then backward, scaled by 1/N^3."""
    import torch
    P, L = 4, 32
    spec = "packed:block(%d,2)|block(%d,2)|local(%d)" % (L, L, L)
    r = Run(P, spec, (L, L, L), cuda)
    glob = np.arange(L ** 3, dtype=np.float64).reshape(L, L, L) + 0j
    r.dat.copy_(torch.from_numpy(O.scatter_global(P, spec, glob, r.dp)))
    r.forward()
    back = r.inverse()
    g = O.gather_global(P, spec, back, r.dp, (L, L, L)) / L ** 3
    assert np.max(np.abs(g - glob)) < 1e-9


@pytest.mark.parametrize("schedule", [api.SCHEDULE_LINES, api.SCHEDULE_SPLIT], ids=["lines", "split"])
@pytest.mark.parametrize("P,spec,shape,mode,B", [CASES[0], CASES[2], CASES[4], CASES[6], CASES[8], CASES[10]],
                         ids=["64c", "48c", "14x21x11", "allA1", "1d", "frev128"])
def test_forward_and_inverse_native_fp64(P, spec, shape, mode, B, schedule, cuda):
    """The same transforms in native FP64 arithmetic (DMG_ARITH_FP64)."""
    r = Run(P, spec, shape, cuda, mode, B, arith=api.ARITH_FP64, schedule=schedule)
    assert r.plan.arith == api.ARITH_FP64
    got = r.forward()
    exp, mask = O.split_expected_output(P, spec, r.glob, r.wl, mode, B)
    assert _rel(got[mask], exp[mask]) < TOL_C128
    back = r.inverse()
    g = O.gather_global(P, spec, back, r.dp, r.shape) / np.prod(r.shape)
    assert _rel(g, r.glob) < TOL_C128


@pytest.mark.parametrize("scale", [1e300, 1e-300, 2.0 ** 600, 3e-310])
def test_double_float_extreme_magnitudes(scale, cuda):
    """Double-float runs scale by a power of two, so FP64 magnitudes beyond FP32's range keep their accuracy."""
    P, spec, shape = 4, "packed:block(16,2)|block(24,2)|local(10)", (16, 24, 10)
    r = Run(P, spec, shape, cuda, scale=scale)
    assert r.plan.arith == api.ARITH_DF
    got = r.forward()
    exp, mask = O.split_expected_output(P, spec, r.glob, r.wl)
    if scale < 1e-307:  # denormal inputs: accuracy relative to the largest value
        assert np.max(np.abs(got[mask] - exp[mask])) <= 1e-12 * np.max(np.abs(exp[mask])) + 1e-320
        return
    assert np.all(np.isfinite(got[mask]))
    assert _rel(got[mask], exp[mask]) < TOL_C128
    back = r.inverse()
    g = O.gather_global(P, spec, back, r.dp, r.shape) / np.prod(r.shape)
    assert _rel(g, r.glob) < TOL_C128


def test_double_float_zero_input(cuda):
    import torch
    P, spec, shape = 4, "packed:block(8,2)|block(8,2)|local(8)", (8, 8, 8)
    r = Run(P, spec, shape, cuda)
    r.dat.zero_()
    got = r.forward()
    assert not np.any(got)
    assert r.plan.arith == api.ARITH_DF
    del torch


@pytest.mark.parametrize("dtype", [api.C128, api.C64], ids=["c128", "c64"])
def test_long_dimension_schedules(dtype, cuda):
    """2048-point dimensions: auto picks the split schedule for complex128 and lines for complex64; both
    schedules give the same slots."""
    P, spec, shape = 4, "packed:block(2048,2)|block(24,2)", (2048, 24)
    tol = TOL_C128 if dtype == api.C128 else TOL_C64
    r = Run(P, spec, shape, cuda, dtype=dtype)
    assert r.plan.schedule == (api.SCHEDULE_SPLIT if dtype == api.C128 else api.SCHEDULE_LINES)
    for sched in (api.SCHEDULE_LINES, api.SCHEDULE_SPLIT):
        r.plan.set_schedule(sched)
        got = r.forward().astype(np.complex128)
        exp, mask = O.split_expected_output(P, spec, r.glob, r.wl)
        assert _rel(got[mask], exp[mask]) < tol
        back = r.inverse().astype(np.complex128)
        g = O.gather_global(P, spec, back, r.dp, r.shape) / np.prod(r.shape)
        assert _rel(g, r.glob) < tol
        r.dat /= float(np.prod(r.shape))  # the unnormalised inverse left N times the input


def test_schedule_rejects_too_long_lines(cuda):
    """A dimension longer than a tile cannot run as one line pass."""
    import torch
    P, spec = 4, "packed:block(4096,2)|block(8,2)"
    comm = api.Comm(P)
    S = api.decomp_from_spec(comm, spec)
    work = torch.zeros(P * 4 * S.extent(), dtype=torch.complex128, device=cuda)
    dat = torch.zeros(P * S.extent(), dtype=torch.complex128, device=cuda)
    plan = api.SplitPlan(S, dat.data_ptr(), 4 * S.extent(), work.data_ptr())
    assert plan.schedule == api.SCHEDULE_SPLIT
    with pytest.raises(RuntimeError):
        plan.set_schedule(api.SCHEDULE_LINES)
    assert plan.schedule == api.SCHEDULE_SPLIT


@pytest.mark.parametrize("dtype", [api.C128, api.C64], ids=["c128", "c64"])
def test_cuda_graph_replay_matches_eager(dtype, cuda):
    """A forward + inverse captured into a CUDA graph (after a first run has put the plan's tables on the
    device) replays to the same bits as the eager runs."""
    import torch
    r = Run(16, "packed:block(48,4)|rotate(5,block(48,4))|local(64)", (48, 48, 64), cuda, dtype=dtype,
            schedule=api.SCHEDULE_LINES)
    start = r.dat.clone()
    want_fwd = r.forward()
    want_back = r.inverse()
    r.dat.copy_(start)
    r.work.zero_()
    torch.cuda.synchronize()
    cap = torch.cuda.Stream(cuda)
    cap.wait_stream(torch.cuda.current_stream(cuda))
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=cap):
        hs = torch.cuda.current_stream(cuda).cuda_stream
        r.plan.run(api.FFTW_FORWARD, hs)
    g2 = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g2, stream=cap):
        hs = torch.cuda.current_stream(cuda).cuda_stream
        r.plan.run(api.FFTW_BACKWARD, hs)
    for _ in range(2):
        r.dat.copy_(start)
        g.replay()
        torch.cuda.synchronize()
        assert np.array_equal(r.work.cpu().numpy(), want_fwd)
        g2.replay()
        torch.cuda.synchronize()
        assert np.array_equal(r.dat.cpu().numpy(), want_back)


def test_autotune_small_cube(cuda):
    """autotuneParallelPlan (reference split_fft.c:78-247) on an 8x12x16 complex128 cube over a 2x2 grid:
    it returns one of the makeParallelPlan plans in one of the two pass schedules, with a tile size and radix
    schedule of its choice; its forward transform is the oracle's spectrum in that plan's slots, and has the
    same bits as makeParallelPlan with its factors, schedule, tile and radix schedule.  A second call with the
    same start decomposition builds the cached choice without timing."""
    import torch
    P, spec, shape = 4, "packed:local(8)|block(12,2)|block(16,2)", (8, 12, 16)
    comm = api.Comm(P)
    S = api.decomp_from_spec(comm, spec)
    dp, wl = S.extent(), 2 * int(np.prod(shape))
    rng = np.random.default_rng(11)
    glob = rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)
    host = O.scatter_global(P, spec, glob, dp)
    dat = torch.from_numpy(host).to(cuda)
    work = torch.zeros(P * wl, dtype=torch.complex128, device=cuda)
    stream = torch.cuda.current_stream(cuda).cuda_stream
    api.autotune_cache_clear()
    sp = api.SplitPlan(S, dat.data_ptr(), wl, work.data_ptr(), autotune=True)
    assert api.autotune_last_timed() > 20 and api.autotune_cache_entries() == 1
    B = [L // a for L, a in zip(shape, sp.A_factors)]
    dat.copy_(torch.from_numpy(host))  # the search ran forward transforms over the buffers
    sp.run(api.FFTW_FORWARD, stream)
    torch.cuda.synchronize()
    got = work.cpu().numpy()
    exp, mask = O.split_expected_output(P, spec, glob, wl, 2, B)
    assert _rel(got[mask], exp[mask]) < TOL_C128
    work2 = torch.zeros_like(work)
    ref = api.SplitPlan(S, dat.data_ptr(), wl, work2.data_ptr(), B=B, schedule=sp.schedule)
    ref.set_tile(sp.tile)
    ref.set_radix(sp.radix)
    ref.run(api.FFTW_FORWARD, stream)
    torch.cuda.synchronize()
    assert np.array_equal(work2.cpu().numpy()[mask], got[mask])
    # the cached choice
    again = api.SplitPlan(S, dat.data_ptr(), wl, work2.data_ptr(), autotune=True)
    assert api.autotune_last_timed() == 0
    assert (again.A_factors, again.schedule, again.tile, again.radix) == (sp.A_factors, sp.schedule, sp.tile, sp.radix)


@pytest.mark.parametrize("dtype", [api.C128, api.C64], ids=["c128", "c64"])
def test_autotune_complex64_and_full_grid(dtype, cuda):
    """The typed autotuner with the full grid search (every grid of A and B, as the reference walks them) on
    a 2D array: the chosen plan's forward transform matches the oracle in the plan's own output slots."""
    import torch
    P, spec, shape = 4, "packed:block(8,2)|block(12,2)", (8, 12)
    r = Run(P, spec, shape, cuda, dtype=dtype, seed=4)
    tdt = torch.complex128 if dtype == api.C128 else torch.complex64
    work = torch.zeros(P * r.wl, dtype=tdt, device=cuda)
    sp = api.SplitPlan(r.S, r.dat.data_ptr(), r.wl, work.data_ptr(), autotune=True, dtype=dtype, full_grid=True)
    assert api.autotune_last_timed() > 20
    host = O.scatter_global(P, spec, r.glob, r.dp).astype(r.npdt)
    r.dat.copy_(torch.from_numpy(host))
    sp.run(api.FFTW_FORWARD, r.stream)
    torch.cuda.synchronize()
    got = work.cpu().numpy().astype(np.complex128)
    # the chosen plan's B layout (its own grids) holds frequency k1 + B k2 in slot k2 + A k1 of each dimension
    Bd = sp.decomp_B() or sp.decomp_A()
    off = np.array([Bd.global_offset(c, r.wl) for c in np.ndindex(*shape)]).reshape(shape)
    A = sp.A_factors
    k = [np.arange(L) // a + (L // a) * (np.arange(L) % a) for L, a in zip(shape, A)]
    want = O.fftn64(r.glob)[np.ix_(*k)]
    tol = TOL_C128 if dtype == api.C128 else TOL_C64
    assert _rel(got[off], want) < tol


@pytest.mark.parametrize("tile,radix", [(1024, api.RADIX_FIXED), (512, api.RADIX_FIXED), (0, api.RADIX_PLAN8),
                                        (0, api.RADIX_PLAN4), (256, api.RADIX_PLAN4)])
@pytest.mark.parametrize("dtype", [api.C128, api.C64], ids=["c128", "c64"])
def test_tile_and_radix_choices(tile, radix, dtype, cuda):
    """Every tile size and radix schedule the autotuner may choose gives the oracle's forward spectrum and
    the exact inverse."""
    P, spec, shape = 16, "packed:block(48,4)|rotate(5,block(64,4))|local(32)", (48, 64, 32)
    r = Run(P, spec, shape, cuda, dtype=dtype, seed=6)
    r.plan.set_tile(tile)
    r.plan.set_radix(radix)
    assert r.plan.radix == radix
    got = r.forward()
    exp, mask = O.split_expected_output(P, spec, r.glob, r.wl)
    tol = TOL_C128 if dtype == api.C128 else TOL_C64
    assert _rel(got[mask].astype(np.complex128), exp[mask]) < tol
    back = r.inverse()
    g = O.gather_global(P, spec, back.astype(np.complex128), r.dp, r.shape) / np.prod(r.shape)
    assert _rel(g, r.glob) < tol


@pytest.mark.parametrize("schedule", [api.SCHEDULE_LINES, api.SCHEDULE_SPLIT], ids=["lines", "split"])
@pytest.mark.parametrize("P,spec,shape", [
    (16, "packed:block(48,4)|rotate(5,block(64,4))|local(32)", (48, 64, 32)),
    (16, "packed:block(64,4)|block(16,4)|local(1024)", (64, 16, 1024)),
    (64, "packed:frev(16,8,block(128,8))|rotate(3,block(64,8))|local(32)", (128, 64, 32)),
])
@pytest.mark.parametrize("dtype", [api.C128, api.C64], ids=["c128", "c64"])
def test_wide_tiles(dtype, P, spec, shape, schedule, cuda):
    """Tiles of twice the default values (the 512-thread wide kernels for the power-of-two lengths; the others
    keep the default) give the oracle's spectrum and the exact inverse; complex64 also in the tensor-core form,
    whose 1024-point passes keep four-line tiles."""
    ariths = [None] if dtype == api.C128 else [api.ARITH_FP32, api.ARITH_TC16]
    for ar in ariths:
        r = Run(P, spec, shape, cuda, dtype=dtype, seed=8, arith=ar, schedule=schedule)
        r.plan.set_tile(8192 if dtype == api.C64 else 4096)
        got = r.forward()
        exp, mask = O.split_expected_output(P, spec, r.glob, r.wl)
        tol = TOL_C128 if dtype == api.C128 else TOL_C64
        assert _rel(got[mask].astype(np.complex128), exp[mask]) < tol, ar
        back = r.inverse()
        g = O.gather_global(P, spec, back.astype(np.complex128), r.dp, r.shape) / np.prod(r.shape)
        assert _rel(g, r.glob) < tol, ar
    if dtype == api.C128:
        with pytest.raises(Exception):
            r.plan.set_tile(8192)
