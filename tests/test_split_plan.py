"""Split-FFT planning on the host against the oracle and the reference's fixtures (no GPU)."""
import numpy as np
import pytest

from decomp_mpi_gb300 import api
from oracle import oracle as O
from tests.golden_cases import meta, split_case, split_names

PLAN_CASES = [
    (4, "packed:local(8)|block(12,2)|block(16,2)", 0, None),
    (4, "packed:block(16,2)|block(16,2)|local(16)", 0, None),
    (6, "packed:block(12,3)|block(10,2)|local(6)", 0, None),
    (4, "packed:local(8)|block(12,2)|block(16,2)", 1, None),
    (4, "packed:local(8)|block(12,2)|block(16,2)", 2, [1, 12, 16]),
    (64, "packed:block(512,8)|block(512,8)|local(512)", 0, None),
    (16, "packed:block(120,4)|block(120,4)|local(120)", 0, None),
    (16, "packed:block(48,4)|rotate(5,block(48,4))|local(48)", 0, None),
    (4, "packed:block(64,2)|block(64,2)|local(64)", 0, None),
    (8, "packed:block(14,2)|block(21,4)|local(11)", 0, None),
    (4, "packed:block(30,4)", 0, None),
    (4, "packed:block(12,2)|block(18,2)", 0, None),
]


def _work_len(shape):
    return 2 * int(np.prod(shape))


def _shape(P, spec):
    c = api.Comm(P)
    return c, api.decomp_from_spec(c, spec)


@pytest.mark.parametrize("P,spec,mode,B", PLAN_CASES)
def test_factors_grids_and_layout_match_oracle(P, spec, mode, B):
    c, S = _shape(P, spec)
    lib = S.lib
    sizes = []
    import ctypes

    class DS(ctypes.Structure):
        _fields_ = [("ndim", ctypes.c_int), ("comm", ctypes.c_void_p), ("proc_used", ctypes.c_int),
                    ("dims", ctypes.POINTER(ctypes.c_void_p))]

    class AD(ctypes.Structure):
        _fields_ = [("decomp", ctypes.c_void_p)]
    ds = DS.from_address(S.h)
    for i in range(ds.ndim):
        sizes.append(lib.sizeDimDecomp(AD.from_address(ds.dims[i]).decomp))
    wl = _work_len(sizes)
    sp = api.SplitPlan(S, 0x100000, wl, 0x200000, slab=mode if mode < 2 else 0, B=B if mode == 2 else None)
    A, Bf, ga, gb, a_spec, b_spec = O.split_factors(P, spec, mode, B)
    assert sp.A_factors == A
    use_first = all(a == 1 for a in A)
    out_spec = a_spec if use_first else b_spec
    out_dec = sp.decomp_A() if use_first else sp.decomp_B()
    want = O.global_offsets(P, out_spec, wl, tuple(sizes)).ravel()
    rng = np.random.default_rng(0)
    total = int(np.prod(sizes))
    idx = range(total) if total <= 4096 else rng.integers(0, total, 2000)
    for g in idx:
        coord = np.unravel_index(int(g), sizes)
        assert out_dec.global_offset([int(x) for x in coord], wl) == want[g]


@pytest.mark.parametrize("name", split_names())
def test_extent_matches_reference(name):
    m, z = split_case(name)
    c, S = _shape(m["P"], m["spec"])
    sp = api.SplitPlan(S, 0x100000, m["work_len"], 0x200000, slab=m["mode"] if m["mode"] < 2 else 0,
                       B=m["B"] if m["mode"] == 2 else None)
    assert sp.extent == int(z["info"][:, 0].max())
    assert sp.A_factors == [int(a) for a in z["info"][0, 1:1 + len(m["shape"])]]


def test_processor_grid_matches_reference():
    for case in meta()["grid"]:
        c = api.Comm(case["P"])
        assert api.processor_grid(c, case["tasks"]) == case["grid"], case


def test_workspace_too_small_rejected():
    c, S = _shape(4, "packed:block(16,2)|block(16,2)|local(16)")
    with pytest.raises(api.DecompError):
        api.SplitPlan(S, 0x1000, 2 * 1024 - 1, 0x2000)  # needs 2 * extent = 2048


def test_invalid_factor_rejected():
    c, S = _shape(4, "packed:block(16,2)|block(16,2)|local(16)")
    with pytest.raises(api.DecompError):
        api.SplitPlan(S, 0x1000, 4096, 0x2000, B=[3, 4, 4])


def test_reference_descriptor_and_exact_descriptor():
    """getTransformed is the reference's factor_reverse(A,B) over B; it agrees with the exact
    descriptor when A == B and differs otherwise (the reference's defect)."""
    for spec, same in [("packed:block(16,2)|block(16,2)|local(16)", True),
                       ("packed:local(8)|block(12,2)|block(16,2)", False)]:
        c, S = _shape(4, spec)
        sp = api.SplitPlan(S, 0x1000, 8192, 0x2000)
        ref = sp.transformed()
        ex = sp.transformed_exact()
        sizes = [16, 16, 16] if same else [8, 12, 16]
        diff = 0
        for g in range(int(np.prod(sizes))):
            coord = [int(x) for x in np.unravel_index(g, sizes)]
            diff += ref.global_offset(coord, 8192) != ex.global_offset(coord, 8192)
        assert (diff == 0) == same


def test_gcd():
    lib = api.load()
    for u, v in [(0, 5), (5, 0), (12, 18), (17, 5), (1 << 20, 3 << 10)]:
        assert lib.gcd(u, v) == np.gcd(u, v)


def _plan_offsets(dec, shape, wl):
    import itertools
    return [dec.global_offset(list(x), wl) for x in itertools.product(*[range(n) for n in shape])]


def test_propose_parallel_plan_is_make_parallel_plan():
    """proposeParallelPlan with no flags (split_fft.c:747-787) is the plan makeParallelPlan builds: the same
    factors and the same A and B layouts."""
    P, spec, shape, B = 4, "packed:local(8)|block(12,2)|block(16,2)", (8, 12, 16), [2, 3, 4]
    c, S = _shape(P, spec)
    wl = _work_len(shape)
    sp = api.propose_parallel_plan(api.NO_FLAGS, S, B, 0x100000, wl, 0x200000)
    ref = api.SplitPlan(S, 0x100000, wl, 0x200000, B=B)
    assert sp.A_factors == ref.A_factors == [4, 4, 4]
    assert _plan_offsets(sp.decomp_A(), shape, wl) == _plan_offsets(ref.decomp_A(), shape, wl)
    assert _plan_offsets(sp.decomp_B(), shape, wl) == _plan_offsets(ref.decomp_B(), shape, wl)


def test_propose_parallel_plan_declines_and_rejects():
    """Every B_i = 1 is declined (NULL, no error) under PREFER_STAGE1 and planned without it; a factor
    that does not divide its length is an error (the reference aborts, split_fft.c:761-763)."""
    P, spec, shape = 4, "packed:local(8)|block(12,2)|block(16,2)", (8, 12, 16)
    c, S = _shape(P, spec)
    wl = _work_len(shape)
    assert api.propose_parallel_plan(api.PREFER_STAGE1, S, [1, 1, 1], 0x100000, wl, 0x200000) is None
    sp = api.propose_parallel_plan(api.NO_FLAGS, S, [1, 1, 1], 0x100000, wl, 0x200000)
    assert sp.A_factors == [8, 12, 16]
    with pytest.raises(api.DecompError):
        api.propose_parallel_plan(api.NO_FLAGS, S, [3, 3, 4], 0x100000, wl, 0x200000)


def test_build_parallel_plan_explicit_grids():
    """buildParallelPlan with explicit processor grids: A's owner depends only on the dimensions its grid
    splits (grid (1, 2, 2): not on x0), B's likewise (grid (2, 2, 1): not on x2), over all four ranks."""
    import itertools
    P, spec, shape = 4, "packed:local(8)|block(12,2)|block(16,2)", (8, 12, 16)
    c, S = _shape(P, spec)
    wl = _work_len(shape)
    sp = api.build_parallel_plan(api.NO_FLAGS, 0, 0, S, [4, 4, 4], [2, 3, 4], list(shape), [1, 2, 2], [2, 2, 1],
                                 0x100000, wl, 0x200000)
    assert sp.A_factors == [4, 4, 4]
    A, B = sp.decomp_A(), sp.decomp_B()
    own_a, own_b = {}, {}
    for x in itertools.product(*[range(n) for n in shape]):
        own_a.setdefault(x[1:], set()).add(A.owner(list(x)))
        own_b.setdefault(x[:2], set()).add(B.owner(list(x)))
    assert all(len(v) == 1 for v in own_a.values()) and all(len(v) == 1 for v in own_b.values())
    assert set().union(*own_a.values()) == set().union(*own_b.values()) == {0, 1, 2, 3}


@pytest.mark.parametrize("dtype", [api.C128, api.C64], ids=["c128", "c64"])
def test_measured_split_plan_form(dtype):
    """The measured 512^3 transform on the 8x8 grid (factor_reverse start, workspace twice the extent)
    plans three one-pass-per-dimension passes of compile-time length 512 whose sides all take the
    separable walks (orders tab / atb / abt, no per-value layout evaluation)."""
    import re
    c = api.Comm(64)
    n = 512
    spec = "packed:frev(16,32,block(%d,8))|frev(32,16,block(%d,8))|local(%d)" % (n, n, n)
    S = api.decomp_from_spec(c, spec)
    probe = api.SplitPlan(S, 1 << 20, 1 << 40, 1 << 21, dtype=dtype)
    length = 2 * probe.extent
    probe.free()
    d = api.SplitPlan(S, 1 << 20, length, 1 << 21, dtype=dtype).describe()
    assert " lines passes=3:" in d, d
    passes = re.findall(r"\[d=(\d) n=(\d+) [^\]]* in=(\w+) out=(\w+)\]", d)
    assert [(p[0], p[1]) for p in passes] == [("2", "512"), ("1", "512"), ("0", "512")], d
    assert [(p[2], p[3]) for p in passes] == [("tab", "tab"), ("atb", "atb"), ("abt", "abt")], d
    assert "per value" not in d and "shared dim" not in d, d


def test_tile_choices_in_the_pass_list():
    """Host side of the tile choice: complex64 FP32 plans give the strided 1024-point passes wide tiles (eight
    lines) by default and the contiguous one four; the tensor-core form keeps four lines on its 1024-point
    passes; an explicit tile size applies to every pass; complex128 refuses twice its wide size."""
    import re
    comm = api.Comm(64)
    D = api.decomp_from_spec(comm, "packed:block(1024,8)|block(1024,8)|local(1024)")
    sp = api.SplitPlan(D, 1 << 20, 2 * 1024 ** 3 // 64 + 1024, 1 << 21, dtype=api.C64)

    def lines():
        return [int(x) for x in re.findall(r" x(\d+) v2", sp.describe())]

    assert sp.tile == 0 and lines() == [4, 8, 8]
    sp.set_arith(api.ARITH_TC16)
    assert lines() == [4, 4, 4]
    sp.set_arith(api.ARITH_FP32)
    sp.set_tile(2048)
    assert sp.tile == 2048 and lines() == [2, 2, 2]
    sp.set_tile(8192)
    assert lines() == [8, 8, 8]
    for bad in (32, 3000, 16384):
        with pytest.raises(Exception):
            sp.set_tile(bad)
    D2 = api.decomp_from_spec(comm, "packed:block(512,8)|block(512,8)|local(512)")
    sp2 = api.SplitPlan(D2, 1 << 20, 2 * 512 ** 3 // 64 + 1024, 1 << 21)
    sp2.set_tile(4096)
    with pytest.raises(Exception):
        sp2.set_tile(8192)
    sp2.set_radix(api.RADIX_PLAN4)
    assert sp2.radix == api.RADIX_PLAN4
    with pytest.raises(Exception):
        sp2.set_radix(7)


def test_native_fp64_tiles_and_paired_split_sides():
    """Native FP64 passes take tiles of at most 1024 values (two 512-point lines where double-float takes
    four, whatever tile the plan asks for); the split schedule's sides whose shared dimension is a sum of
    sub-axis parts walk as separable ("(paired)"), while a start decomposition with uneven blocks (per-rank
    strides) keeps the per-value walk."""
    import re
    comm = api.Comm(64)
    blk, rotd, frv = _bench_specs(512)
    D = api.decomp_from_spec(comm, frv)
    probe = api.SplitPlan(D, 1 << 20, 1 << 40, 1 << 21)
    length = 2 * probe.extent64
    sp = api.SplitPlan(D, 1 << 20, length, 1 << 21)

    def lines():
        return [int(x) for x in re.findall(r" x(\d+) v2", sp.describe())]

    assert lines() == [4, 4, 4]
    sp.set_arith(api.ARITH_FP64)
    assert lines() == [2, 2, 2]
    sp.set_tile(4096)
    assert lines() == [2, 2, 2]
    sp.set_tile(512)
    assert lines() == [1, 1, 1]
    sp.set_tile(0)
    sp.set_schedule(api.SCHEDULE_SPLIT)
    d = sp.describe()
    assert d.count("(paired)") == 12 and "shared dim" not in d, d
    # 4 x 3 ranks: 30 values in blocks of 8 (uneven), so the first pass reads the start layout per value
    comm2 = api.Comm(12)
    D2 = api.decomp_from_spec(comm2, "packed:block(30,4)|block(28,3)|local(12)")
    sp2 = api.SplitPlan(D2, 1 << 20, 1 << 20, 1 << 21, B=[3, 4, 2])
    sp2.set_schedule(api.SCHEDULE_SPLIT)
    d2 = sp2.describe()
    first = re.findall(r"\[t=\d[^\]]*\]", d2)[0]
    assert "in=atb(per value)" in first and "(paired)" in d2, d2


def _bench_specs(n):
    g0 = g1 = 8
    blk = "packed:block(%d,%d)|block(%d,%d)|local(%d)" % (n, g0, n, g1, n)
    rotd = "packed:rotate(1,block(%d,%d))|rotate(%d,block(%d,%d))|local(%d)" % (n, g0, n // 3, n, g1, n)
    frv = "packed:frev(16,%d,block(%d,%d))|frev(%d,16,block(%d,%d))|local(%d)" % (n // 16, n, g0, n // 16, n, g1, n)
    return blk, rotd, frv
