"""Host-side descriptor and planner logic against the oracle (no GPU needed)."""
import numpy as np
import pytest

from decomp_mpi_gb300 import api
from decomp_mpi_gb300._lib import load
from oracle import oracle as O
from tests.golden_cases import reshape_case, reshape_names

SPECS = [
    (4, "axes:single(10,0,1)@1,1|single(10,0,4)@10,1"),
    (4, "axes:rotate(2,local(10))@1,1|rotate(1,block(10,4))@10,1"),
    (4, "axes:rotate(3,block(10,2))@1,1|rotate(3,block(10,2))@5,2"),
    (4, "packed:local(8)|block(12,2)|block(16,2)"),
    (6, "packed:block(10,3)|block(7,2)|local(9)"),
    (6, "packed:rotate(3,block(10,2))|local(7)|block(9,3)"),
    (16, "packed:local(16)|rotate(5,block(12,4))|frev(4,5,block(20,4))"),
    (4, "packed:interleave(block(4,2),2)|local(12)|interleave(block(4,2),4)"),
    (64, "packed:interleave(block(16,4),32)|interleave(block(16,4),32)|interleave(block(16,4),32)"),
    (64, "packed:blockf(512,16,4)|blockf(512,16,4)|blockf(512,16,4)"),
    (16, "packed:interleave(block(10,3),12)|interleave(block(10,2),12)|interleave(block(10,2),12)"),
    (16, "packed:blockf(120,10,3)|blockf(120,10,2)|blockf(120,10,2)"),
    (5, "packed:block(11,5)|local(6)"),
]


def _shape(P, spec):
    c = api.Comm(P)
    d = api.decomp_from_spec(c, spec)
    return c, d


@pytest.mark.parametrize("P,spec", SPECS)
def test_extents_match_oracle(P, spec):
    c, d = _shape(P, spec)
    ext, pu = O.decomp_info(P, spec)
    assert d.proc_used == pu
    assert d.extent() == max(ext[:pu])
    for r in range(pu):
        assert d.rank_extent(r) == ext[r]


@pytest.mark.parametrize("P,spec", SPECS)
def test_global_offsets_match_oracle(P, spec):
    c, d = _shape(P, spec)
    pitch = d.extent()
    import itertools
    from decomp_mpi_gb300.api import _SpecParser  # noqa: F401  (spec grammar shared by tests)
    lens = []
    s = spec.split(":", 1)[1]
    # global sizes via the oracle, offsets via the product
    ext, pu = O.decomp_info(P, spec)
    nd = s.count("|") + 1
    # find the global sizes by probing the oracle's offsets with the product's decomp sizes
    lib = load()
    sizes = []
    import ctypes

    class AD(ctypes.Structure):
        _fields_ = [("decomp", ctypes.c_void_p)]

    class DS(ctypes.Structure):
        _fields_ = [("ndim", ctypes.c_int), ("comm", ctypes.c_void_p), ("proc_used", ctypes.c_int),
                    ("dims", ctypes.POINTER(ctypes.c_void_p))]
    ds = DS.from_address(d.h)
    for i in range(nd):
        ax = AD.from_address(ds.dims[i])
        sizes.append(lib.sizeDimDecomp(ax.decomp))
    want = O.global_offsets(P, spec, pitch, tuple(sizes))
    total = int(np.prod(sizes))
    if total <= 4096:
        coords = list(itertools.product(*[range(n) for n in sizes]))
    else:  # a seeded sample of coordinates for the large decompositions
        rng = np.random.default_rng(total)
        coords = [tuple(int(rng.integers(0, n)) for n in sizes) for _ in range(3000)]
    for idx in coords:
        assert d.global_offset(idx, pitch) == want[idx], (idx,)


@pytest.mark.parametrize("name", reshape_names())
def test_golden_cases_plan(name):
    m, *_ = reshape_case(name)
    c = api.Comm(m["P"])
    s = api.decomp_from_spec(c, m["src_spec"])
    d = api.decomp_from_spec(c, m["dst_spec"])
    pl = api.ReshapePlan(c, m["esize"], s, d)
    assert pl.src_pitch == m["src_pitch"] and pl.dest_pitch == m["dst_pitch"]
    assert pl.check_bounds(m["esize"], m["src_pitch"], m["dst_pitch"]) == 0
    assert pl.check_bounds(m["esize"], m["src_pitch"] - 1, m["dst_pitch"]) != 0
    assert pl.launches == 1
    assert pl.bytes_moved == 2 * pl.elements * m["esize"]


def test_incompatible_sizes_rejected():
    c = api.Comm(4)
    s = api.decomp_from_spec(c, "packed:block(8,2)|block(8,2)")
    d = api.decomp_from_spec(c, "packed:block(8,2)|block(9,2)")
    with pytest.raises(api.DecompError):
        api.ReshapePlan(c, 8, s, d)


def test_illegal_rank_stride_rejected():
    c = api.Comm(4)
    with pytest.raises(api.DecompError):
        api.decomp_from_spec(c, "axes:block(8,4)@1,2|local(8)@8,1")


def test_rank_out_of_range_rejected():
    c = api.Comm(3)
    with pytest.raises(api.DecompError):
        api.decomp_from_spec(c, "packed:block(8,2)|block(8,2)")


def test_replicated_ranks_rejected():
    """rank strides (1,4) with 2x2 positions over 8 ranks: rank 2 would hold a copy of rank 0."""
    c = api.Comm(8)
    s = api.decomp_from_spec(c, "axes:block(8,2)@1,1|block(8,2)@8,4")
    d = api.decomp_from_spec(c, "packed:block(8,2)|local(8)")
    with pytest.raises(api.DecompError):
        api.ReshapePlan(c, 8, s, d)
    assert load().dmg_last_error_code() == 2


def test_pitch_override():
    c = api.Comm(4)
    s = api.decomp_from_spec(c, "packed:block(8,2)|block(8,2)")
    d = api.decomp_from_spec(c, "packed:local(8)|block(8,4)")
    pl = api.ReshapePlan(c, 8, s, d)
    with pytest.raises(api.DecompError):
        pl.set_pitch(src_pitch=pl.src_pitch - 1)
    pl.set_pitch(src_pitch=100, dest_pitch=64)
    assert (pl.src_pitch, pl.dest_pitch) == (100, 64)


def test_view_rank_fields():
    """The reference fields of a descriptor describe the communicator's view rank."""
    lib = load()
    c = api.Comm(4)
    c.set_view_rank(3)
    d = api.decomp_from_spec(c, "packed:block(8,2)|block(8,2)")
    assert lib.myRank(d.h) == 3
    for pos in [(0, 0), (7, 7), (4, 3)]:
        assert d.owner(pos) == (pos[0] // 4) * 2 + pos[1] // 4


VISIT_SPECS = [
    (4, "axes:rotate(3,block(10,2))@1,1|rotate(3,block(10,2))@5,2"),
    (4, "packed:local(8)|block(12,2)|block(16,2)"),
    (6, "packed:block(10,3)|block(7,2)|local(9)"),
    (4, "packed:interleave(block(4,2),2)|local(12)|interleave(block(4,2),4)"),
    (5, "packed:block(11,5)|local(6)"),
]


@pytest.mark.parametrize("P,spec", VISIT_SPECS)
def test_visit_data_slots_and_positions(P, spec):
    """visitData (reference split_fft.c:862-889) calls the visitor once per slot 0..max_local of the
    buffer of the rank the descriptor describes; here the position is the slot's global coordinate (-1
    entries where the slot holds nothing), which must match the oracle's offsets on every rank."""
    import ctypes
    c, d = _shape(P, spec)
    lib = load()

    class AD(ctypes.Structure):
        _fields_ = [("decomp", ctypes.c_void_p)]

    class DS(ctypes.Structure):
        _fields_ = [("ndim", ctypes.c_int), ("comm", ctypes.c_void_p), ("proc_used", ctypes.c_int),
                    ("dims", ctypes.POINTER(ctypes.c_void_p))]
    ds = DS.from_address(d.h)
    sizes = tuple(lib.sizeDimDecomp(AD.from_address(ds.dims[i]).decomp) for i in range(ds.ndim))
    pitch = d.extent()
    off = O.global_offsets(P, spec, pitch, sizes)
    VIS = ctypes.CFUNCTYPE(None, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double))
    lib.visitData.restype, lib.visitData.argtypes = None, [ctypes.c_void_p, VIS, ctypes.POINTER(ctypes.c_double)]
    for r in range(P):
        # like an MPI rank, the view rank makes its own descriptor, whose fields describe it
        c.set_view_rank(r)
        d = api.decomp_from_spec(c, spec)
        buf = (ctypes.c_double * (2 * pitch))()
        seen = {}

        def visit(nd, pos, dat):
            slot = (ctypes.addressof(dat.contents) - ctypes.addressof(buf)) // 16
            assert 0 <= slot < pitch
            seen.setdefault(slot, []).append(tuple(pos[i] for i in range(nd)))

        cb = VIS(visit)
        lib.visitData(d.h, cb, buf)
        held = {int(o % pitch): g for g, o in np.ndenumerate(off) if o >= 0 and o // pitch == r}
        got = {s: p[0] for s, p in seen.items() if -1 not in p[0]}
        assert got == held
        assert all(len(p) == 1 for p in seen.values())


@pytest.mark.parametrize("A,B", [(3, 4), (4, 3), (2, 6), (12, 1)])
def test_factor_reverse_axis_decomp(A, B):
    """makeFactorReverseAxisDecomp (reference factor_reverse_decomp.c:56-58): the axis of
    factor_reverse(A, B, nested) keeps the original axis's memory and rank strides."""
    import ctypes
    lib = load()
    P = 4
    c = api.Comm(P)
    ax0 = lib.makeAxisDecomp(c.h, lib.makeBlockDecomp(12, 2), 1, 1)
    fr = lib.makeFactorReverseAxisDecomp(A, B, ax0)
    ax1 = lib.makeAxisDecomp(c.h, lib.makeBlockDecomp(8, 2), 6, 2)
    D = api.Decomp(c, lib.makeDecomp(2, (ctypes.c_void_p * 2)(fr, ax1)))
    lib.freeAxisDecomp(ax0)
    spec = "axes:frev(%d,%d,block(12,2))@1,1|block(8,2)@6,2" % (A, B)
    pitch = O.pitch_of(P, spec)
    assert D.extent() == pitch
    want = O.global_offsets(P, spec, pitch, (12, 8))
    for g in np.ndindex(12, 8):
        assert D.global_offset(list(g), pitch) == want[g]


def _bench_module():
    import importlib.util
    import os
    spec = importlib.util.spec_from_file_location(
        "bench_specs", os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "bench.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


@pytest.mark.parametrize("es", [16, 8, 4, 1])
def test_measured_reshapes_plan_direct_16_byte_moves(es):
    """The reshapes that are measured (the 512^3 chain on 8x8 and the sweep's transitions) plan onto
    separable address tables with 16-byte moves (elements narrower than 16 bytes fused along the
    contiguous axis): the kernel form that runs near the HBM copy rate."""
    bench = _bench_module()
    c = api.Comm(64)
    D = [api.decomp_from_spec(c, s) for s in bench.specs(512)]
    plans = [api.ReshapePlan(c, es, D[0], D[1]), api.ReshapePlan(c, es, D[1], D[2])]
    for shape, g in [((256, 256, 256), 16), ((1024, 1024, 512), 32)]:
        cg = api.Comm(g * g)
        blk, other = bench.sweep_specs(shape, g)
        S = api.decomp_from_spec(cg, blk)
        for spec in other.values():
            O_ = api.decomp_from_spec(cg, spec)
            plans += [api.ReshapePlan(cg, es, S, O_), api.ReshapePlan(cg, es, O_, S)]
    for p in plans:
        d = p.describe()
        assert d.startswith("src=separable dst=separable unit=%dB fuse=%d " % (es, 16 // es)), d
