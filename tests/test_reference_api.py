"""The reference's smaller C entry points through the C-ABI, against the reference's semantics and the
oracle (no GPU): run-length index sets, the locality and offset queries of a descriptor's view rank,
the stage decompositions of the split FFT, DimDecomp cloning, the global-order decomposition and the
stream setting."""
import ctypes

import numpy as np
import pytest

from decomp_mpi_gb300 import api
from decomp_mpi_gb300._lib import load
from oracle import oracle as O


class _Index(ctypes.Structure):
    _fields_ = [("size", ctypes.c_int), ("count", ctypes.c_int), ("offsets", ctypes.POINTER(ctypes.c_int)),
                ("counts", ctypes.POINTER(ctypes.c_int))]


def _runs(h):
    ix = _Index.from_address(h)
    return [(ix.offsets[i], ix.counts[i]) for i in range(ix.count)]


def test_index_runs():
    """addIndex merges an offset that continues the last run and starts a new run otherwise; the arrays
    grow past their initial 16 entries (reference index.c:23-42)."""
    lib = load()
    h = lib.makeIndex()
    for o in [0, 1, 2, 5, 6, 9, 3]:
        lib.addIndex(h, o)
    assert _runs(h) == [(0, 3), (5, 2), (9, 1), (3, 1)]
    assert lib.sizeIndex(h) == 7
    lib.freeIndex(h)
    h = lib.makeIndex()
    for o in range(0, 80, 2):
        lib.addIndex(h, o)
    assert _runs(h) == [(o, 1) for o in range(0, 80, 2)]
    assert _Index.from_address(h).size >= 40
    lib.freeIndex(h)


LOCAL_SPECS = [
    (4, "packed:local(8)|block(12,2)|rotate(3,block(16,2))", (8, 12, 16)),
    (6, "packed:block(10,3)|frev(7,1,block(7,2))|local(9)", (10, 7, 9)),
    (4, "packed:interleave(block(4,2),2)|local(5)|interleave(block(4,2),3)", (8, 5, 12)),
]


@pytest.mark.parametrize("P,spec,shape", LOCAL_SPECS)
def test_locality_and_offsets_of_the_view_rank(P, spec, shape):
    """isCoordLocal / areCoordsLocal / getOffset / myRank (reference reshape.h:185-201) describe the rank
    that made the descriptor: a coordinate is local where the oracle puts it in that rank's buffer, at the
    oracle's offset inside the buffer."""
    lib = load()
    c = api.Comm(P)
    pitch = O.pitch_of(P, spec)
    off = O.global_offsets(P, spec, pitch, shape)
    for r in range(P):
        c.set_view_rank(r)
        d = api.decomp_from_spec(c, spec)
        assert lib.myRank(d.h) == r
        for g in np.ndindex(*shape):
            pos = (ctypes.c_int * len(shape))(*g)
            mine = bool(off[g] >= 0 and off[g] // pitch == r)
            assert bool(lib.areCoordsLocal(d.h, pos)) == mine
            if mine:
                assert lib.getOffset(d.h, pos) == off[g] % pitch
        # per dimension: a position is local when some held coordinate of the rank has it
        for dim, n in enumerate(shape):
            held = {g[dim] for g in np.ndindex(*shape) if off[g] >= 0 and off[g] // pitch == r}
            for x in range(n):
                assert bool(lib.isCoordLocal(d.h, dim, x)) == (x in held)


def _ints(v):
    return (ctypes.c_int * len(v))(*v)


@pytest.mark.parametrize("A,B,grid", [([4, 3, 2], [2, 4, 5], [2, 2, 1]), ([8, 1, 6], [1, 12, 2], [1, 2, 2])])
def test_stage_decompositions(A, B, grid):
    """makeInterleavedDecomp is interleave(block(A_i, grid_i), B_i) per dimension and makeBlockedDecomp is
    block of A_i B_i with factor A_i over grid_i, both packed (reference split_fft.c:36-77)."""
    lib = load()
    P = 4
    c = api.Comm(P)
    shape = tuple(a * b for a, b in zip(A, B))
    for maker, dims in [
        (lib.makeInterleavedDecomp, ["interleave(block(%d,%d),%d)" % (a, g, b) for a, b, g in zip(A, B, grid)]),
        (lib.makeBlockedDecomp, ["blockf(%d,%d,%d)" % (a * b, a, g) for a, b, g in zip(A, B, grid)]),
    ]:
        d = api.Decomp(c, maker(len(A), c.h, _ints(A), _ints(B), _ints(grid)))
        spec = "packed:" + "|".join(dims)
        pitch = O.pitch_of(P, spec)
        assert d.extent() == pitch
        want = O.global_offsets(P, spec, pitch, shape)
        for g in np.ndindex(*shape):
            assert d.global_offset(list(g), pitch) == want[g], (spec, g)


def test_clone_dim_decomp():
    """cloneDimDecomp copies a decorated DimDecomp: the clone lays out a decomposition identically and
    outlives the original."""
    lib = load()
    P = 4
    c = api.Comm(P)
    orig = lib.makeRotatedDecomp(5, lib.makeFactorReverseDecomp(4, 3, lib.makeBlockDecomp(12, 2)))
    clone = lib.cloneDimDecomp(orig)
    assert lib.sizeDimDecomp(clone) == lib.sizeDimDecomp(orig) == 12
    lib.freeDimDecomp(orig)
    d = api.Decomp(c, lib.makePackedDecomp(c.h, 2, (ctypes.c_void_p * 2)(clone, lib.makeBlockDecomp(8, 2))))
    spec = "packed:rotate(5,frev(4,3,block(12,2)))|block(8,2)"
    pitch = O.pitch_of(P, spec)
    want = O.global_offsets(P, spec, pitch, (12, 8))
    for g in np.ndindex(12, 8):
        assert d.global_offset(list(g), pitch) == want[g]


def test_global_decomp_is_c_order_on_rank_zero():
    """dmg_makeGlobalDecomp: every element on rank 0, at its C-order linear index."""
    lib = load()
    c = api.Comm(4)
    shape = (5, 3, 4)
    d = api.Decomp(c, lib.dmg_makeGlobalDecomp(c.h, 3, _ints(shape)))
    assert d.extent() == 60
    for i, g in enumerate(np.ndindex(*shape)):
        assert d.owner(list(g)) == 0
        assert d.global_offset(list(g), 60) == i


def test_stream_setting():
    """dmg_set_stream / dmg_get_stream: the stream the reference-signature runs enqueue on (no CUDA call)."""
    lib = load()
    before = lib.dmg_get_stream()
    try:
        lib.dmg_set_stream(ctypes.c_void_p(0x1234))
        assert lib.dmg_get_stream() == 0x1234
    finally:
        lib.dmg_set_stream(ctypes.c_void_p(before))
    assert lib.dmg_get_stream() == before


def test_error_printing_switch_is_per_thread():
    """dmg_set_error_printing returns the previous setting and applies to the calling thread only."""
    import threading
    lib = load()
    prev = lib.dmg_set_error_printing(0)
    try:
        seen = []
        t = threading.Thread(target=lambda: seen.append(lib.dmg_set_error_printing(1)))
        t.start()
        t.join()
        assert seen == [1]  # a new thread starts with printing on
        assert lib.dmg_set_error_printing(0) == 0  # this thread's setting was not touched by the other
    finally:
        lib.dmg_set_error_printing(prev)


@pytest.mark.parametrize("spec", ["packed:block(8,2", "packed:blok(8,2)", "cols:block(8,2)", "packed:block(8)",
                                  "packed:", "packed:block(8,2)|", "axes:block(8,2)",
                                  "packed:frev(3,3,block(8,2))", "packed:block(8,5)"])
def test_bad_decomposition_specs_are_rejected(spec):
    """Malformed spec strings and decompositions the constructors refuse (factors that do not multiply to
    the length, a grid larger than the communicator) raise instead of returning a descriptor."""
    c = api.Comm(4)
    lib = load()
    prev = lib.dmg_set_error_printing(0)
    try:
        with pytest.raises((ValueError, api.DecompError)):
            api.decomp_from_spec(c, spec)
    finally:
        lib.dmg_set_error_printing(prev)
