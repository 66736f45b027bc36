"""GPU reshape through the C-ABI against the golden fixtures and the oracle (bit-exact)."""
import numpy as np
import pytest

from decomp_mpi_gb300 import api
from oracle import oracle as O
from tests.golden_cases import reshape_case, reshape_names

pytestmark = pytest.mark.gpu


def _run_gpu(P, s_spec, d_spec, esize, src_bytes: np.ndarray, fill_bytes: np.ndarray, cuda, stream=None):
    import torch
    comm = api.Comm(P)
    S = api.decomp_from_spec(comm, s_spec)
    D = api.decomp_from_spec(comm, d_spec)
    plan = api.ReshapePlan(comm, esize, S, D)
    ds = torch.from_numpy(src_bytes.view(np.uint8).copy()).to(cuda)
    dd = torch.from_numpy(fill_bytes.view(np.uint8).copy()).to(cuda)
    s = stream if stream is not None else torch.cuda.current_stream(cuda)
    with torch.cuda.stream(s):
        plan.run(ds.data_ptr(), dd.data_ptr(), s.cuda_stream)
    s.synchronize()
    return dd.cpu().numpy(), plan


@pytest.mark.parametrize("name", reshape_names())
def test_golden(name, cuda):
    m, src, out, fill = reshape_case(name)
    got, _ = _run_gpu(m["P"], m["src_spec"], m["dst_spec"], m["esize"], src, fill, cuda)
    assert np.array_equal(got, out)


def _pencils(n, g0, g1):
    x = "packed:block(%d,%d)|block(%d,%d)|local(%d)" % (n, g0, n, g1, n)
    y = "packed:block(%d,%d)|local(%d)|block(%d,%d)" % (n, g0, n, n, g1)
    z = "packed:local(%d)|block(%d,%d)|block(%d,%d)" % (n, n, g0, n, g1)
    return x, y, z


X64, Y64, Z64 = _pencils(64, 2, 2)
CASES = [
    # config "plain method": 64^3 complex128 on a 2x2 grid, x -> y -> z pencils
    ("c1_x_to_y", 4, X64, Y64, "complex128"),
    ("c1_y_to_z", 4, Y64, Z64, "complex128"),
    ("c1_z_to_x", 4, Z64, X64, "complex128"),
    # the transitions of the bandwidth sweep at a small size on 4x4
    ("block_to_interleave", 16, "packed:block(32,4)|block(32,4)|local(32)",
     "packed:interleave(block(8,4),4)|interleave(block(8,4),4)|local(32)", "int64"),
    ("interleave_to_block", 16, "packed:interleave(block(8,4),4)|interleave(block(8,4),4)|local(32)",
     "packed:block(32,4)|block(32,4)|local(32)", "complex64"),
    ("block_to_rotate", 16, "packed:block(32,4)|block(32,4)|local(32)",
     "packed:rotate(3,block(32,4))|rotate(11,block(32,4))|local(32)", "int64"),
    ("rotate_to_block", 16, "packed:rotate(3,block(32,4))|rotate(11,block(32,4))|local(32)",
     "packed:block(32,4)|block(32,4)|local(32)", "complex64"),
    ("block_to_frev", 16, "packed:block(32,4)|block(32,4)|local(32)",
     "packed:frev(4,8,block(32,4))|frev(8,4,block(32,4))|local(32)", "int64"),
    ("frev_to_block", 16, "packed:frev(4,8,block(32,4))|frev(8,4,block(32,4))|local(32)",
     "packed:block(32,4)|block(32,4)|local(32)", "complex64"),
    ("frev_last_axis", 16, "packed:block(32,4)|block(32,4)|local(32)",
     "packed:block(32,4)|local(32)|frev(8,4,block(32,4))", "complex128"),
    # uneven blocks: ranked address tables on one or both sides
    ("uneven_both", 12, "packed:block(30,4)|block(14,3)|local(9)", "packed:local(30)|block(14,4)|block(9,3)",
     "complex128"),
    ("uneven_ranked_to_sep", 6, "packed:block(10,3)|block(7,2)|local(9)",
     "packed:local(10)|local(7)|block(9,6)", "int32"),
    # element sizes and dimensionalities
    ("int16_2d", 8, "packed:block(40,8)|local(24)", "packed:local(40)|block(24,8)", "int16"),
    ("bytes_1d", 3, "packed:block(100,3)", "packed:rotate(7,block(100,3))", "uint8"),
    ("struct48_3d", 4, "packed:block(8,2)|block(6,2)|local(5)", "packed:local(8)|local(6)|block(5,4)", "V48"),
    ("four_dims", 8, "packed:block(6,2)|block(4,2)|block(6,2)|local(10)",
     "packed:local(6)|rotate(1,block(4,4))|local(6)|block(10,2)", "complex64"),
    # explicit strides whose fast axes differ: the shared-memory transpose kernel
    ("transpose_2d", 4, "axes:block(64,2)@1,1|block(48,2)@32,2", "axes:block(64,2)@24,1|block(48,2)@1,2",
     "complex128"),
    ("transpose_3d_int64", 8, "axes:block(40,2)@1,1|block(36,2)@20,2|block(10,2)@360,4",
     "axes:local(40)@180,1|block(36,4)@1,2|block(10,2)@9,1", "int64"),
    ("transpose_uneven_ranked", 6, "packed:block(10,3)|block(7,2)|local(9)",
     "axes:local(10)@9,1|block(7,3)@1,1|block(9,2)@30,3", "float32"),
    ("transpose_int8", 4, "axes:block(33,2)@1,1|block(20,2)@17,2", "axes:block(33,2)@10,1|block(20,2)@1,2", "int8"),
    # explicit strides with padding, single-rank source (test.c pattern)
    ("single_source_3d", 4, "axes:single(12,0,1)@1,1|single(10,0,4)@12,1|local(6)@130,1",
     "axes:rotate(2,local(12))@1,1|rotate(1,block(10,4))@12,1|local(6)@40,1", "float64"),
]


@pytest.mark.parametrize("name,P,s,d,dt", CASES, ids=[c[0] for c in CASES])
def test_against_oracle(name, P, s, d, dt, cuda):
    dt = np.dtype(dt)
    sp, dp = O.pitch_of(P, s), O.pitch_of(P, d)
    rng = np.random.default_rng(5)
    src = np.frombuffer(rng.integers(0, 256, P * sp * dt.itemsize, dtype=np.uint8).tobytes(), dtype=dt)
    fill = np.frombuffer(np.full(P * dp * dt.itemsize, 0x5A, np.uint8).tobytes(), dtype=dt)
    want = fill.copy()
    O.reshape(P, s, d, src.copy(), sp, want, dp)
    got, plan = _run_gpu(P, s, d, dt.itemsize, src, fill, cuda)
    assert np.array_equal(got, want.view(np.uint8)), plan.describe()


def test_non_default_stream(cuda):
    import torch
    s = torch.cuda.Stream(cuda)
    dt = np.dtype("complex128")
    P, a, b = 4, X64, Y64
    sp, dp = O.pitch_of(P, a), O.pitch_of(P, b)
    rng = np.random.default_rng(1)
    src = rng.uniform(-1, 1, P * sp).astype(dt)
    want = np.zeros(P * dp, dt)
    O.reshape(P, a, b, src, sp, want, dp)
    got, _ = _run_gpu(P, a, b, 16, src, np.zeros(P * dp, dt), cuda, stream=s)
    assert np.array_equal(got, want.view(np.uint8))


def test_pitch_override_gpu(cuda):
    """Arrays with a larger per-rank pitch than the extent (split_plan_test.c allocates 2N/P per rank)."""
    import torch
    P, a, b = 4, X64, Z64
    comm = api.Comm(P)
    S, D = api.decomp_from_spec(comm, a), api.decomp_from_spec(comm, b)
    plan = api.ReshapePlan(comm, 16, S, D)
    sp, dp = plan.src_pitch + 100, plan.dest_pitch + 36
    plan.set_pitch(sp, dp)
    rng = np.random.default_rng(2)
    src = rng.uniform(-1, 1, P * sp) + 0j
    want = np.zeros(P * dp, np.complex128)
    O.reshape(P, a, b, src, sp, want, dp)
    ds = torch.from_numpy(src).to(cuda)
    dd = torch.zeros(P * dp, dtype=torch.complex128, device=cuda)
    plan.run(ds.data_ptr(), dd.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(dd.cpu().numpy(), want)


def _index_roundtrip(P, a, b, shape, torch_dtype, cuda):
    """Values = global linear index; forward must be a permutation onto the held slots and the
    reverse reshape must restore the source exactly (a size-independent property)."""
    import torch
    comm = api.Comm(P)
    S, D = api.decomp_from_spec(comm, a), api.decomp_from_spec(comm, b)
    esize = torch.empty(0, dtype=torch_dtype).element_size()
    fwd = api.ReshapePlan(comm, esize, S, D)
    bwd = api.ReshapePlan(comm, esize, D, S)
    N = int(np.prod(shape))
    off = torch.from_numpy(O.global_offsets(P, a, fwd.src_pitch, shape).ravel()).to(cuda)
    src = torch.full((P * fwd.src_pitch,), -1, dtype=torch.int64, device=cuda)
    src[off] = torch.arange(N, device=cuda)
    if torch_dtype == torch.complex64:
        src = src.to(torch.float32)
        src = torch.complex(src, -src)
    dst = torch.full((P * fwd.dest_pitch,), -7, dtype=src.dtype, device=cuda)
    st = torch.cuda.current_stream().cuda_stream
    fwd.run(src.data_ptr(), dst.data_ptr(), st)
    back = torch.full_like(src, -3)
    bwd.run(dst.data_ptr(), back.data_ptr(), st)
    torch.cuda.synchronize()
    assert torch.equal(back[off], src[off])
    doff = torch.from_numpy(O.global_offsets(P, b, fwd.dest_pitch, shape).ravel()).to(cuda)
    assert torch.equal(dst[doff], src[off])


@pytest.mark.parametrize("tdt", ["int64", "complex64"])
@pytest.mark.parametrize("kind", ["interleave", "rotate", "frev"])
def test_sweep_256_cubed(kind, tdt, cuda):
    import torch
    n, g = 256, 16
    blk = "packed:block(%d,%d)|block(%d,%d)|local(%d)" % (n, g, n, g, n)
    other = {
        "interleave": "packed:interleave(block(16,%d),16)|interleave(block(16,%d),16)|local(%d)" % (g, g, n),
        "rotate": "packed:rotate(1,block(%d,%d))|rotate(85,block(%d,%d))|local(%d)" % (n, g, n, g, n),
        "frev": "packed:frev(16,16,block(%d,%d))|frev(32,8,block(%d,%d))|local(%d)" % (n, g, n, g, n),
    }[kind]
    _index_roundtrip(g * g, blk, other, (n, n, n), getattr(torch, tdt), cuda)


LARGEST = [
    ((1024, 1024, 512), 32, "packed:frev(16,64,block(1024,32))|frev(64,16,block(1024,32))|local(512)"),
    ((512, 512, 1024), 16, "packed:interleave(block(32,16),16)|interleave(block(32,16),16)|local(1024)"),
]


@pytest.mark.parametrize("shape,g,other", LARGEST, ids=["1024x1024x512-32x32-frev", "512x512x1024-16x16-interleave"])
def test_sweep_largest_arrays(shape, g, other, cuda):
    """The reshape sweep's largest arrays, 4 GiB over 1024 virtual ranks and 2 GiB over 256, in 8-byte
    elements (int64 or complex64: the move is the same).  The source holds every slot's global linear
    index; the reshape must give that pattern in the destination decomposition (both patterns written
    by the device index visitor, which its own tests pin to the oracle), and the reverse reshape must
    restore the source exactly."""
    import torch
    P = g * g
    L0, L1, L2 = shape
    comm = api.Comm(P)
    S = api.decomp_from_spec(comm, "packed:block(%d,%d)|block(%d,%d)|local(%d)" % (L0, g, L1, g, L2))
    D = api.decomp_from_spec(comm, other)
    fwd, bwd = api.ReshapePlan(comm, 8, S, D), api.ReshapePlan(comm, 8, D, S)
    st = torch.cuda.current_stream(cuda).cuda_stream
    src = torch.full((P * fwd.src_pitch,), -1, dtype=torch.int64, device=cuda)
    want = torch.full((P * fwd.dest_pitch,), -7, dtype=torch.int64, device=cuda)
    api.fill_index(S, 8, src.data_ptr(), st)
    api.fill_index(D, 8, want.data_ptr(), st)
    dst = torch.full_like(want, -7)
    fwd.run(src.data_ptr(), dst.data_ptr(), st)
    back = torch.full_like(src, -1)
    bwd.run(dst.data_ptr(), back.data_ptr(), st)
    torch.cuda.synchronize()
    assert int((src >= 0).sum()) == L0 * L1 * L2
    assert torch.equal(dst, want)
    assert torch.equal(back, src)


def test_cuda_graph_replay(cuda):
    """A reshape run captured into a CUDA graph (after a first run has put its tables on the device)
    replays to the eager result; a second source buffer gives its own permutation."""
    import torch
    P = 16
    comm = api.Comm(P)
    S = api.decomp_from_spec(comm, "packed:block(32,4)|block(32,4)|local(32)")
    D = api.decomp_from_spec(comm, "packed:rotate(3,block(32,4))|rotate(11,block(32,4))|local(32)")
    plan = api.ReshapePlan(comm, 16, S, D)
    rng = np.random.default_rng(5)
    src = torch.from_numpy(rng.standard_normal(2 * P * plan.src_pitch)).view(torch.complex128).to(cuda)
    want = torch.zeros(P * plan.dest_pitch, dtype=torch.complex128, device=cuda)
    got = torch.zeros_like(want)
    stream = torch.cuda.current_stream(cuda)
    plan.run(src.data_ptr(), want.data_ptr(), stream.cuda_stream)
    torch.cuda.synchronize()
    cap = torch.cuda.Stream(cuda)
    cap.wait_stream(stream)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=cap):
        plan.run(src.data_ptr(), got.data_ptr(), torch.cuda.current_stream(cuda).cuda_stream)
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(got, want)
    src.copy_(src * 2)
    g.replay()
    plan.run(src.data_ptr(), want.data_ptr(), stream.cuda_stream)
    torch.cuda.synchronize()
    assert torch.equal(got, want)


def test_grouped_reshapes_of_mixed_sizes(cuda):
    """dmg_reshape_run_group: reshapes of different sizes, decompositions and element sizes, and one that
    transposes the fast axis, enqueued together; the contiguous ones of one element size share a launch.
    Every result equals the same plan's single run bit for bit."""
    import torch
    cases = [
        (4, "packed:block(48,2)|block(48,2)|local(48)", "packed:rotate(16,block(48,2))|rotate(1,block(48,2))|local(48)",
         16),
        (16, "packed:block(64,4)|block(32,4)|local(96)", "packed:frev(8,8,block(64,4))|block(32,4)|local(96)", 16),
        (16, "packed:block(120,4)|block(120,4)|local(120)",
         "packed:rotate(40,block(120,4))|rotate(1,block(120,4))|local(120)", 16),
        (4, "packed:block(32,2)|block(16,2)|local(64)", "packed:interleave(block(4,2),8)|local(16)|block(64,2)", 8),
        (4, "axes:block(64,2)@1,1|block(48,2)@32,2", "axes:block(64,2)@24,1|block(48,2)@1,2", 16),  # transposes
        (9, "packed:block(30,3)|block(21,3)|local(16)", "packed:local(30)|rotate(2,block(21,3))|block(16,3)", 8),
    ]
    plans, srcs, want, got, keep = [], [], [], [], []
    st = torch.cuda.current_stream(cuda).cuda_stream
    rng = np.random.default_rng(9)
    for P, a, b, es in cases:
        comm = api.Comm(P)
        S, D = api.decomp_from_spec(comm, a), api.decomp_from_spec(comm, b)
        pl = api.ReshapePlan(comm, es, S, D)
        src = torch.from_numpy(rng.integers(0, 1 << 62, (P * pl.src_pitch * es) // 8)).to(cuda)
        w = torch.full(((P * pl.dest_pitch * es) // 8,), -1, dtype=torch.int64, device=cuda)
        g = torch.full_like(w, -1)
        pl.run(src.data_ptr(), w.data_ptr(), st)
        plans.append(pl)
        srcs.append(src)
        want.append(w)
        got.append(g)
        keep.append((comm, S, D))
    api.reshape_group(plans, [x.data_ptr() for x in srcs], [x.data_ptr() for x in got], st)
    torch.cuda.synchronize()
    for i in range(len(cases)):
        assert torch.equal(got[i], want[i]), cases[i][1]
