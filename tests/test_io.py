"""Global-order I/O: the per-rank file view (makeIOType) and file write/read through the C-ABI."""
import os

import numpy as np
import pytest

from decomp_mpi_gb300 import api
from oracle import oracle as O

SPECS = [
    # (P, spec, shape)
    (4, "packed:block(10,2)|block(7,2)|local(5)", (10, 7, 5)),          # uneven blocks
    (6, "packed:rotate(3,block(12,3))|block(8,2)", (12, 8)),            # rotated 2D
    (8, "packed:interleave(block(4,2),3)|block(9,2)|block(6,2)", (12, 9, 6)),
    (16, "packed:frev(4,8,block(32,4))|rotate(5,block(24,4))|local(3)", (32, 24, 3)),
    (4, "axes:block(6,2)@1,1|local(4)@3,1|block(10,2)@12,2", (6, 4, 10)),  # Fortran order, rank strides 1, 2
]


@pytest.mark.parametrize("P,spec,shape", SPECS)
def test_file_view_matches_oracle_offsets(P, spec, shape):
    """Every rank's view lists its elements in global C order, at their C-order file positions and
    their buffer offsets (reference writeFile, fftw_bench.c:26-63)."""
    comm = api.Comm(P)
    d = api.decomp_from_spec(comm, spec)
    pitch = d.extent()
    off = O.global_offsets(P, spec, pitch, shape).ravel()
    seen = np.zeros(off.size, dtype=bool)
    for r in range(P):
        f, m = api.io_view(d, r)
        assert np.all(np.diff(f) > 0)  # C order
        held = np.nonzero((off >= r * pitch) & (off < (r + 1) * pitch))[0]
        assert np.array_equal(f, held)
        assert np.array_equal(r * pitch + m, off[f])
        seen[f] = True
    assert seen.all()


@pytest.mark.gpu
@pytest.mark.parametrize("P,spec,shape", SPECS)
@pytest.mark.parametrize("dtype", [np.complex128, np.int32, np.dtype("V3")], ids=["c128", "i32", "b3"])
def test_write_then_read_file(P, spec, shape, dtype, tmp_path, cuda):
    import torch
    comm = api.Comm(P)
    d = api.decomp_from_spec(comm, spec)
    pitch = d.extent()
    es = np.dtype(dtype).itemsize
    rng = np.random.default_rng(3)
    raw = rng.integers(0, 256, size=P * pitch * es, dtype=np.uint8)
    src = torch.from_numpy(raw.copy()).to(cuda)
    path = str(tmp_path / "array.bin")
    api.write_file(path, d, es, src.data_ptr())
    got = np.fromfile(path, dtype=np.uint8)
    off = O.global_offsets(P, spec, pitch, shape).ravel()
    want = raw.reshape(-1, es)[off].ravel()
    assert got.size == int(np.prod(shape)) * es
    assert np.array_equal(got, want)
    # read back into a fresh array: every held slot restored, bit for bit
    dst = torch.zeros(P * pitch * es, dtype=torch.uint8, device=cuda)
    api.read_file(path, d, es, dst.data_ptr())
    back = dst.cpu().numpy().reshape(-1, es)
    assert np.array_equal(back[off], raw.reshape(-1, es)[off])
    os.remove(path)


@pytest.mark.gpu
def test_read_file_into_another_decomposition(tmp_path, cuda):
    """Write in one decomposition and read in another: the file is decomposition-independent."""
    import torch
    P, shape = 16, (32, 24, 3)
    a = api.decomp_from_spec(api.Comm(P), SPECS[3][1])
    comm = api.Comm(P)
    b = api.decomp_from_spec(comm, "packed:block(32,4)|block(24,4)|local(3)")
    n = int(np.prod(shape))
    glob = np.arange(n, dtype=np.int64)
    src = torch.from_numpy(O.scatter_global(P, SPECS[3][1], glob.reshape(shape), a.extent())).to(cuda)
    path = str(tmp_path / "g.bin")
    api.write_file(path, a, 8, src.data_ptr())
    dst = torch.full((P * b.extent(),), -1, dtype=torch.int64, device=cuda)
    api.read_file(path, b, 8, dst.data_ptr())
    g = O.gather_global(P, "packed:block(32,4)|block(24,4)|local(3)", dst.cpu().numpy(), b.extent(), shape)
    assert np.array_equal(g.ravel(), glob)


@pytest.mark.gpu
def test_read_file_too_short(tmp_path, cuda):
    import torch
    P, spec, shape = SPECS[0]
    d = api.decomp_from_spec(api.Comm(P), spec)
    path = str(tmp_path / "short.bin")
    np.zeros(10, dtype=np.uint8).tofile(path)
    dst = torch.zeros(P * d.extent() * 8, dtype=torch.uint8, device=cuda)
    with pytest.raises(RuntimeError):
        api.read_file(path, d, 8, dst.data_ptr())
