"""Device visitors: index fill (the reference's test.c pattern) and decomp_scale, against the oracle."""
import numpy as np
import pytest

from decomp_mpi_gb300 import api
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SPECS = [
    (4, "packed:block(10,2)|block(7,2)|local(5)", (10, 7, 5)),
    (8, "packed:interleave(block(4,2),3)|block(9,2)|block(6,2)", (12, 9, 6)),
    (16, "packed:frev(4,8,block(32,4))|rotate(5,block(24,4))|local(3)", (32, 24, 3)),
    (4, "axes:block(6,2)@1,1|local(4)@3,1|block(10,2)@12,2", (6, 4, 10)),
    (6, "packed:rotate(3,block(12,3))|block(8,2)", (12, 8)),
]


@pytest.mark.parametrize("P,spec,shape", SPECS)
@pytest.mark.parametrize("ts", [4, 8])
def test_fill_index(P, spec, shape, ts, cuda):
    import torch
    d = api.decomp_from_spec(api.Comm(P), spec)
    tdt = torch.int32 if ts == 4 else torch.int64
    x = torch.full((P * d.extent(),), -1, dtype=tdt, device=cuda)
    api.fill_index(d, ts, x.data_ptr())
    off = O.global_offsets(P, spec, d.extent(), shape).ravel()
    got = x.cpu().numpy()
    assert np.array_equal(got[off], np.arange(off.size))


@pytest.mark.parametrize("P,spec,shape", SPECS)
@pytest.mark.parametrize("complex64", [False, True], ids=["c128", "c64"])
@pytest.mark.parametrize("sign", [-1, 1])
def test_decomp_scale(P, spec, shape, complex64, sign, cuda):
    """data *= prod_d f_d[x_d] (conjugate for sign 1), slots whose product is 0 untouched (dimscale.c:7-67)."""
    import torch
    rng = np.random.default_rng(5)
    npdt = np.complex64 if complex64 else np.complex128
    d = api.decomp_from_spec(api.Comm(P), spec)
    glob = (rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)).astype(npdt)
    facs = []
    for i, L in enumerate(shape):
        f = (rng.uniform(-1, 1, L) + 1j * rng.uniform(-1, 1, L)).astype(npdt)
        f[0] = 0  # an unused index
        facs.append(f if i != 1 else None)
    x = torch.from_numpy(O.scatter_global(P, spec, glob, d.extent())).to(cuda)
    api.decomp_scale(d, complex64, x.data_ptr(), facs, sign)
    prod = np.ones(shape, dtype=np.complex128)
    for i, f in enumerate(facs):
        if f is not None:
            sh = [1] * len(shape)
            sh[i] = shape[i]
            prod = prod * f.astype(np.complex128).reshape(sh)
    if sign == 1:
        prod = np.conj(prod)
    exp = np.where(prod == 0, glob.astype(np.complex128), glob.astype(np.complex128) * prod)
    got = O.gather_global(P, spec, x.cpu().numpy().astype(np.complex128), d.extent(), shape)
    tol = 1e-6 if complex64 else 1e-15
    assert np.max(np.abs(got - exp)) <= tol * max(1.0, np.max(np.abs(exp)))
