"""The tensor-core form of the complex64 split FFT (DMG_ARITH_TC16) through the C-ABI: the 1024-point
passes compute their DFT as two 32-point DFT products on the tensor cores (FP16 hi + lo operands, three
products, FP32 accumulation).  Forward spectra against the FP64 oracle and inverses back to N times the
input, within 1e-6 relative L2 (the precision form's bar), in both directions of every axis order that
puts a 1024-point line in a different place of the tile, with tiles of 4, 2 and 1 lines."""
import numpy as np
import pytest

from decomp_mpi_gb300 import api
from oracle import oracle as O
from tests.test_split_fft_gpu import Run, _rel

pytestmark = pytest.mark.gpu

TOL_TC = 1e-6  # relative L2


CASES = [
    # (P, start spec, shape): the 1024-point dimension last (contiguous lines), middle, first
    (4, "packed:block(16,2)|block(8,2)|local(1024)", (16, 8, 1024)),
    (4, "packed:block(16,2)|local(1024)|block(8,2)", (16, 1024, 8)),
    (4, "packed:local(1024)|block(12,2)|block(6,2)", (1024, 12, 6)),
    (16, "packed:block(1024,4)|block(32,4)|local(16)", (1024, 32, 16)),
    # two lines per tile (one vector axis of length 2) and a 2D array
    (2, "packed:block(2,2)|local(1024)", (2, 1024)),
    (1, "packed:local(1024)", (1024,)),
]


@pytest.mark.parametrize("P,spec,shape", CASES, ids=[str(c[2]) for c in CASES])
def test_tc_forward_and_inverse(P, spec, shape, cuda):
    r = Run(P, spec, shape, cuda, dtype=api.C64, seed=5, arith=api.ARITH_TC16, schedule=api.SCHEDULE_LINES)
    assert r.plan.arith == api.ARITH_TC16
    got = r.forward().astype(np.complex128)
    assert r.plan.device_status() == 0
    exp, mask = O.split_expected_output(P, spec, r.glob, r.wl)
    assert _rel(got[mask], exp[mask]) < TOL_TC
    back = r.inverse().astype(np.complex128)
    assert r.plan.device_status() == 0
    g = O.gather_global(P, spec, back, r.dp, r.shape) / np.prod(r.shape)
    assert _rel(g, r.glob) < TOL_TC


def test_tc_row_scaling_keeps_relative_accuracy(cuda):
    """Values near 1e-6 and near 1e6 (outside FP16's range either way): each row's power-of-two scale keeps
    the relative error at the FP32 level."""
    for scale in (1e-6, 1e6):
        P, spec, shape = 4, "packed:block(16,2)|block(8,2)|local(1024)", (16, 8, 1024)
        r = Run(P, spec, shape, cuda, dtype=api.C64, seed=7, arith=api.ARITH_TC16, scale=scale)
        got = r.forward().astype(np.complex128)
        exp, mask = O.split_expected_output(P, spec, r.glob, r.wl)
        assert _rel(got[mask], exp[mask]) < TOL_TC, scale


def test_tc_and_fp32_agree(cuda):
    """The tensor-core and FP32 forms of one plan give spectra within 1e-6 of each other; other lengths (here
    32 and 16) run the FP32 stages in both."""
    P, spec, shape = 16, "packed:block(1024,4)|block(32,4)|local(16)", (1024, 32, 16)
    a = Run(P, spec, shape, cuda, dtype=api.C64, seed=9, arith=api.ARITH_FP32)
    b = Run(P, spec, shape, cuda, dtype=api.C64, seed=9, arith=api.ARITH_TC16)
    fa, fb = a.forward(), b.forward()
    _, mask = O.split_expected_output(P, spec, a.glob, a.wl)
    assert _rel(fb[mask].astype(np.complex128), fa[mask].astype(np.complex128)) < TOL_TC
