"""Parity at the full sizes of the benchmark configurations, through the C-ABI.

* 512^3 complex128 on an 8x8 virtual grid: the chain block -> rotate(1,170)
  -> factor_reverse((16,32),(32,16)) lands every value in its destination
  slot (bit-exact), and the split FFT's forward spectrum matches the FP64
  oracle (pocketfft on the host) in the B layout's slots within 1e-12
  relative L2, in double-float and in native FP64 arithmetic; the inverse
  returns N times the input.
* The reshape sweep (int64 / complex64 elements, 256^3, 512x512x1024,
  1024x1024x512, block <-> interleave / rotate / factor_reverse on 4x4,
  16x16 and 32x32 grids): every forward reshape gives the destination's
  global-index pattern bit for bit, and the reverse reshape restores the
  source.
* 1024^3 complex64 (complex Gaussian, 16 planted plane waves): the FP32
  and the tensor-core transforms against the FP64 oracle on whole planes of the spectrum
  (relative L2 and max-abs within 1e-6), Parseval's identity and the
  planted peaks.
"""
import math

import numpy as np
import pytest

from decomp_mpi_gb300 import api
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _chain_specs(n, g):
    blk = "packed:block(%d,%d)|block(%d,%d)|local(%d)" % (n, g, n, g, n)
    rot = "packed:rotate(1,block(%d,%d))|rotate(%d,block(%d,%d))|local(%d)" % (n, g, n // 3, n, g, n)
    frv = "packed:frev(16,%d,block(%d,%d))|frev(%d,16,block(%d,%d))|local(%d)" % (n // 16, n, g, n // 16, n, g, n)
    return blk, rot, frv


def _slot_freq(A, B, n):
    """Frequency held by each slot of one dimension of the B layout: slot k2 + A k1 holds k1 + B k2."""
    s = np.arange(n)
    return s // A + B * (s % A)


def test_c2_chain_and_split_fft_512_cubed(cuda):
    import torch
    n, g = 512, 8
    P = g * g
    shape = (n, n, n)
    N = n ** 3
    blk, rot, frv = _chain_specs(n, g)
    comm = api.Comm(P)
    D0, D1, D2 = (api.decomp_from_spec(comm, s) for s in (blk, rot, frv))
    r01 = api.ReshapePlan(comm, 16, D0, D1)
    r12 = api.ReshapePlan(comm, 16, D1, D2)
    st = torch.cuda.current_stream(cuda).cuda_stream

    rng = np.random.default_rng(1)
    glob = np.empty(shape, np.complex128)
    glob.real = rng.uniform(-1, 1, shape)
    glob.imag = rng.uniform(-1, 1, shape)
    glob_d = torch.from_numpy(glob.reshape(-1)).to(cuda)
    a0 = torch.zeros(P * r01.src_pitch, dtype=torch.complex128, device=cuda)
    api.io_scatter(D0, 16, glob_d.data_ptr(), a0.data_ptr(), st)
    a1 = torch.zeros(P * r01.dest_pitch, dtype=torch.complex128, device=cuda)
    a2 = torch.zeros(P * r12.dest_pitch, dtype=torch.complex128, device=cuda)
    r01.run(a0.data_ptr(), a1.data_ptr(), st)
    r12.run(a1.data_ptr(), a2.data_ptr(), st)
    torch.cuda.synchronize()
    # every global coordinate is in its destination slot, bit for bit (offsets from the oracle)
    for spec, arr, pitch in ((rot, a1, r01.dest_pitch), (frv, a2, r12.dest_pitch)):
        off = torch.from_numpy(O.global_offsets(P, spec, pitch, shape).reshape(-1)).to(cuda)
        assert torch.equal(arr[off].view(torch.float64), glob_d.view(torch.float64)), spec
        del off

    probe = api.SplitPlan(D2, 1 << 20, 1 << 40, 1 << 21)
    wl = 2 * probe.extent64
    probe.free()
    work = torch.zeros(P * wl, dtype=torch.complex128, device=cuda)
    sp = api.SplitPlan(D2, a2.data_ptr(), wl, work.data_ptr())
    A, Bf, _, _, _, b_spec = O.split_factors(P, frv)
    off_b = torch.from_numpy(O.global_offsets(P, b_spec, wl, shape).reshape(-1)).to(cuda)
    # the oracle: FP64 DFT of the global array, read in the B layout's slot order
    F = O.fftn64(glob)
    k = [_slot_freq(A[d], Bf[d], n) for d in range(3)]
    want = F[np.ix_(*k)].reshape(-1)
    del F
    wnorm = np.linalg.norm(want)
    keep = a2.clone()
    for arith in (api.ARITH_DF, api.ARITH_FP64):
        sp.set_arith(arith)
        a2.copy_(keep)
        work.zero_()
        sp.run(api.FFTW_FORWARD, st)
        torch.cuda.synchronize()
        got = work[off_b].cpu().numpy()
        err = np.linalg.norm(got - want) / wnorm
        assert err < 1e-12, (arith, err)
        sp.run(api.FFTW_BACKWARD, st)
        torch.cuda.synchronize()
        back = a2 / N
        rt = float((torch.linalg.vector_norm(back - keep) / torch.linalg.vector_norm(keep)).item())
        assert rt < 1e-12, (arith, rt)
        del got, back


SWEEP_SHAPES = [(256, 256, 256), (512, 512, 1024), (1024, 1024, 512)]


def _sweep_specs(shape, g):
    L0, L1, L2 = shape

    def il(L):
        A = 2 * g if L % (2 * g) == 0 else g
        return "interleave(block(%d,%d),%d)" % (A, g, L // A)

    blk = "packed:block(%d,%d)|block(%d,%d)|local(%d)" % (L0, g, L1, g, L2)
    return blk, {
        "interleave": "packed:%s|%s|local(%d)" % (il(L0), il(L1), L2),
        "rotate": "packed:rotate(%d,block(%d,%d))|rotate(1,block(%d,%d))|local(%d)" % (L0 // 3, L0, g, L1, g, L2),
        "factor_reverse": "packed:frev(16,%d,block(%d,%d))|frev(%d,16,block(%d,%d))|local(%d)" % (
            L0 // 16, L0, g, L1 // 16, L1, g, L2),
    }


@pytest.mark.parametrize("kind", ["interleave", "rotate", "factor_reverse"])
@pytest.mark.parametrize("g", [4, 16, 32])
@pytest.mark.parametrize("shape", SWEEP_SHAPES, ids=["256^3", "512x512x1024", "1024x1024x512"])
def test_c3_sweep_placement(shape, g, kind, cuda):
    """Both directions of the transition, in 8-byte elements (int64 and complex64 are the same move for
    the kernel, which copies bytes): the destination holds every coordinate's global index in its slot,
    and the reverse reshape restores the source."""
    import torch
    P = g * g
    blk, others = _sweep_specs(shape, g)
    comm = api.Comm(P)
    B = api.decomp_from_spec(comm, blk)
    D = api.decomp_from_spec(comm, others[kind])
    st = torch.cuda.current_stream(cuda).cuda_stream
    for s, d in ((B, D), (D, B)):
        fwd, bwd = api.ReshapePlan(comm, 8, s, d), api.ReshapePlan(comm, 8, d, s)
        src = torch.full((P * fwd.src_pitch,), -1, dtype=torch.int64, device=cuda)
        want = torch.full((P * fwd.dest_pitch,), -7, dtype=torch.int64, device=cuda)
        api.fill_index(s, 8, src.data_ptr(), st)
        api.fill_index(d, 8, want.data_ptr(), st)
        dst = torch.full_like(want, -7)
        back = torch.full_like(src, -1)
        fwd.run(src.data_ptr(), dst.data_ptr(), st)
        bwd.run(dst.data_ptr(), back.data_ptr(), st)
        torch.cuda.synchronize()
        assert torch.equal(dst, want), kind
        assert torch.equal(back, src), kind
        del dst, back
        assert int((src >= 0).sum()) == shape[0] * shape[1] * shape[2]
        fwd.free()
        bwd.free()
        del src, want


def _c4_input(cuda, n):
    """1024^3 complex64 in global C order on the device: complex Gaussian N(0,1) (seed 2) plus 16 unit plane
    waves at wavenumbers drawn from seed 2; returns (values, wavenumbers)."""
    import torch
    N = n ** 3
    gen = torch.Generator(device=cuda)
    gen.manual_seed(2)
    glob = torch.empty(N, dtype=torch.complex64, device=cuda)
    glob.real.normal_(0, math.sqrt(0.5), generator=gen)
    glob.imag.normal_(0, math.sqrt(0.5), generator=gen)
    waves = np.random.default_rng(2).integers(0, n, size=(16, 3))
    idx = torch.arange(n, device=cuda, dtype=torch.float64)
    g3 = glob.view(n, n, n)
    for kv in waves:
        e = [torch.exp(2j * math.pi * float(kv[d]) * idx / n) for d in range(3)]
        g3 += (e[0][:, None, None] * e[1][None, :, None] * e[2][None, None, :]).to(torch.complex64)
    return glob, waves


def _plane_oracle(x_host, n, k0s):
    """FP64 spectrum planes X[k0, :, :] of a global n^3 array (host, C order) by the definition along the
    first dimension (a weighted sum of the n planes, in FP64) and pocketfft over the other two."""
    w = np.exp(-2j * np.pi * np.outer(np.asarray(k0s), np.arange(n)) / n)  # (K, n)
    x2 = x_host.reshape(n, n * n)
    acc = np.zeros((len(k0s), n * n), np.complex128)
    step = 1 << 16
    for c in range(0, n * n, step):
        acc[:, c:c + step] = w @ x2[:, c:c + step].astype(np.complex128)
    return np.stack([O.fftn64(acc[i].reshape(n, n)) for i in range(len(k0s))])


@pytest.mark.parametrize("arith", [api.ARITH_FP32, api.ARITH_TC16], ids=["fp32", "tensor-core"])
def test_c4_precision_1024_cubed(arith, cuda):
    import torch
    n, g = 1024, 8
    P = g * g
    N = n ** 3
    st = torch.cuda.current_stream(cuda).cuda_stream
    comm = api.Comm(P)
    spec = "packed:block(%d,%d)|block(%d,%d)|local(%d)" % (n, g, n, g, n)
    D = api.decomp_from_spec(comm, spec)
    glob, waves = _c4_input(cuda, n)
    x_host = glob.cpu().numpy()
    energy = float(torch.sum(glob.abs().to(torch.float64) ** 2).item())
    x = torch.empty(P * D.extent(), dtype=torch.complex64, device=cuda)
    api.io_scatter(D, 8, glob.data_ptr(), x.data_ptr(), st)
    del glob
    probe = api.SplitPlan(D, 1 << 20, 1 << 40, 1 << 21, dtype=api.C64)
    ext = probe.extent64
    probe.free()
    wl = 2 * ext
    work = torch.empty(P * wl, dtype=torch.complex64, device=cuda)
    sp = api.SplitPlan(D, x.data_ptr(), wl, work.data_ptr(), dtype=api.C64)
    sp.set_arith(arith)
    sp.run(api.FFTW_FORWARD, st)
    assert sp.device_status() == 0
    A, Bf, _, _, _, b_spec = O.split_factors(P, spec)
    assert sp.decomp_B().extent() == ext  # the gather below reads rank r's slots at r * ext
    # the spectrum in global frequency order on the device
    out = torch.empty(N, dtype=torch.complex64, device=cuda)
    api.io_gather(sp.decomp_B(), 8, work.view(P, wl)[:, :ext].contiguous().data_ptr(), out.data_ptr(), st)
    torch.cuda.synchronize()
    del work, x
    # slots -> frequencies: global slot s holds frequency k(s); the plane of frequency k0 along dim 0
    # sits at slot s0 with k(s0) = k0
    k = [_slot_freq(A[d], Bf[d], n) for d in range(3)]
    inv = [np.argsort(kd) for kd in k]
    k0s = [0, int(waves[0][0]), int(waves[5][0]), 777]
    want = _plane_oracle(x_host, n, k0s)
    o3 = out.view(n, n, n)
    rows = torch.from_numpy(inv[1]).to(cuda)
    cols = torch.from_numpy(inv[2]).to(cuda)
    num = den = 0.0
    max_abs = 0.0
    for i, k0 in enumerate(k0s):
        plane = o3[int(inv[0][k0])][rows][:, cols].cpu().numpy().astype(np.complex128)
        d = plane - want[i]
        num += float(np.sum(np.abs(d) ** 2))
        den += float(np.sum(np.abs(want[i]) ** 2))
        max_abs = max(max_abs, float(np.abs(d).max()))
    rel = math.sqrt(num / den)
    peak = float(np.abs(want).max())
    assert rel < 1e-6, rel
    assert max_abs / peak < 1e-6, max_abs / peak
    # Parseval over the whole spectrum (an amplitude error of 1e-6 moves the energy by up to 2e-6), and the
    # planted waves at N (plus the noise's own coefficient)
    spec_energy = float(torch.sum(out.abs().to(torch.float64) ** 2).item())
    assert abs(spec_energy / N - energy) / energy < 2e-6
    for kv in waves:
        s = [int(inv[d][int(kv[d])]) for d in range(3)]
        v = complex(o3[s[0], s[1], s[2]].item())
        assert abs(v - N) / N < 1e-3
