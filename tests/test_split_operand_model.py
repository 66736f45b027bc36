"""Numerics of DFT stages computed as matrix products of split operands, on the CPU.

A tensor-core stage multiplies 16-point (or 4-point) complex blocks, written as real vectors of
interleaved (re, im) pairs, by the real form of the DFT matrix.  The tensor pipes take 16-bit
operands, so each FP32 operand x is split into parts (x = hi + lo, hi = round16(x),
lo = round16(x - hi)) and the product is the sum of a few part products accumulated in FP32.  This
module models that arithmetic on 1024-point lines (16 * 16 * 4 four-step, FP64 twiddle tables
rounded to FP32, twiddles applied in FP32) and pins which operand split reaches FP32-level error:

* BF16 hi + lo with 3 products (hi*hi + lo*hi + hi*lo) keeps about 16 significant bits and lands
  near 5e-6 relative L2, outside a 1e-6 bar;
* FP16 hi + lo with 3 products keeps about 22 bits and lands near 1.2e-7, as does BF16 with three
  parts and 6 products, both within a factor two of plain FP32 arithmetic (7.7e-8);
* FP16's range needs a power-of-two scale per block for inputs far from 1; scaling by the block's
  largest power of two leaves the error unchanged.

The model accumulates each part product in FP64 and rounds it into an FP32 running sum, which is
at least as accurate as the tensor pipe's FP32 accumulation: the figures are lower bounds on the
error of such a stage.
"""
import numpy as np
import pytest

N = 1024
LINES = 64


def _bf16(x):
    b = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16  # round to nearest even on the top 16 bits
    return r.astype(np.uint32).view(np.float32)


def _f16(x):
    return np.asarray(x, np.float32).astype(np.float16).astype(np.float32)


def _f32(x):
    return np.asarray(x, np.float32)


def _split(x, rnd, parts):
    out, r = [], np.asarray(x, np.float32)
    for _ in range(parts):
        h = rnd(r)
        out.append(h)
        r = (r - h).astype(np.float32)
    return out


def _dft_real(n):
    k = np.arange(n)
    w = np.exp(-2j * np.pi * np.outer(k, k) / n)
    m = np.zeros((2 * n, 2 * n))
    m[0::2, 0::2], m[0::2, 1::2] = w.real, -w.imag
    m[1::2, 0::2], m[1::2, 1::2] = w.imag, w.real
    return m


def _block_dft(x, rnd, terms, scale):
    """DFT of the last axis (length <= 16) as one split-operand matrix product."""
    n = x.shape[-1]
    xr = np.stack([x.real, x.imag], -1).reshape(*x.shape[:-1], 2 * n).astype(np.float32)
    s = np.ones(xr.shape[:-1] + (1,), np.float32)
    if scale:
        m = np.max(np.abs(xr), axis=-1, keepdims=True)
        m[m == 0] = 1
        s = np.exp2(np.floor(np.log2(m))).astype(np.float32)
    xs = _split(xr / s, rnd, 3)
    ms = _split(_dft_real(n).astype(np.float32), rnd, 3)
    acc = np.zeros_like(xr)
    for i, j in terms:
        acc = (acc + (xs[i].astype(np.float64) @ ms[j].T.astype(np.float64)).astype(np.float32)).astype(np.float32)
    acc = acc * s
    return (acc[..., 0::2] + 1j * acc[..., 1::2]).astype(np.complex64)


def _fft(x, rnd, terms, scale=False):
    """Four-step FFT of the last axis: 16-point blocks on the model, the rest recursively."""
    n = x.shape[-1]
    if n <= 16:
        return _block_dft(x, rnd, terms, scale)
    n1, n2 = 16, n // 16
    a = _fft(np.swapaxes(x.reshape(*x.shape[:-1], n1, n2), -1, -2), rnd, terms, scale)  # [j2, k1]
    tw = np.exp(-2j * np.pi * np.outer(np.arange(n2), np.arange(n1)) / n).astype(np.complex64)
    b = _fft(np.swapaxes((a * tw).astype(np.complex64), -1, -2), rnd, terms, scale)  # [k1, k2]
    return np.swapaxes(b, -1, -2).reshape(*x.shape[:-1], n)  # k = k1 + 16 k2


THREE = [(0, 0), (1, 0), (0, 1)]
SIX = [(0, 0), (1, 0), (0, 1), (1, 1), (2, 0), (0, 2)]


@pytest.fixture(scope="module")
def lines():
    rng = np.random.default_rng(0)
    x = rng.uniform(-1, 1, (LINES, N)) + 1j * rng.uniform(-1, 1, (LINES, N))
    return x, np.fft.fft(x, axis=-1)


def _rel(got, want):
    return float(np.linalg.norm(got - want) / np.linalg.norm(want))


def test_fp32_products_reach_fp32_level(lines):
    x, want = lines
    assert _rel(_fft(x.astype(np.complex64), _f32, [(0, 0)]), want) < 1.5e-7


def test_bf16_three_products_miss_the_bar(lines):
    x, want = lines
    e = _rel(_fft(x.astype(np.complex64), _bf16, THREE), want)
    assert 1e-6 < e < 2e-5


@pytest.mark.parametrize("rnd,terms,scale", [(_f16, THREE, False), (_f16, THREE, True), (_bf16, SIX, False)],
                         ids=["fp16-3", "fp16-3-scaled", "bf16-6"])
def test_splits_at_fp32_level(lines, rnd, terms, scale):
    x, want = lines
    fp32 = _rel(_fft(x.astype(np.complex64), _f32, [(0, 0)]), want)
    e = _rel(_fft(x.astype(np.complex64), rnd, terms, scale), want)
    assert e < 2.0 * fp32 and e < 3e-7


def test_fp16_needs_the_scale_far_from_one(lines):
    """Inputs near 1e-6 leave FP16's lo parts subnormal: the per-block scale restores the error."""
    x, want = lines
    tiny = (x * 1e-6).astype(np.complex64)
    e_raw = _rel(_fft(tiny, _f16, THREE), want * 1e-6)
    e_scaled = _rel(_fft(tiny, _f16, THREE, scale=True), want * 1e-6)
    assert e_scaled < 3e-7 < e_raw
