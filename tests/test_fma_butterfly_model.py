"""Host model of the native-FP64 twiddled stages (no GPU).

The FP64 pass kernel runs a twiddled radix-8 stage, y_s = sum_q w^q x_q W8^(q s), as three layers of
radix-2 butterflies y0 = a + t b, y1 = 2 a - y0 whose twiddle t is one complex number per butterfly
(w^4; w^2 and w^2 W4; w, w W4, w W8 and w W8 W4), and a twiddled radix-4 stage the same way
(dft8_tw_fma / dft4_tw_fma in csrc/kernels/fft_pass.cuh).  This model replays that order of
operations in float64 and checks it against the direct sum for both directions, with the outputs in
the kernel's bit-reversed places, and checks that its rounding error stays at the level of the
conventional form (seven twiddle products, then the 8-point DFT).
"""
import numpy as np
import pytest


def _bfly(a, b, t):
    y0 = a + t * b
    return y0, 2 * a - y0


def _root(num, den, sign, dtype=np.complex128):
    """exp(sign 2 pi i num / den), rounded once to dtype (the kernels' tables)."""
    ang = np.longdouble(sign) * 2 * np.pi * np.longdouble(num) / np.longdouble(den)
    return dtype(complex(np.cos(ang), np.sin(ang))) if dtype is np.complex128 else \
        np.clongdouble(np.cos(ang)) + 1j * np.clongdouble(np.sin(ang))


def dft8_tw_layers(x, j, lp, sign):
    """w = w_(8 lp)^j; the twiddles w, w^2, w^4 and w W8 as table entries."""
    n = 8 * lp
    w1, w2, w4, v = (_root(j, n, sign), _root(2 * j, n, sign), _root(4 * j, n, sign), _root(j + lp, n, sign))
    W4 = 1j * sign
    a = list(x)
    for q in range(4):
        a[q], a[q + 4] = _bfly(a[q], a[q + 4], w4)
    a[0], a[2] = _bfly(a[0], a[2], w2)
    a[1], a[3] = _bfly(a[1], a[3], w2)
    a[4], a[6] = _bfly(a[4], a[6], w2 * W4)
    a[5], a[7] = _bfly(a[5], a[7], w2 * W4)
    a[0], a[1] = _bfly(a[0], a[1], w1)
    a[2], a[3] = _bfly(a[2], a[3], w1 * W4)
    a[4], a[5] = _bfly(a[4], a[5], v)
    a[6], a[7] = _bfly(a[6], a[7], v * W4)
    return np.array([a[0], a[4], a[2], a[6], a[1], a[5], a[3], a[7]])


def dft4_tw_layers(x, j, lp, sign):
    n = 4 * lp
    w1, w2 = _root(j, n, sign), _root(2 * j, n, sign)
    W4 = 1j * sign
    a = list(x)
    a[0], a[2] = _bfly(a[0], a[2], w2)
    a[1], a[3] = _bfly(a[1], a[3], w2)
    a[0], a[1] = _bfly(a[0], a[1], w1)
    a[2], a[3] = _bfly(a[2], a[3], w1 * W4)
    return np.array([a[0], a[2], a[1], a[3]])


def dft8_tw_conventional(x, j, lp, sign):
    """The conventional form: seven twiddle products, then the 8-point DFT as radix-2 layers (a +- t b)."""
    n = 8 * lp
    a = [x[q] * _root(j * q, n, sign) if q else x[0] for q in range(8)]
    W8, W4 = _root(lp, n, sign), 1j * sign

    def pm(u, v, t):
        return u + t * v, u - t * v
    for q in range(4):
        a[q], a[q + 4] = pm(a[q], a[q + 4], 1)
    a[0], a[2] = pm(a[0], a[2], 1)
    a[1], a[3] = pm(a[1], a[3], 1)
    a[4], a[6] = pm(a[4], a[6], W4)
    a[5], a[7] = pm(a[5], a[7], W4)
    a[0], a[1] = pm(a[0], a[1], 1)
    a[2], a[3] = pm(a[2], a[3], W4)
    a[4], a[5] = pm(a[4], a[5], W8)
    a[6], a[7] = pm(a[6], a[7], W8 * W4)
    return np.array([a[0], a[4], a[2], a[6], a[1], a[5], a[3], a[7]])


def _direct(x, j, lp, sign, dtype=np.complex128):
    r = len(x)
    n = r * lp
    return np.array([sum(_root(j * q, n, sign, dtype) * x[q] * _root(q * s * lp, n, sign, dtype) for q in range(r))
                     for s in range(r)])


@pytest.mark.parametrize("sign", [-1, 1], ids=["forward", "inverse"])
@pytest.mark.parametrize("radix", [8, 4])
def test_layers_equal_the_twiddled_dft(sign, radix):
    rng = np.random.default_rng(7)
    for lp in (1, 2, 8, 64):
        for j in range(lp):
            x = rng.standard_normal(radix) + 1j * rng.standard_normal(radix)
            got = dft8_tw_layers(x, j, lp, sign) if radix == 8 else dft4_tw_layers(x, j, lp, sign)
            assert np.allclose(got, _direct(x, j, lp, sign), rtol=0, atol=1e-13), (lp, j)


def test_layer_rounding_matches_the_conventional_form():
    """Against a long-double evaluation, the layered form's error stays at the conventional form's level
    (seven twiddle products, then the 8-point DFT as radix-2 layers), a few units in the last place of
    float64 (this model rounds every product; the kernel's fused multiply-adds round less)."""
    rng = np.random.default_rng(11)
    sign, lp = -1, 64
    err_layers, err_conv = [], []
    for _ in range(400):
        j = int(rng.integers(0, lp))
        x = rng.standard_normal(8) + 1j * rng.standard_normal(8)
        exact = _direct(x.astype(np.clongdouble), j, lp, sign, np.clongdouble)
        lay = dft8_tw_layers(x, j, lp, sign)
        conv = dft8_tw_conventional(x, j, lp, sign)
        scale = float(np.max(np.abs(exact)))
        err_layers.append(float(np.max(np.abs(lay - exact))) / scale)
        err_conv.append(float(np.max(np.abs(conv - exact))) / scale)
    assert max(err_layers) < 8 * np.finfo(np.float64).eps
    assert np.mean(err_layers) < 1.5 * np.mean(err_conv)
