"""The oracle restatement against the golden fixtures made by the reference itself."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.golden_cases import meta, reshape_case, reshape_names, split_case, split_names


@pytest.mark.parametrize("name", reshape_names())
def test_oracle_reshape_matches_reference(name):
    m, src, out, fill = reshape_case(name)
    dt = np.dtype(m["dtype"])
    s = src.view(dt)
    d = fill.view(dt).copy()
    O.reshape(m["P"], m["src_spec"], m["dst_spec"], s, m["src_pitch"], d, m["dst_pitch"], nthreads=4)
    assert np.array_equal(d.view(np.uint8), out), name


@pytest.mark.parametrize("name", reshape_names())
def test_oracle_pitch_matches_reference(name):
    m, *_ = reshape_case(name)
    assert O.pitch_of(m["P"], m["src_spec"]) == m["src_pitch"]
    assert O.pitch_of(m["P"], m["dst_spec"]) == m["dst_pitch"]


def test_testc_known_answer():
    """test.c's pass criterion: every local slot holds its global linear index j + 10*i (test.c:16-43)."""
    m, src, out, fill = reshape_case("testc_orig_to_new")
    P, sp, dp = m["P"], m["src_pitch"], m["dst_pitch"]
    s = np.full(P * sp, -1, np.int32)
    s[:100] = np.arange(100)  # the array lives on rank 0, C order with dim 0 fastest (stride 1)
    d = np.full(P * dp, -9, np.int32)
    O.reshape(P, m["src_spec"], m["dst_spec"], s, sp, d, dp)
    off = O.global_offsets(P, m["dst_spec"], dp, (10, 10))
    for j in range(10):
        for i in range(10):
            assert d[off[j, i]] == j + 10 * i


@pytest.mark.parametrize("name", split_names())
def test_oracle_split_matches_reference(name):
    m, z = split_case(name)
    P, wl = m["P"], m["work_len"]
    sp = O.SplitPlanCPU(P, m["spec"], wl, m["mode"], m["B"])
    work = np.zeros(P * wl, np.complex128)
    dat = z["dat"].copy()
    sp.run(dat, m["dat_pitch"], work, -1, nthreads=4)
    held = z["slot"] >= 0
    ref = z["work"][held]
    err = np.linalg.norm(work[held] - ref) / np.linalg.norm(ref)
    assert err < 1e-14, err


@pytest.mark.parametrize("name", split_names())
def test_reference_split_layout_is_true_frequency_map(name):
    """Pins the output layout: B-layout slot s = k2 + A*k1 holds frequency k1 + B*k2 (FP64 numpy oracle)."""
    m, z = split_case(name)
    P, wl = m["P"], m["work_len"]
    exp, mask = O.split_expected_output(P, m["spec"], z["glob"], wl, m["mode"], m["B"])
    held = z["slot"] >= 0
    assert np.array_equal(held, mask)
    err = np.linalg.norm(z["work"][held] - exp[held]) / np.linalg.norm(exp[held])
    assert err < 1e-12, err


@pytest.mark.parametrize("name", split_names())
def test_oracle_split_roundtrip(name):
    m, z = split_case(name)
    P, wl, dp = m["P"], m["work_len"], m["dat_pitch"]
    shape = tuple(m["shape"])
    sp = O.SplitPlanCPU(P, m["spec"], wl, m["mode"], m["B"])
    work = np.zeros(P * wl, np.complex128)
    dat = z["dat"].copy()
    sp.run(dat, dp, work, -1)
    back = np.zeros_like(dat)
    sp.run(back, dp, work, +1)
    g = O.gather_global(P, m["spec"], back, dp, shape) / np.prod(shape)
    assert np.linalg.norm(g - z["glob"]) / np.linalg.norm(z["glob"]) < 1e-13


def test_processor_grid_matches_reference():
    for c in meta()["grid"]:
        assert O.processor_grid(c["P"], c["tasks"]) == c["grid"], c


def test_fft_oracle_small_against_direct_dft():
    """The FP64 numpy oracle itself against a direct DFT in long double."""
    rng = np.random.default_rng(3)
    for n in (6, 8, 10, 15):
        x = rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)
        k = np.arange(n)
        w = np.exp(-2j * np.pi * np.outer(k, k).astype(np.longdouble) / n)
        ref = (w * x[None, :]).sum(axis=1)
        assert np.max(np.abs(np.fft.fft(x) - ref)) < 1e-13
