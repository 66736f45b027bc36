"""Batched split-FFT runs and the request server: batched results equal single runs, every job's result is
the same alone and in a mix of sizes and types, and the results match the FP64 oracle."""
import numpy as np
import pytest

from decomp_mpi_gb300 import api
from oracle import oracle as O

pytestmark = pytest.mark.gpu

GRID = 4
P = GRID * GRID
TOL = {api.C128: 1e-12, api.C64: 2e-6}


def _rel(a, b):
    m = float(np.max(np.abs(b)))
    return float(np.linalg.norm((a - b) / m) / np.linalg.norm(b / m)) if m else float(np.max(np.abs(a)))


def _cube(side, dtype, seed):
    rng = np.random.default_rng(seed)
    g = rng.uniform(-1, 1, (side,) * 3) + 1j * rng.uniform(-1, 1, (side,) * 3)
    return g if dtype == api.C128 else g.astype(np.complex64)


@pytest.mark.parametrize("dtype", [api.C128, api.C64], ids=["c128", "c64"])
def test_batched_run_equals_single_runs(dtype, cuda):
    """dmg_split_run_batch over three arrays gives, bit for bit, what three dmg_split_run calls give."""
    import torch
    side = 24
    _, rot = api.cube_specs(side, GRID)
    comm = api.Comm(P)
    D = api.decomp_from_spec(comm, rot)
    tdt = torch.complex128 if dtype == api.C128 else torch.complex64
    probe = api.SplitPlan(D, 1 << 20, 1 << 40, 1 << 21, dtype=dtype)
    length = 2 * probe.extent64
    probe.free()
    dats = [torch.from_numpy(O.scatter_global(P, rot, _cube(side, dtype, s), D.extent())).to(cuda) for s in range(3)]
    works = [torch.zeros(P * length, dtype=tdt, device=cuda) for _ in range(3)]
    scales = torch.zeros(3 * 64, dtype=torch.int32, device=cuda)
    sp = api.SplitPlan(D, dats[0].data_ptr(), length, works[0].data_ptr(), dtype=dtype)
    st = torch.cuda.current_stream().cuda_stream
    single_w, single_d = [], []
    for i in range(3):
        d = dats[i].clone()
        w = torch.zeros_like(works[i])
        sp.set_buffers(d.data_ptr(), w.data_ptr())
        sp.run(api.FFTW_FORWARD, st)
        single_w.append(w.clone())
        sp.run(api.FFTW_BACKWARD, st)
        single_d.append(d)
    sptr = [scales.data_ptr() + 256 * i for i in range(3)]
    sp.run_batch(api.FFTW_FORWARD, [d.data_ptr() for d in dats], [w.data_ptr() for w in works], sptr, st)
    torch.cuda.synchronize()
    for i in range(3):
        assert torch.equal(works[i], single_w[i])
    sp.run_batch(api.FFTW_BACKWARD, [d.data_ptr() for d in dats], [w.data_ptr() for w in works], sptr, st)
    torch.cuda.synchronize()
    for i in range(3):
        assert torch.equal(dats[i], single_d[i])


def _job_list():
    rng = np.random.default_rng(3)
    sides = [16, 24, 32, 48]
    return [(int(rng.choice(sides)), api.C128 if rng.random() < 0.5 else api.C64, 100 + i) for i in range(20)]


def _run(server, jobs, cuda, one_at_a_time):
    import torch
    bufs = []
    for side, dtype, seed in jobs:
        blk, _ = api.cube_specs(side, GRID)
        n_in, n_spec, n_out = server.sizes(side, dtype)
        npdt = np.complex128 if dtype == api.C128 else np.complex64
        comm = api.Comm(P)
        pitch = api.decomp_from_spec(comm, blk).extent()
        host_in = torch.from_numpy(O.scatter_global(P, blk, _cube(side, dtype, seed), pitch).astype(npdt)).pin_memory()
        assert host_in.numel() == n_in
        spec = torch.zeros(n_spec, dtype=host_in.dtype).pin_memory()
        out = torch.zeros(n_out, dtype=host_in.dtype).pin_memory()
        bufs.append((host_in, spec, out))
    done = []
    for (side, dtype, _), (hi, hs, ho) in zip(jobs, bufs):
        server.submit(side, dtype, hi.data_ptr(), hs.data_ptr(), ho.data_ptr())
        if one_at_a_time:
            server.drain()
    server.drain()
    done += server.poll()
    assert len(done) == len(jobs) and all(d["status"] == 0 for d in done)
    return bufs, done


def test_results_alone_equal_results_in_the_mix(cuda):
    """Each job's spectrum and inverse are the same run alone (one slot, no batching, one job at a time)
    and run in a mix (several slots, batching, all submitted at once)."""
    jobs = _job_list()
    alone = api.Server(GRID, 1 << 30, slots=1, max_batch=1)
    a_bufs, _ = _run(alone, jobs, cuda, one_at_a_time=True)
    alone.close()
    mix = api.Server(GRID, 1 << 30, slots=3, max_batch=8)
    m_bufs, m_done = _run(mix, jobs, cuda, one_at_a_time=False)
    mix.close()
    assert max(d["batch"] for d in m_done) > 1  # some launches were shared
    srv = api.Server(GRID, 1 << 26, slots=1, max_batch=1)
    for (side, dtype, _), a, m in zip(jobs, a_bufs, m_bufs):
        # the same kernels on the same data: identical bits in every slot a rank holds
        spec_held, out_held = _held(srv, side, dtype)
        assert np.array_equal(a[1].numpy()[spec_held], m[1].numpy()[spec_held])
        assert np.array_equal(a[2].numpy()[out_held], m[2].numpy()[out_held])
    srv.close()


def _held(server, side, dtype):
    """Masks of the spectrum and output slots some rank holds (the rest is padding)."""
    _, rot = api.cube_specs(side, GRID)
    n_in, n_spec, n_out = server.sizes(side, dtype)
    ext = n_spec // P
    _, mask = O.split_expected_output(P, rot, np.zeros((side,) * 3), 2 * ext)
    spec = mask.reshape(P, 2 * ext)[:, :ext].ravel()
    out = np.zeros(n_out, dtype=bool)
    out[O.global_offsets(P, rot, n_out // P, (side,) * 3).ravel()] = True
    return spec, out


def test_server_results_match_oracle(cuda):
    """Spectrum against the FP64 oracle in the plan's B slots, inverse back to N times the input."""
    jobs = [(24, api.C128, 7), (24, api.C64, 8), (48, api.C128, 9), (16, api.C64, 10)]
    srv = api.Server(GRID, 1 << 30, slots=2, max_batch=4)
    bufs, _ = _run(srv, jobs, cuda, one_at_a_time=False)
    for (side, dtype, seed), (hi, hs, ho) in zip(jobs, bufs):
        blk, rot = api.cube_specs(side, GRID)
        g = _cube(side, dtype, seed).astype(np.complex128)
        n_in, n_spec, n_out = srv.sizes(side, dtype)
        ext = n_spec // P
        exp, mask = O.split_expected_output(P, rot, g, 2 * ext)
        exp = exp.reshape(P, 2 * ext)[:, :ext].ravel()
        mask = mask.reshape(P, 2 * ext)[:, :ext].ravel()
        got = hs.numpy().astype(np.complex128)
        assert _rel(got[mask], exp[mask]) < TOL[dtype]
        comm = api.Comm(P)
        pitch_rot = api.decomp_from_spec(comm, rot).extent()
        back = O.gather_global(P, rot, ho.numpy().astype(np.complex128), pitch_rot, (side,) * 3) / side ** 3
        assert _rel(back, g) < TOL[dtype]
    srv.close()


def test_server_refuses_a_job_larger_than_the_arena(cuda):
    srv = api.Server(GRID, 1 << 20, slots=1, max_batch=1)
    import torch
    n_in, _, _ = srv.sizes(64, api.C128)
    x = torch.zeros(n_in, dtype=torch.complex128).pin_memory()
    with pytest.raises(RuntimeError):
        srv.submit(64, api.C128, x.data_ptr())
    srv.close()


C5_SIDES = [48, 64, 96, 120, 128, 160, 192, 240, 256, 320, 384, 480, 512]


def _check_job(srv, side, dtype, g, hs, ho):
    """A served job's spectrum against the FP64 oracle (global frequency order) and its inverse against
    N times the input."""
    blk, rot = api.cube_specs(side, GRID)
    shape = (side,) * 3
    _, n_spec, n_out = srv.sizes(side, dtype)
    ext = n_spec // P
    A, Bf, _, _, _, b_spec = O.split_factors(P, rot)
    got = hs.numpy()[O.global_offsets(P, b_spec, ext, shape)].astype(np.complex128)
    F = O.fftn64(g)
    k = [np.arange(side) // A[d] + Bf[d] * (np.arange(side) % A[d]) for d in range(3)]
    want = F[np.ix_(*k)]
    del F
    e_spec = _rel(got, want)
    del got, want
    back = ho.numpy()[O.global_offsets(P, rot, n_out // P, shape)].astype(np.complex128) / side ** 3
    e_back = _rel(back, g)
    return e_spec, e_back


@pytest.mark.parametrize("sides", [C5_SIDES[:9], [320], [384], [480], [512]],
                         ids=["48-256", "320", "384", "480", "512"])
def test_server_every_c5_side_both_types(sides, cuda):
    """Every cube side of the served stream, in complex64 and complex128, through the server in one mix
    (several slots, batching on): spectra against the FP64 oracle and inverses back to N times the
    input, within 1e-12 (complex128) and 2e-6 (complex64)."""
    import torch
    jobs = [(s, dt, 1000 + 2 * s + dt) for s in sides for dt in (api.C128, api.C64)]
    srv = api.Server(GRID, 32 << 30, slots=3, max_batch=8)
    bufs = []
    for side, dtype, seed in jobs:
        blk, _ = api.cube_specs(side, GRID)
        n_in, n_spec, n_out = srv.sizes(side, dtype)
        g = _cube(side, dtype, seed)
        pitch = n_in // P
        hi = torch.from_numpy(O.scatter_global(P, blk, g, pitch)).pin_memory()
        assert hi.numel() == n_in
        hs = torch.zeros(n_spec, dtype=hi.dtype).pin_memory()
        ho = torch.zeros(n_out, dtype=hi.dtype).pin_memory()
        bufs.append((g, hi, hs, ho))
        srv.submit(side, dtype, hi.data_ptr(), hs.data_ptr(), ho.data_ptr())
    srv.drain()
    done = srv.poll()
    assert len(done) == len(jobs) and all(d["status"] == 0 for d in done)
    for (side, dtype, _), (g, hi, hs, ho) in zip(jobs, bufs):
        e_spec, e_back = _check_job(srv, side, dtype, g.astype(np.complex128), hs, ho)
        assert e_spec < TOL[dtype], (side, dtype, e_spec)
        assert e_back < TOL[dtype], (side, dtype, e_back)
    srv.close()


def test_server_arithmetic_choice(cuda):
    """dmg_server_set_arith: complex128 jobs in native FP64 and complex64 jobs in the tensor-core form give the
    FP64 oracle's spectra and round trips; the choice is refused while jobs are queued."""
    jobs = [(24, api.C128, 31), (32, api.C64, 32)]
    srv = api.Server(GRID, 1 << 30, slots=2, max_batch=4)
    srv.set_arith(api.C128, api.ARITH_FP64)
    srv.set_arith(api.C64, api.ARITH_TC16)
    with pytest.raises(Exception):
        srv.set_arith(api.C128, api.ARITH_FP32)
    bufs, _ = _run(srv, jobs, cuda, one_at_a_time=False)
    for (side, dtype, seed), (hi, hs, ho) in zip(jobs, bufs):
        g = _cube(side, dtype, seed).astype(np.complex128)
        e_spec, e_back = _check_job(srv, side, dtype, g, hs, ho)
        assert e_spec < TOL[dtype] and e_back < TOL[dtype], (side, dtype, e_spec, e_back)
    srv.close()


@pytest.mark.parametrize("arith128", [None, api.ARITH_FP64], ids=["df", "fp64"])
def test_mixed_sides_share_launches(arith128, cuda):
    """dmg_server_set_mixing: jobs of different sides (one element type per batch) share the reshape and pass
    launches.  Each job's spectrum and inverse are the same bits as on a one-slot server that runs it alone
    with the same plans, and match the FP64 oracle; some batch holds more jobs than any one (side, type)
    class has, so it mixed sides; the setting is refused while jobs are queued."""
    jobs = _job_list() + [(40, api.C128, 300), (40, api.C64, 301), (60, api.C128, 302)]
    classes = {}
    for side, dtype, _ in jobs:
        classes[(side, dtype)] = classes.get((side, dtype), 0) + 1
    alone = api.Server(GRID, 1 << 30, slots=1, max_batch=1)
    alone.set_mixing(64)
    if arith128 is not None:
        alone.set_arith(api.C128, arith128)
    a_bufs, _ = _run(alone, jobs, cuda, one_at_a_time=True)
    alone.close()
    mix = api.Server(GRID, 1 << 30, slots=1, max_batch=16)
    mix.set_mixing(64)
    if arith128 is not None:
        mix.set_arith(api.C128, arith128)
    m_bufs, m_done = _run(mix, jobs, cuda, one_at_a_time=False)
    assert max(d["batch"] for d in m_done) > max(classes.values())
    srv = api.Server(GRID, 1 << 26, slots=1, max_batch=1)
    for (side, dtype, seed), a, m in zip(jobs, a_bufs, m_bufs):
        spec_held, out_held = _held(srv, side, dtype)
        assert np.array_equal(a[1].numpy()[spec_held], m[1].numpy()[spec_held]), (side, dtype)
        assert np.array_equal(a[2].numpy()[out_held], m[2].numpy()[out_held]), (side, dtype)
        g = _cube(side, dtype, seed).astype(np.complex128)
        e_spec, e_back = _check_job(srv, side, dtype, g, m[1], m[2])
        assert e_spec < TOL[dtype] and e_back < TOL[dtype], (side, dtype, e_spec, e_back)
    srv.close()
    import torch
    n_in, _, _ = mix.sizes(24, api.C128)
    x = torch.zeros(n_in, dtype=torch.complex128).pin_memory()
    for _ in range(4):
        mix.submit(24, api.C128, x.data_ptr())
    with pytest.raises(Exception):
        mix.set_mixing(0)
    mix.drain()
    mix.poll()
    mix.set_mixing(0)
    mix.close()
