"""The power-of-two stages' buffer swizzles (fft_pass.cuh), checked on the CPU: each is a bijection of the tile,
and under the shared-memory bank model (a wavefront serves 16 lanes x 8 bytes or 8 lanes x 16 bytes, 32 banks of
4 bytes) every stage's loads and the previous stage's stores take one wavefront per phase."""
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KERNELS = os.path.join(ROOT, "decomp_mpi_gb300", "csrc", "kernels")


@pytest.fixture(scope="module")
def dump():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "swizzle_dump")
        subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "--expt-relaxed-constexpr",
                        "-I" + os.path.join(ROOT, "include"),
                        "-I" + os.path.join(ROOT, "decomp_mpi_gb300", "csrc", "host"), "-I" + KERNELS,
                        os.path.join(ROOT, "tests", "host", "swizzle_dump.cu"), "-o", exe],
                       check=True, capture_output=True, timeout=600)
        out = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=120).stdout
    stages = []
    for line in out.splitlines():
        if line.startswith("stage"):
            kv = dict(t.split("=") for t in line.split()[1:])
            stages.append({k: int(v) for k, v in kv.items()})
        elif line.startswith("g"):
            stages[-1]["g"] = [int(t) for t in line.split()[1:]]
    return stages


def _wavefronts(addrs, w):
    per = 128 // w
    tot = 0
    for ph in range(0, len(addrs), per):
        banks = {}
        for a in addrs[ph:ph + per]:
            for k in range(w // 4):
                word = a // 4 + k
                banks.setdefault(word % 32, set()).add(word)
        tot += max(len(v) for v in banks.values())
    return tot


def test_swizzles_are_bijections(dump):
    for st in dump:
        if "g" in st:
            assert sorted(st["g"]) == list(range(len(st["g"]))), (st["es"], st["nf"], st["lp"])


def test_stage_accesses_are_conflict_free(dump):
    by = {}
    for st in dump:
        by.setdefault((st["es"], st["nf"]), []).append(st)
    for (es, nf), sts in by.items():
        tile = len(next(s["g"] for s in sts if "g" in s)) if any("g" in s for s in sts) else None
        for i, st in enumerate(sts):
            if "g" not in st:
                continue  # the first stage reads the line-padded staging buffer
            g, lp, r = st["g"], st["lp"], st["r"]
            prev = sts[i - 1]
            nl = tile // nf
            ideal = 32 * es // 128
            # this stage's loads
            nr, m = nf // r, nf // r // lp
            for w0 in range(0, min(nl * nr, 32 * 16), 32):
                for q in range(r):
                    xs = []
                    for b in range(w0, w0 + 32):
                        l, bb = divmod(b, nr)
                        j, k = divmod(bb, m)
                        xs.append(g[l * nf + j * r * m + q * m + k] * es)
                    assert _wavefronts(xs, es) == ideal, ("load", es, nf, lp, q)
            # the previous stage's stores into this buffer
            pr = prev["r"]
            pnr = nf // pr
            for w0 in range(0, min(nl * pnr, 32 * 16), 32):
                for s_ in range(pr):
                    xs = [g[(b // pnr) * nf + (b % pnr) + s_ * pnr] * es for b in range(w0, w0 + 32)]
                    assert _wavefronts(xs, es) == ideal, ("store", es, nf, lp, s_)
