"""The request server's device arena (decomp_mpi_gb300/csrc/host/arena.h), compiled alone on the CPU and driven
through tests/host/arena_check.c: first-fit placement at 256-byte granularity, freed blocks merged with their
neighbours, the bytes in use accounted, checked step by step against a plain model of the same policy."""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ALIGN = 256


@pytest.fixture(scope="module")
def harness():
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "arena_check")
        subprocess.run([cc, "-std=gnu11", "-O1", "-Wall", "-I" + os.path.join(ROOT, "decomp_mpi_gb300", "csrc", "host"),
                        os.path.join(ROOT, "tests", "host", "arena_check.c"), "-o", exe], check=True,
                       capture_output=True, timeout=120)
        p = subprocess.Popen([exe], stdin=subprocess.PIPE, stdout=subprocess.PIPE, text=True)

        def cmd(line):
            p.stdin.write(line + "\n")
            p.stdin.flush()
            return p.stdout.readline().strip()
        yield cmd
        p.stdin.close()
        p.wait(timeout=30)


class Model:
    """First fit over an offset-sorted free list with merging of neighbours."""

    def __init__(self, size):
        self.size = size // ALIGN * ALIGN
        self.free = [(0, self.size)] if self.size else []
        self.used = 0

    @staticmethod
    def up(b):
        b = max(b, 1)
        return (b + ALIGN - 1) // ALIGN * ALIGN

    def alloc(self, b):
        b = self.up(b)
        for i, (o, s) in enumerate(self.free):
            if s >= b:
                self.free[i] = (o + b, s - b)
                if s == b:
                    del self.free[i]
                self.used += b
                return o
        return -1

    def release(self, o, b):
        b = self.up(b)
        self.free.append((o, b))
        self.free.sort()
        merged = []
        for fo, fs in self.free:
            if merged and merged[-1][0] + merged[-1][1] == fo:
                merged[-1] = (merged[-1][0], merged[-1][1] + fs)
            else:
                merged.append((fo, fs))
        self.free = merged
        self.used -= b

    def state(self):
        return "used %d free%s" % (self.used, "".join(" %d:%d" % f for f in self.free))


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_arena_matches_first_fit_model(harness, seed):
    rng = np.random.default_rng(seed)
    size = 1 << 20
    assert int(harness("i %d" % (size + 77))) == size  # rounded down to the alignment
    model = Model(size + 77)
    live = []
    for step in range(3000):
        if live and (rng.random() < 0.45 or len(live) > 60):
            o, b = live.pop(int(rng.integers(0, len(live))))
            assert harness("f %d %d" % (o, b)) == "0"
            model.release(o, b)
        else:
            b = int(rng.choice([1, 255, 256, 257, 1000, 4096, 30000, 100000]))
            got = int(harness("a %d" % b))
            assert got == model.alloc(b), step
            if got >= 0:
                assert got % ALIGN == 0 and got + Model.up(b) <= size
                live.append((got, b))
        if step % 50 == 0:
            assert harness("s") == model.state(), step
    # the live blocks never overlap
    spans = sorted((o, o + Model.up(b)) for o, b in live)
    assert all(a[1] <= b[0] for a, b in zip(spans, spans[1:]))
    for o, b in live:
        assert harness("f %d %d" % (o, b)) == "0"
    assert harness("s") == "used 0 free 0:%d" % size  # everything merged back into one block


def test_arena_exhaustion_and_reuse(harness):
    assert int(harness("i %d" % (4 * ALIGN))) == 4 * ALIGN
    offs = [int(harness("a %d" % ALIGN)) for _ in range(4)]
    assert offs == [0, ALIGN, 2 * ALIGN, 3 * ALIGN]
    assert int(harness("a 1")) == -1
    assert harness("f %d %d" % (ALIGN, ALIGN)) == "0"
    assert harness("f %d %d" % (2 * ALIGN, ALIGN)) == "0"
    assert harness("s") == "used %d free %d:%d" % (2 * ALIGN, ALIGN, 2 * ALIGN)
    assert int(harness("a %d" % (2 * ALIGN))) == ALIGN  # the two freed neighbours serve one larger block
