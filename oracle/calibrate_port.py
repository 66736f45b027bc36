"""TEST INFRASTRUCTURE: time the oracle's CPU port of the benchmark step against the reference's own code.

The reference (reshape.c, split_fft.c and the decomposition sources, compiled unmodified against the
project's MPI/FFTW shims into _ref/libref.so) can only be built where its checkout is present, so the
benchmark's CPU arm runs the oracle's step-for-step restatement instead.  This script runs both on the same
host and the same workload (the benchmark's chain and split FFT forward + backward on the 8x8 virtual grid,
n^3 complex128) and prints their mean step times: the ratio says how far the port's timing stands from the
reference's.  Both use the oracle's FP64 FFT for the FFTW stages.

    DMG_REFERENCE_DIR=<checkout> python -c "from oracle import oracle as O; O.build()"
    python oracle/calibrate_port.py 128 256
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path[0] = os.path.dirname(HERE)  # the repository root, not this folder

from oracle import oracle as O  # noqa: E402

P = 64


def specs(n, g=8):
    blk = "packed:block(%d,%d)|block(%d,%d)|local(%d)" % (n, g, n, g, n)
    rot = "packed:rotate(1,block(%d,%d))|rotate(%d,block(%d,%d))|local(%d)" % (n, g, n // 3, n, g, n)
    frv = "packed:frev(16,%d,block(%d,%d))|frev(%d,16,block(%d,%d))|local(%d)" % (n // 16, n, g, n // 16, n, g, n)
    return blk, rot, frv


def main(sizes, steps=3):
    threads = os.cpu_count() or 1
    for n in sizes:
        s = specs(n)
        p = [O.pitch_of(P, x) for x in s]
        wl = 4 * n ** 3 // P + 64
        rng = np.random.default_rng(1)
        a0 = rng.uniform(-1, 1, P * p[0]) + 1j * rng.uniform(-1, 1, P * p[0])
        a1 = np.zeros(P * p[1], np.complex128)
        a2 = np.zeros(P * p[2], np.complex128)
        work = np.zeros(P * wl, np.complex128)
        r1 = O.ReshapePlanCPU(P, s[0], s[1], 16)
        r2 = O.ReshapePlanCPU(P, s[1], s[2], 16)
        fft = O.SplitPlanCPU(P, s[2], wl)

        def port_step():
            r1.run(a0, p[0], a1, p[1], threads)
            r2.run(a1, p[1], a2, p[2], threads)
            fft.run(a2, p[2], work, -1, threads)
            fft.run(a2, p[2], work, +1, threads)

        port_step()
        t = time.perf_counter()
        for _ in range(steps):
            port_step()
        port = (time.perf_counter() - t) / steps
        ref = O.ref_time_step(P, s, p, wl, (a0, a1, a2, work), 1, steps) / steps
        print("n=%d: port %.1f ms per step on %d threads, reference %.1f ms per step on %d thread-ranks, "
              "port / reference = %.2f" % (n, 1e3 * port, threads, 1e3 * ref, P, port / ref), flush=True)


if __name__ == "__main__":
    main([int(x) for x in sys.argv[1:]] or [128, 256])
