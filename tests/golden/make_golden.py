"""Generate the golden fixtures from the reference itself.

Runs the reference's own C sources (built unmodified against the project's
MPI/FFTW shims into oracle/_ref/libref.so by ``make -C oracle ref``) on the
cases below and stores inputs and outputs under tests/golden/.  The
reference ships no golden data; these fixtures pin the oracle restatement
(tests/test_oracle_golden.py) and the GPU path.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import zlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402

# (name, P, src spec, dst spec, numpy dtype).  The test.c scenarios
# (test.c:118-215) use int and value = global linear index.
RESHAPE_CASES = [
    ("testc_orig_to_new", 4, "axes:single(10,0,1)@1,1|single(10,0,4)@10,1",
     "axes:rotate(2,local(10))@1,1|rotate(1,block(10,4))@10,1", "int32"),
    ("testc_orig_to_d2", 4, "axes:single(10,0,1)@1,1|single(10,0,4)@10,1",
     "axes:rotate(3,block(10,2))@1,1|rotate(3,block(10,2))@5,2", "int32"),
    ("testc_new_to_d2", 4, "axes:rotate(2,local(10))@1,1|rotate(1,block(10,4))@10,1",
     "axes:rotate(3,block(10,2))@1,1|rotate(3,block(10,2))@5,2", "int32"),
    ("testc_orig_to_new_p6", 6, "axes:single(10,0,1)@1,1|single(10,0,6)@10,1",
     "axes:rotate(2,local(10))@1,1|rotate(1,block(10,6))@10,1", "int32"),
    ("pencil_x_to_y", 4, "packed:block(16,2)|block(16,2)|local(16)", "packed:block(16,2)|local(16)|block(16,2)",
     "complex128"),
    ("pencil_y_to_z", 4, "packed:block(16,2)|local(16)|block(16,2)", "packed:local(16)|block(16,2)|block(16,2)",
     "complex128"),
    ("uneven_block_rotate", 6, "packed:block(10,3)|block(7,2)|local(9)",
     "packed:rotate(3,block(10,2))|local(7)|block(9,3)", "int64"),
    ("interleave", 4, "packed:block(8,2)|block(12,2)|local(16)",
     "packed:interleave(block(4,2),2)|local(12)|interleave(block(4,2),4)", "int64"),
    ("factor_reverse", 16, "packed:block(16,4)|block(12,4)|local(20)",
     "packed:local(16)|rotate(5,block(12,4))|frev(4,5,block(20,4))", "complex64"),
    ("chain_block_rotate_frev", 16, "packed:rotate(3,block(16,4))|rotate(7,block(16,4))|local(16)",
     "packed:frev(4,4,block(16,4))|local(16)|frev(2,8,block(16,4))", "complex128"),
    ("single_to_block_2d", 5, "packed:block(11,5)|local(6)", "packed:local(11)|block(6,5)", "float32"),
    ("int8_elements", 4, "packed:block(12,2)|block(10,2)", "packed:block(12,4)|local(10)", "int8"),
    ("struct24_elements", 4, "packed:block(6,2)|block(10,2)", "packed:local(6)|block(10,4)", "V24"),
]

# (name, P, start spec, global shape, mode, B)
SPLIT_CASES = [
    ("split_8x12x16_p4", 4, "packed:local(8)|block(12,2)|block(16,2)", (8, 12, 16), 0, None),
    ("split_16cube_p4", 4, "packed:block(16,2)|block(16,2)|local(16)", (16, 16, 16), 0, None),
    ("split_12x10x6_p6", 6, "packed:block(12,3)|block(10,2)|local(6)", (12, 10, 6), 0, None),
    ("slab_8x12x16_p4", 4, "packed:local(8)|block(12,2)|block(16,2)", (8, 12, 16), 1, None),
    ("given_B_8x12x16_p4", 4, "packed:local(8)|block(12,2)|block(16,2)", (8, 12, 16), 2, [1, 12, 16]),
    ("split_16cube_p8", 8, "packed:block(16,2)|block(16,4)|local(16)", (16, 16, 16), 0, None),
]

GRID_CASES = [
    (4, [10, 10, 10]), (64, [16, 16, 16]), (64, [32, 32, 32]), (16, [6, 10, 10]), (6, [3, 2, 2]),
    (6, [4, 5, 3]), (12, [8, 12, 16]), (7, [5, 5, 5]), (64, [512, 512, 512]), (16, [48, 48, 48]),
    (16, [8, 6, 10]), (1024, [32, 32]),
]


def _dtype(name):
    return np.dtype(name)


def make_reshape(name, P, s, d, dt):
    dt = _dtype(dt)
    sp = O.pitch_of(P, s)
    dp = O.pitch_of(P, d)
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    nbytes = P * sp * dt.itemsize
    src = np.frombuffer(rng.integers(0, 256, nbytes, dtype=np.uint8).tobytes(), dtype=dt).copy()
    fill = np.frombuffer(np.full(P * dp * dt.itemsize, 0xA5, np.uint8).tobytes(), dtype=dt).copy()
    out = fill.copy()
    O.ref_reshape(P, s, d, src, sp, out, dp)
    return dict(src=src.view(np.uint8), out=out.view(np.uint8), fill=fill.view(np.uint8)), dict(
        P=P, src_spec=s, dst_spec=d, dtype=dt.str, esize=dt.itemsize, src_pitch=sp, dst_pitch=dp)


def make_split(name, P, spec, shape, mode, B):
    rng = np.random.default_rng(7)
    glob = rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)
    dp = O.pitch_of(P, spec)
    dat = O.scatter_global(P, spec, glob, dp)
    work_len = 2 * int(np.prod(shape))
    work, info, slot = O.ref_split(P, spec, dat, dp, work_len, mode, B)
    return dict(dat=dat, work=work, slot=slot, info=info, glob=glob), dict(
        P=P, spec=spec, shape=list(shape), mode=mode, B=B, dat_pitch=dp, work_len=work_len)


def main():
    if not O.ref_available():
        O.build(ref=True)
    meta = {"reshape": {}, "split": {}, "grid": []}
    for name, P, s, d, dt in RESHAPE_CASES:
        arrays, m = make_reshape(name, P, s, d, dt)
        np.savez_compressed(os.path.join(HERE, "reshape_%s.npz" % name), **arrays)
        meta["reshape"][name] = m
    for name, P, spec, shape, mode, B in SPLIT_CASES:
        arrays, m = make_split(name, P, spec, shape, mode, B)
        np.savez_compressed(os.path.join(HERE, "split_%s.npz" % name), **arrays)
        meta["split"][name] = m
    for P, tasks in GRID_CASES:
        meta["grid"].append({"P": P, "tasks": tasks, "grid": O.ref_processor_grid(P, tasks)})
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print("wrote", len(meta["reshape"]), "reshape,", len(meta["split"]), "split,", len(meta["grid"]), "grid cases")


if __name__ == "__main__":
    main()
