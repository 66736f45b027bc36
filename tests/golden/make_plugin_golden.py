"""Generate the golden fixture of the caller-defined plugin test from the reference itself.

Compiles tests/plugin/block_cyclic.c (a block-cyclic DimDecomp written against the plugin API only) and
tests/plugin/ref_plugin_driver.c against the reference's own headers, links them with the reference library
(oracle/_ref/libref.so: the reference's sources compiled unmodified against the project's MPI/FFTW shims),
and runs the reference's reshape block -> block_cyclic and its forward split FFT on the block-cyclic
decomposition, one thread per virtual rank.  Writes tests/golden/plugin_block_cyclic.npz.

    DMG_REFERENCE_DIR=<checkout> python -c "from oracle import oracle as O; O.build()"
    DMG_REFERENCE_DIR=<checkout> python tests/golden/make_plugin_golden.py
"""
from __future__ import annotations

import ctypes
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

CASE = {"g0": 2, "g1": 2, "L0": 24, "L1": 12, "L2": 10, "b": 3}


def build(ref_dir):
    out_dir = os.path.join(ROOT, "tests", "plugin", "_ref")
    os.makedirs(out_dir, exist_ok=True)
    lib = os.path.join(out_dir, "libplugin_ref.so")
    plug = os.path.join(ROOT, "tests", "plugin")
    subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-std=gnu99", "-w", "-I" + os.path.join(ROOT, "oracle", "shim"),
                    "-I" + ref_dir, os.path.join(plug, "block_cyclic.c"), os.path.join(plug, "ref_plugin_driver.c"),
                    "-L" + os.path.dirname(O.REF_LIB), "-lref", "-Wl,-rpath," + os.path.dirname(O.REF_LIB),
                    "-o", lib], check=True)
    return lib


def main():
    ref_dir = os.environ.get("DMG_REFERENCE_DIR", "")
    if not ref_dir or not os.path.isdir(ref_dir) or not O.ref_available():
        sys.exit("needs DMG_REFERENCE_DIR and oracle/_ref/libref.so (see the module docstring)")
    lib = ctypes.CDLL(build(ref_dir))
    f = lib.plugin_ref_run
    vp, ll = ctypes.c_void_p, ctypes.c_longlong
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int] * 6 + [ll, ll, ll, vp, vp, vp, vp, vp, ctypes.c_char_p, ctypes.c_int]
    c = CASE
    P = c["g0"] * c["g1"]
    N = c["L0"] * c["L1"] * c["L2"]
    err = ctypes.create_string_buffer(512)
    ext = np.zeros(3 * P, np.int32)
    rc = f(c["g0"], c["g1"], c["L0"], c["L1"], c["L2"], c["b"], 0, 0, 0, None, None, None, None,
           ext.ctypes.data, err, 512)
    assert rc == 0, err.value
    sp, dp = int(ext[0::3].max()), int(ext[1::3].max())
    wl = 2 * N
    rng = np.random.default_rng(21)
    src = rng.uniform(-1, 1, P * sp) + 1j * rng.uniform(-1, 1, P * sp)
    dst = np.zeros(P * dp, np.complex128)
    work = np.zeros(P * wl, np.complex128)
    slot = np.full(P * wl, -1, np.int64)
    rc = f(c["g0"], c["g1"], c["L0"], c["L1"], c["L2"], c["b"], sp, dp, wl, src.ctypes.data, dst.ctypes.data,
           work.ctypes.data, slot.ctypes.data, ext.ctypes.data, err, 512)
    assert rc == 0, err.value
    meta = dict(CASE, src_pitch=sp, dst_pitch=dp, work_len=wl, split_extent=int(ext[2::3].max()))
    out = os.path.join(HERE, "plugin_block_cyclic.npz")
    # dst is the reshape's output and the split FFT's input; the reference's split FFT leaves dat as scratch,
    # so the reshape output is recorded before the transform by re-running the reshape alone
    dst_only = np.zeros(P * dp, np.complex128)
    rc = f(c["g0"], c["g1"], c["L0"], c["L1"], c["L2"], c["b"], sp, dp, wl, src.ctypes.data, dst_only.ctypes.data,
           None, None, None, err, 512)
    assert rc == 0, err.value
    np.savez_compressed(out, meta=json.dumps(meta), src=src, reshaped=dst_only, work=work, slot=slot)
    print("wrote", out, meta)


if __name__ == "__main__":
    main()
