"""TEST INFRASTRUCTURE (oracle).

ctypes wrappers for the oracle restatement (``_build/liboracle.so``) and,
when it has been built here, for the reference library compiled against the
project's shims (``_ref/libref.so``).  Only tests, the smoke check and the
benchmark's CPU-baseline leg import this module; the product never does.

Arrays are virtual-grid arrays: numpy arrays holding ``P`` consecutive
per-rank buffers of ``pitch`` elements each.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libref.so")
# the reference checkout, when one is present: DMG_REFERENCE_DIR names it (no default)
REF_SOURCES = os.environ.get("DMG_REFERENCE_DIR", "")

_c_ll = ctypes.c_longlong
_c_ll_p = ctypes.POINTER(ctypes.c_longlong)
_c_int_p = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p
_cp = ctypes.c_char_p


def build(ref: bool = True) -> None:
    """Compile the oracle restatement, and the reference library when its sources are present."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    if ref and REF_SOURCES and os.path.isdir(REF_SOURCES):
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + REF_SOURCES], check=True)


def _sig(lib, name, res, args):
    f = getattr(lib, name)
    f.restype = res
    f.argtypes = args
    return f


_oracle = None
_ref = None


def oracle_lib():
    global _oracle
    if _oracle is None:
        if not os.path.exists(ORACLE_LIB):
            build(ref=False)
        lib = ctypes.CDLL(ORACLE_LIB)
        _sig(lib, "oracle_decomp_info", ctypes.c_int, [ctypes.c_int, _cp, _c_ll_p, _c_int_p])
        _sig(lib, "oracle_global_offsets", ctypes.c_int, [ctypes.c_int, _cp, _c_ll, _c_ll_p])
        _sig(lib, "oracle_reshape", ctypes.c_int,
             [ctypes.c_int, _cp, _cp, ctypes.c_int, _c_ll, _c_ll, _vp, _vp, ctypes.c_int])
        _sig(lib, "oracle_reshape_plan", _vp, [ctypes.c_int, _cp, _cp, ctypes.c_int])
        _sig(lib, "oracle_reshape_exec", ctypes.c_int, [_vp, _vp, _c_ll, _vp, _c_ll, ctypes.c_int])
        _sig(lib, "oracle_reshape_free", None, [_vp])
        _sig(lib, "oracle_processor_grid", ctypes.c_int, [ctypes.c_int, ctypes.c_int, _c_int_p, _c_int_p])
        _sig(lib, "oracle_split_factors", ctypes.c_int,
             [ctypes.c_int, _cp, ctypes.c_int, _c_int_p, _c_int_p, _c_int_p, _c_int_p, _c_int_p, _cp, _cp,
              ctypes.c_int])
        _sig(lib, "oracle_split_fft", ctypes.c_int,
             [ctypes.c_int, _cp, ctypes.c_int, _c_int_p, _c_ll, _c_ll, _vp, _vp, ctypes.c_int, ctypes.c_int])
        _sig(lib, "oracle_split_plan", _vp, [ctypes.c_int, _cp, ctypes.c_int, _c_int_p, _c_ll])
        _sig(lib, "oracle_split_exec", ctypes.c_int, [_vp, _c_ll, _c_ll, _vp, _vp, ctypes.c_int, ctypes.c_int])
        _sig(lib, "oracle_split_extent", _c_ll, [_vp, ctypes.c_int])
        _sig(lib, "oracle_split_free", None, [_vp])
        _oracle = lib
    return _oracle


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def ref_lib():
    global _ref
    if _ref is None:
        lib = ctypes.CDLL(REF_LIB)
        _sig(lib, "ref_reshape", ctypes.c_int,
             [ctypes.c_int, _cp, _cp, ctypes.c_int, _c_ll, _c_ll, _vp, _vp, _c_int_p, _c_int_p, _cp, ctypes.c_int])
        _sig(lib, "ref_processor_grid", ctypes.c_int, [ctypes.c_int, ctypes.c_int, _c_int_p, _c_int_p])
        _sig(lib, "ref_time_step", ctypes.c_int,
             [ctypes.c_int, _cp, _cp, _cp, _c_ll, _c_ll, _c_ll, _c_ll, _vp, _vp, _vp, _vp, ctypes.c_int,
              ctypes.c_int, ctypes.POINTER(ctypes.c_double), _cp, ctypes.c_int])
        _sig(lib, "ref_split", ctypes.c_int,
             [ctypes.c_int, _cp, ctypes.c_int, _c_int_p, _c_ll, _c_ll, _vp, _vp, _c_int_p, _c_ll_p, ctypes.c_int,
              _cp, ctypes.c_int])
        _ref = lib
    return _ref


def _ints(vals):
    arr = (ctypes.c_int * max(1, len(vals)))(*vals)
    return arr


# ---------------------------------------------------------------- oracle

def decomp_info(P: int, spec: str):
    """Per-rank extents and proc_used of a decomposition (oracle; extent as reshape.c:47-324 computes it)."""
    ext = (ctypes.c_longlong * P)()
    pu = ctypes.c_int()
    rc = oracle_lib().oracle_decomp_info(P, spec.encode(), ext, ctypes.byref(pu))
    if rc:
        raise ValueError("oracle_decomp_info(%s) failed: %d" % (spec, rc))
    return list(ext), pu.value


def pitch_of(P: int, spec: str) -> int:
    ext, pu = decomp_info(P, spec)
    return max(ext[:pu])


def global_offsets(P: int, spec: str, pitch: int, shape) -> np.ndarray:
    """Element offset of each global coordinate (C order) in the virtual-grid array; -1 when unheld
    (rank r's buffer at r * pitch, getOffset of reshape.h:201 inside it)."""
    out = np.empty(int(np.prod(shape)), dtype=np.int64)
    rc = oracle_lib().oracle_global_offsets(P, spec.encode(), pitch, out.ctypes.data_as(_c_ll_p))
    if rc:
        raise ValueError("oracle_global_offsets failed: %d" % rc)
    return out.reshape(shape)


def reshape(P, src_spec, dst_spec, src: np.ndarray, src_pitch, dst: np.ndarray, dst_pitch, nthreads=8):
    """Reshape src into dst (in place in dst) following the reference's message algorithm
    (makeReshapePlan / runReshapePlan, reshape.c:351-492; typemaps as typelist.c:74-119 builds them)."""
    assert src.dtype == dst.dtype and src.flags.c_contiguous and dst.flags.c_contiguous
    rc = oracle_lib().oracle_reshape(P, src_spec.encode(), dst_spec.encode(), src.dtype.itemsize, src_pitch,
                                     dst_pitch, src.ctypes.data, dst.ctypes.data, nthreads)
    if rc:
        raise RuntimeError("oracle_reshape failed: %d" % rc)
    return dst


class ReshapePlanCPU:
    """Planned oracle reshape, so that timing covers only the run (like runReshapePlan)."""

    def __init__(self, P, src_spec, dst_spec, esize):
        self.h = oracle_lib().oracle_reshape_plan(P, src_spec.encode(), dst_spec.encode(), esize)
        if not self.h:
            raise ValueError("oracle_reshape_plan failed")

    def run(self, src, src_pitch, dst, dst_pitch, nthreads=8):
        rc = oracle_lib().oracle_reshape_exec(self.h, src.ctypes.data, src_pitch, dst.ctypes.data, dst_pitch,
                                              nthreads)
        if rc:
            raise RuntimeError("oracle_reshape_exec failed: %d" % rc)

    def __del__(self):
        if getattr(self, "h", None):
            oracle_lib().oracle_reshape_free(self.h)
            self.h = None


def processor_grid(P: int, tasks):
    """makeProcessorGrid (processor_grid.c:73-97) restated by the oracle."""
    g = (ctypes.c_int * len(tasks))()
    oracle_lib().oracle_processor_grid(P, len(tasks), _ints(tasks), g)
    return list(g)


def split_factors(P: int, start_spec: str, mode: int = 0, B=None):
    """(A, B, grid_a, grid_b, a_spec, b_spec) of the split plan the reference would build
    (makeSplitPlan / makeParallelPlan, split_fft.c:570-614 and 747-788)."""
    nd = start_spec.count("|") + 1
    A = (ctypes.c_int * nd)()
    Bo = (ctypes.c_int * nd)()
    ga = (ctypes.c_int * nd)()
    gb = (ctypes.c_int * nd)()
    asp = ctypes.create_string_buffer(1024)
    bsp = ctypes.create_string_buffer(1024)
    rc = oracle_lib().oracle_split_factors(P, start_spec.encode(), mode, _ints(B or [1] * nd), A, Bo, ga, gb, asp,
                                           bsp, 1024)
    if rc:
        raise ValueError("oracle_split_factors failed: %d" % rc)
    return list(A), list(Bo), list(ga), list(gb), asp.value.decode(), bsp.value.decode()


class SplitPlanCPU:
    """Planned oracle split FFT (the reference's algorithm on CPU threads: runSplitPlan, split_fft.c:622-744)."""

    def __init__(self, P, start_spec, work_len, mode=0, B=None):
        nd = start_spec.count("|") + 1
        self.P = P
        self.h = oracle_lib().oracle_split_plan(P, start_spec.encode(), mode, _ints(B or [1] * nd), work_len)
        if not self.h:
            raise ValueError("oracle_split_plan failed (workspace too small or bad factors)")
        self.work_len = work_len

    def extent(self, r):
        return oracle_lib().oracle_split_extent(self.h, r)

    def run(self, dat: np.ndarray, dat_pitch: int, work: np.ndarray, direction: int = -1, nthreads: int = 8):
        assert dat.dtype == np.complex128 and work.dtype == np.complex128
        rc = oracle_lib().oracle_split_exec(self.h, dat_pitch, self.work_len, dat.ctypes.data, work.ctypes.data,
                                            direction, nthreads)
        if rc:
            raise RuntimeError("oracle_split_exec failed: %d" % rc)

    def __del__(self):
        if getattr(self, "h", None):
            oracle_lib().oracle_split_free(self.h)
            self.h = None


# ---------------------------------------------------------------- reference (shim build)

def ref_reshape(P, src_spec, dst_spec, src: np.ndarray, src_pitch, dst: np.ndarray, dst_pitch):
    err = ctypes.create_string_buffer(512)
    rc = ref_lib().ref_reshape(P, src_spec.encode(), dst_spec.encode(), src.dtype.itemsize, src_pitch, dst_pitch,
                               src.ctypes.data, dst.ctypes.data, None, None, err, 512)
    if rc:
        raise RuntimeError("reference reshape failed: %s" % err.value.decode())
    return dst


def ref_extents(P, src_spec, dst_spec):
    ext = (ctypes.c_int * (2 * P))()
    pu = (ctypes.c_int * 2)()
    err = ctypes.create_string_buffer(512)
    rc = ref_lib().ref_reshape(P, src_spec.encode(), dst_spec.encode(), 1, 0, 0, None, None, ext, pu, err, 512)
    if rc:
        raise RuntimeError("reference plan failed: %s" % err.value.decode())
    return list(ext[0::2]), list(ext[1::2]), list(pu)


def ref_processor_grid(P, tasks):
    g = (ctypes.c_int * len(tasks))()
    ref_lib().ref_processor_grid(P, len(tasks), _ints(tasks), g)
    return list(g)


def ref_split(P, start_spec, dat: np.ndarray, dat_pitch, work_len, mode=0, B=None):
    """Run the reference's forward split FFT; returns (work, info, slot_map)."""
    nd = start_spec.count("|") + 1
    work = np.zeros(P * work_len, dtype=np.complex128)
    info = (ctypes.c_int * (8 * P))()
    slot = np.full(P * work_len, -1, dtype=np.int64)
    err = ctypes.create_string_buffer(512)
    d = np.ascontiguousarray(dat.copy())
    rc = ref_lib().ref_split(P, start_spec.encode(), mode, _ints(B or [1] * nd), dat_pitch, work_len, d.ctypes.data,
                             work.ctypes.data, info, slot.ctypes.data_as(_c_ll_p), 0, err, 512)
    if rc:
        raise RuntimeError("reference split failed: %s" % err.value.decode())
    info = np.array(list(info), dtype=np.int64).reshape(P, 8)
    return work, info, slot


def ref_time_step(P, specs, pitches, work_len, arrays, warmup, steps):
    """Wall seconds of `steps` benchmark steps (two reshapes, split FFT forward and backward) run by the
    reference's own code on P thread-ranks, after `warmup` steps."""
    err = ctypes.create_string_buffer(512)
    sec = ctypes.c_double()
    a0, a1, a2, work = arrays
    rc = ref_lib().ref_time_step(P, specs[0].encode(), specs[1].encode(), specs[2].encode(), pitches[0], pitches[1],
                                 pitches[2], work_len, a0.ctypes.data, a1.ctypes.data, a2.ctypes.data,
                                 work.ctypes.data, warmup, steps, ctypes.byref(sec), err, 512)
    if rc:
        raise RuntimeError("reference step failed: %s" % err.value.decode())
    return sec.value


# ---------------------------------------------------------------- FFT value oracle

def fftn64(x: np.ndarray, inverse: bool = False) -> np.ndarray:
    """FP64 n-dimensional DFT (forward sign -1, unnormalised) on the host: pocketfft through scipy on every
    host core when scipy is present, numpy's pocketfft otherwise."""
    x = np.asarray(x, dtype=np.complex128)
    try:
        import scipy.fft as sf
        f = sf.ifftn if inverse else sf.fftn
        return f(x, workers=os.cpu_count() or 1, norm="forward" if inverse else "backward")
    except ImportError:
        return np.fft.ifftn(x) * x.size if inverse else np.fft.fftn(x)


def gather_global(P, spec, arr: np.ndarray, pitch, shape) -> np.ndarray:
    """Global array (C order) from a virtual-grid array."""
    off = global_offsets(P, spec, pitch, shape)
    assert (off >= 0).all(), "decomposition does not hold every coordinate"
    return arr[off]


def scatter_global(P, spec, glob: np.ndarray, pitch, fill=0):
    """Virtual-grid array of a decomposition holding a global array."""
    off = global_offsets(P, spec, pitch, glob.shape)
    out = np.full(P * pitch, fill, dtype=glob.dtype)
    out[off.ravel()] = glob.ravel()
    return out


def split_expected_output(P, start_spec, glob_in: np.ndarray, work_len, mode=0, B=None):
    """Expected forward split-FFT output: numpy FP64 fftn placed in the reference's B layout
    (the slots runSplitPlan's second stage writes, split_fft.c:690-700; getTransformed, split_fft.c:615-621).

    Global slot s_i = k2_i + A_i*k1_i of the B decomposition holds frequency
    k_i = k1_i + B_i*k2_i.  Returns (work array, mask of held slots).
    """
    A, Bf, ga, gb, a_spec, b_spec = split_factors(P, start_spec, mode, B)
    F = fftn64(glob_in)
    shape = glob_in.shape
    use_first = all(a == 1 for a in A)
    out_spec = a_spec if use_first else b_spec
    idx = [np.arange(n) for n in shape]
    k = []
    for i, n in enumerate(shape):
        s = idx[i]
        k2 = s % A[i]
        k1 = s // A[i]
        k.append(k1 + Bf[i] * k2)
    ex = F[np.ix_(*k)]
    off = global_offsets(P, out_spec, work_len, shape)
    work = np.zeros(P * work_len, dtype=np.complex128)
    mask = np.zeros(P * work_len, dtype=bool)
    work[off.ravel()] = ex.ravel()
    mask[off.ravel()] = True
    return work, mask
