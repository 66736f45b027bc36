"""Python mirror of the reference's reshape / split-FFT interface.

Thin objects over the C-ABI library (``libdecomp_gb300.so``).  The names
follow the reference (reshape.h, split_fft.h): a :class:`Comm` is a virtual
communicator over ``P`` virtual ranks, a :class:`Decomp` a decomposition of
a global array over them, a :class:`ReshapePlan` the move between two of
them.  Device buffers are passed as raw pointers (``tensor.data_ptr()``) to
virtual-grid arrays: rank ``r``'s local buffer starts at element
``r * pitch``.
"""
from __future__ import annotations

import ctypes
import re

from ._lib import DecompError, check, last_error, load

__all__ = [
    "Comm", "Decomp", "ReshapePlan", "SplitPlan", "decomp_from_spec", "processor_grid", "DecompError",
    "propose_parallel_plan", "build_parallel_plan",
    "FFTW_FORWARD", "FFTW_BACKWARD", "C128", "C64",
]

FFTW_FORWARD = -1
FFTW_BACKWARD = 1
C128 = 0
C64 = 1
ARITH_FP64 = 0
ARITH_FP32 = 1
ARITH_DF = 2
ARITH_TC16 = 3
SCHEDULE_AUTO = 0
SCHEDULE_LINES = 1
SCHEDULE_SPLIT = 2
RADIX_FIXED = 0
RADIX_PLAN8 = 1
RADIX_PLAN4 = 2
# SearchFlags of split_fft.h
NO_FLAGS = 0x00
PREFER_LARGE_FFT = 0x01
PREFER_STAGE1 = 0x02
FORCE_USE_FIRST = 0x04


class _DecompStruct(ctypes.Structure):
    _fields_ = [("ndim", ctypes.c_int), ("comm", ctypes.c_void_p), ("proc_used", ctypes.c_int),
                ("dims", ctypes.c_void_p)]


class Comm:
    """Virtual communicator of ``nranks`` virtual ranks (replaces the MPI_Comm that reshape.h:77 keeps in
    every AxisDecomp)."""

    def __init__(self, nranks: int):
        self.lib = load()
        self.h = self.lib.dmg_comm_create(int(nranks))
        if not self.h:
            raise DecompError("dmg_comm_create(%d): %s" % (nranks, last_error()))
        self.size = int(nranks)
        self._children = []

    def set_view_rank(self, rank: int):
        check(self.lib.dmg_comm_set_rank(self.h, int(rank)), "dmg_comm_set_rank")

    def __del__(self):
        # descriptors made on the communicator hold a pointer to it; free it last
        if getattr(self, "h", None) and not self._children:
            self.lib.dmg_comm_free(self.h)
            self.h = None


# ------------------------------------------------------------------ DimDecomp builders

def _dim(kind, *args):
    lib = load()
    f = {
        "block": lib.makeBlockDecomp,
        "blockf": lib.makeBlockDecompWithFactor,
        "local": lib.makeLocalDecomp,
        "single": lib.makeSingleDecomp,
    }[kind]
    h = f(*[int(a) for a in args])
    if not h:
        raise DecompError("make %s%r failed" % (kind, args))
    return h


def _wrap(kind, nested, *args):
    """Decorators clone `nested`; the caller's copy is freed here."""
    lib = load()
    if kind == "rotate":
        h = lib.makeRotatedDecomp(int(args[0]), nested)
    elif kind == "interleave":
        h = lib.makeInterleaveDecomp(nested, int(args[0]))
    elif kind == "frev":
        h = lib.makeFactorReverseDecomp(int(args[0]), int(args[1]), nested)
    else:
        raise ValueError(kind)
    lib.freeDimDecomp(nested)
    if not h:
        raise DecompError("make %s%r failed" % (kind, args))
    return h


_TOKEN = re.compile(r"\s*([A-Za-z_]+|-?\d+|[(),|@:])")


def _tokens(s):
    pos, out = 0, []
    while pos < len(s):
        m = _TOKEN.match(s, pos)
        if not m:
            if s[pos:].strip() == "":
                break
            raise ValueError("bad decomposition spec near %r" % s[pos:])
        out.append(m.group(1))
        pos = m.end()
    return out


class _SpecParser:
    """Parser of decomposition spec strings (see decomp_from_spec)."""

    def __init__(self, text):
        self.t = _tokens(text)
        self.i = 0

    def peek(self):
        return self.t[self.i] if self.i < len(self.t) else None

    def take(self, want=None):
        tok = self.peek()
        if tok is None or (want is not None and tok != want):
            raise ValueError("spec: expected %r got %r" % (want, tok))
        self.i += 1
        return tok

    def num(self):
        return int(self.take())

    def dim(self):
        kind = self.take()
        self.take("(")
        if kind in ("block", "local", "single", "blockf"):
            n = {"block": 2, "local": 1, "single": 3, "blockf": 3}[kind]
            args = [self.num()]
            for _ in range(n - 1):
                self.take(",")
                args.append(self.num())
            self.take(")")
            return _dim(kind, *args)
        if kind == "rotate":
            r = self.num()
            self.take(",")
            nested = self.dim()
            self.take(")")
            return _wrap("rotate", nested, r)
        if kind == "interleave":
            nested = self.dim()
            self.take(",")
            b = self.num()
            self.take(")")
            return _wrap("interleave", nested, b)
        if kind == "frev":
            a = self.num()
            self.take(",")
            b = self.num()
            self.take(",")
            nested = self.dim()
            self.take(")")
            return _wrap("frev", nested, a, b)
        raise ValueError("spec: unknown decomposition %r" % kind)


class Decomp:
    """An N-D decomposition, the reference's Decomp (reshape.h:134-142; owns its C handle)."""

    def __init__(self, comm: Comm, handle):
        if not handle:
            raise DecompError("decomposition failed: %s" % last_error())
        self.comm = comm
        self.h = handle
        self.lib = load()
        comm._children.append(self)

    @property
    def _s(self):
        return _DecompStruct.from_address(self.h)

    @property
    def ndim(self) -> int:
        return self._s.ndim

    @property
    def proc_used(self) -> int:
        return self._s.proc_used

    def extent(self) -> int:
        """Largest per-rank extent: the default pitch of a virtual-grid array."""
        return int(self.lib.extent64(self.h))

    def rank_extent(self, r: int) -> int:
        return int(self.lib.rankExtent64(self.h, int(r)))

    def owner(self, pos) -> int:
        arr = (ctypes.c_int * len(pos))(*pos)
        return self.lib.ownerRank(self.h, arr)

    def global_offset(self, pos, pitch=None) -> int:
        arr = (ctypes.c_int * len(pos))(*pos)
        return int(self.lib.globalOffset64(self.h, arr, int(self.extent() if pitch is None else pitch)))

    def free(self):
        if self.h:
            self.lib.freeDecomp(self.h)
            self.h = None
            if self in self.comm._children:
                self.comm._children.remove(self)


def decomp_from_spec(comm: Comm, spec: str) -> Decomp:
    """Build a Decomp from a spec string.

    ``packed:d0|d1|...`` (makePackedDecomp) or
    ``axes:d0@stride,rank_stride|...`` (makeAxisDecomp + makeDecomp), each
    ``d`` one of ``block(len,procs)``, ``blockf(len,factor,procs)``,
    ``local(len)``, ``single(len,rank,procs)``, ``rotate(r,d)``,
    ``interleave(d,B)``, ``frev(A,B,d)``.
    """
    lib = load()
    spec = spec.strip()
    if spec.startswith("packed:"):
        p = _SpecParser(spec[len("packed:"):])
        dims = [p.dim()]
        while p.peek() == "|":
            p.take("|")
            dims.append(p.dim())
        if p.peek() is not None:
            raise ValueError("trailing spec text")
        arr = (ctypes.c_void_p * len(dims))(*dims)
        return Decomp(comm, lib.makePackedDecomp(comm.h, len(dims), arr))
    if spec.startswith("axes:"):
        p = _SpecParser(spec[len("axes:"):])
        axes = []
        while True:
            d = p.dim()
            p.take("@")
            stride = p.num()
            p.take(",")
            rs = p.num()
            a = lib.makeAxisDecomp(comm.h, d, stride, rs)
            if not a:
                raise DecompError("makeAxisDecomp: %s" % last_error())
            axes.append(a)
            if p.peek() != "|":
                break
            p.take("|")
        arr = (ctypes.c_void_p * len(axes))(*axes)
        return Decomp(comm, lib.makeDecomp(len(axes), arr))
    raise ValueError("spec must start with packed: or axes:")


class ReshapePlan:
    """makeReshapePlan / runReshapePlan (reshape.h:272-301, reshape.c:351-492) on the virtual grid."""

    def __init__(self, comm: Comm, elem_bytes: int, src: Decomp, dest: Decomp):
        self.lib = load()
        self.comm, self.src, self.dest = comm, src, dest
        self.h = self.lib.makeReshapePlan(comm.h, int(elem_bytes), src.h, dest.h)
        if not self.h:
            raise DecompError("makeReshapePlan: %s" % last_error())
        self.elem_bytes = int(elem_bytes)

    def set_pitch(self, src_pitch=0, dest_pitch=0):
        check(self.lib.dmg_reshape_set_pitch(self.h, int(src_pitch), int(dest_pitch)), "dmg_reshape_set_pitch")

    @property
    def src_pitch(self) -> int:
        return int(self.lib.dmg_reshape_pitch(self.h, 0))

    @property
    def dest_pitch(self) -> int:
        return int(self.lib.dmg_reshape_pitch(self.h, 1))

    @property
    def bytes_moved(self) -> int:
        return int(self.lib.dmg_reshape_bytes(self.h))

    @property
    def elements(self) -> int:
        return int(self.lib.dmg_reshape_elements(self.h))

    @property
    def launches(self) -> int:
        return int(self.lib.dmg_reshape_launches(self.h))

    def describe(self) -> str:
        return self.lib.dmg_reshape_describe(self.h).decode()

    def run(self, src_ptr: int, dest_ptr: int, stream=None):
        """Enqueue the reshape on `stream` (a CUDA stream handle, int; None = default stream)."""
        check(self.lib.dmg_reshape_run(self.h, ctypes.c_void_p(src_ptr), ctypes.c_void_p(dest_ptr),
                                       ctypes.c_void_p(stream or 0)), "runReshapePlan")

    def check_bounds(self, type_size: int, src_len: int, dest_len: int) -> int:
        return self.lib.checkReshapePlanBounds(self.h, int(type_size), int(src_len), int(dest_len))

    def free(self):
        if self.h:
            self.lib.freeReshapePlan(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def reshape_group(plans, srcs, dsts, stream=None):
    """dmg_reshape_run_group: several reshapes (any plans) in as few launches as their kernels allow."""
    n = len(plans)
    P = (ctypes.c_void_p * n)(*[p.h for p in plans])
    S = (ctypes.c_void_p * n)(*srcs)
    D = (ctypes.c_void_p * n)(*dsts)
    check(load().dmg_reshape_run_group(n, P, S, D, ctypes.c_void_p(stream or 0)), "dmg_reshape_run_group")


def _int_array(vals):
    return (ctypes.c_int * len(vals))(*[int(v) for v in vals])


def processor_grid(comm: Comm, tasks):
    """makeProcessorGrid (processor_grid.c:73-97): the reference's grid search over the communicator's ranks."""
    lib = load()
    ptr = lib.makeProcessorGrid(comm.h, len(tasks), _int_array(tasks))
    if not ptr:
        raise DecompError("makeProcessorGrid: %s" % last_error())
    out = [ptr[i] for i in range(len(tasks))]
    ctypes.CDLL(None).free(ctypes.cast(ptr, ctypes.c_void_p))
    return out


class _SplitStruct(ctypes.Structure):
    _fields_ = [("comm", ctypes.c_void_p), ("A_factors", ctypes.POINTER(ctypes.c_int)), ("A", ctypes.c_void_p),
                ("B", ctypes.c_void_p), ("B_flipped", ctypes.c_void_p), ("src", ctypes.c_void_p),
                ("work", ctypes.c_void_p), ("extent", ctypes.c_int), ("plan_a", ctypes.c_void_p),
                ("plan_b", ctypes.c_void_p), ("plan_a_back", ctypes.c_void_p), ("plan_b_back", ctypes.c_void_p),
                ("start_to_A", ctypes.c_void_p), ("A_to_start", ctypes.c_void_p), ("A_to_B", ctypes.c_void_p),
                ("B_to_A", ctypes.c_void_p), ("twiddle", ctypes.c_void_p),
                ("times", ctypes.POINTER(ctypes.c_double)), ("impl", ctypes.c_void_p)]


class _BorrowedDecomp(Decomp):
    """A Decomp owned by a plan (not freed from Python)."""

    def __init__(self, comm, handle):
        self.comm, self.h, self.lib = comm, handle, load()

    def free(self):
        pass


class SplitPlan:
    """Split 3D FFT plan (makeSplitPlan / makeParallelPlan / autotuneParallelPlan, split_fft.h:10-63).

    ``dat`` and ``work`` are device pointers; ``length`` is the per-rank
    workspace length in elements.  ``dtype`` is C128 (FP64) or C64 (FP32).
    """

    def __init__(self, start: Decomp, dat_ptr: int, length: int, work_ptr: int, slab: int = 0, B=None,
                 dtype: int = C128, autotune: bool = False, arith=None, schedule=None, full_grid: bool = False):
        self.lib = load()
        self.start = start
        if autotune and dtype == C128 and not full_grid:
            h = self.lib.autotuneParallelPlan(start.h, ctypes.c_void_p(dat_ptr), int(length), ctypes.c_void_p(work_ptr))
        elif autotune:
            h = self.lib.dmg_autotuneParallelPlanTyped(start.h, ctypes.c_void_p(dat_ptr), int(length),
                                                       ctypes.c_void_p(work_ptr), int(dtype), int(bool(full_grid)))
        elif B is not None:
            h = self.lib.dmg_makeParallelPlanTyped(start.h, _int_array(B), ctypes.c_void_p(dat_ptr), int(length),
                                                   ctypes.c_void_p(work_ptr), int(dtype))
        else:
            h = self.lib.dmg_makeSplitPlanTyped(int(slab), start.h, ctypes.c_void_p(dat_ptr), int(length),
                                                ctypes.c_void_p(work_ptr), int(dtype))
        if not h:
            raise DecompError("split plan: %s" % last_error())
        self.h = h
        self.length = int(length)
        self.dtype = dtype
        if arith is not None:
            self.set_arith(arith)
        if schedule is not None:
            self.set_schedule(schedule)

    def set_arith(self, arith):
        """ARITH_DF (default for complex128) or ARITH_FP64; ARITH_FP32 (default for complex64) or ARITH_TC16
        (the 1024-point passes' DFTs on the tensor cores) for complex64."""
        check(self.lib.dmg_split_set_arith(self.h, int(arith)), "dmg_split_set_arith")

    def device_status(self):
        """0 when every tensor-core pass completed its products (reads the device word after the queued work)."""
        st = self.lib.dmg_split_device_status(self.h)
        if st < 0:
            raise DecompError("dmg_split_device_status: %s" % last_error())
        return st

    @property
    def arith(self):
        return self.lib.dmg_split_get_arith(self.h)

    def run_batch(self, direction, dats, works, scales=None, stream=None):
        """dmg_split_run_batch: one run over several (dat, work) device arrays; scales: device int pointers
        (needed for double-float plans)."""
        n = len(dats)
        D = (ctypes.c_void_p * n)(*[ctypes.c_void_p(x) for x in dats])
        W = (ctypes.c_void_p * n)(*[ctypes.c_void_p(x) for x in works])
        S = (ctypes.c_void_p * n)(*[ctypes.c_void_p(x) for x in (scales or [0] * n)])
        check(self.lib.dmg_split_run_batch(self.h, int(direction), ctypes.c_void_p(stream or 0), n, D, W, S),
              "dmg_split_run_batch")

    @property
    def extent64(self):
        return self.lib.dmg_split_extent64(self.h)

    def set_schedule(self, schedule):
        """SCHEDULE_AUTO, SCHEDULE_LINES (one pass per dimension) or SCHEDULE_SPLIT (two per dimension)."""
        check(self.lib.dmg_split_set_schedule(self.h, int(schedule)), "dmg_split_set_schedule")

    @property
    def schedule(self):
        return self.lib.dmg_split_get_schedule(self.h)

    def set_tile(self, values):
        """Values per pass tile (0: the default)."""
        check(self.lib.dmg_split_set_tile(self.h, int(values)), "dmg_split_set_tile")

    @property
    def tile(self):
        return self.lib.dmg_split_get_tile(self.h)

    def set_radix(self, radix):
        """RADIX_FIXED (compile-time radix schedules), RADIX_PLAN8 or RADIX_PLAN4 (the plan's radices)."""
        check(self.lib.dmg_split_set_radix(self.h, int(radix)), "dmg_split_set_radix")

    @property
    def radix(self):
        return self.lib.dmg_split_get_radix(self.h)

    @property
    def _s(self):
        return _SplitStruct.from_address(self.h)

    @property
    def ndim(self):
        return self.start.ndim

    @property
    def A_factors(self):
        s = self._s
        return [s.A_factors[i] for i in range(self.ndim)]

    @property
    def extent(self):
        return self._s.extent

    def decomp_A(self):
        return _BorrowedDecomp(self.start.comm, self._s.A)

    def decomp_B(self):
        return _BorrowedDecomp(self.start.comm, self._s.B) if self._s.B else None

    def transformed(self):
        """getTransformed(): the reference's descriptor (right only when A_i == B_i)."""
        return _BorrowedDecomp(self.start.comm, self.lib.getTransformed(self.h))

    def transformed_exact(self):
        """getTransformedExact(): a new Decomp owned by the caller."""
        return Decomp(self.start.comm, self.lib.getTransformedExact(self.h))

    def set_buffers(self, dat_ptr, work_ptr):
        check(self.lib.dmg_split_set_buffers(self.h, ctypes.c_void_p(dat_ptr), ctypes.c_void_p(work_ptr)),
              "dmg_split_set_buffers")

    def set_dat_pitch(self, pitch):
        check(self.lib.dmg_split_set_dat_pitch(self.h, int(pitch)), "dmg_split_set_dat_pitch")

    def run(self, direction=FFTW_FORWARD, stream=None):
        check(self.lib.dmg_split_run(self.h, int(direction), ctypes.c_void_p(stream or 0)), "runSplitPlan")

    def set_timing(self, on=True):
        check(self.lib.dmg_split_set_timing(self.h, int(bool(on))), "dmg_split_set_timing")

    def pass_times(self, direction=FFTW_FORWARD):
        """Milliseconds of each pass of the last timed run in `direction`."""
        buf = (ctypes.c_float * 16)()
        k = self.lib.dmg_split_pass_times(self.h, int(direction), buf, 16)
        if k < 0:
            raise DecompError("dmg_split_pass_times: %s" % last_error())
        return [buf[i] for i in range(k)]

    def times(self):
        """plan->times after dmg_split_collect_times: {name: seconds}."""
        check(self.lib.dmg_split_collect_times(self.h), "dmg_split_collect_times")
        t = self._s.times
        return {n: t[i] for i, n in enumerate(["RESHAPE_1", "FFT_1", "TWIDDLE", "RESHAPE_2", "FFT_2", "ALL"])}

    def launches(self, direction=FFTW_FORWARD):
        return self.lib.dmg_split_launches(self.h, int(direction))

    @property
    def flops(self):
        return float(self.lib.dmg_split_flops(self.h))

    def describe(self):
        return self.lib.dmg_split_describe(self.h).decode()

    def free(self):
        if getattr(self, "h", None):
            self.lib.freeSplitPlan(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def split_run_group(plans, direction, stream=None):
    """dmg_split_run_group: runSplitPlan on several plans (any sizes; runtime radix schedules, one arithmetic),
    the k-th passes of all of them in one launch."""
    n = len(plans)
    P = (ctypes.c_void_p * n)(*[p.h for p in plans])
    check(load().dmg_split_run_group(n, P, int(direction), ctypes.c_void_p(stream or 0)), "dmg_split_run_group")


def split_run_group_batch(plans, njobs, dats, works, scales, direction, stream=None):
    """dmg_split_run_group_batch: plan i transforms njobs[i] arrays; dats / works / scales list them plan by plan
    (scales: device int words, for double-float plans)."""
    n, m = len(plans), len(dats)
    P = (ctypes.c_void_p * n)(*[p.h for p in plans])
    J = (ctypes.c_int * n)(*[int(x) for x in njobs])
    D = (ctypes.c_void_p * m)(*[ctypes.c_void_p(x) for x in dats])
    W = (ctypes.c_void_p * m)(*[ctypes.c_void_p(x) for x in works])
    S = (ctypes.c_void_p * m)(*[ctypes.c_void_p(x) for x in (scales or [0] * m)])
    check(load().dmg_split_run_group_batch(n, P, J, D, W, S, int(direction), ctypes.c_void_p(stream or 0)),
          "dmg_split_run_group_batch")


def split_group_launches(plans, direction) -> int:
    n = len(plans)
    P = (ctypes.c_void_p * n)(*[p.h for p in plans])
    return load().dmg_split_group_launches(n, P, int(direction))


def autotune_cache_clear():
    """Forget every cached autotuning winner."""
    load().dmg_autotune_cache_clear()


def autotune_cache_entries() -> int:
    return load().dmg_autotune_cache_entries()


def autotune_last_timed() -> int:
    """Configurations the last autotuning call timed (0 when it built a cached choice)."""
    return load().dmg_autotune_last_timed()


def _wrap_plan(start: Decomp, handle, length: int) -> "SplitPlan":
    sp = SplitPlan.__new__(SplitPlan)
    sp.lib, sp.start, sp.h, sp.length, sp.dtype = load(), start, handle, int(length), C128
    return sp


def propose_parallel_plan(flags: int, start: Decomp, B, dat_ptr: int, length: int, work_ptr: int):
    """proposeParallelPlan: the plan of the given second-stage factors B (A = L / B), grids from
    makeProcessorGrid; None where the reference declines (every B_i = 1 under PREFER_STAGE1)."""
    lib = load()
    lib.dmg_clear_error()
    h = lib.proposeParallelPlan(int(flags), start.h, _int_array(B), ctypes.c_void_p(dat_ptr), int(length),
                                ctypes.c_void_p(work_ptr))
    if not h:
        if lib.dmg_last_error_code():
            raise DecompError("proposeParallelPlan: %s" % last_error())
        return None
    return _wrap_plan(start, h, length)


def build_parallel_plan(flags: int, use_first: int, use_second: int, start: Decomp, A, B, L, grid_a, grid_b,
                        dat_ptr: int, length: int, work_ptr: int):
    """buildParallelPlan: the plan of explicit factors and processor grids for the A and B stages."""
    lib = load()
    nd = len(L)
    h = lib.buildParallelPlan(int(flags), int(use_first), int(use_second), start.h, nd, _int_array(A), _int_array(B),
                              _int_array(L), _int_array(grid_a), _int_array(grid_b), ctypes.c_void_p(dat_ptr),
                              int(length), ctypes.c_void_p(work_ptr))
    if not h:
        raise DecompError("buildParallelPlan: %s" % last_error())
    return _wrap_plan(start, h, length)


# ---------------------------------------------------------------- global-order I/O

def io_view(decomp: "Decomp", rank: int):
    """makeIOType's file view (reshape.c:137-172) for one rank: (file positions, buffer offsets) of its
    elements in C order."""
    import numpy as np
    lib = load()
    n = lib.dmg_io_view(decomp.h, int(rank), None, None, 0)
    if n < 0:
        raise DecompError("dmg_io_view: %s" % last_error())
    f = np.empty(max(n, 1), dtype=np.int64)
    m = np.empty(max(n, 1), dtype=np.int64)
    P = ctypes.POINTER(ctypes.c_longlong)
    lib.dmg_io_view(decomp.h, int(rank), f.ctypes.data_as(P), m.ctypes.data_as(P), n)
    return f[:n], m[:n]


def io_gather(decomp: "Decomp", elem_size: int, src_ptr: int, global_ptr: int, stream=None):
    """Device to device: the array in `decomp` to global C order."""
    check(load().dmg_io_gather(decomp.h, int(elem_size), ctypes.c_void_p(src_ptr), ctypes.c_void_p(global_ptr),
                               ctypes.c_void_p(stream)), "dmg_io_gather")


def io_scatter(decomp: "Decomp", elem_size: int, global_ptr: int, dst_ptr: int, stream=None):
    """Device to device: global C order into the array in `decomp`."""
    check(load().dmg_io_scatter(decomp.h, int(elem_size), ctypes.c_void_p(global_ptr), ctypes.c_void_p(dst_ptr),
                                ctypes.c_void_p(stream)), "dmg_io_scatter")


def write_file(path: str, decomp: "Decomp", elem_size: int, src_ptr: int, stream=None):
    """Write the distributed array to `path` as the global array in C order (the reference's writeFile)."""
    check(load().dmg_io_write_file(path.encode(), decomp.h, int(elem_size), ctypes.c_void_p(src_ptr),
                                   ctypes.c_void_p(stream)), "dmg_io_write_file")


def read_file(path: str, decomp: "Decomp", elem_size: int, dst_ptr: int, stream=None):
    """Read a global C-order file into the distributed array (the reference's readFile)."""
    check(load().dmg_io_read_file(path.encode(), decomp.h, int(elem_size), ctypes.c_void_p(dst_ptr),
                                  ctypes.c_void_p(stream)), "dmg_io_read_file")


# ---------------------------------------------------------------- device visitors

def decomp_scale(decomp: "Decomp", complex64: bool, data_ptr: int, factors, sign: int = -1, stream=None):
    """dmg_decomp_scale, the device form of decomp_scale (dimscale.c:7-67): data *= prod_d factors[d][x_d]
    (conjugated for sign == 1); factors[d] a complex numpy array of length L_d (complex128, or complex64 when
    complex64) or None."""
    import numpy as np
    keep = []
    arr = (ctypes.c_void_p * 3)()
    for d in range(3):
        f = factors[d] if factors is not None and d < len(factors) else None
        if f is not None:
            f = np.ascontiguousarray(f, dtype=np.complex64 if complex64 else np.complex128)
            keep.append(f)
            arr[d] = f.ctypes.data
        else:
            arr[d] = None
    check(load().dmg_decomp_scale(decomp.h, int(bool(complex64)), ctypes.c_void_p(data_ptr), arr, int(sign),
                                  ctypes.c_void_p(stream)), "dmg_decomp_scale")
    del keep


def fill_index(decomp: "Decomp", type_size: int, data_ptr: int, stream=None):
    """dmg_visit_fill_index: every held slot = its global C-order linear index."""
    check(load().dmg_visit_fill_index(decomp.h, int(type_size), ctypes.c_void_p(data_ptr), ctypes.c_void_p(stream)),
          "dmg_visit_fill_index")


# ---------------------------------------------------------------- request server

class _JobDesc(ctypes.Structure):
    _fields_ = [("side", ctypes.c_int), ("dtype", ctypes.c_int), ("input", ctypes.c_void_p),
                ("spectrum", ctypes.c_void_p), ("output", ctypes.c_void_p)]


class _JobDone(ctypes.Structure):
    _fields_ = [("id", ctypes.c_longlong), ("t_submit", ctypes.c_double), ("t_start", ctypes.c_double),
                ("t_done", ctypes.c_double), ("batch", ctypes.c_int), ("status", ctypes.c_int)]


class Server:
    """dmg_server_*: reshape + split-FFT jobs of mixed sizes with admission by free HBM, plan caching,
    stream slots and same-shape batching (include/dmg_serve.h)."""

    def __init__(self, grid=4, arena_bytes=8 << 30, slots=4, max_batch=8):
        self.lib = load()
        self.h = self.lib.dmg_server_create(int(grid), int(arena_bytes), int(slots), int(max_batch))
        if not self.h:
            raise DecompError("dmg_server_create: %s" % last_error())
        self.grid = grid

    def set_arith(self, dtype, arith):
        """Arithmetic of the server's plans of one element type (C128: ARITH_DF or ARITH_FP64; C64: ARITH_FP32 or
        ARITH_TC16); call it while no job is queued or running."""
        check(self.lib.dmg_server_set_arith(self.h, int(dtype), int(arith)), "dmg_server_set_arith")

    def set_mixing(self, max_side):
        """Jobs of sides up to max_side may share launches with other sides (0: only one side per batch)."""
        check(self.lib.dmg_server_set_mixing(self.h, int(max_side)), "dmg_server_set_mixing")

    def sizes(self, side, dtype):
        """Element counts of a job's host arrays: (input, spectrum, output)."""
        a, b, c = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_longlong()
        check(self.lib.dmg_server_job_sizes(self.h, int(side), int(dtype), ctypes.byref(a), ctypes.byref(b),
                                            ctypes.byref(c)), "dmg_server_job_sizes")
        return a.value, b.value, c.value

    def submit(self, side, dtype, input_ptr, spectrum_ptr=0, output_ptr=0):
        j = _JobDesc(int(side), int(dtype), ctypes.c_void_p(input_ptr), ctypes.c_void_p(spectrum_ptr or None),
                     ctypes.c_void_p(output_ptr or None))
        jid = self.lib.dmg_server_submit(self.h, ctypes.byref(j))
        if jid < 0:
            raise DecompError("dmg_server_submit: %s" % last_error())
        return jid

    def poll(self, max_jobs=4096):
        buf = (_JobDone * max_jobs)()
        n = self.lib.dmg_server_poll(self.h, buf, max_jobs)
        if n < 0:
            raise DecompError("dmg_server_poll: %s" % last_error())
        return [{"id": d.id, "t_submit": d.t_submit, "t_start": d.t_start, "t_done": d.t_done, "batch": d.batch,
                 "status": d.status} for d in buf[:n]]

    def drain(self):
        check(self.lib.dmg_server_drain(self.h), "dmg_server_drain")

    def status(self):
        q, r, u = ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong()
        check(self.lib.dmg_server_status(self.h, ctypes.byref(q), ctypes.byref(r), ctypes.byref(u)),
              "dmg_server_status")
        return {"queued": q.value, "running": r.value, "arena_used": u.value}

    def close(self):
        if self.h:
            self.lib.dmg_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def cube_specs(side, grid=4):
    """The served jobs' decompositions: (block spec, rotate spec)."""
    blk = "packed:block(%d,%d)|block(%d,%d)|local(%d)" % (side, grid, side, grid, side)
    rot = "packed:rotate(%d,block(%d,%d))|rotate(1,block(%d,%d))|local(%d)" % (side // 3, side, grid, side, grid, side)
    return blk, rot
