"""The C-ABI library loads on a machine without a GPU and exports every
function that the public headers in include/ declare."""
import ctypes
import os
import re

import pytest

from decomp_mpi_gb300 import _lib
from decomp_mpi_gb300.build import INCLUDE_DIR, LIB_PATH

def _strip_comments(text):
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return re.sub(r"//[^\n]*", "", text)


def _strip_blocks(text):
    """Drop brace blocks (struct bodies, inline function bodies)."""
    out, depth = [], 0
    for ch in text:
        if ch == "{":
            depth += 1
            continue
        if ch == "}":
            depth -= 1
            continue
        if depth == 0:
            out.append(ch)
    return "".join(out)


_FUNC = re.compile(r"\b([A-Za-z_]\w*)\s*\(([^()]|\([^()]*\))*\)\s*$", re.S)


def declared_functions():
    """Names of the functions the public headers declare (not static inline, not typedefs)."""
    names = {}
    for fn in sorted(os.listdir(INCLUDE_DIR)):
        if not fn.endswith(".h"):
            continue
        text = _strip_comments(open(os.path.join(INCLUDE_DIR, fn)).read())
        text = "\n".join(l for l in text.splitlines() if not l.strip().startswith("#"))
        text = text.replace('extern "C" {', "")
        text = "\n".join(l for l in text.splitlines() if l.strip() != "}")
        text = _strip_blocks(text)
        for stmt in text.split(";"):
            stmt = " ".join(stmt.split())
            if not stmt or stmt.startswith(("typedef", "static", "struct", "enum")):
                continue
            m = _FUNC.search(stmt)
            if m:
                names.setdefault(m.group(1), fn)
    return names


def test_library_is_built_in_tree():
    assert os.path.exists(LIB_PATH)


def test_library_loads_without_gpu():
    lib = _lib.load()
    assert lib.dmg_last_error_code() == 0


def test_every_declared_function_is_exported():
    lib = ctypes.CDLL(LIB_PATH)
    names = declared_functions()
    assert len(names) > 60
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_no_mpi_symbols_exported():
    """The virtual-MPI helpers are header-inline; a process may also load a real MPI."""
    lib = ctypes.CDLL(LIB_PATH)
    for n in ("MPI_Comm_rank", "MPI_Comm_size", "MPI_Type_contiguous"):
        assert not hasattr(lib, n), n


@pytest.mark.parametrize("name", sorted(_lib.SIGNATURES))
def test_python_signatures_exist(name):
    assert hasattr(_lib.load(), name)


_DROP_IN = r"""
#include <stdio.h>
#include "reshape.h"
#include "split_fft.h"
#include "index.h"
#include "block_decomp.h"
#include "interleave_decomp.h"
#include "rotate_decomp.h"
#include "factor_reverse_decomp.h"
#include "single_decomp.h"
#include "local_decomp.h"
#include "dmg_gb300.h"
#include "dmg_io.h"
#include "dmg_visit.h"
#include "dmg_serve.h"

/* test.c's first scenario, planned only (running needs a GPU): 10x10 from rank 0 to a rotated block */
int main(void) {
  int P = 4;
  MPI_Comm comm = dmg_comm_create(P);
  AxisDecomp o[2] = {makeAxisDecomp(comm, makeSingleDecomp(10, 0, 1), 1, 1),
                     makeAxisDecomp(comm, makeSingleDecomp(10, 0, P), 10, 1)};
  Decomp orig = makeDecomp(2, o);
  AxisDecomp n[2] = {makeAxisDecomp(comm, makeRotatedDecomp(2, makeLocalDecomp(10)), 1, 1),
                     makeAxisDecomp(comm, makeRotatedDecomp(1, makeBlockDecomp(10, P)), 10, 1)};
  Decomp next = makeDecomp(2, n);
  ReshapePlan plan = makeReshapePlan(comm, MPI_INT, orig, next);
  if (!plan) return 1;
  printf("%d %d %d\n", extent(orig), extent(next), checkReshapePlanBounds(plan, 4, 100, 100));
  freeReshapePlan(plan);
  freeDecomp(orig);
  freeDecomp(next);
  dmg_comm_free(comm);
  return 0;
}
"""


@pytest.mark.parametrize("compiler,std", [("gcc", "c99"), ("gcc", "c11"), ("g++", "c++17")])
def test_headers_compile_for_c_and_cpp_programs(tmp_path, compiler, std):
    """Every public header compiles with -pedantic -Werror as C99, C11 and C++17, as a reference program
    would include them."""
    import shutil
    import subprocess
    cc = shutil.which(compiler)
    if not cc:
        pytest.skip("%s not available" % compiler)
    src = tmp_path / ("drop_in.cpp" if compiler == "g++" else "drop_in.c")
    src.write_text(_DROP_IN)
    subprocess.run([cc, "-std=" + std, "-Wall", "-Wextra", "-pedantic", "-Werror", "-I" + INCLUDE_DIR,
                    "-fsyntax-only", str(src)], check=True, capture_output=True, timeout=120)


def test_c_program_links_and_plans(tmp_path):
    """A C program in the reference's style links against the library and plans test.c's first scenario
    on a machine without a GPU (planning is host work; the run needs the device)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc")
    if not cc:
        pytest.skip("gcc not available")
    src = tmp_path / "drop_in.c"
    src.write_text(_DROP_IN)
    exe = tmp_path / "drop_in"
    subprocess.run([cc, "-std=c99", "-I" + INCLUDE_DIR, str(src), LIB_PATH, "-Wl,-rpath," + os.path.dirname(LIB_PATH),
                    "-o", str(exe)], check=True, capture_output=True, timeout=120)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True, timeout=60).stdout.split()
    assert out == ["100", "30", "0"]
