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
