"""The C ABI library on a CPU-only machine: it loads, exports every entry point include/rq.h
declares, its structs have the reference byte sizes, and device calls fail loudly without a GPU."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import candela_gb300 as R
from candela_gb300 import _lib as L

from .conftest import gpu_available

HEADERS = sorted((Path(__file__).resolve().parents[1] / "include").glob("*.h"))


def declared_functions():
    names = set()
    for h in HEADERS:
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(rq_\w+)\s*\(", text, re.M):
            names.add(m.group(1))
    return names


def test_every_declared_symbol_is_exported_and_bound():
    names = declared_functions()
    assert len(names) >= 20
    lib = L.lib()
    for n in sorted(names):
        assert hasattr(lib, n), f"librq.so does not export {n}"
        assert n in L.SIGNATURES, f"{n} has no ctypes signature in candela_gb300/_lib.py"


def test_abi_version_and_status_strings():
    assert L.lib().rq_abi_version() == 1
    assert L.lib().rq_status_string(L.RQ_EINVAL) == b"invalid argument"


def test_struct_sizes_match_reference_layouts():
    assert R.VERTEX_DTYPE.itemsize == 32         # Candela::Vertex
    assert L.TRI_DTYPE.itemsize == 16            # BVH::Triangle
    assert L.STACK_NODE_DTYPE.itemsize == 64     # FlattenedStackNode
    assert L.STACKLESS_NODE_DTYPE.itemsize == 32  # FlattenedNode
    assert L.ENTITY_DTYPE.itemsize == 192        # BVHEntity
    assert C.sizeof(L.RqOpts) == 32
    assert C.sizeof(L.RqGiParams) == 80
    assert C.sizeof(L.RqProbeParams) == 108     # rq_probe_params, the oracle's orc_probe_params
    from oracle import oracle as O
    assert C.sizeof(O.OrcProbeParams) == C.sizeof(L.RqProbeParams)


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU failure path")
def test_context_creation_fails_without_gpu():
    with pytest.raises(R.RqError) as e:
        R.Context(0)
    assert e.value.status == L.RQ_ECUDA


def test_null_arguments_rejected():
    h = C.c_void_p()
    assert L.lib().rq_create(0, None) == L.RQ_EINVAL
    assert L.lib().rq_closest(None, None, None, 0, None, None, None) == L.RQ_EINVAL
    assert L.lib().rq_build_bvh(None, 0, None, 0, None, 0, 1, None, C.byref(h)) == L.RQ_EINVAL
