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
    assert L.lib().rq_abi_version() == L.ABI_VERSION == 3
    assert L.lib().rq_status_string(L.RQ_EINVAL) == b"invalid argument"


def test_struct_sizes_match_reference_layouts():
    assert R.VERTEX_DTYPE.itemsize == 32         # Candela::Vertex
    assert L.TRI_DTYPE.itemsize == 16            # BVH::Triangle
    assert L.STACK_NODE_DTYPE.itemsize == 64     # FlattenedStackNode
    assert L.STACKLESS_NODE_DTYPE.itemsize == 32  # FlattenedNode
    assert L.ENTITY_DTYPE.itemsize == 192        # BVHEntity
    assert C.sizeof(L.RqOpts) == 32
    assert C.sizeof(L.RqGiParams) == 88
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


def test_ctypes_structs_match_the_c_header(tmp_path):
    """Every struct the Python mirror declares has the size and field offsets the C compiler gives
    include/rq.h (a small C program prints them)."""
    import subprocess
    from pathlib import Path
    inc = Path(__file__).resolve().parents[1] / "include"
    structs = {"rq_opts": L.RqOpts, "rq_tune_result": L.RqTuneResult, "rq_batch_tune": L.RqBatchTune,
               "rq_gi_params": L.RqGiParams, "rq_gi_tune": L.RqGiTune, "rq_probe_params": L.RqProbeParams,
               "rq_frame_stats": L.RqFrameStats, "rq_diff_params": L.RqDiffParams,
               "rq_specular_params": L.RqSpecularParams}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "rq.h"', "int main(void) {"]
    for name, cls in structs.items():
        lines.append(f'printf("{name} %zu\\n", sizeof({name}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{name}.{f} %zu\\n", offsetof({name}, {f}));')
    lines += ['printf("rq_hit_attrib %zu\\n", sizeof(rq_hit_attrib));', "return 0; }"]
    src = tmp_path / "sizes.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-I", str(inc), str(src), "-o", str(exe)], check=True)
    got = dict(ln.split() for ln in subprocess.run([str(exe)], capture_output=True, text=True,
                                                   check=True).stdout.splitlines())
    for name, cls in structs.items():
        assert int(got[name]) == C.sizeof(cls), name
        for f, _ in cls._fields_:
            assert int(got[f"{name}.{f}"]) == getattr(cls, f).offset, f"{name}.{f}"
    assert int(got["rq_hit_attrib"]) == 32
