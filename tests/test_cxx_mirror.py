"""The C++ host mirror of RayIntersector<T> (include/rq_intersector.hpp) through its example
program: on CPU its global buffers equal the Python mirror's byte for byte; on the GPU its
closest-hit / any-hit results equal the oracle's."""
import subprocess

import numpy as np
import pytest

import candela_gb300 as R
from candela_gb300 import _build
from candela_gb300 import scenes as S
from oracle import oracle as O

from .helpers import assert_hits_identical, mesh

LAYOUTS = {"stack": R.STACK, "stackless": R.STACKLESS}
ENTS = [(1, 0.0, 0.0, 0.0, 0.0), (2, 0.25, -0.5, 0.125, 0.0), (1, 0.0, 0.0, 0.3, 0.5)]


def _write_inputs(d, rays=None):
    objs = [(1, mesh("hf32"), 3), (2, mesh("ico2"), 7)]
    with open(d / "objects.txt", "w") as f:
        f.write(f"{len(objs)}\n")
        for k, (oid, m, mid) in enumerate(objs):
            f.write(f"{oid} {mid}\n")
            m.vertices.tofile(d / f"verts_{k}.bin")
            m.indices.astype(np.uint32).tofile(d / f"idx_{k}.bin")
    with open(d / "entities.txt", "w") as f:
        for e in ENTS:
            f.write(" ".join(str(x) for x in e) + "\n")
    if rays is not None:
        rays.tofile(d / "rays.bin")
    return objs


def _python_mirror(objs, layout):
    ri = R.RayIntersector(layout)
    for oid, m, mid in objs:
        m2 = S.Mesh(m.vertices, m.indices, np.full(m.n_tris, mid, dtype=np.int32))
        ri.add_object(oid, [m2])
    for oid, tx, ty, tz, tr in ENTS:
        T = np.eye(4)
        T[:3, 3] = [tx, ty, tz]
        ri.push_entity(oid, model=T, translucency=tr)
    ri.buffer_entities()
    return ri


@pytest.mark.parametrize("name", ["stack", "stackless"])
def test_cxx_mirror_buffers_equal_python_mirror(tmp_path, name):
    objs = _write_inputs(tmp_path)
    r = subprocess.run([str(_build.EXAMPLE), name, str(tmp_path), str(tmp_path)], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    v, t, n, e = _python_mirror(objs, LAYOUTS[name]).global_buffers()
    assert np.fromfile(tmp_path / "nodes.bin", np.uint8).tobytes() == np.ascontiguousarray(n).tobytes()
    assert np.fromfile(tmp_path / "tris.bin", np.uint8).tobytes() == np.ascontiguousarray(t).tobytes()
    assert np.fromfile(tmp_path / "verts.bin", np.uint8).tobytes() == np.ascontiguousarray(v).tobytes()
    assert np.fromfile(tmp_path / "ents.bin", np.uint8).tobytes() == np.ascontiguousarray(e).tobytes()


def test_cxx_mirror_rejects_unknown_object(tmp_path):
    _write_inputs(tmp_path)
    with open(tmp_path / "entities.txt", "a") as f:
        f.write("99 0 0 0 0\n")
    r = subprocess.run([str(_build.EXAMPLE), "stack", str(tmp_path), str(tmp_path)], capture_output=True,
                       text=True)
    assert r.returncode == 1 and "hasn't been added" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["stack", "stackless"])
def test_cxx_mirror_queries_on_gpu(ctx, tmp_path, name):
    rays = S.sphere_rays(50_000, (-1.5, -1.5, -0.5), (1.5, 1.5, 1.5), seed=31)
    objs = _write_inputs(tmp_path, rays)
    boxes = S.query_boxes(20_000, (-1.2, -1.2, -0.4), (1.2, 1.2, 1.2), 0.005, 0.1, seed=32)
    boxes.tofile(tmp_path / "boxes.bin")
    r = subprocess.run([str(_build.EXAMPLE), name, str(tmp_path), str(tmp_path), "--gpu"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    v, t, n, e = _python_mirror(objs, LAYOUTS[name]).global_buffers()
    osc = O.OracleScene(O.ORC_STACK if name == "stack" else O.ORC_STACKLESS, v, t, n, e)
    hits = np.fromfile(tmp_path / "hits.bin", dtype=R.HIT_DTYPE)
    assert_hits_identical(hits, osc.closest(rays), "C++ mirror")
    occ = np.fromfile(tmp_path / "occ.bin", dtype=np.uint8)
    np.testing.assert_array_equal(occ, osc.anyhit(rays))
    coll = np.fromfile(tmp_path / "coll.bin", dtype=np.int32).reshape(-1, 4)
    want = osc.collide(boxes)
    np.testing.assert_array_equal(coll, want)
    assert 0 < want[:, 0].sum() < len(boxes)
