"""The restatement against fixtures taken from the reference's own shaders: tests/golden/glsl_pins.json
holds SHA-256 hashes of what TraverseBVHStack[less].glsl (with GetData), CollideBVHStack[less].glsl, the shading
statements of DiffuseTrace.glsl / SpecularTrace.glsl and UpdateRadianceProbes.glsl, compiled as C++
from the reference tree, return on seeded inputs (tests/golden/make_golden.py).  The oracle must
reproduce every hash; no reference tree is needed here."""
import hashlib
import importlib.util
import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).parent / "golden"


def _make_golden():
    spec = importlib.util.spec_from_file_location("make_golden", GOLDEN / "make_golden.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="module")
def outputs():
    return _make_golden().glsl_case_outputs(reference=False)


def test_every_shader_fixture_is_reproduced(outputs):
    pins = json.loads((GOLDEN / "glsl_pins.json").read_text())
    assert len(pins) >= 15 and set(pins) == set(outputs)
    bad = [k for k, v in outputs.items()
           if hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest() != pins[k]]
    assert not bad, bad


def test_fixture_cases_exercise_the_path(outputs):
    """The hashed cases are not trivial: hits and misses, occluded and free rays, collided and free
    boxes, lit and shadowed shading, reprojected probes."""
    for name in ("closest_hf32_stack", "closest_ico2_stackless"):
        hit = outputs[name][:, 0].view(np.float32) > 0
        assert 0.1 < hit.mean() < 0.95
    assert 0.05 < outputs["occluded_ico2_stack"].mean() < 0.95
    assert 0.1 < (outputs["collide_ico2_stack"][:, 0] == 1).mean() < 0.95
    assert (outputs["shade_diffuse"][:, :3] > 0).any(1).mean() > 0.3
    frames = outputs["probe_frame1"][:, 7]
    assert (frames > 0).mean() > 0.5
