"""Pins the CPU restatement to the reference's own shader source compiled as C++ (oracle/Makefile,
ref_glsl_harness.cpp): the traversal functions of TraverseBVHStack.glsl and TraverseBVHStackless.glsl
give the same TUVW, triangle, mesh, entity and iteration outputs, and the same occlusion answers, as
rq_oracle.cpp with the reference's own conventions (first-found ties, the `TriangleIdx > 0` test);
likewise the collision shaders, GetData, the samplers and the diffuse / specular shading
statements.  Runs where the reference source tree is mounted."""
import numpy as np
import pytest

import candela_gb300 as R
from candela_gb300 import scenes as S
from oracle import oracle as O

from .helpers import ORC_LAYOUT, mesh, oracle_scene, single_object

pytestmark = pytest.mark.skipif(not O.ref_glsl_available(), reason="reference source tree not mounted")

FIELDS_F = ("t", "u", "v", "w")
FIELDS_I = ("tri", "mesh", "entity")


def _rays(lo, hi, n, seed, camera=None):
    parts = [S.sphere_rays(n, lo, hi, seed=seed)]
    if camera:
        parts.append(S.camera_rays(96, 72, **camera))
    edge = np.zeros(5, dtype=R.RAY_DTYPE)
    edge["o"] = [[0, 0, 5], [0, 0, 5], [0.1, 0.2, 3], [0, 0, 5], [-3, 0.1, 0.05]]
    edge["d"] = [[np.nan, 0, -1], [0, 0, 0], [0, 0, -1], [1e-30, 0, -1], [1, 0, 0]]
    edge["tmax"] = 1e6
    parts.append(edge)
    return np.concatenate(parts)


def _compare(ref, ours, iters=True):
    for f in FIELDS_F:
        np.testing.assert_array_equal(ours[f].view(np.uint32), ref[f].view(np.uint32), err_msg=f)
    hit = ref["t"] > 0
    for f in FIELDS_I:
        np.testing.assert_array_equal(ours[f][hit], ref[f][hit], err_msg=f)
    if iters:
        np.testing.assert_array_equal(ours["iters"], ref["iters"])
    return hit


@pytest.mark.parametrize("name", ["hf32", "ico2", "c1"])
@pytest.mark.parametrize("layout", [R.STACK, R.STACKLESS])
def test_single_object_matches_reference_shader(name, layout):
    bufs = single_object(name, layout)
    osc = oracle_scene(bufs, layout)
    rays = _rays((-1.5, -1.5, -0.3), (1.5, 1.5, 1.2), 30_000, seed=4, camera=S.C1_CAMERA)
    ref = O.ref_glsl_closest(ORC_LAYOUT[layout], *bufs, rays)
    ours = osc.closest(rays, tie=O.ORC_TIE_FIRST_FOUND, flags=O.ORC_FLAG_REF_COMPAT)
    hit = _compare(ref, ours)
    assert 0.1 < hit.mean() < 0.95
    np.testing.assert_array_equal(osc.anyhit(rays), O.ref_glsl_occluded(ORC_LAYOUT[layout], *bufs, rays))


@pytest.mark.parametrize("layout", [R.STACK, R.STACKLESS])
def test_entities_and_transparency_match_reference_shader(layout):
    """Several entities with rotations, scales and translations, some translucent: the scene loop,
    the entity transform and IntersectSceneIgnoreTransparent.  The shader hands the same `out int
    Iters` to every entity's walk, so its iteration output is the last walked entity's count; with
    the reference-compat flag the restatement reports that too (by default it sums over entities),
    and iterations are compared as well."""
    ri = R.RayIntersector(layout)
    ri.add_object(1, [mesh("hf32")])
    ri.add_object(2, [mesh("ico2")])
    M = S.instance_transforms(12, (-3.0, -3.0, 0.0), (3.0, 3.0, 1.0), 0.4, 1.2, seed=5, anisotropic=0.3,
                              tilt=0.1)
    for i in range(12):
        ri.push_entity(1 + (i % 2), model=M[i].astype(np.float64), translucency=0.5 if i % 4 == 1 else 0.0)
    ri.buffer_entities()
    v, t, n, e = ri.global_buffers()
    osc = O.OracleScene(ORC_LAYOUT[layout], v, t, n, e)
    rays = _rays((-4.0, -4.0, -0.5), (4.0, 4.0, 2.0), 20_000, seed=8,
                 camera=dict(eye=(0.0, -8.0, 5.0), target=(0.0, 0.0, 0.3)))
    for ignore in (False, True):
        ref = O.ref_glsl_closest(ORC_LAYOUT[layout], v, t, n, e, rays, ignore_transparent=ignore)
        flags = O.ORC_FLAG_REF_COMPAT | (O.ORC_FLAG_IGNORE_TRANSPARENT if ignore else 0)
        ours = osc.closest(rays, tie=O.ORC_TIE_FIRST_FOUND, flags=flags)
        hit = _compare(ref, ours)
        assert hit.mean() > 0.1 and len(np.unique(ref["entity"][hit])) >= 6
    np.testing.assert_array_equal(osc.anyhit(rays), O.ref_glsl_occluded(ORC_LAYOUT[layout], v, t, n, e, rays))
    # the last entity alone: its iteration count is the shader's output
    last = e[-1:].copy()
    ref = O.ref_glsl_closest(ORC_LAYOUT[layout], v, t, n, last, rays)
    ours = O.OracleScene(ORC_LAYOUT[layout], v, t, n, last).closest(rays, tie=O.ORC_TIE_FIRST_FOUND,
                                                                    flags=O.ORC_FLAG_REF_COMPAT)
    _compare(ref, ours)


def test_cos_hemisphere_matches_reference_sampler():
    """CosWeightedHemisphere (Sampling.glsl:1-12) compiled from the reference with the C library's
    cos / sin, against the restatement's turn-based sine / cosine: within a few ulps."""
    rng = np.random.default_rng(1)
    n = rng.normal(size=(50_000, 3)).astype(np.float32)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    r = (rng.integers(0, 1 << 24, size=(50_000, 2)) / 2.0 ** 24).astype(np.float32)
    ours, ref = O.cos_hemisphere(n, r), O.ref_glsl_cos_hemisphere(n, r)
    assert np.abs(ours - ref).max() < 2e-6
    assert (ours == ref).all(1).mean() > 0.2


@pytest.mark.parametrize("layout", [R.STACK, R.STACKLESS])
def test_collide_matches_reference_shader(layout):
    """CollideScene of CollideBVHStack.glsl / CollideBVHStackless.glsl compiled as C++ against the
    restatement with the reference's conventions (RQ_FLAG_REF_COMPAT: the repeated separating
    axis, the within-leaf triangle index on the stack layout): identical records."""
    from .test_oracle_collide import _scene_boxes
    ri = R.RayIntersector(layout)
    ri.add_object(1, [mesh("hf32")])
    ri.add_object(2, [mesh("ico2")])
    M = S.instance_transforms(6, (-2.0, -2.0, 0.0), (2.0, 2.0, 0.5), 0.6, 1.2, seed=7, tilt=0.05)
    ri.push_entity(1)
    for i in range(6):
        ri.push_entity(1 + (i % 2), model=M[i].astype(np.float64))
    ri.buffer_entities()
    v, t, n, e = ri.global_buffers()
    osc = O.OracleScene(ORC_LAYOUT[layout], v, t, n, e)
    boxes = np.concatenate([_scene_boxes("hf32", 4000, seed=3), _scene_boxes("ico2", 4000, seed=4)])
    ref = O.ref_glsl_collide(ORC_LAYOUT[layout], v, t, n, e, boxes)
    ours = osc.collide(boxes, flags=O.ORC_FLAG_REF_COMPAT)
    np.testing.assert_array_equal(ours[:, 0], ref[:, 0])
    hit = ref[:, 0] == 1
    np.testing.assert_array_equal(ours[hit], ref[hit])
    assert 0.2 < hit.mean() < 0.95 and len(np.unique(ref[hit, 1])) >= 3


def test_getdata_matches_reference_shader():
    """GetData (TraverseBVHStack.glsl:422-455) compiled as C++: the interpolated half-packed vertex
    normal, the UV the albedo texture is sampled at (its texture() reports the coordinates), the
    ModelColor of untextured meshes, emissive and alpha — against the restatement's hit_normal,
    hit_uv and hit_albedo."""
    m = S.heightfield(32, seed=5)
    pos = m.positions().astype(np.float64)
    verts = S.with_texcoords(m.vertices, np.stack([pos[:, 0] * 1.7 + 0.3, pos[:, 1] * -2.1], 1))
    mids = (np.arange(m.n_tris) % 3).astype(np.int32)
    b = R.build_bvh(verts, m.indices, mids, 0, layout=R.STACK)
    ents = R.identity_entity(0, b.nodes.shape[0], emissive=0.25, alpha=0.75)
    osc = O.OracleScene(O.ORC_STACK, verts, b.tris, b.nodes, ents)
    rays = S.camera_rays(96, 72, **S.C1_CAMERA)
    hits = osc.closest(rays)
    hits = hits[hits["t"] > 0]
    model = np.float32([[0.7, 0.6, 0.5], [0.2, 0.8, 0.4], [0.9, 0.9, 0.2]])
    refs = [5, -1, 9]                                        # texture per mesh id
    ref = O.ref_glsl_getdata(verts, b.tris, ents, model, refs, hits)
    np.testing.assert_array_equal(ref[:, :3], osc.hit_normal(hits, 0))
    uv = osc.hit_uv(hits)
    tex = np.isin(hits["mesh"], [0, 2])
    np.testing.assert_array_equal(ref[tex, 3:5], uv[tex])
    np.testing.assert_array_equal(ref[tex, 5], np.where(hits["mesh"][tex] == 0, 5.0, 9.0))
    np.testing.assert_array_equal(ref[~tex, 3:6], osc.hit_albedo(hits[~tex], model))
    np.testing.assert_array_equal(ref[:, 6], np.float32(0.25))
    np.testing.assert_array_equal(ref[:, 7], np.float32(0.75))
    assert tex.sum() > 100 and (~tex).sum() > 100


def test_specular_direction_matches_reference_sampler():
    """StochasticReflectionDirection (SpecularTrace.glsl:102-135) with SampleGGXVNDF (Sampling.glsl:
    63-83) compiled as C++, its hash2() drawing the same counter-based samples: a mirror is
    reproduced bit for bit; GGX samples agree to a few ulps except where sin(theta) = sqrt(1 -
    cos^2) cancels (cos(theta) within 1e-6 of 1), where both float evaluations carry ~1e-4 error."""
    rng = np.random.default_rng(3)
    n = rng.normal(size=(40_000, 3)).astype(np.float32)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    i = rng.normal(size=(40_000, 3)).astype(np.float32)
    i /= np.linalg.norm(i, axis=1, keepdims=True)
    i = np.where(((i * n).sum(1) > 0)[:, None], -i, i).astype(np.float32)
    rid = np.arange(40_000, dtype=np.uint32)
    for rough in (0.0, 0.005):
        np.testing.assert_array_equal(O.spec_direction(i, n, rough, 7, rid), O.ref_glsl_spec_direction(i, n, rough, 7, rid))
    for rough in (0.3, 0.8, 1.0):
        d = np.abs(O.spec_direction(i, n, rough, 7, rid) - O.ref_glsl_spec_direction(i, n, rough, 7, rid)).max(1)
        assert d.max() < 1e-3 and np.median(d) < 2e-7 and (d < 1e-5).mean() > 0.99


def _shading_scene():
    """Two objects, five entities: emissive 0, 0.5, 2 and +inf (the last drives the specular pass's
    IsValid branch), one tilted; camera rays and sphere rays with misses."""
    ri = R.RayIntersector(R.STACK)
    ri.add_object(1, [mesh("hf32")])
    ri.add_object(2, [mesh("ico2")])
    M = S.instance_transforms(4, (-2.0, -2.0, 0.2), (2.0, 2.0, 0.8), 0.5, 0.9, seed=9, tilt=0.2)
    ri.push_entity(1)
    for i, em in enumerate((0.5, 2.0, 0.0, np.inf)):
        ri.push_entity(2 if i % 2 == 0 else 1, model=M[i].astype(np.float64), emissive=em)
    ri.buffer_entities()
    v, t, n, e = ri.global_buffers()
    osc = O.OracleScene(O.ORC_STACK, v, t, n, e)
    rays = np.concatenate([S.camera_rays(80, 60, eye=(0.0, -5.0, 3.0), target=(0.0, 0.0, 0.3)),
                           S.sphere_rays(20_000, (-2.5, -2.5, -0.2), (2.5, 2.5, 1.5), seed=11)])
    hits = osc.closest(rays)
    emissive = e["data"][:, 0].view(np.float32)
    model = np.float32([[0.7, 0.6, 0.5], [0.2, 0.8, 0.4], [0.9, 0.9, 0.2], [0.3, 0.3, 0.3]])
    alb = np.zeros((rays.shape[0], 4), dtype=np.float32)
    hit = hits["t"] > 0
    alb[hit, :3] = osc.hit_albedo(hits[hit], model)
    alb[hit, 3] = emissive[hits["entity"][hit]]
    nrm = np.full((rays.shape[0], 3), -1.0, dtype=np.float32)
    nrm[hit] = osc.hit_normal(hits[hit], 0)
    lit = np.random.default_rng(2).integers(0, 2, rays.shape[0]).astype(np.uint8)
    return osc, rays, hits, model, alb, nrm, lit


def test_diffuse_shading_matches_reference_shader():
    """The diffuse pass's hit shading (DiffuseTrace.glsl:486-494, GetDirect :368-372) compiled as
    C++ with GetDirectShadow returning the shadow ray's answer and the sky texture a constant:
    the restatement's shade() gives the same radiance and AO bit for bit (its sky_color is the
    shader's texture value times its 2).  Run with the reference's SUN_COLOR_DIFF and with another
    colour."""
    osc, rays, hits, model, alb, nrm, lit = _shading_scene()
    sun_dir, sky = np.float32([0.3, 0.4, -0.866]), np.float32([0.45, 0.6, 0.95])
    ref_sun, _ = O.ref_glsl_sun_colors()
    for sun in (ref_sun, np.float32([4.0, 3.8, 3.5])):
        ref = O.ref_glsl_shade(0, rays, hits, alb, nrm, lit, sun_dir, sun, sky)
        ours = osc.shade(rays, hits, lit, model, sun_dir, sun, sky * np.float32(2.0))
        np.testing.assert_array_equal(ours.view(np.uint32), ref.view(np.uint32))
    hit = hits["t"] > 0
    assert 0.2 < hit.mean() < 0.9 and (ref[hit, :3].sum(1) > 0).mean() > 0.3
    assert np.isinf(ref[hit & (alb[:, 3] == np.inf)]).any()


def test_specular_shading_matches_reference_shader():
    """The specular pass's shading and store (SpecularTrace.glsl:554-563 and 588-596: SampleLighting
    :420-425, Sky :435-437, IsValid Utility.glsl:117-125, TransformReflectionTransversal
    SpatialUtility.glsl:12-14) compiled as C++, SampleProbes returning the ambient term: the
    restatement's spec_shade() stores the same texel bit for bit, including the non-finite
    radiance the +inf emissive entity gives (zeroed, t = -1)."""
    osc, rays, hits, model, alb, nrm, lit = _shading_scene()
    sky, amb = np.float32([0.45, 0.6, 0.95]), np.float32([0.1, 0.1, 0.12])
    _, ref_sun = O.ref_glsl_sun_colors()
    clamped = 0
    for sun in (ref_sun, np.float32([4.0, 3.8, 3.5])):
        for rough in (0.0, 0.35, 1.0):
            ref = O.ref_glsl_shade(1, rays, hits, alb, nrm, lit, (0.0, 0.0, -1.0), sun, sky, amb, rough)
            ours = osc.spec_shade(rays, hits, lit, model, rough, sun, sky, amb)
            np.testing.assert_array_equal(ours.view(np.uint32), ref.view(np.uint32))
            clamped += int((ref[:, :3] == 6.0).sum())
    hit = hits["t"] > 0
    bad = hit & (alb[:, 3] == np.inf)
    assert bad.sum() > 10 and (ref[bad, 3] == np.float32(-1.0 / 48.0)).all()
    assert clamped > 100 and (ref[~hit, :3] > 0).all()


def _probe_scene():
    ri = R.RayIntersector(R.STACK)
    ri.add_object(1, [mesh("hf32")])
    ri.add_object(2, [mesh("ico2")])
    M = S.instance_transforms(6, (-1.5, -1.5, 0.1), (1.5, 1.5, 0.6), 0.4, 0.8, seed=12, tilt=0.1)
    ri.push_entity(1, emissive=0.0)
    for i in range(6):
        ri.push_entity(2, model=M[i].astype(np.float64), emissive=0.3 if i == 2 else 0.0)
    ri.buffer_entities()
    v, t, n, e = ri.global_buffers()
    return O.OracleScene(O.ORC_STACK, v, t, n, e), e


def _probe_inputs(osc, ents, p, model, flags=0):
    rays = O.probe_raygen(p)
    hits = osc.closest(rays, flags=flags)
    hit = hits["t"] > 0
    alb = np.zeros((rays.shape[0], 4), dtype=np.float32)
    alb[hit, :3] = osc.hit_albedo(hits[hit], model)
    alb[hit, 3] = ents["data"][:, 0].view(np.float32)[hits["entity"][hit]]
    nrm = np.full((rays.shape[0], 3), -1.0, dtype=np.float32)
    nrm[hit] = osc.hit_normal(hits[hit], p.normal_mode)
    sr = osc.shadow_raygen(rays, hits, np.array(p.sun_dir, dtype=np.float32), p.shadow_offset, p.normal_mode)
    lit = 1 - osc.anyhit(sr)
    return rays, hits, alb, nrm, lit


def test_probe_update_matches_reference_shader():
    """UpdateRadianceProbes.glsl main (with SampleProbes, Trilinear, GetVisibility, Reproject,
    GetDirect, the SH encode / pack / unpack of SphericalHarmonics.glsl and UnitVectorToOctahedron)
    compiled as C++, fed the restatement's rays, hits, GetData values and shadow answers: the packed
    SH volume, the raw radiance and the depth-moment map are identical bit for bit over three frames
    -- the first from an empty volume, then with the volume moved by a fraction of a probe spacing
    (reprojection, temporal blending, SampleProbes from the previous frame) and with
    u_Temporal off."""
    from candela_gb300.engine import probe_params, probe_volumes
    osc, ents = _probe_scene()
    model = np.float32([[0.7, 0.6, 0.5], [0.3, 0.8, 0.4]])
    sun = O.ref_glsl_probe_sun_color()
    origins = [(0.0, 0.0, 0.6), (0.13, -0.07, 0.62), (0.3, 0.05, 0.55)]
    sh, raw, pmap = probe_volumes(probe_params(grid=(10, 6, 8)))
    prev = origins[0]
    stats = []
    for k, org in enumerate(origins):
        p = probe_params(grid=(10, 6, 8), origin=org, prev_origin=prev, size=(2.0, 1.0, 1.6), seed=5 + k,
                         temporal=k < 2, sun_color=sun, sky_color=(0.4, 0.55, 0.9))
        rays, hits, alb, nrm, lit = _probe_inputs(osc, ents, p, model)
        want = O.ref_glsl_probe(p, rays, hits, alb, nrm, lit, sh, raw, pmap)
        got = osc.probe_shade(p, rays, hits, lit, model, sh, raw, pmap)
        for a, b, name in zip(got, want, ("sh", "raw", "map")):
            np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32), err_msg=f"frame {k} {name}")
        sh, raw, pmap = got
        prev = org
        hit = hits["t"] > 0
        stats.append((hit.mean(), (sh[:, 7] > 0).mean(), (lit[hit] == 0).mean()))
    assert all(0.2 < s[0] < 0.95 for s in stats)
    assert stats[1][1] > 0.5 and stats[2][1] > 0.5           # reprojected probes
    assert 0.05 < stats[0][2] < 0.95                          # some hits in shadow
    assert (np.abs(raw[:, :3]).sum(1) > 0).mean() > 0.5


def test_probe_direction_matches_reference_sampler():
    """normalize(LambertBRDF(h)) (UpdateRadianceProbes.glsl:351-372) with the C library's acos,
    pow, sin and cos, fed the same hash values, against the restatement's sqrt(1 - c^2) form with
    the turn-based sine / cosine: within 1e-6 (the radius cancels in the normalisation)."""
    ids = np.arange(100_000, dtype=np.uint32)
    for seed in (0, 7):
        ours = O.probe_direction(seed, ids)
        h = np.stack([O.sample_u01(seed, ids, 0), O.sample_u01(seed, ids, 1), np.full(ids.shape, 0.5, np.float32)], 1)
        d = np.abs(ours - O.ref_glsl_lambert_direction(h)).max(1)
        assert d.max() < 1e-6 and np.median(d) < 1e-7


def test_bounce_loop_matches_reference_shader():
    """The RT second-bounce loop (DiffuseTrace.glsl:499-535) compiled as C++, fed the restatement's
    GI hits, bounce directions, bounce hits (GetData values) and shadow answers: the bounce ray
    origins (HitPosition + iNormal * 0.02) and FinalRadiance + Bounced equal the restatement's
    (orc_bounce_raygen, orc_bounce_accumulate with the reference's silent misses) bit for bit."""
    osc, rays, hits, model, alb, nrm, lit = _shading_scene()
    sd, sun, sky = np.float32([0.3, 0.4, -0.866]), np.float32([4.0, 3.8, 3.5]), np.float32([0.45, 0.6, 0.95])
    bounces, seed = 3, 13
    sec = osc.gi_raygen(rays, hits, 1, seed, 0.05)
    sh = osc.closest(sec)
    emissive = osc.entities["data"][:, 0].view(np.float32)
    glit = 1 - osc.anyhit(osc.shadow_raygen(sec, sh, sd, 1e-3))
    fr = osc.shade(sec, sh, glit, model, sd, sun, sky)[:, :3]
    alive = sh["t"] > 0
    n = len(sec)
    slot = np.zeros((n, 20), dtype=np.float32)
    slot[:, 0:3], slot[:, 3:6] = sec["o"], sec["d"]
    slot[:, 6], slot[:, 7], slot[:, 8], slot[:, 9] = sh["t"], sh["u"], sh["v"], sh["w"]
    gn = np.full((n, 3), -1.0, dtype=np.float32)
    gn[alive] = osc.hit_normal(sh[alive], 0)
    flip = (gn * sec["d"]).astype(np.float32)
    facing = (flip[:, 0] + flip[:, 1]) + flip[:, 2] > np.float32(0.0001)
    gn[facing] = -gn[facing]
    thr0 = np.zeros((n, 3), dtype=np.float32)
    thr0[alive] = osc.hit_albedo(sh[alive], model)
    slot[alive, 10:13] = thr0[alive]
    slot[alive, 13] = emissive[sh["entity"][alive]]
    slot[:, 14:17], slot[:, 17:20] = gn, fr
    per = np.zeros((n, bounces, 15), dtype=np.float32)
    per[:, :, 3:7] = -1.0
    per[:, :, 11:14] = -1.0
    ours_in = np.zeros((n, bounces, 12), dtype=np.float32)
    ours_in[:, :, 0] = -1.0
    prev_r, prev_h, live = sec, sh, alive.copy()
    origins = []
    for b in range(bounces):
        br = osc.bounce_raygen(prev_r, prev_h, live, np.arange(n, dtype=np.uint32), seed, b, 0.02, 1e6)
        bh = osc.closest(br)
        blit = 1 - osc.anyhit(osc.shadow_raygen(br, bh, sd, 1e-3))
        hit = live & (bh["t"] > 0)
        per[live, b, 0:3] = br["d"][live]
        per[hit, b, 3], per[hit, b, 4], per[hit, b, 5], per[hit, b, 6] = (bh["t"][hit], bh["u"][hit], bh["v"][hit],
                                                                          bh["w"][hit])
        balb = osc.hit_albedo(bh[hit], model)
        per[hit, b, 7:10], per[hit, b, 10] = balb, emissive[bh["entity"][hit]]
        bn = osc.hit_normal(bh[hit], 0)
        per[hit, b, 11:14], per[:, b, 14] = bn, blit
        ours_in[hit, b, 0], ours_in[hit, b, 1:4], ours_in[hit, b, 4] = bh["t"][hit], balb, emissive[bh["entity"][hit]]
        ours_in[hit, b, 5:8], ours_in[hit, b, 8:11], ours_in[hit, b, 11] = bn, br["d"][hit], blit[hit]
        origins.append((live.copy(), br["o"].copy()))
        prev_r, prev_h, live = br, bh, hit
    ours = O.bounce_accumulate(fr, thr0, ours_in, sd, sun, sky, ref_miss=True)
    ref_fr, ref_org = O.ref_glsl_bounce(slot, per, sd, sun, sky)
    np.testing.assert_array_equal(ours.view(np.uint32), ref_fr.view(np.uint32))
    for b, (traced, o) in enumerate(origins):
        np.testing.assert_array_equal(ref_org[traced, b].view(np.uint32), o[traced].view(np.uint32), err_msg=f"b{b}")
    assert alive.sum() > 2000 and (ours != fr).any(1).mean() > 0.05 and origins[1][0].sum() > 100
