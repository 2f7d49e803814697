"""Known answers of the radiance-probe restatement (orc_probe_raygen / orc_probe_shade,
UpdateRadianceProbes.glsl), independent of the reference tree: probe positions, the direction
distribution, the sky term of a miss, the SH encoding and its packing, the depth-moment map and
the temporal blend."""
import numpy as np

from candela_gb300.engine import probe_params, probe_volumes
from oracle import oracle as O

from .helpers import oracle_scene, single_object

import candela_gb300 as R

Y00, Y1 = np.float32(0.28209479177387814347), np.float32(0.48860251190291992159)


def _decode(sh):
    """Unpacked SH (n, 4, 3) in the struct order L00, L11, L10, L1_1 (UnpackSH)."""
    w = sh[:, :6].astype(np.uint32)
    lo = (w & 0xFFFF).astype(np.uint16).view(np.int16).astype(np.float32)
    hi = (w >> 16).astype(np.uint16).view(np.int16).astype(np.float32)
    u = np.stack([lo, hi], 2).reshape(-1, 12) / np.float32(32767.0)
    return (u * sh[:, 6].view(np.float32)[:, None]).reshape(-1, 4, 3)


def test_probe_rays_positions_and_directions():
    p = probe_params(grid=(8, 4, 6), origin=(1.0, 2.0, 3.0), size=(4.0, 2.0, 3.0), seed=3)
    rays = O.probe_raygen(p)
    assert rays.shape == (8 * 4 * 6,)
    i = np.arange(rays.shape[0])
    x, y, z = i % 8, (i // 8) % 4, i // 32
    want = np.stack([1.0 + (2.0 * x / 8 - 1) * 4.0, 2.0 + (2.0 * y / 4 - 1) * 2.0, 3.0 + (2.0 * z / 6 - 1) * 3.0], 1)
    np.testing.assert_allclose(rays["o"], want, atol=1e-6)
    np.testing.assert_allclose(np.linalg.norm(rays["d"], axis=1), 1.0, atol=2e-7)
    assert (rays["tmin"] == 0).all() and (rays["tmax"] == np.float32(1e6)).all()
    # uniform on the sphere: the mean direction vanishes, each |component| averages 1/2
    d = O.probe_direction(11, np.arange(200_000, dtype=np.uint32))
    assert np.abs(d.mean(0)).max() < 0.01
    np.testing.assert_allclose(np.abs(d).mean(0), 0.5, atol=0.01)


def test_probe_miss_sky_map_and_sh():
    """All rays miss: radiance sky x 2.2 x clamp(d.y, 0, 1), depth moments (256, 256^2) at the
    direction's octahedral pixel, the SH decodes to EncodeSH within the snorm16 step, nothing
    reprojects (the previous volume sits far away) so the frame count is 0."""
    bufs = single_object("ico2", R.STACK)
    osc = oracle_scene(bufs, R.STACK)
    p = probe_params(grid=(6, 5, 4), origin=(100.0, 100.0, 100.0), prev_origin=(-100.0, 0.0, 0.0), size=(1.0, 1.0, 1.0),
                     seed=9, sky_color=(0.5, 0.25, 1.0))
    rays = O.probe_raygen(p)
    hits = np.zeros(rays.shape[0], dtype=O.HIT_DTYPE)
    hits["t"] = -1.0
    sh, raw, pmap = probe_volumes(p)
    osh, oraw, omap = osc.probe_shade(p, rays, hits, None, [[0.5, 0.5, 0.5]], sh, raw, pmap)
    d = rays["d"]
    ls = np.clip(d[:, 1], 0.0, 1.0).astype(np.float32)
    want = (np.float32([0.5, 0.25, 1.0]) * np.float32(2.2))[None, :] * ls[:, None]
    np.testing.assert_array_equal(oraw[:, :3], want.astype(np.float32))
    assert (oraw[:, 3] == 0).all() and (osh[:, 7] == 0).all()
    written = (omap != 0).reshape(-1, 64, 2).any(2)
    assert (written.sum(1) == 1).all()
    np.testing.assert_array_equal(omap.reshape(-1, 64, 2)[written], np.float32([[256.0, 65536.0]]).repeat(written.sum(), 0))
    # the SH: L00 = Y00 * L * 2 pi, L1 lobes = Y1 * (-d.x, d.z, -d.y) * L * 4 pi / 3, packed to 1/32767
    c = _decode(osh)
    a0, a1 = np.float32(2 * np.pi), np.float32(4 * np.pi / 3)
    ref = np.stack([Y00 * oraw[:, :3] * a0, -Y1 * d[:, 0:1] * oraw[:, :3] * a1, Y1 * d[:, 2:3] * oraw[:, :3] * a1,
                    -Y1 * d[:, 1:2] * oraw[:, :3] * a1], 1)
    scale = np.abs(ref).reshape(-1, 12).max(1)
    assert (np.abs(c - ref).reshape(-1, 12).max(1) <= scale / 32767.0 * 0.51 + 1e-7).all()


def test_probe_temporal_blend():
    """Every probe reprojects onto itself (unmoved volume) except the first row, column and layer
    (their SamplePoint is exactly 0, and Reproject wants it inside (0, 1)); with u_Temporal the
    frame count advances from the previous volume's and the raw radiance and depth moments blend
    by min(1 - 1/frames, 0.98); without it they are replaced."""
    bufs = single_object("ico2", R.STACK)
    osc = oracle_scene(bufs, R.STACK)
    n = 5 * 4 * 3
    prev_sh = np.zeros((n, 8), dtype=np.uint32)
    prev_sh[:, 7] = 4                                     # 4 frames so far -> 5, alpha 0.8
    prev_raw = np.full((n, 4), 2.0, dtype=np.float32)
    pmap = np.full((n, 128), 10.0, dtype=np.float32)
    for temporal in (True, False):
        p = probe_params(grid=(5, 4, 3), origin=(50.0, 0.0, 0.0), size=(1.0, 1.0, 1.0), temporal=temporal,
                         sky_color=(1.0, 1.0, 1.0))
        rays = O.probe_raygen(p)
        hits = np.zeros(n, dtype=O.HIT_DTYPE)
        hits["t"] = -1.0
        osh, oraw, omap = osc.probe_shade(p, rays, hits, None, [[0.5, 0.5, 0.5]], prev_sh, prev_raw, pmap)
        i = np.arange(n)
        inner = (i % 5 > 0) & ((i // 5) % 4 > 0) & (i // 20 > 0)
        np.testing.assert_array_equal(osh[:, 7], np.where(inner, 5, 0))
        a = np.float32(min(1.0 - 1.0 / 5.0, 0.98)) if temporal else np.float32(0.0)
        fr = np.clip(rays["d"][:, 1], 0, 1)[:, None] * np.float32(2.2)
        want = np.where(inner[:, None], fr * (np.float32(1) - a) + np.float32(2.0) * a, fr).astype(np.float32)
        np.testing.assert_allclose(oraw[:, :3], np.broadcast_to(want, (n, 3)), rtol=1e-6, atol=1e-7)
        moved = (omap != 10.0).reshape(n, 64, 2).any(2)
        assert (moved.sum(1) == 1).all()
        got = omap.reshape(n, 64, 2)[moved]
        np.testing.assert_allclose(got[:, 0], np.where(inner, 256 * (1 - a) + 10 * a, 256.0), rtol=1e-6)
