"""Differentiation form: forward depth + Lambert image, adjoint w.r.t. vertex positions.

* the forward depth equals the strict closest-hit t of the oracle bit for bit;
* the adjoint equals an FP64 host evaluation of the same closed-form derivatives;
* it matches central finite differences (h = 1e-3) on vertices whose neighbourhood does not
  change which triangle a pixel sees (away from silhouettes and triangle switches);
* it is bit-reproducible, and recompute mode equals taped mode;
* refit after a position update gives tight, containing boxes."""
import numpy as np
import pytest

import candela_gb300 as R
from candela_gb300 import _lib as L
from candela_gb300 import scenes as S
from candela_gb300.engine import diff_params
from oracle import oracle as O

from .helpers import assert_hits_identical, hits_from_device, rays_to_device

pytestmark = pytest.mark.gpu

CAM = dict(eye=(0.0, -1.6, 2.2), target=(0.0, 0.0, 0.0), vfov_deg=60.0)


def _setup(ctx, n=64, res=160, seed=5):
    import torch
    m = S.heightfield(n, seed=seed)
    b = R.build_bvh(m.vertices, m.indices, m.mesh_ids, 0, layout=R.STACK)
    ent = R.identity_entity(0, b.nodes.shape[0])
    sc = ctx.scene(R.STACK, m.vertices, b.tris, b.nodes, ent)
    rays = S.camera_rays(res, res, **CAM)
    tgt_mesh = S.heightfield(n, seed=seed + 1)
    tb = R.build_bvh(tgt_mesh.vertices, tgt_mesh.indices, tgt_mesh.mesh_ids, 0, layout=R.STACK)
    tsc = ctx.scene(R.STACK, tgt_mesh.vertices, tb.tris, tb.nodes, R.identity_entity(0, tb.nodes.shape[0]))
    d_rays = rays_to_device(rays)
    zero = torch.zeros((len(rays), 2), dtype=torch.float32, device="cuda")
    return m, b, ent, sc, rays, d_rays, tsc, zero


def _host_grad(m, b, ent, rays, hits, image, target, p):
    """FP64 evaluation of the adjoint formulas on the oracle's hit records."""
    P = m.vertices["pos"][:, :3].astype(np.float64)
    grad = np.zeros_like(P)
    hit = hits["t"] > 0
    tri = hits["tri"][hit]
    tv = b.tris[tri, :3]
    A, B, C = P[tv[:, 0]], P[tv[:, 1]], P[tv[:, 2]]
    d = rays["d"][hit].astype(np.float64)
    n = np.cross(B - A, C - A)
    ndotd = (n * d).sum(1)
    w = np.stack([hits["u"][hit], hits["v"][hit], hits["w"][hit]], 1).astype(np.float64)
    depth = hits["t"][hit].astype(np.float64)
    rad = image[hit, 1].astype(np.float64)
    T = target[hit].astype(np.float64)
    gt = 2 * p.w_depth * (depth - T[:, 0])
    gr = 2 * p.w_radiance * (rad - T[:, 1])
    m_ = -np.array(p.sun_dir[:], dtype=np.float64)
    ln = np.sqrt((n * n).sum(1))
    nh = n / ln[:, None]
    sgn = np.where(ndotd > 0, -1.0, 1.0)
    f = sgn * (nh @ m_)
    c = p.albedo * p.sun_color
    g = (sgn / ln)[:, None] * (m_[None, :] - (nh @ m_)[:, None] * nh)
    on = (f > 0) & (gr != 0)
    E = [B - C, C - A, A - B]
    for k in range(3):
        ck = (gt / ndotd)[:, None] * w[:, k:k + 1] * n
        ck = ck + np.where(on[:, None], (gr * c)[:, None] * np.cross(E[k], g), 0.0)
        np.add.at(grad, tv[:, k], ck)
    return grad


def test_forward_depth_bit_exact_and_adjoint_vs_fp64(ctx):
    import torch
    m, b, ent, sc, rays, d_rays, tsc, zero = _setup(ctx)
    p = diff_params(shadow_rays=False)
    target, _, ttape = tsc.forward(d_rays, zero, p)
    ttape.close()
    image, loss, tape = sc.forward(d_rays, target, p)
    grad = tape.backward().cpu().numpy()
    img = image.cpu().numpy()
    osc = O.OracleScene(O.ORC_STACK, m.vertices, b.tris, b.nodes, ent)
    hits = osc.closest(rays)
    hit = hits["t"] > 0
    assert hit.sum() > 5000
    assert np.array_equal(img[hit, 0].view(np.uint32), hits["t"][hit].view(np.uint32))
    assert (img[~hit] == 0).all()
    want = _host_grad(m, b, ent, rays, hits, img, target.cpu().numpy(), p)
    err = np.linalg.norm(grad - want) / np.linalg.norm(want)
    assert err < 1e-4, err
    big = np.abs(want) > 1e-3 * np.abs(want).max()
    rel = np.abs(grad[big] - want[big]) / np.abs(want[big])
    assert np.percentile(rel, 99) < 1e-3
    tloss = ((img[hit] - target.cpu().numpy()[hit]).astype(np.float64) ** 2).sum()
    assert abs(loss - tloss) <= 1e-4 * tloss


def test_adjoint_deterministic_and_recompute(ctx):
    m, b, ent, sc, rays, d_rays, tsc, zero = _setup(ctx)
    p = diff_params(shadow_rays=True)
    target, _, tt = tsc.forward(d_rays, zero, p)
    _, l1, t1 = sc.forward(d_rays, target, p)
    g1 = t1.backward().cpu().numpy()
    _, l2, t2 = sc.forward(d_rays, target, p)
    g2 = t2.backward().cpu().numpy()
    assert l1 == l2
    assert np.array_equal(g1.view(np.uint32), g2.view(np.uint32))
    pr = diff_params(shadow_rays=True, recompute=True)
    _, l3, t3 = sc.forward(d_rays, target, pr)
    assert t3.nbytes() < t1.nbytes()
    g3 = t3.backward().cpu().numpy()
    assert l3 == l1
    assert np.array_equal(g3.view(np.uint32), g1.view(np.uint32))


def test_adjoint_vs_central_differences(ctx):
    import torch
    m, b, ent, sc, rays, d_rays, tsc, zero = _setup(ctx, n=48, res=200)
    p = diff_params(shadow_rays=True)
    target, _, tt = tsc.forward(d_rays, zero, p)
    tgt = target.cpu().numpy().astype(np.float64)
    _, _, tape = sc.forward(d_rays, target, p)
    gz = tape.backward().cpu().numpy()[:, 2]
    base = torch.from_numpy(m.vertices["pos"][:, :3].copy()).cuda()
    h = 1e-3

    def render(dz, v):
        xyz = base.clone()
        xyz[v, 2] += dz
        sc.update_positions(xyz)
        img, _, t = sc.forward(d_rays, target, p, want_loss=False)
        t.close()
        tri = sc.closest(d_rays).cpu().numpy().view(R.HIT_DTYPE)["tri"]
        im = img.cpu().numpy().astype(np.float64)
        hitm = im[:, 0] > 0
        l = np.where(hitm, (im[:, 0] - tgt[:, 0]) ** 2 + (im[:, 1] - tgt[:, 1]) ** 2, 0.0)
        return l, tri

    rng = np.random.default_rng(3)
    cand = np.nonzero(np.abs(gz) > 1e-2 * np.abs(gz).max())[0]
    rng.shuffle(cand)
    checked, rels = 0, []
    for v in cand:
        lp, tp = render(+h, v)
        lm, tm = render(-h, v)
        if not np.array_equal(tp, tm):
            continue  # a pixel switches triangle: silhouette / edge crossing, not differentiable
        fd = (lp - lm).sum() / (2 * h)
        rels.append(abs(fd - gz[v]) / max(abs(fd), 1e-12))
        checked += 1
        if checked == 24:
            break
    sc.update_positions(base)
    assert checked >= 12
    rels = np.array(rels)
    assert np.median(rels) < 1e-3 and rels.max() < 1e-2, rels


def test_refit_tight_and_containing(ctx):
    import torch
    m, b, ent, sc, rays, d_rays, tsc, zero = _setup(ctx, n=32)
    xyz = torch.from_numpy(m.vertices["pos"][:, :3].copy()).cuda()
    xyz[:, 2] += torch.linspace(0, 0.3, xyz.shape[0], device="cuda")
    sc.update_positions(xyz)
    # the oracle on the moved vertices with its own (host) refit must agree with the GPU hits
    P = xyz.cpu().numpy()
    v2 = m.vertices.copy()
    v2["pos"][:, :3] = P
    nodes = b.nodes.copy()
    w = nodes.view(np.int32)

    def box(j):  # host refit, recursive over the stack layout
        out = []
        for s in (0, 8):
            if w[j, s + 3] == -1:
                lo, hi = box(w[j, s + 7])
            else:
                st, ln = w[j, s + 3] >> 4, w[j, s + 3] & 15
                pts = P[b.tris[st:st + ln, :3].ravel()]
                lo, hi = pts.min(0), pts.max(0)
            nodes[j, s:s + 3] = lo
            nodes[j, s + 4:s + 7] = hi
            out.append((lo, hi))
        return np.minimum(out[0][0], out[1][0]), np.maximum(out[0][1], out[1][1])

    box(0)
    osc = O.OracleScene(O.ORC_STACK, v2, b.tris, nodes, ent)
    want = osc.closest(rays)
    got = sc.closest(d_rays).cpu().numpy().view(np.uint32).reshape(-1, 8)
    assert np.array_equal(got, want.view(np.uint32).reshape(-1, 8))


def _host_refit(b, P):
    """The stack-layout BVH2 of b with every box recomputed from positions P (bottom-up, exact)."""
    nodes = b.nodes.copy()
    w = nodes.view(np.int32)

    def box(j):
        out = []
        for s in (0, 8):
            if w[j, s + 3] == -1:
                lo, hi = box(w[j, s + 7])
            else:
                st, ln = w[j, s + 3] >> 4, w[j, s + 3] & 15
                pts = P[b.tris[st:st + ln, :3].ravel()]
                lo, hi = pts.min(0), pts.max(0)
            nodes[j, s:s + 3] = lo
            nodes[j, s + 4:s + 7] = hi
            out.append((lo, hi))
        return np.minimum(out[0][0], out[1][0]), np.maximum(out[0][1], out[1][1])

    box(0)
    return nodes


def test_bvh8_refit_follows_vertex_moves(ctx):
    """rq_scene_update_positions refits the BVH8 (records and quantised boxes, topology kept): after
    three successive moves, small and large, BVH8q closest hits and occlusion equal the oracle's walk
    over the host-refitted BVH2 (or are proven by a brute force), in one-thread-per-ray and
    persistent launches at every group-stack depth, and equal a BVH8 built afresh from the moved
    positions."""
    import torch
    from .helpers import assert_equal_or_proven, assert_occlusion_equal_or_proven, same_records
    m = S.heightfield(64, seed=5)
    b = R.build_bvh(m.vertices, m.indices, m.mesh_ids, 0, layout=R.STACK)
    ent = R.identity_entity(0, b.nodes.shape[0])
    sc = ctx.scene(R.STACK, m.vertices, b.tris, b.nodes, ent)
    sc.build_bvh8()
    rays = np.concatenate([S.camera_rays(160, 120, **CAM),
                           S.sphere_rays(40_000, (-1.3, -1.3, -0.6), (1.3, 1.3, 1.0), seed=17)])
    d_rays = rays_to_device(rays)
    base = m.vertices["pos"][:, :3].astype(np.float64)
    rng = np.random.default_rng(3)
    for step, amp in enumerate((0.002, 0.05, 0.3)):
        P = base.copy()
        P[:, 2] += amp * np.sin(7.0 * base[:, 0] + step) * np.cos(5.0 * base[:, 1])
        P[:, :2] += rng.uniform(-0.3, 0.3, (len(P), 2)) * (2.0 / 64) * (amp > 0.01)
        P = P.astype(np.float32)
        sc.update_positions(torch.from_numpy(P).cuda())
        v2 = m.vertices.copy()
        v2["pos"][:, :3] = P
        osc = O.OracleScene(O.ORC_STACK, v2, b.tris, _host_refit(b, P), ent)
        want = osc.closest(rays)
        want_occ = osc.anyhit(rays)
        assert_hits_identical(hits_from_device(sc.closest(d_rays)), want, f"strict after move {step}")
        for kw in (dict(), dict(block_size=128, min_blocks=7, persistent=1),
                   dict(block_size=128, min_blocks=7, persistent=1, stack_depth=24)):
            got = hits_from_device(sc.closest(d_rays, layout=L.LAYOUT_BVH8Q, **kw))
            assert_equal_or_proven(got, want, osc, rays, what=f"bvh8 refit move {step} {kw}")
            occ = sc.anyhit(d_rays, layout=L.LAYOUT_BVH8Q, **kw).cpu().numpy()
            assert_occlusion_equal_or_proven(occ, want_occ, osc, rays, what=f"bvh8 refit any {step} {kw}")
        # a BVH8 built afresh over the moved positions (same BVH2 topology) finds the same hits
        fresh = ctx.scene(R.STACK, v2, b.tris, _host_refit(b, P), ent)
        fresh.build_bvh8()
        f_hits = hits_from_device(fresh.closest(d_rays, layout=L.LAYOUT_BVH8Q))
        assert same_records(got, f_hits).all()
        fresh.close()
        assert (want["t"] > 0).mean() > 0.2
    assert ctx.device_status() == 0
    sc.close()


def test_adjoint_on_bvh8_equals_bvh2(ctx):
    """rq_fwd / rq_bwd tracing the BVH8q give the BVH2 image, loss and gradients bit for bit, also
    after a refit, taped and in recompute mode."""
    import torch
    m, b, ent, sc, rays, d_rays, tsc, zero = _setup(ctx, n=48)
    sc.build_bvh8()
    p2 = diff_params(shadow_rays=True)
    target, _, t0 = tsc.forward(d_rays, zero, p2)
    t0.close()
    for moved in (False, True):
        if moved:
            xyz = torch.from_numpy(m.vertices["pos"][:, :3].copy()).cuda()
            xyz[:, 2] += 0.05 * torch.sin(11.0 * xyz[:, 0])
            sc.update_positions(xyz)
        for recompute in (False, True):
            img2, l2, tp2 = sc.forward(d_rays, target, diff_params(shadow_rays=True, recompute=recompute))
            g2 = tp2.backward().cpu().numpy()
            img8, l8, tp8 = sc.forward(d_rays, target, diff_params(shadow_rays=True, recompute=recompute,
                                                                   layout=L.LAYOUT_BVH8Q))
            g8 = tp8.backward().cpu().numpy()
            np.testing.assert_array_equal(img8.cpu().numpy().view(np.uint32), img2.cpu().numpy().view(np.uint32))
            assert l8 == l2
            np.testing.assert_array_equal(g8.view(np.uint32), g2.view(np.uint32))
            tp2.close()
            tp8.close()
    assert ctx.device_status() == 0
