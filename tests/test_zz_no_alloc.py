"""rq_gi_frame_noalloc — the GI pass for callers that cannot allocate device memory mid-frame.

Frame loops that must keep their timing, and host applications that own all device memory and
forbid plugins from calling cudaMalloc, cannot use rq_gi_frame (it grows its scratch on demand).
rq_gi_frame_noalloc runs the same kernels with their intermediates in a fixed device array.  These
tests call it through the C ABI twice in a row, with different parameters and launch forms, and
check each result against rq_gi_frame's on the same inputs bit for bit (the two run the same
arithmetic in the same order), and that the device's free memory does not move across a call.
The file is named to be collected last so a stop-at-first-failure run has already run everything
else.
"""
import ctypes as C

import numpy as np
import pytest

import candela_gb300 as R
from candela_gb300 import _lib as L
from candela_gb300 import scenes as S
from candela_gb300.engine import _opts, gi_params

from .helpers import rays_to_device, single_object

pytestmark = pytest.mark.gpu


def _noalloc(ctx, sc, d_rays, n, params, out, **launch):
    import torch
    stream = torch.cuda.current_stream(d_rays.device).cuda_stream
    o = _opts(**launch)
    st = L.lib().rq_gi_frame_noalloc(ctx.handle, sc.handle, L.ptr(d_rays), n, C.byref(params),
                                     C.byref(o), L.ptr(out), stream)
    L.check(st, ctx.handle)
    return out


def _free_bytes():
    import torch
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def test_noalloc_matches_gi_frame_two_calls(ctx):
    import torch
    bufs = single_object("hf64", R.STACK)
    sc = ctx.scene(R.STACK, *bufs)
    sc.set_materials(np.array([[0.7, 0.6, 0.5]], dtype=np.float32))
    sc.build_bvh8()

    # call 1: GI with shadow rays, 4 samples per pixel (49,152 secondary rays), BVH8q with the
    # persistent ray-queue launch
    rays1 = S.camera_rays(128, 96, **S.C1_CAMERA)
    p1 = gi_params(spp=4, seed=11, origin_offset=1e-3, shadow_rays=True, shadow_offset=1e-3)
    d1 = rays_to_device(rays1)
    launch1 = dict(layout=L.LAYOUT_BVH8Q, block_size=128, min_blocks=7, persistent=1)
    out1 = torch.empty((len(rays1), 4), dtype=torch.float32, device="cuda")
    want1 = sc.gi_frame(d1, p1, **launch1).cpu().numpy()
    free0 = _free_bytes()
    got1 = _noalloc(ctx, sc, d1, len(rays1), p1, out1, **launch1)
    assert _free_bytes() == free0, "the no-alloc pass changed the device's free memory"
    np.testing.assert_array_equal(got1.cpu().numpy().view(np.uint32), want1.view(np.uint32))

    # call 2 right after: other camera, 2 samples, no shadows, strict BVH2 one thread per ray —
    # must not see call 1's contents
    rays2 = S.camera_rays(160, 120, eye=(0.3, -2.0, 1.2), target=(0.0, 0.1, 0.0))
    p2 = gi_params(spp=2, seed=12, origin_offset=2e-3)
    d2 = rays_to_device(rays2)
    out2 = torch.empty((len(rays2), 4), dtype=torch.float32, device="cuda")
    want2 = sc.gi_frame(d2, p2).cpu().numpy()
    free0 = _free_bytes()
    got2 = _noalloc(ctx, sc, d2, len(rays2), p2, out2).cpu().numpy()
    assert _free_bytes() == free0, "the no-alloc pass changed the device's free memory"
    np.testing.assert_array_equal(got2.view(np.uint32), want2.view(np.uint32))
    assert np.abs(want2).sum() > 0 and not np.array_equal(got1.cpu().numpy()[: len(got2)], got2)

    # RTAO on the same array: any-hit AO rays
    p3 = gi_params(spp=1, seed=7, origin_offset=1e-3, ray_tmax=0.25, query=1)
    want3 = sc.gi_frame(d2, p3).cpu().numpy()
    got3 = _noalloc(ctx, sc, d2, len(rays2), p3, out2).cpu().numpy()
    np.testing.assert_array_equal(got3.view(np.uint32), want3.view(np.uint32))
    assert ctx.device_status() == 0


def test_noalloc_rejects_oversized_pass(ctx):
    import torch
    bufs = single_object("hf32", R.STACK)
    sc = ctx.scene(R.STACK, *bufs)
    rays = S.camera_rays(256, 256, **S.C1_CAMERA)  # 65,536 pixels x 2 spp > capacity
    out = torch.empty((len(rays), 4), dtype=torch.float32, device="cuda")
    with pytest.raises(R.RqError) as e:
        _noalloc(ctx, sc, rays_to_device(rays), len(rays), gi_params(spp=2), out)
    assert e.value.status == L.RQ_EINVAL
    assert L.NOALLOC_MAX_RAYS == 65536
