"""First-bounce closest hits of the wavefront path at full scene scale.

pt_primary_hits returns every camera ray of a render and its closest hit, computed as
the render computes it: rasterised (raster_primary.cuh: each triangle visits the
samples inside its pixel rectangle and cone of directions) or traced through the
4-wide BVH. For the same rays both must give the same triangle and the same distance
bits, and both must be the reference traversal's answer (the oracle's restatement of
BinnedSAHBVH::Intersect, Core/Accel/BinnedSAHBVH.cpp:272-374, exact ties included).
The scenes are the 1.0M-triangle benchmark scene and the largest scene of the batched
workload (1.5M triangles, 825x441).
"""
import numpy as np
import pytest

import oracle
from petrichor_gb300 import capi, synth

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _hits(ctx, sid, cam, st, traversal):
    """Device tensors: rays (n, 6), triangle ids (n), distances (n)."""
    ctx.set_tuning(primary_traversal=traversal)
    try:
        n = st.width * st.height * st.spp
        rays = torch.empty((n, 6), dtype=torch.float32, device="cuda")
        tri = torch.empty(n, dtype=torch.int32, device="cuda")
        dist = torch.empty(n, dtype=torch.float32, device="cuda")
        ctx.primary_hits(sid, cam, st, rays.data_ptr(), tri.data_ptr(), dist.data_ptr())
        torch.cuda.synchronize()
        return rays, tri, dist
    finally:
        ctx.set_tuning()


def _scene(case):
    """The scene and its spp: every camera ray of a full render (one wave)."""
    if case == "benchmark_1M":
        return synth.spheres_grids(), 64      # 132.7M rays, 133 per triangle
    return synth.batch_instance(40), 256      # 93.1M rays, 62 per triangle


@pytest.mark.parametrize("case", ["benchmark_1M", "batch_1_5M"])
def test_rasterised_first_bounce_equals_traced_and_reference(gpu_ctx, case):
    sc, spp = _scene(case)
    st = capi.settings_from_scene(sc, capi.MODE_WAVEFRONT, seed=3, spp=spp)
    cam = capi.camera_from_scene(sc)
    sid = gpu_ctx.upload(sc)
    try:
        r_tr, t_tr, d_tr = _hits(gpu_ctx, sid, cam, st, 1)   # traced
        r_ra, t_ra, d_ra = _hits(gpu_ctx, sid, cam, st, 2)   # rasterised
    finally:
        gpu_ctx.release(sid)
    n = t_tr.numel()
    assert torch.equal(r_tr.view(torch.int32), r_ra.view(torch.int32))  # the same camera rays
    assert (t_ra >= 0).float().mean().item() > 0.2                       # the camera sees the scene
    bad = torch.nonzero((t_tr != t_ra) | (d_tr.view(torch.int32) != d_ra.view(torch.int32)))
    bad = bad.flatten().cpu().numpy()
    rng = np.random.default_rng(5)
    idx = np.unique(np.concatenate([rng.choice(n, 20000, replace=False), bad[:256]]))
    it = torch.from_numpy(idx).cuda()
    rays = r_tr[it].cpu().numpy()
    tt, dt = t_tr[it].cpu().numpy(), d_tr[it].cpu().numpy()
    tr, dr = t_ra[it].cpu().numpy(), d_ra[it].cpu().numpy()
    o = oracle.OracleScene(sc)
    ref_t, ref_d = o.trace(rays)
    detail = ""
    if bad.size:
        k = np.isin(idx, bad[:256])
        j = int(np.nonzero(k)[0][0])
        detail = (f"{bad.size} of {n} rays differ; of the first {int(k.sum())}, the traced hit is "
                  f"the reference's for {int((tt[k] == ref_t[k]).sum())}, the rasterised for "
                  f"{int((tr[k] == ref_t[k]).sum())}; e.g. ray {idx[j]} {rays[j].tolist()}: traced "
                  f"{tt[j]} {dt[j]!r}, rasterised {tr[j]} {dr[j]!r}, reference {ref_t[j]} {ref_d[j]!r}")
    assert bad.size == 0, detail
    assert np.array_equal(tt, ref_t)
    hit = ref_t >= 0
    assert np.array_equal(dt[hit].view(np.uint32), ref_d[hit].view(np.uint32))
