"""Failure detection without a GPU fault.

Device side: a bounded wait that cannot succeed (a decoupled look-back on a
predecessor that nothing publishes) gives up after its poll limit, latches
the timeout bit, and the host reads WFPT_ERR_TIMEOUT; the context stays
usable.  Host side: an injected allocation failure surfaces as
WFPT_ERR_OUT_OF_MEMORY and the renderer recovers once allocation works."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

WFPT_ERR_TIMEOUT = 4
WFPT_ERR_OUT_OF_MEMORY = 3


def _sort_still_works(wf, dev):
    import torch
    rng = np.random.default_rng(21)
    keys = rng.integers(0, 2**32, 100000, dtype=np.uint32)
    k = torch.from_numpy(keys.view(np.int32)).to(dev)
    v = torch.arange(100000, dtype=torch.int32, device=dev)
    wf.api.sort_pairs(k, v, 32)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(v.cpu().numpy(), order.astype(np.int32))
    assert wf.api.device_status() == 0


@pytest.mark.parametrize("which", [0, 1])
def test_lookback_wait_times_out(wf, dev, which):
    assert wf.api.device_status() == 0
    assert wf.api.selftest_wait_timeout(which) == WFPT_ERR_TIMEOUT
    assert wf.api.device_status() == 0  # the timeout bit was read and cleared
    _sort_still_works(wf, dev)


def test_injected_allocation_failure_and_recovery(wf, dev):
    import torch
    pos, nrm, idx = wf.api.generate_scene(0, 5, 4000)
    sc = wf.api.Scene(pos, idx)
    geom = wf.api.Geometry(pos, nrm, idx, device=dev)
    cam = wf.api.make_camera(position=(0.5, 0.5, 2.2), rotation_deg=(0.0, 0.0, 0.0), fov_deg=45.0, znear=0.001,
                             zfar=10.0)
    w, h = 64, 48
    cfg = dict(ray_type=wf.PATH_RAYS, recursion_depth=2, num_shadow_samples=2, shadow_radius=0.1,
               bvh_kind=wf.BVH8_Q8, sort_path_rays=1, reorder_path_rays=1, morton_kind=2)
    outs = []
    for inject in (True, False):
        r = wf.api.Renderer(**cfg)
        r.set_scene(sc, geom, (0.5, 1.6, 0.5), (0.53, 0.81, 0.98))
        px = torch.zeros((w * h, 4), dtype=torch.float32, device=dev)
        fp = torch.zeros((w * h, 4), dtype=torch.float32, device=dev)
        if inject:
            old = wf.api.tune_get("debug.fail_alloc_after")
            wf.api.tune_set("debug.fail_alloc_after", 3)
            try:
                with pytest.raises(wf.WfptError) as err:
                    r.render(cam, w, h, px, fp)
                assert err.value.status == WFPT_ERR_OUT_OF_MEMORY
            finally:
                wf.api.tune_set("debug.fail_alloc_after", old)
        r.render(cam, w, h, px, fp)  # recovers: the missing buffers are allocated now
        outs.append(fp.cpu().numpy())
        r.close()
    assert np.array_equal(outs[0].view(np.uint32), outs[1].view(np.uint32))
    assert wf.api.device_status() == 0
