"""hrt_build_accel_static: the BVH build that allocates nothing.

It serves callers that cannot call cudaMalloc (an arena or framework allocator
owns all device memory, or a latency-critical loop must not synchronise on an
allocation).  Through the C ABI, with caller-owned device buffers, its output must
equal the context build's (hrt_build_accel + hrt_get_bvh) bit for bit, on two calls
in a row of different sizes (the shared static scratch keeps the previous call's
contents, so the second call checks that what must start at zero is cleared).
This file is collected last so that a failure here leaves every other test run.
"""
import numpy as np
import pytest

from helios_gb300 import _hrt, scenes

pytestmark = pytest.mark.gpu


def _scene(seed, n_leaf, n_tri):
    a = scenes.homogeneous_canopy(n_leaves=n_leaf, leaf=0.2, domain=4, seed=seed)
    b = scenes.orchard(nx=1, ny=1, leaves_per_tree=n_tri, side=0.2, seed=seed + 1)
    return (np.concatenate([a.T, b.T]).astype(np.float32), np.concatenate([a.ptype, b.ptype]).astype(np.uint32),
            np.concatenate([a.twosided, b.twosided]))


def _static_build(lib, T, ty):
    import torch

    n = T.shape[0]
    dT = torch.from_numpy(T.reshape(-1)).cuda()
    dty = torch.from_numpy(ty.view(np.int32)).cuda()
    rec = torch.empty(n * 16, dtype=torch.float32, device="cuda")
    org = torch.empty(n * 16, dtype=torch.float32, device="cuda")
    nodes = torch.empty(max(n - 1, 1) * 16, dtype=torch.int32, device="cuda")
    codes = torch.empty(n, dtype=torch.int64, device="cuda")
    perm = torch.empty(n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = lib.hrt_build_accel_static(dT.data_ptr(), dty.data_ptr(), n, rec.data_ptr(), org.data_ptr(),
                                    nodes.data_ptr(), codes.data_ptr(), perm.data_ptr(), None)
    assert rc == _hrt.HRT_OK, rc
    return (codes.cpu().numpy().view(np.uint64), perm.cpu().numpy().view(np.uint32),
            nodes.cpu().numpy().view(np.uint32).reshape(-1, 16))


def test_static_build_matches_context_build(hrt_lib):
    pytest.importorskip("torch")
    ctx = _hrt.Context(0)
    for seed, n_leaf, n_tri in ((3, 9000, 7000), (5, 1500, 2500)):
        T, ty, ts = _scene(seed, n_leaf, n_tri)
        c1, p1, n1 = _static_build(hrt_lib, T, ty)
        ctx.update_geometry(T, ty, ts)
        ctx.build_accel()
        c2, p2, n2 = ctx.bvh()
        assert np.array_equal(c1, c2)
        assert np.array_equal(p1, p2)
        assert np.array_equal(n1[:, 12:14], n2[:, 12:14])
        assert np.array_equal(n1[:, :12].view(np.float32), n2[:, :12].view(np.float32))


def test_static_build_rejects_oversize(hrt_lib):
    n = 32769  # one above HRT_STATIC_MAX_PRIMS: rejected before any device work
    rc = hrt_lib.hrt_build_accel_static(1, 1, n, 1, 1, 1, 1, 1, None)
    assert rc == _hrt.HRT_EINVAL
