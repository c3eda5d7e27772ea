"""Host-side logic of the package (no GPU): parameter layout, config, synthetic
ray geometry, and the error behaviour of the Python mirror without a device."""
import numpy as np
import pytest


def test_weights_layout_roundtrip(ng):
    blob = ng.weights.glorot_blob(3)
    assert blob.dtype == np.float32 and blob.size == ng.weights.PARAM_COUNT
    d = ng.weights.to_dict(blob, "fine")
    assert d["fine/dense_5/kernel:0"].shape == (319, 256)
    assert d["fine/dense_9/kernel:0"].shape == (283, 128)
    assert d["fine/sigma/kernel:0"].shape == (256, 1)
    assert d["fine/rgb/bias:0"].shape == (3,)
    assert np.array_equal(ng.weights.from_dict(d, "fine"), blob)


def test_glorot_limits(ng):
    d = ng.weights.to_dict(ng.weights.glorot_blob(0))
    for name, i, o in ng.weights.LAYERS:
        W = d[f"coarse/{name}/kernel:0"]
        lim = np.sqrt(6.0 / (i + o))
        assert np.abs(W).max() <= lim
        assert np.all(d[f"coarse/{name}/bias:0"] == 0)


def test_make_params_defaults(ng):
    p = ng.make_params()
    assert (p.sampling.N_coarse, p.sampling.N_fine) == (64, 128)
    assert p.sampling.perturb and p.sampling.lin_inv_depth and not p.system.white_bg


def test_sphere_rays_geometry(ng):
    o, d, n, f = ng.synthetic.sphere_rays(1000, 0)
    assert o.dtype == np.float32 and o.shape == (1000, 3) and n.shape == (1000, 1)
    np.testing.assert_allclose(np.linalg.norm(o, axis=1), 4.0, rtol=1e-6)
    np.testing.assert_allclose(np.linalg.norm(d, axis=1), 1.0, rtol=1e-6)
    cosang = -np.sum(o * d, axis=1) / 4.0
    assert cosang.min() > 0.9  # directions point at the centre
    assert np.all(n == 2.0) and np.all(f == 6.0)


def test_frame_rays_pinhole(ng):
    o, d, n, f = ng.synthetic.frame_rays(1, H=40, W=30, focal=50.0)
    assert o.shape == (1200, 3)
    # centre pixel looks at the origin (camera z towards the centre)
    K = ng.synthetic.intrinsic(40, 30, 50.0)
    assert K[0, 2] == 15.0
    c = d[20 * 30 + 15]
    np.testing.assert_allclose(c, -o[0] / np.linalg.norm(o[0]), atol=1e-6)


def test_look_at_pose_is_rotation(ng):
    P = ng.synthetic.look_at_pose(0.3, 1.1)
    R = P[:3, :3]
    np.testing.assert_allclose(R.T @ R, np.eye(3), atol=1e-12)
    np.testing.assert_allclose(np.linalg.norm(P[:3, 3]), 4.0)


def test_no_device_raises_loudly(ng):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is visible")
    with pytest.raises(RuntimeError, match="CUDA device"):
        ng.PositionalEncoder(10)(np.zeros((4, 3), np.float32))
