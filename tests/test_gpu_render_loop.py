"""The render loop (nerf/main/render.py:27-117) on the GPU: render_cameras
with a real NeRF on the device at a small frame size, its files checked
against the device render of the same cameras and the oracle's depth map."""
import importlib
import os

import numpy as np
import pytest
import torch

from test_render_loop import decode_png

pytestmark = pytest.mark.gpu


def test_render_cameras_on_device(ng, oracle, cuda, tmp_path):
    rl = importlib.import_module("nerf-tf2_gb300.render_loop")
    H, W = 20, 28
    K = ng.synthetic.intrinsic(H, W, 30.0)
    poses = rl.create_spherical_path(4.0, 60.0, 3)
    nerf = ng.NeRF(ng.make_params(), precision="bf16", coarse_params=ng.weights.glorot_blob(1),
                   fine_params=ng.weights.glorot_blob(2))
    bounds = rl.default_bounds(4.0)
    names = rl.render_cameras(nerf, poses, K, H, W, bounds, str(tmp_path), scale_factor=0.5, seed=4, chunk=256)
    nerf.coarse_model.check_device_errors()
    assert names == ["render_00000", "render_00001", "render_00002"]
    for name, c2w in zip(names, poses):
        fr = nerf.render_frame(H, W, K, c2w, bounds=bounds, seed=4, chunk=256)
        img = decode_png(os.path.join(tmp_path, "rgb", name + ".png"))
        assert np.array_equal(img, fr["image_u8"].cpu().numpy())
        depth = fr["depth"].cpu().numpy()
        d1 = np.load(os.path.join(tmp_path, "depth_type_1", name + ".npy"))
        d2 = np.load(os.path.join(tmp_path, "depth_type_2", name + ".npy"))
        acc = np.load(os.path.join(tmp_path, "acc_map", name + ".npy"))
        np.testing.assert_allclose(d1, oracle.create_depth_map(depth.reshape(-1), H, W, 0.5, "type_1"), rtol=1e-6)
        want2 = oracle.create_depth_map(depth.reshape(-1), H, W, 0.5, "type_2", K, c2w)
        np.testing.assert_allclose(d2, want2, atol=2e-5 * np.abs(want2).max())
        assert np.array_equal(acc, fr["acc"].cpu().numpy())
        assert 0.0 <= acc.min() and acc.max() <= 1.0 + 1e-6
