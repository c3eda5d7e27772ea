"""Parity of the ray kernels (coarse sampler, fine sampler, compositor,
encoder, uniforms) with the CPU oracle on the same inputs.

Integer and index outputs, and every float the reference computes with plain
IEEE arithmetic only (sampling, CDF, inverse transform, sort), are compared
bit-exactly. Transcendental results (exp, sin, cos) are compared within the
tolerances written in each test.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
F32, F64 = np.float32, np.float64


def dev(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def host(x):
    return x.detach().cpu().numpy()


def rays(ng, R, seed, vary_bounds=True):
    o, d, n, f = ng.synthetic.sphere_rays(R, seed)
    if vary_bounds:
        rng = np.random.default_rng(seed + 100)
        n = rng.uniform(0.5, 3.0, (R, 1)).astype(F32)
        f = (n + rng.uniform(0.5, 10.0, (R, 1))).astype(F32)
    return o, d, n, f


@pytest.mark.parametrize("lin_inv", [False, True])
@pytest.mark.parametrize("perturb", [True, False])
@pytest.mark.parametrize("S", [64, 7])
def test_coarse_sampler_bit_exact(ng, oracle, cuda, lin_inv, perturb, S):
    R = 777
    p = ng.make_params(N_coarse=S, perturb=perturb, lin_inv_depth=lin_inv)
    o, d, n, f = rays(ng, R, 1)
    u = np.random.default_rng(2).random((R, S), dtype=F32)
    got = ng.create_input_batch_coarse_model(p, dev(o), dev(d), dev(n), dev(f), u_vals=dev(u))
    want = oracle.create_input_batch_coarse_model(p, o, d, n, f, u)
    for k in ("xyz_inputs", "dir_inputs", "t_vals"):
        assert np.array_equal(host(got[k]), want[k]), k
    for k in ("bin_edges", "left_edges", "right_edges", "bin_widths"):
        assert np.array_equal(host(got["bin_data"][k]), want["bin_data"][k]), k


def test_coarse_sampler_empty(ng, cuda):
    p = ng.make_params()
    z3 = torch.zeros(0, 3, device=cuda)
    z1 = torch.zeros(0, 1, device=cuda)
    out = ng.create_input_batch_coarse_model(p, z3, z3, z1, z1, u_vals=torch.zeros(0, 64, device=cuda))
    assert out["xyz_inputs"].shape == (0, 3) and out["t_vals"].shape == (0, 64)


def _fine_inputs(ng, oracle, R, seed, Sc=64, lin_inv=True):
    p = ng.make_params(N_coarse=Sc, lin_inv_depth=lin_inv)
    o, d, n, f = rays(ng, R, seed)
    rng = np.random.default_rng(seed + 7)
    uc = rng.random((R, Sc), dtype=F32)
    cm = oracle.create_input_batch_coarse_model(p, o, d, n, f, uc)
    w = rng.random((R, Sc)).astype(F32) ** 4
    w[::5] = 0.0                                  # all-transparent rays
    w[1::7] = 0.0
    w[1::7, Sc // 3] = 1.0                        # one-hot rays
    return p, o, d, n, f, cm, w, rng


@pytest.mark.parametrize("Sf", [128, 33])
def test_fine_sampler_bit_exact(ng, oracle, cuda, Sf):
    R = 517
    p, o, d, n, f, cm, w, rng = _fine_inputs(ng, oracle, R, 3)
    p.sampling.N_fine = Sf
    u = rng.random((R, Sf), dtype=F32)
    # u exactly on an inner CDF edge (searchsorted side='right', :363), u = 0, u -> 1-
    wp = w + F32(1e-5)
    pdf = wp / oracle.seq_sum(wp * cm["bin_data"]["bin_widths"])[:, None]
    agg = oracle.seq_cumsum(pdf * cm["bin_data"]["bin_widths"])
    u[:, 0] = agg[:, 20]
    u[:, 1] = 0.0
    u[:, 2] = np.nextafter(F32(1), F32(0))
    u[:, 3] = u[:, 4]  # duplicate fine samples -> equal t, stable order
    want = oracle.create_input_batch_fine_model(p, o, d, w, cm["bin_data"], cm["t_vals"], u,
                                                return_indices=True)
    bd = {k: dev(v) for k, v in cm["bin_data"].items()}
    bd["left_edges"] = dev(cm["bin_data"]["bin_edges"])[:, :-1]  # strided view, as produced
    got = ng.create_input_batch_fine_model(p, dev(o), dev(d), dev(w), bd, dev(cm["t_vals"]),
                                           u_vals=dev(u), return_indices=True)
    assert np.array_equal(host(got["piece_idxs"]), want["piece_idxs"])
    assert np.array_equal(host(got["sort_perm"]), want["sort_perm"])
    assert np.array_equal(host(got["t_vals"]), want["t_vals"])
    assert np.array_equal(host(got["xyz_inputs"]), want["xyz_inputs"])
    assert np.array_equal(host(got["dir_inputs"]), want["dir_inputs"])


@pytest.mark.parametrize("Sf", [128, 33, 256, 512])
def test_fine_sampler_sort_paths(ng, oracle, cuda, Sf):
    """The stable sort of concat(t_c, t_f) (ray_utils.py:380-385) on its fast
    path (non-decreasing t_c, no NaN: bitonic sort of the fine draws, then a
    merge) and its fallback (rank sort), bit-exact: ties between coarse and
    fine depths, ties among fine draws, unsorted coarse depths, NaN."""
    R = 200
    p, o, d, n, f, cm, w, rng = _fine_inputs(ng, oracle, R, 11)
    p.sampling.N_fine = Sf
    u = rng.random((R, Sf), dtype=F32)
    u[:, 1] = 0.0                       # t_f = near ...
    u[:, 2] = u[:, 3] = u[:, 4]         # fine ties
    t_c = cm["t_vals"].copy()
    t_c[20:40, 0] = cm["bin_data"]["bin_edges"][20:40, 0]   # ... = t_c[0]: coarse/fine ties
    t_c[40:50, 5] = t_c[40:50, 6]                           # coarse ties
    t_c[0:10] = t_c[0:10, ::-1]                             # unsorted: rank-sort fallback
    t_c[10:15, 7] = np.nan                                  # NaN: fallback, NaN last
    u[15:18, 9] = np.nan
    want = oracle.create_input_batch_fine_model(p, o, d, w, cm["bin_data"], t_c, u, return_indices=True)
    got = ng.create_input_batch_fine_model(p, dev(o), dev(d), dev(w),
                                           {k: dev(v) for k, v in cm["bin_data"].items()},
                                           dev(t_c), u_vals=dev(u), return_indices=True)
    assert np.array_equal(host(got["sort_perm"]), want["sort_perm"])
    np.testing.assert_array_equal(host(got["t_vals"]), want["t_vals"])
    np.testing.assert_array_equal(host(got["xyz_inputs"]), want["xyz_inputs"])


def test_fine_sampler_pdf_mask(ng, oracle, cuda):
    """pdf < 1e-8 (ray_utils.py:372-373): zero weights over huge bins."""
    R = 40
    p = ng.make_params(lin_inv_depth=False)
    o = np.zeros((R, 3), F32)
    d = np.tile(np.array([[0, 0, 1]], F32), (R, 1))
    n = np.ones((R, 1), F32)
    f = np.full((R, 1), 1e12, F32)
    cm = oracle.create_input_batch_coarse_model(p, o, d, n, f, np.full((R, 64), 0.5, F32))
    w = np.zeros((R, 64), F32)
    u = np.random.default_rng(0).random((R, 128), dtype=F32)
    want = oracle.create_input_batch_fine_model(p, o, d, w, cm["bin_data"], cm["t_vals"], u,
                                                return_indices=True)
    got = ng.create_input_batch_fine_model(p, dev(o), dev(d), dev(w),
                                           {k: dev(v) for k, v in cm["bin_data"].items()},
                                           dev(cm["t_vals"]), u_vals=dev(u), return_indices=True)
    assert np.array_equal(host(got["t_vals"]), want["t_vals"])
    assert np.array_equal(host(got["piece_idxs"]), want["piece_idxs"])


@pytest.mark.parametrize("S", [64, 192, 256, 5])
@pytest.mark.parametrize("white_bg", [False, True])
def test_composite_vs_oracle(ng, oracle, cuda, S, white_bg):
    rng = np.random.default_rng(S)
    R = 301
    t = np.sort(rng.uniform(2, 6, (R, S)), axis=1).astype(F32)
    sig = (rng.exponential(3.0, (R * S, 1)) * (rng.random((R * S, 1)) < 0.7)).astype(F32)
    sig[:S] = 0.0          # a transparent ray
    sig[S + 3] = 1e9       # an opaque sample
    rgb = rng.random((R * S, 3), dtype=F32)
    want32 = oracle.post_process_model_output(rgb, sig, t, white_bg)
    want64 = oracle.post_process_model_output(rgb.astype(F64), sig.astype(F64), t.astype(F64),
                                              white_bg)
    for mode in (ng._lib.TRANS_CUMPROD, ng._lib.TRANS_LOGSUM):
        got = ng.post_process_model_output(dev(rgb), dev(sig), dev(t), white_bg, trans_mode=mode)
        for k in ("weights", "pred_rgb", "pred_depth", "acc_map"):
            g = host(got[k])
            # tolerance: fp32 exp/log ulps and a different product order
            np.testing.assert_allclose(g, want32[k], atol=5e-6 * (6 if k == "pred_depth" else 1),
                                       rtol=5e-5, err_msg=f"{k} mode={mode}")
            np.testing.assert_allclose(g, want64[k], atol=1e-5 * (6 if k == "pred_depth" else 1),
                                       rtol=1e-4, err_msg=f"{k} vs fp64 mode={mode}")


def test_compute_weights_and_alpha(ng, oracle, cuda):
    rng = np.random.default_rng(1)
    R, S = 64, 64
    t = np.sort(rng.uniform(2, 6, (R, S)), axis=1).astype(F32)
    sig = rng.exponential(2.0, (R * S, 1)).astype(F32)
    w = host(ng.compute_weights(dev(sig), dev(t), S))
    np.testing.assert_allclose(w, oracle.compute_weights(sig, t, S), atol=5e-6, rtol=5e-5)
    diffs = rng.uniform(0, 0.2, (R, S)).astype(F32)
    a = host(ng.sigma_to_alpha(dev(sig.reshape(R, S)), dev(diffs)))
    np.testing.assert_allclose(a, oracle.sigma_to_alpha(sig.reshape(R, S), diffs), atol=2e-7,
                               rtol=1e-6)


def test_long_ray_logsum_drift(ng, oracle, cuda):
    """2048 samples of low density: the compensated log-sum stays closer to
    the fp64 transmittance than the fp32 product."""
    S, R = 2048, 8
    t = np.tile(np.linspace(2, 6, S, dtype=F32), (R, 1))
    sig = np.full((R * S, 1), 0.05, F32)
    rgb = np.full((R * S, 3), 0.5, F32)
    want = oracle.post_process_model_output(rgb.astype(F64), sig.astype(F64), t.astype(F64))
    errs = {}
    for mode in (ng._lib.TRANS_CUMPROD, ng._lib.TRANS_LOGSUM):
        got = ng.post_process_model_output(dev(rgb), dev(sig), dev(t), trans_mode=mode)
        errs[mode] = np.abs(host(got["weights"]) - want["weights"]).max()
    assert errs[ng._lib.TRANS_LOGSUM] <= errs[ng._lib.TRANS_CUMPROD] * 1.5 + 1e-9


@pytest.mark.parametrize("L", [10, 4])
def test_encoder_vs_oracle(ng, oracle, cuda, L):
    rng = np.random.default_rng(L)
    x = rng.uniform(-4.5, 4.5, (1001, 3)).astype(F32)
    got = host(ng.PositionalEncoder(L)(dev(x)))
    want = oracle.positional_encoding(x, L)
    assert np.array_equal(got[:, :3], x)
    # sinf/cosf of identical fp32 arguments: a few ulp apart
    np.testing.assert_allclose(got, want, atol=1e-6, rtol=0)


def test_uniforms_match_philox(ng, oracle, cuda):
    ng.set_seed(1234)
    a = host(ng.ray_utils.uniform((37, 64)))
    b = host(ng.ray_utils.uniform((5,)))
    assert np.array_equal(a.reshape(-1), oracle.philox_uniform(1234, 0, 37 * 64))
    assert np.array_equal(b, oracle.philox_uniform(1234, 37 * 64, 5))


@pytest.mark.parametrize("H,W", [(800, 800), (7, 13), (1, 1)])
def test_get_rays_bit_exact(ng, oracle, cuda, H, W):
    """get_rays_tf (ray_utils.py:53-106) on the device, bit-exact against the
    float32 restatement."""
    K = ng.synthetic.intrinsic(H, W, 1111.111 * W / 800)
    pose = ng.synthetic.random_pose(H * 31 + W)
    o, d = ng.ray_utils.get_rays_tf(H, W, K, pose)
    wo, wd = oracle.get_rays_tf(H, W, K, pose)
    assert o.shape == (H * W, 3) and d.shape == (H * W, 3)
    assert np.array_equal(host(d), wd)
    assert np.array_equal(host(o), wo)


def test_sample_mode_batch_bit_exact(ng, oracle, cuda):
    """The sample-mode map function (base_dataset.py:555-621) on the device
    with supplied indices, bit-exact: rays, bounds, rgb = img / 255; an
    out-of-range index gives zeros."""
    H, W, B = 30, 50, 777
    rng = np.random.default_rng(2)
    img = rng.integers(0, 256, (H, W, 3), dtype=np.uint8)
    K = ng.synthetic.intrinsic(H, W, 41.0)
    pose = ng.synthetic.random_pose(8)
    idxs = rng.integers(0, H * W, B).astype(np.int32)
    idxs[:3] = [0, H * W - 1, W]
    (o, d, n, f), (rgb,) = ng.ray_utils.sample_mode_batch(img, pose, (2.0, 6.0), K, B, idxs=idxs)
    (wo, wd, wn, wf), (wrgb,) = oracle.sample_mode_batch(img, pose, (2.0, 6.0), K, idxs)
    for got, want in ((o, wo), (d, wd), (n, wn), (f, wf), (rgb, wrgb)):
        assert np.array_equal(host(got), want)
    bad = idxs.copy()
    bad[5] = -1
    bad[6] = H * W
    (o2, d2, n2, f2), (rgb2,) = ng.ray_utils.sample_mode_batch(img, pose, (2.0, 6.0), K, B, idxs=bad)
    assert not host(d2)[5:7].any() and not host(rgb2)[5:7].any() and not host(n2)[5:7].any()


def test_uniform_int_matches_philox(ng, oracle, cuda):
    """Indices drawn from the library's Philox stream: (word * maxval) >> 32
    of the same words as the float uniforms, in [0, maxval)."""
    n, maxval, seed, off = 10001, 640000, 1234, 8
    out = torch.empty(n, dtype=torch.int32, device="cuda")
    ng._lib.call("nerfgb_uniform_int", ctypes.c_ulonglong(seed), ctypes.c_ulonglong(off), n, maxval,
                 out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    want = oracle.philox_uniform_int(seed, off, n, maxval)
    got = host(out)
    assert np.array_equal(got, want)
    assert got.min() >= 0 and got.max() < maxval
    (o, d, _, _), _ = ng.ray_utils.sample_mode_batch(np.zeros((800, 800, 3), np.uint8), ng.synthetic.random_pose(1),
                                                       (2.0, 6.0), ng.synthetic.intrinsic(), 4096, seed=7)
    assert torch.isfinite(d).all() and o.shape == (4096, 3)


@pytest.mark.parametrize("map_type", ["type_1", "type_2"])
def test_create_depth_map(ng, oracle, cuda, map_type):
    """create_depth_map (ray_utils.py:108-135): type_1 to float32 rounding,
    type_2 (float32 rays and points against the reference's float64) within
    2e-5 relative."""
    H, W = 20, 31
    rng = np.random.default_rng(4)
    depth = rng.uniform(2.0, 6.0, H * W).astype(F32)
    K = ng.synthetic.intrinsic(H, W, 27.0)
    pose = ng.synthetic.random_pose(9)
    got = host(ng.ray_utils.create_depth_map(dev(depth), H, W, 0.5, map_type, intrinsic=K, C_to_W2=pose))
    want = oracle.create_depth_map(depth, H, W, 0.5, map_type, intrinsic=K, C_to_W2=pose)
    assert got.shape == (H, W)
    np.testing.assert_allclose(got, want, rtol=2e-5, atol=2e-5)
