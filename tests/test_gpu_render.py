"""End-to-end parity of NeRF.forward (nerf/core/model.py:57-125) and of the fused
render with the CPU oracle on the same rays, weights and uniforms."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
F32, F64 = np.float32, np.float64


def dev(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def host(x):
    return x.detach().cpu().numpy()


@pytest.fixture(scope="module")
def case(ng):
    R = 96
    o, d, n, f = ng.synthetic.sphere_rays(R, 42)
    rng = np.random.default_rng(43)
    uc = rng.random((R, 64), dtype=F32)
    uf = rng.random((R, 128), dtype=F32)
    bc, bf = ng.weights.glorot_blob(1), ng.weights.glorot_blob(2)
    return R, o, d, n, f, uc, uf, bc, bf


@pytest.mark.parametrize("white_bg", [False, True])
def test_forward_fp32_vs_oracle(ng, oracle, cuda, case, white_bg):
    R, o, d, n, f, uc, uf, bc, bf = case
    p = ng.make_params(white_bg=white_bg)
    nerf = ng.NeRF(p, precision="fp32", coarse_params=bc, fine_params=bf,
                   trans_mode=ng._lib.TRANS_CUMPROD)
    cm, fm = nerf.forward(dev(o), dev(d), dev(n), dev(f), u_coarse=dev(uc), u_fine=dev(uf))
    wcm, wfm = oracle.nerf_forward(p, oracle.unpack_params(bc), oracle.unpack_params(bf),
                                   o, d, n, f, uc, uf, F32)
    for got, want in ((cm, wcm), (fm, wfm)):
        assert set(got) == {"acc_map", "weights", "pred_rgb", "pred_depth"}
        np.testing.assert_allclose(host(got["pred_rgb"]), want["pred_rgb"], atol=1e-4)
        np.testing.assert_allclose(host(got["acc_map"]), want["acc_map"], atol=1e-4)
        np.testing.assert_allclose(host(got["pred_depth"]), want["pred_depth"], atol=5e-4)
        np.testing.assert_allclose(host(got["weights"]), want["weights"], atol=1e-4)


def test_forward_fp32_vs_fp64_oracle(ng, oracle, cuda, case):
    R, o, d, n, f, uc, uf, bc, bf = case
    p = ng.make_params()
    nerf = ng.NeRF(p, precision="fp32", coarse_params=bc, fine_params=bf)
    _, fm = nerf.forward(dev(o), dev(d), dev(n), dev(f), u_coarse=dev(uc), u_fine=dev(uf))
    _, wfm = oracle.nerf_forward(p, oracle.unpack_params(bc, F64), oracle.unpack_params(bf, F64),
                                 o, d, n, f, uc.astype(F64), uf.astype(F64), F64)
    err = np.abs(host(fm["pred_rgb"]) - wfm["pred_rgb"]).max()
    assert err < 2e-3, err


@pytest.mark.parametrize("precision", ["fp32", "bf16", "fp8"])
def test_fused_render_matches_forward(ng, cuda, case, precision):
    R, o, d, n, f, uc, uf, bc, bf = case
    p = ng.make_params()
    nerf = ng.NeRF(p, precision=precision, coarse_params=bc, fine_params=bf)
    cm, fm = nerf.forward(dev(o), dev(d), dev(n), dev(f), u_coarse=dev(uc), u_fine=dev(uf))
    out = nerf.render(dev(o), dev(d), dev(n), dev(f), u_coarse=dev(uc), u_fine=dev(uf), chunk=40,
                      return_coarse=True)
    nerf.coarse_model.check_device_errors()
    assert torch.equal(out["rgb"], fm["pred_rgb"])
    assert torch.equal(out["depth"], fm["pred_depth"])
    assert torch.equal(out["acc"], fm["acc_map"])
    assert torch.equal(out["rgb_coarse"], cm["pred_rgb"])


def test_render_default_uniforms_deterministic(ng, cuda, case):
    R, o, d, n, f, uc, uf, bc, bf = case
    nerf = ng.NeRF(ng.make_params(), coarse_params=bc, fine_params=bf)
    a = nerf.render(dev(o), dev(d), dev(n), dev(f), seed=7)
    b = nerf.render(dev(o), dev(d), dev(n), dev(f), seed=7)
    c = nerf.render(dev(o), dev(d), dev(n), dev(f), seed=8)
    assert torch.equal(a["rgb"], b["rgb"])
    assert not torch.equal(a["rgb"], c["rgb"])


def test_render_frame_is_render_of_device_rays(ng, cuda):
    """NeRF.render_frame (the render loop, nerf/main/render.py:79-97) equals
    NeRF.render on get_rays_tf's rays, and its uint8 image is the clipped,
    truncated rgb."""
    H, W = 24, 40
    K = ng.synthetic.intrinsic(H, W, 33.3)
    pose = ng.synthetic.random_pose(5)
    nerf = ng.NeRF(ng.make_params(), precision="bf16", coarse_params=ng.weights.glorot_blob(1),
                   fine_params=ng.weights.glorot_blob(2))
    fr = nerf.render_frame(H, W, K, pose, bounds=(2.0, 6.0), seed=3, chunk=256)
    o, d = ng.ray_utils.get_rays_tf(H, W, K, pose)
    n = o.shape[0]
    ref = nerf.render(o, d, torch.full((n, 1), 2.0, device="cuda"), torch.full((n, 1), 6.0, device="cuda"),
                      seed=3, chunk=256)
    assert fr["rgb"].shape == (H, W, 3) and fr["depth"].shape == (H, W)
    assert torch.equal(fr["rgb"].reshape(-1, 3), ref["rgb"])
    assert torch.equal(fr["depth"].reshape(-1), ref["depth"])
    img = np.clip(host(ref["rgb"]) * 255.0, 0.0, 255.0).astype(np.uint8).reshape(H, W, 3)
    assert np.array_equal(host(fr["image_u8"]), img)


@pytest.fixture(scope="module")
def case1024(ng):
    R = 1024
    o, d, n, f = ng.synthetic.sphere_rays(R, 44)
    rng = np.random.default_rng(45)
    uc = rng.random((R, 64), dtype=F32)
    uf = rng.random((R, 128), dtype=F32)
    rng_b = np.random.default_rng(46)
    bc, bf = ng.weights.glorot_blob(1), ng.weights.glorot_blob(2)
    for blob in (bc, bf):  # non-zero biases, so that the bias paths are used
        for name, (ko, bo, i, o_) in ng.weights.offsets().items():
            blob[bo:bo + o_] = rng_b.uniform(-0.1, 0.1, o_)
    return R, o, d, n, f, uc, uf, bc, bf


def _row_err(got, want):
    return np.abs(np.asarray(got, F64) - np.asarray(want, F64)).reshape(len(got), -1).max(axis=1)


@pytest.mark.parametrize("precision", ["bf16", "fp8"])
def test_fused_render_lowp_vs_oracle(ng, oracle, cuda, case1024, precision):
    """The fused render (nerfgb_render_rays) in BF16 / FP8 on 1,024 rays
    against (1) the FP64 oracle of NeRF.forward: the format's own error,
    reported and bounded, and (2) the oracle's FP32 chain with the MLPs
    emulated in the kernels' arithmetic (oracle.mlp_forward_lowp): tight on
    all but a few rays. On those few the fine sampler's CDF, built from
    coarse weights that differ in the last FP32 bits, puts a draw on the
    other side of a bin edge; t is continuous across the edge, so such a ray
    moves by little."""
    R, o, d, n, f, uc, uf, bc, bf = case1024
    p = ng.make_params()
    nerf = ng.NeRF(p, precision=precision, coarse_params=bc, fine_params=bf,
                   trans_mode=ng._lib.TRANS_CUMPROD)
    out = nerf.render(dev(o), dev(d), dev(n), dev(f), u_coarse=dev(uc), u_fine=dev(uf), chunk=512)
    nerf.coarse_model.check_device_errors()
    got = {k: host(out[k]) for k in ("rgb", "depth", "acc")}
    _, w64 = oracle.nerf_forward(p, oracle.unpack_params(bc, F64), oracle.unpack_params(bf, F64),
                                 o, d, n, f, uc.astype(F64), uf.astype(F64), F64)
    e64 = _row_err(got["rgb"], w64["pred_rgb"])
    psnr64 = oracle.psnr(w64["pred_rgb"], got["rgb"])
    print(f"{precision} fused render vs FP64 oracle, 1024 rays: rgb max {e64.max():.2e} "
          f"p90 {np.quantile(e64, 0.9):.2e} mean {e64.mean():.2e}; PSNR {psnr64:.1f} dB")
    emul = lambda pp, x, dd: oracle.mlp_forward_lowp(pp, x, dd, precision)  # noqa: E731
    _, we = oracle.nerf_forward(p, oracle.unpack_params(bc, F32), oracle.unpack_params(bf, F32),
                                o, d, n, f, uc, uf, F32, mlp=emul)
    stats = {}
    for key, wkey in (("rgb", "pred_rgb"), ("acc", "acc_map"), ("depth", "pred_depth")):
        e = _row_err(got[key], we[wkey])
        stats[key] = e
        print(f"  vs emulation {key}: max {e.max():.2e} p96 {np.quantile(e, 0.96):.2e} mean {e.mean():.2e}")
    # The format's own error against FP64: this random-init network's density
    # is rough, so a fine draw that the coarse pass's rounding moves samples
    # a different value on a few rays; the mean and the PSNR bound the rest.
    mean64, min_psnr = {"bf16": (5e-3, 30.0), "fp8": (3e-2, 20.0)}[precision]
    assert e64.mean() < mean64 and psnr64 > min_psnr, (e64.mean(), psnr64)
    # Against the emulation the MLPs differ only in FP32 summation order and
    # the BF16/E4M3 roundings it flips (rgb 5e-4 max per sample, see
    # test_mlp_lowp_vs_emulation); the fine sampler then moves draws by the
    # coarse weights' difference, which the rough density amplifies. The
    # encoding's octaves come from a sincos every fourth octave and up to
    # three doublings (oracle.positional_encoding_kernel); CUDA's sincosf and
    # numpy's sin differ by a few ulps there, which the doublings multiply by
    # up to 8, so a few more BF16 roundings of the encoding flip.
    tight = {"bf16": 1.5e-3, "fp8": 5e-3}[precision]
    for key, scale in (("rgb", 1.0), ("acc", 1.0), ("depth", 10.0)):
        e = stats[key]
        assert np.quantile(e, 0.96) < tight * scale, (key, np.quantile(e, 0.96))
        assert e.mean() < 0.25 * tight * scale, (key, e.mean())


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_render_coarse_vs_oracle(ng, oracle, cuda, case, precision):
    """NeRF.render_coarse (the coarse pass, model.py:88-100) against the
    oracle's coarse pass: FP32 at the chain's FP32 tolerance, BF16 against
    the emulated-BF16 chain."""
    R, o, d, n, f, uc, uf, bc, bf = case
    p = ng.make_params()
    nerf = ng.NeRF(p, precision=precision, coarse_params=bc, fine_params=bf,
                   trans_mode=ng._lib.TRANS_CUMPROD)
    got = nerf.render_coarse(dev(o), dev(d), dev(n), dev(f), u_coarse=dev(uc))
    nerf.coarse_model.check_device_errors()
    mlp = None if precision == "fp32" else (lambda pp, x, dd: oracle.mlp_forward_lowp(pp, x, dd, "bf16"))
    want, _ = oracle.nerf_forward(p, oracle.unpack_params(bc), oracle.unpack_params(bf), o, d, n, f, uc, uf,
                                  F32, mlp=mlp)
    tol = 1e-4 if precision == "fp32" else 5e-4
    np.testing.assert_allclose(host(got["pred_rgb"]), want["pred_rgb"], atol=tol)
    np.testing.assert_allclose(host(got["acc_map"]), want["acc_map"], atol=tol)
    np.testing.assert_allclose(host(got["pred_depth"]), want["pred_depth"], atol=5 * tol)
    np.testing.assert_allclose(host(got["weights"]), want["weights"], atol=tol)
