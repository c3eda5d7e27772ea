"""Training-side kernels against the oracle: compositing backward, losses,
Adam, and the proposal network (forward, backward, training)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
F32, F64 = np.float32, np.float64


def dev(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def host(x):
    return x.detach().cpu().numpy()


@pytest.mark.parametrize("S,white_bg", [(64, False), (192, True), (7, False)])
def test_composite_backward_vs_oracle(ng, oracle, cuda, S, white_bg):
    rng = np.random.default_rng(S)
    R = 123
    t = np.sort(rng.uniform(2, 6, (R, S)), 1).astype(F32)
    sig = (rng.exponential(1.5, R * S) * (rng.random(R * S) < 0.8)).astype(F32)
    rgb = rng.random((R * S, 3), dtype=F32)
    G = rng.normal(size=(R, 3)).astype(F32)
    gw = rng.normal(size=(R, S)).astype(F32)
    want_s, want_c = oracle.composite_backward(sig.astype(F64), t.astype(F64), rgb.astype(F64),
                                               G.astype(F64), gw.astype(F64), white_bg)
    gs = torch.empty(R * S, device="cuda")
    gc = torch.empty(R * S, 3, device="cuda")
    d_sig, d_t, d_rgb, d_G, d_gw = dev(sig), dev(t), dev(rgb), dev(G), dev(gw)  # keep alive
    ng._lib.call("nerfgb_composite_backward", d_sig.data_ptr(), d_t.data_ptr(), d_rgb.data_ptr(),
                 d_G.data_ptr(), d_gw.data_ptr(), R, S, int(white_bg), gs.data_ptr(), gc.data_ptr(), None)
    scale = np.abs(want_s).max()
    # fp32 products/exp vs fp64: relative to the gradient's scale
    np.testing.assert_allclose(host(gs), want_s, atol=2e-5 * scale, rtol=1e-3)
    np.testing.assert_allclose(host(gc), want_c, atol=1e-6, rtol=1e-4)


def test_losses_vs_oracle(ng, oracle, cuda):
    rng = np.random.default_rng(0)
    p, y = rng.random((500, 3), dtype=F32), rng.random((500, 3), dtype=F32)
    loss = torch.zeros(1, device="cuda")
    grad = torch.empty(500, 3, device="cuda")
    d_p, d_y = dev(p), dev(y)
    ng._lib.call("nerfgb_mse_loss", d_p.data_ptr(), d_y.data_ptr(), 1500, ng._lib.F(1.0),
                 loss.data_ptr(), grad.data_ptr(), None)
    wl, wg = oracle.mse(y, p)
    assert abs(float(loss.item()) - wl) < 1e-6
    np.testing.assert_allclose(host(grad), wg, rtol=1e-5, atol=1e-9)
    wp, wt = rng.random((64, 64), dtype=F32), rng.random((64, 64), dtype=F32)
    loss.zero_()
    g2 = torch.empty(64, 64, device="cuda")
    d_wp, d_wt = dev(wp), dev(wt)
    ng._lib.call("nerfgb_envelope_loss", d_wp.data_ptr(), d_wt.data_ptr(), 64, 64, ng._lib.F(3.0),
                 loss.data_ptr(), g2.data_ptr(), None)
    wl, wg = oracle.prop_loss(wp, wt, 3.0)
    assert abs(float(loss.item()) - wl) < 1e-4 * wl
    np.testing.assert_allclose(host(g2), wg, rtol=1e-5, atol=1e-9)


def test_proposal_weights_vs_oracle(ng, oracle, cuda):
    rng = np.random.default_rng(4)
    R, S = 77, 64
    t = np.sort(rng.uniform(2, 6, (R, S)), 1).astype(F32)
    sig = rng.exponential(1.0, R * S).astype(F32)
    d_t, d_s = dev(t), dev(sig)
    w = host(ng.proposal.proposal_weights(d_s, d_t))
    want = oracle.proposal_weights(sig.astype(F64), t.astype(F64))
    np.testing.assert_allclose(w, want, atol=5e-6, rtol=5e-5)
    assert np.all(want.sum(1) < 1.0)  # the last bin no longer absorbs the rest
    gw = rng.normal(size=(R, S)).astype(F32)
    d_gw = dev(gw)
    gs = torch.empty(R * S, device="cuda")
    ng._lib.call("nerfgb_proposal_weights_backward", d_s.data_ptr(), d_t.data_ptr(), d_gw.data_ptr(), R, S,
                 gs.data_ptr(), None)
    ws, _ = oracle.composite_backward(sig.astype(F64), t.astype(F64), np.zeros((R * S, 3)), None,
                                      gw.astype(F64), False, last_delta=None)
    np.testing.assert_allclose(host(gs), ws, atol=2e-5 * np.abs(ws).max(), rtol=1e-3)


def test_adam_vs_oracle(ng, oracle, cuda):
    rng = np.random.default_rng(1)
    n = 1000
    var = rng.normal(size=n).astype(F32)
    m, v = np.zeros(n, F32), np.zeros(n, F32)
    tv, tm, tvv = dev(var), dev(m), dev(v)
    for step in range(1, 6):
        g = rng.normal(size=n).astype(F32)
        ng.proposal.adam_step(tv, tm, tvv, dev(g), step, 5e-4)
        var, m, v = oracle.apply_adam(var.astype(F64), m.astype(F64), v.astype(F64), g.astype(F64), step, 5e-4)
    np.testing.assert_allclose(host(tv), var, atol=1e-6)
    np.testing.assert_allclose(host(tm), m, atol=1e-6)


def test_proposal_forward_backward_vs_oracle(ng, oracle, cuda):
    rng = np.random.default_rng(3)
    blob = ng.proposal.glorot_blob(4)
    blob[2496:2560] = rng.uniform(-0.1, 0.1, 64)
    n = 1000
    x = rng.uniform(-4, 4, (n, 3)).astype(F32)
    prop = ng.ProposalNetwork(blob)
    sig = host(prop(dev(x)))[:, 0]
    want = oracle.prop_forward(blob, x, F64)
    np.testing.assert_allclose(sig, want, rtol=1e-4, atol=1e-5)
    ds = rng.normal(size=n).astype(F32)
    g = host(prop.backward(dev(x), dev(ds)))
    wg = oracle.prop_backward(blob.astype(F64), x.astype(F64), ds.astype(F64))
    np.testing.assert_allclose(g, wg, atol=1e-3 * np.abs(wg).max(), rtol=1e-3)


def _bf16(a):
    """Round-to-nearest-even to BF16, returned as float32."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


@pytest.mark.parametrize("n", [1000, 13])
def test_proposal_forward_bf16_vs_oracle(ng, oracle, cuda, n):
    """The tensor-core proposal forward (BF16 operands, FP32 accumulation)
    against (1) a float64 evaluation with the same BF16 roundings of the
    encoding, W1, h1 and W2 (checks the fragment layout: tight) and (2) the
    float64 oracle (BF16-sized tolerance)."""
    rng = np.random.default_rng(n)
    blob = ng.proposal.glorot_blob(4)
    blob[2496:2560] = rng.uniform(-0.1, 0.1, 64)
    blob[6656:6720] = rng.uniform(-0.1, 0.1, 64)
    x = rng.uniform(-4, 4, (n, 3)).astype(F32)
    prop = ng.ProposalNetwork(blob)
    sig = host(prop(dev(x), precision="bf16"))[:, 0]
    p = oracle.prop_unpack(blob, F32)
    enc = oracle.proposal_encoding_kernel(x)
    h1 = np.maximum(_bf16(enc).astype(F64) @ _bf16(p["W1"]).astype(F64) + p["b1"], 0)
    z2 = _bf16(h1.astype(F32)).astype(F64) @ _bf16(p["W2"]).astype(F64) + p["b2"]
    z3 = np.maximum(z2, 0) @ p["W3"].astype(F64) + p["b3"][0]
    emul = oracle.softplus(z3)
    np.testing.assert_allclose(sig, emul, rtol=2e-4, atol=2e-5)
    want = oracle.prop_forward(blob, x, F64)
    assert np.abs(sig - want).max() < 3e-2 * max(1.0, np.abs(want).max())
    assert np.abs(sig - host(prop(dev(x)))[:, 0]).max() > 0  # not the FP32 kernel


@pytest.fixture(scope="module")
def proposal_case(ng):
    """A band-limited sparse scene (one random-init network as coarse and
    fine), 200k training rays from 8 random 200x200 frames and the plain
    path's coarse-pass weight histograms as targets."""
    p = ng.make_params()
    blob = ng.synthetic.sparse_scene_blob(21, max_freq_log2=5)
    nerf = ng.NeRF(p, precision="bf16", coarse_params=blob, fine_params=blob)
    rays = [torch.from_numpy(x).cuda()
            for x in ng.synthetic.training_rays(100, 8, 25000, H=200, W=200, focal=277.78)]
    g = torch.Generator(device="cuda")
    g.manual_seed(0)
    uc = torch.rand(rays[0].shape[0], 64, device="cuda", generator=g)
    w_t = ng.proposal.coarse_histograms(nerf, *rays, uc)
    return nerf, blob, rays, uc, w_t


def test_proposal_training_reduces_loss_and_gains(ng, cuda, proposal_case):
    """Trained by the library's own kernels, the proposal beats what the
    method has without it (a flat PDF for the fine samples) against a dense
    64+512-sample render, and its histograms approach the coarse pass's."""
    nerf, blob, rays, uc, w_t = proposal_case
    prop = ng.ProposalNetwork(seed=7)
    trainer = ng.ProposalTrainer(prop, nerf.params, lr=3e-3)
    losses = trainer.fit(*rays, uc, w_t, steps=1500, batch=4096)
    assert losses[-1] < 0.5 * losses[0], losses
    # histogram agreement on rays that hit something
    idx = torch.arange(0, 20000, device="cuda")
    d = ng.create_input_batch_coarse_model(nerf.params, *(r[idx] for r in rays), u_vals=uc[idx])
    w = ng.proposal.proposal_weights(prop(d["xyz_inputs"]), d["t_vals"])
    wt = w_t[idx]
    hit = wt.sum(1) > 0.2
    pw = (w + 1e-5) / (w + 1e-5).sum(1, keepdim=True)
    pt = (wt + 1e-5) / (wt + 1e-5).sum(1, keepdim=True)
    tv = float((0.5 * (pw - pt).abs().sum(1))[hit].mean())
    assert tv < 0.3, tv
    # held-out frame, same uniforms for every path
    o, d, n, f = [torch.from_numpy(x).cuda() for x in ng.synthetic.frame_rays(999, H=200, W=200, focal=277.78)]
    gt = ng.NeRF(ng.make_params(N_fine=512), precision="fp32", coarse_params=blob,
                 fine_params=blob).render(o, d, n, f, seed=9)["rgb"]
    fast = nerf.render(o, d, n, f, seed=5, proposal=prop)["rgb"]
    flat_blob = np.zeros(ng.proposal.PARAM_COUNT, np.float32)
    flat_blob[-1] = -30.0  # density ~1e-13 everywhere: the fine sampler's PDF is flat (w + 1e-5)
    flat = ng.ProposalNetwork(flat_blob)
    base = nerf.render(o, d, n, f, seed=5, proposal=flat)["rgb"]
    nerf.fine_model.check_device_errors()
    p_trained, p_flat = ng.psnr(gt, fast), ng.psnr(gt, base)
    assert p_trained > p_flat + 0.5, (p_trained, p_flat)
