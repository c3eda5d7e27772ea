"""The hand-written backward (the gradient tf.GradientTape takes at
nerf/core/model.py:148-170) against the oracle's analytic gradients, which
tests/test_oracle_grad.py checks by finite differences in float64."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
F32, F64 = np.float32, np.float64


def dev(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def host(x):
    return x.detach().cpu().numpy()


def biased_blob(ng, seed):
    blob = ng.weights.glorot_blob(seed)
    rng = np.random.default_rng(seed + 99)
    for name, (ko, bo, i, o) in ng.weights.offsets().items():
        blob[bo:bo + o] = rng.uniform(-0.1, 0.1, o)
    return blob


def flat_grads(ng, g):
    parts = []
    for name, i, o in ng.weights.LAYERS:
        W, b = g[name]
        parts += [np.asarray(W).reshape(-1), np.asarray(b).reshape(-1)]
    return np.concatenate(parts)


def compare(ng, got, want, rel=2e-3, norm=False):
    """Layer by layer: max error relative to the layer's largest entry, or
    (norm=True) the relative L2 error of the layer's gradient."""
    for name, (ko, bo, i, o) in ng.weights.offsets().items():
        for lo, hi in ((ko, ko + i * o), (bo, bo + o)):
            w = want[lo:hi]
            if norm:
                err = np.linalg.norm(got[lo:hi] - w) / max(np.linalg.norm(w), 1e-12)
            else:
                err = np.abs(got[lo:hi] - w).max() / max(np.abs(w).max(), 1e-12)
            assert err < rel, (name, lo == bo, err)


@pytest.mark.parametrize("n", [300, 64])
def test_mlp_backward_vs_oracle(ng, oracle, cuda, n):
    blob = biased_blob(ng, 3)
    rng = np.random.default_rng(n)
    x = rng.uniform(-3, 3, (n, 3)).astype(F32)
    d = rng.normal(size=(n, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(F32)
    dr = rng.normal(size=(n, 3)).astype(F32)
    ds = rng.normal(size=(n,)).astype(F32)
    mlp = ng.get_coarse_or_fine_model("fine", params=blob)
    X, D = dev(x), dev(d)
    rgb, sig, acts = mlp.forward_train(X, D)
    r2, s2 = mlp((X, D))
    assert torch.equal(rgb, r2) and torch.equal(sig, s2)  # the tape does not change the forward
    g = torch.zeros(ng.weights.PARAM_COUNT, device="cuda")
    mlp.backward(acts, dev(dr), dev(ds), g)
    # the tape matches the oracle's fp32 forward
    _, _, a32 = oracle.mlp_forward(oracle.unpack_params(blob, F32), x, d, F32, cache=True)
    tape = oracle.acts_from_tape(host(acts), F32)
    for k in ("enc_xyz", "h0", "h4", "h7", "bott", "enc_dir", "h9"):
        np.testing.assert_allclose(tape[k], a32[k], atol=2e-4, rtol=1e-3, err_msg=k)
    # backward kernels against the float64 chain on the same tape (same ReLU masks)
    want = flat_grads(ng, oracle.mlp_backward_cached(oracle.unpack_params(blob, F64),
                                                     oracle.acts_from_tape(host(acts)), dr.astype(F64),
                                                     ds.astype(F64)))
    compare(ng, host(g), want, rel=1e-4)


def test_train_step_gradients_vs_oracle(ng, oracle, cuda):
    """Loss = MSE(coarse) + MSE(fine) (model.py:157-168): GPU gradients of
    both networks against the oracle's chain (compositing backward, MLP
    backward) on the same rays, uniforms and sample positions."""
    R = 48
    o, d, n, f = ng.synthetic.sphere_rays(R, 5)
    rng = np.random.default_rng(6)
    uc = rng.random((R, 64), dtype=F32)
    uf = rng.random((R, 128), dtype=F32)
    target = rng.random((R, 3), dtype=F32)
    bc, bf = biased_blob(ng, 11), biased_blob(ng, 12)
    p = ng.make_params()
    nerf = ng.NeRF(p, precision="fp32", coarse_params=bc, fine_params=bf, trans_mode=ng._lib.TRANS_CUMPROD)
    out = nerf.train_step(((dev(o), dev(d), dev(n), dev(f)), (dev(target),)), u_coarse=dev(uc),
                          u_fine=dev(uf), lr=0.0)
    gc, gf = (host(g) for g in nerf.gradients())
    # oracle chain in float64 on the float32 sample positions the kernels used
    cm = oracle.create_input_batch_coarse_model(p, o, d, n, f, uc)
    pc64 = oracle.unpack_params(bc, F64)
    rgb_c, sig_c = oracle.mlp_forward(pc64, cm["xyz_inputs"].astype(F64), cm["dir_inputs"].astype(F64), F64)
    pp_c = oracle.post_process_model_output(rgb_c, sig_c, cm["t_vals"].astype(F64))
    fm = oracle.create_input_batch_fine_model(p, o, d, pp_c["weights"].astype(F32), cm["bin_data"],
                                              cm["t_vals"], uf)
    pf64 = oracle.unpack_params(bf, F64)
    rgb_f, sig_f = oracle.mlp_forward(pf64, fm["xyz_inputs"].astype(F64), fm["dir_inputs"].astype(F64), F64)
    pp_f = oracle.post_process_model_output(rgb_f, sig_f, fm["t_vals"].astype(F64))
    lc, Gc = oracle.mse(target, pp_c["pred_rgb"])
    lf, Gf = oracle.mse(target, pp_f["pred_rgb"])
    assert abs(out["loss"] - (lc + lf)) < 1e-4 * (lc + lf)
    # (1) the oracle chain in float64 on this step's own tape: tight
    tape = nerf._train_state()["tape"]
    for key, pb, got in (("coarse", pc64, gc), ("fine", pf64, gf)):
        t, sig, rgb_s, acts, pred = (host(x).astype(F64) for x in tape[key])
        _, G = oracle.mse(target.astype(F64), pred)
        ds, dr = oracle.composite_backward(sig.reshape(-1), t, rgb_s, G)
        want = flat_grads(ng, oracle.mlp_backward_cached(pb, oracle.acts_from_tape(acts), dr, ds))
        compare(ng, got, want, rel=2e-3, norm=True)
    # (2) a fully independent float64 forward: fp32 encodings of frequencies
    #     up to 2^9 pi and ReLU masks flipping near zero move dense_0 by ~2%
    for G, t, rgb_s, sig, xyz, dirs, pb, got in (
            (Gc, cm["t_vals"], rgb_c, sig_c, cm["xyz_inputs"], cm["dir_inputs"], pc64, gc),
            (Gf, fm["t_vals"], rgb_f, sig_f, fm["xyz_inputs"], fm["dir_inputs"], pf64, gf)):
        ds, dr = oracle.composite_backward(sig[:, 0], t.astype(F64), rgb_s, G)
        want = flat_grads(ng, oracle.mlp_backward(pb, xyz.astype(F64), dirs.astype(F64), dr, ds))
        compare(ng, got, want, rel=5e-2, norm=True)


def test_training_reduces_loss(ng, cuda):
    """A few hundred steps on one batch of a fixed teacher's renders drive the
    loss down (Adam lr 5e-4 as in setup_model, model.py:413-418)."""
    p = ng.make_params()
    teacher = ng.NeRF(p, precision="fp32", seed=40)
    o, d, n, f = [torch.from_numpy(x).cuda() for x in ng.synthetic.sphere_rays(512, 7)]
    tgt = teacher.render(o, d, n, f, seed=3)["rgb"]
    student = ng.NeRF(p, precision="fp32", seed=50)
    first = None
    for i in range(150):
        out = student.train_step(((o, d, n, f), (tgt,)))
        first = out["loss"] if first is None else first
    assert out["loss"] < 0.5 * first, (first, out["loss"])
