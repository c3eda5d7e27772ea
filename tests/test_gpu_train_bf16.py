"""BF16 training (tensor-core GEMMs, FP32 master weights): the tape of the
BF16 forward and the BF16 backward against the oracle's float64 chain on the
same tape (the gradient tf.GradientTape takes at nerf/core/model.py:148-170)."""
import numpy as np
import pytest
import torch

from test_gpu_backward import biased_blob, compare, dev, flat_grads, host

pytestmark = pytest.mark.gpu
F32, F64 = np.float32, np.float64


def tape64(acts):
    """The BF16 tape (int16 bits) as float64."""
    assert acts.dtype == torch.int16
    return acts.view(torch.bfloat16).float().cpu().numpy().astype(F64)


@pytest.mark.parametrize("n", [300, 2048])
def test_mlp_backward_bf16_vs_oracle(ng, oracle, cuda, n):
    blob = biased_blob(ng, 3)
    rng = np.random.default_rng(n)
    x = rng.uniform(-3, 3, (n, 3)).astype(F32)
    d = rng.normal(size=(n, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(F32)
    dr = rng.normal(size=(n, 3)).astype(F32)
    ds = rng.normal(size=(n,)).astype(F32)
    mlp = ng.get_coarse_or_fine_model("fine", params=blob, precision="bf16")
    X, D = dev(x), dev(d)
    rgb, sig, acts = mlp.forward_train(X, D, precision="bf16")
    r2, s2 = mlp((X, D))
    mlp.check_device_errors()
    assert torch.equal(rgb, r2) and torch.equal(sig, s2)  # the tape does not change the forward
    # the tape: BF16 activations within BF16 rounding of the fp32 oracle's
    # (relative L2 per activation, 8 layers of 8-bit-mantissa operands)
    _, _, a32 = oracle.mlp_forward(oracle.unpack_params(blob, F32), x, d, F32, cache=True)
    tape = oracle.acts_from_tape(tape64(acts))
    for k in ("enc_xyz", "h0", "h4", "h7", "bott", "enc_dir", "h9"):
        err = np.linalg.norm(tape[k] - a32[k]) / np.linalg.norm(a32[k])
        assert err < 2e-2, (k, err)
    g = torch.zeros(ng.weights.PARAM_COUNT, device="cuda")
    mlp.backward(acts, dev(dr), dev(ds), g)
    # float64 chain on the same tape (same ReLU masks); the GPU rounds dZ and
    # W to BF16 for every product (8-bit mantissa, ~10 layers deep)
    want = flat_grads(ng, oracle.mlp_backward_cached(oracle.unpack_params(blob, F64), tape, dr.astype(F64),
                                                     ds.astype(F64)))
    compare(ng, host(g), want, rel=3e-2, norm=True)
    # and distinctly closer than zero / a scaled copy would be: the heads are FP32
    for name in ("rgb", "sigma"):
        ko, bo, i, o = ng.weights.offsets()[name]
        w = want[ko:ko + i * o]
        assert np.linalg.norm(host(g)[ko:ko + i * o] - w) / np.linalg.norm(w) < 1e-4, name


def test_train_step_bf16_gradients_vs_oracle(ng, oracle, cuda):
    R = 48
    o, d, n, f = ng.synthetic.sphere_rays(R, 5)
    rng = np.random.default_rng(6)
    uc = rng.random((R, 64), dtype=F32)
    uf = rng.random((R, 128), dtype=F32)
    target = rng.random((R, 3), dtype=F32)
    bc, bf = biased_blob(ng, 11), biased_blob(ng, 12)
    p = ng.make_params()
    nerf = ng.NeRF(p, precision="bf16", coarse_params=bc, fine_params=bf, trans_mode=ng._lib.TRANS_CUMPROD)
    out = nerf.train_step(((dev(o), dev(d), dev(n), dev(f)), (dev(target),)), u_coarse=dev(uc),
                          u_fine=dev(uf), lr=0.0)
    nerf.coarse_model.check_device_errors()
    assert np.isfinite(out["loss"])
    gc, gf = (host(g) for g in nerf.gradients())
    tape = nerf._train_state()["tape"]
    for key, blob, got in (("coarse", bc, gc), ("fine", bf, gf)):
        t, sig, rgb_s, acts, pred = tape[key]
        t, sig, rgb_s, pred = (host(x).astype(F64) for x in (t, sig, rgb_s, pred))
        _, G = oracle.mse(target.astype(F64), pred)
        dsig, drgb = oracle.composite_backward(sig.reshape(-1), t, rgb_s, G)
        want = flat_grads(ng, oracle.mlp_backward_cached(oracle.unpack_params(blob, F64),
                                                         oracle.acts_from_tape(tape64(acts)), drgb, dsig))
        compare(ng, got, want, rel=3e-2, norm=True)


def test_train_bf16_reduces_loss(ng, cuda):
    """Twenty BF16 steps on one batch lower the loss (Keras Adam, lr 5e-4)."""
    R = 1024
    rays = [dev(x) for x in ng.synthetic.sphere_rays(R, 9)]
    teacher = ng.NeRF(ng.make_params(), precision="fp32", seed=1)
    target = teacher.render(*rays, seed=3)["rgb"]
    student = ng.NeRF(ng.make_params(), precision="bf16", seed=2)
    losses = [student.train_step((tuple(rays), (target,)))["loss"] for _ in range(20)]
    student.coarse_model.check_device_errors()
    assert all(np.isfinite(losses))
    assert losses[-1] < 0.8 * losses[0], losses


def test_train_step_resumes_loaded_adam_state(ng, oracle, cuda):
    """NeRF.load_optimizer_state (what load_model reads from the reference's
    <tag>_optimizer.npz) sets the step and the m/v slots; the next train_step
    is Adam step t+1 from them (model.py:246-276, then :171)."""
    p = ng.make_params()
    nerf = ng.NeRF(p, precision="fp32", seed=60)
    rays = [dev(x) for x in ng.synthetic.sphere_rays(256, 9)]
    target = torch.rand(256, 3, device="cuda", generator=torch.Generator(device="cuda").manual_seed(1))
    rng = np.random.default_rng(2)
    P = ng.weights.PARAM_COUNT
    st = {"step": 41, "m": {k: (rng.normal(size=P) * 1e-3).astype(F32) for k in ("coarse", "fine")},
          "v": {k: (rng.random(P) * 1e-6).astype(F32) for k in ("coarse", "fine")}}
    nerf.load_optimizer_state(st)
    before = [host(m.params).astype(F64) for m in (nerf.coarse_model, nerf.fine_model)]
    uc = dev(rng.random((256, 64), dtype=F32))
    uf = dev(rng.random((256, 128), dtype=F32))
    nerf.train_step((tuple(rays), (target,)), u_coarse=uc, u_fine=uf, lr=1e-3)
    grads = [host(g).astype(F64) for g in nerf.gradients()]
    for k, (name, model) in enumerate((("coarse", nerf.coarse_model), ("fine", nerf.fine_model))):
        want, _, _ = oracle.apply_adam(before[k], st["m"][name].astype(F64), st["v"][name].astype(F64), grads[k],
                                       42, 1e-3)
        # FP32 Adam against float64: where v is tiny, m / (sqrt(v) + eps) amplifies
        # FP32 rounding; 2e-3 of the step size
        np.testing.assert_allclose(host(model.params), want, rtol=1e-5, atol=2e-3 * 1e-3)
        fresh, _, _ = oracle.apply_adam(before[k], 0.0, 0.0, grads[k], 1, 1e-3)
        assert np.abs(fresh - want).max() > 1e-4  # the loaded state matters
    assert nerf._train_state()["step"] == 42


def test_bf16_tape_rows_permute_and_stop_at_n(ng, cuda):
    """The tape at a ragged size (several 512-row pair tiles, a partial last
    one): each row's tape is its own row's operands, bit for bit under a row
    permutation, including the encodings (columns 0-63 and enc_dir) and h9;
    rows past n of a larger buffer are not written."""
    lib = ng._lib
    n = 100_003
    g = torch.Generator(device="cuda")
    g.manual_seed(23)
    xyz = torch.rand(n, 3, device="cuda", generator=g) * 4 - 2
    dirs = torch.nn.functional.normalize(torch.randn(n, 3, device="cuda", generator=g), dim=1)
    mlp = ng.get_coarse_or_fine_model("fine", params=biased_blob(ng, 5), precision="bf16")
    _, _, acts = mlp.forward_train(xyz, dirs, precision="bf16")
    perm = torch.randperm(n, device="cuda", generator=g)
    _, _, acts_p = mlp.forward_train(xyz[perm], dirs[perm], precision="bf16")
    mlp.check_device_errors()
    assert torch.equal(acts_p, acts[perm])
    ld = acts.shape[1]
    assert bool((acts[:, :63] != 0).any(dim=1).all())  # every row's encoding written
    # rows past n: a buffer of n + 700 rows holding a sentinel
    big = torch.full((n + 700, ld), 0x7BCD, dtype=torch.int16, device="cuda")
    rgb, sig = torch.empty(n, 3, device="cuda"), torch.empty(n, 1, device="cuda")
    lib.call("nerfgb_mlp_forward_train_bf16", mlp.packed("bf16").data_ptr(), xyz.data_ptr(), dirs.data_ptr(), n,
             1, rgb.data_ptr(), sig.data_ptr(), big.data_ptr(), mlp.err_word.data_ptr(),
             torch.cuda.current_stream().cuda_stream)
    mlp.check_device_errors()
    assert torch.equal(big[:n], acts)
    assert bool((big[n:] == 0x7BCD).all())
