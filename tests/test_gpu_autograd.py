"""NeRF.forward's maps through torch.autograd (autograd.RenderFunction and
MSEFunction): loss.backward() runs the library's hand-written backward
(tf.GradientTape at nerf/core/model.py:148-170), recomputing the activation
tape per ray tile."""
import numpy as np
import pytest

from test_gpu_backward import biased_blob, compare, dev, flat_grads, host

pytestmark = pytest.mark.gpu
F32, F64 = np.float32, np.float64


def _case(ng, R=48, seed=5):
    o, d, n, f = ng.synthetic.sphere_rays(R, seed)
    rng = np.random.default_rng(seed + 1)
    uc = rng.random((R, 64), dtype=F32)
    uf = rng.random((R, 128), dtype=F32)
    target = rng.random((R, 3), dtype=F32)
    return (o, d, n, f), uc, uf, target


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_recompute_per_tile_equals_stored_tape(ng, cuda, precision):
    """Gradients with the tape recomputed over tiles of 16 rays (three tiles)
    equal those from the forward's own tape, up to the FP32 summation order of
    the row reductions; the maps equal the fused render's bit for bit."""
    (o, d, n, f), uc, uf, target = _case(ng)
    p = ng.make_params()
    bc, bf = biased_blob(ng, 11), biased_blob(ng, 12)
    ag = ng.autograd
    res = {}
    for tile in (None, 16):
        nerf = ng.NeRF(p, precision=precision, coarse_params=bc, fine_params=bf)
        rgb_c, rgb_f = ag.render_with_grad(nerf, dev(o), dev(d), dev(n), dev(f), u_coarse=dev(uc),
                                           u_fine=dev(uf), tile_rays=tile)
        loss = ag.mse(rgb_c, dev(target)) + ag.mse(rgb_f, dev(target))
        loss.backward()
        nerf.coarse_model.check_device_errors()
        res[tile] = (host(nerf.coarse_model.params.grad), host(nerf.fine_model.params.grad), host(rgb_c),
                     host(rgb_f), float(loss.detach()))
        out = nerf.render(dev(o), dev(d), dev(n), dev(f), u_coarse=dev(uc), u_fine=dev(uf), return_coarse=True,
                          precision=precision)
        assert np.array_equal(host(out["rgb"]), res[tile][3])
        assert np.array_equal(host(out["rgb_coarse"]), res[tile][2])
    a, b = res[None], res[16]
    assert np.array_equal(a[2], b[2]) and np.array_equal(a[3], b[3]) and a[4] == b[4]
    for ga, gb in ((a[0], b[0]), (a[1], b[1])):
        assert np.abs(ga).max() > 0
        np.testing.assert_allclose(gb, ga, rtol=1e-4, atol=1e-5 * np.abs(ga).max())


def test_function_gradients_vs_oracle(ng, oracle, cuda):
    """loss.backward() through the Function (FP32, tiles of 20 rays) against
    the oracle's float64 chain on the same rays, uniforms and tape (the
    last tile's, so the comparison runs on those 8 rays' contribution via a
    loss on them alone)."""
    (o, d, n, f), uc, uf, target = _case(ng, R=48, seed=9)
    p = ng.make_params()
    bc, bf = biased_blob(ng, 3), biased_blob(ng, 4)
    nerf = ng.NeRF(p, precision="fp32", coarse_params=bc, fine_params=bf, trans_mode=ng._lib.TRANS_CUMPROD)
    rgb_c, rgb_f = ng.autograd.render_with_grad(nerf, dev(o), dev(d), dev(n), dev(f), u_coarse=dev(uc),
                                                u_fine=dev(uf), tile_rays=20)
    (ng.autograd.mse(rgb_c, dev(target)) + ng.autograd.mse(rgb_f, dev(target))).backward()
    got_c, got_f = host(nerf.coarse_model.params.grad), host(nerf.fine_model.params.grad)
    # the oracle chain on the sample positions of every tile, re-taped here
    nerf2 = ng.NeRF(p, precision="fp32", coarse_params=bc, fine_params=bf, trans_mode=ng._lib.TRANS_CUMPROD)
    want = {"coarse": 0.0, "fine": 0.0}
    for s in range(0, 48, 20):
        sl = slice(s, min(48, s + 20))
        passes = ng.autograd._taped_passes(nerf2, dev(o[sl]), dev(d[sl]), dev(n[sl]), dev(f[sl]), dev(uc[sl]),
                                           dev(uf[sl]), "fp32")
        for key, blob, (t, sig, rgb_s, acts, pp) in zip(("coarse", "fine"), (bc, bf), passes):
            t, sig, rgb_s, acts, pred = (host(x).astype(F64) for x in (t, sig, rgb_s, acts, pp["pred_rgb"]))
            # dL/dpred of MSE over all 48 rays, restricted to this tile's rows
            G = 2.0 * (pred - target[sl].astype(F64)) / (48 * 3)
            ds, dr = oracle.composite_backward(sig.reshape(-1), t, rgb_s, G)
            want[key] = want[key] + flat_grads(ng, oracle.mlp_backward_cached(oracle.unpack_params(blob, F64),
                                                                              oracle.acts_from_tape(acts), dr, ds))
    compare(ng, got_c, want["coarse"], rel=2e-3, norm=True)
    compare(ng, got_f, want["fine"], rel=2e-3, norm=True)


def test_only_fine_loss_leaves_coarse_gradient_zero(ng, cuda):
    """The fine samples' positions carry no gradient into the coarse network
    (ray_utils.py:377 stop_gradient): a loss on the fine map alone gives the
    coarse network a zero gradient."""
    (o, d, n, f), uc, uf, target = _case(ng, R=32, seed=2)
    nerf = ng.NeRF(ng.make_params(), precision="bf16", coarse_params=biased_blob(ng, 1),
                   fine_params=biased_blob(ng, 2))
    _, rgb_f = ng.autograd.render_with_grad(nerf, dev(o), dev(d), dev(n), dev(f), u_coarse=dev(uc),
                                            u_fine=dev(uf), tile_rays=8)
    ng.autograd.mse(rgb_f, dev(target)).backward()
    nerf.coarse_model.check_device_errors()
    assert float(nerf.coarse_model.params.grad.abs().max()) == 0.0
    assert float(nerf.fine_model.params.grad.abs().max()) > 0.0


def test_single_tile_keeps_forward_tape(ng, cuda):
    """A tile covering every ray is one tile: the forward keeps its tape (no
    second render); maps as the stored tape's bit for bit, gradients up to the
    FP32 order of the backward's atomic row reductions (bias and head sums)."""
    (o, d, n, f), uc, uf, target = _case(ng, R=40, seed=13)
    p = ng.make_params()
    bc, bf = biased_blob(ng, 21), biased_blob(ng, 22)
    res = []
    for tile in (None, 40, 4096):
        nerf = ng.NeRF(p, precision="bf16", coarse_params=bc, fine_params=bf)
        rgb_c, rgb_f = ng.autograd.render_with_grad(nerf, dev(o), dev(d), dev(n), dev(f), u_coarse=dev(uc),
                                                    u_fine=dev(uf), tile_rays=tile)
        (ng.autograd.mse(rgb_c, dev(target)) + ng.autograd.mse(rgb_f, dev(target))).backward()
        nerf.coarse_model.check_device_errors()
        assert "tape" in nerf._train_state()  # the forward's tape was kept
        res.append((host(nerf.coarse_model.params.grad), host(nerf.fine_model.params.grad), host(rgb_c),
                    host(rgb_f)))
    for r in res[1:]:
        assert np.array_equal(r[2], res[0][2]) and np.array_equal(r[3], res[0][3])
        for ga, gb in ((res[0][0], r[0]), (res[0][1], r[1])):
            np.testing.assert_allclose(gb, ga, rtol=1e-4, atol=1e-6 * np.abs(ga).max())


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_backward_streams_give_the_same_gradients(ng, cuda, precision):
    """The coarse network's backward on a side stream beside the fine
    network's (NeRF.backward_streams = 2) gives the one-stream gradients, up
    to the FP32 order of the backward's atomic row reductions, and a full
    train_step after it the same loss; the gradients are complete when the
    caller's stream reads them."""
    (o, d, n, f), uc, uf, target = _case(ng, R=64, seed=17)
    p = ng.make_params()
    bc, bf = biased_blob(ng, 31), biased_blob(ng, 32)
    res = {}
    for streams in (1, 2):
        nerf = ng.NeRF(p, precision=precision, coarse_params=bc, fine_params=bf)
        nerf.backward_streams = streams
        for tile in (None, 16):
            for m in (nerf.coarse_model, nerf.fine_model):
                m.params.grad = None
            rgb_c, rgb_f = ng.autograd.render_with_grad(nerf, dev(o), dev(d), dev(n), dev(f), u_coarse=dev(uc),
                                                        u_fine=dev(uf), tile_rays=tile)
            (ng.autograd.mse(rgb_c, dev(target)) + ng.autograd.mse(rgb_f, dev(target))).backward()
            res[streams, tile] = (nerf.coarse_model.params.grad.double().sum().cpu(),
                                  host(nerf.coarse_model.params.grad), host(nerf.fine_model.params.grad))
        data = ((dev(o), dev(d), dev(n), dev(f)), (dev(target),))
        res[streams, "step"] = nerf.train_step(data, u_coarse=dev(uc), u_fine=dev(uf))["loss"]
        nerf.coarse_model.check_device_errors()
    for tile in (None, 16):
        a, b = res[1, tile], res[2, tile]
        assert float(a[0]) != 0.0
        np.testing.assert_allclose(float(b[0]), float(a[0]), rtol=1e-4)
        for ga, gb in ((a[1], b[1]), (a[2], b[2])):
            assert np.abs(ga).max() > 0
            np.testing.assert_allclose(gb, ga, rtol=1e-4, atol=1e-6 * np.abs(ga).max())
    assert res[1, "step"] == res[2, "step"]
