"""Size-independent properties at the benchmark's full size: an 800x800 frame
(640,000 rays, 64 coarse + 128 fine samples, 4096-ray chunks) and the MLP
at the fine pass's launch shape (786,432 rows). Every check is bit for bit:
the fused render against the op-by-op NeRF.forward (model.py:57-125), the
gate with every sample on against the plain chain, the gated render under a
permutation of the rays, and the MLP under a permutation of its rows."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

H = W = 800
FOCAL = 1111.111


@pytest.fixture(scope="module")
def frame(ng):
    rays = [torch.from_numpy(x).cuda() for x in ng.synthetic.frame_rays(3, H, W, FOCAL)]
    R = rays[0].shape[0]
    g = torch.Generator(device="cuda")
    g.manual_seed(11)
    uc = torch.rand(R, 64, device="cuda", generator=g)
    uf = torch.rand(R, 128, device="cuda", generator=g)
    blob = ng.synthetic.sparse_scene_blob(21, max_freq_log2=6)
    return rays, uc, uf, blob


def test_full_frame_fused_equals_forward(ng, cuda, frame):
    rays, uc, uf, blob = frame
    nerf = ng.NeRF(ng.make_params(), precision="bf16", coarse_params=blob, fine_params=blob)
    fused = nerf.render(*rays, u_coarse=uc, u_fine=uf, chunk=4096, return_coarse=True)
    pc, pf = nerf.forward(*rays, u_coarse=uc, u_fine=uf)
    nerf.coarse_model.check_device_errors()
    assert torch.equal(fused["rgb"], pf["pred_rgb"].reshape(-1, 3))
    assert torch.equal(fused["depth"], pf["pred_depth"].reshape(-1))
    assert torch.equal(fused["acc"], pf["acc_map"].reshape(-1))
    assert torch.equal(fused["rgb_coarse"], pc["pred_rgb"].reshape(-1, 3))


def test_full_frame_gate_all_on_equals_plain(ng, cuda, frame):
    rays, uc, uf, blob = frame
    nerf = ng.NeRF(ng.make_params(), precision="bf16", coarse_params=blob, fine_params=blob)
    prop = ng.ProposalNetwork(seed=7)
    plain = nerf.render(*rays, u_coarse=uc, u_fine=uf, chunk=4096)
    gated = nerf.render(*rays, u_coarse=uc, u_fine=uf, chunk=4096, proposal=prop, proposal_mode="gate",
                        gate_tau=-1.0)
    nerf.coarse_model.check_device_errors()
    for k in ("rgb", "depth", "acc"):
        assert torch.equal(gated[k], plain[k]), k


def test_full_frame_gated_render_commutes_with_ray_permutation(ng, cuda, frame):
    """Rays are independent: rendering the frame's rays in another order (the
    gates' row maps, filled by atomics, come out in another order too) gives
    the same maps, permuted."""
    rays, uc, uf, blob = frame
    nerf = ng.NeRF(ng.make_params(), precision="bf16", coarse_params=blob, fine_params=blob)
    prop = ng.ProposalNetwork(seed=7)
    kw = dict(chunk=4096, proposal=prop, proposal_mode="gate", gate_tau=1e-4, gate_fine_draws=True)
    a = nerf.render(*rays, u_coarse=uc, u_fine=uf, **kw)
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    perm = torch.randperm(rays[0].shape[0], device="cuda", generator=g)
    b = nerf.render(*[x[perm] for x in rays], u_coarse=uc[perm], u_fine=uf[perm], **kw)
    nerf.coarse_model.check_device_errors()
    for k in ("rgb", "depth", "acc"):
        assert torch.equal(b[k], a[k][perm]), k
    # the gate is not trivially on or off on this frame
    assert 0.0 < float(a["acc"].mean()) < 1.0


@pytest.mark.parametrize("mode", ["plain", "gate", "replace"])
def test_full_frame_streams_do_not_change_maps(ng, cuda, frame, mode):
    """Chunks alternate over the caller's stream and side streams with their
    own workspaces: one, two and three streams give the same maps bit for
    bit, and the maps are complete when the caller's stream reaches them
    (read here on that stream without another synchronisation)."""
    rays, uc, uf, blob = frame
    nerf = ng.NeRF(ng.make_params(), precision="bf16", coarse_params=blob, fine_params=blob)
    kw = dict(chunk=4096, u_coarse=uc, u_fine=uf)
    if mode != "plain":
        kw.update(proposal=ng.ProposalNetwork(seed=7), proposal_mode=mode, gate_tau=1e-4)
    maps = {n: nerf.render(*rays, streams=n, **kw) for n in (1, 2, 3)}
    sums = {n: torch.stack([m[k].double().sum() for k in ("rgb", "depth", "acc")]).cpu() for n, m in maps.items()}
    nerf.coarse_model.check_device_errors()
    for n in (2, 3):
        for k in ("rgb", "depth", "acc"):
            assert torch.equal(maps[n][k], maps[1][k]), (n, k)
        assert torch.equal(sums[n], sums[1]), n


def test_render_streams_argument(ng, cuda):
    nerf = ng.NeRF(ng.make_params(), precision="bf16")
    rays = [torch.from_numpy(x).cuda() for x in ng.synthetic.frame_rays(3, 8, 8, 10.0)]
    with pytest.raises(ValueError):
        nerf.render(*rays, streams=0)
    one = nerf.render(*rays, chunk=16, seed=3, streams=1)
    many = nerf.render(*rays, chunk=16, seed=3, streams=8)  # more streams than chunks
    for k in ("rgb", "depth", "acc"):
        assert torch.equal(one[k], many[k]), k


@pytest.mark.parametrize("precision", ["bf16", "fp8"])
def test_fine_pass_mlp_row_permutation(ng, cuda, precision):
    """The tensor-core MLP at its fine-pass launch shape: every row is computed
    on its own, so permuting the rows permutes the outputs bit for bit."""
    n = 4096 * 192
    g = torch.Generator(device="cuda")
    g.manual_seed(17)
    xyz = torch.rand(n, 3, device="cuda", generator=g) * 4 - 2
    dirs = torch.nn.functional.normalize(torch.randn(n, 3, device="cuda", generator=g), dim=1)
    mlp = ng.get_coarse_or_fine_model("fine", seed=1, precision=precision)
    rgb, sig = mlp((xyz, dirs))
    perm = torch.randperm(n, device="cuda", generator=g)
    rgb2, sig2 = mlp((xyz[perm], dirs[perm]))
    mlp.check_device_errors()
    assert torch.equal(rgb2, rgb[perm]) and torch.equal(sig2.reshape(-1), sig.reshape(-1)[perm])
    assert bool(torch.isfinite(rgb).all()) and float(sig.max()) > 0
