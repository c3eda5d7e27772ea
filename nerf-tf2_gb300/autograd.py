"""The hierarchical render and the MSE loss as torch.autograd.Functions whose
backward is the library's hand-written one (the gradient tf.GradientTape
takes at nerf/core/model.py:148-170).

``render_with_grad(nerf, rays_o, rays_d, near, far, ...)`` returns the coarse
and fine rgb maps [R, 3] (model.py:88-123), differentiable with respect to the
two networks' flat parameter blobs. Two ways to keep what backward needs:

* ``tile_rays=T`` (recompute): forward runs the fused render (one library
  call per ray chunk) and keeps only the rays, the jitter uniforms and the
  parameters; backward walks the rays in tiles of T, and for each tile runs
  the coarse and fine passes again with the activation tape
  (``NerfMLP.forward_train``), the compositing backward and the MLP
  backward, accumulating the parameter gradients. The tape never holds more
  than one tile (T x (Nc + Nc + Nf) rows).
* ``tile_rays=None`` (stored tape): forward runs the taped passes over all
  rays once and backward uses that tape; faster, R rows of tape. A tile that
  covers every ray (tile_rays >= R) is the same single tile, so forward keeps
  its tape then too rather than rendering twice.

The fine samples' positions do not carry gradient into the coarse network
(ray_utils.py:377 stop_gradient), so each network's gradient comes from its
own map's loss. Adam (model.py:171) is applied by ``NeRF.train_step``.
"""
import torch

from . import _lib, ray_utils
from ._tensors import as_cuda, empty, ptr, stream


def _precision_for_training(nerf, precision):
    return precision or ("fp32" if nerf.precision == "fp32" else "bf16")


def _taped_passes(nerf, rays_o, rays_d, near, far, u_c, u_f, tp):
    """Coarse and fine passes of one ray range with the activation tape:
    per network (t, sigma, sample_rgb, tape, post-processed dict)."""
    p = nerf.params
    d_cm = ray_utils.create_input_batch_coarse_model(p, rays_o, rays_d, near, far, u_vals=u_c)
    t_c = d_cm["t_vals"]
    Sc = t_c.shape[1]
    rgb_c, sig_c, acts_c = nerf.coarse_model.forward_train(d_cm["xyz_inputs"], rays_d, rows_per_dir=Sc,
                                                           precision=tp)
    pp_c = ray_utils.post_process_model_output(rgb_c, sig_c, t_c, nerf.white_bg, trans_mode=nerf.trans_mode)
    d_fm = ray_utils.create_input_batch_fine_model(p, rays_o, rays_d, pp_c["weights"], d_cm["bin_data"], t_c,
                                                   u_vals=u_f)
    t_f = d_fm["t_vals"]
    rgb_f, sig_f, acts_f = nerf.fine_model.forward_train(d_fm["xyz_inputs"], rays_d, rows_per_dir=t_f.shape[1],
                                                         precision=tp)
    pp_f = ray_utils.post_process_model_output(rgb_f, sig_f, t_f, nerf.white_bg, trans_mode=nerf.trans_mode)
    return (t_c, sig_c, rgb_c, acts_c, pp_c), (t_f, sig_f, rgb_f, acts_f, pp_f)


def _keep_tape(nerf, passes):
    """The last taped passes stay inspectable until the next step."""
    nerf._train_state()["tape"] = {k: (t, s, r, a, pp["pred_rgb"])
                                   for k, (t, s, r, a, pp) in zip(("coarse", "fine"), passes)}


def _backward_pass(nerf, model, t, sig, rgb_s, acts, g_map, g):
    """Compositing backward then MLP backward of one network, on the current
    stream, its gradient accumulated into g."""
    n, S = t.shape
    d_sig, d_rgb = empty(n * S), empty(n * S, 3)
    _lib.call("nerfgb_composite_backward", ptr(sig), ptr(t), ptr(rgb_s), ptr(g_map), None, n, S,
              int(nerf.white_bg), ptr(d_sig), ptr(d_rgb), stream())
    model.backward(acts, d_rgb, d_sig, g)


def _backward_passes(nerf, passes, grad_maps, grads):
    """Both networks' backward, gradients accumulated into grads = (coarse
    blob grad, fine blob grad). The two are independent (the fine samples
    carry no gradient into the coarse network), so with
    nerf.backward_streams > 1 the coarse network's runs on a side stream
    beside the fine network's on the current stream, which waits for it
    before returning."""
    jobs = [(model, t, sig, rgb_s, acts, g_map.contiguous(), g)
            for model, (t, sig, rgb_s, acts, _), g_map, g in zip((nerf.coarse_model, nerf.fine_model), passes,
                                                                  grad_maps, grads)]
    if getattr(nerf, "backward_streams", 1) <= 1:
        for job in jobs:
            _backward_pass(nerf, *job)
        return
    main = torch.cuda.current_stream()
    side = nerf._side_streams(1)[0]
    fork = torch.cuda.Event()
    fork.record(main)
    side.wait_event(fork)
    for x in jobs[0][1:]:
        x.record_stream(side)
    with torch.cuda.stream(side):
        _backward_pass(nerf, *jobs[0])
    _backward_pass(nerf, *jobs[1])
    join = torch.cuda.Event()
    join.record(side)
    main.wait_event(join)


class RenderFunction(torch.autograd.Function):
    """(params_coarse, params_fine) -> (rgb_coarse [R,3], rgb_fine [R,3]).
    The other arguments are constants; see the module docstring."""

    @staticmethod
    def forward(ctx, params_c, params_f, nerf, rays_o, rays_d, near, far, u_c, u_f, tp, tile_rays):
        R = rays_o.shape[0]
        if tile_rays is not None and int(tile_rays) >= R:
            tile_rays = None  # one tile: its tape is the forward's
        ctx.nerf, ctx.tp, ctx.tile_rays, ctx.R = nerf, tp, tile_rays, R
        if tile_rays is None:
            passes = _taped_passes(nerf, rays_o, rays_d, near, far, u_c, u_f, tp)
            ctx.passes = passes
            _keep_tape(nerf, passes)
            return passes[0][4]["pred_rgb"], passes[1][4]["pred_rgb"]
        # the fused render at the training precision gives the taped passes' maps bit for bit
        out = nerf.render(rays_o, rays_d, near, far, chunk=max(int(tile_rays), 1), u_coarse=u_c, u_fine=u_f,
                          precision=tp, return_coarse=True)
        ctx.save_for_backward(rays_o, rays_d, near, far, u_c, u_f)
        return out["rgb_coarse"], out["rgb"]

    @staticmethod
    def backward(ctx, g_rgb_c, g_rgb_f):
        nerf, tp, R = ctx.nerf, ctx.tp, ctx.R
        dev = nerf.coarse_model.params.device
        g_rgb_c = torch.zeros(R, 3, device=dev) if g_rgb_c is None else g_rgb_c.contiguous()
        g_rgb_f = torch.zeros(R, 3, device=dev) if g_rgb_f is None else g_rgb_f.contiguous()
        grads = (torch.zeros_like(nerf.coarse_model.params), torch.zeros_like(nerf.fine_model.params))
        if ctx.tile_rays is None:
            _backward_passes(nerf, ctx.passes, (g_rgb_c, g_rgb_f), grads)
            ctx.passes = None
        else:
            rays_o, rays_d, near, far, u_c, u_f = ctx.saved_tensors
            T = max(int(ctx.tile_rays), 1)
            for s in range(0, R, T):
                sl = slice(s, min(R, s + T))
                passes = _taped_passes(nerf, rays_o[sl], rays_d[sl], near[sl], far[sl], u_c[sl], u_f[sl], tp)
                _backward_passes(nerf, passes, (g_rgb_c[sl], g_rgb_f[sl]), grads)
                _keep_tape(nerf, passes)
        return grads[0], grads[1], None, None, None, None, None, None, None, None, None


class MSEFunction(torch.autograd.Function):
    """keras.losses.MeanSquaredError (model.py:32, :157-168) by the library's
    kernel: loss and gradient in one pass, the gradient kept for backward."""

    @staticmethod
    def forward(ctx, pred, target):
        pred = pred.contiguous()
        loss = torch.zeros(1, device=pred.device)
        g = torch.empty_like(pred)
        _lib.call("nerfgb_mse_loss", ptr(pred), ptr(target), pred.numel(), 1.0, ptr(loss), ptr(g), stream())
        ctx.save_for_backward(g)
        return loss[0]

    @staticmethod
    def backward(ctx, g_out):
        (g,) = ctx.saved_tensors
        return g * g_out, None


def render_with_grad(nerf, rays_o, rays_d, near, far, *, u_coarse=None, u_fine=None, precision=None,
                     tile_rays=4096):
    """Coarse and fine rgb maps [R, 3] of NeRF.forward, differentiable with
    respect to nerf.coarse_model.params and nerf.fine_model.params (their
    .grad accumulates on backward). Jitter uniforms are drawn from the
    library's stream when not given (and reused by the recompute)."""
    tp = _precision_for_training(nerf, precision)
    if tp not in ("fp32", "bf16"):
        raise ValueError(f"training precision must be fp32 or bf16, not {tp!r}")
    rays_o = as_cuda(rays_o, name="rays_o")
    R = rays_o.shape[0]
    rays_d = as_cuda(rays_d, shape=(R, 3), name="rays_d")
    near = as_cuda(near, shape=(R, 1), name="near")
    far = as_cuda(far, shape=(R, 1), name="far")
    Sc, Sf = int(nerf.params.sampling.N_coarse), int(nerf.params.sampling.N_fine)
    u_c = ray_utils.uniform((R, Sc)) if u_coarse is None else as_cuda(u_coarse, shape=(R, Sc), name="u_coarse")
    u_f = ray_utils.uniform((R, Sf)) if u_fine is None else as_cuda(u_fine, shape=(R, Sf), name="u_fine")
    pc, pf = nerf.coarse_model.params, nerf.fine_model.params
    pc.requires_grad_(True)
    pf.requires_grad_(True)
    return RenderFunction.apply(pc, pf, nerf, rays_o, rays_d, near, far, u_c, u_f, tp, tile_rays)


def mse(pred, target):
    """MSEFunction on pred and target (same shape)."""
    return MSEFunction.apply(pred, as_cuda(target, shape=tuple(pred.shape), name="target"))
