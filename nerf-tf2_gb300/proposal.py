"""Learned proposal sampler (not in the reference).

A 2x64 ReLU MLP on the L=6 encoding of xyz predicts a density whose
composited weights over the 64 stratified bins replace the coarse MLP's
weights (nerf/core/model.py:94-111) as the PDF of the inverse-transform fine
sampler (nerf/utils/ray_utils.py:276-406). It is trained on the GPU with the
library's own kernels (forward, compositing backward, backward, Adam) on the
coarse-pass weight histograms that the plain hierarchical path produces.
"""
import ctypes

import numpy as np
import torch

from . import _lib, ray_utils
from ._tensors import as_cuda, empty, ptr, stream

PARAM_COUNT = 6785
SHAPES = (("W1", (39, 64)), ("b1", (64,)), ("W2", (64, 64)), ("b2", (64,)), ("W3", (64,)), ("b3", (1,)))


def glorot_blob(seed):
    """Glorot-uniform kernels, zero biases (the Keras Dense defaults)."""
    rng = np.random.default_rng(seed)
    parts = []
    for name, shp in SHAPES:
        if name.startswith("W"):
            fan_in, fan_out = (shp[0], shp[1]) if len(shp) == 2 else (shp[0], 1)
            lim = np.sqrt(6.0 / (fan_in + fan_out))
            parts.append(rng.uniform(-lim, lim, size=shp).astype(np.float32).reshape(-1))
        else:
            parts.append(np.zeros(shp, np.float32).reshape(-1))
    return np.concatenate(parts)


class ProposalNetwork:
    def __init__(self, params=None, seed=0):
        blob = glorot_blob(seed) if params is None else params
        self.params = as_cuda(blob, shape=(PARAM_COUNT,), name="proposal params").clone()

    def __call__(self, xyz, precision="fp32"):
        """sigma [n,1] at xyz [n,3]. "fp32": the SIMT kernel (training uses
        it); "bf16": tensor cores, BF16 operands and FP32 accumulation."""
        if precision not in ("fp32", "bf16"):
            raise ValueError(f"proposal precision must be fp32 or bf16, not {precision!r}")
        xyz = as_cuda(xyz, name="xyz")
        n = xyz.shape[0]
        sigma = empty(n, 1)
        _lib.call("nerfgb_proposal_forward" if precision == "fp32" else "nerfgb_proposal_forward_bf16",
                  ptr(self.params), ptr(xyz), n, ptr(sigma), stream())
        return sigma

    def backward(self, xyz, grad_sigma, grad_params=None):
        """Accumulates d(sum grad_sigma * sigma)/dparams into grad_params."""
        xyz = as_cuda(xyz, name="xyz")
        n = xyz.shape[0]
        g = as_cuda(grad_sigma, shape=(n,), name="grad_sigma")
        if grad_params is None:
            grad_params = torch.zeros(PARAM_COUNT, device=self.params.device)
        _lib.call("nerfgb_proposal_backward", ptr(self.params), ptr(xyz), ptr(g), n, ptr(grad_params), stream())
        return grad_params


def proposal_weights(sigma, t_vals, trans_mode=None):
    """Weights [R, S] of proposal densities: compute_weights with the last
    interval equal to the previous spacing (not 1e10), so the last bin's
    weight can be 0 and is differentiable."""
    t_vals = as_cuda(t_vals, name="t_vals")
    R, S = t_vals.shape
    sigma = as_cuda(sigma, shape=(R * S,), name="sigma")
    w = empty(R, S)
    mode = ray_utils.DEFAULT_TRANS_MODE if trans_mode is None else trans_mode
    _lib.call("nerfgb_proposal_weights", ptr(sigma), ptr(t_vals), R, S, int(mode), ptr(w), stream())
    return w


def adam_step(params, m, v, grads, step, lr, beta1=0.9, beta2=0.999, eps=1e-7):
    """Keras Adam step (TensorFlow ApplyAdam) on flat device tensors."""
    _lib.call("nerfgb_adam_step", ptr(params), ptr(m), ptr(v), ptr(grads), params.numel(),
              ctypes.c_float(lr), ctypes.c_float(beta1), ctypes.c_float(beta2), ctypes.c_float(eps),
              int(step), stream())


def coarse_histograms(nerf, rays_o, rays_d, near, far, u_coarse, chunk=4096):
    """The plain path's coarse-pass weights [R, N_coarse] on the given rays and
    jitter uniforms: the proposal's training targets."""
    R = rays_o.shape[0]
    out = empty(R, int(nerf.params.sampling.N_coarse))
    for s in range(0, R, chunk):
        sl = slice(s, min(R, s + chunk))
        d = ray_utils.create_input_batch_coarse_model(nerf.params, rays_o[sl], rays_d[sl], near[sl], far[sl],
                                                      u_vals=u_coarse[sl])
        rgb, sig = nerf.coarse_model((d["xyz_inputs"], rays_d[sl]), rows_per_dir=d["t_vals"].shape[1])
        out[sl] = ray_utils.compute_weights(sig, d["t_vals"], d["t_vals"].shape[1], trans_mode=nerf.trans_mode)
    return out


class ProposalTrainer:
    """Trains a ProposalNetwork on (rays, jitter, target weights) with the
    envelope loss: per bin (1 + lam [w_p < w_t]) (w_p - w_t)^2, mean over
    rays."""

    def __init__(self, proposal, params, lr=3e-3, lam=3.0, trans_mode=None):
        self.prop, self.params = proposal, params
        self.lr, self.lam = lr, lam
        self.trans_mode = ray_utils.DEFAULT_TRANS_MODE if trans_mode is None else trans_mode
        n = proposal.params.numel()
        self.m = torch.zeros(n, device=proposal.params.device)
        self.v = torch.zeros(n, device=proposal.params.device)
        self.grads = torch.zeros(n, device=proposal.params.device)
        self.loss = torch.zeros(1, device=proposal.params.device)
        self.step_count = 0

    def step(self, rays_o, rays_d, near, far, u_coarse, w_target):
        """One Adam step on a batch; returns the loss tensor (device)."""
        R, S = w_target.shape
        d = ray_utils.create_input_batch_coarse_model(self.params, rays_o, rays_d, near, far, u_vals=u_coarse)
        xyz, t = d["xyz_inputs"], d["t_vals"]
        sigma = self.prop(xyz)
        w = proposal_weights(sigma, t, self.trans_mode)
        gw = empty(R, S)
        self.loss.zero_()
        _lib.call("nerfgb_envelope_loss", ptr(w), ptr(w_target), R, S, ctypes.c_float(self.lam),
                  ptr(self.loss), ptr(gw), stream())
        gs = empty(R * S)
        _lib.call("nerfgb_proposal_weights_backward", ptr(sigma), ptr(t), ptr(gw), R, S, ptr(gs), stream())
        self.grads.zero_()
        self.prop.backward(xyz, gs, self.grads)
        self.step_count += 1
        adam_step(self.prop.params, self.m, self.v, self.grads, self.step_count, self.lr)
        return self.loss

    def fit(self, rays_o, rays_d, near, far, u_coarse, w_target, steps, batch=4096, seed=0):
        """`steps` Adam steps on random batches of the training set."""
        g = torch.Generator(device=rays_o.device)
        g.manual_seed(seed)
        R = rays_o.shape[0]
        losses = []
        for i in range(steps):
            idx = torch.randint(0, R, (batch,), device=rays_o.device, generator=g)
            loss = self.step(rays_o[idx], rays_d[idx], near[idx], far[idx], u_coarse[idx], w_target[idx])
            if i % 50 == 0 or i == steps - 1:
                losses.append(float(loss.item()))
        return losses
