"""Drop-in for nerf/utils/ray_utils.py's render-path functions, on CUDA.

Same names, argument names, dict keys and shapes as the reference. Tensors
are torch CUDA tensors (numpy arrays and host tensors are moved to the
device). Two keyword-only additions:

* ``u_vals=`` on both samplers supplies the jitter uniforms that the
  reference draws internally with tf.random.uniform (ray_utils.py:230, :355).
  When omitted they come from the library's Philox stream (``set_seed``).
* ``return_indices=True`` on the fine sampler also returns the searchsorted
  bin indices and the sort permutation (int32).

Every call is one or two kernel launches in libnerfgb.so on the current
torch stream. There is no CPU path.
"""
import ctypes

import torch

from . import _lib
from ._tensors import as_cuda, empty, ptr, stream

# Transmittance evaluation used by compute_weights/post_process_model_output:
# TRANS_LOGSUM (exp of a compensated log-sum) or TRANS_CUMPROD (the
# reference's product as written, ray_utils.py:480).
DEFAULT_TRANS_MODE = _lib.TRANS_LOGSUM


class _Philox:
    """Counter state of the library's Philox4x32-10 stream."""

    def __init__(self, seed=0):
        self.seed, self.offset = int(seed), 0

    def draw(self, shape):
        n = 1
        for s in shape:
            n *= int(s)
        out = empty(*shape)
        _lib.call("nerfgb_uniform", ctypes.c_ulonglong(self.seed), ctypes.c_ulonglong(self.offset),
                  n, ptr(out), stream())
        self.offset += n
        return out


_rng = _Philox(0)


def set_seed(seed):
    """Re-keys the uniform stream (the analogue of tf.random.set_seed)."""
    global _rng
    _rng = _Philox(seed)


def uniform(shape):
    """Uniforms in [0, 1) from the library's stream (tf.random.uniform)."""
    return _rng.draw(shape)


def get_rays_tf(H, W, intrinsic, c2w):
    """ray_utils.py:53-106 on the device: (rays_o, rays_d), each [H*W, 3]
    float32, for the pinhole camera `intrinsic` [3,3] at pose `c2w` [4,4]
    (numpy arrays or tensors). The 3x3 rotation and the norm are sequential
    float32 sums."""
    K = as_cuda(torch.as_tensor(intrinsic, dtype=torch.float32), shape=(3, 3), name="intrinsic")
    T = as_cuda(torch.as_tensor(c2w, dtype=torch.float32), shape=(4, 4), name="c2w")
    n = int(H) * int(W)
    rays_o, rays_d = empty(n, 3), empty(n, 3)
    _lib.call("nerfgb_get_rays", int(H), int(W), ptr(K), ptr(T), ptr(rays_o), ptr(rays_d), stream())
    return rays_o, rays_d


def sample_mode_batch(img, pose, bounds, intrinsic, batch_size, *, idxs=None, seed=0):
    """base_dataset.py:555-621 (the sample-mode map function) for one image
    on the device: ((rays_o, rays_d, near, far), (rgb,)) for batch_size rays
    drawn uniformly with replacement among the image's H*W. ``img`` is uint8
    [H, W, 3]; ``idxs`` (int32 [batch_size]) replaces the reference's
    tf.random.uniform draw, else it comes from the Philox stream keyed by
    ``seed``."""
    img = torch.as_tensor(img)
    if img.dtype != torch.uint8 or img.dim() != 3 or img.shape[2] != 3:
        raise ValueError("img must be a uint8 [H, W, 3] array")
    img = img.to(device="cuda").contiguous()
    H, W = int(img.shape[0]), int(img.shape[1])
    K = as_cuda(torch.as_tensor(intrinsic, dtype=torch.float32), shape=(3, 3), name="intrinsic")
    T = as_cuda(torch.as_tensor(pose, dtype=torch.float32), shape=(4, 4), name="pose")
    B = int(batch_size)
    if idxs is None:
        idxs = torch.empty(B, dtype=torch.int32, device="cuda")
        _lib.call("nerfgb_uniform_int", ctypes.c_ulonglong(int(seed)), ctypes.c_ulonglong(0), B, H * W,
                  ptr(idxs), stream())
    else:
        idxs = as_cuda(idxs, dtype=torch.int32, shape=(B,), name="idxs")
    rays_o, rays_d, rgb = empty(B, 3), empty(B, 3), empty(B, 3)
    near, far = empty(B, 1), empty(B, 1)
    _lib.call("nerfgb_sample_rays", ptr(img), H, W, ptr(K), ptr(T), ctypes.c_float(float(bounds[0])),
              ctypes.c_float(float(bounds[1])), ptr(idxs), B, ptr(rays_o), ptr(rays_d), ptr(near), ptr(far),
              ptr(rgb), stream())
    return (rays_o, rays_d, near, far), (rgb,)


def create_depth_map(pred_depth, H, W, scale_factor, map_type, intrinsic=None, C_to_W2=None):
    """ray_utils.py:108-135 on the device: "type_1" = pred_depth /
    scale_factor as [H, W]; "type_2" = the camera-frame z of the depth
    points along get_rays_tf's rays (float32; the reference computes it in
    float64 with NumPy)."""
    d = as_cuda(pred_depth, name="pred_depth").reshape(-1)
    n = int(H) * int(W)
    if d.numel() != n:
        raise ValueError(f"pred_depth has {d.numel()} values, H*W = {n}")
    out = empty(n)
    if map_type == "type_1":
        _lib.call("nerfgb_depth_map", ptr(d), n, ctypes.c_float(float(scale_factor)), 1, None, None, None,
                  ptr(out), stream())
    elif map_type == "type_2":
        if intrinsic is None or C_to_W2 is None:
            raise ValueError("type_2 needs intrinsic and C_to_W2")
        rays_o, rays_d = get_rays_tf(H, W, intrinsic, C_to_W2)
        import numpy as np
        w2c = as_cuda(torch.as_tensor(np.linalg.inv(np.asarray(C_to_W2, np.float64)), dtype=torch.float32),
                      shape=(4, 4), name="w2c")
        _lib.call("nerfgb_depth_map", ptr(d), n, ctypes.c_float(float(scale_factor)), 2, ptr(rays_o),
                  ptr(rays_d), ptr(w2c), ptr(out), stream())
    else:
        raise ValueError(f"Invalid map_type: {map_type}")
    return out.reshape(int(H), int(W))


def create_input_batch_coarse_model(params, rays_o, rays_d, near, far, *, u_vals=None):
    """ray_utils.py:137-274. Returns {"xyz_inputs", "dir_inputs", "bin_data",
    "t_vals"}; bin_data holds "bin_edges", "left_edges", "right_edges",
    "bin_widths" (left/right are views of bin_edges). Unlike the reference,
    perturb=False does not raise NameError at :263: the widths are always
    computed."""
    S = int(params.sampling.N_coarse)
    perturb = bool(params.sampling.perturb)
    rays_o = as_cuda(rays_o, name="rays_o")
    R = rays_o.shape[0]
    rays_o = as_cuda(rays_o, shape=(R, 3), name="rays_o")
    rays_d = as_cuda(rays_d, shape=(R, 3), name="rays_d")
    near = as_cuda(near, shape=(R, 1), name="near")
    far = as_cuda(far, shape=(R, 1), name="far")
    if perturb:
        u_vals = uniform((R, S)) if u_vals is None else as_cuda(u_vals, shape=(R, S), name="u_vals")
    else:
        u_vals = None
    xyz = empty(R * S, 3)
    dirs = empty(R * S, 3)
    t = empty(R, S)
    edges = empty(R, S + 1)
    widths = empty(R, S)
    _lib.call("nerfgb_coarse_sample", ptr(rays_o), ptr(rays_d), ptr(near), ptr(far), ptr(u_vals),
              R, S, int(perturb), int(bool(params.sampling.lin_inv_depth)), ptr(xyz), ptr(dirs),
              ptr(t), ptr(edges), ptr(widths), stream())
    bin_data = {"bin_edges": edges, "left_edges": edges[:, :-1],
                "right_edges": edges[:, 1:], "bin_widths": widths}
    return {"xyz_inputs": xyz, "dir_inputs": dirs, "bin_data": bin_data, "t_vals": t}


def create_input_batch_fine_model(params, rays_o, rays_d, bin_weights, bin_data, t_vals_coarse,
                                  *, u_vals=None, return_indices=False):
    """ray_utils.py:276-406. Returns {"xyz_inputs", "dir_inputs", "t_vals"}
    (+ "piece_idxs" [R,N_fine] and "sort_perm" [R,N_coarse+N_fine] int32 when
    return_indices). t_vals is sorted ascending (:385)."""
    Sf = int(params.sampling.N_fine)
    rays_o = as_cuda(rays_o, name="rays_o")
    R = rays_o.shape[0]
    rays_o = as_cuda(rays_o, shape=(R, 3), name="rays_o")
    rays_d = as_cuda(rays_d, shape=(R, 3), name="rays_d")
    t_c = as_cuda(t_vals_coarse, name="t_vals_coarse")
    Sc = t_c.shape[1]
    w = as_cuda(bin_weights, shape=(R, Sc), name="bin_weights")
    widths = as_cuda(bin_data["bin_widths"], shape=(R, Sc), name="bin_widths")
    left = bin_data["left_edges"]
    if not (isinstance(left, torch.Tensor) and left.is_cuda and left.dtype == torch.float32
            and left.dim() == 2 and left.stride(1) == 1 and left.shape == (R, Sc)):
        left = as_cuda(left, shape=(R, Sc), name="left_edges")
    u_vals = uniform((R, Sf)) if u_vals is None else as_cuda(u_vals, shape=(R, Sf), name="u_vals")
    S = Sc + Sf
    xyz = empty(R * S, 3)
    dirs = empty(R * S, 3)
    t = empty(R, S)
    idx = empty(R, Sf, dtype=torch.int32) if return_indices else None
    perm = empty(R, S, dtype=torch.int32) if return_indices else None
    _lib.call("nerfgb_fine_sample", ptr(rays_o), ptr(rays_d), ptr(w), ptr(left), left.stride(0),
              ptr(widths), ptr(t_c), ptr(u_vals), R, Sc, Sf, ptr(xyz), ptr(dirs), ptr(t), ptr(idx),
              ptr(perm), stream())
    out = {"xyz_inputs": xyz, "dir_inputs": dirs, "t_vals": t}
    if return_indices:
        out["piece_idxs"] = idx
        out["sort_perm"] = perm
    return out


def sigma_to_alpha(sigma, diffs):
    """ray_utils.py:408-424: alpha = 1 - exp(-sigma * diffs)."""
    diffs = as_cuda(diffs, name="diffs")
    sigma = as_cuda(sigma, shape=tuple(diffs.shape), name="sigma")
    alpha = torch.empty_like(diffs)
    _lib.call("nerfgb_sigma_to_alpha", ptr(sigma), ptr(diffs), diffs.numel(), ptr(alpha), stream())
    return alpha


def _composite(sample_rgb, sigma, t_vals, white_bg, trans_mode, want_weights=True):
    t_vals = as_cuda(t_vals, name="t_vals")
    R, S = t_vals.shape
    sigma = as_cuda(sigma, shape=(R * S,), name="sigma")
    sample_rgb = as_cuda(sample_rgb, shape=(R * S, 3), name="sample_rgb")
    weights = empty(R, S) if want_weights else None
    rgb = empty(R, 3)
    depth = empty(R)
    acc = empty(R)
    _lib.call("nerfgb_composite", ptr(sample_rgb), ptr(sigma), ptr(t_vals), R, S, int(bool(white_bg)),
              int(trans_mode), ptr(weights), ptr(rgb), ptr(depth), ptr(acc), stream())
    return weights, rgb, depth, acc


def compute_weights(sigma, t_vals, N_samples, *, trans_mode=None):
    """ray_utils.py:426-482: weights [R, N_samples]."""
    t_vals = as_cuda(t_vals, name="t_vals")
    if int(N_samples) != t_vals.shape[1]:
        raise ValueError(f"N_samples={int(N_samples)} does not match t_vals {tuple(t_vals.shape)}")
    R, S = t_vals.shape
    dummy_rgb = torch.zeros(R * S, 3, device=t_vals.device)
    mode = DEFAULT_TRANS_MODE if trans_mode is None else trans_mode
    return _composite(dummy_rgb, sigma, t_vals, False, mode)[0]


def post_process_model_output(sample_rgb, sigma, t_vals, white_bg=False, *, trans_mode=None):
    """ray_utils.py:484-551: {"acc_map" [R], "weights" [R,S], "pred_rgb"
    [R,3], "pred_depth" [R]}."""
    mode = DEFAULT_TRANS_MODE if trans_mode is None else trans_mode
    weights, rgb, depth, acc = _composite(sample_rgb, sigma, t_vals, white_bg, mode)
    return {"acc_map": acc, "weights": weights, "pred_rgb": rgb, "pred_depth": depth}
