"""numpy restatement of the nerf-tf2 render path. TEST INFRASTRUCTURE ONLY.

Parity unpinned: TensorFlow 2.6 (the reference's runtime, pinned at
requirements.txt:44) is absent, and the reference has no tests or golden
vectors. Every function below restates the reference line by line and cites it.
Each runs in float32 (the reference's precision) or float64 (the FP64 oracle
pass), chosen by ``dtype``.

The TensorFlow ops the reference calls are restated from their published
semantics (tensorflow==2.6.0):
  * ``tf.linspace(start, stop, num, axis)``: first point = start, last
    point = stop, interior points ``start + i * ((stop - start) / (num - 1))``,
    one multiply and one add per point (TF's ``linspace_nd``).
  * ``tf.searchsorted(a, v, side='right')``: per row, ``std::upper_bound``
    binary search. It returns the count of elements <= v on a sorted row.
  * ``tf.reduce_sum`` and ``tf.cumsum``: TF does not specify an order. Here
    both are sequential left to right in the working dtype. The CUDA kernels
    use the same order, so the fine sampler's CDF and indices are bit-exact.
  * ``tf.sort``: ascending. The permutation returned with it is the stable
    argsort (ties keep concatenation order).
"""
import numpy as np

F32 = np.float32
F64 = np.float64

# ---------------------------------------------------------------------------
# Parameter layout of one coarse/fine network (nerf/core/model.py:334-394).
# Flat blob order: dense_0..dense_7, sigma, dense_8, dense_9, rgb; per layer
# the Keras kernel [in, out] row-major, then the bias [out].
# ---------------------------------------------------------------------------
LAYERS = (
    ("dense_0", 63, 256), ("dense_1", 256, 256), ("dense_2", 256, 256),
    ("dense_3", 256, 256), ("dense_4", 256, 256), ("dense_5", 319, 256),
    ("dense_6", 256, 256), ("dense_7", 256, 256), ("sigma", 256, 1),
    ("dense_8", 256, 256), ("dense_9", 283, 128), ("rgb", 128, 3),
)


def param_count():
    return sum(i * o + o for _, i, o in LAYERS)


def unpack_params(blob, dtype=F32):
    """Flat blob -> {name: (W[in,out], b[out])}."""
    blob = np.asarray(blob)
    out, off = {}, 0
    for name, i, o in LAYERS:
        W = blob[off:off + i * o].reshape(i, o).astype(dtype)
        off += i * o
        b = blob[off:off + o].astype(dtype)
        off += o
        out[name] = (W, b)
    assert off == blob.size
    return out


def pack_params(p):
    parts = []
    for name, i, o in LAYERS:
        W, b = p[name]
        parts += [np.asarray(W).reshape(-1), np.asarray(b).reshape(-1)]
    return np.concatenate(parts)


def glorot_params(seed, dtype=F32):
    """Keras defaults: GlorotUniform kernel (limit sqrt(6/(in+out))), zero bias
    (Dense defaults used at model.py:368,375,378,384,387)."""
    rng = np.random.default_rng(seed)
    p = {}
    for name, i, o in LAYERS:
        lim = np.sqrt(6.0 / (i + o))
        p[name] = (rng.uniform(-lim, lim, size=(i, o)).astype(dtype),
                   np.zeros(o, dtype))
    return p


# ---------------------------------------------------------------------------
# Stratified coarse sampler: ray_utils.py:137-274
# ---------------------------------------------------------------------------
def tf_linspace(start, stop, num, dtype=F32):
    """tf.linspace(start, stop, num, axis=1) for [R,1] start/stop -> [R,num]."""
    start = np.asarray(start, dtype).reshape(-1, 1)
    stop = np.asarray(stop, dtype).reshape(-1, 1)
    n_steps = max(num - 1, 1)
    delta = (stop - start) / dtype(n_steps)
    i = np.arange(1, num - 1, dtype=dtype)[None, :]
    mid = start + delta * i
    return np.concatenate([start, mid, stop], axis=1)[:, :num]


def bin_edges(near, far, n_coarse, lin_inv_depth, dtype=F32):
    """ray_utils.py:183-206: linear in t, or linear in inverse depth."""
    near = np.asarray(near, dtype).reshape(-1, 1)
    far = np.asarray(far, dtype).reshape(-1, 1)
    if not lin_inv_depth:
        return tf_linspace(near, far, n_coarse + 1, dtype)
    one = dtype(1)
    return one / tf_linspace(one / near, one / far, n_coarse + 1, dtype)


def create_input_batch_coarse_model(params, rays_o, rays_d, near, far,
                                    u_vals=None, dtype=F32):
    """ray_utils.py:137-274. ``u_vals`` [R, N_coarse] in [0,1) replaces the
    internal tf.random.uniform draw at :230. When perturb is False the
    reference raises NameError at :263 (bin_widths undefined); here the widths
    are computed in both branches."""
    S = params.sampling.N_coarse
    rays_o = np.asarray(rays_o, dtype)
    rays_d = np.asarray(rays_d, dtype)
    edges = bin_edges(near, far, S, params.sampling.lin_inv_depth, dtype)  # :183-206
    left = edges[:, :-1]                                                   # :212
    right = edges[:, 1:]                                                   # :214
    widths = right - left                                                  # :226
    if params.sampling.perturb:
        u = np.asarray(u_vals, dtype)
        t = left + (u * widths)                                            # :234
    else:
        t = dtype(0.5) * (left + right)                                    # :243
    xyz = rays_o[:, None, :] + t[..., None] * rays_d[:, None, :]           # :251
    dirs = np.broadcast_to(rays_d[:, None, :], xyz.shape)                  # :253
    return {
        "xyz_inputs": xyz.reshape(-1, 3),
        "dir_inputs": np.ascontiguousarray(dirs).reshape(-1, 3),
        "bin_data": {"bin_edges": edges, "left_edges": left,
                     "right_edges": right, "bin_widths": widths},
        "t_vals": t,
    }


# ---------------------------------------------------------------------------
# Inverse-transform fine sampler: ray_utils.py:276-406
# ---------------------------------------------------------------------------
def seq_sum(x):
    """Left-to-right sum along axis 1 in x's dtype."""
    acc = np.zeros(x.shape[0], x.dtype)
    for j in range(x.shape[1]):
        acc = acc + x[:, j]
    return acc


def seq_cumsum(x):
    out = np.empty_like(x)
    acc = np.zeros(x.shape[0], x.dtype)
    for j in range(x.shape[1]):
        acc = acc + x[:, j]
        out[:, j] = acc
    return out


def upper_bound(a, v):
    """Row-wise std::upper_bound(a[r], v[r, k]) (tf.searchsorted side='right',
    ray_utils.py:363). a [R, n], v [R, m] -> int32 [R, m]."""
    R, n = a.shape
    first = np.zeros(v.shape, np.int64)
    count = np.full(v.shape, n, np.int64)
    rows = np.arange(R)[:, None]
    while True:
        active = count > 0
        if not active.any():
            break
        step = count // 2
        it = np.minimum(first + step, n - 1)
        go_right = active & ~(v < a[rows, it])
        first = np.where(go_right, first + step + 1, first)
        count = np.where(active, np.where(go_right, count - step - 1, step), 0)
    return first.astype(np.int32)


def create_input_batch_fine_model(params, rays_o, rays_d, bin_weights, bin_data,
                                  t_vals_coarse, u_vals, dtype=F32,
                                  return_indices=False):
    """ray_utils.py:276-406 with ``u_vals`` [R, N_fine] supplied in place of the
    tf.random.uniform draw at :355 (``det`` is hard-wired False at :348)."""
    rays_o = np.asarray(rays_o, dtype)
    rays_d = np.asarray(rays_d, dtype)
    left = np.asarray(bin_data["left_edges"], dtype)                       # :330
    widths = np.asarray(bin_data["bin_widths"], dtype)                     # :331
    w = np.asarray(bin_weights, dtype) + dtype(1e-5)                       # :335
    denom = seq_sum(w * widths)[:, None]                                   # :338
    pdf = w / denom                                                        # :339
    agg = seq_cumsum(pdf * widths)                                         # :342
    agg = np.concatenate([np.zeros_like(agg[:, :1]), agg], axis=1)         # :345
    u = np.asarray(u_vals, dtype)
    idx = upper_bound(agg[:, 1:-1], u)                                     # :363
    rows = np.arange(u.shape[0])[:, None]
    agg_ = agg[:, :-1][rows, idx]                                          # :366
    pdf_ = pdf[rows, idx]                                                  # :367
    left_ = left[rows, idx]                                                # :368
    mask = np.where(pdf_ < dtype(1e-8), dtype(0), dtype(1))                # :372
    pdf_ = np.maximum(pdf_, dtype(1e-8))                                   # :373
    t_fine = (((u - agg_) / pdf_) * mask) + left_                          # :376
    t_cat = np.concatenate([np.asarray(t_vals_coarse, dtype), t_fine], 1)  # :380
    perm = np.argsort(t_cat, axis=1, kind="stable").astype(np.int32)       # :385
    t = np.take_along_axis(t_cat, perm, axis=1)
    xyz = rays_o[:, None, :] + t[..., None] * rays_d[:, None, :]           # :389
    dirs = np.broadcast_to(rays_d[:, None, :], xyz.shape)                  # :392
    out = {"xyz_inputs": xyz.reshape(-1, 3),
           "dir_inputs": np.ascontiguousarray(dirs).reshape(-1, 3),
           "t_vals": t}
    if return_indices:
        out["piece_idxs"] = idx
        out["sort_perm"] = perm
        out["t_vals_fine"] = t_fine
    return out


# ---------------------------------------------------------------------------
# Compositing: ray_utils.py:408-551
# ---------------------------------------------------------------------------
def sigma_to_alpha(sigma, diffs):
    """ray_utils.py:423."""
    return 1 - np.exp(-sigma * diffs)


def compute_weights(sigma, t_vals, N_samples):
    """ray_utils.py:426-482. The exclusive cumprod is sequential (TF does not
    specify an order)."""
    dtype = t_vals.dtype.type
    EPS, INF = dtype(1e-10), dtype(1e10)                                   # :458-459
    diffs = t_vals[:, 1:] - t_vals[:, :-1]                                 # :462
    diffs_ = np.concatenate(
        [diffs, np.full((t_vals.shape[0], 1), INF, dtype)], axis=-1)       # :465-468
    sigma_ = np.asarray(sigma, dtype).reshape(-1, N_samples)               # :474
    alpha = sigma_to_alpha(sigma_, diffs_)                                 # :476
    fac = dtype(1) - alpha + EPS                                           # :480
    T = np.empty_like(fac)
    acc = np.ones(fac.shape[0], dtype)
    for j in range(fac.shape[1]):
        T[:, j] = acc
        acc = acc * fac[:, j]
    return alpha * T


def post_process_model_output(sample_rgb, sigma, t_vals, white_bg=False):
    """ray_utils.py:484-551."""
    t_vals = np.asarray(t_vals)
    dtype = t_vals.dtype.type
    N = t_vals.shape[1]
    weights = compute_weights(np.asarray(sigma, dtype), t_vals, N)         # :528
    rgb_ = np.asarray(sample_rgb, dtype).reshape(-1, N, 3)                 # :531
    pred_rgb = np.sum(weights[..., None] * rgb_, axis=1)                   # :534
    pred_depth = np.sum(t_vals * weights, axis=1)                          # :537
    acc_map = np.sum(weights, axis=1)                                      # :540
    if white_bg:
        pred_rgb = pred_rgb + (1 - acc_map[:, None])                       # :544
    return {"acc_map": acc_map, "weights": weights,
            "pred_rgb": pred_rgb, "pred_depth": pred_depth}


# ---------------------------------------------------------------------------
# Positional encoder and MLP: model.py:289-394
# ---------------------------------------------------------------------------
def encoder_multipliers(L, dtype=F32):
    """model.py:309-311: (2 ** range(L)) * pi. In float32, pi is rounded to
    float32 first (np.pi enters a float32 tensor)."""
    return (np.float64(2.0) ** np.arange(L)).astype(dtype) * dtype(np.pi)


def positional_encoding(x, L, dtype=F32):
    """model.py:319-331: [x, sin/cos interleaved], coordinate-major, then
    frequency, then (sin, cos)."""
    x = np.asarray(x, dtype)
    expanded = x[..., None] * encoder_multipliers(L, dtype)[None, None, :]  # :323
    sincos = np.stack([np.sin(expanded), np.cos(expanded)], axis=-1)       # :325-328
    return np.concatenate([x, sincos.reshape(x.shape[0], -1)], axis=-1)    # :329-330


def relu(x):
    return np.maximum(x, 0)


def sigmoid(x):
    one = x.dtype.type(1)
    return one / (one + np.exp(-x))


def mlp_forward(p, xyz, dirs, dtype=F32, cache=False):
    """get_coarse_or_fine_model (model.py:334-394) applied to (xyz, dirs).
    Returns (rgb [M,3], sigma [M,1]) and, when ``cache``, the activations."""
    p = {k: (np.asarray(W, dtype), np.asarray(b, dtype)) for k, (W, b) in p.items()}
    enc_xyz = positional_encoding(xyz, 10, dtype)                          # :359
    enc_dir = positional_encoding(dirs, 4, dtype)                          # :362
    acts = {"enc_xyz": enc_xyz, "enc_dir": enc_dir}
    h = enc_xyz
    for i in range(8):                                                     # :366-372
        W, b = p[f"dense_{i}"]
        h = relu(h @ W + b)
        acts[f"h{i}"] = h
        if i == 4:
            h = np.concatenate([h, enc_xyz], axis=-1)
    W, b = p["sigma"]
    sigma = relu(h @ W + b)                                                # :375
    W, b = p["dense_8"]
    bott = h @ W + b                                                       # :378
    h9in = np.concatenate([bott, enc_dir], axis=-1)                        # :381
    W, b = p["dense_9"]
    h9 = relu(h9in @ W + b)                                                # :384
    W, b = p["rgb"]
    rgb = sigmoid(h9 @ W + b)                                              # :387
    acts.update(bott=bott, h9=h9, sigma_pre=None)
    if cache:
        return rgb, sigma, acts
    return rgb, sigma


def nerf_forward(params, p_coarse, p_fine, rays_o, rays_d, near, far,
                 u_coarse, u_fine, dtype=F32, mlp=None):
    """NeRF.forward (model.py:57-125) with supplied uniforms. ``mlp(p, xyz,
    dirs)`` replaces mlp_forward when given (e.g. mlp_forward_lowp)."""
    if mlp is None:
        mlp = lambda p, x, d: mlp_forward(p, x, d, dtype)  # noqa: E731
    d_cm = create_input_batch_coarse_model(params, rays_o, rays_d, near, far,
                                           u_coarse, dtype)
    rgb_c, sig_c = mlp(p_coarse, d_cm["xyz_inputs"], d_cm["dir_inputs"])
    pp_cm = post_process_model_output(rgb_c, sig_c, d_cm["t_vals"],
                                      params.system.white_bg)
    d_fm = create_input_batch_fine_model(params, rays_o, rays_d, pp_cm["weights"],
                                         d_cm["bin_data"], d_cm["t_vals"], u_fine,
                                         dtype)
    rgb_f, sig_f = mlp(p_fine, d_fm["xyz_inputs"], d_fm["dir_inputs"])
    pp_fm = post_process_model_output(rgb_f, sig_f, d_fm["t_vals"],
                                      params.system.white_bg)
    return pp_cm, pp_fm


def psnr(y_true, y_pred):
    """nerf/core/ops.py:249-257 (per-element mean)."""
    mse = np.mean(np.square(np.asarray(y_true, F64) - np.asarray(y_pred, F64)))
    return -10.0 * (np.log(mse) / np.log(10.0))


# ---------------------------------------------------------------------------
# Synthetic rays (test-side restatement of ray_utils.get_rays, :6-51)
# ---------------------------------------------------------------------------
def get_rays(H, W, intrinsic, c2w):
    """ray_utils.py:6-51 in float64 (pose_utils.normalize uses EPS 1e-8)."""
    u, v = np.meshgrid(np.arange(W, dtype=F64), np.arange(H, dtype=F64), indexing="xy")
    x = (u - intrinsic[0, 2]) / intrinsic[0, 0]
    y = (v - intrinsic[1, 2]) / intrinsic[1, 1]
    d = np.stack([x, y, np.ones_like(x)], -1).reshape(-1, 3)
    d = d @ c2w[:3, :3].T
    d = d / (np.sqrt(np.sum(d ** 2, axis=1, keepdims=True)) + 1e-8)
    o = np.broadcast_to(c2w[:3, 3], d.shape)
    return o, d


def get_rays_tf(H, W, intrinsic, c2w):
    """ray_utils.py:53-106 in float32. The matmul (:96) and the reduce_sum
    (:99) are sequential left-to-right sums without FMA (TF leaves their
    order open); z = 1 makes the third product exact."""
    K = np.asarray(intrinsic, F32)
    T = np.asarray(c2w, F32)
    u, v = np.meshgrid(np.arange(W, dtype=F32), np.arange(H, dtype=F32), indexing="xy")
    x = ((u - K[0, 2]) / K[0, 0]).reshape(-1)                              # :86
    y = ((v - K[1, 2]) / K[1, 1]).reshape(-1)                              # :87
    d = np.stack([(x * T[i, 0] + y * T[i, 1]) + T[i, 2] for i in range(3)], -1)  # :94-96
    m = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]       # :99
    d = d / (np.sqrt(m) + F32(1e-8))[:, None]                              # :100
    o = np.broadcast_to(T[:3, 3], d.shape)                                 # :103
    return o, d


def sample_mode_batch(img, pose, bounds, intrinsic, idxs):
    """base_dataset.py:555-621 with the indices supplied (the reference
    draws them with tf.random.uniform at :605-608)."""
    H, W = img.shape[:2]
    o, d = get_rays_tf(H, W, intrinsic, pose)                               # :589-591
    rgb = img.reshape(-1, 3).astype(F32) / F32(255.0)                      # :595-597
    n = o.shape[0]
    near = np.full((n, 1), bounds[0], F32)
    far = np.full((n, 1), bounds[1], F32)                                  # :599-602
    i = np.asarray(idxs)
    return (o[i], d[i], near[i], far[i]), (rgb[i],)                        # :610-614


def create_depth_map(pred_depth, H, W, scale_factor, map_type, intrinsic=None, C_to_W2=None):
    """ray_utils.py:108-135 (float64, NumPy get_rays)."""
    ds = np.asarray(pred_depth, F64) * (1 / scale_factor)                 # :117
    if map_type == "type_1":
        return ds.reshape(H, W)                                            # :120
    o, d = get_rays(H, W, np.asarray(intrinsic, F64), np.asarray(C_to_W2, F64))  # :123
    pts = o + d * ds[:, None]                                              # :124
    w2c = np.linalg.inv(np.asarray(C_to_W2, F64))                          # :126
    cam = pts @ w2c[:3, :3].T + w2c[:3, 3]                                 # :127
    return cam[:, 2].reshape(H, W)                                         # :129-130


# ---------------------------------------------------------------------------
# Philox4x32-10 in numpy (Salmon et al., SC 2011), to check the library's
# device uniforms: element e of the stream keyed by seed is output (e mod 4)
# of counter (e div 4), top 24 bits scaled to [0, 1).
# ---------------------------------------------------------------------------
def philox4x32_10(x0, x1, x2, x3, k0, k1):
    """Ten Philox4x32 rounds on uint32 arrays; returns the four output words."""
    M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
    W0, W1 = np.uint32(0x9E3779B9), np.uint32(0xBB67AE85)
    x0, x1, x2, x3 = (np.asarray(v, np.uint32) for v in (x0, x1, x2, x3))
    k0, k1 = np.uint32(k0), np.uint32(k1)
    with np.errstate(over="ignore"):
        for _ in range(10):
            p0 = M0 * x0.astype(np.uint64)
            p1 = M1 * x2.astype(np.uint64)
            hi0, lo0 = (p0 >> np.uint64(32)).astype(np.uint32), p0.astype(np.uint32)
            hi1, lo1 = (p1 >> np.uint64(32)).astype(np.uint32), p1.astype(np.uint32)
            x0, x1, x2, x3 = hi1 ^ x1 ^ k0, lo1, hi0 ^ x3 ^ k1, lo0
            k0 = np.uint32(k0 + W0)
            k1 = np.uint32(k1 + W1)
    return x0, x1, x2, x3


def philox_words(seed, offset, n):
    """Words offset .. offset + n - 1 of the stream keyed by seed (uint32)."""
    e = np.arange(offset, offset + n, dtype=np.uint64)
    c = e >> np.uint64(2)
    lo = (c & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    hi = (c >> np.uint64(32)).astype(np.uint32)
    z = np.zeros_like(lo)
    words = np.stack(philox4x32_10(lo, hi, z, z, seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF), axis=1)
    return words[np.arange(n), (e & np.uint64(3)).astype(np.int64)]


def philox_uniform(seed, offset, n):
    w = philox_words(seed, offset, n)
    return (w >> np.uint32(8)).astype(np.float32) * np.float32(1.0 / 16777216.0)


def philox_uniform_int(seed, offset, n, maxval):
    """Integers in [0, maxval): (word * maxval) >> 32."""
    w = philox_words(seed, offset, n).astype(np.uint64)
    return ((w * np.uint64(maxval)) >> np.uint64(32)).astype(np.int32)


# ---------------------------------------------------------------------------
# Gradients (the reference takes them with tf.GradientTape, model.py:148-171)
# ---------------------------------------------------------------------------
def composite_backward(sigma, t_vals, sample_rgb, grad_rgb_map=None, grad_weights=None,
                       white_bg=False, last_delta=1e10):
    """Analytic gradient of compute_weights/post_process_model_output
    (ray_utils.py:426-551) w.r.t. sigma [R*S] and sample_rgb [R*S,3], given
    dL/dpred_rgb [R,3] and/or dL/dweights [R,S]."""
    t = np.asarray(t_vals)
    dtype = t.dtype.type
    R, S = t.shape
    sig = np.asarray(sigma, dtype).reshape(R, S)
    rgb = np.asarray(sample_rgb, dtype).reshape(R, S, 3)
    dl = t[:, -1:] - t[:, -2:-1] if last_delta is None else np.full((R, 1), dtype(last_delta), dtype)
    delta = np.concatenate([t[:, 1:] - t[:, :-1], dl], 1)
    e = np.exp(-sig * delta)
    alpha = 1 - e
    fac = dtype(1) - alpha + dtype(1e-10)
    T = np.concatenate([np.ones((R, 1), dtype), np.cumprod(fac, axis=1)[:, :-1]], 1)
    w = alpha * T
    g = np.zeros((R, S), dtype) if grad_weights is None else np.asarray(grad_weights, dtype).copy()
    d_rgb = np.zeros_like(rgb)
    if grad_rgb_map is not None:
        G = np.asarray(grad_rgb_map, dtype)
        g = g + np.einsum("rsc,rc->rs", rgb, G)
        if white_bg:
            g = g - G.sum(1, keepdims=True)
        d_rgb = w[..., None] * G[:, None, :]
    gw = g * w
    suffix = np.concatenate([np.cumsum(gw[:, ::-1], axis=1)[:, ::-1][:, 1:], np.zeros((R, 1), dtype)], 1)
    d_alpha = g * T - suffix / fac
    d_sigma = d_alpha * delta * e
    return d_sigma.reshape(-1), d_rgb.reshape(-1, 3)


def proposal_weights(sigma, t_vals):
    """compute_weights with the last interval = the previous spacing."""
    t = np.asarray(t_vals)
    dtype = t.dtype.type
    R, S = t.shape
    delta = np.concatenate([t[:, 1:] - t[:, :-1], t[:, -1:] - t[:, -2:-1]], 1)
    alpha = 1 - np.exp(-np.asarray(sigma, dtype).reshape(R, S) * delta)
    fac = dtype(1) - alpha + dtype(1e-10)
    T = np.concatenate([np.ones((R, 1), dtype), np.cumprod(fac, axis=1)[:, :-1]], 1)
    return alpha * T


def apply_adam(var, m, v, grad, step, lr, beta1=0.9, beta2=0.999, eps=1e-7):
    """TensorFlow's ApplyAdam as Keras' Adam calls it (model.py:418 uses
    Keras defaults): lr_t = lr sqrt(1-b2^t)/(1-b1^t); m += (g-m)(1-b1);
    v += (g^2-v)(1-b2); var -= lr_t m/(sqrt(v)+eps). Returns new (var, m, v)."""
    b1p, b2p = beta1 ** step, beta2 ** step
    lr_t = lr * np.sqrt(1 - b2p) / (1 - b1p)
    m = m + (grad - m) * (1 - beta1)
    v = v + (grad * grad - v) * (1 - beta2)
    var = var - lr_t * m / (np.sqrt(v) + eps)
    return var, m, v


def lr_schedule(step):
    """ExponentialDecay(5e-4, 500000, 0.1), not staircase (model.py:413-417)."""
    return 5e-4 * 0.1 ** (step / 500000.0)


# ---------------------------------------------------------------------------
# Proposal network (not in the reference): 2x64 ReLU MLP on the L=6 encoding
# of xyz (39 inputs, model.py:330 concatenation convention), softplus density;
# its weights are composited over finite bins (last interval = the previous
# spacing instead of ray_utils.py:465's 1e10).
# Flat blob: W1 [39,64], b1 [64], W2 [64,64], b2 [64], W3 [64], b3 [1].
# ---------------------------------------------------------------------------
PROP_SHAPES = (("W1", (39, 64)), ("b1", (64,)), ("W2", (64, 64)), ("b2", (64,)),
               ("W3", (64,)), ("b3", (1,)))


def prop_unpack(blob, dtype=F32):
    out, off = {}, 0
    for name, shp in PROP_SHAPES:
        n = int(np.prod(shp))
        out[name] = np.asarray(blob[off:off + n], dtype).reshape(shp)
        off += n
    return out


def prop_pack(p):
    return np.concatenate([np.asarray(p[name]).reshape(-1) for name, _ in PROP_SHAPES])


def softplus(x):
    return np.maximum(x, 0) + np.log1p(np.exp(-np.abs(x)))


def prop_forward(blob, xyz, dtype=F32, cache=False):
    p = prop_unpack(blob, dtype)
    enc = positional_encoding(xyz, 6, dtype)
    z1 = enc @ p["W1"] + p["b1"]
    h1 = relu(z1)
    z2 = h1 @ p["W2"] + p["b2"]
    h2 = relu(z2)
    z3 = h2 @ p["W3"] + p["b3"][0]
    sigma = softplus(z3)
    if cache:
        return sigma, dict(enc=enc, z1=z1, h1=h1, z2=z2, h2=h2, z3=z3)
    return sigma


def prop_backward(blob, xyz, d_sigma, dtype=F64):
    """Gradient of sum(d_sigma * prop_forward(xyz)) w.r.t. the flat blob."""
    p = prop_unpack(blob, dtype)
    _, c = prop_forward(blob, xyz, dtype, cache=True)
    dz3 = np.asarray(d_sigma, dtype) / (1 + np.exp(-c["z3"]))
    g = {"W3": c["h2"].T @ dz3, "b3": np.array([dz3.sum()])}
    dz2 = np.outer(dz3, p["W3"]) * (c["z2"] > 0)
    g["W2"] = c["h1"].T @ dz2
    g["b2"] = dz2.sum(0)
    dz1 = (dz2 @ p["W2"].T) * (c["z1"] > 0)
    g["W1"] = c["enc"].T @ dz1
    g["b1"] = dz1.sum(0)
    return prop_pack(g)


def prop_loss(w_prop, w_target, lam=3.0):
    """Envelope loss on the 64-bin weight histograms: squared error, with
    under-estimates of the target weighted (1 + lam). Mean over rays.
    Returns (loss, dL/dw_prop)."""
    diff = np.asarray(w_prop) - np.asarray(w_target)
    rho = 1 + lam * (diff < 0)
    R = diff.shape[0]
    return float(np.sum(rho * diff * diff) / R), 2 * rho * diff / R


# ---------------------------------------------------------------------------
# Proposal-gated render (not in the reference): the chain of nerf_forward in
# which the coarse samples whose proposal weight is at most tau have sigma 0,
# in the coarse pass and again in the fine pass's sorted union (fine draws
# are always evaluated; a skipped sample's rgb is 0).
# ---------------------------------------------------------------------------
def gate_coarse(w_prop, tau):
    """On/off of each coarse sample [R, Sc]: w_prop > tau (NaN: off)."""
    return np.asarray(w_prop) > tau


def gate_fine(sort_perm, mask_c, piece_idxs=None):
    """On/off of each member of the sorted union [R, S]: a coarse sample
    whose gate is on, or a fine draw (sort_perm >= Sc). With piece_idxs
    [R, Sf] (the fine sampler's bin of each draw) a fine draw is on only
    where its bin's coarse gate is on."""
    mask_c = np.asarray(mask_c, bool)
    Sc = mask_c.shape[1]
    perm = np.asarray(sort_perm)
    on_c = np.take_along_axis(mask_c, np.minimum(perm, Sc - 1), axis=1)
    if piece_idxs is None:
        on_f = np.ones(perm.shape, bool)
    else:
        piece = np.asarray(piece_idxs)
        bins = np.take_along_axis(piece, np.clip(perm - Sc, 0, piece.shape[1] - 1), axis=1)
        on_f = np.take_along_axis(mask_c, bins, axis=1)
    return np.where(perm >= Sc, on_f, on_c)


def nerf_render_gated(params, prop_blob, p_coarse, p_fine, rays_o, rays_d, near, far,
                      u_coarse, u_fine, tau, dtype=F32, mlp=None, prop=None, mask_c=None,
                      gate_draws=False):
    """Returns (fine post_process_model_output, coarse mask [R,Sc], union
    mask [R,S], proposal weights [R,Sc]). ``mlp(p, xyz, dirs)`` and
    ``prop(blob, xyz)`` replace mlp_forward and prop_forward when given;
    ``mask_c`` [R,Sc] replaces the coarse gate's decisions (e.g. the ones a
    device run made); ``gate_draws`` gates the fine draws by their bins'
    coarse decisions too."""
    if mlp is None:
        mlp = lambda p, x, d: mlp_forward(p, x, d, dtype)  # noqa: E731
    if prop is None:
        prop = lambda b, x: prop_forward(b, x, dtype)  # noqa: E731
    d_cm = create_input_batch_coarse_model(params, rays_o, rays_d, near, far, u_coarse, dtype)
    t_c = d_cm["t_vals"]
    Sc = t_c.shape[1]
    w_p = proposal_weights(prop(prop_blob, d_cm["xyz_inputs"]), t_c)
    m_c = gate_coarse(w_p, tau) if mask_c is None else np.asarray(mask_c, bool).reshape(t_c.shape)
    _, sig_c = mlp(p_coarse, d_cm["xyz_inputs"], d_cm["dir_inputs"])
    sig_c = np.where(m_c.reshape(-1), sig_c.reshape(-1), dtype(0))
    w_c = compute_weights(sig_c, t_c, Sc)
    d_fm = create_input_batch_fine_model(params, rays_o, rays_d, w_c, d_cm["bin_data"], t_c,
                                         u_fine, dtype, return_indices=True)
    rgb_f, sig_f = mlp(p_fine, d_fm["xyz_inputs"], d_fm["dir_inputs"])
    m_f = gate_fine(d_fm["sort_perm"], m_c, d_fm["piece_idxs"] if gate_draws else None)
    on = m_f.reshape(-1)
    sig_f = np.where(on, sig_f.reshape(-1), dtype(0))
    rgb_f = np.where(on[:, None], rgb_f, dtype(0))
    pp = post_process_model_output(rgb_f, sig_f, d_fm["t_vals"], params.system.white_bg)
    return pp, m_c, m_f, w_p


def mlp_backward(p, xyz, dirs, d_rgb, d_sigma, dtype=F64):
    """Gradient of sum(d_rgb * rgb + d_sigma * sigma) of mlp_forward
    (model.py:334-394) w.r.t. every layer: {name: (dW, db)}."""
    p = {k: (np.asarray(W, dtype), np.asarray(b, dtype)) for k, (W, b) in p.items()}
    _, _, a = mlp_forward(p, xyz, dirs, dtype, cache=True)
    return mlp_backward_cached(p, a, d_rgb, d_sigma, dtype)


def acts_from_tape(tape, dtype=F64):
    """The activation cache of mlp_forward from a stored tape [n, 2528]:
    enc_xyz [64] | h0..h7 [8 x 256] | bottleneck [256] | enc_dir [32] | h9."""
    t = np.asarray(tape, dtype)
    a = {"enc_xyz": t[:, 0:63], "enc_dir": t[:, 2368:2395], "bott": t[:, 2112:2368], "h9": t[:, 2400:2528]}
    for i in range(8):
        a[f"h{i}"] = t[:, 64 + 256 * i:64 + 256 * (i + 1)]
    return a


def mlp_backward_cached(p, a, d_rgb, d_sigma, dtype=F64):
    """mlp_backward on a given activation cache (the heads are recomputed
    from h7 and h9)."""
    p = {k: (np.asarray(W, dtype), np.asarray(b, dtype)) for k, (W, b) in p.items()}
    rgb = sigmoid(a["h9"] @ p["rgb"][0] + p["rgb"][1])
    sigma = relu(a["h7"] @ p["sigma"][0] + p["sigma"][1])
    d_sigma = np.asarray(d_sigma, dtype).reshape(-1, 1)
    g = {}
    dz = np.asarray(d_rgb, dtype) * rgb * (1 - rgb)                      # sigmoid
    g["rgb"] = (a["h9"].T @ dz, dz.sum(0))
    dh9 = dz @ p["rgb"][0].T
    dz9 = dh9 * (a["h9"] > 0)
    h9in = np.concatenate([a["bott"], a["enc_dir"]], -1)
    g["dense_9"] = (h9in.T @ dz9, dz9.sum(0))
    dbott = (dz9 @ p["dense_9"][0].T)[:, :256]
    g["dense_8"] = (a["h7"].T @ dbott, dbott.sum(0))
    dh7 = dbott @ p["dense_8"][0].T
    dzs = d_sigma * (sigma > 0)                                          # sigma ReLU
    g["sigma"] = (a["h7"].T @ dzs, dzs.sum(0))
    dh7 = dh7 + dzs @ p["sigma"][0].T
    dh = dh7
    for i in range(7, -1, -1):
        dz_i = dh * (a[f"h{i}"] > 0)
        if i == 0:
            inp = a["enc_xyz"]
        elif i == 5:
            inp = np.concatenate([a["h4"], a["enc_xyz"]], -1)
        else:
            inp = a[f"h{i - 1}"]
        g[f"dense_{i}"] = (inp.T @ dz_i, dz_i.sum(0))
        dinp = dz_i @ p[f"dense_{i}"][0].T
        dh = dinp[:, :256] if i == 5 else dinp
    return g


def mse(y_true, y_pred):
    """keras.losses.MeanSquaredError: mean over every element (model.py:32)."""
    d = np.asarray(y_pred) - np.asarray(y_true)
    return float(np.mean(d * d)), 2 * d / d.size


# ---------------------------------------------------------------------------
# Low-precision emulation (not in the reference): the arithmetic that the
# build's tensor-core MLPs are specified to do, evaluated in float64 so that
# only the specified roundings differ from the FP64 oracle. BF16: every GEMM
# operand (encodings, activations, weights) rounded to BF16, products summed
# exactly, the sum rounded to FP32, the FP32 bias added in FP32. FP8: E4M3
# operands, each weight column n divided by s_n = max_k |W[k,n]| / 448 before
# rounding, the sum rounded to FP32 and mapped back as fma(sum, s_n, b_n).
# The sigma and rgb heads run in FP32 on the unrounded activations, as in
# the FP32 path (model.py:374-387).
# ---------------------------------------------------------------------------
E4M3_MAX = 448.0


def round_bf16(a):
    """Round-to-nearest-even of float32 values to BF16 (8 significand bits),
    returned as float32."""
    u = np.array(a, F32, copy=True).view(np.uint32)   # finite values: no overflow below
    r = (u >> 16) & np.uint32(1)
    u += np.uint32(0x7FFF)
    u += r
    u &= np.uint32(0xFFFF0000)
    return u.view(F32).reshape(np.shape(a))


def round_e4m3(a):
    """Round-to-nearest-even of float32 values to FP8 E4M3 (4 significand
    bits, exponents -6..8, subnormal step 2^-9), saturated to +-448
    (OCP FP8 formats, satfinite conversion), returned as float32."""
    x = np.asarray(a, F32)
    # normal range: keep 3 of float32's 23 fraction bits, ties to even (a
    # carry into the exponent is the correct next binade)
    u = np.array(x, F32, copy=True).view(np.uint32)
    r = (u >> 20) & np.uint32(1)
    u += np.uint32(0x7FFFF)
    u += r
    u &= np.uint32(0xFFF00000)
    y = u.view(F32).reshape(x.shape)
    # below 2^-6: multiples of the subnormal step 2^-9 (exact scaling, rint ties to even)
    small = np.abs(x) < F32(2.0 ** -6)
    y = np.where(small, np.rint(x * F32(512.0)) / F32(512.0), y)
    return np.clip(y, F32(-E4M3_MAX), F32(E4M3_MAX)).astype(F32)


def fp8_scales(W):
    """Per-output-channel weight scales s_n = max_k |W[k, n]| / 448 (FP32)."""
    return (np.abs(np.asarray(W, F32)).max(axis=0) / F32(E4M3_MAX)).astype(F32)


def _gemm_lowp(a_q, W, b, fmt):
    """One Dense layer of the tensor-core kernels: a_q [M, K] already in the
    operand format. Returns the FP32 pre-activation."""
    W = np.asarray(W, F32)
    b = np.asarray(b, F32)
    if fmt == "bf16":
        acc = (a_q.astype(F64) @ round_bf16(W).astype(F64)).astype(F32)
        return (acc + b).astype(F32)
    s = fp8_scales(W)
    wq = round_e4m3(np.where(s > 0, W / np.where(s > 0, s, F32(1)), F32(0)).astype(F32))
    acc = (a_q.astype(F64) @ wq.astype(F64)).astype(F32)
    return (acc.astype(F64) * s + b).astype(F32)   # fmaf(acc, s, b): one rounding


def positional_encoding_kernel(x, L):
    """positional_encoding (float32) as the tensor-core MLP kernels compute
    it (nerf-tf2_gb300/csrc/mlp_tc.cu, encode_pairs_q): octave l from sin/cos
    at octave 4*floor(l/4) and l % 4 angle doublings, sin 2a = (2 sin a)
    cos a, cos 2a = cos a cos a - sin a sin a, each operation rounded in
    float32."""
    x = np.asarray(x, F32)
    mult = encoder_multipliers(L, F32)
    out = np.empty((x.shape[0], 3 + 6 * L), F32)
    out[:, :3] = x
    for c in range(3):
        for l0 in range(0, L, 4):
            th = (x[:, c] * mult[l0]).astype(F32)
            s, co = np.sin(th).astype(F32), np.cos(th).astype(F32)
            for l in range(l0, min(l0 + 4, L)):
                if l > l0:
                    s, co = (F32(2) * s) * co, co * co - s * s
                out[:, 3 + c * 2 * L + 2 * l] = s
                out[:, 4 + c * 2 * L + 2 * l] = co
    return out


def mlp_forward_lowp(p, xyz, dirs, fmt):
    """get_coarse_or_fine_model's network (model.py:334-394) as the BF16
    (fmt="bf16") or FP8-e4m3 (fmt="fp8") tensor-core kernels compute it.
    p: unpack_params(blob, F32). Returns (rgb [M,3], sigma [M,1]) float32."""
    q = round_bf16 if fmt == "bf16" else round_e4m3
    enc_xyz = q(positional_encoding_kernel(xyz, 10))
    enc_dir = q(positional_encoding_kernel(dirs, 4))
    h = enc_xyz
    for i in range(8):
        v = _gemm_lowp(h, *p[f"dense_{i}"], fmt)
        h = q(np.maximum(v, 0))
        if i == 4:
            h = np.concatenate([h, enc_xyz], axis=-1)
    W, b = p["sigma"]
    sigma = np.maximum(np.maximum(v, 0).astype(F64) @ np.asarray(W, F64) + np.asarray(b, F64), 0)
    v8 = _gemm_lowp(h, *p["dense_8"], fmt)
    h9in = np.concatenate([q(v8), enc_dir], axis=-1)
    v9 = _gemm_lowp(h9in, *p["dense_9"], fmt)
    W, b = p["rgb"]
    z = np.maximum(v9, 0).astype(F64) @ np.asarray(W, F64) + np.asarray(b, F64)
    rgb = 1.0 / (1.0 + np.exp(-z))
    return rgb.astype(F32), sigma.astype(F32)


def proposal_encoding_kernel(xyz):
    """The L=6 encoding as the proposal's tensor-core kernels compute it
    (nerf-tf2_gb300/csrc/proposal.cu, encode_octaves_bf16): per coordinate
    chain, sin/cos at the first octave of the chain, then each next octave
    by sin 2a = (2 sin a) cos a, cos 2a = cos a cos a - sin a sin a in float32
    (rounded per operation); chains: coordinates 0 and 1 over octaves 0-5,
    coordinate 2 over 0-2 and over 3-5."""
    x = np.asarray(xyz, F32)
    out = np.zeros((x.shape[0], 39), F32)
    out[:, :3] = x
    mult = encoder_multipliers(6, F32)
    for c, l0, l1 in ((0, 0, 6), (1, 0, 6), (2, 0, 3), (2, 3, 6)):
        th = (x[:, c] * mult[l0]).astype(F32)
        s, co = np.sin(th).astype(F32), np.cos(th).astype(F32)
        for l in range(l0, l1):
            if l > l0:
                s, co = (F32(2) * s) * co, co * co - s * s
            out[:, 3 + c * 12 + 2 * l] = s
            out[:, 4 + c * 12 + 2 * l] = co
    return out


def prop_forward_bf16(blob, xyz):
    """The proposal network (prop_forward) as its tensor-core kernel computes
    it: the kernels' encoding (proposal_encoding_kernel) in BF16, W1, h1 and
    W2 in BF16, FP32 biases, the last layer in FP32."""
    p = prop_unpack(blob, F32)
    enc = proposal_encoding_kernel(xyz)
    h1 = np.maximum(round_bf16(enc).astype(F64) @ round_bf16(p["W1"]).astype(F64) + p["b1"], 0)
    z2 = round_bf16(h1.astype(F32)).astype(F64) @ round_bf16(p["W2"]).astype(F64) + p["b2"]
    z3 = np.maximum(z2, 0) @ p["W3"].astype(F64) + p["b3"][0]
    return softplus(z3).astype(F32)
