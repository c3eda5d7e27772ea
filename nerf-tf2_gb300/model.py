"""Drop-in for the render-path parts of nerf/core/model.py, on CUDA.

* ``PositionalEncoder(L, name=None)`` - model.py:289-332.
* ``get_coarse_or_fine_model(model_name, num_units=256)`` - model.py:334-394;
  returns a callable ``model(inputs=(xyz, dir)) -> (rgb [M,3], sigma [M,1])``
  whose weights live on the device as the flat blob of ``weights.py``.
* ``NeRF(params)`` with ``forward(rays_o, rays_d, near, far)`` -
  model.py:18-125; returns ``(post_proc_CM, post_proc_FM)``.

The MLP runs as one kernel per call: FP32 SIMT (``precision="fp32"``, the
plain path), BF16 tcgen05 GEMMs (``precision="bf16"``) or FP8-e4m3 tcgen05
GEMMs with per-output-channel weight scales (``precision="fp8"``), both
accumulating in FP32.
"""
import ctypes

import torch

from . import _lib, h5, ray_utils
from ._tensors import as_cuda, device, empty, ptr, stream
from .weights import PARAM_COUNT, from_dict, glorot_blob, optimizer_state_from_npz, to_dict
from .weights import from_keras_layers as weights_from_keras

PRECISIONS = {"fp32": _lib.PREC_FP32, "bf16": _lib.PREC_BF16, "fp8": _lib.PREC_FP8}


class PositionalEncoder:
    """model.py:289-332: x [n,3] -> [x, sin(x 2^l pi), cos(x 2^l pi)] with the
    reference's interleaving (coordinate-major, then frequency, then
    sin/cos)."""

    def __init__(self, L, name=None):
        self.L = int(L)
        self.name = name

    def __call__(self, x):
        x = as_cuda(x, name="x")
        n = x.shape[0]
        x = as_cuda(x, shape=(n, 3), name="x")
        out = empty(n, 3 + 6 * self.L)
        _lib.call("nerfgb_positional_encode", ptr(x), n, self.L, ptr(out), stream())
        return out

    call = __call__


class NerfMLP:
    """The Keras model of get_coarse_or_fine_model as a device-resident
    callable. ``params`` is the flat float32 blob (``weights.py``)."""

    def __init__(self, model_name, params=None, seed=0, precision="fp32"):
        self.name = model_name
        blob = glorot_blob(seed) if params is None else params
        self.params = as_cuda(blob, shape=(PARAM_COUNT,), name="params").clone()
        self.precision = precision
        self._packed = {}
        self._version = 0
        self.err_word = torch.zeros(1, dtype=torch.int32, device=device())

    # -- weights -------------------------------------------------------------
    def mark_updated(self):
        """Call after changing ``params`` in place; repacks lazily."""
        self._version += 1

    def packed(self, precision=None):
        prec = PRECISIONS[precision or self.precision]
        hit = self._packed.get(prec)
        if hit is not None and hit[0] == self._version:
            return hit[1]
        nbytes = _lib.lib().nerfgb_mlp_packed_bytes(prec)
        buf = torch.empty(nbytes, dtype=torch.uint8, device=self.params.device)
        _lib.call("nerfgb_mlp_pack", ptr(self.params), prec, ptr(buf), stream())
        self._packed[prec] = (self._version, buf)
        return buf

    def get_weights(self):
        """{"<model>/<layer>/kernel:0": ndarray, ...} (Keras variable names)."""
        return to_dict(self.params.detach().cpu().numpy(), self.name)

    def set_weights(self, d):
        blob = from_dict(d, self.name)
        with torch.no_grad():
            self.params.copy_(torch.from_numpy(blob))
        self.mark_updated()

    def load_weights(self, path):
        """Keras's Model.load_weights for an HDF5 weight file written by the
        reference (nerf/core/ops.py:142-143): the file's layers matched to the
        network's by their Keras names, kernel and bias per layer (h5.py
        reads the file without h5py)."""
        self.set_weights(weights_from_keras(h5.keras_layer_weights(path), self.name))

    # -- forward -------------------------------------------------------------
    def __call__(self, inputs, *, precision=None, rows_per_dir=1):
        xyz, dirs = inputs
        xyz = as_cuda(xyz, name="xyz")
        n = xyz.shape[0]
        xyz = as_cuda(xyz, shape=(n, 3), name="xyz")
        nd = (n + rows_per_dir - 1) // rows_per_dir
        dirs = as_cuda(dirs, shape=(nd, 3), name="dir")
        prec = PRECISIONS[precision or self.precision]
        rgb = empty(n, 3)
        sigma = empty(n, 1)
        _lib.call("nerfgb_mlp_forward", ptr(self.packed(precision)), prec, ptr(xyz), ptr(dirs), n,
                  int(rows_per_dir), ptr(rgb), ptr(sigma), ptr(self.err_word), stream())
        return rgb, sigma

    call = __call__

    def forward_train(self, xyz, dirs, rows_per_dir=1, precision="fp32"):
        """Forward that also returns the stored activations for ``backward``
        (the tape of tf.GradientTape, model.py:148). "fp32": the FP32 kernel
        and an FP32 tape; "bf16": the tensor-core kernel and a BF16 tape
        (int16 tensor of BF16 bits) holding the operands its GEMMs read."""
        if precision not in ("fp32", "bf16"):
            raise ValueError(f"training forward precision must be fp32 or bf16, not {precision!r}")
        xyz = as_cuda(xyz, name="xyz")
        n = xyz.shape[0]
        dirs = as_cuda(dirs, shape=((n + rows_per_dir - 1) // rows_per_dir, 3), name="dir")
        rgb, sigma = empty(n, 3), empty(n, 1)
        ld = int(_lib.lib().nerfgb_mlp_acts_floats_per_row())
        if precision == "bf16":
            acts = torch.empty(n, ld, dtype=torch.int16, device=xyz.device)
            _lib.call("nerfgb_mlp_forward_train_bf16", ptr(self.packed("bf16")), ptr(xyz), ptr(dirs), n,
                      int(rows_per_dir), ptr(rgb), ptr(sigma), ptr(acts), ptr(self.err_word), stream())
        else:
            acts = empty(n, ld)
            _lib.call("nerfgb_mlp_forward_train", ptr(self.packed("fp32")), ptr(xyz), ptr(dirs), n,
                      int(rows_per_dir), ptr(rgb), ptr(sigma), ptr(acts), stream())
        return rgb, sigma, acts

    def backward(self, acts, d_rgb, d_sigma, grad_params):
        """Accumulates the parameter gradient of sum(d_rgb*rgb + d_sigma*sigma)
        into grad_params (flat Keras layout). An FP32 tape takes the FP32
        backward; a BF16 tape (from ``forward_train(precision="bf16")``) the
        BF16 one (BF16 tensor-core GEMMs, FP32 accumulation, FP32
        gradients; a bounded-wait timeout lands in err_word)."""
        n = acts.shape[0]
        d_rgb = as_cuda(d_rgb, shape=(n, 3), name="d_rgb")
        d_sigma = as_cuda(d_sigma, shape=(n,), name="d_sigma")
        lib = _lib.lib()
        bf16 = acts.dtype == torch.int16
        nbytes = (lib.nerfgb_mlp_backward_bf16_workspace_bytes if bf16 else lib.nerfgb_mlp_backward_workspace_bytes)(n)
        ws = torch.empty(int(nbytes), dtype=torch.uint8, device=acts.device)
        if bf16:
            _lib.call("nerfgb_mlp_backward_bf16", ptr(self.packed("fp32")), ptr(acts), n, ptr(d_rgb),
                      ptr(d_sigma), ptr(grad_params), ptr(ws), ptr(self.err_word), stream())
        else:
            _lib.call("nerfgb_mlp_backward", ptr(self.packed("fp32")), ptr(acts), n, ptr(d_rgb), ptr(d_sigma),
                      ptr(grad_params), ptr(ws), stream())
        return grad_params

    def check_device_errors(self):
        """Synchronises and raises if a bounded device wait timed out."""
        torch.cuda.synchronize()
        code = int(self.err_word.item())
        if code != 0:
            self.err_word.zero_()
            raise _lib.NerfgbError("nerfgb_mlp_forward (device)", code, _lib.status_name(code))


def get_coarse_or_fine_model(model_name, num_units=256, *, params=None, seed=0, precision="fp32"):
    """model.py:334-394. Only num_units=256 (the reference's value) has
    kernels."""
    assert model_name in ("coarse", "fine")
    if num_units != 256:
        raise ValueError("the CUDA MLP is specialised for num_units=256")
    return NerfMLP(model_name, params=params, seed=seed, precision=precision)


class NeRF:
    """model.py:18-125: coarse and fine networks plus the hierarchical
    render. ``forward`` mirrors the reference op by op and returns its dicts;
    ``render`` runs the same chain as one fused library call per chunk."""

    def __init__(self, params, *, precision="fp32", seed=0, coarse_params=None, fine_params=None,
                 trans_mode=None):
        self.params = params
        self.white_bg = bool(params.system.white_bg)
        self.precision = precision
        self.trans_mode = ray_utils.DEFAULT_TRANS_MODE if trans_mode is None else trans_mode
        self.coarse_model = get_coarse_or_fine_model("coarse", params=coarse_params, seed=seed,
                                                     precision=precision)
        self.fine_model = get_coarse_or_fine_model("fine", params=fine_params, seed=seed + 1,
                                                   precision=precision)
        # 2: the training backward runs the coarse network's gradient on a
        # side stream beside the fine network's (1: one stream)
        self.backward_streams = 2

    def forward(self, rays_o, rays_d, near, far, *, u_coarse=None, u_fine=None):
        """model.py:57-125 with optional explicit jitter uniforms."""
        data_CM = ray_utils.create_input_batch_coarse_model(
            params=self.params, rays_o=rays_o, rays_d=rays_d, near=near, far=far, u_vals=u_coarse)
        rgb_CM, sigma_CM = self.coarse_model(inputs=(data_CM["xyz_inputs"], data_CM["dir_inputs"]))
        post_proc_CM = ray_utils.post_process_model_output(
            sample_rgb=rgb_CM, sigma=sigma_CM, t_vals=data_CM["t_vals"], white_bg=self.white_bg,
            trans_mode=self.trans_mode)
        data_FM = ray_utils.create_input_batch_fine_model(
            params=self.params, rays_o=rays_o, rays_d=rays_d, bin_weights=post_proc_CM["weights"],
            t_vals_coarse=data_CM["t_vals"], bin_data=data_CM["bin_data"], u_vals=u_fine)
        rgb_FM, sigma_FM = self.fine_model(inputs=(data_FM["xyz_inputs"], data_FM["dir_inputs"]))
        post_proc_FM = ray_utils.post_process_model_output(
            sample_rgb=rgb_FM, sigma=sigma_FM, t_vals=data_FM["t_vals"], white_bg=self.white_bg,
            trans_mode=self.trans_mode)
        return post_proc_CM, post_proc_FM

    def __call__(self, inputs):
        """model.py:36-55: inputs[0] = (rays_o, rays_d, near, far)."""
        return self.forward(*inputs[0])

    # -- training (model.py:127-180, :396-432) -------------------------------
    def _train_state(self):
        if not hasattr(self, "_opt"):
            z = lambda: torch.zeros(PARAM_COUNT, device=self.coarse_model.params.device)  # noqa: E731
            self._opt = {"step": 0, "m": [z(), z()], "v": [z(), z()], "g": [z(), z()]}
        return self._opt

    def train_step(self, data, *, u_coarse=None, u_fine=None, lr=None, precision=None, tile_rays=4096):
        """One step of NeRF.train_step (model.py:127-180): the coarse and fine
        maps through autograd.RenderFunction, loss = MSE(coarse) + MSE(fine)
        (:157-168) through autograd.MSEFunction, ``loss.backward()`` (the
        hand-written backward: compositing, then the MLP, recomputing the
        activations per tile of ``tile_rays`` rays; None keeps the forward's
        tape instead), and a Keras Adam step with ExponentialDecay(5e-4,
        500000, 0.1) (:413-418) on the FP32 master weights. ``precision``:
        "fp32" (FP32 GEMMs) or "bf16" (BF16 tensor-core GEMMs forward and
        backward, FP32 accumulation); default: "bf16" for a BF16 or FP8
        model, else "fp32". ``data`` = ((rays_o, rays_d, near, far), (rgb,)).
        Returns {"loss", "coarse_loss", "fine_loss", "psnr"} as floats."""
        from . import autograd
        (rays_o, rays_d, near, far), (rgb,) = data
        rays_o = as_cuda(rays_o, name="rays_o")
        R = rays_o.shape[0]
        target = as_cuda(rgb, shape=(R, 3), name="rgb")
        st = self._train_state()
        st["step"] += 1
        for model in (self.coarse_model, self.fine_model):
            model.params.grad = None
        rgb_c, rgb_f = autograd.render_with_grad(self, rays_o, rays_d, near, far, u_coarse=u_coarse, u_fine=u_fine,
                                                 precision=precision, tile_rays=tile_rays)
        loss_c, loss_f = autograd.mse(rgb_c, target), autograd.mse(rgb_f, target)
        (loss_c + loss_f).backward()
        st["g"] = [self.coarse_model.params.grad, self.fine_model.params.grad]
        step_lr = 5e-4 * 0.1 ** (st["step"] / 500000.0) if lr is None else lr
        for k, model in enumerate((self.coarse_model, self.fine_model)):
            _lib.call("nerfgb_adam_step", ptr(model.params), ptr(st["m"][k]), ptr(st["v"][k]), ptr(st["g"][k]),
                      PARAM_COUNT, step_lr, 0.9, 0.999, 1e-7, st["step"], stream())
            model.mark_updated()
        lc, lf = float(loss_c.detach()), float(loss_f.detach())
        return {"loss": lc + lf, "coarse_loss": lc, "fine_loss": lf,
                "psnr": -10.0 * float(torch.log10(torch.tensor(max(lf, 1e-30))))}

    def gradients(self):
        """Flat parameter gradients of the last train_step: (coarse, fine)."""
        st = self._train_state()
        return st["g"][0], st["g"][1]

    call = __call__
    predict_step = __call__

    # -- fused inference ----------------------------------------------------
    def render_coarse(self, rays_o, rays_d, near, far, *, u_coarse=None, precision=None):
        """The coarse pass alone (model.py:88-100): stratified samples, the
        coarse network and compositing, three launches. Directions are read
        per ray by the MLP (no [R*S,3] dir_inputs tensor). Returns
        post_process_model_output's dict."""
        p = self.params
        rays_o = as_cuda(rays_o, name="rays_o")
        R = rays_o.shape[0]
        rays_d = as_cuda(rays_d, shape=(R, 3), name="rays_d")
        near = as_cuda(near, shape=(R, 1), name="near")
        far = as_cuda(far, shape=(R, 1), name="far")
        S = int(p.sampling.N_coarse)
        perturb = bool(p.sampling.perturb)
        if perturb:
            u = ray_utils.uniform((R, S)) if u_coarse is None else as_cuda(u_coarse, shape=(R, S), name="u_coarse")
        else:
            u = None
        xyz, t, edges, widths = empty(R * S, 3), empty(R, S), empty(R, S + 1), empty(R, S)
        _lib.call("nerfgb_coarse_sample", ptr(rays_o), ptr(rays_d), ptr(near), ptr(far), ptr(u), R, S,
                  int(perturb), int(bool(p.sampling.lin_inv_depth)), ptr(xyz), None, ptr(t), ptr(edges),
                  ptr(widths), stream())
        rgb_s, sig_s = self.coarse_model((xyz, rays_d), precision=precision, rows_per_dir=S)
        return ray_utils.post_process_model_output(rgb_s, sig_s, t, self.white_bg, trans_mode=self.trans_mode)

    def _side_streams(self, n):
        """n CUDA streams of the current device, made once and kept."""
        dev = torch.cuda.current_device()
        cache = self.__dict__.setdefault("_render_streams", {})
        have = cache.setdefault(dev, [])
        while len(have) < n:
            have.append(torch.cuda.Stream(device=dev))
        return have[:n]

    def render(self, rays_o, rays_d, near, far, *, chunk=4096, u_coarse=None, u_fine=None, seed=0,
               precision=None, return_coarse=False, proposal=None, proposal_mode="replace",
               gate_tau=1e-4, gate_fine_draws=True, streams=3):
        """Fine (and optionally coarse) rgb/depth/acc maps for every ray, in
        chunks of `chunk` rays (the reference renders 4096-ray batches,
        base_dataset.py:853-857). Uniforms come from Philox keyed by `seed`
        when not supplied. With `proposal` (a ProposalNetwork) no coarse maps
        are produced, and `proposal_mode` says how the proposal is used:
        "replace": its weights replace the coarse MLP's as the fine sampler's
        PDF (the coarse MLP does not run); "gate": the coarse and fine MLPs
        run as in the plain chain but skip the coarse samples whose proposal
        weight is at most `gate_tau` (sigma = 0 there); with
        `gate_fine_draws` they also skip the fine draws that fall in such a
        coarse bin.

        Chunk k runs on stream k % `streams` (the caller's current stream and
        `streams` - 1 side streams, each with its own workspace), so that one
        chunk's ray kernels fill the SMs another chunk's MLP leaves idle.
        Chunks are independent: the maps do not depend on `streams`. The
        side streams start after the caller's stream has reached this call
        and the caller's stream waits for them before returning, so the maps
        are ordered on the caller's stream like a single-stream render."""
        if proposal is not None and proposal_mode not in ("replace", "gate"):
            raise ValueError(f"proposal_mode must be 'replace' or 'gate', not {proposal_mode!r}")
        gated = proposal is not None and proposal_mode == "gate"
        prec = PRECISIONS[precision or self.precision]
        rays_o = as_cuda(rays_o, name="rays_o")
        R = rays_o.shape[0]
        rays_d = as_cuda(rays_d, shape=(R, 3), name="rays_d")
        near = as_cuda(near, shape=(R, 1), name="near")
        far = as_cuda(far, shape=(R, 1), name="far")
        Sc, Sf = int(self.params.sampling.N_coarse), int(self.params.sampling.N_fine)
        if u_coarse is not None:
            u_coarse = as_cuda(u_coarse, shape=(R, Sc), name="u_coarse")
        if u_fine is not None:
            u_fine = as_cuda(u_fine, shape=(R, Sf), name="u_fine")
        out = {k: empty(R, 3) if k.startswith("rgb") else empty(R)
               for k in (["rgb", "depth", "acc"] + (["rgb_coarse", "depth_coarse", "acc_coarse"]
                                                     if return_coarse else []))}
        if proposal is not None and return_coarse:
            raise ValueError("the proposal paths have no coarse maps")
        if int(streams) < 1:
            raise ValueError(f"streams must be at least 1, not {streams}")
        lib = _lib.lib()
        ws_bytes = (lib.nerfgb_render_gated_workspace_bytes if gated else lib.nerfgb_render_workspace_bytes)(
            min(chunk, R), Sc, Sf)
        pc, pf = self.coarse_model.packed(precision), self.fine_model.packed(precision)
        n_st = min(int(streams), max(1, (R + chunk - 1) // chunk))
        main = torch.cuda.current_stream()
        sts = [main] + self._side_streams(n_st - 1)
        wss = [torch.empty(ws_bytes, dtype=torch.uint8, device=rays_o.device) for _ in range(n_st)]
        if n_st > 1:
            # side streams: start after everything the caller's stream has
            # queued (inputs, outputs, packed weights); the caching allocator
            # learns which streams use each buffer
            fork = torch.cuda.Event()
            fork.record(main)
            used = [rays_o, rays_d, near, far, u_coarse, u_fine, pc, pf, *out.values()]
            if proposal is not None:
                used.append(proposal.params)
            for k, st in enumerate(sts[1:], 1):
                st.wait_event(fork)
                wss[k].record_stream(st)
                for t in used:
                    if t is not None:
                        t.record_stream(st)
        for k, s in enumerate(range(0, R, chunk)):
            e = min(R, s + chunk)
            sl = slice(s, e)
            ws = wss[k % n_st]
            with torch.cuda.stream(sts[k % n_st]):
                self._render_chunk(lib, gated, proposal, pc, pf, prec, rays_o, rays_d, near, far, u_coarse,
                                   u_fine, seed, s, sl, e, Sc, Sf, gate_tau, gate_fine_draws, return_coarse, out,
                                   ws)
        for st in sts[1:]:
            join = torch.cuda.Event()
            join.record(st)
            main.wait_event(join)
        return out

    def _render_chunk(self, lib, gated, proposal, pc, pf, prec, rays_o, rays_d, near, far, u_coarse, u_fine,
                      seed, s, sl, e, Sc, Sf, gate_tau, gate_fine_draws, return_coarse, out, ws):
        """One chunk's library call, on the current stream."""
        if gated:
            _lib.call("nerfgb_render_rays_gated", ptr(proposal.params), ptr(pc), ptr(pf), prec,
                      ptr(rays_o[sl]), ptr(rays_d[sl]), ptr(near[sl]), ptr(far[sl]),
                      ptr(u_coarse[sl]) if u_coarse is not None else None,
                      ptr(u_fine[sl]) if u_fine is not None else None,
                      ctypes.c_ulonglong(int(seed) + s), e - s, Sc, Sf,
                      int(bool(self.params.sampling.perturb)),
                      int(bool(self.params.sampling.lin_inv_depth)), int(self.white_bg),
                      int(self.trans_mode), ctypes.c_float(gate_tau),
                      _lib.GATE_FINE_DRAWS if gate_fine_draws else 0, ptr(out["rgb"][sl]),
                      ptr(out["depth"][sl]), ptr(out["acc"][sl]), ptr(ws),
                      ptr(self.coarse_model.err_word), stream())
            return
        if proposal is not None:
            _lib.call("nerfgb_render_rays_proposal", ptr(proposal.params), ptr(pf), prec,
                      ptr(rays_o[sl]), ptr(rays_d[sl]), ptr(near[sl]), ptr(far[sl]),
                      ptr(u_coarse[sl]) if u_coarse is not None else None,
                      ptr(u_fine[sl]) if u_fine is not None else None,
                      ctypes.c_ulonglong(int(seed) + s), e - s, Sc, Sf,
                      int(bool(self.params.sampling.perturb)),
                      int(bool(self.params.sampling.lin_inv_depth)), int(self.white_bg),
                      int(self.trans_mode), ptr(out["rgb"][sl]), ptr(out["depth"][sl]),
                      ptr(out["acc"][sl]), ptr(ws), ptr(self.fine_model.err_word), stream())
            return
        _lib.call("nerfgb_render_rays", ptr(pc), ptr(pf), prec, ptr(rays_o[sl]), ptr(rays_d[sl]),
                  ptr(near[sl]), ptr(far[sl]),
                  ptr(u_coarse[sl]) if u_coarse is not None else None,
                  ptr(u_fine[sl]) if u_fine is not None else None,
                  ctypes.c_ulonglong(int(seed) + s), e - s, Sc, Sf,
                  int(bool(self.params.sampling.perturb)),
                  int(bool(self.params.sampling.lin_inv_depth)), int(self.white_bg),
                  int(self.trans_mode),
                  ptr(out["rgb_coarse"][sl]) if return_coarse else None,
                  ptr(out["depth_coarse"][sl]) if return_coarse else None,
                  ptr(out["acc_coarse"][sl]) if return_coarse else None,
                  ptr(out["rgb"][sl]), ptr(out["depth"][sl]), ptr(out["acc"][sl]), ptr(ws),
                  ptr(self.coarse_model.err_word), stream())

    def load_model(self, load_dir, load_tag, skip_optimizer=False):
        """NeRF.set_everything (nerf/core/model.py:238-287): unless
        `skip_optimizer` (the reference's params.model.load.skip_optimizer),
        the Adam state from <load_dir>/<load_tag>_optimizer.npz
        (weights.optimizer_state_from_npz: step count and the m/v slots of
        both networks), then the coarse and fine networks' weights from
        <load_tag>_coarse.h5 and <load_tag>_fine.h5 (the files the
        reference's checkpoint callback writes, ops.py:131-149). The next
        train_step continues from the loaded step, as Keras's Adam does."""
        import os
        if not skip_optimizer:
            st = optimizer_state_from_npz(os.path.join(load_dir, f"{load_tag}_optimizer.npz"))
            self.load_optimizer_state(st)
        self.coarse_model.load_weights(os.path.join(load_dir, f"{load_tag}_coarse.h5"))
        self.fine_model.load_weights(os.path.join(load_dir, f"{load_tag}_fine.h5"))

    def load_optimizer_state(self, state):
        """Sets the Adam step and the m/v slots of both networks from
        weights.optimizer_state_from_npz's result."""
        opt = self._train_state()
        opt["step"] = int(state["step"])
        for k, name in enumerate(("coarse", "fine")):
            for slot in ("m", "v"):
                opt[slot][k].copy_(torch.from_numpy(state[slot][name]))

    def render_frame(self, H, W, intrinsic, c2w, bounds=(2.0, 6.0), **render_kw):
        """One image of the render loop (nerf/main/render.py:79-97): the
        frame's rays from the pinhole camera on the device
        (ray_utils.get_rays_tf), near/far = `bounds`, NeRF.render in chunks
        (keyword arguments pass through), and the maps as images: "rgb"
        [H,W,3], "depth" and "acc" [H,W], and "image_u8" [H,W,3] =
        clip(rgb * 255, 0, 255) truncated to uint8 (render.py:96-97)."""
        rays_o, rays_d = ray_utils.get_rays_tf(H, W, intrinsic, c2w)
        n = rays_o.shape[0]
        near = torch.full((n, 1), float(bounds[0]), device=rays_o.device)
        far = torch.full((n, 1), float(bounds[1]), device=rays_o.device)
        out = self.render(rays_o, rays_d, near, far, **render_kw)
        frame = {"rgb": out["rgb"].reshape(H, W, 3), "depth": out["depth"].reshape(H, W),
                 "acc": out["acc"].reshape(H, W)}
        frame["image_u8"] = (frame["rgb"] * 255.0).clamp(0.0, 255.0).to(torch.uint8)
        return frame


def psnr(y_true, y_pred):
    """nerf/core/ops.py:249-257: per-element PSNR in dB (float64)."""
    a = torch.as_tensor(y_true).double()
    b = torch.as_tensor(y_pred).to(a.device).double()
    mse = torch.mean((a - b) ** 2)
    return float(-10.0 * torch.log10(mse))
