"""GB300 (sm_103a) render path of nerf-tf2 behind the reference's API.

    import importlib
    ng = importlib.import_module("nerf-tf2_gb300")
    params = ng.make_params()
    nerf = ng.NeRF(params, precision="bf16")
    post_proc_CM, post_proc_FM = nerf.forward(rays_o, rays_d, near, far)

Submodules mirror the reference's modules: ``ray_utils`` (nerf/utils/
ray_utils.py), ``model`` (nerf/core/model.py) and ``render_loop`` (the
files of nerf/main/render.py's loop). The kernels live in
libnerfgb.so (C ABI: include/nerfgb.h), built by ``build.py``.
"""
from . import autograd, h5, proposal, ray_utils, render_loop, synthetic, weights  # noqa: F401
from ._lib import NerfgbError, lib  # noqa: F401
from .config import make_params  # noqa: F401
from .model import (NeRF, NerfMLP, PositionalEncoder,  # noqa: F401
                    get_coarse_or_fine_model, psnr)
from .proposal import ProposalNetwork, ProposalTrainer  # noqa: F401
from .ray_utils import (compute_weights, create_input_batch_coarse_model,  # noqa: F401
                        create_input_batch_fine_model, post_process_model_output,
                        set_seed, sigma_to_alpha)
