"""The slice of the reference's YAML config that the render path reads.

The reference loads nerf/params/config.yaml into a python-box object and the
path reads ``params.sampling.{N_coarse, N_fine, perturb, lin_inv_depth}``
(config.yaml:364-381) and ``params.system.white_bg`` (config.yaml:15). Any
object with those attributes works here (duck typing, as in the reference);
``make_params`` builds one with the reference's defaults.
"""
from types import SimpleNamespace


def make_params(N_coarse=64, N_fine=128, perturb=True, lin_inv_depth=True,
                white_bg=False):
    return SimpleNamespace(
        sampling=SimpleNamespace(N_coarse=N_coarse, N_fine=N_fine,
                                 perturb=perturb, lin_inv_depth=lin_inv_depth),
        system=SimpleNamespace(white_bg=white_bg),
    )
