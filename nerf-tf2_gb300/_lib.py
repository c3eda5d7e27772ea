"""ctypes binding of libnerfgb.so (declared in include/nerfgb.h).

The library is built in-tree (``build.py``). Nothing here falls back to a
CPU or PyTorch implementation: if the library is missing, loading raises.
"""
import ctypes
import os
import pathlib

HERE = pathlib.Path(__file__).resolve().parent
# NERFGB_LIBRARY names another build of the same library (the bounds-check
# build, libnerfgb_bounds.so) to load instead.
LIB_PATH = pathlib.Path(os.environ.get("NERFGB_LIBRARY", str(HERE / "libnerfgb.so")))

P = ctypes.c_void_p
I = ctypes.c_int
LL = ctypes.c_longlong
ULL = ctypes.c_ulonglong
F = ctypes.c_float

# Status codes and enums (include/nerfgb.h).
OK = 0
E_INVALID_ARG = -1
E_UNSUPPORTED = -2
E_CUDA = -3
E_TIMEOUT = -4
E_DEVICE = -5
E_SCRATCH_LIMIT = -6
PREC_FP32 = 0
PREC_BF16 = 1
PREC_FP8 = 2
GATE_FINE_DRAWS = 1
TRANS_CUMPROD = 0
TRANS_LOGSUM = 1

# name -> (restype, argtypes)
SIGNATURES = {
    "nerfgb_abi_version": (I, []),
    "nerfgb_status_string": (ctypes.c_char_p, [I]),
    "nerfgb_mlp_param_count": (LL, []),
    "nerfgb_mlp_packed_bytes": (LL, [I]),
    "nerfgb_mlp_pack": (I, [P, I, P, P]),
    "nerfgb_coarse_sample": (I, [P, P, P, P, P, I, I, I, I, P, P, P, P, P, P]),
    "nerfgb_fine_sample": (I, [P, P, P, P, I, P, P, P, I, I, I, P, P, P, P, P, P]),
    "nerfgb_composite": (I, [P, P, P, I, I, I, I, P, P, P, P, P]),
    "nerfgb_sigma_to_alpha": (I, [P, P, LL, P, P]),
    "nerfgb_positional_encode": (I, [P, LL, I, P, P]),
    "nerfgb_mlp_forward": (I, [P, I, P, P, LL, I, P, P, P, P]),
    "nerfgb_mlp_forward_mapped": (I, [P, I, P, P, LL, I, P, P, P, P, P, P]),
    "nerfgb_bounds_check_status": (I, [I]),
    "nerfgb_mlp_forward_wait_test": (I, [P, I, P, P, LL, I, P, P, P, ctypes.c_ulonglong, LL, P]),
    "nerfgb_uniform": (I, [ULL, ULL, LL, P, P]),
    "nerfgb_get_rays": (I, [I, I, P, P, P, P, P]),
    "nerfgb_sample_rays": (I, [P, I, I, P, P, F, F, P, I, P, P, P, P, P, P]),
    "nerfgb_uniform_int": (I, [ULL, ULL, LL, I, P, P]),
    "nerfgb_depth_map": (I, [P, LL, F, I, P, P, P, P, P]),
    "nerfgb_render_workspace_bytes": (LL, [I, I, I]),
    "nerfgb_render_rays": (I, [P, P, I, P, P, P, P, P, P, ULL, I, I, I, I, I, I, I,
                               P, P, P, P, P, P, P, P, P]),
    "nerfgb_proposal_param_count": (LL, []),
    "nerfgb_proposal_forward": (I, [P, P, LL, P, P]),
    "nerfgb_proposal_forward_bf16": (I, [P, P, LL, P, P]),
    "nerfgb_proposal_backward": (I, [P, P, P, LL, P, P]),
    "nerfgb_proposal_weights": (I, [P, P, I, I, I, P, P]),
    "nerfgb_proposal_weights_backward": (I, [P, P, P, I, I, P, P]),
    "nerfgb_render_rays_proposal": (I, [P, P, I, P, P, P, P, P, P, ULL, I, I, I, I, I, I, I,
                                        P, P, P, P, P, P]),
    "nerfgb_gate_coarse": (I, [P, I, I, F, P, P, P, P]),
    "nerfgb_gate_fine": (I, [P, P, P, I, I, I, P, P, P]),
    "nerfgb_render_gated_workspace_bytes": (LL, [I, I, I]),
    "nerfgb_render_rays_gated": (I, [P, P, P, I, P, P, P, P, P, P, ULL, I, I, I, I, I, I, I, F, I,
                                     P, P, P, P, P, P]),
    "nerfgb_composite_backward": (I, [P, P, P, P, P, I, I, I, P, P, P]),
    "nerfgb_mse_loss": (I, [P, P, LL, F, P, P, P]),
    "nerfgb_envelope_loss": (I, [P, P, I, I, F, P, P, P]),
    "nerfgb_adam_step": (I, [P, P, P, P, LL, F, F, F, F, LL, P]),
    "nerfgb_mlp_acts_floats_per_row": (LL, []),
    "nerfgb_mlp_forward_train": (I, [P, P, P, LL, I, P, P, P, P]),
    "nerfgb_mlp_backward_workspace_bytes": (LL, [LL]),
    "nerfgb_mlp_backward": (I, [P, P, LL, P, P, P, P, P]),
    "nerfgb_mlp_forward_train_bf16": (I, [P, P, P, LL, I, P, P, P, P, P]),
    "nerfgb_mlp_backward_bf16_workspace_bytes": (LL, [LL]),
    "nerfgb_mlp_backward_bf16": (I, [P, P, LL, P, P, P, P, P, P]),
    "nerfgb_render_rays_noalloc": (I, [P, P, I, P, P, P, P, P, P, ULL, I, I, I, I, I, I, I,
                                       P, P, P, P, P, P, P, P]),
}


class NerfgbError(RuntimeError):
    """A libnerfgb entry point returned a non-zero status."""

    def __init__(self, fn, status, name):
        super().__init__(f"{fn} failed: {name} ({status})")
        self.status = status
        self.code = name


_lib = None


def lib():
    """Loads libnerfgb.so once. Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; "
                "g.build()\"` (requires nvcc). There is no CPU fallback.")
        handle = ctypes.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _lib = handle
    return _lib


def status_name(status):
    return lib().nerfgb_status_string(int(status)).decode()


def call(name, *args):
    """Calls entry point `name`; raises NerfgbError on a non-zero status."""
    rc = getattr(lib(), name)(*args)
    if rc != OK:
        raise NerfgbError(name, rc, status_name(rc))
    return rc
