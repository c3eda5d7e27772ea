"""Tensor plumbing for the ctypes calls: device placement, dtype and layout
checks, raw pointers and the current CUDA stream."""
import numpy as np
import torch


def device():
    if not torch.cuda.is_available():
        raise RuntimeError("libnerfgb needs a CUDA device (sm_103); none is visible")
    return torch.device("cuda", torch.cuda.current_device())


def as_cuda(x, dtype=torch.float32, shape=None, name="tensor"):
    """Returns x as a contiguous CUDA tensor of `dtype` (copying only when x is
    on the host, has another dtype or is strided)."""
    if isinstance(x, np.ndarray):
        x = torch.from_numpy(np.ascontiguousarray(x))
    if not isinstance(x, torch.Tensor):
        x = torch.as_tensor(x)
    if x.device.type != "cuda":
        x = x.to(device())
    if x.dtype != dtype:
        x = x.to(dtype)
    if not x.is_contiguous():
        x = x.contiguous()
    if shape is not None:
        want = tuple(shape)
        if tuple(x.shape) != want:
            if x.numel() == int(np.prod(want)):
                x = x.reshape(want)
            else:
                raise ValueError(f"{name}: expected shape {want}, got {tuple(x.shape)}")
    return x


def ptr(x):
    return None if x is None else x.data_ptr()


def stream():
    return torch.cuda.current_stream().cuda_stream


def empty(*shape, dtype=torch.float32):
    return torch.empty(*shape, dtype=dtype, device=device())
