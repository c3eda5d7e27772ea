"""The tensor-core MLP kernels' failure path: every mbarrier wait is bounded,
and on expiry the kernel reports NERFGB_E_TIMEOUT in the caller's err_word,
drains its copies and MMAs, frees its tensor memory and returns, leaving the
context usable. A diagnostic entry point (nerfgb_mlp_forward_wait_test)
shortens the limit to a few milliseconds and leaves one weight chunk
unloaded, so that a wait runs out; the reference has no counterpart (it
surfaces TensorFlow's errors)."""
import ctypes
import time

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _run(ng, mlp, X, D, wait_ns, withhold):
    lib = ng._lib.lib()
    n = X.shape[0]
    rgb = torch.full((n, 3), -1.0, device="cuda")
    sig = torch.full((n,), -1.0, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    t0 = time.perf_counter()
    rc = lib.nerfgb_mlp_forward_wait_test(mlp.packed().data_ptr(), ng.model.PRECISIONS[mlp.precision],
                                          X.data_ptr(), D.data_ptr(), n, 1, rgb.data_ptr(), sig.data_ptr(),
                                          err.data_ptr(), ctypes.c_ulonglong(wait_ns), withhold,
                                          torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return rc, int(err.item()), rgb, sig, time.perf_counter() - t0


@pytest.mark.parametrize("precision", ["bf16", "fp8"])
def test_wait_runs_out_and_the_next_launch_is_clean(ng, cuda, precision):
    n = 100_000  # several tiles per CTA (pair): a withheld chunk stalls every CTA
    rng = np.random.default_rng(3)
    X = torch.from_numpy(rng.uniform(-3, 3, (n, 3)).astype(np.float32)).cuda()
    d = rng.normal(size=(n, 3))
    D = torch.from_numpy((d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)).cuda()
    mlp = ng.get_coarse_or_fine_model("fine", seed=4, precision=precision)
    rgb0, sig0 = mlp((X, D))
    mlp.check_device_errors()
    # the short limit alone: no wait comes near it, the outputs are the kernel's
    rc, code, rgb, sig, _ = _run(ng, mlp, X, D, 5_000_000, -1)
    assert rc == ng._lib.OK and code == 0
    assert torch.equal(rgb, rgb0) and torch.equal(sig.reshape(-1), sig0.reshape(-1))
    # one chunk withheld: the issuer's wait runs out, the kernel reports it and returns
    rc, code, _, _, secs = _run(ng, mlp, X, D, 2_000_000, 5)
    assert rc == ng._lib.OK
    assert code == ng._lib.E_TIMEOUT, ng._lib.status_name(code)
    assert secs < 5.0
    # the context stays usable: the next launches are bit-identical to the clean run
    for _ in range(2):
        rgb1, sig1 = mlp((X, D))
        mlp.check_device_errors()
        assert torch.equal(rgb1, rgb0) and torch.equal(sig1, sig0)


def test_wait_test_rejects_bad_arguments(ng, cuda):
    mlp = ng.get_coarse_or_fine_model("fine", seed=4, precision="bf16")
    X = torch.zeros(4, 3, device="cuda")
    rc, *_ = _run(ng, mlp, X, X, 10, -1)  # limit below 1 us
    assert rc == ng._lib.E_INVALID_ARG
