"""Parity of the MLP kernels with the CPU oracle (nerf/core/model.py:334-394).

FP32 SIMT against the fp32 and fp64 oracle; BF16 tcgen05 against the fp64
oracle with a BF16-sized tolerance.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
F32, F64 = np.float32, np.float64


def dev(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def host(x):
    return x.detach().cpu().numpy()


def samples(n, seed, rows_per_dir=1):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-4.0, 4.0, (n, 3)).astype(F32)
    nd = (n + rows_per_dir - 1) // rows_per_dir
    d = rng.normal(size=(nd, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(F32)
    return x, d


def biased_blob(ng, seed):
    """Glorot kernels plus non-zero biases, so that every bias path is used."""
    blob = ng.weights.glorot_blob(seed)
    rng = np.random.default_rng(seed + 99)
    for name, (ko, bo, i, o) in ng.weights.offsets().items():
        blob[bo:bo + o] = rng.uniform(-0.1, 0.1, o)
    return blob


@pytest.mark.parametrize("n", [1000, 64, 1, 4097])
def test_mlp_fp32_vs_oracle(ng, oracle, cuda, n):
    blob = biased_blob(ng, 5)
    x, d = samples(n, n)
    mlp = ng.get_coarse_or_fine_model("coarse", params=blob, precision="fp32")
    rgb, sigma = mlp((dev(x), dev(d)))
    assert rgb.shape == (n, 3) and sigma.shape == (n, 1)
    p32 = oracle.unpack_params(blob, F32)
    r32, s32 = oracle.mlp_forward(p32, x, d, F32)
    r64, s64 = oracle.mlp_forward(oracle.unpack_params(blob, F64), x, d, F64)
    # tolerance: fp32 dot products of length <= 320 in another order, 10 layers
    np.testing.assert_allclose(host(rgb), r32, atol=2e-5, rtol=0)
    np.testing.assert_allclose(host(sigma), s32, atol=1e-4, rtol=1e-4)
    np.testing.assert_allclose(host(rgb), r64, atol=1e-3, rtol=0)
    np.testing.assert_allclose(host(sigma), s64, atol=2e-3, rtol=2e-3)


def test_mlp_rows_per_dir(ng, cuda):
    blob = biased_blob(ng, 6)
    S = 192
    x, d = samples(8 * S, 1, rows_per_dir=S)
    mlp = ng.get_coarse_or_fine_model("fine", params=blob)
    a_rgb, a_sig = mlp((dev(x), dev(d)), rows_per_dir=S)
    b_rgb, b_sig = mlp((dev(x), dev(np.repeat(d, S, axis=0))))
    assert torch.equal(a_rgb, b_rgb) and torch.equal(a_sig, b_sig)


def test_mlp_empty(ng, cuda):
    mlp = ng.get_coarse_or_fine_model("coarse")
    rgb, sigma = mlp((torch.zeros(0, 3, device=cuda), torch.zeros(0, 3, device=cuda)))
    assert rgb.shape == (0, 3) and sigma.shape == (0, 1)


@pytest.mark.parametrize("n", [4096, 300, 1])
def test_mlp_bf16_vs_fp64(ng, oracle, cuda, n):
    blob = biased_blob(ng, 8)
    x, d = samples(n, 11 + n)
    mlp = ng.get_coarse_or_fine_model("coarse", params=blob, precision="bf16")
    rgb, sigma = mlp((dev(x), dev(d)))
    mlp.check_device_errors()
    r64, s64 = oracle.mlp_forward(oracle.unpack_params(blob, F64), x, d, F64)
    # BF16 operands (8-bit mantissa), FP32 accumulation over 10 layers
    err_rgb = np.abs(host(rgb) - r64).max()
    err_sig = np.abs(host(sigma) - s64).max() / max(1.0, np.abs(s64).max())
    assert err_rgb < 2e-2, err_rgb
    assert err_sig < 5e-2, err_sig
    assert np.abs(host(rgb) - r64).mean() < 3e-3


def test_mlp_bf16_many_tiles(ng, oracle, cuda):
    """200,003 rows: several 512-row tiles per CTA pair of the persistent
    kernel (and a ragged last tile). Every row is computed the same way
    wherever it lands (tile, pair CTA, sub-tile): a row permutation permutes
    the outputs bit for bit; sampled rows match the fp64 oracle."""
    n = 200003
    blob = biased_blob(ng, 21)
    x, d = samples(n, 23)
    mlp = ng.get_coarse_or_fine_model("fine", params=blob, precision="bf16")
    rgb, sigma = mlp((dev(x), dev(d)))
    perm = np.random.default_rng(5).permutation(n)
    rgb_p, sigma_p = mlp((dev(x[perm]), dev(d[perm])))
    mlp.check_device_errors()
    pt = torch.from_numpy(perm).cuda()
    assert torch.equal(rgb_p, rgb[pt]) and torch.equal(sigma_p, sigma[pt])
    rows = np.concatenate([np.random.default_rng(6).choice(n, 250, replace=False), [0, n - 1]])
    r64, s64 = oracle.mlp_forward(oracle.unpack_params(blob, F64), x[rows], d[rows], F64)
    assert np.abs(host(rgb)[rows] - r64).max() < 2e-2
    assert np.abs(host(sigma)[rows] - s64).max() / max(1.0, np.abs(s64).max()) < 5e-2


@pytest.mark.parametrize("n", [4097, 300])
def test_mlp_fp8_vs_fp64(ng, oracle, cuda, n):
    """FP8-e4m3 operands (3 mantissa bits) with per-output-channel weight
    scales, FP32 accumulation; bounds sized for e4m3 rounding over 10 layers."""
    blob = biased_blob(ng, 8)
    x, d = samples(n, 31 + n)
    mlp = ng.get_coarse_or_fine_model("coarse", params=blob, precision="fp8")
    rgb, sigma = mlp((dev(x), dev(d)))
    mlp.check_device_errors()
    r64, s64 = oracle.mlp_forward(oracle.unpack_params(blob, F64), x, d, F64)
    err_rgb = np.abs(host(rgb) - r64)
    assert err_rgb.max() < 6e-2, err_rgb.max()
    assert err_rgb.mean() < 1e-2, err_rgb.mean()
    assert np.abs(host(sigma) - s64).max() / max(1.0, np.abs(s64).max()) < 0.15
    # and clearly coarser than BF16 on the same inputs (the FP8 path is taken)
    r16, _ = ng.get_coarse_or_fine_model("coarse", params=blob, precision="bf16")((dev(x), dev(d)))
    assert np.abs(host(r16) - r64).mean() < err_rgb.mean()


def _err_stats(got, want, scale=1.0):
    e = np.abs(np.asarray(got, F64) - np.asarray(want, F64)).reshape(len(got), -1).max(axis=1) / scale
    return float(e.max()), float(np.quantile(e, 0.99)), float(e.mean())


@pytest.mark.parametrize("precision,n", [("bf16", 4096), ("bf16", 301), ("fp8", 4097), ("fp8", 300)])
def test_mlp_lowp_vs_emulation(ng, oracle, cuda, precision, n):
    """The tensor-core kernels against the oracle's emulation of their
    specified arithmetic (oracle.mlp_forward_lowp: operands rounded to BF16 or
    to E4M3 with per-channel weight scales, exact products, FP32 sums, FP32
    bias and heads). What remains is the tensor core's FP32 summation order,
    and an activation that lands within that difference of a rounding
    boundary rounding the other way (a BF16 step is 2^-8 relative, an E4M3
    step 2^-3), so the bounds are far below the formats' own error against
    FP64 (test_mlp_bf16_vs_fp64, test_mlp_fp8_vs_fp64)."""
    blob = biased_blob(ng, 8)
    x, d = samples(n, 11 + n)
    mlp = ng.get_coarse_or_fine_model("coarse", params=blob, precision=precision)
    rgb, sigma = mlp((dev(x), dev(d)))
    mlp.check_device_errors()
    er, es = oracle.mlp_forward_lowp(oracle.unpack_params(blob, F32), x, d, precision)
    r_max, r_99, r_mean = _err_stats(host(rgb), er)
    s_max, s_99, s_mean = _err_stats(host(sigma), es, max(1.0, float(np.abs(es).max())))
    print(f"{precision} n={n}: rgb max {r_max:.2e} p99 {r_99:.2e} mean {r_mean:.2e}; "
          f"sigma max {s_max:.2e} p99 {s_99:.2e} mean {s_mean:.2e}")
    tol = {"bf16": dict(mx=2e-3, p99=2e-4, mean=2e-5), "fp8": dict(mx=3e-2, p99=3e-3, mean=3e-4)}[precision]
    for mx, p99, mean in ((r_max, r_99, r_mean), (s_max, s_99, s_mean)):
        assert mx < tol["mx"] and p99 < tol["p99"] and mean < tol["mean"], (mx, p99, mean)
