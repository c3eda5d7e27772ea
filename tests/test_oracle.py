"""Known-answer tests that pin the CPU oracle (no GPU).

The reference ships no tests or golden vectors, so the oracle is pinned by
closed-form cases of the reference's own formulas (nerf/utils/ray_utils.py,
nerf/core/model.py) and by published Philox vectors.
"""
import numpy as np
import pytest

F32, F64 = np.float32, np.float64


def params(ng, **kw):
    return ng.make_params(**kw)


# --- Philox4x32-10: Random123 known-answer vectors -------------------------
@pytest.mark.parametrize("ctr,key,want", [
    ((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
    ((0xffffffff,) * 4, (0xffffffff,) * 2, (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
    ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
     (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)),
])
def test_philox_kat(oracle, ctr, key, want):
    words = oracle.philox4x32_10(*[np.array([c], np.uint32) for c in ctr], *key)
    assert tuple(int(w[0]) for w in words) == want


def test_philox_uniform_range(oracle):
    u = oracle.philox_uniform(123, 0, 100000)
    assert u.dtype == F32 and u.min() >= 0 and u.max() < 1
    assert abs(u.mean() - 0.5) < 0.01


# --- linspace / bins (ray_utils.py:183-247) --------------------------------
def test_linspace_endpoints_exact(oracle):
    near = np.array([[2.0], [0.1]], F32)
    far = np.array([[6.0], [1e3]], F32)
    e = oracle.tf_linspace(near, far, 65)
    assert e.shape == (2, 65)
    assert np.array_equal(e[:, 0], near[:, 0]) and np.array_equal(e[:, -1], far[:, 0])
    assert np.all(np.diff(e, axis=1) > 0)
    np.testing.assert_allclose(e[0], np.linspace(2, 6, 65), rtol=1e-6)


def test_inverse_depth_edges(oracle):
    e = oracle.bin_edges(np.array([[2.0]]), np.array([[6.0]]), 64, True, F64)
    np.testing.assert_allclose(1 / e[0], np.linspace(0.5, 1 / 6, 65), rtol=1e-14)


def test_coarse_mid_points_and_widths(oracle, ng):
    p = params(ng, perturb=False, lin_inv_depth=False)
    o = np.zeros((1, 3), F32)
    d = np.array([[0, 0, 1]], F32)
    out = oracle.create_input_batch_coarse_model(p, o, d, [[2.0]], [[6.0]], None, F64)
    np.testing.assert_allclose(out["t_vals"][0], 2 + (np.arange(64) + 0.5) / 16, rtol=1e-14)
    np.testing.assert_allclose(out["bin_data"]["bin_widths"], 1 / 16, rtol=1e-14)
    np.testing.assert_allclose(out["xyz_inputs"][:, 2], out["t_vals"][0])


def test_coarse_u_bounds(oracle, ng):
    p = params(ng, lin_inv_depth=True)
    o, d, n, f = ng.synthetic.sphere_rays(16, 0)
    u0 = np.zeros((16, 64), F32)
    out = oracle.create_input_batch_coarse_model(p, o, d, n, f, u0)
    assert np.array_equal(out["t_vals"], out["bin_data"]["left_edges"])


# --- compositing (ray_utils.py:408-551) -------------------------------------
def _t(R, S, dtype=F64):
    return np.tile(np.linspace(2, 6, S, dtype=dtype), (R, 1))


def test_composite_zero_density(oracle):
    t = _t(3, 64)
    out = oracle.post_process_model_output(np.full((192, 3), 0.7), np.zeros((192, 1)), t, True)
    assert np.all(out["weights"] == 0) and np.all(out["acc_map"] == 0)
    np.testing.assert_allclose(out["pred_rgb"], 1.0)  # white background (:542-544)


def test_composite_opaque_sample(oracle):
    t = _t(1, 64)
    sigma = np.zeros((64, 1))
    sigma[10] = 1e12
    out = oracle.post_process_model_output(np.ones((64, 3)) * 0.25, sigma, t)
    w = out["weights"][0]
    # ten transparent samples each contribute a factor (1 - 0) + 1e-10 (:480)
    assert w[10] == pytest.approx((1 + 1e-10) ** 10, abs=1e-15)
    assert np.all(w[:10] == 0) and np.all(np.abs(w[11:]) < 1e-9)
    np.testing.assert_allclose(out["pred_depth"][0], t[0, 10])


def test_composite_constant_density_closed_form(oracle):
    S = 64
    t = _t(1, S)
    dt = t[0, 1] - t[0, 0]
    sig = 0.3
    out = oracle.post_process_model_output(np.zeros((S, 3)), np.full((S, 1), sig), t)
    a = 1 - np.exp(-sig * dt)
    i = np.arange(S - 1)
    want = a * (1 - a + 1e-10) ** i
    np.testing.assert_allclose(out["weights"][0, :-1], want, rtol=1e-12)
    # last delta is 1e10 (:465-468) so alpha_last = 1
    T_last = (1 - a + 1e-10) ** (S - 1)
    np.testing.assert_allclose(out["weights"][0, -1], T_last, rtol=1e-12)


def test_composite_fp32_vs_fp64(oracle):
    rng = np.random.default_rng(0)
    R, S = 64, 192
    t = np.sort(rng.uniform(2, 6, (R, S)), axis=1)
    sig = rng.exponential(2.0, (R * S, 1))
    rgb = rng.uniform(0, 1, (R * S, 3))
    a = oracle.post_process_model_output(rgb.astype(F32), sig.astype(F32), t.astype(F32))
    b = oracle.post_process_model_output(rgb, sig, t)
    for k in ("weights", "pred_rgb", "pred_depth", "acc_map"):
        np.testing.assert_allclose(a[k], b[k], atol=2e-5)


# --- positional encoder (model.py:289-332) ----------------------------------
def test_encoder_zero_and_layout(oracle):
    e = oracle.positional_encoding(np.zeros((2, 3), F32), 10)
    assert e.shape == (2, 63)
    assert np.all(e[:, :3] == 0)
    assert np.all(e[:, 3::2] == 0) and np.all(e[:, 4::2] == 1)


def test_encoder_index_convention(oracle):
    x = np.array([[0.1, 0.2, 0.3]], F64)
    e = oracle.positional_encoding(x, 4, F64)
    for c in range(3):
        for l in range(4):
            arg = x[0, c] * (2.0 ** l) * np.pi
            assert e[0, 3 + c * 8 + 2 * l] == pytest.approx(np.sin(arg), abs=1e-15)
            assert e[0, 3 + c * 8 + 2 * l + 1] == pytest.approx(np.cos(arg), abs=1e-15)


def test_encoder_multipliers_fp32(oracle):
    m = oracle.encoder_multipliers(10, F32)
    assert m.dtype == F32
    assert np.array_equal(m, (2.0 ** np.arange(10)).astype(F32) * F32(np.pi))


# --- fine sampler (ray_utils.py:276-406) -------------------------------------
def _coarse(oracle, ng, R, seed=0, lin_inv=False, dtype=F32):
    p = params(ng, lin_inv_depth=lin_inv)
    o, d, n, f = ng.synthetic.sphere_rays(R, seed)
    u = np.random.default_rng(seed + 1).random((R, 64), dtype=F32)
    return p, o, d, oracle.create_input_batch_coarse_model(p, o, d, n, f, u, dtype)


def test_upper_bound_matches_searchsorted(oracle):
    rng = np.random.default_rng(3)
    a = np.sort(rng.random((50, 63)).astype(F32), axis=1)
    a[:, 10] = a[:, 11]  # ties
    v = rng.random((50, 128)).astype(F32)
    v[:, 0] = a[:, 11]   # exactly on an edge
    v[:, 1] = 0.0
    got = oracle.upper_bound(a, v)
    want = np.stack([np.searchsorted(a[r], v[r], side="right") for r in range(50)])
    assert np.array_equal(got, want)


def test_fine_uniform_weights_linear_bins(oracle, ng):
    p, o, d, cm = _coarse(oracle, ng, 4, lin_inv=False, dtype=F64)
    w = np.full((4, 64), 0.5)
    u = np.random.default_rng(9).random((4, 128))
    out = oracle.create_input_batch_fine_model(p, o, d, w, cm["bin_data"], cm["t_vals"], u, F64,
                                               return_indices=True)
    np.testing.assert_allclose(out["t_vals_fine"], 2 + 4 * u, rtol=1e-12)


def test_fine_one_hot_weight(oracle, ng):
    p, o, d, cm = _coarse(oracle, ng, 2)
    w = np.zeros((2, 64), F32)
    w[:, 17] = 1.0
    u = np.random.default_rng(2).random((2, 128)).astype(F32) * F32(0.9) + F32(0.05)
    out = oracle.create_input_batch_fine_model(p, o, d, w, cm["bin_data"], cm["t_vals"], u,
                                               return_indices=True)
    assert np.all(out["piece_idxs"] == 17)
    left = cm["bin_data"]["left_edges"][:, 17:18]
    right = cm["bin_data"]["right_edges"][:, 17:18]
    assert np.all(out["t_vals_fine"] >= left) and np.all(out["t_vals_fine"] <= right * (1 + 1e-6))


def test_fine_edge_rules(oracle, ng):
    p, o, d, cm = _coarse(oracle, ng, 1)
    w = np.random.default_rng(5).random((1, 64)).astype(F32)
    wp = w + F32(1e-5)
    denom = oracle.seq_sum(wp * cm["bin_data"]["bin_widths"])[:, None]
    pdf = wp / denom
    agg = oracle.seq_cumsum(pdf * cm["bin_data"]["bin_widths"])
    u = np.zeros((1, 128), F32)
    u[0, 0] = 0.0                                   # -> 0
    u[0, 1] = agg[0, 9]                             # exactly on inner edge 10 -> 'right' gives 10
    u[0, 2] = np.nextafter(agg[0, 9], F32(0))       # just below -> 9
    u[0, 3] = np.nextafter(F32(1), F32(0))          # u -> 1- -> 63
    out = oracle.create_input_batch_fine_model(p, o, d, w, cm["bin_data"], cm["t_vals"], u,
                                               return_indices=True)
    assert out["piece_idxs"][0, :4].tolist() == [0, 10, 9, 63]


def test_fine_pdf_mask(oracle, ng):
    """pdf < 1e-8 (ray_utils.py:372-373): offset zeroed, t = left edge."""
    p = params(ng, lin_inv_depth=False)
    o = np.zeros((1, 3), F32)
    d = np.array([[0, 0, 1]], F32)
    cm = oracle.create_input_batch_coarse_model(p, o, d, [[1.0]], [[1e12]],
                                                np.full((1, 64), 0.5, F32))
    w = np.zeros((1, 64), F32)
    u = np.full((1, 128), 0.5, F32)
    out = oracle.create_input_batch_fine_model(p, o, d, w, cm["bin_data"], cm["t_vals"], u,
                                               return_indices=True)
    idx = out["piece_idxs"][0, 0]
    assert np.all(out["t_vals_fine"][0] == cm["bin_data"]["left_edges"][0, idx])


def test_fine_sort_is_stable_argsort(oracle, ng):
    p, o, d, cm = _coarse(oracle, ng, 8)
    w = np.random.default_rng(1).random((8, 64)).astype(F32)
    u = np.random.default_rng(2).random((8, 128)).astype(F32)
    u[:, 5] = u[:, 6]  # duplicate fine samples
    out = oracle.create_input_batch_fine_model(p, o, d, w, cm["bin_data"], cm["t_vals"], u,
                                               return_indices=True)
    t_cat = np.concatenate([cm["t_vals"], out["t_vals_fine"]], 1)
    assert np.array_equal(out["t_vals"], np.sort(t_cat, axis=1))
    assert np.array_equal(np.take_along_axis(t_cat, out["sort_perm"], 1), out["t_vals"])
    assert np.all(np.diff(out["t_vals"], axis=1) >= 0)


def test_fine_fp32_vs_fp64(oracle, ng):
    p, o, d, cm32 = _coarse(oracle, ng, 32)
    _, _, _, cm64 = _coarse(oracle, ng, 32, dtype=F64)
    w = np.random.default_rng(4).random((32, 64))
    u = np.random.default_rng(6).random((32, 128)).astype(F32)
    a = oracle.create_input_batch_fine_model(p, o, d, w.astype(F32), cm32["bin_data"],
                                             cm32["t_vals"], u)
    b = oracle.create_input_batch_fine_model(p, o, d, w, cm64["bin_data"], cm64["t_vals"],
                                             u.astype(F64), F64)
    np.testing.assert_allclose(a["t_vals"], b["t_vals"], rtol=1e-5)


# --- MLP (model.py:334-394) ---------------------------------------------------
def test_param_count(oracle, ng):
    assert oracle.param_count() == 595844 == ng.weights.PARAM_COUNT


def test_glorot_matches_package(oracle, ng):
    blob = ng.weights.glorot_blob(7)
    p = oracle.glorot_params(7)
    assert np.array_equal(oracle.pack_params(p), blob)


def test_mlp_single_layer_fp64(oracle):
    """dense_0 of the network against an explicit fp64 matmul."""
    rng = np.random.default_rng(0)
    p = oracle.glorot_params(1, F64)
    x = rng.uniform(-2, 2, (8, 3))
    enc = oracle.positional_encoding(x, 10, F64)
    W, b = p["dense_0"]
    want = np.maximum(np.einsum("mk,kn->mn", enc, W) + b, 0)
    _, _, acts = oracle.mlp_forward(p, x, x, F64, cache=True)
    np.testing.assert_allclose(acts["h0"], want, rtol=1e-12, atol=1e-14)


def test_mlp_fp32_vs_fp64(oracle):
    rng = np.random.default_rng(0)
    p = oracle.glorot_params(2)
    x = rng.uniform(-2, 2, (256, 3)).astype(F32)
    d = rng.normal(size=(256, 3)).astype(F32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r32, s32 = oracle.mlp_forward(p, x, d, F32)
    r64, s64 = oracle.mlp_forward(p, x, d, F64)
    np.testing.assert_allclose(r32, r64, atol=1e-3)
    np.testing.assert_allclose(s32, s64, atol=1e-3, rtol=1e-3)


def test_get_rays_matches_package(oracle, ng):
    K = ng.synthetic.intrinsic(8, 10, 11.0)
    pose = ng.synthetic.random_pose(3)
    o1, d1 = oracle.get_rays(8, 10, K, pose)
    o2, d2 = ng.synthetic.get_rays(8, 10, K, pose)
    np.testing.assert_allclose(d1, d2, rtol=1e-15)
    np.testing.assert_allclose(o1, o2)


# --- proposal-gated render ---------------------------------------------------
def test_gate_fine_hand_case(oracle):
    # Sc = 2 coarse samples (perm 0, 1), fine draws perm 2, 3; coarse 1 gated off
    perm = np.array([[0, 2, 1, 3], [1, 0, 3, 2]])
    m_c = np.array([[True, False], [True, False]])
    want = np.array([[True, True, False, True], [False, True, True, True]])
    assert np.array_equal(oracle.gate_fine(perm, m_c), want)
    # with the draws' bins: ray 0's draw 0 (perm 2) lies in bin 1 (off), draw 1
    # (perm 3) in bin 0 (on); ray 1's draws both in bin 1 (off)
    piece = np.array([[1, 0], [1, 1]])
    want_d = np.array([[True, False, False, True], [False, True, False, False]])
    assert np.array_equal(oracle.gate_fine(perm, m_c, piece), want_d)
    assert not oracle.gate_coarse(np.array([np.nan, 0.5, 0.1]), 0.1).tolist()[0]
    assert oracle.gate_coarse(np.array([np.nan, 0.5, 0.1]), 0.1).tolist() == [False, True, False]


def test_gated_render_all_on_is_forward(oracle, ng):
    """tau < 0 keeps every sample: the gated chain is nerf_forward's fine pass."""
    p = params(ng)
    o, d, n, f = ng.synthetic.sphere_rays(6, 8)
    rng = np.random.default_rng(9)
    uc, uf = rng.random((6, 64)), rng.random((6, 128))
    pc, pf = oracle.glorot_params(1, F64), oracle.glorot_params(2, F64)
    blob = ng.proposal.glorot_blob(4)
    got, m_c, m_f, w_p = oracle.nerf_render_gated(p, blob, pc, pf, o, d, n, f, uc, uf, -1.0, F64)
    _, want = oracle.nerf_forward(p, pc, pf, o, d, n, f, uc, uf, F64)
    assert m_c.all() and m_f.all() and w_p.shape == (6, 64)
    for k in ("pred_rgb", "pred_depth", "acc_map", "weights"):
        np.testing.assert_array_equal(got[k], want[k])


def test_gated_render_skips_gated_samples(oracle, ng):
    """Gating every coarse sample off leaves only the fine draws, which the
    fine sampler then places from a flat PDF (all coarse weights 0)."""
    p = params(ng)
    o, d, n, f = ng.synthetic.sphere_rays(4, 10)
    rng = np.random.default_rng(11)
    uc, uf = rng.random((4, 64)), rng.random((4, 128))
    pc, pf = oracle.glorot_params(1, F64), oracle.glorot_params(2, F64)
    blob = ng.proposal.glorot_blob(4)
    got, m_c, m_f, _ = oracle.nerf_render_gated(p, blob, pc, pf, o, d, n, f, uc, uf, 10.0, F64)
    assert not m_c.any() and m_f.sum() == 4 * 128
    assert np.all(got["weights"][~m_f] == 0)
    # gating the draws by their bins as well leaves nothing: empty rays
    got, _, m_f, _ = oracle.nerf_render_gated(p, blob, pc, pf, o, d, n, f, uc, uf, 10.0, F64, gate_draws=True)
    assert not m_f.any() and np.all(got["acc_map"] == 0) and np.all(got["pred_rgb"] == 0)


# --- ray generation ----------------------------------------------------------
def test_get_rays_tf_matches_float64(oracle, ng):
    """get_rays_tf (float32, ray_utils.py:53-106) against get_rays (float64,
    :6-51): the same rays to float32 rounding."""
    K = ng.synthetic.intrinsic(12, 17, 21.5)
    pose = ng.synthetic.random_pose(4)
    o32, d32 = oracle.get_rays_tf(12, 17, K, pose)
    o64, d64 = oracle.get_rays(12, 17, K, pose)
    assert o32.dtype == np.float32 and d32.shape == (12 * 17, 3)
    np.testing.assert_allclose(d32, d64, atol=2e-6)
    np.testing.assert_allclose(o32, o64, atol=1e-6)
    np.testing.assert_allclose(np.linalg.norm(d32, axis=1), 1.0, atol=1e-6)


def test_low_precision_roundings(oracle):
    """The emulation's format roundings: round-to-nearest-even, E4M3 with
    subnormals (step 2^-9) and saturation to 448 (OCP FP8 formats)."""
    x = np.array([0, 1, 1.0625, 1.125, 1.1875, 448, 460, 1000, -1000, 2.0 ** -6, 2.0 ** -9, 3 * 2.0 ** -10,
                  2.0 ** -10, 2.0 ** -11, -0.3, 240, 232], np.float32)
    want = np.array([0, 1, 1, 1.125, 1.25, 448, 448, 448, -448, 2.0 ** -6, 2.0 ** -9, 2.0 ** -8, 0, 0,
                     -0.3125, 240, 224], np.float32)
    assert np.array_equal(oracle.round_e4m3(x), want)
    b = np.array([1.00390625, 1.01171875, 3.14159, -2.0 ** -130, 65504.0], np.float32)
    assert np.array_equal(oracle.round_bf16(b), np.array([1.0, 1.015625, 3.140625, -2.0 ** -130, 65536.0],
                                                         np.float32))
    # every E4M3 value is a fixed point
    vals = np.array([s * m * 2.0 ** e for s in (1, -1) for e in range(-6, 9) for m in np.arange(8, 16) / 8
                     if m * 2.0 ** e <= 448], np.float32)
    assert np.array_equal(oracle.round_e4m3(vals), vals)


def test_proposal_encoding_kernel_close_to_exact(oracle):
    """The proposal kernels' octave-doubling encoding stays within a few 1e-6
    of sin/cos evaluated at every octave in float32 (the reference encoding's
    arithmetic), far below the BF16 rounding it then gets; both are ~2.5e-5
    from float64 at the top octave (the float32 rounding of the angle)."""
    x = np.random.default_rng(3).uniform(-4, 4, (5000, 3)).astype(np.float32)
    got = oracle.proposal_encoding_kernel(x)
    want = oracle.positional_encoding(x, 6, np.float32)
    assert got.shape == want.shape and np.array_equal(got[:, :3], x)
    assert np.abs(got - want).max() < 4e-6


def test_mlp_encoding_kernel_close_to_float32(oracle):
    """The tensor-core MLP's encoding (octaves by at most three doublings from
    every fourth) stays within 1e-6 of the float32 encoding at every octave."""
    rng = np.random.default_rng(4)
    for L in (10, 4):
        x = rng.uniform(-4, 4, (5000, 3)).astype(np.float32)
        got = oracle.positional_encoding_kernel(x, L)
        want = oracle.positional_encoding(x, L, np.float32)
        assert got.shape == want.shape
        assert np.abs(got - want).max() < 1e-6, (L, float(np.abs(got - want).max()))
