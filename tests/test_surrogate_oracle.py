"""The surrogate's FP64 oracle (oracle/surrogate_ref.py) on the CPU: its
backward pass against central finite differences of its forward pass, its
bf16 rounding, and its patch layout."""
import numpy as np
import pytest

from oracle import surrogate_ref as R

P, C, E, L = 4, 6, 8, 2
NORM = (0.5, 2.0, 0.4, 10.0)
SCALE = (3.0, 5.0)


def _case(seed=0, B=2, H=8, W=12):
    rng = np.random.default_rng(seed)
    params = R.random_params(P, C, E, L, rng)
    for k in params:
        if k.startswith("b"):
            params[k] = rng.normal(0, 0.1, params[k].shape)
    f_old = np.stack([rng.random((B, H, W)), 0.4 + 0.05 * rng.random((B, H, W))], axis=1)
    f_new = f_old + 0.05 * rng.normal(size=f_old.shape)
    return params, f_old, f_new


def _loss(params, f_old, f_new):
    return R.loss_and_grads(params, f_old, f_new, P, L, NORM, SCALE, bf16_ops=False)[0]


def test_patch_roundtrip():
    rng = np.random.default_rng(1)
    f = rng.random((2, 2, 8, 12))
    x = R.patches(f, 4)
    assert x.shape == (2 * 2 * 3, 2 * 16)
    # token 4 = sample 0, patch row 1, patch col 1; column 16 + 5 = channel 1, py 1, px 1
    assert x[4, 16 + 5] == f[0, 1, 4 + 1, 4 + 1]
    np.testing.assert_array_equal(R.unpatch(x, 2, 8, 12, 4), f)


def test_bf16_rounding_is_round_to_nearest_even():
    vals = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -2.5, 3.0e-30])
    got = R.bf16(vals)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: even mantissa (1) wins;
    # 1 + 3 * 2^-8 ties between 1 + 2^-7 and 1 + 2^-6: even is 1 + 2^-6
    np.testing.assert_array_equal(got[:5], [1.0, 1.0, 1.0 + 2 ** -6, 1.0, -2.5])
    assert abs(got[5] - 3.0e-30) <= 3.0e-30 * 2 ** -8


def test_backward_matches_finite_differences():
    params, f_old, f_new = _case()
    loss, grads, _ = R.loss_and_grads(params, f_old, f_new, P, L, NORM, SCALE, bf16_ops=False)
    assert loss > 0
    rng = np.random.default_rng(2)
    h = 1e-6
    for name, g in grads.items():
        assert g.shape == params[name].shape
        flat = params[name].reshape(-1)
        for idx in rng.choice(flat.size, size=min(4, flat.size), replace=False):
            old = flat[idx]
            flat[idx] = old + h
            lp = _loss(params, f_old, f_new)
            flat[idx] = old - h
            lm = _loss(params, f_old, f_new)
            flat[idx] = old
            fd = (lp - lm) / (2 * h)
            an = g.reshape(-1)[idx]
            assert abs(fd - an) <= 1e-6 * max(1.0, abs(an)) + 1e-5 * abs(an), (name, idx, fd, an)


def test_directional_derivative():
    params, f_old, f_new = _case(3)
    _, grads, _ = R.loss_and_grads(params, f_old, f_new, P, L, NORM, SCALE, bf16_ops=False)
    rng = np.random.default_rng(4)
    v = {k: rng.normal(size=p.shape) for k, p in params.items()}
    h = 1e-6
    plus = {k: p + h * v[k] for k, p in params.items()}
    minus = {k: p - h * v[k] for k, p in params.items()}
    fd = (_loss(plus, f_old, f_new) - _loss(minus, f_old, f_new)) / (2 * h)
    an = sum(float((grads[k] * v[k]).sum()) for k in params)
    assert fd == pytest.approx(an, rel=1e-6)


def test_bf16_emulation_stays_close_to_fp64():
    params, f_old, f_new = _case(5)
    l64, g64, o64 = R.loss_and_grads(params, f_old, f_new, P, L, NORM, SCALE, bf16_ops=False)
    l16, g16, o16 = R.loss_and_grads(params, f_old, f_new, P, L, NORM, SCALE, bf16_ops=True)
    assert np.linalg.norm(o16 - o64) / np.linalg.norm(o64) < 2e-2
    assert l16 == pytest.approx(l64, rel=2e-2)
    for k in g64:
        assert np.linalg.norm(g16[k] - g64[k]) <= 5e-2 * np.linalg.norm(g64[k]) + 1e-12, k
