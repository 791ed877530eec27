"""The learned-schedule MLP: the CPU reference's backward pass against finite
differences (CPU), its restatement in the device rounding (bf16 operands,
fp32 accumulation) against the exact one (CPU), and the device training
kernel's gradients against that restatement (GPU)."""
import numpy as np
import pytest


def params_for(nin, nh, seed):
    rng = np.random.default_rng(seed)
    n = nh * nin + nh + nh * nh + nh + 2 * nh + 2
    return (rng.normal(0, 0.3, n)).astype(np.float32)


def test_oracle_backward_matches_finite_differences(po):
    nin, nh, B = 6, 16, 20
    rng = np.random.default_rng(3)
    prm = params_for(nin, nh, 1).astype(np.float64)
    x = rng.normal(size=(B, nin)).astype(np.float32)
    y = rng.normal(size=(B, 2)).astype(np.float32)
    g, L = po.mlp_forward_backward(nin, nh, prm, x, y)
    # central differences through the same code path; a ReLU kink inside the
    # stencil spoils a difference quotient, which shows as disagreement
    # between two step sizes, so those indices are skipped
    def fd(i, h):
        pp, pm = prm.copy(), prm.copy()
        pp[i] += h
        pm[i] -= h
        return (po.mlp_forward_backward(nin, nh, pp, x, y)[1] - po.mlp_forward_backward(nin, nh, pm, x, y)[1]) / (2 * h)

    checked = 0
    for i in rng.choice(len(prm), 60, replace=False):
        f1, f2 = fd(i, 2e-3), fd(i, 1e-3)
        if abs(f1 - f2) > 1e-3 * max(1.0, abs(f1)):
            continue
        checked += 1
        assert abs(f2 - g[i]) < 2e-3 * max(1.0, abs(g[i])), (i, f2, g[i])
    assert checked >= 40


def test_bf16_rounding_helper(po):
    v = np.array([1.0, 1.00390625, 1.005859375, -3.14159], dtype=np.float32)
    r = po.bf16_round(v)
    assert r[0] == 1.0 and r[1] == 1.0  # tie rounds to even
    assert r[2] == np.float32(1.0078125)


def test_device_rounding_restatement_close_to_exact(po):
    """bf16 operands cost about 2^-9 relative per product: the gradient in the
    device rounding stays within 2% of the exact one (max norm)."""
    nin, nh, B = 6, 64, 512
    rng = np.random.default_rng(5)
    prm = po.bf16_round(params_for(nin, nh, 2))
    x = rng.normal(size=(B, nin)).astype(np.float32)
    y = rng.normal(size=(B, 2)).astype(np.float32)
    g_e, L_e = po.mlp_forward_backward(nin, nh, prm, x, y)
    g_d, L_d = po.mlp_forward_backward(nin, nh, prm, x, y, rounding="device")
    assert abs(L_d - L_e) <= 1e-2 * L_e
    assert np.abs(g_d - g_e).max() <= 2e-2 * np.abs(g_e).max()


@pytest.mark.gpu
@pytest.mark.parametrize("nin,nh,B", [(6, 64, 1024), (3, 64, 96), (13, 32, 257), (40, 64, 2048), (20, 48, 33)])
def test_device_gradients_match_reference(pkg, po, nin, nh, B):
    """Tolerance 1e-4 of the largest gradient entry: the tensor cores' fp32
    accumulation order differs from the restatement's, and an activation whose
    fp32 value sits on a bf16 rounding boundary can round the other way."""
    rng = np.random.default_rng(nin * 100 + nh)
    prm = po.bf16_round(params_for(nin, nh, 7))
    x = rng.normal(size=(B, nin)).astype(np.float32)
    y = rng.normal(size=(B, 2)).astype(np.float32)
    h = pkg._handle(0)
    g_dev, L_dev = h.learn_gradcheck(nin, nh, prm, x, y)
    g_ref, L_ref = po.mlp_forward_backward(nin, nh, prm, x, y, rounding="device")
    assert abs(L_dev - L_ref) <= 1e-4 * abs(L_ref)
    scale = np.abs(g_ref).max()
    assert np.abs(g_dev - g_ref).max() <= 1e-4 * scale
