"""The CPU restatement of the learned gas-optics network: its analytic
gradients against central differences (float64), and the bf16-emulating
version against the float64 one.  These pin the checker that the GPU
training kernels are compared with (tests/test_gpu_mlp.py)."""
import numpy as np

import mlp_oracle as M


def _case(rows=6, seed=3):
    rs = np.random.default_rng(seed)
    p = rs.normal(0.0, 0.3, M.NPARAM)
    x = np.zeros((rows, M.KIN))
    x[:, :9] = rs.normal(size=(rows, 9))
    t = np.zeros((rows, M.NOUTP))
    t[:, :M.NOUT] = rs.normal(size=(rows, M.NOUT))
    return p, x, t


def test_gradients_match_central_differences():
    p, x, t = _case()
    _, g = M.forward_backward(p, x, t, emulate=False)
    rs = np.random.default_rng(0)
    idx = []
    for k, (o, n) in M.OFF.items():
        idx += list(o + rs.choice(n, 6, replace=False))
    idx = np.array(idx)
    fd = M.finite_difference(p, x, t, idx)
    scale = np.abs(g).max()
    assert np.abs(fd - g[idx]).max() <= 1e-6 * scale + 1e-9, np.abs(fd - g[idx]).max()


def test_padding_outputs_and_inputs_carry_no_gradient():
    p, x, t = _case()
    _, g = M.forward_backward(p, x, t, emulate=False)
    G = M.unpack(g)
    assert np.all(G["W4"][:, M.NOUT:] == 0) and np.all(G["b4"][M.NOUT:] == 0)
    assert np.all(G["W1"][9:, :] == 0)  # padded inputs are zero


def test_bf16_emulation_close_to_float64():
    p, x, t = _case(rows=16)
    l64, g64 = M.forward_backward(p, x, t, emulate=False)
    l16, g16 = M.forward_backward(p, x, t, emulate=True)
    assert abs(l16 - l64) <= 2e-2 * l64
    assert np.abs(g16 - g64).max() <= 5e-2 * np.abs(g64).max()


def test_bf16_rounding():
    # 1 + 2^-8 and 1 + 3*2^-8 are halfway cases (bf16 spacing at 1 is 2^-7): ties go to the even mantissa
    v = np.array([1.0, 1.00390625, 1.01171875, 1.001953125, 3.0e-3, -2.5, 65504.0], dtype=np.float32)
    r = M.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.015625 and r[3] == 1.0
    assert np.all(np.abs(r - v) <= np.abs(v) * 2.0 ** -8)
