"""The MLP oracle's backward pass against central finite differences (float64,
no BF16 rounding): relative agreement 1e-5 on randomly chosen parameters of
every layer (the activation's erf form has a second derivative that jumps at
0, which central differences over 1e-6 see at the 1e-6 level)."""
import numpy as np

from oracle import mlp_oracle as mo


def test_finite_differences():
    rng = np.random.default_rng(0)
    n = 32
    p = rng.normal(0, 0.1, mo.param_count())
    x = rng.uniform(-1, 1, (n, mo.N_FEAT))
    t = rng.normal(0, 0.3, (n, mo.OUT))
    w = rng.uniform(0.5, 2.0, mo.OUT)
    _, g = mo.loss_and_grad(p, x, t, w, exact=True)
    offs = np.cumsum([0] + [mo.HID * d + mo.HID for d in mo.IN_DIM])
    picks = []
    for l in range(4):
        wl = mo.HID * mo.IN_DIM[l]
        cols = rng.integers(0, min(mo.IN_DIM[l], mo.N_FEAT if l == 0 else mo.IN_DIM[l]), 4)
        rows = rng.integers(0, mo.HID, 4)
        picks += [offs[l] + r * mo.IN_DIM[l] + c for r, c in zip(rows, cols)]
        picks += list(offs[l] + wl + rng.integers(0, mo.HID, 2))
    eps = 1e-6
    for i in picks:
        q = p.copy()
        q[i] += eps
        lp, _ = mo.loss_and_grad(q, x, t, w, exact=True)
        q[i] -= 2 * eps
        lm, _ = mo.loss_and_grad(q, x, t, w, exact=True)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-5 * max(1e-3, abs(g[i])) + 1e-9, (i, fd, g[i])


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -2.5e-3, 3.0e38], np.float32)
    r = mo.bf16(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: ties go to even (1.0)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125
    assert np.all(np.abs(r[:4] - x[:4]) <= np.abs(x[:4]) * 2.0 ** -8)


def test_erf_form_of_the_network():
    """The network's erf (Abramowitz & Stegun 7.1.27) against the exact erf: the
    published bound 5e-4 in float64, and the same with every operation rounded
    to FP32 in the GPU's order, which stays within 1e-6 of the float64 form."""
    from scipy.special import erf
    x = np.linspace(-6.0, 6.0, 200_001)
    assert np.max(np.abs(mo.net_erf(x) - erf(x))) <= 5e-4
    x32 = x.astype(np.float32)
    e32 = mo.erf_as7127_f32(x32).astype(np.float64)
    assert np.max(np.abs(e32 - mo.net_erf(x32.astype(np.float64)))) <= 1e-6
    # saturation: the quartic's fourth power overflows to inf and erf to +-1 exactly
    assert mo.erf_as7127_f32(np.float32(1e12)) == 1.0
    assert mo.erf_as7127_f32(np.float32(-1e12)) == -1.0


def test_gelu_grad_is_the_derivative():
    z = np.linspace(-7.0, 7.0, 2001)
    h = 1e-6
    fd = (mo.gelu(z + h) - mo.gelu(z - h)) / (2 * h)
    assert np.max(np.abs(fd - mo.gelu_grad(z))) <= 1e-7
