"""CPU oracle of the learned control variate's network. TEST INFRASTRUCTURE ONLY.

Restates the forward and backward passes of leo2d_gb300/csrc/mlp.cu
(16 -> 3 x 256 GELU -> 256, parameters W0 [256][64], b0, W1 [256][256], b1,
W2, b2, W3, b3 as one FP32 vector) in float64. With exact=False it applies
BF16 rounding (round to nearest even) where the GPU stores BF16: the input
features, the weights, the activations, the loss gradient and the
back-propagated gradients. The remaining differences to the GPU are then FP32
accumulation order and rare rounding-boundary cases. The activation is GELU
with erf in the form of Abramowitz & Stegun 7.1.27 (within 5e-4 of erf): that
form defines the network, here in float64 and on the GPU in FP32. With
exact=True no rounding is applied (for finite-difference checks of this oracle).

The network has no counterpart in the reference (LEO2D has no learned part);
the site features follow Hstruct::getShiftConfigs (hstruct.cpp:672-820).
"""
import numpy as np

K_IN, HID, OUT, N_FEAT = 64, 256, 256, 16
IN_DIM = (64, 256, 256, 256)


def bf16(x):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint32) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def param_count():
    return sum(HID * d + HID for d in IN_DIM)


def unpack(p):
    p = np.asarray(p, np.float64)
    Ws, bs, off = [], [], 0
    for d in IN_DIM:
        Ws.append(p[off:off + HID * d].reshape(HID, d))
        off += HID * d
        bs.append(p[off:off + HID])
        off += HID
    return Ws, bs


def pack(Ws, bs):
    out = []
    for W, b in zip(Ws, bs):
        out.append(np.ravel(W))
        out.append(np.ravel(b))
    return np.concatenate(out)


# erf(x) ~ 1 - q(x)^-4, q = 1 + a1 x + a2 x^2 + a3 x^3 + a4 x^4 (x >= 0, odd
# extension): Abramowitz & Stegun, Handbook of Mathematical Functions, 7.1.27
AS_A = (0.278393, 0.230389, 0.000972, 0.078108)


def _q(x):
    a1, a2, a3, a4 = AS_A
    return (((a4 * x + a3) * x + a2) * x + a1) * x + 1.0


def net_erf(x):
    """The network's erf (A&S 7.1.27), float64."""
    x = np.asarray(x, np.float64)
    with np.errstate(over="ignore"):
        return np.sign(x) * (1.0 - _q(np.abs(x)) ** -4)


def gelu(z):
    return 0.5 * z * (1.0 + net_erf(z / np.sqrt(2.0)))


def gelu_grad(z):
    a1, a2, a3, a4 = AS_A
    x = np.abs(z) / np.sqrt(2.0)
    dq = ((4 * a4 * x + 3 * a3) * x + 2 * a2) * x + a1
    with np.errstate(over="ignore"):
        derf = 4.0 * dq / _q(x) ** 5
    return 0.5 * (1.0 + net_erf(z / np.sqrt(2.0))) + z * derf / (2.0 * np.sqrt(2.0))


def _round(exact):
    return (lambda a: np.asarray(a, np.float64)) if exact else bf16


def forward(p, x, exact=False):
    r = _round(exact)
    x = np.asarray(x, np.float64)
    X = np.zeros((x.shape[0], K_IN))
    X[:, :x.shape[1]] = x
    Ws, bs = unpack(p)
    A = r(X)
    for l in range(4):
        Z = A @ r(Ws[l]).T + bs[l]
        if l < 3:
            if not exact:
                Z = Z.astype(np.float32).astype(np.float64)
            A = r(gelu(Z))
        else:
            return Z


def loss_and_grad(p, x, t, w=None, exact=False):
    """Loss (1/n) sum w_j (y - t)^2 and its gradient (parameter-vector layout)."""
    r = _round(exact)
    x = np.asarray(x, np.float64)
    t = np.asarray(t, np.float64)
    n = x.shape[0]
    w = np.ones(OUT) if w is None else np.asarray(w, np.float64)
    X = np.zeros((n, K_IN))
    X[:, :x.shape[1]] = x
    Ws, bs = unpack(p)
    Wr = [r(W) for W in Ws]
    A = [r(X)]
    Zs = []
    for l in range(4):
        Z = A[-1] @ Wr[l].T + bs[l]
        if l < 3:
            if not exact:
                Z = Z.astype(np.float32).astype(np.float64)
            Zs.append(Z)
            A.append(r(gelu(Z)))
        else:
            Y = Z
    d = Y - t
    loss = float(np.sum(w * d * d) / n)
    dZf = 2.0 / n * w * d
    dZb = r(dZf)
    gW, gb = [None] * 4, [None] * 4
    for l in range(3, -1, -1):
        gb[l] = dZf.sum(axis=0)
        gW[l] = dZb.T @ A[l]
        if l > 0:
            dZf = (dZb @ Wr[l]) * gelu_grad(Zs[l - 1])
            dZb = r(dZf)
    return loss, pack(gW, gb)


def erf_as7127_f32(x):
    """The network's erf with every operation rounded to FP32 in the GPU's order
    (the GPU's reciprocal is rcp.approx, within an ulp of this)."""
    t = np.float32
    z = np.asarray(x, t)
    ax = np.abs(z)
    a1, a2, a3, a4 = AS_A
    with np.errstate(over="ignore"):
        p = t(a4) * ax + t(a3)
        for c in (a2, a1, 1.0):
            p = (p * ax + t(c)).astype(t)
        for _ in range(2):
            p = (p * p).astype(t)
        e = (t(1.0) - (t(1.0) / p).astype(t)).astype(t)
    return np.copysign(e, z)
