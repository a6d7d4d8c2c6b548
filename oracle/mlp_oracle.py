"""CPU oracle of the learned closure's network (TEST INFRASTRUCTURE ONLY).

The engine's MLP (nimblesm_gb300/csrc/mlp_common.cuh): sigma/G = B(H) +
s_r * |x|^3 * MLP(x), x = H * s_in, B the neo-Hookean stress over G to second
order in H (linear_part + quadratic_part), MLP = 9 -> 64 -> 64 -> 6 with GELU
(sigmoid form), evaluated with BF16 operands and FP32 accumulation on the
tensor cores.  This module restates the
forward pass and the gradient of the training loss in float64 numpy, either
emulating the BF16 roundings at exactly the points where the GPU rounds
(emulate=True, for a tight gradient check) or in exact arithmetic
(emulate=False, the mathematical gradient).
"""
import numpy as np

HID, IN, OUT = 64, 9, 6
oW1, ob1 = 0, HID * IN
oW2, ob2 = ob1 + HID, ob1 + HID + HID * HID
oW3, ob3 = ob2 + HID, ob2 + HID + OUT * HID
NPARAMS = ob3 + OUT


def bf16(x):
    """Round to the nearest BF16 (ties to even), as float64."""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(P):
    P = np.asarray(P, np.float64)
    return (P[oW1:ob1].reshape(HID, IN), P[ob1:oW2], P[oW2:ob2].reshape(HID, HID), P[ob2:oW3],
            P[oW3:ob3].reshape(OUT, HID), P[ob3:])


def linear_part(H, k_over_g):
    """Small-strain neo-Hookean stress over G (symmetric order), H row-major."""
    tr = H[:, 0] + H[:, 4] + H[:, 8]
    a, d = k_over_g * tr, tr / 3.0
    return np.stack([a + 2 * (H[:, 0] - d), a + 2 * (H[:, 4] - d), a + 2 * (H[:, 8] - d),
                     H[:, 1] + H[:, 3], H[:, 5] + H[:, 7], H[:, 6] + H[:, 2]], axis=1)


def quadratic_part(H, k_over_g):
    """The second-order terms of the neo-Hookean stress over G (the reference's
    sigma = K/2 (J - 1/J) I + G J^(-5/3) dev(F F^T), src/nimble_material.cc:252-310,
    expanded in H): -K/(2G) tr(H H) I + H H^T - |H|^2/3 I - 10/3 tr(H) dev(eps)."""
    Hm = np.asarray(H, np.float64).reshape(-1, 3, 3)
    tr = np.trace(Hm, axis1=1, axis2=2)
    trhh = np.einsum("nij,nji->n", Hm, Hm)
    hht = np.einsum("nij,nkj->nik", Hm, Hm)
    n2 = np.einsum("nij,nij->n", Hm, Hm)
    eps = 0.5 * (Hm + Hm.transpose(0, 2, 1))
    dev = eps - (tr / 3.0)[:, None, None] * np.eye(3)[None]
    Q = (-0.5 * k_over_g * trhh - n2 / 3.0)[:, None, None] * np.eye(3)[None] + hht - (10.0 / 3.0) * tr[:, None, None] * dev
    return np.stack([Q[:, 0, 0], Q[:, 1, 1], Q[:, 2, 2], Q[:, 0, 1], Q[:, 1, 2], Q[:, 2, 0]], axis=1)


def base_part(H, k_over_g):
    """The neo-Hookean stress over G to second order in H (the closure's base)."""
    return linear_part(H, k_over_g) + quadratic_part(H, k_over_g)


def act(u):
    """The engine's activation: GELU in its sigmoid form x sigma(1.702 x)
    (Hendrycks & Gimpel 2016), written a(u) = u (1 + tanh u) = 2 u sigma(2u)
    with u = 0.851 x, the constant factors being the adjacent layers'."""
    return u * (1.0 + np.tanh(u))


def act_grad(u):
    t = np.tanh(u)
    return 1.0 + t + u * (1.0 - t * t)


def forward(P, scales, H, emulate=True):
    W1, b1, W2, b2, W3, b3 = unpack(P)
    r = bf16 if emulate else (lambda v: np.asarray(v, np.float64))
    xs = (np.asarray(H, np.float32) * np.float32(scales[0])).astype(np.float32)
    hi = bf16(xs) if emulate else xs.astype(np.float64)
    lo = bf16((xs - hi.astype(np.float32)).astype(np.float32)) if emulate else np.zeros_like(hi)
    n = H.shape[0]
    X = np.zeros((n, 32))
    X[:, :9], X[:, 9], X[:, 16:25] = hi, 1.0, lo
    W1x = np.zeros((HID, 32))
    W1x[:, :9], W1x[:, 9], W1x[:, 16:25] = W1, b1, W1
    z1 = X @ r(W1x).T
    a1 = r(act(z1))
    z2 = a1 @ r(W2).T + b2
    a2 = r(act(z2))
    out = a2 @ r(W3).T + b3
    return dict(X=X, z1=z1, a1=a1, z2=z2, a2=a2, out=out)


def gate(H, scales):
    """The cubic gate |x|^3."""
    xs = (np.asarray(H, np.float32) * np.float32(scales[0])).astype(np.float64)
    return np.maximum((xs * xs).sum(axis=1) ** 1.5, 1e-30)


def stress_over_g(P, scales, H, emulate=True):
    f = forward(P, scales, H, emulate)
    return base_part(np.asarray(H, np.float64), scales[2]) + (scales[1] * gate(H, scales))[:, None] * f["out"]


def loss_and_gradient(P, scales, H, Y, emulate=True):
    """Mean over points of the squared scaled residual and its gradient."""
    W1, b1, W2, b2, W3, b3 = unpack(P)
    r = bf16 if emulate else (lambda v: np.asarray(v, np.float64))
    n = H.shape[0]
    f = forward(P, scales, H, emulate)
    t = (np.asarray(Y, np.float64) - base_part(np.asarray(H, np.float64), scales[2])) / \
        (scales[1] * gate(H, scales))[:, None]
    d = f["out"] - t
    loss = float((d * d).sum() / n)
    g = r(2.0 * d / n)
    dW3, db3 = g.T @ f["a2"], g.sum(axis=0)
    dz2 = r((g @ r(W3)) * act_grad(f["z2"]))
    dW2, db2 = dz2.T @ f["a1"], dz2.sum(axis=0)
    dz1 = r((dz2 @ r(W2)) * act_grad(f["z1"]))
    dW1x = dz1.T @ f["X"]
    grad = np.zeros(NPARAMS)
    grad[oW1:ob1] = (dW1x[:, :9] + dW1x[:, 16:25]).ravel()
    grad[ob1:oW2] = dW1x[:, 9]
    grad[oW2:ob2] = dW2.ravel()
    grad[ob2:oW3] = db2
    grad[oW3:ob3] = dW3.ravel()
    grad[ob3:] = db3
    return loss, grad
