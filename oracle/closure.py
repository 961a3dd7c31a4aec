"""CPU oracle of the learned eddy-viscosity closure (test infrastructure only).

The reference has no learned closure; everything here is a project definition, restated in
numpy FP64 so the GPU kernels (ark-cpp-mpi_gb300/csrc/ark_closure.cu) can be checked against
it.  Arrays are interior cells [k, j, i] (C3, C2, C1) unless a name says otherwise.

Definitions:
  * box filter: three-point means along x, then y, then z (3 x 3 x 3 box); x and z periodic;
    a solid neighbour in y contributes -a (velocities: no-slip reflection) or +a (products).
  * gradient A[m][d] = d u_m / d x_d by central differences, a solid neighbour counting as -u_c.
  * features (10): with S = (A + A^T)/2 and W = (A - A^T)/2,
      tr S, sqrt(tr S^2), sqrt(-tr W^2), cbrt(tr S^3), cbrt(tr W^2 S), root4(tr W^2 S^2),
      root6(tr W^2 S W S^2), -sgn(y) S_12, -sgn(y) W_12, y+ = (ly/2 - |y|) u_tau / nu
    (signed roots keep every invariant in units of 1/time; the two wall-frame components are
    positive near both walls in the mean shear).
  * target: nu* / nu with nu* = max(0, -tau^d : S^d / (2 S^d : S^d)), tau = filter(u_i u_j) -
    filter(u_i) filter(u_j), ^d the deviatoric parts; 0 where S^d : S^d < 1e-30.
  * network: x_n = (x - mu) / sd; h1 = GELU(W1 x_n + b1) (32); h2 = GELU(W2 h1 + b2) (32);
    y = softplus(w3 . h2 + b3) = nu_t / nu.  GELU in its tanh form:
    GELU(z) = z (1 + tanh(sqrt(2/pi) (z + 0.044715 z^3))) / 2.
    Parameters (1441) in the order W1[32][10], b1[32], W2[32][32], b2[32], w3[32], b3[1]; the
    forward and backward passes use them rounded to BF16 (nearest even).
  * loss: mean over the batch of (y - target)^2.
"""
from __future__ import annotations

import math

import numpy as np

NIN, NH = 10, 32
NPARAM = NH * NIN + NH + NH * NH + NH + NH + 1


def split(theta):
    """Flat parameters -> (W1, b1, W2, b2, w3, b3)."""
    t = np.asarray(theta, dtype=np.float64)
    o = 0
    W1 = t[o:o + NH * NIN].reshape(NH, NIN); o += NH * NIN
    b1 = t[o:o + NH]; o += NH
    W2 = t[o:o + NH * NH].reshape(NH, NH); o += NH * NH
    b2 = t[o:o + NH]; o += NH
    w3 = t[o:o + NH]; o += NH
    b3 = t[o]
    return W1, b1, W2, b2, w3, b3


def bf16(a):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    u = np.ascontiguousarray(np.asarray(a, dtype=np.float32)).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


_K0, _K1 = math.sqrt(2.0 / math.pi), 0.044715


def gelu(z):
    return 0.5 * z * (1.0 + np.tanh(_K0 * (z + _K1 * z ** 3)))


def gelu_grad(z):
    th = np.tanh(_K0 * (z + _K1 * z ** 3))
    return 0.5 * (1.0 + th) + 0.5 * z * (1.0 - th * th) * _K0 * (1.0 + 3.0 * _K1 * z * z)


def softplus(z):
    return np.maximum(z, 0.0) + np.log1p(np.exp(-np.abs(z)))


def sigmoid(z):
    return 1.0 / (1.0 + np.exp(-z))


def forward(theta, mu, sd, X):
    """nu_t / nu for raw features X (n, 10); theta used as given (round it with bf16 first)."""
    W1, b1, W2, b2, w3, b3 = split(theta)
    xn = (np.asarray(X, np.float64) - mu) / sd
    h1 = gelu(xn @ W1.T + b1)
    h2 = gelu(h1 @ W2.T + b2)
    return softplus(h2 @ w3 + b3)


def loss_and_grad(theta, mu, sd, X, target):
    """(mean squared error, gradient over the 1441 parameters), FP64."""
    W1, b1, W2, b2, w3, b3 = split(theta)
    X = np.asarray(X, np.float64)
    t = np.asarray(target, np.float64)
    n = X.shape[0]
    xn = (X - mu) / sd
    z1 = xn @ W1.T + b1
    h1 = gelu(z1)
    z2 = h1 @ W2.T + b2
    h2 = gelu(z2)
    z3 = h2 @ w3 + b3
    y = softplus(z3)
    r = y - t
    loss = float(np.mean(r * r))
    dz3 = (2.0 / n) * r * sigmoid(z3)
    gw3 = h2.T @ dz3
    gb3 = dz3.sum()
    dz2 = np.outer(dz3, w3) * gelu_grad(z2)
    gW2 = dz2.T @ h1
    gb2 = dz2.sum(0)
    dz1 = (dz2 @ W2) * gelu_grad(z1)
    gW1 = dz1.T @ xn
    gb1 = dz1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gw3, [gb3]])
    return loss, g


# ---- fields -------------------------------------------------------------------------------

def _shift(a, d, s, solid_lo, solid_hi, sign):
    """a shifted by s (+1: neighbour i+1) along axis d of [k, j, i] arrays; y (d = 1) uses the
    solid-neighbour rule (sign * a_c), x and z wrap."""
    if d == 1:
        out = np.roll(a, -s, axis=1)
        if s > 0:
            edge = solid_hi
            out[:, -1, :] = np.where(edge, sign * a[:, -1, :], out[:, -1, :])
        else:
            edge = solid_lo
            out[:, 0, :] = np.where(edge, sign * a[:, 0, :], out[:, 0, :])
        return out
    axis = 2 if d == 0 else 0
    return np.roll(a, -s, axis=axis)


def box_filter(a, sign):
    """3 x 3 x 3 box filter of an interior array of the channel (walls below j = 1 and above
    j = C2), x then y then z; sign -1 for velocities, +1 for products."""
    b = np.asarray(a, np.float64)
    for d in (0, 1, 2):
        b = (_shift(b, d, -1, True, True, sign) + b + _shift(b, d, 1, True, True, sign)) / 3.0
    return b


def gradient(u, dx):
    """A[m][d] (3, 3, C3, C2, C1) of interior velocity arrays u[m] in the channel."""
    A = np.empty((3, 3) + u[0].shape)
    for m in range(3):
        for d in range(3):
            A[m, d] = (_shift(u[m], d, 1, True, True, -1.0) - _shift(u[m], d, -1, True, True, -1.0)) / (2.0 * dx[d])
    return A


def _sroot(x, n):
    return np.sign(x) * np.abs(x) ** (1.0 / n)


def features(u, dx, ly, u_tau, nu):
    """(C3, C2, C1, 10) raw features of interior velocity arrays u[m] of the channel."""
    A = gradient(u, dx)
    A = np.moveaxis(A, (0, 1), (-2, -1))  # (..., 3, 3)
    S = 0.5 * (A + np.swapaxes(A, -1, -2))
    W = 0.5 * (A - np.swapaxes(A, -1, -2))
    S2 = S @ S
    W2 = W @ W
    tr = lambda M: np.trace(M, axis1=-2, axis2=-1)
    C2 = u[0].shape[1]
    y = -0.5 * ly + (np.arange(C2) + 0.5) * (ly / C2)
    sg = -np.sign(y)[None, :, None]
    f = np.empty(u[0].shape + (NIN,))
    f[..., 0] = tr(S)
    f[..., 1] = np.sqrt(np.maximum(tr(S2), 0.0))
    f[..., 2] = np.sqrt(np.maximum(-tr(W2), 0.0))
    f[..., 3] = _sroot(tr(S2 @ S), 3)
    f[..., 4] = _sroot(tr(W2 @ S), 3)
    f[..., 5] = _sroot(tr(W2 @ S2), 4)
    f[..., 6] = _sroot(tr(W2 @ S @ W @ S2), 6)
    f[..., 7] = sg * S[..., 0, 1]
    f[..., 8] = sg * W[..., 0, 1]
    f[..., 9] = ((0.5 * ly - np.abs(y)) * (u_tau / nu))[None, :, None] * np.ones(u[0].shape)
    return f


def target(u, dx, nu):
    """nu* / nu (C3, C2, C1) from interior velocity arrays u[m] (unfiltered)."""
    ub = [box_filter(u[m], -1.0) for m in range(3)]
    tau = np.empty((3, 3) + u[0].shape)
    for a in range(3):
        for b in range(a, 3):
            tau[a, b] = box_filter(u[a] * u[b], 1.0) - ub[a] * ub[b]
            tau[b, a] = tau[a, b]
    A = gradient(ub, dx)
    S = 0.5 * (A + np.swapaxes(A, 0, 1))
    trS = S[0, 0] + S[1, 1] + S[2, 2]
    trT = tau[0, 0] + tau[1, 1] + tau[2, 2]
    num = 0.0
    den = 0.0
    for a in range(3):
        for b in range(3):
            sd = S[a, b] - (trS / 3.0 if a == b else 0.0)
            td = tau[a, b] - (trT / 3.0 if a == b else 0.0)
            num = num - td * sd
            den = den + 2.0 * sd * sd
    nut = np.where(den > 1e-30, np.maximum(num / np.where(den > 1e-30, den, 1.0), 0.0), 0.0)
    return nut / nu, ub
