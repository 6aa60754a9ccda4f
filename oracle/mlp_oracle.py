"""CPU oracle of the learned warm start.

Test infrastructure only: the tests and the bench's CPU leg use it as the
checker of the GPU kernels; the product never imports it.

The network has no counterpart in the reference (fem_conjugate_gradients.h:44-46
starts CG from the previous velocity).  This module restates the library's
definition of it (include/otfem_gpu.h, "learned warm start"):

- inputs per node: v, dv_prev, f_ext, and the mean of the 9 entries of Re over
  the tets that contain the node; normalised as (x - mean) / std;
- 18 -> 64 -> 64 -> 64 -> 3, GELU in tanh form on the hidden layers;
- every matrix product takes BF16-rounded operands (weights, activations and
  back-propagated errors) and accumulates in FP32, as the tensor cores do;
- loss: mean over samples and outputs of the squared error against the
  normalised target (dv - dv_prev); gradient w.r.t. the FP32 weights;
- Adam (Kingma & Ba 2015) with beta 0.9 / 0.999 and eps 1e-8.

With ``exact=True`` the same function is evaluated in float64 without BF16
rounding, for finite-difference checks of the gradient formulas.
"""
import numpy as np

N_IN, N_HID, N_OUT = 18, 64, 3
SHAPES = [("W1", (N_HID, N_IN)), ("b1", (N_HID,)), ("W2", (N_HID, N_HID)), ("b2", (N_HID,)),
          ("W3", (N_HID, N_HID)), ("b3", (N_HID,)), ("W4", (N_OUT, N_HID)), ("b4", (N_OUT,))]
NUM_WEIGHTS = sum(int(np.prod(s)) for _, s in SHAPES)  # 9731
NUM_NORM = 2 * N_IN + 2 * N_OUT
STATE_SIZE = NUM_WEIGHTS + NUM_NORM
GELU_C, GELU_A = np.float32(0.7978845608028654), np.float32(0.044715)


def unpack(state):
    """Weights (dict of arrays, weight[out][in]) and normalisation of a state vector."""
    state = np.asarray(state)
    w, off = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        w[name] = state[off:off + n].reshape(shape)
        off += n
    norm = state[off:off + NUM_NORM]
    return w, {"mu_x": norm[:N_IN], "sd_x": norm[N_IN:2 * N_IN], "mu_y": norm[2 * N_IN:2 * N_IN + N_OUT],
               "sd_y": norm[2 * N_IN + N_OUT:]}


def pack(w, norm):
    parts = [np.asarray(w[name], np.float32).reshape(-1) for name, _ in SHAPES]
    parts += [np.asarray(norm[k], np.float32) for k in ("mu_x", "sd_x", "mu_y", "sd_y")]
    return np.concatenate(parts).astype(np.float32)


def bf16(x):
    """Round float32 to the nearest bfloat16 (ties to even), returned as float32."""
    x = np.ascontiguousarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def gelu(z):
    return 0.5 * z * (1 + np.tanh(GELU_C * (z + GELU_A * z * z * z)))


def gelu_grad(z):
    th = np.tanh(GELU_C * (z + GELU_A * z * z * z))
    return 0.5 * (1 + th) + 0.5 * z * (1 - th * th) * GELU_C * (1 + 3 * GELU_A * z * z)


def _ops(exact):
    if exact:
        return np.float64, (lambda a: np.asarray(a, np.float64))
    return np.float32, bf16


def forward(state, x, exact=False):
    """Normalised outputs (n x 3) and the cache of the backward pass."""
    dt, rnd = _ops(exact)
    w, nm = unpack(np.asarray(state, dt))
    xn = ((np.asarray(x, dt) - nm["mu_x"].astype(dt)) / nm["sd_x"].astype(dt)).astype(dt)
    a = rnd(xn)
    cache = {"a": [a], "g": []}
    for l in (1, 2, 3):
        z = (a @ rnd(w[f"W{l}"]).T + w[f"b{l}"].astype(dt)).astype(dt)
        cache["g"].append(gelu_grad(z).astype(dt))
        a = rnd(gelu(z).astype(dt))
        cache["a"].append(a)
    y = (a @ rnd(w["W4"]).T + w["b4"].astype(dt)).astype(dt)
    return y, cache


def loss_and_gradient(state, x, y, exact=False):
    """Mean squared normalised error and its gradient (NUM_WEIGHTS values,
    in the state's weight order)."""
    dt, rnd = _ops(exact)
    w, nm = unpack(np.asarray(state, dt))
    out, cache = forward(state, x, exact)
    yn = ((np.asarray(y, dt) - nm["mu_y"].astype(dt)) / nm["sd_y"].astype(dt)).astype(dt)
    e = out - yn
    n = x.shape[0]
    loss = float(np.mean(np.asarray(e, np.float64) ** 2))
    d = (dt(2.0 / (3.0 * n)) * e).astype(dt)
    grads = {"W4": rnd(d).T @ cache["a"][3], "b4": d.sum(0)}
    dh = rnd(d) @ rnd(w["W4"])
    for l in (3, 2, 1):
        dz = (dh * cache["g"][l - 1]).astype(dt)
        grads[f"W{l}"] = rnd(dz).T @ cache["a"][l - 1]
        grads[f"b{l}"] = dz.sum(0)
        if l > 1:
            dh = rnd(dz) @ rnd(w[f"W{l}"])
    g = np.concatenate([np.asarray(grads[name], dt).reshape(-1) for name, _ in SHAPES])
    return loss, g


def predict(state, x, exact=False):
    """De-normalised outputs (the predicted dv - dv_prev)."""
    dt, _ = _ops(exact)
    _, nm = unpack(np.asarray(state, dt))
    out, _ = forward(state, x, exact)
    return out * nm["sd_y"].astype(dt) + nm["mu_y"].astype(dt)


def adam_step(state, grad, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update of the weights of `state` (float32); returns the new
    state, m, v."""
    p = np.asarray(state, np.float32).copy()
    g = np.asarray(grad, np.float32)
    m = (np.float32(b1) * m + np.float32(1 - b1) * g).astype(np.float32)
    v = (np.float32(b2) * v + np.float32(1 - b2) * g * g).astype(np.float32)
    c1, c2 = np.float32(1 - b1 ** t), np.float32(1 - b2 ** t)
    p[:NUM_WEIGHTS] -= np.float32(lr) * (m / c1) / (np.sqrt(v / c2) + np.float32(eps))
    return p, m, v


def node_features(tets, v, dv_prev, fext, re):
    """Network inputs of every node (N x 18): v, dv_prev, f_ext and the mean
    of the 9 entries of Re (re: T x 9, row-major) over the node's tets."""
    N = v.shape[0]
    acc = np.zeros((N, 9))
    cnt = np.zeros(N)
    for k in range(4):
        np.add.at(acc, tets[:, k], re)
        np.add.at(cnt, tets[:, k], 1)
    ring = acc / np.maximum(cnt, 1)[:, None]
    return np.concatenate([v, dv_prev, fext, ring], axis=1).astype(np.float32)
