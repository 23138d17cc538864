"""CPU restatement of the learned warm-start network (include/plume_net.h).

TEST INFRASTRUCTURE ONLY: the parity tests compare the CUDA forward and
backward passes of cfs_plume_gb300/csrc/unet.cu against this module; no
product path imports it.

The network has no counterpart in the reference (its solve always starts from
p = 0, FLUID_3D_MIC.cpp:360), so this restatement follows the layer order and
rounding points the C header documents:

* 16-channel input, channel 0 = the normalised right-hand side, rounded to BF16;
* ten 3x3x3 convolutions with zero padding, BF16 weights and inputs, wide
  accumulation, + FP32 bias, ReLU, output rounded to BF16;
* 2x2x2 mean pooling (rounded to BF16), nearest upsampling, skip
  concatenation [upsampled, skip];
* 1x1x1 output convolution 16 -> 1 with FP32 weights;
* loss = mean over interior cells of (y - t)^2, or of the energy norm
  e (A e) + 1e-4 e^2 of the error e = y - t (A the closed-box 7-point operator);
* gradient tensors are rounded to BF16 where the GPU stores them.

With bf16=False every rounding is skipped and the arithmetic is float64, which
is what the finite-difference check of the backward pass uses.
"""
import numpy as np

LAYERS = [("e1a", 16, 16, 0), ("e1b", 16, 16, 0), ("e2a", 16, 32, 1), ("e2b", 32, 32, 1),
          ("b3a", 32, 64, 2), ("b3b", 64, 64, 2), ("d2a", 96, 32, 1), ("d2b", 32, 32, 1),
          ("d1a", 48, 16, 0), ("d1b", 16, 16, 0)]


def num_params():
    return sum(27 * ci * co + co for _, ci, co, _ in LAYERS) + 17


def round_bf16(a):
    """Round-to-nearest-even to BF16, returned as float64."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params):
    p = np.asarray(params, dtype=np.float64)
    out, k = {}, 0
    for name, ci, co, _ in LAYERS:
        out[name + ".w"] = p[k:k + 27 * ci * co].reshape(27, ci, co)
        k += 27 * ci * co
        out[name + ".b"] = p[k:k + co]
        k += co
    out["out.w"] = p[k:k + 16]
    out["out.b"] = p[k + 16]
    assert k + 17 == p.size
    return out


def pack(grads):
    parts = []
    for name, ci, co, _ in LAYERS:
        parts.append(grads[name + ".w"].reshape(-1))
        parts.append(grads[name + ".b"].reshape(-1))
    parts.append(grads["out.w"].reshape(-1))
    parts.append(np.atleast_1d(grads["out.b"]))
    return np.concatenate(parts)


def _offsets():
    for off in range(27):
        yield off, off // 9 - 1, (off // 3) % 3 - 1, off % 3 - 1


def _shift(xp, dz, dy, dx, Z, Y, X):
    return xp[:, 1 + dz:1 + dz + Z, 1 + dy:1 + dy + Y, 1 + dx:1 + dx + X, :]


def conv3(x, w):
    """y[p] = sum_off x[p + d(off)] @ w[off]; x (B, Z, Y, X, Cin), zero padded."""
    B, Z, Y, X, _ = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (1, 1), (0, 0)))
    y = np.zeros((B, Z, Y, X, w.shape[2]))
    for off, dz, dy, dx in _offsets():
        y += _shift(xp, dz, dy, dx, Z, Y, X) @ w[off]
    return y


def conv3_input_grad(g, w):
    """dx[q] = sum_off g[q - d(off)] @ w[off]^T."""
    B, Z, Y, X, _ = g.shape
    gp = np.pad(g, ((0, 0), (1, 1), (1, 1), (1, 1), (0, 0)))
    dx_ = np.zeros((B, Z, Y, X, w.shape[1]))
    for off, dz, dy, dx in _offsets():
        dx_ += _shift(gp, -dz, -dy, -dx, Z, Y, X) @ w[off].T
    return dx_


def conv3_weight_grad(x, g):
    """dW[off] = sum_p x[p + d(off)]^T g[p]."""
    B, Z, Y, X, ci = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (1, 1), (0, 0)))
    dw = np.zeros((27, ci, g.shape[4]))
    g2 = g.reshape(-1, g.shape[4])
    for off, dz, dy, dx in _offsets():
        dw[off] = _shift(xp, dz, dy, dx, Z, Y, X).reshape(-1, ci).T @ g2
    return dw


def pool(x):
    B, Z, Y, X, C = x.shape
    return x.reshape(B, Z // 2, 2, Y // 2, 2, X // 2, 2, C).mean(axis=(2, 4, 6))


def pool_grad(g):
    return np.repeat(np.repeat(np.repeat(g, 2, 1), 2, 2), 2, 3) * 0.125


def up(x):
    return np.repeat(np.repeat(np.repeat(x, 2, 1), 2, 2), 2, 3)


def up_grad(g):
    B, Z, Y, X, C = g.shape
    return g.reshape(B, Z // 2, 2, Y // 2, 2, X // 2, 2, C).sum(axis=(2, 4, 6))


def interior_mask(res):
    X, Y, Z = res
    m = np.zeros((Z, Y, X))
    m[1:-1, 1:-1, 1:-1] = 1.0
    return m


def closed_box_operator(e, m):
    """A e on interior cells: (number of interior neighbours) * e minus the
    sum of the interior neighbours; e and the result are 0 outside the
    interior (m is the interior mask, shape (Z, Y, X))."""
    q = np.zeros_like(e)
    for ax in (1, 2, 3):
        for s in (1, -1):
            nb = np.roll(m, s, ax - 1)
            q += nb * (e - np.roll(e, s, ax))
    return q * m


class UNetOracle:
    def __init__(self, params, bf16=True):
        self.p = unpack(params)
        self.bf16 = bf16
        self.r = round_bf16 if bf16 else (lambda a: np.asarray(a, dtype=np.float64))
        self.w = {n: self.r(self.p[n + ".w"]) for n, _, _, _ in LAYERS}

    def _conv(self, name, x):
        return self.r(np.maximum(conv3(x, self.w[name]) + self.p[name + ".b"], 0.0))

    def forward(self, inp, res, batch):
        """inp: (batch, X*Y*Z) normalised right-hand sides in cell order."""
        X, Y, Z = res
        a = {}
        x = np.zeros((batch, Z, Y, X, 16))
        x[..., 0] = self.r(np.asarray(inp, dtype=np.float64).reshape(batch, Z, Y, X))
        a["x"] = x
        a["e1a"] = self._conv("e1a", x)
        a["e1b"] = self._conv("e1b", a["e1a"])
        a["p1"] = self.r(pool(a["e1b"]))
        a["e2a"] = self._conv("e2a", a["p1"])
        a["e2b"] = self._conv("e2b", a["e2a"])
        a["p2"] = self.r(pool(a["e2b"]))
        a["b3a"] = self._conv("b3a", a["p2"])
        a["b3b"] = self._conv("b3b", a["b3a"])
        a["cat2"] = np.concatenate([up(a["b3b"]), a["e2b"]], axis=-1)
        a["d2a"] = self._conv("d2a", a["cat2"])
        a["d2b"] = self._conv("d2b", a["d2a"])
        a["cat1"] = np.concatenate([up(a["d2b"]), a["e1b"]], axis=-1)
        a["d1a"] = self._conv("d1a", a["cat1"])
        a["d1b"] = self._conv("d1b", a["d1a"])
        y = a["d1b"] @ self.p["out.w"] + self.p["out.b"]
        if self.bf16:
            y = y.astype(np.float32).astype(np.float64)
        a["y"] = y
        return y.reshape(batch, -1), a

    def loss_grad(self, inp, tgt, res, batch, loss="mse"):
        """loss "mse": mean of e^2; "energy": mean of e (A e) + 1e-4 e^2 with A
        the closed-box 7-point operator on interior cells (e = y - t)."""
        X, Y, Z = res
        y, a = self.forward(inp, res, batch)
        t = np.asarray(tgt, dtype=np.float64).reshape(batch, Z, Y, X)
        m = interior_mask(res)
        count = batch * (X - 2) * (Y - 2) * (Z - 2)
        e = (a["y"] - t) * m
        if loss == "energy":
            if self.bf16:  # the GPU forms e and A e in FP32
                e = e.astype(np.float32).astype(np.float64)
            ae = closed_box_operator(e, m)
            w = 1e-4
            loss = float((e * ae + w * e * e).sum() / count)
            gy = 2.0 * (ae + w * e) / count
        else:
            loss = float((e * e).sum() / count)
            gy = 2.0 * e / count
        r, w, g = self.r, self.w, {}
        relu_mask = lambda act: (act > 0).astype(np.float64)

        def layer(name, xin, gout):
            g[name + ".w"] = conv3_weight_grad(xin, gout)
            g[name + ".b"] = gout.sum(axis=(0, 1, 2, 3))

        g["out.w"] = (a["d1b"] * gy[..., None]).sum(axis=(0, 1, 2, 3))
        g["out.b"] = gy.sum()
        g_d1b = r(relu_mask(a["d1b"]) * (gy[..., None] * self.p["out.w"]))
        layer("d1b", a["d1a"], g_d1b)
        g_d1a = r(relu_mask(a["d1a"]) * conv3_input_grad(g_d1b, w["d1b"]))
        layer("d1a", a["cat1"], g_d1a)
        g_cat1 = r(conv3_input_grad(g_d1a, w["d1a"]))
        g_d2b = r(relu_mask(a["d2b"]) * up_grad(g_cat1[..., :32]))
        layer("d2b", a["d2a"], g_d2b)
        g_d2a = r(relu_mask(a["d2a"]) * conv3_input_grad(g_d2b, w["d2b"]))
        layer("d2a", a["cat2"], g_d2a)
        g_cat2 = r(conv3_input_grad(g_d2a, w["d2a"]))
        g_b3b = r(relu_mask(a["b3b"]) * up_grad(g_cat2[..., :64]))
        layer("b3b", a["b3a"], g_b3b)
        g_b3a = r(relu_mask(a["b3a"]) * conv3_input_grad(g_b3b, w["b3b"]))
        layer("b3a", a["p2"], g_b3a)
        g_p2 = r(conv3_input_grad(g_b3a, w["b3a"]))
        g_e2b = r(relu_mask(a["e2b"]) * (pool_grad(g_p2) + g_cat2[..., 64:]))
        layer("e2b", a["e2a"], g_e2b)
        g_e2a = r(relu_mask(a["e2a"]) * conv3_input_grad(g_e2b, w["e2b"]))
        layer("e2a", a["p1"], g_e2a)
        g_p1 = r(conv3_input_grad(g_e2a, w["e2a"]))
        g_e1b = r(relu_mask(a["e1b"]) * (pool_grad(g_p1) + g_cat1[..., 32:]))
        layer("e1b", a["e1a"], g_e1b)
        g_e1a = r(relu_mask(a["e1a"]) * conv3_input_grad(g_e1b, w["e1b"]))
        layer("e1a", a["x"], g_e1a)
        return loss, pack(g)
