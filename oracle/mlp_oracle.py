"""CPU oracle of the learned predictor's network (TEST INFRASTRUCTURE ONLY).

A numpy restatement of the 8 -> 64 -> 64 -> 64 -> 3 GELU MLP of the library
(csrc/mlp.cuh): forward pass, training loss and its gradient.  Two modes:
  * bf16=True mirrors where the GPU kernels round to BF16 (weights, the
    normalised input, every hidden activation, and the output / hidden
    gradients that enter a matrix product), accumulating in FP64;
  * bf16=False is plain FP64, which the tests check against central finite
    differences to pin the backward formulas themselves.
Only tests/ use this module; the product never imports it.
"""
import numpy as np

IN, HID, OUT = 8, 64, 3
OFF_W1 = 0
OFF_B1 = OFF_W1 + IN * HID
OFF_W2 = OFF_B1 + HID
OFF_B2 = OFF_W2 + HID * HID
OFF_W3 = OFF_B2 + HID
OFF_B3 = OFF_W3 + HID * HID
OFF_W4 = OFF_B3 + HID
OFF_B4 = OFF_W4 + HID * OUT
NPARAM = OFF_B4 + OUT
OFF_XMEAN, OFF_XSCALE = NPARAM, NPARAM + IN
OFF_YMEAN, OFF_YSCALE = NPARAM + 2 * IN, NPARAM + 2 * IN + 1
OFF_CMEAN, OFF_CSCALE = OFF_YSCALE + 1, OFF_YSCALE + 2
NET_FLOATS = OFF_CSCALE + 1
C_GELU = 0.7978845608028654  # sqrt(2 / pi)


def bf16(a):
    """Round to BF16 (round to nearest even), returned as float32."""
    a = np.ascontiguousarray(a, np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def gelu(z):
    return 0.5 * z * (1.0 + np.tanh(C_GELU * (z + 0.044715 * z ** 3)))


def gelu_grad(z):
    th = np.tanh(C_GELU * (z + 0.044715 * z ** 3))
    return 0.5 * (1.0 + th) + 0.5 * z * (1.0 - th * th) * C_GELU * (1.0 + 3 * 0.044715 * z * z)


def unpack(net):
    net = np.asarray(net, np.float64)
    return dict(W1=net[OFF_W1:OFF_B1].reshape(IN, HID), b1=net[OFF_B1:OFF_W2],
                W2=net[OFF_W2:OFF_B2].reshape(HID, HID), b2=net[OFF_B2:OFF_W3],
                W3=net[OFF_W3:OFF_B3].reshape(HID, HID), b3=net[OFF_B3:OFF_W4],
                W4=net[OFF_W4:OFF_B4].reshape(HID, OUT), b4=net[OFF_B4:NPARAM],
                xmean=net[OFF_XMEAN:OFF_XSCALE], xscale=net[OFF_XSCALE:OFF_YMEAN],
                ymean=net[OFF_YMEAN], yscale=net[OFF_YSCALE],
                cmean=net[OFF_CMEAN], cscale=net[OFF_CSCALE])


def forward(net, x, bf=True):
    """Returns y[n][3] and the saved activations."""
    P = unpack(net)
    r = bf16 if bf else (lambda a: np.asarray(a, np.float64))
    xn = r((np.asarray(x, np.float32) - P["xmean"].astype(np.float32)) *
           P["xscale"].astype(np.float32)).astype(np.float64)
    W = [r(P[k]).astype(np.float64) for k in ("W1", "W2", "W3", "W4")]
    z1 = xn @ W[0] + P["b1"]
    h1 = r(gelu(z1)).astype(np.float64)
    z2 = h1 @ W[1] + P["b2"]
    h2 = r(gelu(z2)).astype(np.float64)
    z3 = h2 @ W[2] + P["b3"]
    h3 = r(gelu(z3)).astype(np.float64)
    y = h3 @ W[3] + P["b4"]
    return y, dict(xn=xn, W=W, z=(z1, z2, z3), h=(h1, h2, h3))


def loss_and_grad(net, x, t, bf=True):
    """Mean loss over the batch and its gradient w.r.t. the NPARAM weights.
    t[n][3]: log10 first accepted dt (squared error on the normalised value),
    stiff label (binary cross-entropy on the logit), log2 attempted steps
    (squared error on the normalised value); NaN = no label."""
    P = unpack(net)
    r = bf16 if bf else (lambda a: np.asarray(a, np.float64))
    y, S = forward(net, x, bf)
    n = y.shape[0]
    t = np.asarray(t, np.float64)
    m0, m1, m2 = ~np.isnan(t[:, 0]), ~np.isnan(t[:, 1]), ~np.isnan(t[:, 2])
    tn = np.where(m0, (t[:, 0] - P["ymean"]) / P["yscale"], 0.0)
    t1 = np.where(m1, t[:, 1], 0.0)
    cn = np.where(m2, (t[:, 2] - P["cmean"]) / P["cscale"], 0.0)
    y0, y1, y2 = y[:, 0], y[:, 1], y[:, 2]
    loss = np.sum(np.where(m0, (y0 - tn) ** 2, 0.0))
    loss += np.sum(np.where(m1, np.maximum(y1, 0) + np.log1p(np.exp(-np.abs(y1))) - t1 * y1, 0.0))
    loss += np.sum(np.where(m2, (y2 - cn) ** 2, 0.0))
    loss /= n
    dy = np.zeros_like(y)
    dy[:, 0] = np.where(m0, 2 * (y0 - tn), 0.0) / n
    dy[:, 1] = np.where(m1, 1 / (1 + np.exp(-y1)) - t1, 0.0) / n
    dy[:, 2] = np.where(m2, 2 * (y2 - cn), 0.0) / n
    g = np.zeros(NPARAM)
    dyb = r(dy).astype(np.float64)
    z1, z2, z3 = S["z"]
    h1, h2, h3 = S["h"]
    W1, W2, W3, W4 = S["W"]
    g[OFF_W4:OFF_B4] = (h3.T @ dyb).ravel()
    g[OFF_B4:NPARAM] = dy.sum(0)
    dz3 = (dyb @ W4.T) * gelu_grad(z3)
    dz3b = r(dz3).astype(np.float64)
    g[OFF_B3:OFF_W4] = dz3.sum(0)
    g[OFF_W3:OFF_B3] = (h2.T @ dz3b).ravel()
    dz2 = (dz3b @ W3.T) * gelu_grad(z2)
    dz2b = r(dz2).astype(np.float64)
    g[OFF_B2:OFF_W3] = dz2.sum(0)
    g[OFF_W2:OFF_B2] = (h1.T @ dz2b).ravel()
    dz1 = (dz2b @ W2.T) * gelu_grad(z1)
    dz1b = r(dz1).astype(np.float64)
    g[OFF_B1:OFF_W2] = dz1.sum(0)
    g[OFF_W1:OFF_B1] = (S["xn"].T @ dz1b).ravel()
    return loss, g
