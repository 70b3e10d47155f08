"""Float64 numpy restatement of the selector network (test infrastructure only).

Same flat parameter layout and loss as hyset_gb300/csrc/mlp.cu:
W1[12][64] b1[64] W2[64][64] b2[64] W3[64][3] b3[3]; ReLU hidden layers;
loss = sum(mask * (y - t)^2) / sum(mask).  Used to check the GPU kernels'
forward pass and gradients."""
import numpy as np

F, H, O = 12, 64, 3


def unpack(p):
    p = np.asarray(p, np.float64)
    o = 0
    out = []
    for shape in ((F, H), (H,), (H, H), (H,), (H, O), (O,)):
        size = int(np.prod(shape))
        out.append(p[o:o + size].reshape(shape))
        o += size
    assert o == p.size
    return out


def forward(p, x):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    x = np.asarray(x, np.float64)
    z1 = x @ W1 + b1
    h1 = np.maximum(z1, 0)
    z2 = h1 @ W2 + b2
    h2 = np.maximum(z2, 0)
    return h2 @ W3 + b3, (x, z1, h1, z2, h2)


def loss_grad(p, x, t, m):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    y, (x, z1, h1, z2, h2) = forward(p, x)
    t = np.asarray(t, np.float64)
    m = np.asarray(m, np.float64)
    denom = m.sum()
    loss = float((m * (y - t) ** 2).sum() / denom)
    dy = 2.0 * m * (y - t) / denom
    gW3, gb3 = h2.T @ dy, dy.sum(0)
    d2 = (dy @ W3.T) * (z2 > 0)
    gW2, gb2 = h1.T @ d2, d2.sum(0)
    d1 = (d2 @ W2.T) * (z1 > 0)
    gW1, gb1 = x.T @ d1, d1.sum(0)
    g = np.concatenate([a.ravel() for a in (gW1, gb1, gW2, gb2, gW3, gb3)])
    return loss, g
