"""FP64 numpy restatement of the warm-start MLP (forward and backward).

TEST INFRASTRUCTURE: the checker of the GPU training kernels' gradients
(tests/). Parameter layout as hz_mlp_train_step: W1[32][64], b1[64],
W2[64][64], b2[64], W3[64], b3; ReLU hidden layers; loss = mean((y - t)^2).

``forward`` / ``loss_and_grad`` are the exact network in FP64.
``forward_bf16`` / ``loss_and_grad_bf16`` restate the GPU kernels' mixed
precision (csrc/hz_learn.cu): weights and biases rounded to BF16 (pass
``bf16_round(p)``), the inputs X and the first hidden layer's activations
rounded to BF16 before their products, and in the backward pass G2 =
dL/da2 and G1 = dL/da1 rounded to BF16 before the products G2 W2^T, H1^T G2
and X^T G1; every sum is taken in FP64 here (FP32 on the GPU).
"""
import numpy as np

N_IN, N_HID = 32, 64
N_PARAMS = N_IN * N_HID + N_HID + N_HID * N_HID + N_HID + N_HID + 1


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + N_IN * N_HID].reshape(N_IN, N_HID); o += N_IN * N_HID
    b1 = p[o:o + N_HID]; o += N_HID
    W2 = p[o:o + N_HID * N_HID].reshape(N_HID, N_HID); o += N_HID * N_HID
    b2 = p[o:o + N_HID]; o += N_HID
    W3 = p[o:o + N_HID]; o += N_HID
    b3 = p[o]
    return W1, b1, W2, b2, W3, b3


def bf16_round(x):
    """Round-to-nearest-even to bfloat16, returned as float32 values."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    rounding = ((u >> 16) & 1) + 0x7FFF
    u = ((u + rounding) >> 16) << 16
    return u.astype(np.uint32).view(np.float32)


def forward(p, X):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    a1 = X @ W1 + b1
    h1 = np.maximum(a1, 0.0)
    a2 = h1 @ W2 + b2
    h2 = np.maximum(a2, 0.0)
    y = h2 @ W3 + b3
    return y, (X, a1, h1, a2, h2)


def loss_and_grad(p, X, T):
    """Mean squared error and its gradient w.r.t. the packed parameters."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    y, (X, a1, h1, a2, h2) = forward(p, X)
    n = X.shape[0]
    d = y - np.asarray(T, dtype=np.float64)
    loss = np.mean(d * d)
    g = 2.0 * d / n
    gW3 = h2.T @ g
    gb3 = g.sum()
    g2 = np.outer(g, W3) * (a2 > 0)
    gW2 = h1.T @ g2
    gb2 = g2.sum(0)
    g1 = (g2 @ W2.T) * (a1 > 0)
    gW1 = X.T @ g1
    gb1 = g1.sum(0)
    grad = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3, [gb3]])
    return loss, grad


def _bf16_64(x):
    """BF16 rounding of FP64 values through FP32, as the GPU rounds its FP32
    intermediates."""
    return bf16_round(np.asarray(x, dtype=np.float64).astype(np.float32)).astype(np.float64)


def forward_bf16(p, X):
    """The GPU forward pass: y and the intermediates (Xb, a1, h1b, a2, h2)."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    Xb = _bf16_64(X)
    a1 = Xb @ W1 + b1
    h1b = _bf16_64(np.maximum(a1, 0.0))
    a2 = h1b @ W2 + b2
    h2 = np.maximum(a2, 0.0)
    y = h2 @ W3 + b3
    return y, (Xb, a1, h1b, a2, h2)


def loss_and_grad_bf16(p, X, T):
    """Mean squared error and the gradient the GPU training kernel computes."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    y, (Xb, a1, h1b, a2, h2) = forward_bf16(p, X)
    n = Xb.shape[0]
    d = y - np.asarray(T, dtype=np.float64)
    loss = np.mean(d * d)
    g = 2.0 * d / n
    gW3 = h2.T @ g
    gb3 = g.sum()
    G2 = np.outer(g, W3) * (a2 > 0)
    gb2 = G2.sum(0)
    G2b = _bf16_64(G2)
    gW2 = h1b.T @ G2b
    G1 = (G2b @ W2.T) * (h1b > 0)
    gb1 = G1.sum(0)
    gW1 = Xb.T @ _bf16_64(G1)
    grad = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3, [gb3]])
    return loss, grad
