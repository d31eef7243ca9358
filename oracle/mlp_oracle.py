"""CPU oracle of the rank predictor's network (test infrastructure only).

The reference has no learned component; this restates the network the GPU
kernels implement (a 3-layer perceptron of width 128 with ReLU, BF16 weights
and activations, FP32 arithmetic) together with its mean-squared-error
gradient (backpropagation) and the Adam update of Kingma & Ba (2015,
"Adam: a method for stochastic optimization", Algorithm 1 with bias
correction).  Only the tests and the CPU checks may import it.

Parameter vector layout: W1[128 x nin] b1[128] W2[128 x 128] b2[128] w3[128] b3[1].
"""
import numpy as np

H = 128


def num_params(nin):
    return H * nin + H + H * H + H + H + 1


def unpack(theta, nin):
    o = 0
    W1 = theta[o:o + H * nin].reshape(H, nin)
    o += H * nin
    b1 = theta[o:o + H]
    o += H
    W2 = theta[o:o + H * H].reshape(H, H)
    o += H * H
    b2 = theta[o:o + H]
    o += H
    w3 = theta[o:o + H]
    o += H
    b3 = theta[o:o + 1]
    return W1, b1, W2, b2, w3, b3


def bf16_round(a):
    """Round FP32 values to the nearest BF16 (ties to even), returned as FP32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def forward(theta16, X16, nin, bf16=True, dtype=np.float64):
    """Activations of the network.  With ``bf16`` the hidden activations are
    rounded to BF16 after the ReLU, as the kernels store them."""
    W1, b1, W2, b2, w3, b3 = (p.astype(dtype) for p in unpack(theta16, nin))
    X = X16.astype(dtype)
    rnd = (lambda v: bf16_round(v).astype(dtype)) if bf16 else (lambda v: v)
    h1 = rnd(np.maximum(X @ W1.T + b1, 0))
    h2 = rnd(np.maximum(h1 @ W2.T + b2, 0))
    y = h2 @ w3 + b3[0]
    return X, h1, h2, y


def loss_and_grad(theta16, X16, t, nin, bf16=True, dtype=np.float64):
    """Mean squared error and its gradient w.r.t. the parameter vector
    (evaluated at the BF16 parameters, through the stored activations)."""
    W1, b1, W2, b2, w3, b3 = (p.astype(dtype) for p in unpack(theta16, nin))
    X, h1, h2, y = forward(theta16, X16, nin, bf16, dtype)
    n = X.shape[0]
    e = y - t.astype(dtype)
    loss = float(np.mean(e * e))
    dy = 2.0 * e / n
    gw3 = h2.T @ dy
    gb3 = np.array([dy.sum()])
    d2 = np.outer(dy, w3) * (h2 > 0)
    gW2 = d2.T @ h1
    gb2 = d2.sum(0)
    d1 = (d2 @ W2) * (h1 > 0)
    gW1 = d1.T @ X
    gb1 = d1.sum(0)
    g = np.concatenate((gW1.ravel(), gb1, gW2.ravel(), gb2, gw3, gb3))
    return loss, g


def adam_step(theta, m, v, g, step, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One bias-corrected Adam step (FP32 state), in place; returns theta."""
    m[:] = beta1 * m + (1 - beta1) * g
    v[:] = beta2 * v + (1 - beta2) * g * g
    mh = m / (1 - beta1 ** step)
    vh = v / (1 - beta2 ** step)
    theta -= lr * mh / (np.sqrt(vh) + eps)
    return theta
