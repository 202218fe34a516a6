"""FP64 restatement of the learned proposal -- TEST INFRASTRUCTURE.

The reference has no learned proposal (this component is this project's own); this
module is the checker for the CUDA kernels in annongpu_gb300/csrc/made.cu:

* MADE (Germain, Gregor, Murray, Larochelle, "MADE: Masked Autoencoder for
  Distribution Estimation", ICML 2015) with one hidden layer of width H over N
  spins, natural ordering: hidden unit k has degree d_k in [1, N-1]; input i feeds
  unit k iff i < d_k; unit k feeds output j iff d_k <= j. x_i = 1 for spin up.
      pre = W1 x + b1,  h = relu(pre),  l = W2 h + b2
      log q(s) = sum_j x_j log sigmoid(l_j) + (1 - x_j) log sigmoid(-l_j)
* training loss: mean over the batch of -log q(s); its gradient by backpropagation.
* Adam (Kingma & Ba, 2015) with bias correction.
* autoregressive sampling: x_j = 1 iff u_j < sigmoid(l_j(x_<j)).
Weights are passed as the BF16-rounded values the GPU computes with.
"""

import numpy as np


def degrees(N, H):
    """Hidden-unit degrees: cycle through 1..N-1 (deterministic)."""
    return (np.arange(H) % max(1, N - 1)) + 1


def masks(N, H):
    d = degrees(N, H)
    m1 = (np.arange(N)[None, :] < d[:, None]).astype(np.float64)      # H x N
    m2 = (d[None, :] <= np.arange(N)[:, None]).astype(np.float64)     # N x H
    return m1, m2


def bits(confs, N):
    confs = np.asarray(confs, dtype=np.uint64).reshape(-1)
    return ((confs[:, None] >> np.arange(N, dtype=np.uint64)[None, :]) & np.uint64(1)).astype(np.float64)


def softplus(z):
    return np.logaddexp(0.0, z)


def forward(x, W1, b1, W2, b2):
    pre = x @ W1.T + b1
    h = np.maximum(pre, 0.0)
    l = h @ W2.T + b2
    logq = -(x * softplus(-l) + (1 - x) * softplus(l)).sum(axis=1)
    return pre, h, l, logq


def log_prob(confs, N, W1, b1, W2, b2):
    return forward(bits(confs, N), W1, b1, W2, b2)[3]


def loss_and_grad(confs, N, W1, b1, W2, b2):
    x = bits(confs, N)
    B = x.shape[0]
    pre, h, l, logq = forward(x, W1, b1, W2, b2)
    loss = -logq.mean()
    dl = (1.0 / (1.0 + np.exp(-l)) - x) / B          # d loss / d logits
    m1, m2 = masks(N, W1.shape[0])
    dW2 = (dl.T @ h) * m2
    db2 = dl.sum(axis=0)
    dh = (dl @ W2) * (pre > 0)
    dW1 = (dh.T @ x) * m1
    db1 = dh.sum(axis=0)
    return loss, dW1, db1, dW2, db2


def adam(p, g, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** t)
    vh = v / (1 - b2 ** t)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v


def sample(u, N, W1, b1, W2, b2):
    """u: (B, N) uniforms; returns configurations (uint64) and log q."""
    B = u.shape[0]
    x = np.zeros((B, N))
    for j in range(N):
        _, _, l, _ = forward(x, W1, b1, W2, b2)
        x[:, j] = (u[:, j] < 1.0 / (1.0 + np.exp(-l[:, j]))).astype(np.float64)
    confs = (x.astype(np.uint64) << np.arange(N, dtype=np.uint64)[None, :]).sum(axis=1).astype(np.uint64)
    return confs, forward(x, W1, b1, W2, b2)[3]


def bf16_round(a):
    """Round float32 values to bfloat16 (round to nearest even) and back."""
    f = np.asarray(a, np.float32).copy()
    u = f.view(np.uint32)
    r = ((u >> 16) & 1) + np.uint32(0x7FFF)
    u = (u + r) & np.uint32(0xFFFF0000)
    return u.view(np.float32).astype(np.float64)
