"""Initial-network constructors with the reference's signatures
(pyANNonGPU/new_RBM.py:14-29, pyANNonGPU/new_neural_network.py:31-131).

Initialisation: identity-like couplings of strength ``initial_value`` plus
uniform noise in [-noise, noise] (real and imaginary parts), final weights
``final_weight(s)``. ``rng`` (numpy Generator) makes them reproducible.
"""

import math

import numpy as np

from .api import PsiCNN, PsiDeep, PsiRBM


def _noise(rng, shape, scale, complex_=True):
    r = 2 * rng.random(shape) - 1
    if complex_:
        r = r + 1j * (2 * rng.random(shape) - 1)
    return scale * r


def new_RBM(N, M, initial_value=(0.01 + 1j * math.pi / 4), noise=1e-4, gpu=True, final_weight=10, rng=None,
            **kwargs):
    if M < N:
        raise ValueError("new_RBM needs M >= N")
    rng = np.random.default_rng() if rng is None else rng
    W = _noise(rng, (N, M), noise)
    for k in range(M // N):
        W[:, k * N:(k + 1) * N] += initial_value * np.eye(N)
    return PsiRBM(W, final_weight, 0.0, gpu, **kwargs)


def _block_offset(n, m, c):
    # stride between the windows of consecutive hidden units
    if m > n:
        return 1
    if n % m == 0:
        return n // m
    return c


def new_deep_neural_network(num_sites, N, M, C, initial_value=(0.01 + 1j * math.pi / 4), a=0, noise=1e-4,
                            gpu=True, noise_modulation="auto", final_weights=10, rng=None, **kwargs):
    """One hidden layer: M = [m], C = [c]; hidden unit j connects to sites (j * delta + i) % N, i < c."""
    if not isinstance(M, (list, tuple)):
        M, C = [M], [C]
    if len(M) != 1:
        raise NotImplementedError("this build supports PsiDeep with one hidden layer")
    if isinstance(N, (list, tuple)):
        raise NotImplementedError("multi-dimensional PsiDeep layouts are not built")
    m, c = M[0], C[0]
    if (m * c) % N != 0 or c > N:
        raise ValueError("need (M * C) % N == 0 and C <= N")
    rng = np.random.default_rng() if rng is None else rng
    a = np.full(N, a, dtype=np.complex128) if np.isscalar(a) else np.asarray(a, np.complex128)
    is_real = complex(initial_value).imag == 0
    b = _noise(rng, m, noise, not is_real)
    w = _noise(rng, (c, m), noise, not is_real)
    w[c // 2, :] += initial_value
    delta = _block_offset(N, m, c)
    conn = np.array([[(j * delta + i) % N for j in range(m)] for i in range(c)], np.uint32)
    fw = final_weights * np.ones(m) if np.isscalar(final_weights) else np.asarray(final_weights)
    return PsiDeep(num_sites, a, [b], [conn], [w], fw, 0.0, gpu, **kwargs)


def new_convolutional_network(L, layers, initial_value=(0.01 + 1j * math.pi / 4), noise=1e-4, final_factor=10,
                              symmetry_classes=None, real=False, gpu=True, rng=None, **kwargs):
    """``layers`` = [(channels, connectivity), ...]; kernels start as noise, the first
    layer with ``initial_value`` at the window centre, deeper layers with a Glorot-scaled
    real uniform part (pyANNonGPU/new_convolutional_network.py:30-82)."""
    rng = np.random.default_rng() if rng is None else rng
    L = list(L) if isinstance(L, (list, tuple)) else [L]
    channels = [c for c, _ in layers]
    conns = [list(k) if isinstance(k, (list, tuple)) else [k] for _, k in layers]
    n_sites = int(np.prod(L))
    symmetry_classes = np.zeros(n_sites, np.uint32) if symmetry_classes is None else np.asarray(symmetry_classes)
    ncls = len(set(np.asarray(symmetry_classes).tolist()))
    params = []
    for layer, (ch, conn) in enumerate(zip(channels, conns)):
        vol = int(np.prod(conn))
        prev = channels[layer - 1] if layer else 1
        for _ in range(ch * prev):
            for _ in range(ncls):
                w = _noise(rng, vol, noise, not real)
                if layer == 0:
                    w[vol // 2] = initial_value.real if real else initial_value
                else:
                    w = w + math.sqrt(6 / (vol * prev + vol * ch)) * (2 * rng.random(vol) - 1)
                params.extend(w)
    return PsiCNN(L, channels, conns, symmetry_classes, np.array(params), final_factor, 0.0, gpu, **kwargs)
