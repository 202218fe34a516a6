"""Initial-network constructors with the reference's signatures
(pyANNonGPU/new_RBM.py:14-29, pyANNonGPU/new_neural_network.py:31-131).

Initialisation: identity-like couplings of strength ``initial_value`` plus
uniform noise in [-noise, noise] (real and imaginary parts), final weights
``final_weight(s)``. ``rng`` (numpy Generator) makes them reproducible.
"""

import math

import numpy as np

from .api import (PsiCNN, PsiClassicalANN_1, PsiClassicalANN_2, PsiClassicalFP_1, PsiClassicalFP_2, PsiDeep,
                  PsiFullyPolarized, PsiRBM)
from .expression import PauliExpression


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
    # stride between the windows of consecutive units of a layer
    if m > n:
        return 1
    if n % m == 0:
        return n // m
    return c


def _layer_connections(n, m, c):
    """Connection block (C x M) of a layer over a lattice of shape n (1 to 3 dimensions):
    unit j (multi-index j_ids over m) reads units (j_d * delta_d + i_d) % n_d for every
    window multi-index i_ids over c, flattened row-major."""
    n, m, c = [list(x) for x in (n, m, c)]
    deltas = [_block_offset(n_, m_, c_) for n_, m_, c_ in zip(n, m, c)]
    strides = [int(np.prod(n[d + 1:])) for d in range(len(n))]
    rows = []
    for i_ids in np.ndindex(*c):
        rows.append([sum(((jd * dd + idd) % nd) * sd for jd, dd, idd, nd, sd in zip(j_ids, deltas, i_ids, n, strides))
                     for j_ids in np.ndindex(*m)])
    return np.array(rows, np.uint32)


def new_deep_neural_network(num_sites, N, M, C, initial_value=(0.01 + 1j * math.pi / 4), a=0, noise=1e-4,
                            gpu=True, noise_modulation="auto", final_weights=10, rng=None, **kwargs):
    """PsiDeep with len(M) hidden layers (pyANNonGPU/new_neural_network.py:31-131).

    N, and each entry of M and C, is an int (1-d chain of units) or a 2-/3-tuple
    (lattice of units, flattened row-major). Layer k has M[k] units; each reads a window
    of C[k] units of the layer below, windows spaced as the reference spaces them. The
    first layer's weights are noise plus ``initial_value`` on the window centre row;
    deeper layers are a real Glorot-uniform term of scale sqrt(6 / (C_k + C_{k+1})) plus
    noise. Biases are noise; ``final_weights`` a scalar or one value per last-layer unit.
    As in the reference, an explicit ``noise_modulation`` list only bounds the number of
    deeper layers built; their scale is the Glorot one.
    """
    rng = np.random.default_rng() if rng is None else rng
    dim = len(N) if isinstance(N, (list, tuple)) else 1
    if not isinstance(M, (list, tuple)) or (dim > 1 and not isinstance(M[0], (list, tuple))):
        M, C = [M], [C]
    M, C = list(M), list(C)
    as_shape = (lambda x: [int(x)]) if dim == 1 else (lambda x: [int(v) for v in x])
    shapes = [as_shape(N)] + [as_shape(m) for m in M]
    windows = [as_shape(c) for c in C]
    for n, m, c in zip(shapes[:-1], shapes[1:], windows):
        for nd, md, cd in zip(n, m, c):
            if (md * cd) % nd != 0 or cd > nd:
                raise ValueError("every layer needs (M * C) % N == 0 and C <= N in each dimension")
    N_lin = int(np.prod(shapes[0]))
    M_lin = [int(np.prod(m)) for m in shapes[1:]]
    C_lin = [int(np.prod(c)) for c in windows]
    a = np.full(N_lin, a, dtype=np.complex128) if np.isscalar(a) else np.asarray(a, np.complex128)
    is_real = complex(initial_value).imag == 0
    b = [_noise(rng, m, noise, not is_real) for m in M_lin]
    w0 = _noise(rng, (C_lin[0], M_lin[0]), noise, not is_real)
    w0[C_lin[0] // 2, :] += initial_value
    W = [w0]
    nexts = C_lin[2:] + [1]
    if noise_modulation == "auto":
        noise_modulation = [math.sqrt(6 / (c + nc)) for c, nc in zip(C_lin[1:], nexts)]
    for c, m, nc, _ in zip(C_lin[1:], M_lin[1:], nexts, noise_modulation):
        W.append(math.sqrt(6 / (c + nc)) * (2 * rng.random((c, m)) - 1) + _noise(rng, (c, m), noise, not is_real))
    if len(W) < len(M_lin):
        raise ValueError("noise_modulation has fewer entries than deeper layers")
    conns = [_layer_connections(n, m, c) for n, m, c in zip(shapes[:-1], shapes[1:], windows)]
    fw = final_weights * np.ones(M_lin[-1]) if np.isscalar(final_weights) else np.asarray(final_weights)
    if fw.size != M_lin[-1]:
        raise ValueError("final_weights needs one entry per unit of the last layer")
    return PsiDeep(num_sites, a, b, conns, W, fw, 0.0, gpu, **kwargs)


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


def new_classical_network(num_sites, order, H_local, symmetric=False, distance="max", params=0,
                          psi_ref="fully polarized", use_super_operator=False, gpu=True, **kwargs):
    """Classical network (pyANNonGPU/new_classical_network.py:6-66): one parameter per operator
    of ``H_local`` (a list, or a Pauli expression whose terms become the operators), zero
    initial parameters, log_prefactor log(2^(-N/2)) over the fully polarized reference or 0 over
    a PsiDeep reference (copied; its parameters join the variational ones at order 2)."""
    if order not in (1, 2):
        raise ValueError("order must be 1 or 2")
    if symmetric or use_super_operator:
        raise NotImplementedError("symmetric classical networks and super-operator features are not built")
    if isinstance(H_local, PauliExpression):
        H_local = [PauliExpression({k: c}) for k, c in H_local.terms.items()]
    H_local = list(H_local)
    if isinstance(params, (int, float)) and params == 0:
        params = np.zeros(len(H_local), dtype=complex)
    if isinstance(psi_ref, str):
        lp = math.log(1 / 2 ** (num_sites / 2))
        cls = PsiClassicalFP_1 if order == 1 else PsiClassicalFP_2
        return cls(num_sites, H_local, params, PsiFullyPolarized(num_sites, lp), lp, gpu, **kwargs)
    cls = PsiClassicalANN_1 if order == 1 else PsiClassicalANN_2
    return cls(num_sites, H_local, params, psi_ref, 0.0, gpu, **kwargs)

