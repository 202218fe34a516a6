"""Pauli-sum expressions: the (a, b, coefficient) triples an ``Operator`` is built from.

The reference builds its ``Operator`` from a ``QuantumExpression.PauliExpression``
(source/operator/Operator.cpp:18-39) and reads exactly ``(term.first.a,
term.first.b, term.second)`` from every term. That package is a separate,
unvendored dependency, so this module provides a minimal compatible builder:
``sigma_x/sigma_y/sigma_z`` terms with ``+``, ``-``, ``*`` and scalar factors.

Per-site encoding (include/basis/PauliString.hpp:37-56):
(a, b) = (0, 0) identity, (1, 0) sigma_x, (0, 1) sigma_y, (1, 1) sigma_z.
Site products follow the Pauli algebra sigma_i sigma_j = delta_ij + i eps_ijk sigma_k.

``matrix(num_sites)`` returns the dense matrix whose action matches the
reference's ``PauliString::apply`` (PauliString.hpp:242-254), so
``vdot(psi, H.matrix(N) @ psi)`` is the exact-summation expectation value.
"""

from __future__ import annotations

import numbers

import numpy as np

__all__ = [
    "PauliExpression", "sigma_x", "sigma_y", "sigma_z", "identity",
    "transverse_field_ising_1d", "transverse_field_ising_2d", "heisenberg_j1j2_2d",
    "square_lattice_bonds",
]

# single-site products: (p, q) -> (phase, r) with sigma_p sigma_q = phase * sigma_r
# types: 0 = I, 1 = X, 2 = Y, 3 = Z
_PRODUCT = {}
for _p in range(4):
    _PRODUCT[(0, _p)] = (1, _p)
    _PRODUCT[(_p, 0)] = (1, _p)
for _p in (1, 2, 3):
    _PRODUCT[(_p, _p)] = (1, 0)
_PRODUCT[(1, 2)] = (1j, 3)
_PRODUCT[(2, 1)] = (-1j, 3)
_PRODUCT[(2, 3)] = (1j, 1)
_PRODUCT[(3, 2)] = (-1j, 1)
_PRODUCT[(3, 1)] = (1j, 2)
_PRODUCT[(1, 3)] = (-1j, 2)

_TYPE_TO_AB = {0: (0, 0), 1: (1, 0), 2: (0, 1), 3: (1, 1)}


def _site_type(a: int, b: int, i: int) -> int:
    ai = (a >> i) & 1
    bi = (b >> i) & 1
    return {(0, 0): 0, (1, 0): 1, (0, 1): 2, (1, 1): 3}[(ai, bi)]


class PauliExpression:
    """A sum of Pauli strings with complex coefficients, keyed by (a, b) bit masks."""

    def __init__(self, terms=None):
        self.terms: dict[tuple[int, int], complex] = {}
        if terms:
            for key, c in terms.items():
                if c != 0:
                    self.terms[key] = self.terms.get(key, 0) + complex(c)

    # -- algebra -----------------------------------------------------------------
    @staticmethod
    def _coerce(x) -> "PauliExpression":
        if isinstance(x, PauliExpression):
            return x
        if isinstance(x, numbers.Number):
            return PauliExpression({(0, 0): complex(x)})
        raise TypeError(f"cannot combine PauliExpression with {type(x)!r}")

    def __add__(self, other):
        other = self._coerce(other)
        out = PauliExpression(self.terms)
        for k, c in other.terms.items():
            out.terms[k] = out.terms.get(k, 0) + c
        out.terms = {k: c for k, c in out.terms.items() if c != 0}
        return out

    __radd__ = __add__

    def __neg__(self):
        return PauliExpression({k: -c for k, c in self.terms.items()})

    def __sub__(self, other):
        return self + (-self._coerce(other))

    def __rsub__(self, other):
        return self._coerce(other) - self

    def __mul__(self, other):
        if isinstance(other, numbers.Number):
            return PauliExpression({k: c * other for k, c in self.terms.items()})
        other = self._coerce(other)
        out: dict[tuple[int, int], complex] = {}
        for (a1, b1), c1 in self.terms.items():
            for (a2, b2), c2 in other.terms.items():
                phase = 1 + 0j
                a = (a1 | a2) & ~((a1 | b1) & (a2 | b2))
                b = (b1 | b2) & ~((a1 | b1) & (a2 | b2))
                both = (a1 | b1) & (a2 | b2)
                i = 0
                while both >> i:
                    if (both >> i) & 1:
                        ph, r = _PRODUCT[(_site_type(a1, b1, i), _site_type(a2, b2, i))]
                        phase *= ph
                        ra, rb = _TYPE_TO_AB[r]
                        a |= ra << i
                        b |= rb << i
                    i += 1
                key = (a, b)
                out[key] = out.get(key, 0) + c1 * c2 * phase
        return PauliExpression({k: c for k, c in out.items() if c != 0})

    def __rmul__(self, other):
        if isinstance(other, numbers.Number):
            return self * other
        return self._coerce(other) * self

    def __truediv__(self, x):
        return self * (1.0 / x)

    def __len__(self):
        return len(self.terms)

    def __iter__(self):
        """Yields ((a, b), coefficient) like the reference's term iteration."""
        return iter(self.terms.items())

    def __repr__(self):
        return f"PauliExpression({len(self.terms)} strings)"

    # -- export --------------------------------------------------------------------
    def arrays(self, num_words: int = 1):
        """(a, b, coeff) as uint64 arrays of shape (n, num_words) and complex128 (n,)."""
        n = len(self.terms)
        a = np.zeros((n, num_words), np.uint64)
        b = np.zeros((n, num_words), np.uint64)
        coeff = np.zeros(n, np.complex128)
        for k, ((am, bm), c) in enumerate(self.terms.items()):
            for w in range(num_words):
                a[k, w] = (am >> (64 * w)) & 0xFFFFFFFFFFFFFFFF
                b[k, w] = (bm >> (64 * w)) & 0xFFFFFFFFFFFFFFFF
            coeff[k] = c
        return a, b, coeff

    def max_site(self) -> int:
        m = 0
        for (a, b) in self.terms:
            m = max(m, (a | b).bit_length())
        return m

    def matrix(self, num_sites: int, basis: str = "spins") -> np.ndarray:
        """Dense 2^N x 2^N matrix with <s|H|s'> = c * factor(s), s' = s ^ (a ^ b)."""
        if basis != "spins":
            raise ValueError("only the spin basis is supported")
        dim = 1 << num_sites
        H = np.zeros((dim, dim), np.complex128)
        s = np.arange(dim, dtype=np.int64)
        full = (1 << num_sites) - 1
        for (a, b), c in self.terms.items():
            flip = a ^ b
            y = (~a) & b & full
            zy = ((a & b) | y) & full
            ny = bin(y).count("1")
            pref = (-1j) ** ny
            neg = np.array([bin((~int(x)) & zy).count("1") & 1 for x in s])
            fac = pref * np.where(neg, -1.0, 1.0)
            H[s, s ^ flip] += c * fac
        return H

    def __matmul__(self, vec):
        vec = np.asarray(vec)
        n = int(np.log2(vec.shape[0]))
        return self.matrix(n) @ vec


def _single(i: int, t: int) -> PauliExpression:
    a, b = _TYPE_TO_AB[t]
    return PauliExpression({(a << i, b << i): 1.0})


def sigma_x(i: int) -> PauliExpression:
    return _single(i, 1)


def sigma_y(i: int) -> PauliExpression:
    return _single(i, 2)


def sigma_z(i: int) -> PauliExpression:
    return _single(i, 3)


def identity() -> PauliExpression:
    return PauliExpression({(0, 0): 1.0})


def transverse_field_ising_1d(L: int, h: float = 1.0, J: float = 1.0) -> PauliExpression:
    """H = -J sum_i Z_i Z_{i+1} - h sum_i X_i on a periodic chain."""
    H = PauliExpression()
    for i in range(L):
        H = H + (-J) * sigma_z(i) * sigma_z((i + 1) % L)
    for i in range(L):
        H = H + (-h) * sigma_x(i)
    return H


def square_lattice_bonds(Lx: int, Ly: int, diagonal: bool = False):
    """Periodic nearest-neighbour (and optionally next-nearest, diagonal) bonds, site = y * Lx + x."""
    nn, nnn = [], []
    for y in range(Ly):
        for x in range(Lx):
            i = y * Lx + x
            nn.append((i, y * Lx + (x + 1) % Lx))
            nn.append((i, ((y + 1) % Ly) * Lx + x))
            if diagonal:
                nnn.append((i, ((y + 1) % Ly) * Lx + (x + 1) % Lx))
                nnn.append((i, ((y + 1) % Ly) * Lx + (x - 1) % Lx))
    return nn, nnn


def transverse_field_ising_2d(Lx: int, Ly: int, h: float = 3.04, J: float = 1.0) -> PauliExpression:
    """H = -J sum_<ij> Z_i Z_j - h sum_i X_i on a periodic Lx x Ly square lattice."""
    nn, _ = square_lattice_bonds(Lx, Ly)
    H = PauliExpression()
    for i, j in nn:
        H = H + (-J) * sigma_z(i) * sigma_z(j)
    for i in range(Lx * Ly):
        H = H + (-h) * sigma_x(i)
    return H


def heisenberg_j1j2_2d(Lx: int, Ly: int, J1: float = 1.0, J2: float = 0.5) -> PauliExpression:
    """H = J1 sum_<ij> S_i.S_j + J2 sum_<<ij>> S_i.S_j with S.S = XX + YY + ZZ (Pauli units)."""
    nn, nnn = square_lattice_bonds(Lx, Ly, diagonal=True)
    H = PauliExpression()
    for J, bonds in ((J1, nn), (J2, nnn)):
        for i, j in bonds:
            H = H + J * (sigma_x(i) * sigma_x(j) + sigma_y(i) * sigma_y(j) + sigma_z(i) * sigma_z(j))
    return H
