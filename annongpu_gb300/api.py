"""The pyANNonGPU-compatible Python surface over the C ABI (include/annongpu.h).

Names, argument order and return shapes follow the reference's pybind11 module
_pyANNonGPU (pyANNonGPU/main.cpp.template:65-541) and the monkeypatched helpers
of pyANNonGPU/{PsiRBM,PsiDeep,PsiCNN}.py, so the reference's user code and tests
run unchanged for the VMC path. Every computation runs in libannongpu.so on the
GPU; the `gpu` arguments are kept for signature compatibility (there is no CPU
path to select).
"""

from __future__ import annotations

import ctypes as ct
import json

import numpy as np

from . import _lib as L
from ._lib import call, cbuf, c128, ptr, stream_ptr
from .expression import PauliExpression
from .json_numpy import NumpyDecoder, NumpyEncoder

_ACT = {"poly": L.ACT_POLY, "logcosh": L.ACT_LOGCOSH, 0: L.ACT_POLY, 1: L.ACT_LOGCOSH}
_PREC = {"fp32": L.PREC_FP32, "fp64": L.PREC_FP64, "complex64": L.PREC_FP32, "complex128": L.PREC_FP64}


def _conf_words(conf, num_words: int) -> np.ndarray:
    if isinstance(conf, Spins):
        conf = conf.configuration
    conf = int(conf)
    return np.array([(conf >> (64 * w)) & 0xFFFFFFFFFFFFFFFF for w in range(num_words)], np.uint64)


class _Handle:
    _destroy = None

    def __init__(self):
        self._h = ct.c_void_p()

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value and self._destroy:
            try:
                getattr(L.lib, self._destroy)(h)
            except Exception:
                pass
            self._h = ct.c_void_p()

    @property
    def handle(self):
        return self._h


# ----------------------------------------------------------------------------------
# Spins (include/basis/Spins.h:273-403; binding main.cpp.template:340-344)
class Spins:
    def __init__(self, configuration: int, num_spins: int):
        configuration = int(configuration)
        if num_spins < 128:
            configuration &= (1 << num_spins) - 1
        self.configuration = configuration
        self.num_spins = num_spins

    @staticmethod
    def enumerate(index: int) -> "Spins":
        return Spins(int(index), 128)

    def roll(self, shift: int, N: int) -> "Spins":
        c = self.configuration & ((1 << N) - 1)
        shift %= N
        return Spins(((c << shift) | (c >> (N - shift))) & ((1 << N) - 1), N)

    def array(self, num_spins: int) -> np.ndarray:
        return np.array([1.0 if (self.configuration >> i) & 1 else -1.0 for i in range(num_spins)])

    def __int__(self):
        return self.configuration

    def __eq__(self, other):
        return isinstance(other, Spins) and other.configuration == self.configuration

    def __hash__(self):
        return hash(self.configuration)

    def __repr__(self):
        return f"Spins({self.configuration:#x})"


# ----------------------------------------------------------------------------------
class _Psi(_Handle):
    _destroy = "ann_psi_destroy"

    def _init_common(self, gpu):
        self.gpu = bool(gpu)
        n = ct.c_uint()
        call("ann_psi_num_params", self._h, ct.byref(n))
        self._num_params = n.value

    @property
    def num_params(self) -> int:
        return self._num_params

    @property
    def params(self) -> np.ndarray:
        out = cbuf(self._num_params)
        call("ann_psi_get_params", self._h, ptr(out))
        return out

    @params.setter
    def params(self, value):
        v = c128(value).reshape(-1)
        if v.size != self._num_params:
            raise ValueError(f"expected {self._num_params} parameters, got {v.size}")
        call("ann_psi_set_params", self._h, ptr(v))

    def set_params_async(self, host_params, stream):
        """Copies parameters (complex128, ideally pinned host memory) on `stream`;
        `host_params` may be a numpy array or a torch CPU tensor of float64 pairs."""
        if hasattr(host_params, "data_ptr"):
            p = ct.c_void_p(host_params.data_ptr())
        else:
            self._pending = c128(host_params)
            p = ptr(self._pending)
        call("ann_psi_set_params_async", self._h, p, stream_ptr(stream))

    @property
    def log_prefactor(self) -> complex:
        out = np.zeros(2)
        call("ann_psi_get_log_prefactor", self._h, ptr(out))
        return complex(out[0], out[1])

    @log_prefactor.setter
    def log_prefactor(self, value):
        value = complex(value)
        call("ann_psi_set_log_prefactor", self._h, value.real, value.imag)

    @property
    def symmetric(self) -> bool:
        return False

    def copy(self):
        other = object.__new__(type(self))
        _Handle.__init__(other)
        call("ann_psi_copy", self._h, ct.byref(other._h))
        other.__dict__.update({k: v for k, v in self.__dict__.items() if k != "_h"})
        return other

    def __pos__(self):
        return self.copy()

    # PsiDeep.py:47-57 / PsiRBM.py:39-49 / PsiCNN.py:47-57
    def _vector(self, exact_summation):
        return psi_vector(self, exact_summation)

    def vector(self, exact_summation):
        return self._vector(exact_summation)

    def norm(self, exact_summation) -> float:
        out = np.zeros(1)
        call("ann_psi_norm", self._h, exact_summation.handle, None, ptr(out))
        return float(out[0])

    def normalize(self, exact_summation):
        self.log_prefactor -= np.log(self.norm(exact_summation))

    def calibrate(self, ensemble):
        if type(ensemble).__name__.startswith("ExactSummation"):
            self.normalize(ensemble)
            self.log_prefactor -= 1j * log_psi(self, ensemble).imag
        else:
            self.log_prefactor = 0
            self.log_prefactor -= log_psi(self, ensemble)

    def _device_params(self) -> int:
        p = ct.c_void_p()
        call("ann_psi_params_device", self._h, ct.byref(p))
        return p.value


def _make_rbm(obj, N, M, C, conn, params, fw, log_prefactor, layout, a_in_log_psi, activation, precision, gpu):
    params = c128(params).reshape(-1)
    fw = c128(np.broadcast_to(np.asarray(fw, np.complex128), (M,)))
    conn_a = None if conn is None else np.ascontiguousarray(np.asarray(conn, np.uint32).reshape(-1))
    lp = complex(log_prefactor)
    d = L.RbmDesc(N, M, C, ptr(conn_a), ptr(params), ptr(fw), (ct.c_double * 2)(lp.real, lp.imag), layout,
                  int(bool(a_in_log_psi)), _ACT[activation], _PREC[precision])
    _Handle.__init__(obj)
    call("ann_psi_create_rbm", ct.byref(d), ct.byref(obj._h))
    obj._init_common(gpu)


class PsiRBM(_Psi):
    """Restricted Boltzmann machine (include/quantum_state/PsiRBM.hpp:41-262).

    Reference form: ``PsiRBM(W, final_weight, log_prefactor, gpu)`` with
    log psi = log_prefactor + final_weight * sum_j f(sum_i W_ij s_i) and params = W.
    Optional visible/hidden biases ``a``, ``b`` switch to params = [a | b | W] with
    log psi += a.s (the standard complex RBM).
    """

    def __init__(self, W, final_weight=1.0, log_prefactor=0.0, gpu=True, *, a=None, b=None,
                 activation="poly", precision="fp32", a_in_log_psi=True):
        W = c128(W)
        N, M = W.shape
        self.N, self.M = N, M
        self.num_sites = N
        self.final_weight = complex(final_weight)
        self.activation = activation
        self.precision = precision
        self._biased = a is not None or b is not None
        if self._biased:
            a = np.zeros(N, np.complex128) if a is None else c128(a)
            b = np.zeros(M, np.complex128) if b is None else c128(b)
            params = np.concatenate([a, b, W.reshape(-1)])
            layout = L.LAYOUT_DEEP
        else:
            params = W.reshape(-1)
            layout = L.LAYOUT_RBM
        _make_rbm(self, N, M, N, None, params, self.final_weight, log_prefactor, layout, a_in_log_psi,
                  activation, precision, gpu)

    @property
    def W(self) -> np.ndarray:
        p = self.params
        off = self.N + self.M if self._biased else 0
        return p[off:].reshape(self.N, self.M)

    @property
    def a(self):
        return self.params[:self.N] if self._biased else np.zeros(self.N, np.complex128)

    @property
    def b(self):
        return self.params[self.N:self.N + self.M] if self._biased else np.zeros(self.M, np.complex128)

    # PsiRBM.py:7-36
    def to_json(self):
        obj = dict(type="PsiRBM", W=self.W, final_weight=self.final_weight,
                   log_prefactor_re=self.log_prefactor.real, log_prefactor_im=self.log_prefactor.imag)
        if self._biased:
            obj.update(a=self.a, b=self.b)
        return json.loads(json.dumps(obj, cls=NumpyEncoder, default=_json_default))

    @staticmethod
    def from_json(json_obj, gpu=True):
        obj = json.loads(json.dumps(json_obj, cls=NumpyEncoder), cls=NumpyDecoder)
        fw = obj["final_weight"]
        if isinstance(fw, dict):
            fw = complex(fw["re"], fw["im"])
        return PsiRBM(obj["W"], fw, obj["log_prefactor_re"] + 1j * obj["log_prefactor_im"], gpu,
                      a=obj.get("a"), b=obj.get("b"))


def _json_default(o):
    if isinstance(o, complex):
        return {"re": o.real, "im": o.imag}
    raise TypeError(type(o))


class PsiDeep(_Psi):
    """Feed-forward network with sparse connectivity (include/quantum_state/PsiDeep.hpp:70-471).

    Hidden layer l has M_l units; unit j reads C_l units of the layer below (the spins
    for l = 0) through ``connections[l]`` (C_l x M_l):
        z_0,j = b_0,j + sum_i W_0[i,j] s[connections[0][i,j]]
        z_l,j = b_l,j + sum_i W_l[i,j] f(z_{l-1})[connections[l][i,j]]
        log psi = log_prefactor + (a.s) + sum_j final_weights_j f(z_L,j)
    params = [a | b_0 | W_0 | b_1 | W_1 | ...]. f is the reference's log-cosh polynomial
    on the first layer and its odd polynomial deeper (``activation="logcosh"``: log cosh
    on every layer). One hidden layer runs on the RBM-family kernels (which also take the
    learned proposal); more layers (up to 4; the reference allows 3) on kernels that keep
    the first layer's pre-activations per chain and run the deeper layers in full.

    ``a_in_log_psi=False`` reproduces the reference exactly, whose log psi omits a.s
    (PsiDeep.hpp:260-264) while its O_k still reports s for the a entries.
    """

    def __init__(self, num_sites, a, b, connections, W, final_weights, log_prefactor=0.0, gpu=True, *,
                 a_in_log_psi=True, activation="poly", precision="fp32"):
        if isinstance(b, np.ndarray) and b.ndim == 1:
            b, connections, W = [b], [connections], [W]
        if not (len(b) == len(connections) == len(W)) or len(W) < 1:
            raise ValueError("b, connections and W need one entry per hidden layer")
        a = c128(a).reshape(-1)
        bs = [c128(x).reshape(-1) for x in b]
        Ws = [c128(x) for x in W]
        conns = [np.asarray(x, np.uint32) for x in connections]
        N = a.size
        below = N
        for l, (bl, Wl, cl) in enumerate(zip(bs, Ws, conns)):
            if Wl.ndim != 2 or cl.shape != Wl.shape or Wl.shape[1] != bl.size:
                raise ValueError(f"layer {l}: W and connections must be (C, M) with M = len(b)")
            if cl.size and int(cl.max()) >= below:
                raise ValueError(f"layer {l}: connection index beyond the {below} units below")
            below = bl.size
        self.num_sites = int(num_sites)
        self.N = N
        self.N_i = 0
        self.N_j = 0
        self._sizes = [bl.size for bl in bs]
        self._C = [Wl.shape[0] for Wl in Ws]
        self._M, self._C0 = self._sizes[0], self._C[0]
        self._connections = [c.copy() for c in conns]
        self._final_weights = c128(final_weights).reshape(-1)
        if self._final_weights.size == 1 and self._sizes[-1] > 1:
            self._final_weights = np.full(self._sizes[-1], self._final_weights[0])
        if self._final_weights.size != self._sizes[-1]:
            raise ValueError("final_weights needs one entry per unit of the last layer")
        self.activation = activation
        self.precision = precision
        self.a_in_log_psi = a_in_log_psi
        params = np.concatenate([a] + [np.concatenate([bl, Wl.reshape(-1)]) for bl, Wl in zip(bs, Ws)])
        if len(Ws) == 1:
            _make_rbm(self, N, self._M, self._C0, conns[0], params, self._final_weights, log_prefactor,
                      L.LAYOUT_DEEP, a_in_log_psi, activation, precision, gpu)
            return
        sizes = np.ascontiguousarray(self._sizes, np.uint32)
        cc = np.ascontiguousarray(self._C, np.uint32)
        cat = np.ascontiguousarray(np.concatenate([c.reshape(-1) for c in conns]).astype(np.uint32))
        fw = np.ascontiguousarray(self._final_weights)
        lp = complex(log_prefactor)
        d = L.DeepDesc(N, len(Ws), ptr(sizes), ptr(cc), ptr(cat), ptr(params), params.size, ptr(fw),
                       (ct.c_double * 2)(lp.real, lp.imag), int(bool(a_in_log_psi)), _ACT[activation],
                       _PREC[precision])
        _Handle.__init__(self)
        call("ann_psi_create_deep", ct.byref(d), ct.byref(self._h))
        self._init_common(gpu)

    @property
    def num_layers(self):
        return len(self._sizes)

    def _layer_offsets(self):
        off, out = self.N, []
        for m, c in zip(self._sizes, self._C):
            out.append((off, off + m, off + m + c * m))
            off += m * (1 + c)
        return out

    @property
    def a(self):
        return self.params[:self.N]

    input_weights = a

    @property
    def b(self):
        p = self.params
        return [p[b0:w0] for b0, w0, _ in self._layer_offsets()]

    @property
    def W(self):
        p = self.params
        return [p[w0:e].reshape(c, m) for (_, w0, e), m, c in zip(self._layer_offsets(), self._sizes, self._C)]

    @property
    def connections(self):
        return [c.copy() for c in self._connections]

    @property
    def final_weights(self):
        return self._final_weights.copy()

    @property
    def first_layer_params_slice(self):
        return slice(self.N, self.N + self._M * (1 + self._C0))

    # PsiDeep.py:7-44
    def to_json(self):
        obj = dict(type="PsiDeep", num_sites=self.num_sites, a=self.a, b=self.b, connections=self.connections,
                   W=self.W, final_weights=self.final_weights, log_prefactor_re=self.log_prefactor.real,
                   log_prefactor_im=self.log_prefactor.imag)
        return json.loads(json.dumps(obj, cls=NumpyEncoder))

    @staticmethod
    def from_json(json_obj, gpu=True, **kwargs):
        """``kwargs`` (activation, precision, a_in_log_psi) are not part of the reference's format."""
        obj = json.loads(json.dumps(json_obj, cls=NumpyEncoder), cls=NumpyDecoder)
        return PsiDeep(obj["num_sites"], obj["a"], obj["b"], obj["connections"], obj["W"], obj["final_weights"],
                       obj["log_prefactor_re"] + 1j * obj["log_prefactor_im"], gpu, **kwargs)


def _pad3(v):
    v = [int(x) for x in np.asarray(v).reshape(-1)]
    return [1] * (3 - len(v)) + v


class PsiCNN(_Psi):
    """Periodic convolutional network (include/quantum_state/PsiCNN.hpp:34-383), one or two layers.

    ``PsiCNN(extent, num_channels_list, connectivity_list, symmetry_classes, params,
    final_factor, log_prefactor, gpu)`` as the reference (main.cpp.template:161-170):
    extent and each connectivity are 3-vectors (shorter ones are padded with leading 1s),
    params are ordered per layer, per channel link (c_in * C_out + c_out), per symmetry
    class, per window offset (source/quantum_state/PsiCNN.cpp:38-45).
    ``activation="logcosh"`` uses log cosh on every layer instead of the reference's
    layer polynomials.
    """

    dim = 3

    def __init__(self, extent, num_channels_list, connectivity_list, symmetry_classes, params, final_factor=1.0,
                 log_prefactor=0.0, gpu=True, *, activation="poly", precision="fp32"):
        self.extent = _pad3(extent)
        self.num_channels_list = np.asarray(num_channels_list, np.uint32).reshape(-1)
        L_ = len(self.num_channels_list)
        conn = np.asarray(connectivity_list).reshape(L_, -1)
        self.connectivity_list = np.array([_pad3(c) for c in conn], np.uint32)
        self.N = int(np.prod(self.extent))
        self.num_sites = self.N
        sym = np.asarray(symmetry_classes).reshape(-1).astype(np.uint32)
        self.symmetry_classes = sym
        self.num_symmetry_classes = len(set(sym.tolist()))
        self.final_factor = float(final_factor)
        self.activation = activation
        self.precision = precision
        p = c128(params).reshape(-1)
        lp = complex(log_prefactor)
        self._keep = (np.ascontiguousarray(self.num_channels_list), np.ascontiguousarray(self.connectivity_list),
                      np.ascontiguousarray(sym), p)
        d = L.CnnDesc((ct.c_uint * 3)(*self.extent), L_, ptr(self._keep[0]), ptr(self._keep[1]), ptr(self._keep[2]),
                      ptr(p), p.size, self.final_factor, (ct.c_double * 2)(lp.real, lp.imag), _ACT[activation],
                      _PREC[precision])
        _Handle.__init__(self)
        call("ann_psi_create_cnn", ct.byref(d), ct.byref(self._h))
        self._init_common(gpu)

    def init_gradient(self, num_steps):
        """No-op: O_k rows are written directly (the reference records angles per sample, PsiCNN.cpp:74-78)."""

    # PsiCNN.py:60-83
    def channel_link(self, layer, i, j):
        offset = 0
        vol = [int(np.prod(c)) for c in self.connectivity_list]
        for l in range(layer):
            prev = self.num_channels_list[l - 1] if l > 0 else 1
            offset += int(self.num_channels_list[l] * prev) * self.num_symmetry_classes * vol[l]
        offset += (i * int(self.num_channels_list[layer]) + j) * self.num_symmetry_classes * vol[layer]
        return self.params[offset:offset + self.num_symmetry_classes * vol[layer]]

    # PsiCNN.py:7-44
    def to_json(self):
        obj = dict(type="PsiCNN", extent=np.array(self.extent), num_channels_list=self.num_channels_list,
                   connectivity_list=self.connectivity_list, symmetry_classes=self.symmetry_classes,
                   params=self.params, final_factor=self.final_factor, log_prefactor_re=self.log_prefactor.real,
                   log_prefactor_im=self.log_prefactor.imag)
        return json.loads(json.dumps(obj, cls=NumpyEncoder))

    @staticmethod
    def from_json(json_obj, gpu=True):
        obj = json.loads(json.dumps(json_obj, cls=NumpyEncoder), cls=NumpyDecoder)
        return PsiCNN(obj["extent"], obj["num_channels_list"], obj["connectivity_list"], obj["symmetry_classes"],
                      obj["params"], obj["final_factor"], obj["log_prefactor_re"] + 1j * obj["log_prefactor_im"], gpu)


# ----------------------------------------------------------------------------------
class Operator(_Handle):
    """Sum of Pauli strings (include/operator/Operator.hpp:26-214)."""

    _destroy = "ann_op_destroy"

    def __init__(self, expr, gpu=True):
        _Handle.__init__(self)
        if not isinstance(expr, PauliExpression):
            expr = PauliExpression({(int(a), int(b)): c for (a, b), c in expr})
        self.expr = expr
        self.gpu = bool(gpu)
        a, b, c = expr.arrays(2)
        a = np.ascontiguousarray(a)
        b = np.ascontiguousarray(b)
        c = c128(c)
        call("ann_op_create_pauli", len(c), 2, ptr(a), ptr(b), ptr(c), ct.byref(self._h))
        self.num_strings = len(c)


# ----------------------------------------------------------------------------------
class PauliString:
    """A Pauli string over sites as the words (a, b): per site (a, b) = (0, 0) I, (1, 0) X,
    (0, 1) Y, (1, 1) Z; ``[i]`` is the type 0..3 of site i (include/basis/PauliString.hpp:18-80)."""

    def __init__(self, a: int, b: int):
        self.a, self.b = int(a), int(b)

    @staticmethod
    def enumerate(index: int) -> "PauliString":
        """Base-4 digit i of ``index`` is the type of site i (PauliString.hpp:30-35)."""
        index = int(index)
        a = b = 0
        for i in range(32):
            a |= ((index >> (2 * i)) & 1) << i
            b |= ((index >> (2 * i + 1)) & 1) << i
        return PauliString(a, b)

    def __getitem__(self, i: int) -> int:
        return ((self.a >> i) & 1) | (((self.b >> i) & 1) << 1)

    def array(self, num_sites: int) -> np.ndarray:
        return np.array([self[i] for i in range(num_sites)], np.uint32)

    def __eq__(self, other):
        return isinstance(other, PauliString) and (self.a, self.b) == (other.a, other.b)

    def __hash__(self):
        return hash((self.a, self.b))

    def __repr__(self):
        return f"PauliString(a={self.a:#x}, b={self.b:#x})"


def _pauli_rows(strings) -> np.ndarray:
    """PauliStrings or (a, b) pairs -> (n, 2) uint64 rows."""
    rows = [(p.a, p.b) if isinstance(p, PauliString) else (int(p[0]), int(p[1])) for p in strings]
    return np.ascontiguousarray(np.array(rows, np.uint64).reshape(-1, 2))


class ExactSummationSpins(_Handle):
    """All 2^N configurations, weight |psi(s)|^2 unnormalised (include/ensembles/ExactSummation.hpp:33-72)."""

    _destroy = "ann_ens_destroy"

    def __init__(self, num_sites, gpu=True):
        _Handle.__init__(self)
        self.num_sites = int(num_sites)
        self.gpu = bool(gpu)
        call("ann_ens_create_exact", self.num_sites, ct.byref(self._h))

    @property
    def num_steps(self) -> int:
        return 1 << self.num_sites


class ExactSummationPaulis(ExactSummationSpins):
    """All 4^N Pauli strings over N sites, weight |psi(x)|^2 unnormalised
    (ExactSummation_t<PauliString>, include/ensembles/ExactSummation.hpp:125). The
    wavefunction sees three input units per site (PsiDeep of any depth, 3 N inputs)."""

    def __init__(self, num_sites, gpu=True):
        ExactSummationSpins.__init__(self, num_sites, gpu)
        call("ann_ens_set_basis", self._h, L.BASIS_PAULIS)

    @property
    def num_steps(self) -> int:
        return 1 << (2 * self.num_sites)


_MOVES = {"single_flip": L.MOVE_FLIP, "flip": L.MOVE_FLIP, "exchange": L.MOVE_EXCHANGE_BONDS,
          "exchange_bonds": L.MOVE_EXCHANGE_BONDS, "exchange_pairs": L.MOVE_EXCHANGE_PAIRS}


class MonteCarloSpins(_Handle):
    """Metropolis chains (include/ensembles/MonteCarlo.hpp:28-259).

    ``MonteCarloSpins(num_samples, num_sweeps, num_thermalization_sweeps, num_markov_chains, gpu)``
    as in the reference; ``MonteCarloSpins(other)`` copies. Extensions (keyword-only):
    ``move`` ("single_flip", "exchange" over ``bonds``, "exchange_pairs"), ``n_up``
    (fixed-magnetisation initial configurations), ``seed`` (Philox key) and
    ``persistent`` (chains continue across calls instead of being re-drawn and
    re-thermalised each call as the reference does, MonteCarlo.hpp:79, 89-93).
    """

    _destroy = "ann_ens_destroy"

    def __init__(self, num_samples, num_sweeps=None, num_thermalization_sweeps=None, num_markov_chains=None,
                 gpu=True, *, move="single_flip", bonds=None, n_up=None, seed=0, persistent=False):
        _Handle.__init__(self)
        if isinstance(num_samples, MonteCarloSpins):
            other = num_samples
            call("ann_ens_copy", other._h, ct.byref(self._h))
            self.__dict__.update({k: v for k, v in other.__dict__.items() if k != "_h"})
            return
        self.num_samples = int(num_samples)
        self.num_sweeps = int(num_sweeps)
        self.num_thermalization_sweeps = int(num_thermalization_sweeps)
        self.num_markov_chains = int(num_markov_chains)
        self.gpu = bool(gpu)
        self.move = move
        self._bonds = None if bonds is None else np.ascontiguousarray(np.asarray(bonds, np.uint32).reshape(-1, 2))
        d = L.McDesc(self.num_samples, self.num_sweeps, self.num_thermalization_sweeps, self.num_markov_chains,
                     _MOVES[move], ptr(self._bonds), 0 if self._bonds is None else len(self._bonds),
                     -1 if n_up is None else int(n_up), int(seed) & 0xFFFFFFFFFFFFFFFF, int(bool(persistent)))
        call("ann_ens_create_mc", ct.byref(d), ct.byref(self._h))

    @property
    def num_steps(self) -> int:
        return self.num_samples

    @property
    def acceptance_rate(self) -> float:
        out = np.zeros(1)
        call("ann_ens_acceptance_rate", self._h, ptr(out))
        return float(out[0])

    def refresh_stats(self, stream=None):
        """Reads the acceptance counters of the last sampling pass and applies the learned
        proposal's drop rule (TDVP evaluations and SR steps leave this to the caller)."""
        call("ann_ens_refresh_stats", self._h, stream_ptr(stream))

    def get_chains(self):
        conf = np.zeros((self.num_markov_chains, 2), np.uint64)
        ctr = np.zeros(self.num_markov_chains, np.uint64)
        call("ann_ens_get_chains", self._h, ptr(conf), ptr(ctr))
        return conf, ctr

    def set_chains(self, conf, counter):
        conf = np.ascontiguousarray(np.asarray(conf, np.uint64).reshape(self.num_markov_chains, -1))
        if conf.shape[1] == 1:
            conf = np.concatenate([conf, np.zeros_like(conf)], axis=1)
        ctr = np.ascontiguousarray(np.asarray(counter, np.uint64))
        call("ann_ens_set_chains", self._h, ptr(conf), ptr(ctr))

    def set_tape(self, init_conf, sites, u):
        """Replays recorded proposals: init_conf (chains,), sites/u (chains, len)."""
        if sites is None:
            call("ann_ens_set_tape", self._h, None, None, None, 0)
            return
        init = np.zeros((self.num_markov_chains, 2), np.uint64)
        init[:, 0] = np.asarray(init_conf, np.uint64).reshape(-1)
        s = np.ascontiguousarray(np.asarray(sites, np.uint32).reshape(self.num_markov_chains, -1))
        uu = np.ascontiguousarray(np.asarray(u, np.float64).reshape(self.num_markov_chains, -1))
        self._tape = (init, s, uu)
        call("ann_ens_set_tape", self._h, ptr(init), ptr(s), ptr(uu), s.shape[1])

    def samples(self):
        """(configurations (num_steps, 2) uint64, log psi, local energy) of the last call."""
        n = (self.num_samples // self.num_markov_chains) * self.num_markov_chains
        conf = np.zeros((n, 2), np.uint64)
        lp = cbuf(n)
        el = cbuf(n)
        call("ann_ens_get_samples", self._h, ptr(conf), ptr(lp), ptr(el))
        return conf, lp, el


    # learned proposal (made.cu)
    def set_proposal(self, made, indep_per_sample=1, min_acceptance=0.0):
        """Adds `indep_per_sample` Metropolis-Hastings independence moves drawn from the
        MADE `made` after the local sweeps of every sample; the proposal is dropped once
        its acceptance in a call falls below `min_acceptance`."""
        self._made = made
        call("ann_ens_set_proposal", self._h, None if made is None else made.handle, int(indep_per_sample),
             float(min_acceptance))

    @property
    def proposal_acceptance(self) -> float:
        out = np.zeros(1)
        call("ann_ens_proposal_stats", self._h, ptr(out), None)
        return float(out[0])

    @property
    def proposal_dropped(self) -> bool:
        out = ct.c_int()
        call("ann_ens_proposal_stats", self._h, None, ct.byref(out))
        return bool(out.value)

    def set_history(self, capacity):
        """Keeps the configurations of the last `capacity` samples as proposal training data."""
        call("ann_ens_set_history", self._h, int(capacity))


MonteCarloLoop = MonteCarloSpins


class MonteCarloPaulis(MonteCarloSpins):
    """Metropolis chains over Pauli strings (MonteCarlo_tt<PauliString>,
    include/ensembles/MonteCarlo.hpp:266-280): each move sets a random site to a random
    type I, X, Y, Z (Update_Policy.hpp:41-57); a sweep is one move per input unit of the
    wavefunction (3 per site). ``seed`` and ``persistent`` as for MonteCarloSpins."""

    def __init__(self, num_samples, num_sweeps=None, num_thermalization_sweeps=None, num_markov_chains=None,
                 gpu=True, *, seed=0, persistent=False):
        if isinstance(num_samples, MonteCarloPaulis):
            MonteCarloSpins.__init__(self, num_samples)
            return
        MonteCarloSpins.__init__(self, num_samples, num_sweeps, num_thermalization_sweeps, num_markov_chains, gpu,
                                 seed=seed, persistent=persistent)
        call("ann_ens_set_basis", self._h, L.BASIS_PAULIS)


# ----------------------------------------------------------------------------------
def _conf_rows(confs) -> np.ndarray:
    """Configurations (ints or Spins, or a (n,) / (n, 2) uint64 array) -> (n, 2) uint64 rows."""
    if isinstance(confs, np.ndarray) and confs.dtype == np.uint64:
        c = confs.reshape(len(confs), -1)
        if c.shape[1] == 2:
            return np.ascontiguousarray(c)
        return np.ascontiguousarray(np.concatenate([c[:, :1], np.zeros((len(c), 1), np.uint64)], axis=1))
    return np.ascontiguousarray(np.stack([_conf_words(c, 2) for c in confs]) if len(confs) else
                                np.zeros((0, 2), np.uint64))


class MADE(_Handle):
    """Masked autoregressive MLP q(s) over N spins with one hidden layer of width H
    (the learned Metropolis-Hastings proposal; this project's own component)."""

    _destroy = "ann_made_destroy"

    def __init__(self, N, H=256, seed=0):
        _Handle.__init__(self)
        self.N, self.H = int(N), int(H)
        call("ann_made_create", self.N, self.H, int(seed) & 0xFFFFFFFFFFFFFFFF, ct.byref(self._h))

    @property
    def params(self):
        W1 = np.zeros((self.H, self.N), np.float32)
        b1 = np.zeros(self.H, np.float32)
        W2 = np.zeros((self.N, self.H), np.float32)
        b2 = np.zeros(self.N, np.float32)
        call("ann_made_get_params", self._h, ptr(W1), ptr(b1), ptr(W2), ptr(b2))
        return W1, b1, W2, b2

    @params.setter
    def params(self, value):
        W1, b1, W2, b2 = (np.ascontiguousarray(np.asarray(v, np.float32)) for v in value)
        call("ann_made_set_params", self._h, ptr(W1), ptr(b1), ptr(W2), ptr(b2))

    def log_prob(self, confs):
        rows = _conf_rows(confs)
        out = np.zeros(len(rows))
        call("ann_made_log_prob", self._h, ptr(rows), len(rows), ptr(out))
        return out

    def sample(self, n, seed=0, first=0):
        confs = np.zeros((n, 2), np.uint64)
        logq = np.zeros(n)
        call("ann_made_sample", self._h, int(n), int(seed), int(first), ptr(confs), ptr(logq))
        return confs, logq

    def gradient(self, confs):
        rows = _conf_rows(confs)
        g = [np.zeros((self.H, self.N), np.float32), np.zeros(self.H, np.float32),
             np.zeros((self.N, self.H), np.float32), np.zeros(self.N, np.float32)]
        loss = np.zeros(1)
        call("ann_made_gradient", self._h, ptr(rows), len(rows), *[ptr(x) for x in g], ptr(loss))
        return (*g, float(loss[0]))

    def train(self, confs, steps, batch=4096, lr=1e-3, stream=None):
        rows = _conf_rows(confs)
        loss = np.zeros(1)
        call("ann_made_train", self._h, ptr(rows), len(rows), int(steps), int(batch), float(lr), stream_ptr(stream),
             ptr(loss))
        return float(loss[0])

    def train_on_samples(self, ensemble, steps, batch=4096, lr=1e-3, stream=None):
        loss = np.zeros(1)
        call("ann_made_train_on_samples", self._h, ensemble.handle, int(steps), int(batch), float(lr),
             stream_ptr(stream), ptr(loss))
        return float(loss[0])


# ----------------------------------------------------------------------------------
class ExpectationValue:
    """source/network_functions/ExpectationValue.cu.template"""

    def __init__(self, gpu=True, stream=None):
        self.gpu = bool(gpu)
        self.stream = stream

    def __call__(self, operator, psi, ensemble):
        if isinstance(operator, (list, tuple)):
            hs = (ct.c_void_p * len(operator))(*[o.handle.value for o in operator])
            out = cbuf(len(operator))
            call("ann_expectation_list", hs, len(operator), psi.handle, ensemble.handle, stream_ptr(self.stream),
                 ptr(out))
            return out
        out = np.zeros(2)
        call("ann_expectation", operator.handle, psi.handle, ensemble.handle, stream_ptr(self.stream), ptr(out))
        return complex(out[0], out[1])

    def fluctuation(self, operator, psi, ensemble):
        out = np.zeros(3)
        call("ann_fluctuation", operator.handle, psi.handle, ensemble.handle, stream_ptr(self.stream), ptr(out))
        return float(out[0]), complex(out[1], out[2])

    def gradient(self, operator, psi, ensemble):
        g = cbuf(psi.num_params)
        v = np.zeros(2)
        call("ann_gradient", operator.handle, psi.handle, ensemble.handle, stream_ptr(self.stream), ptr(g), ptr(v))
        return g, complex(v[0], v[1])

    gradient_with_noise = gradient  # bound to gradient in the reference (main.cpp.template:428)

    def exp_sigma_z(self, operator, psi, ensemble):
        out = np.zeros(2)
        call("ann_exp_sigma_z", operator.handle, psi.handle, ensemble.handle, stream_ptr(self.stream), ptr(out))
        return complex(out[0], out[1])


_S_MODES = {"fp32": L.S_FP32, "plain": L.S_FP32, "bf16": L.S_BF16, "bf16_split": L.S_BF16_SPLIT}
_SOLVERS = {"fp64": L.SOLVER_FP64, "mixed": L.SOLVER_MIXED, "fp32": L.SOLVER_FP32}


class TDVP(_Handle):
    """S matrix, F vector and energy moments (include/network_functions/TDVP.hpp,
    source/network_functions/TDVP.cu.template), plus the GPU SR solve this build adds."""

    _destroy = "ann_tdvp_destroy"

    def __init__(self, num_params, gpu=True, *, s_mode="fp32", solver="fp64", max_iter=10, tol=1e-12,
                 stream=None):
        _Handle.__init__(self)
        self.num_params = int(num_params)
        self.gpu = bool(gpu)
        self.threshold = -1e6
        self.stream = stream
        call("ann_tdvp_create", self.num_params, ct.byref(self._h))
        self.s_mode = s_mode
        self.set_solver(solver, max_iter, tol)

    def set_solver(self, solver="fp64", max_iter=10, tol=1e-12):
        """SR solver: "fp64" (FP64 Cholesky + one refinement step), "mixed" (FP32
        Cholesky + refinement with FP64 residuals until ||r||/||F|| <= tol, at most
        max_iter FP32 solves; a stalled eager solve is redone in FP64) or "fp32" (one
        FP32 Cholesky solve without refinement, the plain FP32 form)."""
        call("ann_tdvp_set_solver", self._h, _SOLVERS[solver], int(max_iter), float(tol))
        self.solver = solver

    @property
    def chol_update(self):
        """Trailing update of the FP32 Cholesky: "tc" (tcgen05, split TF32) or "simt"."""
        return getattr(self, "_chol_update", "tc")

    @chol_update.setter
    def chol_update(self, mode):
        call("ann_tdvp_set_chol_update", self._h, {"simt": 0, "tc": 1}[mode])
        self._chol_update = mode

    @property
    def solver_info(self):
        """{'solves', 'residual_first', 'residual_last', 'fell_back', 'update_form'} of the last
        SR solve; update_form names the FP32 factorisation's trailing-update form."""
        out = np.zeros(4)
        call("ann_tdvp_solver_info", self._h, ptr(out))
        form = ct.c_int()
        call("ann_tdvp_solver_form", self._h, ct.byref(form))
        return {"solves": int(out[0]), "residual_first": float(out[1]), "residual_last": float(out[2]),
                "fell_back": bool(out[3]),
                "update_form": {0: None, 1: "FP32 SIMT", 2: "tensor core, rank 64 per panel",
                                3: "tensor core, rank 128 per panel pair"}[form.value]}

    @property
    def s_mode(self):
        return self._s_mode

    @s_mode.setter
    def s_mode(self, mode):
        call("ann_tdvp_set_s_mode", self._h, _S_MODES[mode])
        self._s_mode = mode

    def eval(self, operator, psi, ensemble):
        call("ann_tdvp_eval", self._h, operator.handle, psi.handle, ensemble.handle, stream_ptr(self.stream))

    def eval_F(self, operator, psi, ensemble):
        call("ann_tdvp_eval_F", self._h, operator.handle, psi.handle, ensemble.handle, stream_ptr(self.stream))

    @property
    def S_matrix(self):
        out = cbuf(self.num_params * self.num_params)
        call("ann_tdvp_get_S", self._h, ptr(out))
        return out.reshape(self.num_params, self.num_params)

    @property
    def F_vector(self):
        out = cbuf(self.num_params)
        call("ann_tdvp_get_F", self._h, ptr(out))
        return out

    @property
    def O_k_vector(self):
        out = cbuf(self.num_params)
        call("ann_tdvp_get_O", self._h, ptr(out))
        return out

    def _energy(self):
        E = np.zeros(2)
        E2 = np.zeros(1)
        call("ann_tdvp_get_energy", self._h, ptr(E), ptr(E2))
        return complex(E[0], E[1]), float(E2[0])

    @property
    def E_local(self):
        return self._energy()[0]

    @property
    def var_H(self):
        E, E2 = self._energy()
        return E2 - abs(E) ** 2

    @property
    def total_weight(self):
        out = np.zeros(1)
        call("ann_tdvp_get_total_weight", self._h, ptr(out))
        return float(out[0])

    @property
    def O_k_samples(self):
        n = ct.c_uint()
        out = None
        # rows of the last eval
        out = cbuf(self._rows() * self.num_params)
        call("ann_tdvp_get_O_samples", self._h, ptr(out))
        return out

    def _rows(self):
        return self._last_rows

    def S_dot_vector(self, vec, ensemble=None):
        v = c128(vec)
        out = cbuf(self.num_params)
        call("ann_tdvp_S_dot_vector", self._h, ptr(v), stream_ptr(self.stream), ptr(out))
        return out

    def solve(self, diag_shift, return_info=False):
        """delta = (S + diag_shift I)^{-1} F on the GPU with the configured solver; info =
        relative residuals ||F - (S + shift) delta|| / ||F|| of the first and final solution."""
        delta = cbuf(self.num_params)
        info = np.zeros(2)
        call("ann_tdvp_solve", self._h, float(diag_shift), stream_ptr(self.stream), ptr(delta), ptr(info))
        return (delta, info) if return_info else delta

    def update(self, psi, lr):
        call("ann_sr_update", self._h, psi.handle, float(lr), stream_ptr(self.stream))

    def sr_step(self, operator, psi, ensemble, diag_shift, lr):
        """One stochastic-reconfiguration step: eval, solve, params -= lr * delta (all on the device)."""
        call("ann_sr_step", self._h, operator.handle, psi.handle, ensemble.handle, float(diag_shift), float(lr),
             stream_ptr(self.stream))

    def capture_sr_step(self, operator, psi, ensemble, diag_shift, lr, stream):
        call("ann_sr_graph_capture", self._h, operator.handle, psi.handle, ensemble.handle, float(diag_shift),
             float(lr), stream_ptr(stream))

    def launch_sr_step(self, stream):
        call("ann_sr_graph_launch", self._h, stream_ptr(stream))


def _track_rows(fn):
    def wrapped(self, operator, psi, ensemble):
        fn(self, operator, psi, ensemble)
        self._last_rows = ensemble.num_steps if isinstance(ensemble, ExactSummationSpins) else \
            (ensemble.num_samples // ensemble.num_markov_chains) * ensemble.num_markov_chains
    return wrapped


TDVP.eval = _track_rows(TDVP.eval)
TDVP.eval_F = _track_rows(TDVP.eval_F)


# ----------------------------------------------------------------------------------
class HilbertSpaceDistance:
    """Distance between psi_prime and U psi and its gradient in the parameters of psi_prime
    (source/network_functions/HilbertSpaceDistance.cu.template:16-168; binding
    pyANNonGPU/main.cpp.template:436-442)."""

    def __init__(self, num_params, gpu=True, stream=None):
        self.num_params = int(num_params)
        self.gpu = bool(gpu)
        self.stream = stream

    def __call__(self, psi, psi_prime, operator_, is_unitary, spin_ensemble) -> float:
        out = np.zeros(1)
        call("ann_hsd_distance", psi.handle, psi_prime.handle, operator_.handle, int(bool(is_unitary)),
             spin_ensemble.handle, stream_ptr(self.stream), ptr(out))
        return float(out[0])

    def gradient(self, psi, psi_prime, operator_, is_unitary, spin_ensemble, nu=1.0):
        """(gradient, distance), as gradient_py (HilbertSpaceDistance.hpp:103-112)."""
        grad = cbuf(psi_prime.num_params)
        d = np.zeros(1)
        call("ann_hsd_gradient", psi.handle, psi_prime.handle, operator_.handle, int(bool(is_unitary)),
             spin_ensemble.handle, float(nu), stream_ptr(self.stream), ptr(grad), ptr(d))
        return grad, float(d[0])


# ----------------------------------------------------------------------------------
class PsiFullyPolarized:
    """The trivial reference of a classical network: log psi = 0, no parameters
    (include/quantum_state/PsiFullyPolarized.hpp:16-120)."""

    def __init__(self, num_sites, log_prefactor=0.0):
        self.num_sites = int(num_sites)
        self.log_prefactor = complex(log_prefactor)
        self.num_params = 0
        self.params = np.zeros(0, np.complex128)


def _feature_strings(H_local, nw):
    """(feature_begin, a, b, coeff) of a list of operators / Pauli expressions."""
    beg, A, B, C = [0], [], [], []
    for h in H_local:
        expr = h.expr if isinstance(h, Operator) else h
        if not isinstance(expr, PauliExpression):
            expr = PauliExpression({(int(a), int(b)): c for (a, b), c in expr})
        a, b, c = expr.arrays(nw)
        A.append(np.asarray(a, np.uint64).reshape(-1, nw))
        B.append(np.asarray(b, np.uint64).reshape(-1, nw))
        C.append(np.asarray(c, np.complex128))
        beg.append(beg[-1] + len(C[-1]))
    cat = lambda xs, shape: np.ascontiguousarray(np.concatenate(xs) if xs else np.zeros(shape))
    return (np.ascontiguousarray(beg, np.uint32), cat(A, (0, nw)).astype(np.uint64), cat(B, (0, nw)).astype(np.uint64),
            cat(C, 0).astype(np.complex128))


class PsiClassical(_Psi):
    """Variational classical network (vCN; include/quantum_state/PsiClassical.hpp:48-260):
    log psi(s) = log_prefactor + sum_k params_k h_k(s) (+ log psi_ref(s) for order 2), with
    h_k(s) = fast_local_energy of the k-th operator of H_local (Operator.hpp:122-133).
    ``params`` are [classical params | reference params]; psi_ref is a PsiDeep (any depth,
    copied at construction) or PsiFullyPolarized. Runs on the PsiDeep kernels."""

    def __init__(self, num_sites, H_local, params, psi_ref, log_prefactor=0.0, gpu=True, *, order=1,
                 precision="fp64"):
        self.num_sites = int(num_sites)
        self.N = self.num_sites
        self.order = int(order)
        self.H_local = list(H_local)
        p = c128(params).reshape(-1)
        if p.size != len(self.H_local):
            raise ValueError("params needs one value per operator of H_local")
        self._ref = psi_ref
        nw = 2 if self.num_sites > 64 else 1
        beg, A, B, C = _feature_strings(self.H_local, nw)
        self._keep = (beg, A, B, C, p)
        ref = psi_ref if (self.order > 1 and isinstance(psi_ref, _Psi)) else None
        self.precision = ref.precision if ref is not None else precision
        lp = complex(log_prefactor)
        d = L.ClassicalDesc(self.num_sites, len(self.H_local), ptr(beg), nw, ptr(A), ptr(B), ptr(C), ptr(p),
                            (ct.c_double * 2)(lp.real, lp.imag), self.order,
                            None if ref is None else ref.handle, _PREC[self.precision])
        _Handle.__init__(self)
        call("ann_psi_create_classical", ct.byref(d), ct.byref(self._h))
        self._init_common(gpu)

    @property
    def ref_log_prefactor(self) -> complex:
        out = np.zeros(2)
        call("ann_psi_ref_log_prefactor", self._h, None, ptr(out))
        return complex(out[0], out[1])

    @ref_log_prefactor.setter
    def ref_log_prefactor(self, value):
        v = np.array([complex(value).real, complex(value).imag])
        call("ann_psi_ref_log_prefactor", self._h, ptr(v), None)

    @property
    def psi_ref(self):
        """The reference with this network's current reference parameters (a copy)."""
        if not isinstance(self._ref, _Psi):
            return self._ref
        r = +self._ref
        if self.order > 1:
            r.params = self.params[len(self.H_local):]
            r.log_prefactor = self.ref_log_prefactor
        return r

    def calibrate(self, ensemble):
        if type(ensemble).__name__.startswith("ExactSummation"):
            _Psi.calibrate(self, ensemble)
            return
        # main.cpp.template:253-260: the reference part first, then the whole
        if self.order > 1 and isinstance(self._ref, _Psi):
            self.ref_log_prefactor -= log_psi(self.psi_ref, ensemble)
        self.log_prefactor -= log_psi(self, ensemble)


def _classical_factory(name, order, ann):
    def init(self, num_sites, H_local, params, psi_ref, log_prefactor=0.0, gpu=True, **kwargs):
        if ann and not isinstance(psi_ref, _Psi):
            raise ValueError(name + " needs a PsiDeep reference")
        PsiClassical.__init__(self, num_sites, H_local, params, psi_ref, log_prefactor, gpu, order=order, **kwargs)
    return type(name, (PsiClassical,), {"__init__": init, "__doc__": f"PsiClassical of order {order} "
                                         f"({'PsiDeep' if ann else 'fully polarized'} reference)."})


PsiClassicalFP_1 = _classical_factory("PsiClassicalFP_1", 1, False)
PsiClassicalFP_2 = _classical_factory("PsiClassicalFP_2", 2, False)
PsiClassicalANN_1 = _classical_factory("PsiClassicalANN_1", 1, True)
PsiClassicalANN_2 = _classical_factory("PsiClassicalANN_2", 2, True)


class KullbackLeibler(_Handle):
    """Kullback-Leibler-type divergence of psi (a classical network) from psi_prime over
    psi_prime's ensemble, its gradient in psi_prime's parameters and the gradient's noise
    (source/network_functions/KullbackLeibler.cu.template:17-329; binding
    main.cpp.template:445-461). The mean deviation of a call is subtracted in the next."""

    _destroy = "ann_kl_destroy"

    def __init__(self, num_params, gpu=True, stream=None):
        _Handle.__init__(self)
        self.num_params = int(num_params)
        self.gpu = bool(gpu)
        self.stream = stream
        call("ann_kl_create", self.num_params, ct.byref(self._h))

    def __call__(self, psi, psi_prime, ensemble, threshold=0.0) -> float:
        out = np.zeros(1)
        call("ann_kl_value", self._h, psi.handle, psi_prime.handle, ensemble.handle, float(threshold),
             stream_ptr(self.stream), ptr(out))
        return float(out[0])

    def gradient(self, psi, psi_prime, ensemble, nu=1.0, threshold=0.0):
        """(gradient, value), as gradient_py (KullbackLeibler.hpp:100-112)."""
        grad = cbuf(psi_prime.num_params)
        v = np.zeros(1)
        call("ann_kl_gradient", self._h, psi.handle, psi_prime.handle, ensemble.handle, float(nu), float(threshold),
             stream_ptr(self.stream), ptr(grad), None, ptr(v))
        return grad, float(v[0])

    def gradient_with_noise(self, psi, psi_prime, ensemble, nu=1.0, threshold=0.0):
        """(gradient, noise, value)."""
        grad = cbuf(psi_prime.num_params)
        noise = np.zeros(psi_prime.num_params)
        v = np.zeros(1)
        call("ann_kl_gradient", self._h, psi.handle, psi_prime.handle, ensemble.handle, float(nu), float(threshold),
             stream_ptr(self.stream), ptr(grad), ptr(noise), ptr(v))
        return grad, noise, float(v[0])

    def _stats(self):
        w = np.zeros(1)
        m = np.zeros(2)
        call("ann_kl_stats", self._h, ptr(w), ptr(m))
        return float(w[0]), complex(m[0], m[1])

    @property
    def total_weight(self) -> float:
        return self._stats()[0]

    @property
    def mean_deviation(self) -> complex:
        return self._stats()[1]

    @property
    def log_psi_scale(self) -> float:
        out = np.zeros(1)
        call("ann_kl_log_psi_scale", self._h, None, ptr(out))
        return float(out[0])

    @log_psi_scale.setter
    def log_psi_scale(self, value):
        v = np.array([float(value)])
        call("ann_kl_log_psi_scale", self._h, ptr(v), None)


# ----------------------------------------------------------------------------------
class Batch(_Handle):
    """Many (psi, operator, Monte Carlo ensemble[, TDVP]) instances of uneven size in one
    persistent sampling launch, with per-instance SR solves (this project's addition)."""

    _destroy = "ann_batch_destroy"

    def __init__(self, psis, operators, ensembles, tdvps=None, stream=None):
        _Handle.__init__(self)
        n = len(psis)
        self._members = (list(psis), list(operators), list(ensembles), None if tdvps is None else list(tdvps))
        arr = lambda objs: (ct.c_void_p * n)(*[o.handle.value for o in objs])
        self.stream = stream
        call("ann_batch_create", n, arr(psis), arr(operators), arr(ensembles),
             None if tdvps is None else arr(tdvps), ct.byref(self._h))
        self.n = n

    def sample(self):
        call("ann_batch_sample", self._h, stream_ptr(self.stream))

    def energies(self):
        out = cbuf(self.n)
        call("ann_batch_energies", self._h, ptr(out))
        return out

    def sr_step(self, diag_shift, lr):
        call("ann_batch_sr_step", self._h, float(diag_shift), float(lr), stream_ptr(self.stream))

    def capture_sr_step(self, diag_shift, lr, stream):
        call("ann_batch_graph_capture", self._h, float(diag_shift), float(lr), stream_ptr(stream))

    def launch_sr_step(self, stream):
        call("ann_batch_graph_launch", self._h, stream_ptr(stream))


# ----------------------------------------------------------------------------------
# free functions (main.cpp.template:495-540)
def _nwords(psi):
    return 2 if psi.N > 64 else 1


def log_psi_s(psi, spins) -> complex:
    """log psi of one configuration: Spins (or an int) or a PauliString."""
    if isinstance(spins, PauliString):
        return complex(log_psi_batch(psi, [spins])[0])
    w = _conf_words(spins, _nwords(psi))
    out = np.zeros(2)
    call("ann_log_psi_s", psi.handle, ptr(w), ptr(out))
    return complex(out[0], out[1])


def log_psi_batch(psi, confs) -> np.ndarray:
    confs = list(confs)
    if confs and isinstance(confs[0], PauliString):
        rows = _pauli_rows(confs)
        out = cbuf(len(rows))
        call("ann_log_psi_paulis", psi.handle, ptr(rows), len(rows), None, ptr(out))
        return out
    nw = _nwords(psi)
    arr = np.ascontiguousarray(np.concatenate([_conf_words(c, nw) for c in confs]) if confs else
                               np.zeros(0, np.uint64))
    out = cbuf(len(confs))
    call("ann_log_psi_batch", psi.handle, ptr(arr), len(confs), None, ptr(out))
    return out


def local_energies(psi, operator, confs) -> np.ndarray:
    """E_loc(s) of explicit configurations (ints, Spins or (n, 2) uint64 rows) on the device;
    a list of PauliStrings is read in the Pauli-string basis."""
    if len(confs) and isinstance(confs[0], PauliString):
        rows = _pauli_rows(confs)
        out = cbuf(len(rows))
        call("ann_local_energies_paulis", psi.handle, operator.handle, ptr(rows), len(rows), None, ptr(out))
        return out
    rows = _conf_rows(confs)
    nw = _nwords(psi)
    arr = np.ascontiguousarray(rows[:, :nw])
    out = cbuf(len(rows))
    call("ann_local_energies", psi.handle, operator.handle, ptr(arr), len(rows), None, ptr(out))
    return out


def psi_O_k(psi, spins) -> np.ndarray:
    out = cbuf(psi.num_params)
    if isinstance(spins, PauliString):
        call("ann_psi_O_k_paulis", psi.handle, ptr(_pauli_rows([spins])), ptr(out))
        return out
    w = _conf_words(spins, _nwords(psi))
    call("ann_psi_O_k", psi.handle, ptr(w), ptr(out))
    return out


def psi_O_k_vector(psi, ensemble) -> np.ndarray:
    out = cbuf(psi.num_params)
    call("ann_psi_O_k_vector", psi.handle, ensemble.handle, None, ptr(out))
    return out


def log_psi(psi, ensemble) -> complex:
    out = np.zeros(2)
    call("ann_log_psi", psi.handle, ensemble.handle, None, ptr(out))
    return complex(out[0], out[1])


def psi_vector(psi, ensemble) -> np.ndarray:
    out = cbuf(ensemble.num_steps)
    call("ann_psi_vector", psi.handle, ensemble.handle, None, ptr(out))
    return out


def log_psi_vector(psi, ensemble) -> np.ndarray:
    out = cbuf(ensemble.num_steps)
    call("ann_log_psi_vector", psi.handle, ensemble.handle, None, ptr(out))
    return out


def apply_operator(psi, operator, ensemble) -> np.ndarray:
    out = cbuf(ensemble.num_steps)
    call("ann_apply_operator", psi.handle, operator.handle, ensemble.handle, None, ptr(out))
    return out


def activation_function(z, layer=0, activation="poly") -> complex:
    z = complex(z)
    out = np.zeros(2)
    call("ann_activation_function", z.real, z.imag, int(layer), _ACT[activation], ptr(out))
    return complex(out[0], out[1])


# ----------------------------------------------------------------------------------
# autotuner (tuning.cu; this project's addition)
_KNOBS = {0: "rbm_mc.wpb", 1: "stats.slab", 2: "chol.update", 3: "rbm_mc.wsmem", 4: "chol.reserve",
          5: "chol.pair", 6: "rbm_mc.team"}


def autotune(operator, psi, ensemble, tdvp, diag_shift=1e-3, stream=None):
    """Times the candidates of every launch / tile knob on this workload and keeps the
    fastest in the tuning table (sampler warps per CTA, reduction slab rows, Cholesky
    trailing update). Returns {knob: {candidate: median ms}}."""
    rep = np.zeros(3 * 32)
    n = ct.c_uint()
    call("ann_autotune", tdvp.handle, operator.handle, psi.handle, ensemble.handle, float(diag_shift),
         stream_ptr(stream), ptr(rep), 32, ct.byref(n))
    out = {}
    for k in range(min(n.value, 32)):
        knob, cand, ms = rep[3 * k: 3 * k + 3]
        out.setdefault(_KNOBS[int(knob)], {})[int(cand)] = float(ms)
    return out


def tuning_table() -> dict:
    """The tuning table: {"dev<ordinal>/<knob>/<shape>": value}."""
    need = ct.c_size_t()
    call("ann_tuning_dump", None, 0, ct.byref(need))
    buf = ct.create_string_buffer(need.value + 1)
    call("ann_tuning_dump", buf, need.value + 1, ct.byref(need))
    out = {}
    for line in buf.value.decode().splitlines():
        k, v = line.rsplit(" ", 1)
        out[k] = int(v)
    return out


def set_tuning(table: dict, clear=False):
    if clear:
        call("ann_tuning_clear")
    for k, v in table.items():
        call("ann_tuning_set", k.encode(), int(v))


def save_tuning(path):
    import json
    import torch
    with open(path, "w") as f:
        json.dump({"device": torch.cuda.get_device_name(), "table": tuning_table()}, f, indent=1)


def load_tuning(path):
    """Loads a table saved by save_tuning; entries tuned on another GPU model are ignored."""
    import json
    import torch
    with open(path) as f:
        d = json.load(f)
    if d.get("device") == torch.cuda.get_device_name():
        set_tuning(d["table"])
        return True
    return False


def setDevice(device: int):
    call("ann_set_device", int(device))


def start_profiling():
    call("ann_profiler_start")


def stop_profiling():
    call("ann_profiler_stop")
