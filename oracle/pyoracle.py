"""ctypes front end of the FP64 oracle (oracle/liboracle.so) -- TEST INFRASTRUCTURE.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline legs import
this module. It is the checker: nothing in ``annongpu_gb300`` imports it.

``RefHarness`` wraps oracle/_ref/libref.so, the reference's own host code path
(built by ``make -C oracle ref`` where the reference checkout exists); it is used
only to (re)generate the golden fixtures under tests/golden/.
"""

from __future__ import annotations

import ctypes as ct
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
P = ct.c_void_p


def _ptr(x):
    return None if x is None else x.ctypes.data_as(ct.c_void_p)


def build_oracle(quiet: bool = True) -> str:
    so = os.path.join(HERE, "liboracle.so")
    src = [os.path.join(HERE, f) for f in ("oracle.cpp", "oracle.hpp")]
    if not os.path.exists(so) or any(os.path.getmtime(s) > os.path.getmtime(so) for s in src):
        subprocess.run(["make", "-C", HERE, "oracle"], check=True,
                       stdout=subprocess.DEVNULL if quiet else None)
    return so


class OrOp(ct.Structure):
    _fields_ = [("n", ct.c_uint), ("nw", ct.c_uint), ("a", P), ("b", P), ("coeff", P)]


class OrRbm(ct.Structure):
    _fields_ = [("N", ct.c_uint), ("M", ct.c_uint), ("C", ct.c_uint), ("conn", P), ("a", P), ("b", P),
                ("W", P), ("fw", P), ("lp_re", ct.c_double), ("lp_im", ct.c_double),
                ("a_in_log_psi", ct.c_int), ("activation", ct.c_int), ("layout", ct.c_int)]


class OrCnn(ct.Structure):
    _fields_ = [("extent", ct.c_uint * 3), ("num_layers", ct.c_uint), ("channels", P), ("connectivity", P),
                ("sym_classes", P), ("params", P), ("num_params", ct.c_uint), ("final_factor", ct.c_double),
                ("lp_re", ct.c_double), ("lp_im", ct.c_double), ("activation", ct.c_int)]


class OrDeep(ct.Structure):
    _fields_ = [("N", ct.c_uint), ("num_layers", ct.c_uint), ("sizes", P), ("connectivity", P),
                ("connections", P), ("params", P), ("fw", P), ("lp_re", ct.c_double), ("lp_im", ct.c_double),
                ("a_in_log_psi", ct.c_int), ("activation", ct.c_int), ("basis", ct.c_int)]


class OrClassical(ct.Structure):
    _fields_ = [("num_sites", ct.c_uint), ("n_features", ct.c_uint), ("feat_begin", P), ("nw", ct.c_uint),
                ("a", P), ("b", P), ("coeff", P), ("params", P), ("lp_re", ct.c_double), ("lp_im", ct.c_double),
                ("order", ct.c_int), ("ref", P)]


def nwords(N):
    return (N + 63) // 64


def conf_words(conf, N):
    """Python int (or array of words) -> uint64 word array of length nwords(N)."""
    if isinstance(conf, np.ndarray):
        return np.ascontiguousarray(conf, dtype=np.uint64).reshape(-1)
    return np.array([(int(conf) >> (64 * w)) & 0xFFFFFFFFFFFFFFFF for w in range(max(1, nwords(N)))],
                    dtype=np.uint64)


class OpArrays:
    """Keeps the numpy buffers of an operator alive next to its ctypes struct."""

    def __init__(self, expr, N):
        nw = max(1, nwords(N))
        a, b, c = expr.arrays(nw)
        self.a = np.ascontiguousarray(a)
        self.b = np.ascontiguousarray(b)
        self.c = np.ascontiguousarray(c.astype(np.complex128))
        self.struct = OrOp(len(c), nw, _ptr(self.a), _ptr(self.b), _ptr(self.c))


class RbmDesc:
    """An RBM-family wavefunction for the oracle.

    layout 0: reference PsiRBM, params = W (N x M), scalar final weight.
    layout 1: reference PsiDeep with one hidden layer, params = [a | b | W(C x M)].
    """

    def __init__(self, N, M, W, a=None, b=None, fw=None, conn=None, log_prefactor=0j,
                 a_in_log_psi=True, activation=0, layout=1):
        self.N, self.M = N, M
        self.W = np.ascontiguousarray(np.asarray(W, np.complex128).reshape(-1))
        self.C = self.W.size // M
        self.a = None if a is None else np.ascontiguousarray(np.asarray(a, np.complex128))
        self.b = None if b is None else np.ascontiguousarray(np.asarray(b, np.complex128))
        fw = np.ones(M, np.complex128) if fw is None else np.broadcast_to(np.asarray(fw, np.complex128), (M,))
        self.fw = np.ascontiguousarray(fw)
        self.conn = None if conn is None else np.ascontiguousarray(np.asarray(conn, np.uint32).reshape(-1))
        self.lp = complex(log_prefactor)
        self.struct = OrRbm(N, M, self.C, _ptr(self.conn), _ptr(self.a), _ptr(self.b), _ptr(self.W),
                            _ptr(self.fw), self.lp.real, self.lp.imag, int(a_in_log_psi), int(activation),
                            int(layout))

    @property
    def num_params(self):
        return (self.N + self.M + self.C * self.M) if self.struct.layout == 1 else self.C * self.M

    def params(self):
        if self.struct.layout == 0:
            return self.W.copy()
        a = np.zeros(self.N, np.complex128) if self.a is None else self.a
        b = np.zeros(self.M, np.complex128) if self.b is None else self.b
        return np.concatenate([a, b, self.W])


class CnnDesc:
    def __init__(self, extent, channels, connectivity, sym_classes, params, final_factor,
                 log_prefactor=0j, activation=0):
        self.extent = list(extent)
        self.channels = np.ascontiguousarray(np.asarray(channels, np.uint32))
        self.connectivity = np.ascontiguousarray(np.asarray(connectivity, np.uint32).reshape(-1, 3))
        self.N = int(np.prod(extent))
        self.sym = np.ascontiguousarray(np.asarray(sym_classes, np.uint32))
        self.params = np.ascontiguousarray(np.asarray(params, np.complex128))
        self.lp = complex(log_prefactor)
        self.struct = OrCnn((ct.c_uint * 3)(*self.extent), len(self.channels), _ptr(self.channels),
                            _ptr(self.connectivity), _ptr(self.sym), _ptr(self.params), self.params.size,
                            float(final_factor), self.lp.real, self.lp.imag, int(activation))

    @property
    def num_params(self):
        return self.params.size


class DeepDesc:
    """PsiDeep with any number of hidden layers for the oracle.

    ``connections[l]`` is the (C_l x M_l) block of layer l (entry (i, j): the i-th unit
    of the layer below read by unit j); params = [a | b_0 | W_0 | b_1 | W_1 | ...].
    """

    def __init__(self, N, connections, params, fw, log_prefactor=0j, a_in_log_psi=True, activation=0, paulis=False):
        """``paulis``: the Pauli-string basis (N = 3 input units per site; configurations are
        (a, b) word pairs)."""
        self.N = int(N)
        self.paulis = bool(paulis)
        blocks = [np.asarray(c, np.uint32) for c in connections]
        self.sizes = np.ascontiguousarray([b.shape[1] for b in blocks], np.uint32)
        self.connectivity = np.ascontiguousarray([b.shape[0] for b in blocks], np.uint32)
        self.connections = np.ascontiguousarray(np.concatenate([b.reshape(-1) for b in blocks]))
        self.params = np.ascontiguousarray(np.asarray(params, np.complex128))
        self.fw = np.ascontiguousarray(np.broadcast_to(np.asarray(fw, np.complex128), (int(self.sizes[-1]),)))
        self.lp = complex(log_prefactor)
        expect = self.N + int(sum(int(m) * (1 + int(c)) for m, c in zip(self.sizes, self.connectivity)))
        if self.params.size != expect:
            raise ValueError(f"params has {self.params.size} entries, the layer structure needs {expect}")
        self.struct = OrDeep(self.N, len(blocks), _ptr(self.sizes), _ptr(self.connectivity),
                             _ptr(self.connections), _ptr(self.params), _ptr(self.fw), self.lp.real, self.lp.imag,
                             int(a_in_log_psi), int(activation), int(self.paulis))

    @property
    def num_params(self):
        return self.params.size

    def words(self, conf):
        """A configuration as the oracle's words: spins as bits; Pauli strings as (a, b)."""
        if self.paulis:
            a, b = conf
            return np.array([a, b], np.uint64)
        return conf_words(conf, self.N)


class ClassicalDesc:
    """PsiClassical for the oracle: ``features`` is a list of Pauli expressions (one operator
    per feature), ``params`` one complex per feature, ``ref`` a DeepDesc (order 2) or None."""

    def __init__(self, num_sites, features, params, log_prefactor=0j, order=1, ref=None):
        self.N = int(num_sites)
        nw = max(1, nwords(self.N))
        a, b, c, beg = [], [], [], [0]
        for f in features:
            fa, fb, fc = f.arrays(nw)
            a.append(np.asarray(fa, np.uint64).reshape(-1, nw))
            b.append(np.asarray(fb, np.uint64).reshape(-1, nw))
            c.append(np.asarray(fc, np.complex128))
            beg.append(beg[-1] + len(fc))
        self.a = np.ascontiguousarray(np.concatenate(a))
        self.b = np.ascontiguousarray(np.concatenate(b))
        self.c = np.ascontiguousarray(np.concatenate(c))
        self.beg = np.ascontiguousarray(beg, np.uint32)
        self.params = np.ascontiguousarray(np.asarray(params, np.complex128))
        self.ref = ref
        self.order = int(order)
        self.lp = complex(log_prefactor)
        self.struct = OrClassical(self.N, len(features), _ptr(self.beg), nw, _ptr(self.a), _ptr(self.b),
                                  _ptr(self.c), _ptr(self.params), self.lp.real, self.lp.imag, self.order,
                                  ct.cast(ct.pointer(ref.struct), P) if ref is not None else None)

    @property
    def num_params(self):
        return self.params.size + (self.ref.num_params if self.order > 1 and self.ref is not None else 0)


class Oracle:
    def __init__(self):
        self.lib = ct.CDLL(build_oracle())
        L = self.lib
        L.or_rbm_num_params.restype = ct.c_uint
        L.or_rbm_mc_reference.restype = ct.c_uint
        L.or_philox4x32_10.argtypes = [ct.c_uint32, ct.c_uint32, P, P]
        L.or_rbm_mc_philox.argtypes = [P, P, ct.c_uint, ct.c_uint64, ct.c_uint, ct.c_uint, ct.c_uint,
                                       ct.c_int, P, ct.c_uint, ct.c_int, ct.c_int, P, P, P, P, P, P, P, P]
        L.or_rbm_mc_reference.argtypes = [P, P, ct.c_uint, ct.c_uint, ct.c_uint, ct.c_uint,
                                          P, P, P, P, P, P, P, ct.c_uint, P]
        L.or_activation.argtypes = [ct.c_double, ct.c_double, ct.c_uint, ct.c_int, P, P]
        L.or_deep_num_params.restype = ct.c_uint
        L.or_deep_mc_philox.argtypes = L.or_rbm_mc_philox.argtypes
        L.or_classical_num_params.restype = ct.c_uint

    # ---- RBM family ----
    def log_psi(self, psi: RbmDesc, conf):
        out = np.zeros(1, np.complex128)
        w = conf_words(conf, psi.N)
        self.lib.or_rbm_log_psi(ct.byref(psi.struct), _ptr(w), _ptr(out))
        return out[0]

    def O_k(self, psi: RbmDesc, conf):
        out = np.zeros(psi.num_params, np.complex128)
        w = conf_words(conf, psi.N)
        self.lib.or_rbm_O_k(ct.byref(psi.struct), _ptr(w), _ptr(out))
        return out

    def local_energy(self, psi: RbmDesc, expr, conf):
        op = OpArrays(expr, psi.N)
        out = np.zeros(1, np.complex128)
        w = conf_words(conf, psi.N)
        self.lib.or_rbm_local_energy(ct.byref(psi.struct), ct.byref(op.struct), _ptr(w), _ptr(out))
        return out[0]

    def exact(self, psi: RbmDesc, expr=None, want_S=True):
        np_ = psi.num_params
        dim = 1 << psi.N
        r = dict(
            E=np.zeros(1, np.complex128), fluct=np.zeros(3), grad=np.zeros(np_, np.complex128),
            tE=np.zeros(1, np.complex128), tE2=np.zeros(1), tO=np.zeros(np_, np.complex128),
            tF=np.zeros(np_, np.complex128), tS=np.zeros((np_, np_), np.complex128) if want_S else None,
            vec=np.zeros(dim, np.complex128), log_vec=np.zeros(dim, np.complex128), norm=np.zeros(1),
            mean_log_psi=np.zeros(1, np.complex128), O_sum=np.zeros(np_, np.complex128),
            eloc=np.zeros(dim, np.complex128))
        op = OpArrays(expr, psi.N) if expr is not None else None
        self.lib.or_rbm_exact(ct.byref(psi.struct), ct.byref(op.struct) if op else None,
                              *[_ptr(r[k]) for k in ("E", "fluct", "grad", "tE", "tE2", "tO", "tF", "tS",
                                                     "vec", "log_vec", "norm", "mean_log_psi", "O_sum",
                                                     "eloc")])
        return r

    def hsd_exact(self, psi: RbmDesc, psi_p: RbmDesc, expr, unitary, nu=1.0):
        """HilbertSpaceDistance over all 2^N configurations with the exact-summation weights
        |psi(s)|^2: the per-sample sums of source/network_functions/
        HilbertSpaceDistance.cu.template:16-86 and the distance / gradient of :118-168
        (gradient with respect to the parameters of psi_p). Returns (distance, gradient)."""
        r = self.exact(psi, expr, want_S=False)
        rp = self.exact(psi_p, None, want_S=False)
        lp, lpp, e = r["log_vec"], rp["log_vec"], r["eloc"]
        w = np.exp(2.0 * lp.real)
        d = np.conj(lpp - lp)
        if unitary:
            omega = np.exp(d) * e
            nxt = np.abs(e) ** 2
        else:
            omega = np.exp(e + d)
            nxt = np.exp(2.0 * e.real)
        ratio = np.exp(2.0 * (lpp.real - lp.real))
        om, pr, nn = np.sum(w * omega), np.sum(w * ratio), np.sum(w * nxt)
        u = abs(om) ** 2
        v = nn * pr
        dist = np.sqrt(max(1.0 - u / v, 1e-8))
        O = np.array([self.O_k(psi_p, s) for s in range(1 << psi.N)])
        oO = (w * omega) @ np.conj(O)
        rO = (w * ratio) @ np.conj(O)
        grad = -(np.conj(om) * oO * v - u * nn * rO) / v ** 2 / dist ** nu
        return dist, grad

    def mc_reference(self, psi: RbmDesc, expr, num_samples, num_sweeps, num_therm, seed=0, max_props=None):
        N = psi.N
        total = num_therm * N + num_samples * num_sweeps * N
        max_props = total if max_props is None else max_props
        op = OpArrays(expr, N)
        r = dict(sconf=np.zeros(num_samples, np.uint64), slp=np.zeros(num_samples, np.complex128),
                 seloc=np.zeros(num_samples, np.complex128), pconf=np.zeros(max_props, np.uint64),
                 psite=np.zeros(max_props, np.uint32), pu=np.zeros(max_props), pacc=np.zeros(max_props, np.uint8),
                 energy=np.zeros(1, np.complex128))
        n = self.lib.or_rbm_mc_reference(ct.byref(psi.struct), ct.byref(op.struct), num_samples, num_sweeps,
                                         num_therm, seed, *[_ptr(r[k]) for k in ("sconf", "slp", "seloc", "pconf",
                                                                                 "psite", "pu", "pacc")],
                                         max_props, _ptr(r["energy"]))
        r["num_props"] = n
        return r

    def tdvp_samples(self, psi: RbmDesc, expr, confs, weight, want_S=True):
        """The reference's TDVP accumulation over explicit configurations (uniform weight)."""
        np_ = psi.num_params
        op = OpArrays(expr, psi.N)
        c = np.ascontiguousarray(np.asarray(confs, np.uint64).reshape(-1))
        n = c.size // max(1, nwords(psi.N))
        r = dict(E=np.zeros(1, np.complex128), E2=np.zeros(1), O=np.zeros(np_, np.complex128),
                 F=np.zeros(np_, np.complex128), S=np.zeros((np_, np_), np.complex128) if want_S else None)
        self.lib.or_rbm_tdvp_samples(ct.byref(psi.struct), ct.byref(op.struct), _ptr(c), ct.c_uint(n),
                                     ct.c_double(weight), *[_ptr(r[k]) for k in ("E", "E2", "O", "F", "S")])
        return r

    def philox(self, key, ctr):
        out = np.zeros(4, np.uint32)
        c = np.asarray(ctr, np.uint32)
        self.lib.or_philox4x32_10(key & 0xFFFFFFFF, key >> 32, _ptr(c), _ptr(out))
        return out

    def mc_philox(self, psi: RbmDesc, expr, n_chains, seed, samples_per_chain, num_sweeps, num_therm,
                  move_kind=0, bonds=None, init=True, n_up=-1, conf=None, counter=None, _fn=None):
        N = psi.N
        pauli = getattr(psi, "paulis", False)
        nw = 2 if pauli else max(1, nwords(N))
        op = OpArrays(expr, N // 3 if pauli else N) if expr is not None else None
        conf = np.zeros(n_chains * nw, np.uint64) if conf is None else np.ascontiguousarray(conf, np.uint64).copy()
        counter = np.zeros(n_chains, np.uint64) if counter is None else np.ascontiguousarray(counter,
                                                                                            np.uint64).copy()
        ns = samples_per_chain * n_chains
        bonds_a = None if bonds is None else np.ascontiguousarray(np.asarray(bonds, np.uint32).reshape(-1))
        r = dict(sconf=np.zeros(ns * nw, np.uint64), slp=np.zeros(ns, np.complex128),
                 seloc=np.zeros(ns, np.complex128), acc=np.zeros(1, np.uint64), rej=np.zeros(1, np.uint64),
                 tie=np.zeros(1))
        fn = self.lib.or_rbm_mc_philox if _fn is None else _fn
        fn(ct.byref(psi.struct), ct.byref(op.struct) if op else None, n_chains, seed, samples_per_chain, num_sweeps,
           num_therm, move_kind, _ptr(bonds_a), 0 if bonds_a is None else bonds_a.size // 2, int(init), n_up,
           _ptr(conf), _ptr(counter), _ptr(r["sconf"]), _ptr(r["slp"]), _ptr(r["seloc"]), _ptr(r["acc"]),
           _ptr(r["rej"]), _ptr(r["tie"]))
        r["conf"] = conf
        r["counter"] = counter
        return r

    # ---- CNN ----
    def cnn_log_psi(self, psi: CnnDesc, conf):
        out = np.zeros(1, np.complex128)
        w = conf_words(conf, psi.N)
        self.lib.or_cnn_log_psi(ct.byref(psi.struct), _ptr(w), _ptr(out))
        return out[0]

    def cnn_O_k(self, psi: CnnDesc, conf):
        out = np.zeros(psi.num_params, np.complex128)
        w = conf_words(conf, psi.N)
        self.lib.or_cnn_O_k(ct.byref(psi.struct), _ptr(w), _ptr(out))
        return out

    def cnn_local_energy(self, psi: CnnDesc, expr, conf):
        op = OpArrays(expr, psi.N)
        out = np.zeros(1, np.complex128)
        w = conf_words(conf, psi.N)
        self.lib.or_cnn_local_energy(ct.byref(psi.struct), ct.byref(op.struct), _ptr(w), _ptr(out))
        return out[0]

    def cnn_exact(self, psi: CnnDesc, expr, want_S=False):
        np_ = psi.num_params
        r = dict(E=np.zeros(1, np.complex128), norm=np.zeros(1), tE=np.zeros(1, np.complex128), tE2=np.zeros(1),
                 tO=np.zeros(np_, np.complex128), tF=np.zeros(np_, np.complex128),
                 tS=np.zeros((np_, np_), np.complex128) if want_S else None)
        op = OpArrays(expr, psi.N)
        self.lib.or_cnn_exact(ct.byref(psi.struct), ct.byref(op.struct),
                              *[_ptr(r[k]) for k in ("E", "norm", "tE", "tE2", "tO", "tF", "tS")])
        return r

    # ---- PsiDeep, any depth ----
    def deep_log_psi(self, psi: DeepDesc, conf):
        out = np.zeros(1, np.complex128)
        w = psi.words(conf)
        self.lib.or_deep_log_psi(ct.byref(psi.struct), _ptr(w), _ptr(out))
        return out[0]

    def deep_O_k(self, psi: DeepDesc, conf):
        out = np.zeros(psi.num_params, np.complex128)
        w = psi.words(conf)
        self.lib.or_deep_O_k(ct.byref(psi.struct), _ptr(w), _ptr(out))
        return out

    def deep_local_energy(self, psi: DeepDesc, expr, conf):
        op = OpArrays(expr, psi.N // 3 if psi.paulis else psi.N)
        out = np.zeros(1, np.complex128)
        w = psi.words(conf)
        self.lib.or_deep_local_energy(ct.byref(psi.struct), ct.byref(op.struct), _ptr(w), _ptr(out))
        return out[0]

    def deep_exact(self, psi: DeepDesc, expr, want_S=False):
        np_ = psi.num_params
        r = dict(E=np.zeros(1, np.complex128), norm=np.zeros(1), tE=np.zeros(1, np.complex128), tE2=np.zeros(1),
                 tO=np.zeros(np_, np.complex128), tF=np.zeros(np_, np.complex128),
                 tS=np.zeros((np_, np_), np.complex128) if want_S else None)
        op = OpArrays(expr, psi.N // 3 if psi.paulis else psi.N)
        self.lib.or_deep_exact(ct.byref(psi.struct), ct.byref(op.struct),
                               *[_ptr(r[k]) for k in ("E", "norm", "tE", "tE2", "tO", "tF", "tS")])
        return r

    def cnn_mc_philox(self, psi: CnnDesc, expr, n_chains, seed, samples_per_chain, num_sweeps, num_therm,
                      move_kind=0, bonds=None, init=True, n_up=-1, conf=None, counter=None):
        return self.mc_philox(psi, expr, n_chains, seed, samples_per_chain, num_sweeps, num_therm, move_kind,
                              bonds, init, n_up, conf, counter, _fn=self.lib.or_cnn_mc_philox)

    def deep_mc_philox(self, psi: DeepDesc, expr, n_chains, seed, samples_per_chain, num_sweeps, num_therm,
                       move_kind=0, bonds=None, init=True, n_up=-1, conf=None, counter=None):
        return self.mc_philox(psi, expr, n_chains, seed, samples_per_chain, num_sweeps, num_therm, move_kind,
                              bonds, init, n_up, conf, counter, _fn=self.lib.or_deep_mc_philox)

    # ---- PsiClassical and KullbackLeibler ----
    def classical_log_psi(self, psi: ClassicalDesc, conf):
        out = np.zeros(1, np.complex128)
        self.lib.or_classical_log_psi(ct.byref(psi.struct), _ptr(conf_words(conf, psi.N)), _ptr(out))
        return out[0]

    def classical_O_k(self, psi: ClassicalDesc, conf):
        out = np.zeros(psi.num_params, np.complex128)
        self.lib.or_classical_O_k(ct.byref(psi.struct), _ptr(conf_words(conf, psi.N)), _ptr(out))
        return out

    def classical_local_energy(self, psi: ClassicalDesc, expr, conf):
        op = OpArrays(expr, psi.N)
        out = np.zeros(1, np.complex128)
        self.lib.or_classical_local_energy(ct.byref(psi.struct), ct.byref(op.struct), _ptr(conf_words(conf, psi.N)),
                                           _ptr(out))
        return out[0]

    def classical_exact(self, psi: ClassicalDesc, expr, want_S=False):
        np_ = psi.num_params
        r = dict(E=np.zeros(1, np.complex128), norm=np.zeros(1), tE=np.zeros(1, np.complex128), tE2=np.zeros(1),
                 tO=np.zeros(np_, np.complex128), tF=np.zeros(np_, np.complex128),
                 tS=np.zeros((np_, np_), np.complex128) if want_S else None)
        op = OpArrays(expr, psi.N)
        self.lib.or_classical_exact(ct.byref(psi.struct), ct.byref(op.struct),
                                    *[_ptr(r[k]) for k in ("E", "norm", "tE", "tE2", "tO", "tF", "tS")])
        return r

    def kl(self, psi: ClassicalDesc, psi_prime: DeepDesc, confs=None, wprime=None, threshold=0.0, last_mean=0j,
           log_psi_scale=1.0, nu=1.0, gradient=True, noise=False):
        """KullbackLeibler of psi against psi_prime over rows (confs (n, 2) uint64, weights w')
        of psi_prime's ensemble, or exact summation when confs is None."""
        np_ = psi_prime.num_params
        c = None if confs is None else np.ascontiguousarray(np.asarray(confs, np.uint64).reshape(-1, 2))
        w = None if wprime is None else np.ascontiguousarray(np.asarray(wprime, np.float64))
        lm = np.array([complex(last_mean).real, complex(last_mean).imag])
        r = dict(value=np.zeros(1), grad=np.zeros(np_, np.complex128) if gradient else None,
                 noise=np.zeros(np_) if noise else None, total_weight=np.zeros(1),
                 mean_deviation=np.zeros(1, np.complex128))
        self.lib.or_kl(ct.byref(psi.struct), ct.byref(psi_prime.struct), _ptr(c), _ptr(w),
                       ct.c_uint(0 if c is None else len(c)), ct.c_double(threshold), _ptr(lm),
                       ct.c_double(log_psi_scale), ct.c_double(nu), _ptr(r["value"]), _ptr(r["grad"]),
                       _ptr(r["noise"]), _ptr(r["total_weight"]), _ptr(r["mean_deviation"]))
        return r

    def pauli_apply(self, a, b, conf, N):
        nw = max(1, nwords(N))
        aw, bw, cw = conf_words(a, N), conf_words(b, N), conf_words(conf, N)
        f = np.zeros(1, np.complex128)
        out = np.zeros(nw, np.uint64)
        self.lib.or_pauli_apply(_ptr(aw), _ptr(bw), nw, _ptr(cw), _ptr(f), _ptr(out))
        return f[0], out

    def activation(self, z, layer=0, exact=False):
        f = np.zeros(1, np.complex128)
        df = np.zeros(1, np.complex128)
        self.lib.or_activation(z.real, z.imag, layer, int(exact), _ptr(f), _ptr(df))
        return f[0], df[0]


class RefHarness:
    """The reference's own host path (oracle/_ref/libref.so). Fixture generation only."""

    def __init__(self, path=None):
        path = path or os.path.join(HERE, "_ref", "libref.so")
        self.lib = ct.CDLL(path)
        self.lib.ref_deep_mc.restype = ct.c_uint
        self.lib.ref_rbm_mc.restype = ct.c_uint
        U, D = ct.c_uint, ct.c_double
        self.lib.ref_deep_log_psi_s.argtypes = [U, U, U, P, P, P, P, ct.c_uint64, P]
        self.lib.ref_deep_O_k.argtypes = [U, U, U, P, P, P, P, ct.c_uint64, P]
        self.lib.ref_rbm_log_psi_s.argtypes = [U, U, P, P, P, ct.c_uint64, P]
        self.lib.ref_rbm_O_k.argtypes = [U, U, P, P, P, ct.c_uint64, P]
        self.lib.ref_cnn_log_psi_s.argtypes = [P, U, P, P, P, P, U, D, P, ct.c_uint64, P]
        self.lib.ref_cnn_O_k.argtypes = [P, U, P, P, P, P, U, D, P, ct.c_uint64, P]
        self.lib.ref_cnn_exact_energy.argtypes = [P, U, P, P, P, P, U, D, P, P, P, P, U, P, P]
        self.lib.ref_activation.argtypes = [D, D, U, P, P]
        self.lib.ref_deepml_num_params.restype = U
        self.lib.ref_deepml_num_params.argtypes = [U, U, P, P, P, P, P, P]
        self.lib.ref_deepml_log_psi_s.argtypes = [U, U, P, P, P, P, P, P, ct.c_uint64, P]
        self.lib.ref_deepml_O_k.argtypes = [U, U, P, P, P, P, P, P, ct.c_uint64, P]
        self.lib.ref_deepml_pauli_log_psi_s.argtypes = [U, U, P, P, P, P, P, P, ct.c_uint64, ct.c_uint64, P]
        self.lib.ref_deepml_pauli_O_k.argtypes = [U, U, P, P, P, P, P, P, ct.c_uint64, ct.c_uint64, P]
        self.lib.ref_classical_log_psi_s.argtypes = [P, ct.c_uint64, P]
        self.lib.ref_classical_O_k.argtypes = [P, ct.c_uint64, P]
        self.lib.ref_pauli_apply.argtypes = [ct.c_uint64, ct.c_uint64, ct.c_uint64, U, P, P]
        self.lib.ref_deep_hsd_exact.argtypes = [U, U, U, P, P, P, P, P, P, P, P, P, P, U, ct.c_int, D, P, P]
