"""Generate the golden fixtures in this directory from the reference's own host code.

Runs the reference implementation's CPU path (oracle/_ref/libref.so, built by
``make -C oracle ref`` from the reference checkout) on small seeded cases and
stores inputs and outputs as .npz files. The fixtures pin the FP64 oracle
(oracle/oracle.cpp) and, through it, the CUDA path. The reference checkout is
needed only to regenerate them:

    make -C oracle ref REF=<reference checkout> && python tests/golden/gen_golden.py [deep_ml | deep_pauli | classical | hsd]
"""

import ctypes as ct
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from annongpu_gb300.expression import sigma_x, sigma_y, sigma_z, transverse_field_ising_1d  # noqa: E402
from pyoracle import RefHarness  # noqa: E402


def P(x):
    return x.ctypes.data_as(ct.c_void_p)


def cplx(rng, shape, scale):
    return (scale * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))).astype(np.complex128)


def mixed_hamiltonian(N):
    """TFIM plus strings with one, two and three sigma_y factors (phase coverage)."""
    H = transverse_field_ising_1d(N, h=0.9, J=1.1)
    H = H + 0.3 * sigma_y(1) * sigma_y(2) + 0.2 * sigma_x(0) * sigma_z(3)
    H = H + 0.15 * sigma_y(4) + 0.05 * sigma_y(0) * sigma_y(2) * sigma_y(5) + 0.1 * sigma_z(2)
    return H


def op_arrays(H):
    a, b, c = H.arrays(1)
    return (np.ascontiguousarray(a[:, 0]), np.ascontiguousarray(b[:, 0]),
            np.ascontiguousarray(c.astype(np.complex128)), len(c))


def exact_outputs(np_, N):
    dim = 1 << N
    return dict(E=np.zeros(1, np.complex128), fluct=np.zeros(3), grad=np.zeros(np_, np.complex128),
                tE=np.zeros(1, np.complex128), tE2=np.zeros(1), tO=np.zeros(np_, np.complex128),
                tF=np.zeros(np_, np.complex128), tS=np.zeros((np_, np_), np.complex128),
                vec=np.zeros(dim, np.complex128), norm=np.zeros(1), mlp=np.zeros(1, np.complex128),
                O_sum=np.zeros(np_, np.complex128))


KEYS = ("E", "fluct", "grad", "tE", "tE2", "tO", "tF", "tS", "vec", "norm", "mlp", "O_sum")


def mc_outputs(num_samples, total_props):
    return dict(sconf=np.zeros(num_samples, np.uint64), slp=np.zeros(num_samples, np.complex128),
                seloc=np.zeros(num_samples, np.complex128), pconf=np.zeros(total_props, np.uint64),
                psite=np.zeros(total_props, np.uint32), mc_energy=np.zeros(1, np.complex128))


def gen_rbm(ref, rng):
    N, M = 8, 8
    W = cplx(rng, (N, M), 0.15)
    fw = np.array([0.8 + 0.3j])
    lp = np.array([0.1 - 0.2j])
    H = mixed_hamiltonian(N)
    a, b, c, n = op_arrays(H)
    confs = rng.integers(0, 1 << N, 12).astype(np.uint64)
    out = {"N": N, "M": M, "W": W, "fw": fw, "lp": lp, "op_a": a, "op_b": b, "op_c": c, "confs": confs}
    lps, oks = [], []
    for s in confs:
        r = np.zeros(1, np.complex128)
        ref.lib.ref_rbm_log_psi_s(N, M, P(W), P(fw), P(lp), int(s), P(r))
        lps.append(r[0])
        o = np.zeros(N * M, np.complex128)
        ref.lib.ref_rbm_O_k(N, M, P(W), P(fw), P(lp), int(s), P(o))
        oks.append(o)
    out["log_psi"] = np.array(lps)
    out["O_k"] = np.array(oks)
    ex = exact_outputs(N * M, N)
    ref.lib.ref_rbm_exact(N, M, P(W), P(fw), P(lp), P(a), P(b), P(c), n, *[P(ex[k]) for k in KEYS])
    out.update({"ex_" + k: v for k, v in ex.items()})
    ns, sw, th = 40, 2, 3
    total = th * N + ns * sw * N
    mc = mc_outputs(ns, total)
    nprop = ref.lib.ref_rbm_mc(N, M, P(W), P(fw), P(lp), P(a), P(b), P(c), n, ns, sw, th,
                               *[P(mc[k]) for k in ("sconf", "slp", "seloc", "pconf", "psite")], total,
                               P(mc["mc_energy"]))
    assert nprop == total, (nprop, total)
    out.update({"mc_" + k: v for k, v in mc.items()})
    out["mc_params"] = np.array([ns, sw, th])
    np.savez_compressed(os.path.join(HERE, "rbm_n8_m8.npz"), **out)


def gen_deep(ref, rng, name, N, M, C, conn, with_S=True, mc=True, confs_n=12):
    np_ = N + M + C * M
    params = np.concatenate([cplx(rng, N, 0.05), cplx(rng, M, 0.05), cplx(rng, C * M, 0.12)])
    fw = (1.0 + cplx(rng, M, 0.1)).astype(np.complex128)
    lp = np.array([-0.05 + 0.3j])
    H = mixed_hamiltonian(N) if N >= 6 else transverse_field_ising_1d(N)
    a, b, c, n = op_arrays(H)
    connp = None if conn is None else np.ascontiguousarray(conn.astype(np.uint32).reshape(-1))
    cp = P(connp) if connp is not None else None
    confs = rng.integers(0, 1 << N, confs_n).astype(np.uint64)
    out = {"N": N, "M": M, "C": C, "params": params, "fw": fw, "lp": lp, "op_a": a, "op_b": b, "op_c": c,
           "confs": confs}
    if connp is not None:
        out["conn"] = connp
    lps, oks = [], []
    for s in confs:
        r = np.zeros(1, np.complex128)
        ref.lib.ref_deep_log_psi_s(N, M, C, cp, P(params), P(fw), P(lp), int(s), P(r))
        lps.append(r[0])
        o = np.zeros(np_, np.complex128)
        ref.lib.ref_deep_O_k(N, M, C, cp, P(params), P(fw), P(lp), int(s), P(o))
        oks.append(o)
    out["log_psi"] = np.array(lps)
    out["O_k"] = np.array(oks)
    ex = exact_outputs(np_, N)
    ref.lib.ref_deep_exact(N, M, C, cp, P(params), P(fw), P(lp), P(a), P(b), P(c), n, *[P(ex[k]) for k in KEYS])
    if not with_S:
        # keep the fixture small: a checksum and a strided sample of S
        S = ex.pop("tS")
        out["ex_tS_trace"] = np.array([np.trace(S)])
        out["ex_tS_fro"] = np.array([np.linalg.norm(S)])
        idx = np.arange(0, np_ * np_, 97)
        out["ex_tS_idx"] = idx
        out["ex_tS_sample"] = S.reshape(-1)[idx]
        ex.pop("vec")
    out.update({"ex_" + k: v for k, v in ex.items()})
    if mc:
        ns, sw, th = 30, 1, 4
        total = th * N + ns * sw * N
        m = mc_outputs(ns, total)
        nprop = ref.lib.ref_deep_mc(N, M, C, cp, P(params), P(fw), P(lp), P(a), P(b), P(c), n, ns, sw, th,
                                    *[P(m[k]) for k in ("sconf", "slp", "seloc", "pconf", "psite")], total,
                                    P(m["mc_energy"]))
        assert nprop == total
        out.update({"mc_" + k: v for k, v in m.items()})
        out["mc_params"] = np.array([ns, sw, th])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)


def gen_cnn(ref, rng):
    extent = np.array([1, 4, 4], np.uint32)
    channels = np.array([2, 2], np.uint32)
    connectivity = np.array([[1, 3, 3], [1, 2, 2]], np.uint32)
    N = 16
    classes = np.zeros(N, np.uint32)
    classes[N // 2:] = 1  # two symmetry classes
    ncls = 2
    np_ = (2 * 1 * ncls * 9) + (2 * 2 * ncls * 4)
    params = cplx(rng, np_, 0.15)
    ff = 0.7
    lp = np.array([0.02 + 0.01j])
    H = transverse_field_ising_1d(N, h=0.8) + 0.2 * sigma_y(3) * sigma_y(7)
    a, b, c, n = op_arrays(H)
    confs = rng.integers(0, 1 << N, 10).astype(np.uint64)
    lps, oks = [], []
    for s in confs:
        r = np.zeros(1, np.complex128)
        ref.lib.ref_cnn_log_psi_s(P(extent), 2, P(channels), P(connectivity), P(classes), P(params), np_, ff,
                                  P(lp), int(s), P(r))
        lps.append(r[0])
        o = np.zeros(np_, np.complex128)
        ref.lib.ref_cnn_O_k(P(extent), 2, P(channels), P(connectivity), P(classes), P(params), np_, ff,
                            P(lp), int(s), P(o))
        oks.append(o)
    E = np.zeros(1, np.complex128)
    norm = np.zeros(1)
    ref.lib.ref_cnn_exact_energy(P(extent), 2, P(channels), P(connectivity), P(classes), P(params), np_, ff, P(lp),
                                 P(a), P(b), P(c), n, P(E), P(norm))
    np.savez_compressed(os.path.join(HERE, "cnn_4x4.npz"), extent=extent, channels=channels,
                        connectivity=connectivity, classes=classes, params=params, ff=np.array([ff]), lp=lp,
                        op_a=a, op_b=b, op_c=c, confs=confs, log_psi=np.array(lps), O_k=np.array(oks),
                        ex_E=E, ex_norm=norm)


def builder_connections(N, M, C):
    """Connection blocks of the reference's deep-network constructor for a 1-d input
    (pyANNonGPU/new_neural_network.py:88-112): unit j of a layer reads (j * delta + i) % n."""
    out = []
    for n, m, c in zip([N] + M[:-1], M, C):
        delta = 1 if m > n else (n // m if n % m == 0 else c)
        out.append(np.array([[(j * delta + i) % n for j in range(m)] for i in range(c)], np.uint32))
    return out


def gen_deep_ml(ref, rng, name, N, M, C):
    """PsiDeep with several hidden layers through the reference's own kernel."""
    blocks = builder_connections(N, M, C)
    sizes = np.array(M, np.uint32)
    conn_c = np.array(C, np.uint32)
    conn = np.ascontiguousarray(np.concatenate([b.reshape(-1) for b in blocks]))
    np_ = N + sum(m * (1 + c) for m, c in zip(M, C))
    params = cplx(rng, np_, 0.15)
    fw = (1.0 + cplx(rng, M[-1], 0.1)).astype(np.complex128)
    lp = np.array([0.03 - 0.2j])
    H = mixed_hamiltonian(N) if N >= 6 else transverse_field_ising_1d(N, h=0.9, J=1.1)
    a, b, c, n = op_arrays(H)
    confs = np.arange(1 << N, dtype=np.uint64) if N <= 4 else rng.integers(0, 1 << N, 12).astype(np.uint64)
    args = (N, len(M), P(sizes), P(conn_c), P(conn), P(params), P(fw), P(lp))
    assert ref.lib.ref_deepml_num_params(*args) == np_
    lps, oks = [], []
    for s in confs:
        r = np.zeros(1, np.complex128)
        ref.lib.ref_deepml_log_psi_s(*args, int(s), P(r))
        lps.append(r[0])
        o = np.zeros(np_, np.complex128)
        ref.lib.ref_deepml_O_k(*args, int(s), P(o))
        oks.append(o)
    ex = exact_outputs(np_, N)
    ref.lib.ref_deepml_exact(*args, P(a), P(b), P(c), n, *[P(ex[k]) for k in KEYS])
    out = {"N": N, "sizes": sizes, "connectivity": conn_c, "conn": conn, "params": params, "fw": fw, "lp": lp,
           "op_a": a, "op_b": b, "op_c": c, "confs": confs, "log_psi": np.array(lps), "O_k": np.array(oks)}
    out.update({"ex_" + k: v for k, v in ex.items()})
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)


def gen_deep_pauli(ref, rng, name, num_sites, M, C):
    """PsiDeep over the Pauli-string basis (3 input units per site) through the reference's
    own kernel, ExactSummationPaulis and Pauli-string operator products."""
    N = 3 * num_sites
    blocks = builder_connections(N, M, C)
    sizes = np.array(M, np.uint32)
    conn_c = np.array(C, np.uint32)
    conn = np.ascontiguousarray(np.concatenate([b.reshape(-1) for b in blocks]))
    np_ = N + sum(m * (1 + c) for m, c in zip(M, C))
    params = cplx(rng, np_, 0.15)
    fw = (1.0 + cplx(rng, M[-1], 0.1)).astype(np.complex128)
    lp = np.array([0.1 - 0.3j])
    H = transverse_field_ising_1d(num_sites, h=0.7) + 0.3 * sigma_y(0) * sigma_x(1)
    H = H + 0.2 * sigma_z(num_sites - 1) * sigma_y(1) + 0.15 * sigma_y(2)
    a, b, c, n = op_arrays(H)
    pa = rng.integers(0, 1 << num_sites, 12).astype(np.uint64)
    pb = rng.integers(0, 1 << num_sites, 12).astype(np.uint64)
    args = (N, len(M), P(sizes), P(conn_c), P(conn), P(params), P(fw), P(lp))
    lps, oks = [], []
    for x, y in zip(pa, pb):
        r = np.zeros(1, np.complex128)
        ref.lib.ref_deepml_pauli_log_psi_s(*args, int(x), int(y), P(r))
        lps.append(r[0])
        o = np.zeros(np_, np.complex128)
        ref.lib.ref_deepml_pauli_O_k(*args, int(x), int(y), P(o))
        oks.append(o)
    ex = exact_outputs(np_, 2 * num_sites)
    ref.lib.ref_deepml_pauli_exact(*args, P(a), P(b), P(c), n, *[P(ex[k]) for k in KEYS])
    out = {"num_sites": num_sites, "N": N, "sizes": sizes, "connectivity": conn_c, "conn": conn, "params": params,
           "fw": fw, "lp": lp, "op_a": a, "op_b": b, "op_c": c, "conf_a": pa, "conf_b": pb, "log_psi": np.array(lps),
           "O_k": np.array(oks)}
    out.update({"ex_" + k: v for k, v in ex.items()})
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)


class _DeepML(ct.Structure):
    _fields_ = [("N", ct.c_uint), ("L", ct.c_uint), ("sizes", ct.c_void_p), ("connectivity", ct.c_void_p),
                ("conn", ct.c_void_p), ("params", ct.c_void_p), ("final_w", ct.c_void_p), ("log_pref", ct.c_void_p),
                ("num_sites", ct.c_uint)]


class _Classical(ct.Structure):
    _fields_ = [("num_sites", ct.c_uint), ("n_features", ct.c_uint), ("feat_begin", ct.c_void_p),
                ("a", ct.c_void_p), ("b", ct.c_void_p), ("coeff", ct.c_void_p), ("params", ct.c_void_p),
                ("log_pref", ct.c_void_p), ("order", ct.c_uint), ("ref", ct.c_void_p)]


def _deep_arrays(rng, N, M, C, scale):
    blocks = builder_connections(N, M, C)
    np_ = N + sum(m * (1 + c) for m, c in zip(M, C))
    d = dict(sizes=np.array(M, np.uint32), connectivity=np.array(C, np.uint32),
             conn=np.ascontiguousarray(np.concatenate([b.reshape(-1) for b in blocks])),
             params=cplx(rng, np_, scale), fw=(1.0 + cplx(rng, M[-1], 0.1)).astype(np.complex128),
             lp=np.array([0.02 + 0.1j]))
    st = _DeepML(N, len(M), P(d["sizes"]), P(d["connectivity"]), P(d["conn"]), P(d["params"]), P(d["fw"]),
                 P(d["lp"]), 0)
    return d, st


def gen_classical_kl(ref, rng, name, S, features, order, ref_shape, threshold):
    """PsiClassical (features = one Pauli expression each; order 2 with a PsiDeep reference)
    and KullbackLeibler against a PsiDeep psi_prime, through the reference's own kernels."""
    beg, fa, fb, fc = [0], [], [], []
    for f in features:
        a, b, c, n = op_arrays(f)
        fa.append(a)
        fb.append(b)
        fc.append(c)
        beg.append(beg[-1] + n)
    beg = np.array(beg, np.uint32)
    fa, fb, fc = (np.ascontiguousarray(np.concatenate(x)) for x in (fa, fb, fc))
    K = len(features)
    theta = cplx(rng, K, 0.2)
    lp = np.array([0.1 - 0.2j])
    out = {"num_sites": S, "order": order, "feat_begin": beg, "feat_a": fa, "feat_b": fb, "feat_c": fc,
           "theta": theta, "lp": lp, "threshold": np.array([threshold])}
    refst = None
    if ref_shape is not None:
        rd, refst = _deep_arrays(rng, S, *ref_shape, 0.1)
        out.update({"ref_" + k: v for k, v in rd.items()})
    cd = _Classical(S, K, P(beg), P(fa), P(fb), P(fc), P(theta), P(lp), order,
                    ct.cast(ct.pointer(refst), ct.c_void_p) if refst is not None else None)
    np_ = K + (int(rd["params"].size) if refst is not None else 0)
    lps, oks = [], []
    for s in range(1 << S):
        r = np.zeros(1, np.complex128)
        ref.lib.ref_classical_log_psi_s(ct.byref(cd), ct.c_uint64(s), P(r))
        lps.append(r[0])
        o = np.zeros(np_, np.complex128)
        ref.lib.ref_classical_O_k(ct.byref(cd), ct.c_uint64(s), P(o))
        oks.append(o)
    out["log_psi"] = np.array(lps)
    out["O_k"] = np.array(oks)
    H = transverse_field_ising_1d(S, h=0.8) + 0.3 * sigma_y(0) * sigma_y(1)
    a, b, c, n = op_arrays(H)
    out.update({"op_a": a, "op_b": b, "op_c": c})
    ex = exact_outputs(np_, S)
    ref.lib.ref_classical_exact(ct.byref(cd), P(a), P(b), P(c), ct.c_uint(n), *[P(ex[k]) for k in KEYS])
    out.update({"ex_" + k: v for k, v in ex.items()})
    pd, pst = _deep_arrays(rng, S, [2 * S], [3], 0.15)
    out.update({"prime_" + k: v for k, v in pd.items()})
    npp = int(pd["params"].size)
    val = np.zeros(3)
    g = np.zeros(npp, np.complex128)
    g2 = np.zeros(npp, np.complex128)
    nz = np.zeros(npp)
    o4 = np.zeros(4)
    ref.lib.ref_kl_exact(ct.byref(cd), ct.byref(pst), ct.c_double(threshold), ct.c_double(1.0), P(val), P(g), P(g2),
                         P(nz), P(o4))
    out.update({"kl_value": val, "kl_grad": g, "kl_grad_noise_call": g2, "kl_noise": nz, "kl_out4": o4})
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)


def gen_classical_all(ref):
    from annongpu_gb300.expression import PauliExpression

    def terms(expr):
        a, b, c = expr.arrays(1)
        return [PauliExpression({(int(a[k, 0]), int(b[k, 0])): c[k]}) for k in range(len(c))]
    rng = np.random.default_rng(20261206)
    # the reference test suite's classical-network shapes (test/conftest.py)
    gen_classical_kl(ref, rng, "classical_s4_order2_deep", 4, terms(sigma_z(0) * sigma_y(1) + 1.1 * sigma_x(0)), 2,
                     ([4], [4]), 0.0)
    gen_classical_kl(ref, rng, "classical_s6_order1", 6,
                     terms(sigma_z(0) * sigma_x(1) * sigma_z(2) + sigma_y(0) + sigma_x(0) * sigma_x(1)), 1, None, 0.05)


def gen_kats(ref, rng):
    zs = cplx(rng, 24, 0.6)
    f = np.zeros((2, 24), np.complex128)
    df = np.zeros((2, 24), np.complex128)
    for layer in (0, 1):
        for k, z in enumerate(zs):
            o1 = np.zeros(1, np.complex128)
            o2 = np.zeros(1, np.complex128)
            ref.lib.ref_activation(z.real, z.imag, layer, P(o1), P(o2))
            f[layer, k], df[layer, k] = o1[0], o2[0]
    N = 12
    na = 64
    pa = rng.integers(0, 1 << N, na).astype(np.uint64)
    pb = rng.integers(0, 1 << N, na).astype(np.uint64)
    pc = rng.integers(0, 1 << N, na).astype(np.uint64)
    fac = np.zeros(na, np.complex128)
    oc = np.zeros(na, np.uint64)
    for k in range(na):
        o1 = np.zeros(1, np.complex128)
        o2 = np.zeros(1, np.uint64)
        ref.lib.ref_pauli_apply(int(pa[k]), int(pb[k]), int(pc[k]), N, P(o1), P(o2))
        fac[k], oc[k] = o1[0], o2[0]
    np.savez_compressed(os.path.join(HERE, "kats.npz"), z=zs, f=f, df=df, pauli_N=np.array([N]), pauli_a=pa,
                        pauli_b=pb, pauli_conf=pc, pauli_factor=fac, pauli_out=oc)


def main(only=None):
    ref = RefHarness()
    if only == "deep_ml":
        gen_deep_ml_all(ref)
        return
    if only == "deep_pauli":
        gen_deep_pauli_all(ref)
        return
    if only == "classical":
        gen_classical_all(ref)
        return
    if only == "hsd":
        gen_hsd_all(ref)
        return
    rng = np.random.default_rng(20261203)
    gen_kats(ref, rng)
    gen_rbm(ref, rng)
    gen_deep(ref, rng, "deep_n8_m8", 8, 8, 8, None)
    n, m, c = 6, 12, 3
    conn = np.array([[(j * 1 + i) % n for j in range(m)] for i in range(c)])
    gen_deep(ref, rng, "deep_n6_m12_c3", n, m, c, conn)
    gen_deep(ref, rng, "deep_n16_m16", 16, 16, 16, None, with_S=False, mc=False, confs_n=6)
    gen_cnn(ref, rng)
    gen_deep_ml_all(ref)
    gen_deep_pauli_all(ref)
    gen_classical_all(ref)
    gen_hsd_all(ref)
    print("fixtures written to", HERE)


def gen_hsd(ref, rng, name, N, M):
    """HilbertSpaceDistance of psi' to U psi over all 2^N configurations, both one-hidden-layer
    PsiDeep with full connectivity, in the unitary form (U = 1 + i t H) and the exponential
    form (operator i t H): distance() and gradient() for nu = 1 and nu = 0.5."""
    C = N
    np_ = N + M + C * M

    def draw(scale):
        return np.concatenate([cplx(rng, N, 0.05), cplx(rng, M, 0.05), cplx(rng, C * M, scale)])

    params, params_p = draw(0.1), draw(0.12)
    fw = (1.0 + cplx(rng, M, 0.1)).astype(np.complex128)
    fw_p = (1.0 + cplx(rng, M, 0.1)).astype(np.complex128)
    lp, lp_p = np.array([0.02 - 0.1j]), np.array([-0.03 + 0.2j])
    H = mixed_hamiltonian(N)
    t = 1e-2
    out = {"N": N, "M": M, "C": C, "params": params, "fw": fw, "lp": lp, "params_p": params_p, "fw_p": fw_p,
           "lp_p": lp_p, "t": np.array([t])}
    from annongpu_gb300.expression import identity
    for form, expr, unitary in (("unitary", identity() + 1j * t * H, 1), ("exponential", 1j * t * H, 0)):
        a, b, c, n = op_arrays(expr)
        out[f"{form}_op_a"], out[f"{form}_op_b"], out[f"{form}_op_c"] = a, b, c
        for nu in (1.0, 0.5):
            dist = np.zeros(2)
            grad = np.zeros(np_, np.complex128)
            ref.lib.ref_deep_hsd_exact(N, M, C, None, P(params), P(fw), P(lp), P(params_p), P(fw_p), P(lp_p),
                                       P(a), P(b), P(c), n, unitary, nu, P(dist), P(grad))
            tag = f"{form}_nu{nu:g}"
            out[f"{tag}_dist"] = dist
            out[f"{tag}_grad"] = grad
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)


def gen_hsd_all(ref):
    rng = np.random.default_rng(20261206)
    gen_hsd(ref, rng, "hsd_n8_m8", 8, 8)


def gen_deep_ml_all(ref):
    # own generator, so these fixtures do not depend on the ones above
    rng = np.random.default_rng(20261204)
    # the shape of the reference test suite's deep-network fixture (test/conftest.py)
    gen_deep_ml(ref, rng, "deep3_n3_18_9_3", 3, [18, 9, 3], [3, 2, 3])
    gen_deep_ml(ref, rng, "deep3_n8_16_8_4", 8, [16, 8, 4], [4, 4, 2])
    gen_deep_ml(ref, rng, "deep2_n6_12_6", 6, [12, 6], [3, 4])


def gen_deep_pauli_all(ref):
    rng = np.random.default_rng(20261205)
    gen_deep_pauli(ref, rng, "deep_pauli_s3_9_6", 3, [9, 6], [3, 3])
    gen_deep_pauli(ref, rng, "deep_pauli_s4_12_6_3", 4, [12, 6, 3], [4, 4, 2])


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
