"""PsiDeep with several hidden layers on the GPU: against the reference's own kernel
(tests/golden/deep*_*.npz) and the FP64 oracle -- log psi, back-propagated O_k, local
energies, exact-summation TDVP quantities, counter-based Monte Carlo chains (single flip
and exchange moves), Monte Carlo TDVP rows and an SR step."""

import os

import numpy as np
import pytest

from pyoracle import DeepDesc

pytestmark = pytest.mark.gpu

ann = pytest.importorskip("annongpu_gb300")
from annongpu_gb300.builders import _layer_connections  # noqa: E402

GOLD = os.path.join(os.path.dirname(__file__), "golden")
DEEP_ML = ["deep3_n3_18_9_3.npz", "deep3_n8_16_8_4.npz", "deep2_n6_12_6.npz"]


def cplx(rng, shape, scale):
    return scale * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))


def split_params(N, sizes, C, params):
    a = params[:N]
    b, W, off = [], [], N
    for m, c in zip(sizes, C):
        b.append(params[off:off + m])
        W.append(params[off + m:off + m + c * m].reshape(c, m))
        off += m * (1 + c)
    return a, b, W


class Case:
    """A random multi-layer PsiDeep on the GPU and the same network for the oracle."""

    def __init__(self, N, sizes, C, seed, conns=None, a_in=True, activation="poly", precision="fp64",
                 scale=0.15, lp=0.05 - 0.1j):
        rng = np.random.default_rng(seed)
        if conns is None:
            conns = [_layer_connections([n], [m], [c]) for n, m, c in zip([N] + sizes[:-1], sizes, C)]
        np_ = N + sum(m * (1 + c) for m, c in zip(sizes, C))
        self.params = cplx(rng, np_, scale)
        self.fw = 1.0 + cplx(rng, sizes[-1], 0.1)
        a, b, W = split_params(N, sizes, C, self.params)
        self.gpu = ann.PsiDeep(N, a, b, conns, W, self.fw, lp, True, a_in_log_psi=a_in, activation=activation,
                               precision=precision)
        self.conns = conns
        self.a_in = a_in
        self.act = {"poly": 0, "logcosh": 1}[activation]
        self.N = N
        self.ref = self.ref_with(lp)

    def ref_with(self, lp):
        return DeepDesc(self.N, self.conns, self.params, self.fw, log_prefactor=lp, a_in_log_psi=self.a_in,
                        activation=self.act)


def mixed_h(N):
    H = ann.transverse_field_ising_1d(N, 0.8) + 0.3 * ann.sigma_y(1) * ann.sigma_y(2)
    return H + 0.2 * ann.sigma_x(0) * ann.sigma_z(N - 1) + 0.1 * ann.sigma_y(N - 2)


@pytest.mark.parametrize("name", DEEP_ML)
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 5e-5)])
def test_deep_matches_reference_fixture(name, precision, tol):
    g = dict(np.load(os.path.join(GOLD, name)))
    N = int(g["N"])
    sizes = [int(x) for x in g["sizes"]]
    C = [int(x) for x in g["connectivity"]]
    blocks, off = [], 0
    for m, c in zip(sizes, C):
        blocks.append(g["conn"][off:off + m * c].reshape(c, m))
        off += m * c
    a, b, W = split_params(N, sizes, C, g["params"])
    psi = ann.PsiDeep(N, a, b, blocks, W, g["fw"], g["lp"][0], True, a_in_log_psi=False, precision=precision)
    assert psi.num_params == g["params"].size
    for k, s in enumerate(g["confs"]):
        np.testing.assert_allclose(ann.log_psi_s(psi, ann.Spins(int(s), N)), g["log_psi"][k], rtol=tol, atol=tol)
        np.testing.assert_allclose(ann.psi_O_k(psi, ann.Spins(int(s), N)), g["O_k"][k], rtol=10 * tol,
                                   atol=10 * tol * np.abs(g["O_k"][k]).max())
    H = ann.PauliExpression({(int(x), int(y)): c for x, y, c in zip(g["op_a"], g["op_b"], g["op_c"])})
    es = ann.ExactSummationSpins(N)
    np.testing.assert_allclose(ann.ExpectationValue()(ann.Operator(H), psi, es), g["ex_E"][0], rtol=20 * tol)
    np.testing.assert_allclose(psi.norm(es), g["ex_norm"][0], rtol=20 * tol)
    np.testing.assert_allclose(ann.psi_vector(psi, es), g["ex_vec"], rtol=20 * tol, atol=20 * tol)


@pytest.mark.parametrize("sizes,C,a_in,activation", [
    ([20, 10], [3, 4], True, "poly"),
    ([24, 12, 6], [4, 4, 3], False, "poly"),
    ([10, 10, 5, 5], [5, 4, 2, 3], True, "logcosh"),
])
def test_deep_exact_tdvp_fp64(oracle, sizes, C, a_in, activation):
    N = 10
    c = Case(N, sizes, C, seed=len(sizes) * 11 + len(C), a_in=a_in, activation=activation)
    H = mixed_h(N)
    es = ann.ExactSummationSpins(N)
    c.gpu.normalize(es)
    ref = c.ref_with(c.gpu.log_prefactor)
    r = oracle.deep_exact(ref, H, want_S=True)
    td = ann.TDVP(c.gpu.num_params)
    td.eval(ann.Operator(H), c.gpu, es)
    np.testing.assert_allclose(td.E_local, r["tE"][0], rtol=1e-10)
    np.testing.assert_allclose(td.O_k_vector, r["tO"], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(td.F_vector, r["tF"], rtol=1e-9, atol=1e-11)
    np.testing.assert_allclose(td.S_matrix, r["tS"], rtol=1e-9, atol=1e-11)
    for s in [0, 5, 321, 1023]:
        np.testing.assert_allclose(ann.psi_O_k(c.gpu, ann.Spins(s, N)), oracle.deep_O_k(ref, s), rtol=1e-9,
                                   atol=1e-12)


def test_deep_repeated_window_sites_and_two_words(oracle):
    """Windows that read one site twice (first layer recomputed per move) on N = 70
    (two 64-bit words): log psi, O_k and local energies of explicit configurations."""
    N, sizes, C = 70, [35, 14], [4, 5]
    rng = np.random.default_rng(8)
    c0 = _layer_connections([N], [35], [4])
    c0[1, 3] = c0[0, 3]  # unit 3 reads one site twice
    conns = [c0, _layer_connections([35], [14], [5])]
    c = Case(N, sizes, C, seed=3, conns=conns, scale=0.1)
    H = mixed_h(N) + 0.2 * ann.sigma_x(65) * ann.sigma_x(66)
    confs = [int(rng.integers(0, 1 << 62)) | (int(rng.integers(0, 1 << 6)) << 64) for _ in range(6)]
    el = ann.local_energies(c.gpu, ann.Operator(H), confs)
    for k, s in enumerate(confs):
        np.testing.assert_allclose(ann.log_psi_s(c.gpu, ann.Spins(s, N)), oracle.deep_log_psi(c.ref, s),
                                   rtol=1e-11, atol=1e-11)
        np.testing.assert_allclose(ann.psi_O_k(c.gpu, ann.Spins(s, N)), oracle.deep_O_k(c.ref, s), rtol=1e-10,
                                   atol=1e-12)
        np.testing.assert_allclose(el[k], oracle.deep_local_energy(c.ref, H, s), rtol=1e-9, atol=1e-10)


@pytest.mark.parametrize("move", ["single_flip", "exchange", "exchange_pairs"])
def test_deep_mc_philox_stream_matches_oracle(oracle, move):
    N = 12
    c = Case(N, [24, 12, 6], [3, 4, 2], seed=21, a_in=True)
    H = mixed_h(N)
    bonds = np.array([(i, (i + 1) % N) for i in range(N)], np.uint32)
    n_chains, spc, sw, th, seed = 64, 4, 1, 3, 0xBEEF5678
    kind = {"single_flip": 0, "exchange": 1, "exchange_pairs": 2}[move]
    n_up = None if move == "single_flip" else N // 2
    mc = ann.MonteCarloSpins(spc * n_chains, sw, th, n_chains, True, move=move,
                             bonds=bonds if move == "exchange" else None, n_up=n_up, seed=seed, persistent=True)
    ann.ExpectationValue()(ann.Operator(H), c.gpu, mc)
    conf, lp, el = mc.samples()
    ref = oracle.deep_mc_philox(c.ref, H, n_chains, seed, spc, sw, th, move_kind=kind, bonds=bonds,
                                n_up=-1 if n_up is None else n_up)
    assert ref["tie"][0] > 1e-11
    np.testing.assert_array_equal(conf[:, 0], ref["sconf"])
    np.testing.assert_allclose(lp, ref["slp"], rtol=1e-10)
    np.testing.assert_allclose(el, ref["seloc"], rtol=1e-9, atol=1e-11)
    if move != "single_flip":
        pop = np.array([bin(int(x)).count("1") for x in conf[:, 0]])
        assert (pop == N // 2).all()
    ch_conf, ch_ctr = mc.get_chains()
    np.testing.assert_array_equal(ch_conf[:, 0], ref["conf"])
    np.testing.assert_array_equal(ch_ctr, ref["counter"])
    ann.ExpectationValue()(ann.Operator(H), c.gpu, mc)
    conf2, _, _ = mc.samples()
    ref2 = oracle.deep_mc_philox(c.ref, H, n_chains, seed, spc, sw, th, move_kind=kind, bonds=bonds, init=False,
                                 conf=ref["conf"], counter=ref["counter"])
    np.testing.assert_array_equal(conf2[:, 0], ref2["sconf"])


def test_deep_fp32_monte_carlo_energy_sz_sector(oracle):
    """FP32 chains with exchange moves keep Sz = 0; the energy agrees with exact
    summation restricted to the sector within 3 standard errors."""
    N = 12
    c = Case(N, [24, 12], [3, 4], seed=5, precision="fp32", scale=0.2)
    H = ann.PauliExpression()
    for i in range(N):
        j = (i + 1) % N
        H = H + ann.sigma_x(i) * ann.sigma_x(j) + ann.sigma_y(i) * ann.sigma_y(j) + ann.sigma_z(i) * ann.sigma_z(j)
    op = ann.Operator(H)
    bonds = np.array([(i, (i + 1) % N) for i in range(N)], np.uint32)
    mc = ann.MonteCarloSpins(512 * 40, 2, 20, 512, True, move="exchange", bonds=bonds, n_up=N // 2, seed=13)
    e = ann.ExpectationValue()(op, c.gpu, mc)
    conf, lp, el = mc.samples()
    assert (np.array([bin(int(x)).count("1") for x in conf[:, 0]]) == N // 2).all()
    vec = ann.psi_vector(c.gpu, ann.ExactSummationSpins(N))
    mask = np.array([bin(k).count("1") == N // 2 for k in range(1 << N)])
    v = np.where(mask, vec, 0)
    e_exact = np.vdot(v, H.matrix(N) @ v) / np.vdot(v, v)
    se = el.real.reshape(40, 512).mean(axis=0).std(ddof=1) / np.sqrt(512)
    assert abs(e.real - e_exact.real) < 3 * se + 1e-6, (e, e_exact, se)


@pytest.mark.parametrize("s_mode", ["fp32", "bf16"])
def test_deep_monte_carlo_tdvp_rows_and_sr_step(oracle, s_mode):
    """Monte Carlo TDVP of a three-layer network: S and F equal the oracle's sums over the
    same samples (FP32 rows; BF16 tensor-core S within BF16 accuracy), and one SR step
    moves the parameters by -lr (S + shift)^-1 F."""
    N = 16
    c = Case(N, [32, 16, 8], [4, 4, 4], seed=9, precision="fp32", scale=0.1)
    H = ann.transverse_field_ising_1d(N, 1.0) + 0.2 * ann.sigma_y(2) * ann.sigma_y(9)
    op = ann.Operator(H)
    ns = 2000
    mc = ann.MonteCarloSpins(ns, 1, 5, 200, True, seed=4)
    td = ann.TDVP(c.gpu.num_params, s_mode=s_mode)
    td.eval(op, c.gpu, mc)
    conf, _, el = mc.samples()
    ref_el = np.array([oracle.deep_local_energy(c.ref, H, int(s)) for s in conf[:, 0]])
    np.testing.assert_allclose(el, ref_el, rtol=2e-4, atol=2e-4 * np.abs(ref_el).max())
    O = np.array([oracle.deep_O_k(c.ref, int(s)) for s in conf[:, 0]])
    w = 1.0 / ns
    Obar = w * O.sum(axis=0)
    E = w * ref_el.sum()
    S = w * np.conj(O).T @ O - np.outer(np.conj(Obar), Obar)
    F = w * np.conj(O).T @ ref_el - E * np.conj(Obar)
    scale = np.abs(S).max()
    tol = 2e-4 if s_mode == "fp32" else 1e-2
    assert np.abs(td.S_matrix - S).max() / scale < tol
    np.testing.assert_allclose(td.F_vector, F, rtol=1e-3, atol=2e-4 * np.abs(F).max())
    p0 = c.gpu.params
    delta = td.solve(1e-2)
    want = np.linalg.solve(td.S_matrix + 1e-2 * np.eye(c.gpu.num_params), td.F_vector)
    np.testing.assert_allclose(delta, want, rtol=1e-6, atol=1e-8 * np.abs(want).max())
    td.update(c.gpu, 0.05)
    np.testing.assert_allclose(c.gpu.params, p0 - 0.05 * delta, rtol=1e-12, atol=1e-14)


def test_deep_builder_and_json_roundtrip():
    """The reference test suite's deep-network shape (three hidden layers over three
    sites) through the constructor, and a JSON round trip."""
    rng = np.random.default_rng(2)
    psi = ann.new_deep_neural_network(3, 3, [18, 9, 3], [3, 2, 3], a=0, noise=1e-3, rng=rng, precision="fp64")
    assert psi.num_layers == 3
    assert psi.num_params == 3 + 18 * 4 + 9 * 3 + 3 * 4
    assert [w.shape for w in psi.W] == [(3, 18), (2, 9), (3, 3)]
    back = ann.PsiDeep.from_json(psi.to_json(), True, precision="fp64")
    for s in range(8):
        np.testing.assert_allclose(ann.log_psi_s(back, ann.Spins(s, 3)), ann.log_psi_s(psi, ann.Spins(s, 3)),
                                   rtol=1e-14)
    psi2 = ann.new_deep_neural_network(16, (4, 4), [(4, 4), (2, 2)], [(3, 3), (2, 2)], rng=rng)
    assert psi2.num_params == 16 + 16 * 10 + 4 * 5
    cp = +psi2
    np.testing.assert_array_equal(cp.params, psi2.params)
    assert abs(ann.log_psi_s(cp, ann.Spins(77, 16)) - ann.log_psi_s(psi2, ann.Spins(77, 16))) < 1e-6


# ---- the Pauli-string basis (ExactSummationPaulis / MonteCarloPaulis) ----
PAULI_FIX = ["deep_pauli_s3_9_6.npz", "deep_pauli_s4_12_6_3.npz"]


def pauli_h(S):
    H = ann.transverse_field_ising_1d(S, 0.7) + 0.3 * ann.sigma_y(0) * ann.sigma_x(1)
    return H + 0.2 * ann.sigma_z(S - 1) * ann.sigma_y(1) + 0.15 * ann.sigma_y(2) + 0.1


@pytest.mark.parametrize("name", PAULI_FIX)
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 5e-5)])
def test_deep_pauli_matches_reference_fixture(name, precision, tol):
    g = dict(np.load(os.path.join(GOLD, name)))
    S, N = int(g["num_sites"]), int(g["N"])
    sizes = [int(x) for x in g["sizes"]]
    C = [int(x) for x in g["connectivity"]]
    blocks, off = [], 0
    for m, c in zip(sizes, C):
        blocks.append(g["conn"][off:off + m * c].reshape(c, m))
        off += m * c
    a, b, W = split_params(N, sizes, C, g["params"])
    psi = ann.PsiDeep(S, a, b, blocks, W, g["fw"], g["lp"][0], True, a_in_log_psi=False, precision=precision)
    strings = [ann.PauliString(int(x), int(y)) for x, y in zip(g["conf_a"], g["conf_b"])]
    np.testing.assert_allclose(ann.log_psi_batch(psi, strings), g["log_psi"], rtol=tol, atol=tol)
    for k, p in enumerate(strings):
        np.testing.assert_allclose(ann.log_psi_s(psi, p), g["log_psi"][k], rtol=tol, atol=tol)
        np.testing.assert_allclose(ann.psi_O_k(psi, p), g["O_k"][k], rtol=10 * tol,
                                   atol=10 * tol * np.abs(g["O_k"][k]).max())
    H = ann.PauliExpression({(int(x), int(y)): c for x, y, c in zip(g["op_a"], g["op_b"], g["op_c"])})
    op = ann.Operator(H)
    es = ann.ExactSummationPaulis(S)
    assert es.num_steps == 4 ** S
    np.testing.assert_allclose(ann.ExpectationValue()(op, psi, es), g["ex_E"][0], rtol=20 * tol)
    np.testing.assert_allclose(psi.norm(es), g["ex_norm"][0], rtol=20 * tol)
    np.testing.assert_allclose(ann.psi_vector(psi, es), g["ex_vec"], rtol=20 * tol, atol=20 * tol)
    if precision == "fp64":
        td = ann.TDVP(psi.num_params)
        td.eval(op, psi, es)
        np.testing.assert_allclose(td.E_local, g["ex_tE"][0], rtol=1e-10)
        np.testing.assert_allclose(td.O_k_vector, g["ex_tO"], rtol=1e-9, atol=1e-12)
        np.testing.assert_allclose(td.F_vector, g["ex_tF"], rtol=1e-9, atol=1e-10 * np.abs(g["ex_tF"]).max())
        np.testing.assert_allclose(td.S_matrix, g["ex_tS"], rtol=1e-9, atol=1e-10 * np.abs(g["ex_tS"]).max())


def test_deep_pauli_one_layer_and_parameter_updates(oracle):
    """A one-layer PsiDeep (RBM-family kernels over spins) meets Pauli strings: the
    any-depth kernels take it over, with a.s in log psi, and follow parameter updates."""
    S = 4
    N = 3 * S
    c = Case(N, [24], [6], seed=31, a_in=True, scale=0.12)
    H = pauli_h(S)
    op = ann.Operator(H)
    ref = DeepDesc(N, c.conns, c.params, c.fw, log_prefactor=0.05 - 0.1j, a_in_log_psi=True, paulis=True)
    r = oracle.deep_exact(ref, H, want_S=True)
    es = ann.ExactSummationPaulis(S)
    np.testing.assert_allclose(ann.ExpectationValue()(op, c.gpu, es), r["E"][0], rtol=1e-10)
    td = ann.TDVP(c.gpu.num_params)
    td.eval(op, c.gpu, es)
    np.testing.assert_allclose(td.S_matrix, r["tS"], rtol=1e-9, atol=1e-11 * np.abs(r["tS"]).max())
    p2 = c.params * (1 + 0.1j)
    c.gpu.params = p2
    ref2 = DeepDesc(N, c.conns, p2, c.fw, log_prefactor=0.05 - 0.1j, a_in_log_psi=True, paulis=True)
    for x, y in [(0, 0), (5, 3), (15, 9)]:
        np.testing.assert_allclose(ann.log_psi_s(c.gpu, ann.PauliString(x, y)), oracle.deep_log_psi(ref2, (x, y)),
                                   rtol=1e-11, atol=1e-11)
    el = ann.local_energies(c.gpu, op, [ann.PauliString(5, 3), ann.PauliString(1, 14)])
    np.testing.assert_allclose(el, [oracle.deep_local_energy(ref2, H, (5, 3)), oracle.deep_local_energy(ref2, H, (1, 14))],
                               rtol=1e-9, atol=1e-11)


def test_deep_pauli_mc_philox_stream_matches_oracle(oracle):
    S = 5
    N = 3 * S
    c = Case(N, [15, 10], [3, 3], seed=17, a_in=True, scale=0.2)
    H = pauli_h(S)
    ref = DeepDesc(N, c.conns, c.params, c.fw, log_prefactor=0.05 - 0.1j, a_in_log_psi=True, paulis=True)
    n_chains, spc, sw, th, seed = 64, 4, 1, 2, 0x5EED0123
    mc = ann.MonteCarloPaulis(spc * n_chains, sw, th, n_chains, True, seed=seed, persistent=True)
    ann.ExpectationValue()(ann.Operator(H), c.gpu, mc)
    conf, lp, el = mc.samples()
    r = oracle.deep_mc_philox(ref, H, n_chains, seed, spc, sw, th)
    assert r["tie"][0] > 1e-11
    np.testing.assert_array_equal(conf.reshape(-1), r["sconf"])
    np.testing.assert_allclose(lp, r["slp"], rtol=1e-10)
    np.testing.assert_allclose(el, r["seloc"], rtol=1e-9, atol=1e-11)
    ch_conf, ch_ctr = mc.get_chains()
    np.testing.assert_array_equal(ch_conf.reshape(-1), r["conf"])
    np.testing.assert_array_equal(ch_ctr, r["counter"])
    ann.ExpectationValue()(ann.Operator(H), c.gpu, mc)
    conf2, _, _ = mc.samples()
    r2 = oracle.deep_mc_philox(ref, H, n_chains, seed, spc, sw, th, init=False, conf=r["conf"], counter=r["counter"])
    np.testing.assert_array_equal(conf2.reshape(-1), r2["sconf"])


def test_deep_pauli_fp32_monte_carlo_energy(oracle):
    """FP32 chains over Pauli strings: the energy agrees with exact summation within
    3 standard errors."""
    S = 5
    N = 3 * S
    c = Case(N, [15, 10], [3, 3], seed=2, precision="fp32", scale=0.25)
    H = pauli_h(S)
    op = ann.Operator(H)
    es = ann.ExactSummationPaulis(S)
    e_exact = ann.ExpectationValue()(op, c.gpu, es) / c.gpu.norm(es) ** 2
    mc = ann.MonteCarloPaulis(256 * 40, 2, 10, 256, True, seed=3)
    e = ann.ExpectationValue()(op, c.gpu, mc)
    _, _, el = mc.samples()
    se = el.real.reshape(40, 256).mean(axis=0).std(ddof=1) / np.sqrt(256)
    assert abs(e.real - e_exact.real) < 3 * se + 1e-6, (e, e_exact, se)
    assert 0.0 < mc.acceptance_rate <= 1.0
