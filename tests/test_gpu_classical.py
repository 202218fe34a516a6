"""PsiClassical (variational classical network) and KullbackLeibler on the GPU, against the
reference's own kernels (tests/golden/classical_*.npz) and the FP64 oracle: log psi, O_k,
exact-summation energy and TDVP quantities, the divergence with its carried mean deviation,
its gradient (also by finite differences, as the reference's test does) and noise, over exact
summation and Monte Carlo."""

import os

import numpy as np
import pytest

from pyoracle import ClassicalDesc, DeepDesc

pytestmark = pytest.mark.gpu

ann = pytest.importorskip("annongpu_gb300")

GOLD = os.path.join(os.path.dirname(__file__), "golden")
FIX = ["classical_s4_order2_deep.npz", "classical_s6_order1.npz"]


def deep_from(g, prefix, S, precision="fp64", a_in=False):
    blocks, off = [], 0
    sizes = [int(m) for m in g[prefix + "sizes"]]
    C = [int(c) for c in g[prefix + "connectivity"]]
    for m, c in zip(sizes, C):
        blocks.append(g[prefix + "conn"][off:off + m * c].reshape(c, m))
        off += m * c
    p = g[prefix + "params"]
    a, b, W, off = p[:S], [], [], S
    for m, c in zip(sizes, C):
        b.append(p[off:off + m])
        W.append(p[off + m:off + m + c * m].reshape(c, m))
        off += m * (1 + c)
    gpu = ann.PsiDeep(S, a, b, blocks, W, g[prefix + "fw"], g[prefix + "lp"][0], True, a_in_log_psi=a_in,
                      precision=precision)
    ref = DeepDesc(S, blocks, p, g[prefix + "fw"], log_prefactor=g[prefix + "lp"][0], a_in_log_psi=a_in)
    return gpu, ref


def features(g):
    beg = g["feat_begin"]
    return [ann.PauliExpression({(int(g["feat_a"][q]), int(g["feat_b"][q])): g["feat_c"][q]
                                 for q in range(beg[k], beg[k + 1])}) for k in range(len(beg) - 1)]


def classical_from(g, precision="fp64"):
    S = int(g["num_sites"])
    order = int(g["order"])
    ref_gpu = ref_or = None
    if "ref_params" in g:
        ref_gpu, ref_or = deep_from(g, "ref_", S, precision)
    feats = features(g)
    if ref_gpu is not None:
        psi = ann.PsiClassicalANN_2(S, feats, g["theta"], ref_gpu, g["lp"][0], True)
    else:
        psi = ann.PsiClassicalFP_1(S, feats, g["theta"], ann.PsiFullyPolarized(S), g["lp"][0], True,
                                   precision=precision)
    orc = ClassicalDesc(S, feats, g["theta"], log_prefactor=g["lp"][0], order=order, ref=ref_or)
    return psi, orc


@pytest.mark.parametrize("name", FIX)
def test_classical_matches_reference_fixture(name):
    g = dict(np.load(os.path.join(GOLD, name)))
    S = int(g["num_sites"])
    psi, _ = classical_from(g)
    assert psi.num_params == g["O_k"].shape[1]
    lp = ann.log_psi_batch(psi, list(range(1 << S)))
    np.testing.assert_allclose(lp, g["log_psi"], rtol=1e-10, atol=1e-12)
    for s in range(0, 1 << S, 3):
        np.testing.assert_allclose(ann.psi_O_k(psi, ann.Spins(s, S)), g["O_k"][s], rtol=1e-10, atol=1e-12)
    H = ann.PauliExpression({(int(x), int(y)): c for x, y, c in zip(g["op_a"], g["op_b"], g["op_c"])})
    op = ann.Operator(H)
    es = ann.ExactSummationSpins(S)
    np.testing.assert_allclose(ann.ExpectationValue()(op, psi, es), g["ex_E"][0], rtol=1e-10)
    np.testing.assert_allclose(psi.norm(es), g["ex_norm"][0], rtol=1e-10)
    td = ann.TDVP(psi.num_params)
    td.eval(op, psi, es)
    np.testing.assert_allclose(td.O_k_vector, g["ex_tO"], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(td.F_vector, g["ex_tF"], rtol=1e-9, atol=1e-10 * np.abs(g["ex_tF"]).max())
    np.testing.assert_allclose(td.S_matrix, g["ex_tS"], rtol=1e-9, atol=1e-10 * np.abs(g["ex_tS"]).max())


@pytest.mark.parametrize("name", FIX)
def test_kullback_leibler_matches_reference_fixture(name):
    g = dict(np.load(os.path.join(GOLD, name)))
    S = int(g["num_sites"])
    psi, _ = classical_from(g)
    prime, _ = deep_from(g, "prime_", S)
    th = float(g["threshold"][0])
    es = ann.ExactSummationSpins(S)
    kl = ann.KullbackLeibler(prime.num_params)
    np.testing.assert_allclose(kl(psi, prime, es, th), g["kl_value"][0], rtol=1e-10)
    np.testing.assert_allclose(kl.total_weight, g["kl_out4"][0], rtol=1e-10)
    np.testing.assert_allclose(kl.mean_deviation, g["kl_out4"][1] + 1j * g["kl_out4"][2], rtol=1e-10)
    np.testing.assert_allclose(kl(psi, prime, es, th), g["kl_out4"][3], rtol=1e-10)
    grad, v = kl.gradient(psi, prime, es, 1.0, th)
    np.testing.assert_allclose(v, g["kl_value"][1], rtol=1e-10)
    np.testing.assert_allclose(grad, g["kl_grad"], rtol=1e-8, atol=1e-11 * np.abs(g["kl_grad"]).max())
    grad, noise, v = kl.gradient_with_noise(psi, prime, es, 1.0, th)
    np.testing.assert_allclose(v, g["kl_value"][2], rtol=1e-10)
    np.testing.assert_allclose(grad, g["kl_grad_noise_call"], rtol=1e-8,
                               atol=1e-11 * np.abs(g["kl_grad_noise_call"]).max())
    np.testing.assert_allclose(noise, g["kl_noise"], rtol=1e-7, atol=1e-11 * np.abs(g["kl_noise"]).max())


def test_kullback_leibler_gradient_finite_differences():
    """The reference's own check (test/test_KullbackLeibler.py): the gradient in psi_prime's
    parameters against central differences of the divergence (real and imaginary parts).
    psi_prime includes a.s in log psi here: with the reference's convention (a absent from
    log psi, O_a = s) the a entries of the gradient have no finite-difference counterpart."""
    g = dict(np.load(os.path.join(GOLD, FIX[0])))
    S = int(g["num_sites"])
    psi, _ = classical_from(g)
    prime, _ = deep_from(g, "prime_", S, a_in=True)
    es = ann.ExactSummationSpins(S)
    kl = ann.KullbackLeibler(prime.num_params)
    kl(psi, prime, es)
    grad, _ = kl.gradient(psi, prime, es, 1.0)
    p0 = prime.params
    eps = 1e-5
    fd = np.zeros(prime.num_params, complex)
    for k in range(prime.num_params):
        for unit in (1.0, 1j):
            d = np.zeros_like(p0)
            d[k] = unit * eps
            prime.params = p0 + d
            plus = kl(psi, prime, es)
            prime.params = p0 - d
            minus = kl(psi, prime, es)
            fd[k] += unit * (plus - minus) / (2 * eps)
    prime.params = p0
    np.testing.assert_allclose(grad, fd, rtol=1e-4, atol=1e-6)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("fp32", 2e-4)])
def test_kullback_leibler_monte_carlo_rows(oracle, precision, tol):
    """Over psi_prime's Monte Carlo samples: value and gradient equal the oracle's sums over
    the same rows (uniform weights)."""
    g = dict(np.load(os.path.join(GOLD, FIX[0])))
    S = int(g["num_sites"])
    psi, orc = classical_from(g)
    prime, prime_or = deep_from(g, "prime_", S, precision)
    ns = 4096
    mc = ann.MonteCarloSpins(ns, 2, 10, 256, True, seed=5, persistent=True)
    kl = ann.KullbackLeibler(prime.num_params)
    grad, v = kl.gradient(psi, prime, mc, 1.0, 0.0)
    conf, _, _ = mc.samples()
    r = oracle.kl(orc, prime_or, confs=conf, wprime=np.full(ns, 1.0 / ns), nu=1.0)
    np.testing.assert_allclose(v, r["value"][0], rtol=tol)
    np.testing.assert_allclose(kl.total_weight, r["total_weight"][0], rtol=tol)
    np.testing.assert_allclose(grad, r["grad"], rtol=10 * tol, atol=10 * tol * np.abs(r["grad"]).max())


def test_classical_monte_carlo_sr_step(oracle):
    """A classical network over a two-layer PsiDeep: Monte Carlo TDVP S and F equal the
    oracle's sums over the same samples, and one SR step moves all parameters."""
    rng = np.random.default_rng(4)
    S = 8
    blocks = [np.array([[(j + i) % S for j in range(16)] for i in range(3)], np.uint32),
              np.array([[(j * 2 + i) % 16 for j in range(8)] for i in range(4)], np.uint32)]
    np_ref = S + 16 * 4 + 8 * 5
    p = 0.1 * (rng.standard_normal(np_ref) + 1j * rng.standard_normal(np_ref))
    fw = np.ones(8, complex)
    b = [p[S:S + 16], p[S + 64:S + 72]]
    W = [p[S + 16:S + 64].reshape(3, 16), p[S + 72:].reshape(4, 8)]
    ref_gpu = ann.PsiDeep(S, p[:S], b, blocks, W, fw, 0.0, True, precision="fp64")
    feats = [ann.sigma_z(i) * ann.sigma_z((i + 1) % S) for i in range(S)] + [ann.sigma_x(i) for i in range(S)]
    theta = 0.1 * (rng.standard_normal(len(feats)) + 1j * rng.standard_normal(len(feats)))
    psi = ann.new_classical_network(S, 2, feats, psi_ref=ref_gpu)
    psi.params = np.concatenate([theta, p])
    orc = ClassicalDesc(S, feats, theta, order=2, ref=DeepDesc(S, blocks, p, fw))
    H = ann.transverse_field_ising_1d(S, 1.0)
    op = ann.Operator(H)
    mc = ann.MonteCarloSpins(2000, 1, 10, 200, True, seed=8)
    td = ann.TDVP(psi.num_params)
    td.eval(op, psi, mc)
    conf, _, el = mc.samples()
    ref_el = np.array([oracle.classical_local_energy(orc, H, int(s)) for s in conf[:, 0]])
    np.testing.assert_allclose(el, ref_el, rtol=1e-9, atol=1e-11)
    O = np.array([oracle.classical_O_k(orc, int(s)) for s in conf[:, 0]])
    w = 1.0 / len(conf)
    Ob = w * O.sum(axis=0)
    E = w * ref_el.sum()
    S_ = w * np.conj(O).T @ O - np.outer(np.conj(Ob), Ob)
    F = w * np.conj(O).T @ ref_el - E * np.conj(Ob)
    np.testing.assert_allclose(td.S_matrix, S_, rtol=1e-8, atol=1e-10 * np.abs(S_).max())
    np.testing.assert_allclose(td.F_vector, F, rtol=1e-8, atol=1e-10 * np.abs(F).max())
    p_before = psi.params
    delta = td.solve(1e-2)
    td.update(psi, 0.05)
    np.testing.assert_allclose(psi.params, p_before - 0.05 * delta, rtol=1e-12, atol=1e-14)
    assert psi.psi_ref.num_params == np_ref


def test_classical_builder_and_calibrate():
    """new_classical_network over the fully polarized reference: one parameter per term,
    log_prefactor log 2^(-N/2); normalize / calibrate over exact summation."""
    psi = ann.new_classical_network(4, 1, ann.sigma_z(0) * ann.sigma_z(1) + ann.sigma_x(0))
    assert psi.num_params == 2 and psi.order == 1
    np.testing.assert_allclose(psi.log_prefactor, np.log(1 / 2 ** 2))
    es = ann.ExactSummationSpins(4)
    # zero parameters: |psi(s)|^2 = 1/16 for every s, the state is normalised
    np.testing.assert_allclose(psi.norm(es), 1.0, rtol=1e-12)
    psi.params = np.array([0.3 + 0.1j, -0.2j])
    psi.normalize(es)
    np.testing.assert_allclose(psi.norm(es), 1.0, rtol=1e-12)
