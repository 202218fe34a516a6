"""Pins the FP64 oracle (oracle/oracle.cpp) against fixtures produced by the
reference's own host code path (tests/golden/gen_golden.py)."""

import os

import numpy as np
import pytest

from pyoracle import ClassicalDesc, CnnDesc, DeepDesc, RbmDesc

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    return dict(np.load(os.path.join(GOLD, name)))


class _Expr:
    """Operator arrays straight from a fixture."""

    def __init__(self, a, b, c):
        self.a, self.b, self.c = a, b, c

    def arrays(self, nw):
        return self.a.reshape(-1, 1), self.b.reshape(-1, 1), self.c


def rbm_from(g):
    return RbmDesc(int(g["N"]), int(g["M"]), g["W"], fw=np.full(int(g["M"]), g["fw"][0]),
                   log_prefactor=g["lp"][0], layout=0, a_in_log_psi=False)


def deep_from(g):
    N, M, C = int(g["N"]), int(g["M"]), int(g["C"])
    p = g["params"]
    return RbmDesc(N, M, p[N + M:], a=p[:N], b=p[N:N + M], fw=g["fw"], conn=g.get("conn"),
                   log_prefactor=g["lp"][0], layout=1, a_in_log_psi=False)


def deep_ml_from(g):
    """A multi-layer fixture as the oracle's DeepDesc (reference semantics: no a.s in log psi)."""
    N = int(g["N"])
    blocks, off = [], 0
    for m, c in zip(g["sizes"], g["connectivity"]):
        blocks.append(g["conn"][off:off + int(m) * int(c)].reshape(int(c), int(m)))
        off += int(m) * int(c)
    return DeepDesc(N, blocks, g["params"], g["fw"], log_prefactor=g["lp"][0], a_in_log_psi=False)


DEEP_ML = ["deep3_n3_18_9_3.npz", "deep3_n8_16_8_4.npz", "deep2_n6_12_6.npz"]


def close(x, y, rtol=1e-10, atol=1e-12):
    np.testing.assert_allclose(np.asarray(x), np.asarray(y), rtol=rtol, atol=atol)


def test_activation_kats(oracle):
    g = load("kats.npz")
    for layer in (0, 1):
        for k, z in enumerate(g["z"]):
            f, df = oracle.activation(z, layer)
            close(f, g["f"][layer, k], rtol=1e-14)
            close(df, g["df"][layer, k], rtol=1e-14)


def test_pauli_apply_kats(oracle):
    g = load("kats.npz")
    N = int(g["pauli_N"][0])
    for k in range(len(g["pauli_a"])):
        f, out = oracle.pauli_apply(int(g["pauli_a"][k]), int(g["pauli_b"][k]), int(g["pauli_conf"][k]), N)
        assert f == g["pauli_factor"][k]
        assert int(out[0]) == int(g["pauli_out"][k])


@pytest.mark.parametrize("name", ["rbm_n8_m8.npz", "deep_n8_m8.npz", "deep_n6_m12_c3.npz", "deep_n16_m16.npz"])
def test_log_psi_and_O_k(oracle, name):
    g = load(name)
    psi = rbm_from(g) if name.startswith("rbm") else deep_from(g)
    for k, s in enumerate(g["confs"]):
        close(oracle.log_psi(psi, int(s)), g["log_psi"][k])
        close(oracle.O_k(psi, int(s)), g["O_k"][k])


@pytest.mark.parametrize("name", ["rbm_n8_m8.npz", "deep_n8_m8.npz", "deep_n6_m12_c3.npz", "deep_n16_m16.npz"])
def test_exact_summation(oracle, name):
    g = load(name)
    psi = rbm_from(g) if name.startswith("rbm") else deep_from(g)
    expr = _Expr(g["op_a"], g["op_b"], g["op_c"])
    want_S = "ex_tS" in g
    r = oracle.exact(psi, expr, want_S=True)
    close(r["E"][0], g["ex_E"][0])
    close(r["fluct"], g["ex_fluct"], rtol=1e-9)
    close(r["grad"], g["ex_grad"], rtol=1e-9, atol=1e-10)
    close(r["tE"][0], g["ex_tE"][0])
    close(r["tE2"][0], g["ex_tE2"][0])
    close(r["tO"], g["ex_tO"])
    close(r["tF"], g["ex_tF"], rtol=1e-9, atol=1e-10)
    if want_S:
        close(r["tS"], g["ex_tS"], rtol=1e-9, atol=1e-10)
        close(r["vec"], g["ex_vec"])
    else:
        S = r["tS"]
        close(np.trace(S), g["ex_tS_trace"][0], rtol=1e-9)
        close(np.linalg.norm(S), g["ex_tS_fro"][0], rtol=1e-9)
        close(S.reshape(-1)[g["ex_tS_idx"]], g["ex_tS_sample"], rtol=1e-8, atol=1e-10)
    close(r["norm"][0], g["ex_norm"][0])
    close(r["mean_log_psi"][0], g["ex_mlp"][0])
    close(r["O_sum"], g["ex_O_sum"], rtol=1e-9, atol=1e-9)


@pytest.mark.parametrize("name", ["rbm_n8_m8.npz", "deep_n8_m8.npz", "deep_n6_m12_c3.npz"])
def test_mc_trace_bit_exact(oracle, name):
    """The oracle's restatement of the host Monte Carlo, fed the same mt19937 stream,
    visits exactly the reference's configurations, proposal by proposal."""
    g = load(name)
    psi = rbm_from(g) if name.startswith("rbm") else deep_from(g)
    expr = _Expr(g["op_a"], g["op_b"], g["op_c"])
    ns, sw, th = (int(x) for x in g["mc_params"])
    r = oracle.mc_reference(psi, expr, ns, sw, th, seed=0)
    assert r["num_props"] == len(g["mc_psite"])
    np.testing.assert_array_equal(r["psite"], g["mc_psite"])
    np.testing.assert_array_equal(r["pconf"], g["mc_pconf"])
    np.testing.assert_array_equal(r["sconf"], g["mc_sconf"])
    close(r["slp"], g["mc_slp"])
    close(r["seloc"], g["mc_seloc"], rtol=1e-9, atol=1e-11)
    close(r["energy"][0], g["mc_mc_energy"][0], rtol=1e-9)


@pytest.mark.parametrize("name", DEEP_ML)
def test_deep_multilayer(oracle, name):
    """PsiDeep with two and three hidden layers: log psi, O_k (back-propagation) and the
    exact-summation TDVP quantities of the reference's own kernel."""
    g = load(name)
    psi = deep_ml_from(g)
    for k, s in enumerate(g["confs"]):
        close(oracle.deep_log_psi(psi, int(s)), g["log_psi"][k])
        close(oracle.deep_O_k(psi, int(s)), g["O_k"][k], rtol=1e-10, atol=1e-12)
    r = oracle.deep_exact(psi, _Expr(g["op_a"], g["op_b"], g["op_c"]), want_S=True)
    close(r["E"][0], g["ex_E"][0])
    close(r["norm"][0], g["ex_norm"][0])
    close(r["tE"][0], g["ex_tE"][0])
    close(r["tE2"][0], g["ex_tE2"][0])
    close(r["tO"], g["ex_tO"])
    close(r["tF"], g["ex_tF"], rtol=1e-9, atol=1e-10)
    close(r["tS"], g["ex_tS"], rtol=1e-9, atol=1e-10)


@pytest.mark.parametrize("name", ["deep_pauli_s3_9_6.npz", "deep_pauli_s4_12_6_3.npz"])
def test_deep_pauli_string_basis(oracle, name):
    """PsiDeep over Pauli strings (three input units per site), Pauli-string operator
    products and ExactSummationPaulis, against the reference's own kernel."""
    g = load(name)
    N = int(g["N"])
    blocks, off = [], 0
    for m, c in zip(g["sizes"], g["connectivity"]):
        blocks.append(g["conn"][off:off + int(m) * int(c)].reshape(int(c), int(m)))
        off += int(m) * int(c)
    psi = DeepDesc(N, blocks, g["params"], g["fw"], log_prefactor=g["lp"][0], a_in_log_psi=False, paulis=True)
    for k, (a, b) in enumerate(zip(g["conf_a"], g["conf_b"])):
        close(oracle.deep_log_psi(psi, (int(a), int(b))), g["log_psi"][k])
        close(oracle.deep_O_k(psi, (int(a), int(b))), g["O_k"][k])
    r = oracle.deep_exact(psi, _Expr(g["op_a"], g["op_b"], g["op_c"]), want_S=True)
    close(r["E"][0], g["ex_E"][0])
    close(r["norm"][0], g["ex_norm"][0])
    close(r["tE2"][0], g["ex_tE2"][0])
    close(r["tO"], g["ex_tO"])
    close(r["tF"], g["ex_tF"], rtol=1e-9, atol=1e-10)
    close(r["tS"], g["ex_tS"], rtol=1e-9, atol=1e-10)


def classical_from(g):
    """(classical psi, psi_prime) of a classical-network fixture for the oracle."""
    S = int(g["num_sites"])
    beg = g["feat_begin"]
    feats = [_Expr(g["feat_a"][beg[k]:beg[k + 1]], g["feat_b"][beg[k]:beg[k + 1]], g["feat_c"][beg[k]:beg[k + 1]])
             for k in range(len(beg) - 1)]

    def deep(prefix):
        blocks, off = [], 0
        for m, c in zip(g[prefix + "sizes"], g[prefix + "connectivity"]):
            blocks.append(g[prefix + "conn"][off:off + int(m) * int(c)].reshape(int(c), int(m)))
            off += int(m) * int(c)
        return DeepDesc(S, blocks, g[prefix + "params"], g[prefix + "fw"], log_prefactor=g[prefix + "lp"][0],
                        a_in_log_psi=False)
    ref = deep("ref_") if "ref_params" in g else None
    psi = ClassicalDesc(S, feats, g["theta"], log_prefactor=g["lp"][0], order=int(g["order"]), ref=ref)
    return psi, deep("prime_"), ref


@pytest.mark.parametrize("name", ["classical_s4_order2_deep.npz", "classical_s6_order1.npz"])
def test_classical_network_and_kullback_leibler(oracle, name):
    """PsiClassical (order 1, and order 2 over a PsiDeep reference) and KullbackLeibler value,
    gradient and gradient_with_noise (with the carried mean deviation) against the reference."""
    g = load(name)
    psi, prime, ref = classical_from(g)
    S = int(g["num_sites"])
    for s in range(1 << S):
        close(oracle.classical_log_psi(psi, s), g["log_psi"][s])
        close(oracle.classical_O_k(psi, s), g["O_k"][s])
    r = oracle.classical_exact(psi, _Expr(g["op_a"], g["op_b"], g["op_c"]), want_S=True)
    for k in ("E", "norm", "tE", "tO"):
        close(r[k], g["ex_" + k])
    close(r["tF"], g["ex_tF"], rtol=1e-9, atol=1e-11)
    close(r["tS"], g["ex_tS"], rtol=1e-9, atol=1e-11)
    th = float(g["threshold"][0])
    r1 = oracle.kl(psi, prime, threshold=th, gradient=False)
    close(r1["value"][0], g["kl_value"][0])
    close(r1["total_weight"][0], g["kl_out4"][0])
    close(r1["mean_deviation"][0], g["kl_out4"][1] + 1j * g["kl_out4"][2])
    r2 = oracle.kl(psi, prime, threshold=th, last_mean=r1["mean_deviation"][0], gradient=False)
    close(r2["value"][0], g["kl_out4"][3])
    r3 = oracle.kl(psi, prime, threshold=th, last_mean=r2["mean_deviation"][0], nu=1.0)
    close(r3["value"][0], g["kl_value"][1])
    close(r3["grad"], g["kl_grad"], rtol=1e-9, atol=1e-12)
    r4 = oracle.kl(psi, prime, threshold=th, last_mean=r3["mean_deviation"][0], nu=1.0, noise=True)
    close(r4["value"][0], g["kl_value"][2])
    close(r4["grad"], g["kl_grad_noise_call"], rtol=1e-9, atol=1e-12)
    close(r4["noise"], g["kl_noise"], rtol=1e-8, atol=1e-12)


def test_deep_one_layer_equals_rbm_family(oracle):
    """The any-depth restatement with one hidden layer is the RBM-family PsiDeep."""
    g = load("deep_n6_m12_c3.npz")
    N, M, C = int(g["N"]), int(g["M"]), int(g["C"])
    rb = deep_from(g)
    dp = DeepDesc(N, [g["conn"].reshape(C, M)], g["params"], g["fw"], log_prefactor=g["lp"][0],
                  a_in_log_psi=False)
    expr = _Expr(g["op_a"], g["op_b"], g["op_c"])
    for s in range(0, 1 << N, 7):
        close(oracle.deep_log_psi(dp, s), oracle.log_psi(rb, s), rtol=1e-13)
        close(oracle.deep_O_k(dp, s), oracle.O_k(rb, s), rtol=1e-13, atol=1e-14)
        close(oracle.deep_local_energy(dp, expr, s), oracle.local_energy(rb, expr, s), rtol=1e-11, atol=1e-12)


def test_cnn(oracle):
    g = load("cnn_4x4.npz")
    psi = CnnDesc(g["extent"], g["channels"], g["connectivity"], g["classes"], g["params"], g["ff"][0],
                  log_prefactor=g["lp"][0])
    for k, s in enumerate(g["confs"]):
        close(oracle.cnn_log_psi(psi, int(s)), g["log_psi"][k])
        close(oracle.cnn_O_k(psi, int(s)), g["O_k"][k], rtol=1e-9, atol=1e-12)
    r = oracle.cnn_exact(psi, _Expr(g["op_a"], g["op_b"], g["op_c"]))
    close(r["E"][0], g["ex_E"][0], rtol=1e-9)
    close(r["norm"][0], g["ex_norm"][0])


def test_expression_matrix_matches_exact_energy(oracle):
    """The dense builder of annongpu_gb300.expression reproduces the exact-summation
    energy: sum_s |psi(s)|^2 E_loc(s) == psi^H H psi."""
    from annongpu_gb300.expression import sigma_x, sigma_y, sigma_z, transverse_field_ising_1d
    g = load("deep_n8_m8.npz")
    psi = deep_from(g)
    N = psi.N
    H = transverse_field_ising_1d(N, 0.9, 1.1) + 0.3 * sigma_y(1) * sigma_y(2) + 0.2 * sigma_x(0) * sigma_z(3)
    H = H + 0.15 * sigma_y(4) + 0.05 * sigma_y(0) * sigma_y(2) * sigma_y(5) + 0.1 * sigma_z(2)
    r = oracle.exact(psi, H, want_S=False)
    v = r["vec"]
    close(np.vdot(v, H.matrix(N) @ v), r["E"][0], rtol=1e-10)


def test_hsd_restatement_distance_and_gradient():
    """The oracle's HilbertSpaceDistance restatement against the reference's own checks
    (test/test_HilbertSpaceDistance.py): the distance of psi' = psi to U psi with
    U = 1 + i H t against dense matrices, and the gradient against central finite
    differences (d/dRe + i d/dIm, eps 1e-6) of the distance."""
    import annongpu_gb300.expression as ex
    from pyoracle import Oracle
    o = Oracle()
    N, M = 4, 4
    rng = np.random.default_rng(5)
    c = lambda *s: 0.1 * (rng.standard_normal(s) + 1j * rng.standard_normal(s))  # noqa: E731
    a, b, W = c(N), c(M), c(N, M)
    make = lambda p: RbmDesc(N, M, p[N + M:].reshape(N, M), a=p[:N], b=p[N:N + M], layout=1)  # noqa: E731
    p0 = np.concatenate([a, b, W.reshape(-1)])
    H = ex.transverse_field_ising_1d(N, 0.9)
    U = ex.identity() + 0.01j * H
    d, _ = o.hsd_exact(make(p0), make(p0), U, True)
    v = o.exact(make(p0), None, want_S=False)["vec"]
    vp = U.matrix(N) @ v
    d_ref = np.sqrt(1.0 - abs(np.vdot(v / np.linalg.norm(v), vp / np.linalg.norm(vp))) ** 2)
    assert d == pytest.approx(d_ref, rel=1e-9)
    # gradient in psi' for psi' != psi (exponential form), against finite differences
    p1 = p0 + c(p0.size) * 0.3
    op = 0.2j * H
    _, g = o.hsd_exact(make(p0), make(p1), op, False)
    eps = 1e-6
    g_ref = np.zeros(p1.size, complex)
    for k in range(p1.size):
        for unit in (1.0, 1j):
            dp = np.zeros(p1.size, complex)
            dp[k] = eps * unit
            fd = (o.hsd_exact(make(p0), make(p1 + dp), op, False)[0] -
                  o.hsd_exact(make(p0), make(p1 - dp), op, False)[0]) / (2 * eps)
            g_ref[k] += unit * fd
    np.testing.assert_allclose(g, g_ref, rtol=1e-4, atol=1e-7)


def hsd_pair_from(g):
    """psi and psi' of an HSD fixture as oracle descriptors (reference semantics: no a.s)."""
    N, M = int(g["N"]), int(g["M"])

    def one(p, fw, lp):
        return RbmDesc(N, M, p[N + M:], a=p[:N], b=p[N:N + M], fw=fw, log_prefactor=lp[0], layout=1,
                       a_in_log_psi=False)
    return one(g["params"], g["fw"], g["lp"]), one(g["params_p"], g["fw_p"], g["lp_p"])


@pytest.mark.parametrize("form", ["unitary", "exponential"])
@pytest.mark.parametrize("nu", [1.0, 0.5])
def test_hsd_exact_matches_reference(oracle, form, nu):
    """The oracle's HilbertSpaceDistance (distance and gradient in psi', exact summation)
    against the reference's own HilbertSpaceDistance::distance / gradient run on the same
    PsiDeep pair (source/network_functions/HilbertSpaceDistance.cu.template:16-168)."""
    g = load("hsd_n8_m8.npz")
    psi, psi_p = hsd_pair_from(g)
    expr = _Expr(g[f"{form}_op_a"], g[f"{form}_op_b"], g[f"{form}_op_c"])
    d, grad = oracle.hsd_exact(psi, psi_p, expr, form == "unitary", nu=nu)
    tag = f"{form}_nu{nu:g}"
    close(d, g[f"{tag}_dist"][0])
    close(d, g[f"{tag}_dist"][1])
    close(grad, g[f"{tag}_grad"], rtol=1e-9, atol=1e-12)


def test_polynomial_real_part_rearrangement(oracle):
    """The complex64 sampler evaluates the real part of the reference's polynomial activation
    (first layer) as Re f = P/2 - P^2/12 + q^2/3 + (P/45)(P^2 - 12 q^2) with P = x^2 - y^2,
    q = x y (two units per two-wide FP32 instruction). In FP64 the rearrangement equals Re of
    the oracle's activation, which the reference's known-answer values pin."""
    rng = np.random.default_rng(5)
    zs = list(load("kats.npz")["z"]) + list(0.8 * (rng.standard_normal(64) + 1j * rng.standard_normal(64)))
    for z in zs:
        f, _ = oracle.activation(complex(z), 0)
        x, y = z.real, z.imag
        P, q = x * x - y * y, x * y
        re = P / 2 - P * P / 12 + q * q / 3 + (P / 45) * (P * P - 12 * q * q)
        close(re, np.real(f), rtol=1e-13, atol=1e-15)
