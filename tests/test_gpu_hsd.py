"""HilbertSpaceDistance on the GPU (source/network_functions/HilbertSpaceDistance.cu.template):
against the FP64 oracle's restatement over all configurations (unitary and exponential
forms), the reference's own checks (test/test_HilbertSpaceDistance.py: distance against the
dense-matrix formula, gradient against central finite differences of the distance), and a
Monte Carlo estimate against the exact value.

Tolerances: FP64 kernels vs the oracle rtol 1e-10 (distance) and 1e-8 of the largest
gradient entry; finite differences as the reference: rtol 1e-3, atol 1e-4."""

import os

import numpy as np
import pytest

from pyoracle import RbmDesc

pytestmark = pytest.mark.gpu

ann = pytest.importorskip("annongpu_gb300")


def cplx(rng, shape, scale):
    return scale * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))


def deep(N, M, seed, precision="fp64", scale=0.1):
    rng = np.random.default_rng(seed)
    a, b, W = cplx(rng, N, 0.05), cplx(rng, M, 0.05), cplx(rng, (N, M), scale)
    fw = np.ones(M, complex)
    conn = np.array([[(j + i) % N for j in range(M)] for i in range(N)], np.uint32)
    psi = ann.PsiDeep(N, a, [b], [conn], [W], fw, 0.0, True, precision=precision)
    return psi


def desc(psi):
    return RbmDesc(psi.N, psi.b[0].size, psi.W[0], a=psi.a, b=psi.b[0], fw=psi.final_weights,
                   conn=psi.connections[0], log_prefactor=psi.log_prefactor, layout=1)


@pytest.mark.parametrize("unitary", [True, False])
def test_hsd_matches_oracle(oracle, unitary):
    N, M = 8, 8
    psi = deep(N, M, 1)
    psi_p = deep(N, M, 2, scale=0.12)
    es = ann.ExactSummationSpins(N)
    psi.normalize(es)
    psi_p.normalize(es)
    H = ann.transverse_field_ising_1d(N, 0.9)
    t = 1e-2
    expr = (ann.identity() + 1j * t * H) if unitary else (1j * t * H)
    op = ann.Operator(expr)
    hsd = ann.HilbertSpaceDistance(psi_p.num_params)
    d = hsd(psi, psi_p, op, unitary, es)
    g, d2 = hsd.gradient(psi, psi_p, op, unitary, es, 1.0)
    d_ref, g_ref = oracle.hsd_exact(desc(psi), desc(psi_p), expr, unitary)
    np.testing.assert_allclose(d, d_ref, rtol=1e-10)
    np.testing.assert_allclose(d2, d_ref, rtol=1e-10)
    assert np.abs(g - g_ref).max() <= 1e-8 * np.abs(g_ref).max()


def test_hsd_distance_against_dense_matrices():
    """test/test_HilbertSpaceDistance.py:10-41: psi' = psi, U = 1 + i H t."""
    N, M = 8, 8
    psi = deep(N, M, 3)
    es = ann.ExactSummationSpins(N)
    psi.calibrate(es)
    H = ann.transverse_field_ising_1d(N, 1.1)
    t = 1e-2
    U = ann.identity() + 1j * t * H
    d = ann.HilbertSpaceDistance(psi.num_params)(psi, psi, ann.Operator(U), True, es)
    v = ann.psi_vector(psi, es)
    vp = U.matrix(N) @ v
    vp /= np.linalg.norm(vp)
    d_ref = np.sqrt(1.0 - abs(np.vdot(v / np.linalg.norm(v), vp)) ** 2)
    assert d == pytest.approx(d_ref, rel=1e-3, abs=1e-7)


def test_hsd_gradient_finite_differences():
    """test/test_HilbertSpaceDistance.py:69-131: psi' a copy of psi, U a single sigma_x."""
    N, M = 6, 6
    psi = deep(N, M, 4)
    es = ann.ExactSummationSpins(N)
    psi.calibrate(es)
    psi1 = +psi
    op = ann.Operator(ann.sigma_x(2))
    hsd = ann.HilbertSpaceDistance(psi.num_params)
    g, _ = hsd.gradient(psi, psi1, op, True, es, 1.0)
    eps = 1e-6
    p0 = psi.params

    def diff(delta):
        psi1.params = p0 + delta
        plus = hsd(psi, psi1, op, True, es)
        psi1.params = p0 - delta
        minus = hsd(psi, psi1, op, True, es)
        return (plus - minus) / (2 * eps)

    g_ref = np.zeros(psi.num_params, complex)
    for k in range(psi.num_params):
        dk = np.zeros(psi.num_params, complex)
        dk[k] = eps
        g_ref[k] = diff(dk)
        dk[k] = 1j * eps
        g_ref[k] += 1j * diff(dk)
    np.testing.assert_allclose(g, g_ref, rtol=1e-3, atol=1e-4)


def test_hsd_monte_carlo_matches_exact():
    N, M = 10, 20
    psi = deep(N, M, 5, precision="fp32")
    psi_p = deep(N, M, 6, precision="fp32", scale=0.12)
    es = ann.ExactSummationSpins(N)
    psi.normalize(es)
    psi_p.normalize(es)
    op = ann.Operator(ann.identity() + 0.05j * ann.transverse_field_ising_1d(N, 1.0))
    hsd = ann.HilbertSpaceDistance(psi_p.num_params)
    d_ex = hsd(psi, psi_p, op, True, es)
    mc = ann.MonteCarloSpins(1 << 18, 2, 20, 4096, True, seed=9)
    d_mc = hsd(psi, psi_p, op, True, mc)
    assert abs(d_mc - d_ex) < 0.05 * d_ex, (d_mc, d_ex)


@pytest.mark.parametrize("form", ["unitary", "exponential"])
@pytest.mark.parametrize("nu", [1.0, 0.5])
def test_hsd_matches_reference_fixture(form, nu):
    """Distance and gradient on the GPU (FP64 kernels, exact summation) against the
    reference's own HilbertSpaceDistance run on the same PsiDeep pair
    (tests/golden/hsd_n8_m8.npz; source/network_functions/HilbertSpaceDistance.cu.template:16-168).
    The reference's log psi omits a.s, so both networks take a_in_log_psi=False."""
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "hsd_n8_m8.npz")))
    N, M = int(g["N"]), int(g["M"])
    conn = np.array([[i] * M for i in range(N)], np.uint32)

    def make(p, fw, lp):
        return ann.PsiDeep(N, p[:N], [p[N:N + M]], [conn], [p[N + M:].reshape(N, M)], fw, lp[0], True,
                           a_in_log_psi=False, precision="fp64")
    psi = make(g["params"], g["fw"], g["lp"])
    psi_p = make(g["params_p"], g["fw_p"], g["lp_p"])
    a, b, c = g[f"{form}_op_a"], g[f"{form}_op_b"], g[f"{form}_op_c"]
    expr = ann.PauliExpression({(int(ai), int(bi)): complex(ci) for ai, bi, ci in zip(a, b, c)})
    op = ann.Operator(expr)
    es = ann.ExactSummationSpins(N)
    hsd = ann.HilbertSpaceDistance(psi_p.num_params)
    tag = f"{form}_nu{nu:g}"
    d = hsd(psi, psi_p, op, form == "unitary", es)
    grad, d2 = hsd.gradient(psi, psi_p, op, form == "unitary", es, nu)
    np.testing.assert_allclose(d, g[f"{tag}_dist"][0], rtol=1e-10)
    np.testing.assert_allclose(d2, g[f"{tag}_dist"][1], rtol=1e-10)
    assert np.abs(grad - g[f"{tag}_grad"]).max() <= 1e-9 * np.abs(g[f"{tag}_grad"]).max()
