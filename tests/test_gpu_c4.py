"""The alpha = 4 RBM shapes of the learned-proposal workload (N = 64 sites, M = 256 hidden
units, Np = 64 + 256 + 64 * 256 = 16704; the reference stops at M = 128,
include/quantum_state/PsiRBM.hpp:47): log psi, O_k and local energies against the FP64
oracle, Philox chains identical to the oracle's, and Metropolis-Hastings chains with the
learned independence moves sampling the same |psi|^2 as single-flip Metropolis.

Tolerances: complex128 kernels rtol 1e-10 (local energies 1e-9); complex64 kernels 5e-5
of max(1, |value|); Monte Carlo energies within 4 combined standard errors."""

import numpy as np
import pytest

from pyoracle import RbmDesc

pytestmark = pytest.mark.gpu

ann = pytest.importorskip("annongpu_gb300")

N, M = 64, 256


def cplx(rng, shape, scale):
    return scale * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))


def alpha4(precision, scale=0.05, seed=64, activation="poly"):
    rng = np.random.default_rng(seed)
    a, b, W = cplx(rng, N, 0.02), cplx(rng, M, 0.02), cplx(rng, (N, M), scale)
    gpu = ann.PsiRBM(W, 1.0, 0.0, True, a=a, b=b, precision=precision, activation=activation)
    ref = RbmDesc(N, M, W, a=a, b=b, layout=1, activation={"poly": 0, "logcosh": 1}[activation])
    return gpu, ref


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 5e-5)])
def test_alpha4_matches_oracle(oracle, precision, tol):
    gpu, ref = alpha4(precision)
    assert gpu.num_params == 16704
    H = ann.transverse_field_ising_1d(N, 1.0)
    rng = np.random.default_rng(3)
    confs = [int(x) for x in rng.integers(0, 2**63, 6, dtype=np.uint64)]
    el = ann.local_energies(gpu, ann.Operator(H), confs)
    for k, s in enumerate(confs):
        lp = oracle.log_psi(ref, s)
        assert abs(ann.log_psi_s(gpu, ann.Spins(s, N)) - lp) <= tol * max(1.0, abs(lp))
        O_ref = oracle.O_k(ref, s)
        assert np.abs(ann.psi_O_k(gpu, ann.Spins(s, N)) - O_ref).max() <= tol * max(1.0, np.abs(O_ref).max())
        e_ref = oracle.local_energy(ref, H, s)
        assert abs(el[k] - e_ref) <= 10 * tol * max(1.0, abs(e_ref)), (k, el[k], e_ref)


def test_alpha4_philox_chains_match_oracle(oracle):
    gpu, ref = alpha4("fp64", scale=0.1)
    H = ann.transverse_field_ising_1d(N, 1.0)
    n_chains, spc, sw, th, seed = 32, 2, 1, 2, 0xA4A4
    mc = ann.MonteCarloSpins(spc * n_chains, sw, th, n_chains, True, seed=seed, persistent=True)
    ann.ExpectationValue()(ann.Operator(H), gpu, mc)
    conf, lp, el = mc.samples()
    r = oracle.mc_philox(ref, H, n_chains, seed, spc, sw, th)
    assert r["tie"][0] > 1e-12
    np.testing.assert_array_equal(conf[:, 0], r["sconf"])
    np.testing.assert_allclose(lp, r["slp"], rtol=1e-10)
    np.testing.assert_allclose(el, r["seloc"], rtol=1e-9, atol=1e-10)


def test_alpha4_learned_moves_sample_psi2():
    """MADE 64 -> 256 -> 64 trained on 65536 chain configurations; chains that add two
    learned independence moves to one local sweep per sample give the same energy as
    chains of eight local sweeps per sample (log cosh activation: the polynomial grows like
    z^6 at these weights)."""
    gpu, _ = alpha4("fp32", scale=0.05, seed=7, activation="logcosh")
    op = ann.Operator(ann.transverse_field_ising_1d(N, 1.0))
    chains, T = 4096, 16
    prep = ann.MonteCarloSpins(chains, 1, 32, chains, True, seed=2, persistent=True)
    prep.set_history(65536)
    for _ in range(16):
        ann.ExpectationValue()(op, gpu, prep)
    made = ann.MADE(N, 256, seed=3)
    made.train_on_samples(prep, steps=256, batch=4096, lr=3e-3)
    learned = ann.MonteCarloSpins(chains * T, 1, 0, chains, True, seed=4, persistent=True)
    learned.set_chains(*prep.get_chains())
    learned.set_proposal(made, indep_per_sample=2, min_acceptance=0.0)
    e_l = ann.ExpectationValue()(op, gpu, learned).real
    assert learned.proposal_acceptance > 0.02, learned.proposal_acceptance
    _, _, el_l = learned.samples()
    local = ann.MonteCarloSpins(chains * T, 8, 0, chains, True, seed=5, persistent=True)
    local.set_chains(*prep.get_chains())
    e_0 = ann.ExpectationValue()(op, gpu, local).real
    _, _, el_0 = local.samples()
    se = lambda el: el.real.reshape(T, chains).mean(0).std(ddof=1) / np.sqrt(chains)  # noqa: E731
    assert abs(e_l - e_0) < 4 * np.hypot(se(el_l), se(el_0)), (e_l, e_0)
