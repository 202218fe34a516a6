"""Learned proposal (MADE): forward, gradients, Adam and sampling kernels against the
FP64 numpy restatement in oracle/made_oracle.py, and the Metropolis-Hastings chain it
drives: |psi|^2 stays the stationary distribution, and on a bimodal |psi|^2 the learned
moves cross between the modes where single-flip Metropolis stays trapped."""

import numpy as np
import pytest

import made_oracle as mo

pytestmark = pytest.mark.gpu

ann = pytest.importorskip("annongpu_gb300")


def oracle_weights(m):
    W1, b1, W2, b2 = m.params
    # the kernels read BF16 weights and accumulate in FP32
    return mo.bf16_round(W1), b1.astype(np.float64), mo.bf16_round(W2), b2.astype(np.float64)


def randomise(m, rng, scale=0.5):
    W1, b1, W2, b2 = m.params
    m1, m2 = mo.masks(m.N, m.H)
    W1 = (scale * rng.standard_normal(W1.shape) * m1).astype(np.float32)
    W2 = (scale * rng.standard_normal(W2.shape) * m2).astype(np.float32)
    b1 = (0.1 * rng.standard_normal(b1.shape)).astype(np.float32)
    b2 = (0.3 * rng.standard_normal(b2.shape)).astype(np.float32)
    m.params = (W1, b1, W2, b2)


@pytest.mark.parametrize("N,H", [(12, 64), (64, 256), (100, 128)])
def test_log_prob_and_gradient(N, H):
    rng = np.random.default_rng(N + H)
    m = ann.MADE(N, H, seed=3)
    randomise(m, rng)
    confs = [int(rng.integers(0, 2 ** 62)) | (int(rng.integers(0, 2 ** 62)) << 64) for _ in range(200)]
    confs = [c & ((1 << N) - 1) for c in confs]
    rows = np.array([[c & 0xFFFFFFFFFFFFFFFF, c >> 64] for c in confs], np.uint64)
    W1, b1, W2, b2 = oracle_weights(m)
    x = np.array([[(c >> i) & 1 for i in range(N)] for c in confs], np.float64)
    want = mo.forward(x, W1, b1, W2, b2)[3]
    got = m.log_prob(rows)
    np.testing.assert_allclose(got, want, rtol=2e-5, atol=2e-4)
    # gradient of the mean -log q against FP64 backprop (masked entries)
    gW1, gb1, gW2, gb2, loss = m.gradient(rows)
    pre, h, l, logq = mo.forward(x, W1, b1, W2, b2)
    dl = (1 / (1 + np.exp(-l)) - x) / len(x)
    m1, m2 = mo.masks(N, H)
    rW2 = (dl.T @ h) * m2
    rW1 = ((dl @ W2) * (pre > 0)).T @ x * m1
    np.testing.assert_allclose(loss, -logq.mean(), rtol=1e-5)
    for got_g, ref_g in ((gW1 * m1, rW1), (gW2 * m2, rW2), (gb2, dl.sum(0))):
        scale = np.abs(ref_g).max()
        assert np.abs(got_g - ref_g).max() < 2e-4 * scale + 1e-7


def test_adam_step_keeps_masks():
    N, H = 10, 64
    rng = np.random.default_rng(1)
    m = ann.MADE(N, H, seed=9)
    randomise(m, rng, 0.3)
    confs = rng.integers(0, 1 << N, 512).astype(np.uint64)
    W1, b1, W2, b2 = m.params
    g = m.gradient(confs)
    m.train(confs, steps=1, batch=512, lr=1e-2)
    W1n, b1n, W2n, b2n = m.params
    m1, m2 = mo.masks(N, H)
    # first Adam step moves every live weight by lr * sign(g) (bias-corrected moments)
    for old, new, gr, mask in ((W1, W1n, g[0], m1), (W2, W2n, g[2], m2)):
        live = (mask > 0) & (np.abs(gr) > 1e-4)
        np.testing.assert_allclose((old - new)[live], 1e-2 * np.sign(gr[live]), rtol=1e-3, atol=1e-6)
        assert np.all(new[mask == 0] == 0)


def test_sampling_distribution():
    N, H = 6, 32
    rng = np.random.default_rng(5)
    m = ann.MADE(N, H, seed=1)
    randomise(m, rng, 0.8)
    n = 1 << 18
    confs, logq = m.sample(n, seed=77)
    c = confs[:, 0].astype(np.int64)
    np.testing.assert_allclose(logq, m.log_prob(confs), rtol=1e-5, atol=1e-4)
    q = np.exp(m.log_prob(np.arange(1 << N, dtype=np.uint64)))
    np.testing.assert_allclose(q.sum(), 1.0, rtol=1e-4)
    freq = np.bincount(c, minlength=1 << N) / n
    sigma = np.sqrt(q * (1 - q) / n)
    assert np.all(np.abs(freq - q) < 5 * sigma + 1e-6)


def bimodal_rbm(N):
    """W_ij = 0.25 (all-to-all), log-cosh activation: |psi|^2 peaks at magnetisation +-N."""
    W = 0.25 * np.ones((N, N)) + 0.01 * np.random.default_rng(0).standard_normal((N, N))
    return ann.PsiRBM(W, 1.0, 0.0, True, activation="logcosh", precision="fp32")


def test_learned_proposal_crosses_modes_and_keeps_psi2():
    N = 12
    psi = bimodal_rbm(N)
    es = ann.ExactSummationSpins(N)
    psi.normalize(es)
    p = np.abs(ann.psi_vector(psi, es)) ** 2
    p /= p.sum()
    rng = np.random.default_rng(2)
    train = rng.choice(1 << N, size=16384, p=p).astype(np.uint64)
    made = ann.MADE(N, 64, seed=4)
    loss = made.train(train, steps=1500, batch=2048, lr=1e-2)
    entropy = -(p[p > 0] * np.log(p[p > 0])).sum()
    assert loss < entropy + 0.7, (loss, entropy)
    H = ann.transverse_field_ising_1d(N, 1.0)
    op = ann.Operator(H)
    e_exact = ann.ExpectationValue()(op, psi, es)
    mag = np.array([2 * bin(k).count("1") - N for k in range(1 << N)])
    n_chains, T = 256, 64

    def magnetisations(mc):
        conf, _, _ = mc.samples()
        return np.array([2 * bin(int(c)).count("1") - N for c in conf[:, 0]]).reshape(T, n_chains)

    # single-flip Metropolis only: every chain stays in the mode it thermalised into
    local = ann.MonteCarloSpins(n_chains * T, 1, 20, n_chains, True, seed=5)
    ann.ExpectationValue()(op, psi, local)
    m_loc = magnetisations(local)
    crossed_local = np.mean((m_loc.max(0) > 0) & (m_loc.min(0) < 0))
    # learned independence moves (one per sample, no local sweeps)
    learned = ann.MonteCarloSpins(n_chains * T, 0, 20, n_chains, True, seed=5)
    learned.set_proposal(made, indep_per_sample=1)
    e = ann.ExpectationValue()(op, psi, learned)
    m_lrn = magnetisations(learned)
    crossed_learned = np.mean((m_lrn.max(0) > 0) & (m_lrn.min(0) < 0))
    acc = learned.proposal_acceptance
    assert acc > 0.3, acc
    assert crossed_local < 0.05 and crossed_learned > 0.9, (crossed_local, crossed_learned)
    # |psi|^2 is kept: magnetisation histogram and energy agree with exact summation
    _, _, el = learned.samples()
    se = el.real.reshape(T, n_chains).mean(0).std(ddof=1) / np.sqrt(n_chains)
    assert abs(e.real - e_exact.real) < 3 * se + 1e-6, (e, e_exact, se)
    p_up = p[mag > 0].sum()
    frac_up = (m_lrn > 0).mean()
    assert abs(frac_up - p_up) < 0.05


def test_proposal_dropped_below_acceptance_threshold():
    N = 12
    psi = bimodal_rbm(N)
    made = ann.MADE(N, 64, seed=4)  # untrained: proposes almost uniformly
    mc = ann.MonteCarloSpins(256 * 8, 1, 5, 256, True, seed=1)
    mc.set_proposal(made, indep_per_sample=2, min_acceptance=0.2)
    ann.ExpectationValue()(ann.Operator(ann.transverse_field_ising_1d(N)), psi, mc)
    assert mc.proposal_acceptance < 0.2 and mc.proposal_dropped
    # the next call runs local Metropolis alone
    ann.ExpectationValue()(ann.Operator(ann.transverse_field_ising_1d(N)), psi, mc)
    assert mc.acceptance_rate > 0.0


def test_drop_rule_acts_inside_graph_replays_and_rearms():
    """The drop rule runs on the device after each sampling pass (a flag the sampler
    reads), so it also acts in replays of a captured SR step; set_proposal re-arms the
    proposal (the bench does so after each retraining)."""
    import torch
    N = 12
    psi = bimodal_rbm(N)
    es = ann.ExactSummationSpins(N)
    psi.normalize(es)
    p = np.abs(ann.psi_vector(psi, es)) ** 2
    p /= p.sum()
    train = np.random.default_rng(2).choice(1 << N, size=16384, p=p).astype(np.uint64)
    made = ann.MADE(N, 64, seed=4)
    made.train(train, steps=800, batch=2048, lr=1e-2)
    op = ann.Operator(ann.transverse_field_ising_1d(N, 1.0))
    mc = ann.MonteCarloSpins(256, 1, 5, 256, True, seed=1, persistent=True)
    # accepted learned moves fall short of a 99 % threshold: dropped after the first pass
    mc.set_proposal(made, indep_per_sample=2, min_acceptance=0.99)
    st = torch.cuda.Stream()
    td = ann.TDVP(psi.num_params, s_mode="fp32", solver="fp64", stream=st)
    td.capture_sr_step(op, psi, mc, 1e-3, 0.0, st)  # one eager step (the proposal runs), then capture
    mc.refresh_stats(st)
    assert mc.proposal_dropped and mc.proposal_acceptance > 0.1
    td.launch_sr_step(st)
    mc.refresh_stats(st)
    assert mc.proposal_dropped and mc.proposal_acceptance == 0.0  # the replay ran local moves only
    mc.set_proposal(made, indep_per_sample=2, min_acceptance=0.99)
    assert not mc.proposal_dropped
    td.launch_sr_step(st)
    mc.refresh_stats(st)
    assert mc.proposal_dropped and mc.proposal_acceptance > 0.1  # re-armed: learned moves ran once more
