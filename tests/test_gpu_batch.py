"""Batched uneven instances: one persistent sampling launch over 1-D TFIM instances of
different lengths, fields and RBM widths. A batched chain is the same chain as one
sampled alone (bit-identical rows); energies agree with exact summation; batched SR
steps (and their graph replay) equal per-instance SR steps."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ann = pytest.importorskip("annongpu_gb300")

SPECS = [(8, 1), (12, 2), (16, 4), (10, 2), (20, 1), (14, 4)]  # (L, alpha)


def make_instance(L, alpha, seed, tdvp=False, s_mode="bf16"):
    rng = np.random.default_rng(seed)
    M = alpha * L
    a = 0.02 * (rng.standard_normal(L) + 1j * rng.standard_normal(L))
    b = 0.02 * (rng.standard_normal(M) + 1j * rng.standard_normal(M))
    W = 0.05 * (rng.standard_normal((L, M)) + 1j * rng.standard_normal((L, M)))
    h = rng.uniform(0.5, 1.5)
    psi = ann.PsiRBM(W, 1.0, 0.0, True, a=a, b=b, precision="fp32")
    op = ann.Operator(ann.transverse_field_ising_1d(L, h))
    chains = 64 * max(2, int(np.ceil(psi.num_params / 256)))
    mc = ann.MonteCarloSpins(chains * 8, 2, 10, chains, True, seed=1000 + seed, persistent=True)
    td = ann.TDVP(psi.num_params, s_mode=s_mode) if tdvp else None
    return psi, op, mc, td, h


def build(tdvp=False):
    return [make_instance(L, al, seed=i, tdvp=tdvp) for i, (L, al) in enumerate(SPECS)]


def test_batched_chains_equal_single_chains():
    inst = build()
    batch = ann.Batch([x[0] for x in inst], [x[1] for x in inst], [x[2] for x in inst])
    batch.sample()
    E = batch.energies()
    ref = build()
    for k, ((psi, op, mc, _, _), (psi2, op2, mc2, _, _)) in enumerate(zip(inst, ref)):
        e2 = ann.ExpectationValue()(op2, psi2, mc2)
        c1, l1, el1 = mc.samples()
        c2, l2, el2 = mc2.samples()
        np.testing.assert_array_equal(c1, c2)
        np.testing.assert_array_equal(l1, l2)
        np.testing.assert_array_equal(el1, el2)
        assert E[k] == e2


def test_batched_energies_match_exact_summation():
    inst = build()
    batch = ann.Batch([x[0] for x in inst], [x[1] for x in inst], [x[2] for x in inst])
    for _ in range(3):
        batch.sample()  # persistent chains: later passes are equilibrated
    E = batch.energies()
    for k, (psi, op, mc, _, _) in enumerate(inst):
        L = SPECS[k][0]
        es = ann.ExactSummationSpins(L)
        psi.normalize(es)
        e_exact = ann.ExpectationValue()(op, psi, es)
        _, _, el = mc.samples()
        chains = mc.num_markov_chains
        se = el.real.reshape(-1, chains).mean(0).std(ddof=1) / np.sqrt(chains)
        assert abs(E[k].real - e_exact.real) < 4 * se + 1e-6, (k, E[k], e_exact, se)


def test_batched_sr_steps_equal_single_steps_and_graph():
    import torch
    inst = build(tdvp=True)
    ref = build(tdvp=True)
    st = torch.cuda.Stream()
    batch = ann.Batch([x[0] for x in inst], [x[1] for x in inst], [x[2] for x in inst], [x[3] for x in inst],
                      stream=st)
    for _ in range(2):
        batch.sr_step(1e-3, 0.02)
    for psi, op, mc, td, _ in ref:
        for _ in range(2):
            td.sr_step(op, psi, mc, 1e-3, 0.02)
    st.synchronize()
    for (p1, *_), (p2, *_) in zip(inst, ref):
        np.testing.assert_array_equal(p1.params, p2.params)
    # graph: capture (one eager step inside), replay two more
    batch.capture_sr_step(1e-3, 0.02, st)
    batch.launch_sr_step(st)
    batch.launch_sr_step(st)
    for psi, op, mc, td, _ in ref:
        for _ in range(3):
            td.sr_step(op, psi, mc, 1e-3, 0.02)
    st.synchronize()
    torch.cuda.synchronize()
    for (p1, *_), (p2, *_) in zip(inst, ref):
        np.testing.assert_array_equal(p1.params, p2.params)


def test_batched_mixed_solver_steps_equal_single_steps():
    """The same with the mixed-precision solver (FP32 tcgen05 Cholesky + refinement) on every
    instance: the batch runs those solves one instance after another, and each instance's
    parameters after eager and graph-replayed batched steps equal its single-instance steps."""
    import torch
    inst = build(tdvp=True)
    ref = build(tdvp=True)
    for x in inst + ref:
        x[3].set_solver("mixed", 10, 1e-12)
    st = torch.cuda.Stream()
    batch = ann.Batch([x[0] for x in inst], [x[1] for x in inst], [x[2] for x in inst], [x[3] for x in inst],
                      stream=st)
    batch.sr_step(1e-3, 0.02)
    for psi, op, mc, td, _ in ref:
        td.sr_step(op, psi, mc, 1e-3, 0.02)
    st.synchronize()
    torch.cuda.synchronize()
    for (p1, *_), (p2, *_) in zip(inst, ref):
        np.testing.assert_array_equal(p1.params, p2.params)
    batch.capture_sr_step(1e-3, 0.02, st)  # one eager step, then the capture
    batch.launch_sr_step(st)
    for psi, op, mc, td, _ in ref:
        for _ in range(2):
            td.sr_step(op, psi, mc, 1e-3, 0.02)
    st.synchronize()
    torch.cuda.synchronize()
    for (p1, *_, t1, _), (p2, *_, t2, _) in zip(inst, ref):
        assert t1.solver_info["residual_last"] <= 1e-12 and not t2.solver_info["fell_back"]
        np.testing.assert_array_equal(p1.params, p2.params)


def test_batched_learned_proposals_equal_single_chains():
    """Instances with a learned MADE proposal each (two independence moves per sample after
    the local sweeps) in the one persistent launch: every batched chain and its learned-move
    acceptance are the same as the instance sampled alone, and the proposal trains on the
    history ring the batched passes filled (losses as for the single instance; the weights
    themselves are not compared: Adam turns summation-order differences of near-zero
    gradients into steps of +-lr)."""
    def with_proposals(inst):
        mades = []
        for k, (psi, op, mc, _, _) in enumerate(inst):
            made = ann.MADE(psi.N, 64, seed=50 + k)
            mc.set_proposal(made, indep_per_sample=2, min_acceptance=0.0)
            mc.set_history(4 * mc.num_markov_chains)
            mades.append(made)
        return mades

    inst = build()
    m1 = with_proposals(inst)
    batch = ann.Batch([x[0] for x in inst], [x[1] for x in inst], [x[2] for x in inst])
    ref = build()
    m2 = with_proposals(ref)
    for rep in range(2):
        batch.sample()
        for psi2, op2, mc2, _, _ in ref:
            ann.ExpectationValue()(op2, psi2, mc2)
        for (psi, op, mc, _, _), (psi2, op2, mc2, _, _) in zip(inst, ref):
            c1, l1, el1 = mc.samples()
            c2, l2, el2 = mc2.samples()
            np.testing.assert_array_equal(c1, c2)
            np.testing.assert_array_equal(el1, el2)
            mc.refresh_stats()
            mc2.refresh_stats()
            assert mc.proposal_acceptance == mc2.proposal_acceptance
            assert mc.proposal_acceptance > 0.0
    for (made1, made2), (_, _, mc, _, _), (_, _, mc2, _, _) in zip(zip(m1, m2), inst, ref):
        l1 = made1.train_on_samples(mc, steps=4, batch=256, lr=1e-3)
        l2 = made2.train_on_samples(mc2, steps=4, batch=256, lr=1e-3)
        assert np.isfinite(l1) and abs(l1 - l2) <= 1e-2 * abs(l2), (l1, l2)
