"""Autotuner on the GPU: every knob is timed on the workload and the fastest choice
lands in the tuning table; the choices change speed, not results (sampler launch
shapes, whole- and half-warp chains included, give bit-identical chains, reduction slabs agree to the FP32-sum bound
rtol 2e-5, the two Cholesky trailing updates, every count of SMs held back for the
panel and both update ranks (per panel, per panel pair) give the same refined solve to
rtol 1e-8,
the bound of solves refined to ||r||/||F|| <= 1e-12 at condition numbers near 1e3)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ann = pytest.importorskip("annongpu_gb300")


def workload(seed=3, N=16, M=32, chains=2048):
    rng = np.random.default_rng(seed)
    c = lambda *s: 0.02 * (rng.standard_normal(s) + 1j * rng.standard_normal(s))  # noqa: E731
    psi = ann.PsiRBM(c(N, M), 1.0, 0.0, True, a=c(N), b=c(M), precision="fp32")
    op = ann.Operator(ann.transverse_field_ising_1d(N, 1.0))
    mc = ann.MonteCarloLoop(chains, 2, 8, chains, True, seed=seed, persistent=True)
    td = ann.TDVP(psi.num_params, s_mode="bf16", solver="mixed")
    return psi, op, mc, td


def test_autotune_fills_table_and_choices_keep_results():
    ann.set_tuning({}, clear=True)
    psi, op, mc, td = workload()
    td.eval(op, psi, mc)  # thermalises the persistent chains
    conf0, ctr0 = mc.get_chains()
    rep = ann.autotune(op, psi, mc, td)
    # the rank of the updates and the SMs held back for the panel are timed only when the
    # tensor-core update wins (Np = 560 is even: the pair form applies)
    tc_won = min(rep["chol.update"], key=rep["chol.update"].get) == 1
    knobs = {"rbm_mc.team", "rbm_mc.wpb", "rbm_mc.wsmem", "stats.slab", "chol.update"}
    if tc_won:
        knobs |= {"chol.pair", "chol.reserve"}
    assert set(rep) == knobs, rep
    assert set(rep["rbm_mc.wpb"]) == {2, 4, 8} and set(rep["chol.update"]) == {0, 1}
    assert set(rep["rbm_mc.team"]) == {32, 16}
    if tc_won:
        assert set(rep["chol.reserve"]) == {0, 16, 32, 48, 64} and set(rep["chol.pair"]) == {0, 1}
    assert all(ms > 0 for d in rep.values() for ms in d.values())
    # the caller's chains did not move (the sampler was timed on a copy)
    conf1, ctr1 = mc.get_chains()
    assert np.array_equal(conf0, conf1) and np.array_equal(ctr0, ctr1)
    table = ann.tuning_table()
    assert len(table) == len(knobs)
    wkey = next(k for k in table if "/rbm_mc.wpb/" in k)
    skey = next(k for k in table if "/stats.slab/" in k)
    ckey = next(k for k in table if "/chol.update/" in k)
    rkey = ckey.replace("/chol.update/", "/chol.reserve/")
    pkey = ckey.replace("/chol.update/", "/chol.pair/")
    # every sampler launch shape (whole- or half-warp chains, CTA size, W in shared memory
    # or read through L1) gives the same chains, samples and O rows
    mkey = next(k for k in table if "/rbm_mc.wsmem/" in k)
    tkey = next(k for k in table if "/rbm_mc.team/" in k)
    results = []
    for tl, w, m in ((32, 2, 1), (32, 4, 0), (32, 8, 1), (32, 8, 0), (16, 8, 1), (16, 4, 0), (16, 2, 1)):
        ann.set_tuning({tkey: tl, wkey: w, mkey: m})
        mc.set_chains(conf0, ctr0)
        td.eval(op, psi, mc)
        results.append((mc.samples(), td.F_vector))
    for (s, F) in results[1:]:
        for x, y in zip(s, results[0][0]):
            assert np.array_equal(x, y)
        np.testing.assert_array_equal(F, results[0][1])
    # reduction slabs: same F up to FP32 summation order
    Fs = []
    for sl in (128, 512):
        ann.set_tuning({skey: sl})
        mc.set_chains(conf0, ctr0)
        td.eval(op, psi, mc)
        Fs.append(td.F_vector)
    assert np.abs(Fs[0] - Fs[1]).max() <= 2e-5 * np.abs(Fs[1]).max()
    # Cholesky trailing update: the refined solutions agree
    d = []
    for m in (0, 1):
        ann.set_tuning({ckey: m})
        d.append(td.solve(1e-3))
        assert not td.solver_info["fell_back"]
    np.testing.assert_allclose(d[0], d[1], rtol=1e-8, atol=1e-8 * np.abs(d[1]).max())
    # SMs held back for the panel beside the persistent update, updates per panel or per
    # panel pair: the same refined solution
    for r, pr in ((0, 1), (64, 1), (32, 0)):
        ann.set_tuning({ckey: 1, rkey: r, pkey: pr})
        x = td.solve(1e-3)
        assert not td.solver_info["fell_back"]
        np.testing.assert_allclose(x, d[1], rtol=1e-8, atol=1e-8 * np.abs(d[1]).max())
    ann.set_tuning({}, clear=True)


def test_panel_pair_update_alone_matches_per_panel():
    """The rank-128 update per panel pair against one rank-64 update per panel with no
    refinement to hide a wrong factor (solver "fp32": one FP32 Cholesky solve): on the
    same S both unrefined solutions have the FP32 factorisation's residual and agree to
    its bound; in the mixed solver both forms need the same number of refinement solves.
    Np = 560 ends in a partial pair (560 = 4 pairs + one panel of 64 + 48)."""
    ann.set_tuning({}, clear=True)
    psi, op, mc, td = workload()
    assert psi.num_params == 560
    td.eval(op, psi, mc)
    ann.autotune(op, psi, mc, td)  # times the knobs on its own evaluations: S and F move
    td.eval(op, psi, mc)
    ref = td.solve(1e-3)  # mixed: refined to ||r|| / ||F|| <= 1e-12
    table = ann.tuning_table()
    ckey = next(k for k in table if "/chol.update/" in k)
    pkey = ckey.replace("/chol.update/", "/chol.pair/")
    unrefined, iters = {}, {}
    for pair in (0, 1):
        ann.set_tuning({ckey: 1, pkey: pair})
        td.set_solver("fp32")
        unrefined[pair] = td.solve(1e-3)
        info = td.solver_info
        assert info["update_form"] == ("tensor core, rank 128 per panel pair" if pair else
                                       "tensor core, rank 64 per panel"), info
        assert info["residual_first"] < 1e-4, info
        td.set_solver("mixed", 6, 1e-12)
        x = td.solve(1e-3)
        iters[pair] = td.solver_info["solves"]
        np.testing.assert_allclose(x, ref, rtol=1e-8, atol=1e-8 * np.abs(ref).max())
    scale = np.abs(ref).max()
    for pair in (0, 1):
        assert np.abs(unrefined[pair] - ref).max() <= 1e-3 * scale
    assert np.abs(unrefined[0] - unrefined[1]).max() <= 2e-3 * scale
    assert iters[0] == iters[1], iters
    ann.set_tuning({}, clear=True)


@pytest.mark.parametrize("N,M,learned,move", [(64, 128, True, "single_flip"), (70, 40, False, "exchange_pairs")])
def test_half_warp_chains_equal_whole_warp_chains(N, M, learned, move):
    """Half-warp chains (two per warp; at N = 64, M = 128 eight hidden units per lane) keep
    one partial sum per virtual lane, so their chains, log psi, E_loc and O rows equal the
    whole-warp sampler's bit for bit: with the 8x8 TFIM and learned moves, and with
    two-word configurations (N = 70) under exchange moves."""
    import torch
    ann.set_tuning({}, clear=True)
    rng = np.random.default_rng(N)
    c = lambda *s: 0.05 * (rng.standard_normal(s) + 1j * rng.standard_normal(s))  # noqa: E731
    psi = ann.PsiRBM(c(N, M), 1.0, 0.0, True, a=c(N), b=c(M), precision="fp32")
    H = ann.transverse_field_ising_2d(8, 8, h=3.04) if N == 64 else ann.transverse_field_ising_1d(N, 1.0)
    op = ann.Operator(H)
    chains = 2048
    mc = ann.MonteCarloLoop(chains, 4, 4, chains, True, seed=9, persistent=True, move=move,
                            n_up=None if move == "single_flip" else N // 2)
    if learned:
        made = ann.MADE(N, 64, seed=2)
        mc.set_proposal(made, indep_per_sample=2, min_acceptance=0.0)
    td = ann.TDVP(psi.num_params, s_mode="bf16", solver="mixed")
    td.eval(op, psi, mc)  # thermalises the persistent chains
    conf0, ctr0 = mc.get_chains()
    mpad = 32 * ((M + 31) // 32)
    key = (f"dev{torch.cuda.current_device()}/rbm_mc.team/N{N}.M{mpad}.U{mpad // 32}.P0"
           f".made{1 if learned else 0}")
    out = {}
    for tl in (32, 16):
        ann.set_tuning({key: tl}, clear=True)
        mc.set_chains(conf0, ctr0)
        td.eval(op, psi, mc)
        mc.refresh_stats()  # TDVP evaluations leave the acceptance counters to the caller
        out[tl] = (mc.samples(), td.F_vector, mc.get_chains(), mc.acceptance_rate,
                   mc.proposal_acceptance if learned else None)
    (s32, F32, ch32, a32, p32), (s16, F16, ch16, a16, p16) = out[32], out[16]
    for x, y in zip(s16, s32):
        assert np.array_equal(x, y)
    for x, y in zip(ch16, ch32):
        assert np.array_equal(x, y)
    np.testing.assert_array_equal(F16, F32)
    assert a16 == a32 and 0.0 < a32 < 1.0
    if learned:
        assert p16 == p32 and p32 > 0.0, p32
    ann.set_tuning({}, clear=True)
