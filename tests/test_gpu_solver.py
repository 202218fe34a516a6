"""SR solvers on the GPU: the mixed-precision solve (FP32 Cholesky + refinement with
FP64 residuals) against the FP64 oracle's S and F, against numpy on the GPU's own S
at sizes with many 64-wide panels, against the FP64 Cholesky solve, its fallback when
the refinement stalls, and inside a captured SR-step graph.

Tolerances: the refined solution satisfies ||F - (S + shift) x|| / ||F|| <= 1e-12
(checked on the device), so it agrees with numpy.linalg.solve to rtol 1e-8 at the
condition numbers used here (shift 1e-3)."""

import numpy as np
import pytest

from pyoracle import RbmDesc

pytestmark = pytest.mark.gpu

ann = pytest.importorskip("annongpu_gb300")


def cplx(rng, shape, scale):
    return scale * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))


def test_mixed_solver_matches_oracle(oracle):
    """Np = 12 + 24 + 288 = 324: five full 64-wide panels and a ragged one."""
    N, M = 12, 24
    rng = np.random.default_rng(3)
    a, b, W = cplx(rng, N, 0.05), cplx(rng, M, 0.05), cplx(rng, (N, M), 0.12)
    fw = np.ones(M, complex)
    conn = np.array([[(j + i) % N for j in range(M)] for i in range(N)], np.uint32)
    psi = ann.PsiDeep(N, a, [b], [conn], [W], fw, 0.0, True, precision="fp64")
    es = ann.ExactSummationSpins(N)
    psi.normalize(es)
    ref_desc = RbmDesc(N, M, W, a=a, b=b, fw=fw, conn=conn, log_prefactor=psi.log_prefactor, layout=1)
    H = ann.transverse_field_ising_1d(N, 1.0)
    ref = oracle.exact(ref_desc, H)
    td = ann.TDVP(psi.num_params, solver="mixed")
    td.eval(ann.Operator(H), psi, es)
    shift = 1e-3
    want = np.linalg.solve(ref["tS"] + shift * np.eye(psi.num_params), ref["tF"])
    delta, res = td.solve(shift, return_info=True)
    info = td.solver_info
    assert not info["fell_back"] and 1 <= info["solves"] <= 6, info
    assert res[1] <= 1e-12 and info["residual_last"] <= 1e-12, (res, info)
    np.testing.assert_allclose(delta, want, rtol=1e-8, atol=1e-9 * np.abs(want).max())


@pytest.mark.parametrize("update", ["tc", "simt"])
@pytest.mark.parametrize("N,M", [(32, 64), (24, 100)])
def test_mixed_solver_matches_numpy_on_gpu_S(N, M, update):
    """Monte Carlo S of a complex RBM with biases, Np = 2144 (34 panels, 17 tensor-core
    tiles per side) and Np = 2524 (40 panels, ragged last panel and tile), BF16
    tensor-core S; the mixed solve with either trailing update of its FP32 Cholesky
    against numpy on the same S and against the FP64 Cholesky solve."""
    rng = np.random.default_rng(N + M)
    a, b, W = cplx(rng, N, 0.01), cplx(rng, M, 0.01), cplx(rng, (N, M), 0.01)
    psi = ann.PsiRBM(W, 1.0, 0.0, True, a=a, b=b, precision="fp32")
    op = ann.Operator(ann.transverse_field_ising_1d(N, 1.0))
    mc = ann.MonteCarloLoop(4096, 2, 8, 4096, True, seed=11)
    td = ann.TDVP(psi.num_params, s_mode="bf16", solver="mixed")
    td.chol_update = update
    td.eval(op, psi, mc)
    S, F = td.S_matrix, td.F_vector
    shift = 1e-3
    want = np.linalg.solve(S + shift * np.eye(psi.num_params), F)
    d_mixed = td.solve(shift)
    info = td.solver_info
    assert not info["fell_back"] and info["residual_last"] <= 1e-12, info
    np.testing.assert_allclose(d_mixed, want, rtol=1e-8, atol=1e-9 * np.abs(want).max())
    td.set_solver("fp64")
    d_fp64 = td.solve(shift)
    np.testing.assert_allclose(d_mixed, d_fp64, rtol=1e-8, atol=1e-9 * np.abs(d_fp64).max())


def test_mixed_solver_more_block_rows_than_resident_ctas():
    """Np = 80 + 120 + 9600 = 9800: 154 block rows of 64, more than the triangular
    solves' cooperative launch holds at one CTA per SM on a 152-SM GPU, so CTAs own
    several block rows (the hand-off of solution blocks between rounds). The residual is
    checked on the host in FP64 as well as on the device, and the solution against the
    FP64 Cholesky solve."""
    N, M = 80, 120
    rng = np.random.default_rng(5)
    a, b, W = cplx(rng, N, 0.01), cplx(rng, M, 0.01), cplx(rng, (N, M), 0.01)
    psi = ann.PsiRBM(W, 1.0, 0.0, True, a=a, b=b, precision="fp32")
    assert psi.num_params == 9800
    op = ann.Operator(ann.transverse_field_ising_1d(N, 1.0))
    mc = ann.MonteCarloLoop(16384, 2, 8, 16384, True, seed=13)
    # the refinement count depends on the conditioning; the point here is the solves
    td = ann.TDVP(psi.num_params, s_mode="bf16", solver="mixed", max_iter=10)
    td.eval(op, psi, mc)
    shift = 1e-3
    d_mixed = td.solve(shift)
    info = td.solver_info
    assert not info["fell_back"] and info["residual_last"] <= 1e-12, info
    S, F = td.S_matrix, td.F_vector
    r = F - (S @ d_mixed + shift * d_mixed)
    assert np.linalg.norm(r) <= 1e-11 * np.linalg.norm(F)
    td.set_solver("fp64")
    d_fp64 = td.solve(shift)
    np.testing.assert_allclose(d_mixed, d_fp64, rtol=1e-8, atol=1e-9 * np.abs(d_fp64).max())


def test_mixed_solver_stall_falls_back_to_fp64():
    """One FP32 solve cannot reach a residual of 1e-15: the eager solve is redone
    with the FP64 Cholesky and gives exactly its answer."""
    N, M = 16, 32
    rng = np.random.default_rng(1)
    W = cplx(rng, (N, M), 0.05)
    psi = ann.PsiRBM(W, 1.0, 0.0, True, precision="fp32")
    op = ann.Operator(ann.transverse_field_ising_1d(N, 1.0))
    mc = ann.MonteCarloLoop(2048, 2, 8, 1024, True, seed=2)
    td = ann.TDVP(psi.num_params, solver="mixed", max_iter=1, tol=1e-15)
    td.eval(op, psi, mc)
    d1 = td.solve(1e-3)
    assert td.solver_info["fell_back"]
    td.set_solver("fp64")
    d2 = td.solve(1e-3)
    np.testing.assert_array_equal(d1, d2)


def test_mixed_solver_graph_replay_equals_eager():
    import torch
    N, M = 16, 48
    op = ann.Operator(ann.transverse_field_ising_1d(N, 1.0))
    rng = np.random.default_rng(8)
    W = cplx(rng, (N, M), 0.05)
    p1 = ann.PsiRBM(W, 1.0, 0.0, True, precision="fp32")
    p2 = ann.PsiRBM(W, 1.0, 0.0, True, precision="fp32")
    mc1 = ann.MonteCarloSpins(1024 * 2, 2, 5, 1024, True, seed=5, persistent=True)
    mc2 = ann.MonteCarloSpins(1024 * 2, 2, 5, 1024, True, seed=5, persistent=True)
    st = torch.cuda.Stream()
    t1 = ann.TDVP(p1.num_params, s_mode="bf16", solver="mixed", stream=st)
    t2 = ann.TDVP(p2.num_params, s_mode="bf16", solver="mixed", stream=st)
    t2.capture_sr_step(op, p2, mc2, 1e-3, 0.01, st)  # runs one eager step first
    t1.sr_step(op, p1, mc1, 1e-3, 0.01)
    for _ in range(3):
        t1.sr_step(op, p1, mc1, 1e-3, 0.01)
        t2.launch_sr_step(st)
    st.synchronize()
    assert not t1.solver_info["fell_back"] and t2.solver_info["residual_last"] <= 1e-12
    np.testing.assert_array_equal(p1.params, p2.params)


def test_complex64_S_store_keeps_values_and_solutions():
    """With the tensor-core S and the mixed solver, S is kept in complex64 (its values are
    FP32 sums) and the refinement's residual is formed in double-float arithmetic on the
    FP32 pipe. The same chains evaluated for the FP64 solver (S kept in complex128) give a
    bit-identical S and F; the mixed solve from the complex64 S agrees with the mixed
    solve from the complex128 S (FP64 residual) and with the FP64 Cholesky solve to the
    refinement's bound, and its residual checked on the host in FP64 is <= 2e-12; the FP64
    solve of the widened complex64 S equals the one of the complex128 S bit for bit, and a
    stalled refinement falls back to exactly that solve."""
    N, M = 32, 64  # Np = 2144
    rng = np.random.default_rng(21)
    a, b, W = cplx(rng, N, 0.01), cplx(rng, M, 0.01), cplx(rng, (N, M), 0.01)
    psi = ann.PsiRBM(W, 1.0, 0.0, True, a=a, b=b, precision="fp32")
    op = ann.Operator(ann.transverse_field_ising_1d(N, 1.0))
    mc = ann.MonteCarloLoop(4096, 2, 8, 4096, True, seed=17, persistent=True)
    t32 = ann.TDVP(psi.num_params, s_mode="bf16", solver="mixed")
    t32.eval(op, psi, mc)  # thermalises the persistent chains
    conf0, ctr0 = mc.get_chains()
    mc.set_chains(conf0, ctr0)
    t32.eval(op, psi, mc)
    t64 = ann.TDVP(psi.num_params, s_mode="bf16", solver="fp64")
    mc.set_chains(conf0, ctr0)
    t64.eval(op, psi, mc)
    S, F = t64.S_matrix, t64.F_vector
    assert np.array_equal(t32.S_matrix, S) and np.array_equal(t32.F_vector, F)
    shift = 1e-3
    d32 = t32.solve(shift)
    info = t32.solver_info
    assert not info["fell_back"] and info["residual_last"] <= 1e-12, info
    r = F - (S @ d32 + shift * d32)
    assert np.linalg.norm(r) <= 2e-12 * np.linalg.norm(F)
    t64.set_solver("mixed", 6, 1e-12)
    d64 = t64.solve(shift)
    scale = np.abs(d64).max()
    np.testing.assert_allclose(d32, d64, rtol=1e-9, atol=1e-10 * scale)
    t64.set_solver("fp64")
    dref = t64.solve(shift)
    np.testing.assert_allclose(d32, dref, rtol=1e-8, atol=1e-9 * scale)
    t32.set_solver("fp64")
    np.testing.assert_array_equal(t32.solve(shift), dref)
    # a fresh complex64 S (the complex128 copy stale) and a refinement that cannot converge
    t32.set_solver("mixed", 1, 1e-15)
    mc.set_chains(conf0, ctr0)
    t32.eval(op, psi, mc)
    d_fb = t32.solve(shift)
    assert t32.solver_info["fell_back"]
    np.testing.assert_array_equal(d_fb, dref)


def test_factorisation_event_timeline():
    """ann_set_factor_trace records the tagged events of the FP32 factorisation (pair form:
    per panel pair a tile-column update on the main stream, the look-ahead panel kernels);
    the times are ordered per stream and the trace is off again afterwards."""
    import ctypes as ct
    N, M = 32, 64  # Np = 2144: 34 panels of 64 (the last of 32 columns) in 17 pairs
    rng = np.random.default_rng(4)
    a, b, W = cplx(rng, N, 0.01), cplx(rng, M, 0.01), cplx(rng, (N, M), 0.01)
    psi = ann.PsiRBM(W, 1.0, 0.0, True, a=a, b=b, precision="fp32")
    op = ann.Operator(ann.transverse_field_ising_1d(N, 1.0))
    mc = ann.MonteCarloLoop(4096, 2, 8, 4096, True, seed=23)
    td = ann.TDVP(psi.num_params, s_mode="bf16", solver="mixed")
    td.chol_update = "tc"
    td.eval(op, psi, mc)
    td.solve(1e-3)
    if td.solver_info["update_form"] != "tensor core, rank 128 per panel pair":
        pytest.skip("the tuning table chose another update form")
    n_p = psi.num_params
    pairs, panels = (n_p + 127) // 128, (n_p + 63) // 64
    x0 = td.solve(1e-3)
    n = ct.c_uint(0)
    for level in (1, 2):  # 1: panel pairs; 2: also between the panel kernels
        ann._lib.call("ann_set_factor_trace", level)
        x = td.solve(1e-3)
        out = np.zeros(2 * 4096)
        ann._lib.call("ann_get_factor_trace", ann._lib.ptr(out), 4096, ct.byref(n))
        ann._lib.call("ann_set_factor_trace", 0)
        np.testing.assert_array_equal(x, x0)  # the trace changes timing, not results
        ev = out[: 2 * n.value].reshape(-1, 2)
        tags, t = ev[:, 0].astype(int), ev[:, 1]
        assert (tags == 200).sum() == pairs - 1 and (tags == 203).sum() == pairs - 1
        assert (tags == 100).sum() == pairs and (tags == 103).sum() == panels - pairs
        assert (tags == 101).sum() == (pairs if level == 2 else 0)
        assert (tags == 110).sum() == (panels if level == 2 else 0)
        for main in (t[np.isin(tags, [200, 201, 202, 203])], t[np.isin(tags, [100, 110, 101, 103])]):
            assert (np.diff(main) >= -1e-3).all()  # each stream's events in order (ms, event resolution)
        assert t.max() > 0
    # off: the next factorisation records nothing new
    td.solve(1e-3)
    ann._lib.call("ann_get_factor_trace", None, 0, ct.byref(n))
    assert n.value == 0
