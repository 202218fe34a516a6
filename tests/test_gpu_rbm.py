"""CUDA path vs the FP64 oracle for the RBM family (PsiRBM, PsiDeep with one hidden
layer): log psi, O_k, local energies, exact-summation TDVP quantities, Monte Carlo
chains (bit-exact proposal replay and Philox streams), SR solve and update.

Tolerances: complex128 kernels agree with the oracle to rtol 1e-10 (1e-9 for
accumulated quantities); complex64 kernels to the stated FP32 bounds per test.
"""

import numpy as np
import pytest

from pyoracle import RbmDesc

pytestmark = pytest.mark.gpu

ann = pytest.importorskip("annongpu_gb300")


def cplx(rng, shape, scale):
    return scale * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))


def mixed_h(N):
    H = ann.transverse_field_ising_1d(N, h=0.9, J=1.1)
    H = H + 0.3 * ann.sigma_y(1) * ann.sigma_y(2) + 0.2 * ann.sigma_x(0) * ann.sigma_z(3)
    H = H + 0.15 * ann.sigma_y(4 % N) + 0.05 * ann.sigma_y(0) * ann.sigma_y(2) * ann.sigma_y(5 % N)
    return H + 0.1 * ann.sigma_z(2)


class Case:
    """A random RBM-family wavefunction built twice: on the GPU and for the oracle."""

    def __init__(self, kind, N, M, C=None, seed=0, precision="fp64", activation="poly", a_in=True, scale=0.12):
        rng = np.random.default_rng(seed)
        self.N, self.M = N, M
        C = N if C is None else C
        self.C = C
        act = {"poly": 0, "logcosh": 1}[activation]
        if kind == "rbm":
            W = cplx(rng, (N, M), scale)
            fw = 0.8 + 0.3j
            self.gpu = ann.PsiRBM(W, fw, 0.1 - 0.2j, True, precision=precision, activation=activation)
            self.ref = RbmDesc(N, M, W, fw=np.full(M, fw), log_prefactor=0.1 - 0.2j, layout=0, a_in_log_psi=False,
                               activation=act)
        else:
            a = cplx(rng, N, 0.05)
            b = cplx(rng, M, 0.05)
            W = cplx(rng, (C, M), scale)
            fw = 1.0 + cplx(rng, M, 0.1)
            delta = 1 if M > N else (N // M if N % M == 0 else C)
            conn = np.array([[(j * delta + i) % N for j in range(M)] for i in range(C)], np.uint32)
            self.gpu = ann.PsiDeep(N, a, [b], [conn], [W], fw, -0.05 + 0.3j, True, a_in_log_psi=a_in,
                                   precision=precision, activation=activation)
            self.ref = RbmDesc(N, M, W, a=a, b=b, fw=fw, conn=conn, log_prefactor=-0.05 + 0.3j, layout=1,
                               a_in_log_psi=a_in, activation=act)


FP64 = dict(rtol=1e-10, atol=1e-12)


def normalize(c, N):
    """Normalises the GPU wavefunction and rebuilds the oracle description to match."""
    es = ann.ExactSummationSpins(N)
    c.gpu.normalize(es)
    lp = c.gpu.log_prefactor
    d = c.ref
    c.ref = RbmDesc(d.N, d.M, d.W, a=d.a, b=d.b, fw=d.fw, conn=d.conn, log_prefactor=lp, layout=d.struct.layout,
                    a_in_log_psi=d.struct.a_in_log_psi, activation=d.struct.activation)
    return es


@pytest.mark.parametrize("kind,N,M,C", [("rbm", 8, 8, None), ("rbm", 10, 40, None), ("deep", 8, 8, None),
                                        ("deep", 6, 12, 3), ("deep", 12, 64, 6), ("rbm", 70, 33, None)])
@pytest.mark.parametrize("a_in", [True, False])
def test_log_psi_and_O_k_fp64(oracle, kind, N, M, C, a_in):
    if kind == "rbm" and not a_in:
        pytest.skip("PsiRBM has no visible bias")
    c = Case(kind, N, M, C, seed=N + M, a_in=a_in)
    rng = np.random.default_rng(1)
    confs = [int(x) for x in rng.integers(0, 2**62, 6)]
    if N > 64:
        confs = [x | (int(y) << 64) for x, y in zip(confs, rng.integers(0, 2**62, 6))]
    for s in confs:
        s &= (1 << N) - 1
        np.testing.assert_allclose(ann.log_psi_s(c.gpu, ann.Spins(s, N)), oracle.log_psi(c.ref, s), **FP64)
        np.testing.assert_allclose(ann.psi_O_k(c.gpu, ann.Spins(s, N)), oracle.O_k(c.ref, s), **FP64)
    batch = ann.log_psi_batch(c.gpu, [s & ((1 << N) - 1) for s in confs])
    np.testing.assert_allclose(batch, [oracle.log_psi(c.ref, s & ((1 << N) - 1)) for s in confs], **FP64)


@pytest.mark.parametrize("activation", ["poly", "logcosh"])
def test_log_psi_fp32(oracle, activation):
    c = Case("deep", 16, 64, None, seed=5, precision="fp32", activation=activation)
    rng = np.random.default_rng(2)
    for s in rng.integers(0, 1 << 16, 8):
        s = int(s)
        ref = oracle.log_psi(c.ref, s)
        got = ann.log_psi_s(c.gpu, ann.Spins(s, 16))
        assert abs(got - ref) < 2e-5 * max(1.0, abs(ref))
        np.testing.assert_allclose(ann.psi_O_k(c.gpu, ann.Spins(s, 16)), oracle.O_k(c.ref, s), rtol=2e-5, atol=2e-6)


def test_activation_function_matches_reference_polynomial(oracle):
    for z in [0.3 + 0.2j, -0.7 + 0.1j, 1.1 - 0.4j]:
        for layer in (0, 1):
            np.testing.assert_allclose(ann.activation_function(z, layer), oracle.activation(z, layer)[0], rtol=1e-14)
        np.testing.assert_allclose(ann.activation_function(z, 0, "logcosh"), np.log(np.cosh(z)), rtol=1e-12)


@pytest.mark.parametrize("kind,N,M,C", [("rbm", 8, 8, None), ("deep", 8, 8, None), ("deep", 6, 12, 3),
                                        ("deep", 10, 20, 5)])
def test_exact_summation_fp64(oracle, kind, N, M, C):
    c = Case(kind, N, M, C, seed=3 * N + M)
    H = mixed_h(N)
    ref = oracle.exact(c.ref, H)
    op = ann.Operator(H)
    es = ann.ExactSummationSpins(N)
    ev = ann.ExpectationValue()
    np.testing.assert_allclose(ev(op, c.gpu, es), ref["E"][0], **FP64)
    sig, val = ev.fluctuation(op, c.gpu, es)
    np.testing.assert_allclose(sig, ref["fluct"][0], rtol=1e-9)
    np.testing.assert_allclose(val, ref["E"][0], **FP64)
    g, v = ev.gradient(op, c.gpu, es)
    np.testing.assert_allclose(g, ref["grad"], rtol=1e-9, atol=1e-11)
    td = ann.TDVP(c.gpu.num_params)
    td.eval(op, c.gpu, es)
    np.testing.assert_allclose(td.E_local, ref["tE"][0], **FP64)
    np.testing.assert_allclose(td.var_H, ref["tE2"][0] - abs(ref["tE"][0]) ** 2, rtol=1e-9)
    np.testing.assert_allclose(td.O_k_vector, ref["tO"], **FP64)
    np.testing.assert_allclose(td.F_vector, ref["tF"], rtol=1e-9, atol=1e-11)
    np.testing.assert_allclose(td.S_matrix, ref["tS"], rtol=1e-9, atol=1e-11)
    np.testing.assert_allclose(td.total_weight, ref["norm"][0] ** 2, rtol=1e-12)
    np.testing.assert_allclose(c.gpu.norm(es), ref["norm"][0], rtol=1e-12)
    np.testing.assert_allclose(ann.psi_vector(c.gpu, es), ref["vec"], **FP64)
    np.testing.assert_allclose(ann.log_psi(c.gpu, es), ref["mean_log_psi"][0], rtol=1e-10)
    np.testing.assert_allclose(ann.psi_O_k_vector(c.gpu, es), ref["O_sum"], rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(ann.apply_operator(c.gpu, op, es), ref["vec"] * ref["eloc"], rtol=1e-9, atol=1e-12)
    # S . v from the stored samples (TDVP.cu.template:336-443)
    v = np.random.default_rng(0).standard_normal(c.gpu.num_params) + 0j
    np.testing.assert_allclose(td.S_dot_vector(v, es), ref["tS"] @ v, rtol=1e-9, atol=1e-10)
    # list form evaluates every operator on the same configurations
    H2 = ann.transverse_field_ising_1d(N, h=0.3)
    ref2 = oracle.exact(c.ref, H2, want_S=False)
    lst = ev([op, ann.Operator(H2)], c.gpu, es)
    np.testing.assert_allclose(lst, [ref["E"][0], ref2["E"][0]], **FP64)
    # expectation value of a normalised state against the dense matrix
    c.gpu.normalize(es)
    vec = ann.psi_vector(c.gpu, es)
    np.testing.assert_allclose(ev(op, c.gpu, es), np.vdot(vec, H.matrix(N) @ vec), rtol=1e-10)


def test_exact_summation_c1_fp32(oracle):
    """1-D TFIM N=16, M=16 PsiDeep with [a | b | W] (Np = 288), complex64 kernels."""
    rng = np.random.default_rng(1234)
    N = M = 16
    a, b, W = cplx(rng, N, 0.01), cplx(rng, M, 0.01), cplx(rng, (N, M), 0.01)
    psi = ann.PsiRBM(W, 1.0, 0.0, True, a=a, b=b, precision="fp32")
    es = ann.ExactSummationSpins(N)
    psi.normalize(es)
    ref = oracle.exact(RbmDesc(N, M, W, a=a, b=b, layout=1, log_prefactor=psi.log_prefactor),
                       ann.transverse_field_ising_1d(N, 1.0))
    op = ann.Operator(ann.transverse_field_ising_1d(N, 1.0))
    td = ann.TDVP(psi.num_params, s_mode="fp32")
    td.eval(op, psi, es)
    E = ref["tE"][0]
    assert abs(td.E_local - E) < 1e-5 * abs(E)
    Fs = np.abs(ref["tF"]).max()
    assert np.abs(td.F_vector - ref["tF"]).max() < 1e-4 * Fs
    Ss = np.abs(ref["tS"]).max()
    assert np.abs(td.S_matrix - ref["tS"]).max() < 1e-4 * Ss


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("kind", ["rbm", "deep"])
def test_mc_replay_matches_reference_host_chain(oracle, precision, kind):
    """Fed the reference's own proposal sequence (its mt19937 host stream, restated
    bit-exactly by the oracle and pinned by tests/golden), the GPU chains visit the
    same configurations proposal by proposal."""
    N, M = 10, 20
    c = Case(kind, N, M, None, seed=11, precision=precision, a_in=False)
    H = mixed_h(N)
    n_chains, ns, sw, th = 6, 25, 2, 3
    tapes = [oracle.mc_reference(c.ref, H, ns, sw, th, seed=ch) for ch in range(n_chains)]
    init = []
    for t in tapes:
        init.append(int(t["pconf"][0]))
    sites = np.stack([t["psite"] for t in tapes])
    u = np.stack([t["pu"] for t in tapes])
    mc = ann.MonteCarloSpins(ns * n_chains, sw, th, n_chains, True)
    mc.set_tape(init, sites, u)
    e = ann.ExpectationValue()(ann.Operator(H), c.gpu, mc)
    conf, lp, el = mc.samples()
    got = conf[:, 0].reshape(ns, n_chains)
    want = np.stack([t["sconf"] for t in tapes], axis=1)
    if precision == "fp64":
        np.testing.assert_array_equal(got, want)
        np.testing.assert_allclose(lp.reshape(ns, n_chains), np.stack([t["slp"] for t in tapes], 1), rtol=1e-10)
        np.testing.assert_allclose(el.reshape(ns, n_chains), np.stack([t["seloc"] for t in tapes], 1),
                                   rtol=1e-9, atol=1e-11)
        np.testing.assert_allclose(e, np.mean([t["energy"][0] for t in tapes]), rtol=1e-9)
    else:
        # FP32 ratios may flip near-tie decisions; away from ties the chains coincide
        agree = (got == want).mean()
        assert agree > 0.9, agree


@pytest.mark.parametrize("move", ["single_flip", "exchange", "exchange_pairs"])
def test_mc_philox_stream_matches_oracle(oracle, move):
    N, M = 12, 24
    c = Case("deep", N, M, None, seed=21, precision="fp64")
    H = mixed_h(N)
    bonds = np.array([(i, (i + 1) % N) for i in range(N)], np.uint32)
    n_chains, spc, sw, th, seed = 64, 5, 1, 4, 0xDEADBEEF1234
    kind = {"single_flip": 0, "exchange": 1, "exchange_pairs": 2}[move]
    n_up = None if move == "single_flip" else N // 2
    mc = ann.MonteCarloSpins(spc * n_chains, sw, th, n_chains, True, move=move,
                             bonds=bonds if move == "exchange" else None, n_up=n_up, seed=seed, persistent=True)
    ann.ExpectationValue()(ann.Operator(H), c.gpu, mc)
    conf, lp, el = mc.samples()
    ref = oracle.mc_philox(c.ref, H, n_chains, seed, spc, sw, th, move_kind=kind, bonds=bonds,
                           n_up=-1 if n_up is None else n_up)
    assert ref["tie"][0] > 1e-12
    np.testing.assert_array_equal(conf[:, 0], ref["sconf"])
    np.testing.assert_allclose(lp, ref["slp"], rtol=1e-10)
    np.testing.assert_allclose(el, ref["seloc"], rtol=1e-9, atol=1e-11)
    if move != "single_flip":
        pop = np.array([bin(int(x)).count("1") for x in conf[:, 0]])
        assert (pop == N // 2).all()
    # persistent chains continue the stream on the next call
    ch_conf, ch_ctr = mc.get_chains()
    np.testing.assert_array_equal(ch_conf[:, 0], ref["conf"])
    np.testing.assert_array_equal(ch_ctr, ref["counter"])
    ann.ExpectationValue()(ann.Operator(H), c.gpu, mc)
    conf2, lp2, el2 = mc.samples()
    ref2 = oracle.mc_philox(c.ref, H, n_chains, seed, spc, sw, th, move_kind=kind, bonds=bonds, init=False,
                            conf=ref["conf"], counter=ref["counter"])
    np.testing.assert_array_equal(conf2[:, 0], ref2["sconf"])


def test_mc_energy_within_three_standard_errors(oracle):
    N, M = 16, 16
    rng = np.random.default_rng(1234)
    a, b, W = cplx(rng, N, 0.01), cplx(rng, M, 0.01), cplx(rng, (N, M), 0.01)
    H = ann.transverse_field_ising_1d(N, 1.0)
    ref = oracle.exact(RbmDesc(N, M, W, a=a, b=b, layout=1), H, want_S=False)
    e_exact = ref["E"][0] / ref["norm"][0] ** 2
    psi = ann.PsiRBM(W, 1.0, 0.0, True, a=a, b=b, precision="fp32")
    mc = ann.MonteCarloLoop(1024 * 100, 1, 10, 1024, True, seed=99)
    op = ann.Operator(H)
    e = ann.ExpectationValue()(op, psi, mc)
    conf, lp, el = mc.samples()
    # per-chain means -> standard error robust to autocorrelation
    chain_means = el.real.reshape(100, 1024).mean(axis=0)
    se = chain_means.std(ddof=1) / np.sqrt(1024)
    assert abs(e.real - e_exact.real) < 3 * se + 1e-6, (e, e_exact, se)
    assert 0.0 < mc.acceptance_rate < 1.0


def test_sr_solve_and_update(oracle):
    N, M = 8, 16
    c = Case("deep", N, M, None, seed=4, precision="fp64")
    H = ann.transverse_field_ising_1d(N, 1.0)
    es = normalize(c, N)
    ref = oracle.exact(c.ref, H)
    td = ann.TDVP(c.gpu.num_params)
    td.eval(ann.Operator(H), c.gpu, es)
    shift = 1e-3
    A = ref["tS"] + shift * np.eye(c.gpu.num_params)
    want = np.linalg.solve(A, ref["tF"])
    delta, info = td.solve(shift, return_info=True)
    np.testing.assert_allclose(delta, want, rtol=1e-8, atol=1e-10 * np.abs(want).max())
    assert info[1] <= max(info[0], 1e-14) and info[1] < 1e-12
    p0 = c.gpu.params
    td.update(c.gpu, 0.01)
    np.testing.assert_allclose(c.gpu.params, p0 - 0.01 * delta, rtol=1e-13, atol=1e-15)
    # the kernel weights follow the updated parameters
    c2 = RbmDesc(N, M, c.gpu.W[0], a=c.gpu.a, b=c.gpu.b[0], fw=c.gpu.final_weights, conn=c.gpu.connections[0],
                 log_prefactor=c.gpu.log_prefactor, layout=1)
    np.testing.assert_allclose(ann.log_psi_s(c.gpu, ann.Spins(37, N)), oracle.log_psi(c2, 37), **FP64)


def test_sr_not_positive_definite_is_reported(oracle):
    N, M = 6, 6
    c = Case("deep", N, M, None, seed=9, precision="fp64")
    es = normalize(c, N)
    td = ann.TDVP(c.gpu.num_params)
    td.eval(ann.Operator(ann.transverse_field_ising_1d(N)), c.gpu, es)
    with pytest.raises(ann.AnnError, match="positive definite"):
        td.solve(-10.0)
    # the context stays usable
    td.solve(1e-3)


def test_sr_step_graph_replay_equals_eager(oracle):
    import torch
    N, M = 10, 20
    H = ann.transverse_field_ising_1d(N, 1.0)
    op = ann.Operator(H)
    c1 = Case("deep", N, M, None, seed=8, precision="fp32")
    c2 = Case("deep", N, M, None, seed=8, precision="fp32")
    mc1 = ann.MonteCarloSpins(512 * 4, 2, 5, 512, True, seed=5, persistent=True)
    mc2 = ann.MonteCarloSpins(512 * 4, 2, 5, 512, True, seed=5, persistent=True)
    t1 = ann.TDVP(c1.gpu.num_params, s_mode="fp32")
    t2 = ann.TDVP(c2.gpu.num_params, s_mode="fp32")
    st = torch.cuda.Stream()
    t2.stream = st
    t2.capture_sr_step(op, c2.gpu, mc2, 1e-3, 0.01, st)  # runs one eager step first
    t1.stream = st
    t1.sr_step(op, c1.gpu, mc1, 1e-3, 0.01)
    for _ in range(3):
        t1.sr_step(op, c1.gpu, mc1, 1e-3, 0.01)
        t2.launch_sr_step(st)
    st.synchronize()
    np.testing.assert_array_equal(c1.gpu.params, c2.gpu.params)


@pytest.mark.parametrize("mode,tol", [("bf16", 1e-2), ("bf16_split", 2e-4)])
def test_tensor_core_S_matches_oracle(oracle, mode, tol):
    """S from the tcgen05 BF16 HERK (and its hi+lo split form) against the FP64
    oracle; Np = 374 spans three 128-parameter blocks (diagonal, off-diagonal and
    mirrored tiles, ragged last block), K = 2^14 samples."""
    N, M = 14, 24
    c = Case("deep", N, M, None, seed=31, precision="fp32")
    es = normalize(c, N)
    H = ann.transverse_field_ising_1d(N, 0.8)
    ref = oracle.exact(c.ref, H)
    td = ann.TDVP(c.gpu.num_params, s_mode=mode)
    td.eval(ann.Operator(H), c.gpu, es)
    S = td.S_matrix
    scale = np.abs(ref["tS"]).max()
    err = np.abs(S - ref["tS"]).max() / scale
    assert err < tol, err
    # the two triangles of diagonal tiles are separate FP32 sums
    assert np.abs(S - S.conj().T).max() < 1e-5 * scale
    # the plain FP32 form agrees with both
    td32 = ann.TDVP(c.gpu.num_params, s_mode="fp32")
    td32.eval(ann.Operator(H), c.gpu, es)
    assert np.abs(td32.S_matrix - ref["tS"]).max() / scale < 1e-4


def test_tensor_core_S_monte_carlo_rows(oracle):
    """Monte Carlo rows (W = 1, N_s not a multiple of 64): tensor-core S equals the
    FP32 SIMT S of the same samples within BF16 accuracy."""
    N, M = 16, 32
    c = Case("deep", N, M, None, seed=12, precision="fp32")
    H = ann.transverse_field_ising_1d(N, 1.0)
    mc = ann.MonteCarloSpins(1000, 1, 5, 100, True, seed=4)
    td = ann.TDVP(c.gpu.num_params, s_mode="bf16")
    td.eval(ann.Operator(H), c.gpu, mc)
    S_tc = td.S_matrix
    conf, _, _ = mc.samples()
    ref = oracle.tdvp_samples(c.ref, H, conf[:, 0], 1.0 / 1000)
    scale = np.abs(ref["S"]).max()
    assert np.abs(S_tc - ref["S"]).max() / scale < 1e-2
    np.testing.assert_allclose(td.F_vector, ref["F"], rtol=1e-4, atol=1e-5 * np.abs(ref["F"]).max())


def test_exp_sigma_z_matches_oracle(oracle):
    """ExpectationValue.exp_sigma_z (ExpectationValue.cu.template:52-81): sum over the
    exact-summation weights |psi(s)|^2 of exp(sum_n c_n <s|P_n|P_n s>), the per-string
    matrix elements from the oracle's Pauli algebra (pinned to the reference's KATs)."""
    N, M = 8, 16
    c = Case("deep", N, M, None, seed=77)
    H = ann.transverse_field_ising_1d(N, 0.7) + 0.3 * ann.sigma_y(1) * ann.sigma_y(2) + 0.2 * ann.sigma_z(3)
    es = ann.ExactSummationSpins(N)
    got = ann.ExpectationValue().exp_sigma_z(ann.Operator(H), c.gpu, es)
    w = np.abs(ann.psi_vector(c.gpu, es)) ** 2
    want = 0j
    for s in range(1 << N):
        a = sum(complex(coef) * oracle.pauli_apply(ka, kb, s, N)[0] for (ka, kb), coef in H)
        want += w[s] * np.exp(a)
    np.testing.assert_allclose(got, want, rtol=1e-10)


@pytest.mark.parametrize("mode,shift,S_tol,delta_tol", [("bf16", 1e-3, 2e-2, 0.2), ("bf16_split", 1e-4, 2e-4, 0.12)])
def test_tensor_core_S_many_waves_against_fp64(mode, shift, S_tol, delta_tol):
    """Tensor-core S at Np = 4224 (33 parameter blocks of 128: 561 tiles, several waves of
    the S kernel) from 8192 Monte Carlo samples, against a full FP64 evaluation of the same
    samples (complex128 O rows, FP64 HERK), and the SR update delta = (S + shift)^{-1} F
    against the FP64 Cholesky solve of the FP64 S.

    Bounds: relative Frobenius error of S (2e-2 BF16, 2e-4 hi+lo split). The update is
    checked by its backward error: delta solves (S64 + shift) delta = F64 up to exactly the
    perturbation (S - S64) delta - (F - F64) (the mixed solve adds nothing of its own), and
    its forward error is that perturbation amplified by cond(S64 + shift), about 1e3-1e4 for
    this random-init, nearly rank-deficient S: measured 0.083 (BF16, shift 1e-3) and 0.057
    (hi+lo, shift 1e-4), bounded here at 0.2 and 0.12."""
    N, M = 64, 64
    rng = np.random.default_rng(17)
    cc = lambda *s: 0.05 * (rng.standard_normal(s) + 1j * rng.standard_normal(s))  # noqa: E731
    a, b, W = cc(N), cc(M), cc(N, M)
    psi = ann.PsiRBM(W, 1.0, 0.0, True, a=a, b=b, precision="fp32")
    psi64 = ann.PsiRBM(W, 1.0, 0.0, True, a=a, b=b, precision="fp64")
    assert psi.num_params == 4224
    op = ann.Operator(ann.transverse_field_ising_1d(N, 1.0))
    n = 8192
    mc = ann.MonteCarloSpins(n, 4, 16, n, True, seed=5, persistent=True)
    td = ann.TDVP(psi.num_params, s_mode=mode, solver="mixed")
    td.eval(op, psi, mc)
    S, F = td.S_matrix, td.F_vector
    d = td.solve(shift)
    conf, _, _ = mc.samples()
    replay = ann.MonteCarloSpins(n, 0, 0, n, True, persistent=True)
    replay.set_tape(conf[:, 0], np.zeros((n, 1), np.uint32), np.zeros((n, 1)))
    t64 = ann.TDVP(psi.num_params, s_mode="fp32", solver="fp64")
    t64.eval(op, psi64, replay)
    S64, F64 = t64.S_matrix, t64.F_vector
    d64 = t64.solve(shift)
    rel = lambda x, y: np.linalg.norm(x - y) / np.linalg.norm(y)  # noqa: E731
    assert rel(F, F64) < 1e-5, rel(F, F64)
    assert rel(S, S64) < S_tol, rel(S, S64)
    nF = np.linalg.norm(F64)
    backward = np.linalg.norm(S64 @ d + shift * d - F64) / nF
    explained = np.linalg.norm((S - S64) @ d - (F - F64)) / nF
    assert abs(backward - explained) <= 1e-9 + 1e-6 * explained, (backward, explained)
    assert rel(d, d64) < delta_tol, rel(d, d64)
