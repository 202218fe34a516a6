"""PsiCNN on the GPU against the reference's own host outputs (tests/golden/cnn_4x4.npz)
and the FP64 oracle: log psi, O_k, exact-summation energy and TDVP quantities,
Monte Carlo with exchange moves."""

import os

import numpy as np
import pytest

from pyoracle import CnnDesc

pytestmark = pytest.mark.gpu

ann = pytest.importorskip("annongpu_gb300")

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def golden():
    return dict(np.load(os.path.join(GOLD, "cnn_4x4.npz")))


def random_cnn(rng, extent, layers, ncls=1, scale=0.15, ff=0.7, activation="poly", precision="fp64"):
    N = int(np.prod(extent))
    classes = (np.arange(N) % ncls).astype(np.uint32)
    channels = [c for c, _ in layers]
    conns = [k for _, k in layers]
    np_ = sum(c * (channels[l - 1] if l else 1) * ncls * int(np.prod(k)) for l, (c, k) in enumerate(layers))
    params = scale * (rng.standard_normal(np_) + 1j * rng.standard_normal(np_))
    gpu = ann.PsiCNN(extent, channels, conns, classes, params, ff, 0.05 - 0.02j, True, activation=activation,
                     precision=precision)
    ref = CnnDesc(extent, channels, conns, classes, params, ff, log_prefactor=0.05 - 0.02j,
                  activation={"poly": 0, "logcosh": 1}[activation])
    return gpu, ref


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 3e-5)])
def test_cnn_matches_reference_fixture(precision, tol):
    g = golden()
    psi = ann.PsiCNN(g["extent"], g["channels"], g["connectivity"], g["classes"], g["params"], g["ff"][0],
                     g["lp"][0], True, precision=precision)
    for k, s in enumerate(g["confs"]):
        np.testing.assert_allclose(ann.log_psi_s(psi, ann.Spins(int(s), 16)), g["log_psi"][k], rtol=tol, atol=tol)
        np.testing.assert_allclose(ann.psi_O_k(psi, ann.Spins(int(s), 16)), g["O_k"][k], rtol=tol * 10,
                                   atol=tol * 10)
    H = ann.PauliExpression({(int(a), int(b)): c for a, b, c in zip(g["op_a"], g["op_b"], g["op_c"])})
    es = ann.ExactSummationSpins(16)
    np.testing.assert_allclose(ann.ExpectationValue()(ann.Operator(H), psi, es), g["ex_E"][0], rtol=tol * 10)
    np.testing.assert_allclose(psi.norm(es), g["ex_norm"][0], rtol=tol * 10)


@pytest.mark.parametrize("layers,ncls,activation", [
    ([(3, [1, 2, 3])], 1, "poly"),
    ([(2, [1, 3, 3]), (3, [1, 2, 2])], 2, "poly"),
    ([(4, [1, 3, 3]), (2, [1, 3, 3])], 1, "logcosh"),
])
def test_cnn_exact_tdvp_fp64(oracle, layers, ncls, activation):
    rng = np.random.default_rng(len(layers) * 7 + ncls)
    extent = [1, 3, 4]
    gpu, ref = random_cnn(rng, extent, layers, ncls=ncls, activation=activation)
    N = 12
    H = ann.transverse_field_ising_1d(N, 0.7) + 0.3 * ann.sigma_y(2) * ann.sigma_y(5) + 0.2 * ann.sigma_x(1)
    es = ann.ExactSummationSpins(N)
    gpu.normalize(es)
    ref = CnnDesc(extent, ref.channels, ref.connectivity.reshape(-1, 3), ref.sym, ref.params, gpu.final_factor,
                  log_prefactor=gpu.log_prefactor, activation=ref.struct.activation)
    r = oracle.cnn_exact(ref, H, want_S=True)
    td = ann.TDVP(gpu.num_params)
    td.eval(ann.Operator(H), gpu, es)
    np.testing.assert_allclose(td.E_local, r["tE"][0], rtol=1e-10)
    np.testing.assert_allclose(td.O_k_vector, r["tO"], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(td.F_vector, r["tF"], rtol=1e-9, atol=1e-11)
    np.testing.assert_allclose(td.S_matrix, r["tS"], rtol=1e-9, atol=1e-11)
    for s in [0, 5, 1234, 4095]:
        np.testing.assert_allclose(ann.psi_O_k(gpu, ann.Spins(s, N)), oracle.cnn_O_k(ref, s), rtol=1e-9,
                                   atol=1e-12)


def test_cnn_monte_carlo_exchange_sz_sector(oracle):
    """Exchange moves over the bonds of the Heisenberg model keep Sz = 0; the MC
    energy agrees with exact summation restricted to the sector within 3 standard errors."""
    rng = np.random.default_rng(3)
    extent = [1, 3, 4]
    N = 12
    gpu, ref = random_cnn(rng, extent, [(3, [1, 3, 3]), (2, [1, 2, 2])], precision="fp32", scale=0.2)
    nn, _ = ann.square_lattice_bonds(4, 3)
    H = ann.PauliExpression()
    for i, j in nn:
        H = H + ann.sigma_x(i) * ann.sigma_x(j) + ann.sigma_y(i) * ann.sigma_y(j) + ann.sigma_z(i) * ann.sigma_z(j)
    op = ann.Operator(H)
    mc = ann.MonteCarloSpins(512 * 40, 2, 20, 512, True, move="exchange", bonds=nn, n_up=N // 2, seed=11)
    e = ann.ExpectationValue()(op, gpu, mc)
    conf, lp, el = mc.samples()
    pop = np.array([bin(int(x)).count("1") for x in conf[:, 0]])
    assert (pop == N // 2).all()
    # exact energy within the Sz = 0 sector
    vec = ann.psi_vector(gpu, ann.ExactSummationSpins(N))
    mask = np.array([bin(k).count("1") == N // 2 for k in range(1 << N)])
    v = np.where(mask, vec, 0)
    e_exact = np.vdot(v, H.matrix(N) @ v) / np.vdot(v, v)
    se = el.real.reshape(40, 512).mean(axis=0).std(ddof=1) / np.sqrt(512)
    assert abs(e.real - e_exact.real) < 3 * se + 1e-6, (e, e_exact, se)


# ---- the 10 x 10 J1-J2 shape: two 3 x 3 layers of 16 and 8 channels, 100 sites (two words) ----
def c3_case(precision, scale=0.05, seed=31):
    rng = np.random.default_rng(seed)
    extent = [1, 10, 10]
    return random_cnn(rng, extent, [(16, [1, 3, 3]), (8, [1, 3, 3])], ncls=1, scale=scale, ff=0.5,
                      precision=precision)


def sz0_configs(rng, n, N=100):
    out = []
    for _ in range(n):
        up = rng.choice(N, N // 2, replace=False)
        out.append(sum(1 << int(i) for i in up))
    return out


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 2e-4)])
def test_cnn_10x10_16_8_channels_matches_oracle(oracle, precision, tol):
    """log psi, O_k and the J1-J2 local energy of explicit Sz = 0 configurations on the
    10 x 10 lattice (N = 100, two spin words; Np = 16*9 + 16*8*9 = 1296) against the FP64
    oracle's restatement of PsiCNN.hpp:97-266 (the reference caps N at 64 and channels at 6,
    so this shape has no reference output). The local energy's psi ratios come from the
    changed pre-activations of each flip pair (the 3 x 3 / 5 x 5 cones)."""
    gpu, ref = c3_case(precision)
    assert gpu.num_params == 1296
    H = ann.heisenberg_j1j2_2d(10, 10, 1.0, 0.5)
    op = ann.Operator(H)
    confs = sz0_configs(np.random.default_rng(5), 4)
    el = ann.local_energies(gpu, op, confs)
    for k, s in enumerate(confs):
        lp_ref = oracle.cnn_log_psi(ref, s)
        np.testing.assert_allclose(ann.log_psi_s(gpu, ann.Spins(s, 100)), lp_ref, rtol=tol, atol=tol)
        O_ref = oracle.cnn_O_k(ref, s)
        O = ann.psi_O_k(gpu, ann.Spins(s, 100))
        assert np.abs(O - O_ref).max() <= 10 * tol * np.abs(O_ref).max()
        e_ref = oracle.cnn_local_energy(ref, H, s)
        assert abs(el[k] - e_ref) <= 10 * tol * max(1.0, abs(e_ref)), (k, el[k], e_ref)


def test_cnn_10x10_exchange_chains_match_oracle(oracle):
    """Philox chains with exchange moves over the J1-J2 bonds from random Sz = 0 starts
    (50 up spins) on the 10 x 10 two-layer CNN: the FP64 kernels take every decision from
    the incremental psi ratio, the oracle from full forward passes; sampled configurations
    are identical and stay in the Sz = 0 sector, log psi agrees to 1e-10, and persistent
    chains continue the stream."""
    gpu, ref = c3_case("fp64", scale=0.3)
    nn, nnn = ann.square_lattice_bonds(10, 10, diagonal=True)
    bonds = np.array(nn + nnn, np.uint32)
    n_chains, spc, sw, th, seed = 6, 2, 1, 1, 0xC3C3
    mc = ann.MonteCarloSpins(spc * n_chains, sw, th, n_chains, True, move="exchange", bonds=bonds, n_up=50,
                             seed=seed, persistent=True)
    ann.log_psi(gpu, mc)
    conf, lp, _ = mc.samples()
    r = oracle.cnn_mc_philox(ref, None, n_chains, seed, spc, sw, th, move_kind=1, bonds=bonds, n_up=50)
    assert r["tie"][0] > 1e-11
    assert r["acc"][0] > 20  # moves were accepted along the way
    np.testing.assert_array_equal(conf.reshape(-1), r["sconf"])
    np.testing.assert_allclose(lp, r["slp"], rtol=1e-10)
    pop = np.array([bin(int(a)).count("1") + bin(int(b)).count("1") for a, b in conf])
    assert (pop == 50).all()
    ch_conf, ch_ctr = mc.get_chains()
    np.testing.assert_array_equal(ch_conf.reshape(-1), r["conf"])
    np.testing.assert_array_equal(ch_ctr, r["counter"])
    ann.log_psi(gpu, mc)
    conf2, _, _ = mc.samples()
    r2 = oracle.cnn_mc_philox(ref, None, n_chains, seed, spc, sw, th, move_kind=1, bonds=bonds, init=False,
                              conf=r["conf"], counter=r["counter"])
    np.testing.assert_array_equal(conf2.reshape(-1), r2["sconf"])


@pytest.mark.parametrize("layers,ncls,scale", [
    ([(3, [1, 2, 3])], 1, 0.2),
    ([(2, [1, 3, 3]), (3, [1, 2, 2])], 2, 0.15),
])
def test_cnn_single_flip_and_pair_chains_match_oracle(oracle, layers, ncls, scale):
    """Single flips and random-pair exchanges on small lattices with one or two layers and
    two symmetry classes: FP64 chains identical to the oracle's, local energies included
    (weight scales keep Re log psi within a few units: the polynomial activations grow
    like z^6)."""
    rng = np.random.default_rng(9 + ncls)
    extent = [1, 3, 4]
    gpu, ref = random_cnn(rng, extent, layers, ncls=ncls, scale=scale)
    N = 12
    H = ann.transverse_field_ising_1d(N, 0.7) + 0.3 * ann.sigma_y(2) * ann.sigma_y(5) + 0.2 * ann.sigma_x(1) + \
        0.1 * ann.sigma_x(0) * ann.sigma_x(4) * ann.sigma_x(8)
    for move, kind, n_up in (("single_flip", 0, None), ("exchange_pairs", 2, N // 2)):
        n_chains, spc, sw, th, seed = 32, 3, 1, 2, 0x77 + kind
        mc = ann.MonteCarloSpins(spc * n_chains, sw, th, n_chains, True, move=move, n_up=n_up, seed=seed)
        ann.ExpectationValue()(ann.Operator(H), gpu, mc)
        conf, lp, el = mc.samples()
        r = oracle.cnn_mc_philox(ref, H, n_chains, seed, spc, sw, th, move_kind=kind,
                                 n_up=-1 if n_up is None else n_up)
        assert r["tie"][0] > 1e-11
        np.testing.assert_array_equal(conf[:, 0], r["sconf"])
        np.testing.assert_allclose(lp, r["slp"], rtol=1e-10)
        np.testing.assert_allclose(el, r["seloc"], rtol=1e-9, atol=1e-11)
