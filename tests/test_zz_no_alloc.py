"""ann_force_vector_noalloc (E, <O>, F from caller-owned device arrays with a fixed
static scratch, no allocation) called through the C ABI, against ann_tdvp_eval_F on
the same samples, on two calls in a row: the second call has fewer rows and fewer
parameters than the first, so stale scratch from the first call would show.

Tolerance: the energy is an FP64 sum in both paths (rtol 1e-10). For <O> and F the
no-allocation path accumulates the complex64 rows in FP64, while ann_tdvp_eval_F
accumulates them in FP32 within slabs of at most 512 rows (FP64 across slabs), so they
agree to rtol 2e-5 of the largest entry, the bound used for FP32-accumulated sums.
"""

import ctypes as ct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ann = pytest.importorskip("annongpu_gb300")
torch = pytest.importorskip("torch")


def eval_case(L, alpha, seed, chains, rows_per_chain):
    rng = np.random.default_rng(seed)
    M = alpha * L
    W = 0.05 * (rng.standard_normal((L, M)) + 1j * rng.standard_normal((L, M)))
    a = 0.02 * (rng.standard_normal(L) + 1j * rng.standard_normal(L))
    b = 0.02 * (rng.standard_normal(M) + 1j * rng.standard_normal(M))
    psi = ann.PsiRBM(W, 1.0, 0.0, True, a=a, b=b, precision="fp32")
    op = ann.Operator(ann.transverse_field_ising_1d(L, 0.8))
    mc = ann.MonteCarloSpins(chains * rows_per_chain, 2, 10, chains, True, seed=seed)
    td = ann.TDVP(psi.num_params)
    td.eval_F(op, psi, mc)
    n = chains * rows_per_chain
    O = td.O_k_samples.reshape(n, psi.num_params)
    _, _, el = mc.samples()
    return psi.num_params, O, el, td


def call_noalloc(Np, O, el, ld, weights):
    """Device copies of the inputs, then one call through the C ABI on torch's stream."""
    n = O.shape[0]
    rows = np.full((n, ld), np.nan + 1j * np.nan, np.complex64)  # padding must not be read
    rows[:, :Np] = O.astype(np.complex64)
    assert np.array_equal(rows[:, :Np].astype(np.complex128), O)  # float O rows: exact copy
    dev = torch.device("cuda:0")
    d_rows = torch.from_numpy(rows).to(dev)
    d_el = torch.from_numpy(np.ascontiguousarray(el, np.complex128)).to(dev)
    d_w = None if weights is None else torch.from_numpy(weights).to(dev)
    d_Om = torch.full((Np,), 7.0, dtype=torch.complex128, device=dev)
    d_F = torch.full((Np,), 7.0, dtype=torch.complex128, device=dev)
    d_E = torch.full((1,), 7.0, dtype=torch.complex128, device=dev)
    torch.cuda.synchronize()
    st = torch.cuda.current_stream().cuda_stream
    ann._lib.call("ann_force_vector_noalloc", ct.c_void_p(d_rows.data_ptr()), n, ld, Np,
                  None if d_w is None else ct.c_void_p(d_w.data_ptr()), 1.0 / n, ct.c_void_p(d_el.data_ptr()),
                  ct.c_void_p(d_Om.data_ptr()), ct.c_void_p(d_F.data_ptr()), ct.c_void_p(d_E.data_ptr()),
                  ct.c_void_p(st))
    torch.cuda.synchronize()
    return d_Om.cpu().numpy(), d_F.cpu().numpy(), complex(d_E.cpu().numpy()[0])


def close(got, want, rtol):
    scale = np.abs(want).max()
    assert np.abs(got - want).max() <= rtol * scale + 1e-300, (np.abs(got - want).max(), scale)


def test_noalloc_force_vector_matches_eval_F_two_calls():
    # call 1: 16 sites alpha 4 (Np 16+64+1024 = 1104), uniform weights, padded rows
    Np1, O1, el1, td1 = eval_case(16, 4, 11, 512, 8)
    Om1, F1, E1 = call_noalloc(Np1, O1, el1, ld=Np1 + 3, weights=None)
    # call 2: 10 sites alpha 2 (Np 230), fewer rows, explicit weight array
    Np2, O2, el2, td2 = eval_case(10, 2, 12, 256, 4)
    n2 = O2.shape[0]
    Om2, F2, E2 = call_noalloc(Np2, O2, el2, ld=Np2, weights=np.full(n2, 1.0 / n2))
    for Om, F, E, td in ((Om1, F1, E1, td1), (Om2, F2, E2, td2)):
        close(Om, td.O_k_vector, 2e-5)
        close(F, td.F_vector, 2e-5)
        close(np.array([E]), np.array([td.E_local]), 1e-10)


def test_noalloc_rejects_num_params_beyond_scratch():
    d = torch.zeros(8, dtype=torch.complex128, device="cuda:0")
    p = ct.c_void_p(d.data_ptr())
    big = 130817
    with pytest.raises(ann._lib.AnnError, match="exceeds the fixed scratch limit of 130816"):
        ann._lib.call("ann_force_vector_noalloc", p, 1, big, big, None, 1.0, p, p, p, p, None)
