"""Times the reference's own CPU path (oracle/_ref/libref.so, built from the reference
sources by `make -C oracle ref REF=<reference checkout>`) against the FP64 oracle's
restatement of it on the same sample, one core each: the host Monte Carlo of one chain
(MonteCarlo.hpp:55-177) followed by TDVP::eval over its samples (E, F, dense S;
TDVP.cu.template:181-302). Shapes of the 2-D TFIM 8x8 workload with the reference's
PsiRBM (W only, N = 64, M = 128, Np = 8192; its PsiDeep stops at M = 64). TEST
INFRASTRUCTURE: measurement of the checker, never part of the product.

    python oracle/compare_ref_port_speed.py [samples]
"""

import ctypes as ct
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(HERE))

from pyoracle import OpArrays, Oracle, RbmDesc, RefHarness  # noqa: E402
from annongpu_gb300.expression import transverse_field_ising_2d  # noqa: E402


def main(samples=4, sweeps=64):
    N, M = 64, 128
    rng = np.random.default_rng(1234)
    W = 0.01 * (rng.standard_normal((N, M)) + 1j * rng.standard_normal((N, M)))
    fw, lp = np.ones(1, np.complex128), np.zeros(1, np.complex128)
    H = transverse_field_ising_2d(8, 8, h=3.04)
    ref = RefHarness()
    op = OpArrays(H, N)
    a, b, c = (np.ascontiguousarray(x) for x in H.arrays(1))
    a, b = a[:, 0].copy(), b[:, 0].copy()
    c = np.ascontiguousarray(c.astype(np.complex128))
    P = ct.c_void_p
    ref.lib.ref_rbm_tdvp_mc.argtypes = [ct.c_uint, ct.c_uint, P, P, P, P, P, P, ct.c_uint, ct.c_uint, ct.c_uint,
                                        ct.c_uint, P]
    ptr = lambda x: x.ctypes.data_as(P)  # noqa: E731
    tE = np.zeros(1, np.complex128)
    t0 = time.perf_counter()
    ref.lib.ref_rbm_tdvp_mc(N, M, ptr(W), ptr(fw), ptr(lp), ptr(a), ptr(b), ptr(c), len(c), samples, sweeps, 1,
                            ptr(tE))
    t_ref = time.perf_counter() - t0
    o = Oracle()
    psi = RbmDesc(N, M, W, fw=np.ones(M), layout=0, a_in_log_psi=False)
    t0 = time.perf_counter()
    r = o.mc_reference(psi, H, samples, sweeps, 1)
    o.tdvp_samples(psi, H, r["sconf"], 1.0 / samples, want_S=True)
    t_port = time.perf_counter() - t0
    del op
    print(f"samples={samples} sweeps={sweeps}: reference {t_ref / samples:.4f} s/sample, "
          f"port {t_port / samples:.4f} s/sample, port/reference time ratio {t_port / t_ref:.3f}")


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 4)
