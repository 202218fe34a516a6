// HilbertSpaceDistance: distance between psi' and the state U psi (U given as a Pauli
// sum), and its gradient with respect to the parameters of psi', sampled from psi.
//
// Per sample s of the ensemble of psi (source/network_functions/
// HilbertSpaceDistance.cu.template:16-86):
//   E(s)  = local energy of U with respect to psi,
//   omega = exp(conj(log psi'(s) - log psi(s))) E(s)      (unitary U)
//         = exp(E(s) + conj(log psi'(s) - log psi(s)))   (otherwise),
//   next  = |E(s)|^2  (unitary)  or  exp(2 Re E(s)),
//   ratio = exp(2 (Re log psi'(s) - Re log psi(s))),
// averaged with the ensemble weights; the gradient adds sum w omega conj(O'_k) and
// sum w ratio conj(O'_k) with O' the log-derivatives of psi'. Then (:118-168)
//   u = |<omega>|^2, v = <next> <ratio>, distance = sqrt(max(1 - u / v, 1e-8)),
//   grad_k = -(conj(<omega>) <omega O'_k> v - u <next> <ratio O'_k>) / v^2 / distance^nu.
// The rows of psi come from the ensemble kernels (log psi and E(s) in one pass), log psi'
// and O' from the explicit-configuration kernels on the same configurations; the sums
// are deterministic two-pass reductions (FP64 per row, the O' columns as in col_stats).
#include <cmath>

#include "ann_internal.hpp"

namespace ann {

namespace {

constexpr int kHsdThreads = 256;
constexpr int kHsdBlocks = 256;

__device__ __forceinline__ double hsd_block_sum(double v, double* sh) {
    v = warp_sum(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if(l == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if(w == 0) {
        r = (l < (int)(blockDim.x >> 5)) ? sh[l] : 0.0;
        r = warp_sum(r);
    }
    return r;
}

// omega_r, ratio_r per row; per-block sums of w omega (re, im), w ratio, w next
__global__ void __launch_bounds__(kHsdThreads)
hsd_rows_kernel(size_t n, const double* __restrict__ wts, double w0, const cplx<double>* __restrict__ lp,
                const cplx<double>* __restrict__ lpp, const cplx<double>* __restrict__ e, int unitary,
                cplx<double>* __restrict__ omega, cplx<double>* __restrict__ ratio, double* __restrict__ partial) {
    __shared__ double sh[32];
    const size_t per = (n + gridDim.x - 1) / gridDim.x;
    const size_t r0 = (size_t)blockIdx.x * per, r1 = min(n, r0 + per);
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for(size_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        const double w = wts ? wts[r] : w0;
        const cplx<double> d = conj(lpp[r] - lp[r]);
        const cplx<double> E = e[r];
        const cplx<double> om = unitary ? cexp(d) * E : cexp(E + d);
        const double nx = unitary ? norm2(E) : exp(2.0 * E.re);
        const double pr = exp(2.0 * (lpp[r].re - lp[r].re));
        omega[r] = om;
        ratio[r] = mk(pr, 0.0);
        acc[0] += w * om.re;
        acc[1] += w * om.im;
        acc[2] += w * pr;
        acc[3] += w * nx;
    }
    for(int k = 0; k < 4; k++) {
        const double s = hsd_block_sum(acc[k], sh);
        if(threadIdx.x == 0) partial[(size_t)blockIdx.x * 4 + k] = s;
    }
}

__global__ void hsd_final_kernel(const double* __restrict__ partial, int nb, double* __restrict__ out4) {
    if(threadIdx.x == 0) {
        double acc[4] = {0.0, 0.0, 0.0, 0.0};
        for(int b = 0; b < nb; b++)
            for(int k = 0; k < 4; k++) acc[k] += partial[(size_t)b * 4 + k];
        for(int k = 0; k < 4; k++) out4[k] = acc[k];
    }
}

struct HsdScratch {
    DevBuf O, omega, ratio, partial, sums, omega_O, ratio_O, cpart;
    Rows rows2;
};
HsdScratch& hsd_scratch() {
    static thread_local HsdScratch s;
    return s;
}

struct HsdSums {
    zd omega;
    double ratio, next;
};

// the sums of one pass; with `grad` also <omega O'_k> and <ratio O'_k> (device)
HsdSums hsd_pass(ann_psi_impl& psi, ann_psi_impl& psi_p, const ann_op_impl& op, bool unitary, ann_ens_impl& ens,
                 bool grad, cudaStream_t st) {
    if(psi.N != psi_p.N) throw Error(ANN_ERR_INVALID, "psi and psi_prime act on different numbers of sites");
    auto& sc = hsd_scratch();
    run_ensemble(psi, &op, ens, SampleTargets{&ens.rows}, st);
    const size_t n = ens.rows.n;
    const size_t ld = ((size_t)psi_p.Np + 3) & ~(size_t)3;
    void* O = nullptr;
    if(grad) {
        sc.O.ensure(n * ld * psi_p.elem_bytes());
        O = sc.O.p;
    }
    run_confs(psi_p, nullptr, ens.rows.conf.as<uint64_t>(), n, sc.rows2, O, ld, st);
    sc.omega.ensure(n * sizeof(cplx<double>));
    sc.ratio.ensure(n * sizeof(cplx<double>));
    sc.partial.ensure((size_t)kHsdBlocks * 4 * sizeof(double));
    sc.sums.ensure(4 * sizeof(double));
    const double* w = ens.kind == 0 ? ens.rows.weight.as<double>() : nullptr;
    const double w0 = ens.kind == 0 ? 0.0 : ens.uniform_weight();
    hsd_rows_kernel<<<kHsdBlocks, kHsdThreads, 0, st>>>(n, w, w0, ens.rows.log_psi.as<cplx<double>>(),
                                                        sc.rows2.log_psi.as<cplx<double>>(),
                                                        ens.rows.eloc.as<cplx<double>>(), unitary ? 1 : 0,
                                                        sc.omega.as<cplx<double>>(), sc.ratio.as<cplx<double>>(),
                                                        sc.partial.as<double>());
    check_launch("hsd_rows_kernel");
    hsd_final_kernel<<<1, 32, 0, st>>>(sc.partial.as<double>(), kHsdBlocks, sc.sums.as<double>());
    check_launch("hsd_final_kernel");
    if(grad) {
        sc.omega_O.ensure((size_t)psi_p.Np * sizeof(cplx<double>));
        sc.ratio_O.ensure((size_t)psi_p.Np * sizeof(cplx<double>));
        // sum_s w_s c_s conj(O'_sk) for c = omega, ratio
        col_stats(O, psi_p.precision, n, ld, psi_p.Np, w, w0, sc.omega.as<cplx<double>>(), nullptr,
                  sc.omega_O.as<cplx<double>>(), nullptr, nullptr, sc.cpart, st);
        col_stats(O, psi_p.precision, n, ld, psi_p.Np, w, w0, sc.ratio.as<cplx<double>>(), nullptr,
                  sc.ratio_O.as<cplx<double>>(), nullptr, nullptr, sc.cpart, st);
    }
    double h[4];
    ANN_CUDA(cudaMemcpyAsync(h, sc.sums.p, sizeof(h), cudaMemcpyDeviceToHost, st));
    ANN_CUDA(cudaStreamSynchronize(st));
    return HsdSums{zd(h[0], h[1]), h[2], h[3]};
}

double hsd_distance_of(const HsdSums& s) {
    const double u = std::norm(s.omega);
    const double v = s.next * s.ratio;
    return std::sqrt(std::max(1.0 - u / v, 1e-8));
}

template<typename F>
int hguard(F&& f) {
    try {
        f();
        return ANN_OK;
    } catch(const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch(const std::exception& e) {
        set_last_error(e.what());
        return ANN_ERR_CUDA;
    }
}

void hsd_check_status() {
    unsigned v = 0;
    unsigned* p = status_word();
    ANN_CUDA(cudaMemcpy(&v, p, sizeof(unsigned), cudaMemcpyDeviceToHost));
    if(v) {
        ANN_CUDA(cudaMemset(p, 0, sizeof(unsigned)));
        throw Error(ANN_ERR_NUMERIC, "device status: non-finite value in log psi / local energy");
    }
}

}  // namespace

}  // namespace ann

using namespace ann;

extern "C" {

int ann_hsd_distance(ann_psi* psi, ann_psi* psi_prime, ann_op* op, int is_unitary, ann_ens* ens, void* stream,
                     double* distance) {
    return hguard([&] {
        if(!psi || !psi_prime || !op || !ens || !distance) throw Error(ANN_ERR_INVALID, "null argument");
        const HsdSums s = hsd_pass(*psi, *psi_prime, *op, is_unitary != 0, *ens, false,
                                   reinterpret_cast<cudaStream_t>(stream));
        hsd_check_status();
        *distance = hsd_distance_of(s);
    });
}

int ann_hsd_gradient(ann_psi* psi, ann_psi* psi_prime, ann_op* op, int is_unitary, ann_ens* ens, double nu,
                     void* stream, double* grad, double* distance) {
    return hguard([&] {
        if(!psi || !psi_prime || !op || !ens || !grad) throw Error(ANN_ERR_INVALID, "null argument");
        cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
        const HsdSums s = hsd_pass(*psi, *psi_prime, *op, is_unitary != 0, *ens, true, st);
        hsd_check_status();
        const unsigned np = psi_prime->Np;
        std::vector<zd> oo(np), ro(np);
        auto& sc = hsd_scratch();
        ANN_CUDA(cudaMemcpy(oo.data(), sc.omega_O.p, np * sizeof(zd), cudaMemcpyDeviceToHost));
        ANN_CUDA(cudaMemcpy(ro.data(), sc.ratio_O.p, np * sizeof(zd), cudaMemcpyDeviceToHost));
        const double u = std::norm(s.omega);
        const double v = s.next * s.ratio;
        const double d = hsd_distance_of(s);
        const double pref = std::pow(d, nu);
        for(unsigned k = 0; k < np; k++) {
            const zd uk = std::conj(s.omega) * oo[k];
            const zd vk = s.next * ro[k];
            const zd g = -(uk * v - u * vk) / (v * v) / pref;
            grad[2 * k] = g.real();
            grad[2 * k + 1] = g.imag();
        }
        if(distance) *distance = d;
    });
}

}  // extern "C"
