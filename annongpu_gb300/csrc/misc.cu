// Small device paths of the reference's network functions:
//   ExpectationValue::exp_sigma_z (source/network_functions/ExpectationValue.cu.template:52-81,
//     StandartOperator::fast_local_energy_parallel include/operator/Operator.hpp:137-155)
//   activation_function (pyANNonGPU/main.cpp.template:534-536)
#include "ann_internal.hpp"

namespace ann {

namespace {

// per row: v(s) = sum_n c_n <s|P_n|.> (matrix elements only, no psi ratio);
// partial[b] = sum over block b's rows of w exp(v)
__global__ void __launch_bounds__(256)
exp_sigma_z_kernel(OpDev op, size_t n, const uint64_t* __restrict__ conf, const double* __restrict__ wts, double w0,
                   cplx<double>* __restrict__ partial) {
    __shared__ double sh[2][8];
    double re = 0.0, im = 0.0;
    const size_t per = (n + gridDim.x - 1) / gridDim.x;
    const size_t r0 = (size_t)blockIdx.x * per, r1 = min(n, r0 + per);
    for(size_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        const uint64_t* s = conf + r * kMaxWords;
        cplx<double> v = mk(0.0, 0.0);
        for(unsigned d = 0; d < op.n_diag; d++) {
            int neg = 0;
            for(unsigned w = 0; w < op.nw; w++) neg += __popcll((~s[w]) & op.diag_mask[d * op.nw + w]);
            const double sg = (neg & 1) ? -1.0 : 1.0;
            v.re += sg * op.diag_coeff[2 * d];
            v.im += sg * op.diag_coeff[2 * d + 1];
        }
        const unsigned nstr = op.grp_str_begin[op.n_groups];
        for(unsigned k = 0; k < nstr; k++) {
            int neg = 0;
            for(unsigned w = 0; w < op.nw; w++) neg += __popcll((~s[w]) & op.str_mask[k * op.nw + w]);
            const double sg = (neg & 1) ? -1.0 : 1.0;
            v.re += sg * op.str_coeff[2 * k];
            v.im += sg * op.str_coeff[2 * k + 1];
        }
        const double w = wts ? wts[r] : w0;
        const cplx<double> e = cexp(v);
        re += w * e.re;
        im += w * e.im;
    }
    re = warp_sum(re);
    im = warp_sum(im);
    if((threadIdx.x & 31) == 0) {
        sh[0][threadIdx.x >> 5] = re;
        sh[1][threadIdx.x >> 5] = im;
    }
    __syncthreads();
    if(threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for(int k = 0; k < 8; k++) {
            a += sh[0][k];
            b += sh[1][k];
        }
        partial[blockIdx.x] = mk(a, b);
    }
}

__global__ void activation_kernel(double re, double im, unsigned layer, int act, double* out) {
    const cplx<double> f = act == kPoly ? poly_f(mk(re, im), (int)layer) : logcosh(mk(re, im));
    out[0] = f.re;
    out[1] = f.im;
}

}  // namespace

void exp_sigma_z_sum(const ann_op_impl& op, const Rows& rows, const double* wts, double w0, double* out2,
                     cudaStream_t st) {
    constexpr unsigned blocks = 128;
    DevBuf part;
    part.ensure(blocks * sizeof(cplx<double>));
    exp_sigma_z_kernel<<<blocks, 256, 0, st>>>(op.view(), rows.n, rows.conf.as<uint64_t>(), wts, w0,
                                               part.as<cplx<double>>());
    check_launch("exp_sigma_z_kernel");
    std::vector<cplx<double>> h(blocks);
    ANN_CUDA(cudaMemcpyAsync(h.data(), part.p, blocks * sizeof(cplx<double>), cudaMemcpyDeviceToHost, st));
    ANN_CUDA(cudaStreamSynchronize(st));
    double a = 0.0, b = 0.0;
    for(auto& z : h) {
        a += z.re;
        b += z.im;
    }
    out2[0] = a;
    out2[1] = b;
}

void activation_host(double re, double im, unsigned layer, int activation, double* out2) {
    DevBuf d;
    d.ensure(2 * sizeof(double));
    activation_kernel<<<1, 1>>>(re, im, layer, activation, d.as<double>());
    check_launch("activation_kernel");
    ANN_CUDA(cudaMemcpy(out2, d.p, 2 * sizeof(double), cudaMemcpyDeviceToHost));
}

}  // namespace ann
