// Reductions over the sample rows: energy, variance, total weight (FP64), <O>, F,
// S.v (FP64 for complex128 O rows; FP32 within slabs of at most 512 rows and FP64
// across slabs for complex64 O rows). Deterministic: fixed partitions, fixed-order
// combination, no atomics.
//
// Reference semantics: TDVP::compute_averages (source/network_functions/
// TDVP.cu.template:77-126) and its host post-processing (:293-301),
// ExpectationValue::fluctuation / gradient (ExpectationValue.cu.template:175-275),
// TDVP::S_dot_vector (TDVP.cu.template:336-443). The reference accumulates with
// global FP64 atomics; here every block reduces a fixed slab and a second pass
// adds the slabs in order.
#include <algorithm>

#include "ann_internal.hpp"

namespace ann {

namespace {

constexpr int kRowThreads = 256;
constexpr int kRowBlocks = 256;

__device__ __forceinline__ double block_sum(double v, double* sh) {
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

// partial[b] = 6 sums over rows of block b's slab
__global__ void __launch_bounds__(kRowThreads)
row_stats_kernel(size_t n, const double* __restrict__ wts, double w0, const cplx<double>* __restrict__ eloc,
                 const cplx<double>* __restrict__ lpsi, double* __restrict__ partial) {
    __shared__ double sh[32];
    const size_t per = (n + gridDim.x - 1) / gridDim.x;
    const size_t r0 = (size_t)blockIdx.x * per, r1 = min(n, r0 + per);
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for(size_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        const double w = wts ? wts[r] : w0;
        acc[0] += w;
        if(eloc) {
            const cplx<double> e = eloc[r];
            acc[1] += w * e.re;
            acc[2] += w * e.im;
            acc[3] += w * (e.re * e.re + e.im * e.im);
        }
        const cplx<double> l = lpsi[r];
        acc[4] += w * l.re;
        acc[5] += w * l.im;
    }
    for(int k = 0; k < 6; k++) {
        const double s = block_sum(acc[k], sh);
        if(threadIdx.x == 0) partial[(size_t)blockIdx.x * 6 + k] = s;
    }
}

__global__ void row_stats_final(const double* __restrict__ partial, int nb, Stats* out) {
    if(threadIdx.x == 0) {
        double acc[6] = {0, 0, 0, 0, 0, 0};
        for(int b = 0; b < nb; b++)
            for(int k = 0; k < 6; k++) acc[k] += partial[(size_t)b * 6 + k];
        out->W = acc[0];
        out->E[0] = acc[1];
        out->E[1] = acc[2];
        out->E2 = acc[3];
        out->L[0] = acc[4];
        out->L[1] = acc[5];
    }
}

template<typename T>
__device__ __forceinline__ cplx<double> ldO(const void* O, size_t idx) {
    return cvt<double>(reinterpret_cast<const cplx<T>*>(O)[idx]);
}

// per column k, over a slab of rows: sum w O, sum w e conj(O), sum O
template<typename T>
__global__ void __launch_bounds__(256)
col_stats_kernel(const void* __restrict__ O, size_t rows, size_t ld, unsigned Np, const double* __restrict__ wts,
                 double w0, const cplx<double>* __restrict__ e, cplx<double>* __restrict__ part, int want_sum) {
    const unsigned k = blockIdx.x * blockDim.x + threadIdx.x;
    if(k >= Np) return;
    const size_t per = (rows + gridDim.y - 1) / gridDim.y;
    const size_t r0 = (size_t)blockIdx.y * per, r1 = min(rows, r0 + per);
    cplx<double> ao = mk(0.0, 0.0), af = mk(0.0, 0.0), as = mk(0.0, 0.0);
    for(size_t r = r0; r < r1; r++) {
        const double w = wts ? wts[r] : w0;
        const cplx<double> o = ldO<T>(O, r * ld + k);
        ao.re += w * o.re;
        ao.im += w * o.im;
        if(e) {
            const cplx<double> we = w * e[r];
            af += we * conj(o);
        }
        if(want_sum) as += o;
    }
    cplx<double>* p = part + ((size_t)blockIdx.y * Np + k) * 3;
    p[0] = ao;
    p[1] = af;
    p[2] = as;
}

// complex64 O rows: FP32 accumulation over a slab of at most kSlab rows, FP64 across
// slabs. The slab's weights are scaled by their maximum (exact-summation weights are
// unnormalised |psi|^2 and may exceed the FP32 range); with `center` the energies are
// centred, e - E/W, so the sum that becomes F does not cancel:
//   F = sum w e conj(O) - E conj(Obar) = sum w (e - E/W) conj(O) + E (1/W - 1) conj(Obar).
constexpr int kSlab = 512;

__global__ void __launch_bounds__(256)
col_stats_f32_kernel(const cplx<float>* __restrict__ O, size_t rows, size_t ld, unsigned Np, const double* __restrict__ wts,
                     double w0, const cplx<double>* __restrict__ e, const Stats* __restrict__ center,
                     cplx<double>* __restrict__ part, int want_sum, unsigned per) {
    __shared__ float sw[kSlab];
    __shared__ cplx<float> swe[kSlab];
    __shared__ double red[8];
    const size_t r0 = (size_t)blockIdx.y * per, r1 = min(rows, r0 + per);
    const unsigned nr = (unsigned)(r1 - r0);
    // slab scale: the largest weight of the slab
    double wmax = 0.0;
    for(unsigned t = threadIdx.x; t < nr; t += blockDim.x) wmax = fmax(wmax, wts ? wts[r0 + t] : w0);
#pragma unroll
    for(int o = 16; o > 0; o >>= 1) wmax = fmax(wmax, __shfl_xor_sync(0xffffffffu, wmax, o));
    if((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = wmax;
    __syncthreads();
    wmax = 0.0;
    for(int w = 0; w < (int)(blockDim.x >> 5); w++) wmax = fmax(wmax, red[w]);
    const double scale = wmax > 0.0 ? wmax : 1.0;
    cplx<double> shift = mk(0.0, 0.0);
    if(center && e) shift = (1.0 / center->W) * mk(center->E[0], center->E[1]);
    for(unsigned t = threadIdx.x; t < nr; t += blockDim.x) {
        const double wn = (wts ? wts[r0 + t] : w0) / scale;
        sw[t] = (float)wn;
        swe[t] = e ? cvt<float>(wn * (e[r0 + t] - shift)) : mk(0.f, 0.f);
    }
    __syncthreads();
    const unsigned k = blockIdx.x * blockDim.x + threadIdx.x;
    if(k >= Np) return;
    cplx<float> ao = mk(0.f, 0.f), af = mk(0.f, 0.f), as = mk(0.f, 0.f);
    const cplx<float>* Ok = O + r0 * ld + k;
#pragma unroll 8
    for(unsigned t = 0; t < nr; t++) {
        const cplx<float> o = Ok[(size_t)t * ld];
        const float w = sw[t];
        ao.re = fmaf(w, o.re, ao.re);
        ao.im = fmaf(w, o.im, ao.im);
        cmac_conj(af, o, swe[t]);  // += w (e - shift) conj(O)
        as.re += o.re;
        as.im += o.im;
    }
    cplx<double>* p = part + ((size_t)blockIdx.y * Np + k) * 3;
    p[0] = scale * cvt<double>(ao);
    p[1] = scale * cvt<double>(af);
    p[2] = want_sum ? cvt<double>(as) : mk(0.0, 0.0);
}

// centred: the slab sums of F used centred energies (col_stats_f32_kernel with `center`)
__global__ void col_stats_final(const cplx<double>* __restrict__ part, int nslab, unsigned Np,
                                cplx<double>* Obar, cplx<double>* F, const Stats* center, cplx<double>* Osum,
                                int centred) {
    const unsigned k = blockIdx.x * blockDim.x + threadIdx.x;
    if(k >= Np) return;
    cplx<double> ao = mk(0.0, 0.0), af = mk(0.0, 0.0), as = mk(0.0, 0.0);
    for(int s = 0; s < nslab; s++) {
        const cplx<double>* p = part + ((size_t)s * Np + k) * 3;
        ao += p[0];
        af += p[1];
        as += p[2];
    }
    if(Obar) Obar[k] = ao;
    if(F) {
        if(center) {
            const cplx<double> E = mk(center->E[0], center->E[1]);
            if(centred) af = af + ((1.0 / center->W) - 1.0) * (E * conj(ao));
            else af = af - E * conj(ao);
        }
        F[k] = af;
    }
    if(Osum) Osum[k] = as;
}

// y_s = sum_k O_sk v_k, one warp per row
template<typename T>
__global__ void row_dot_kernel(const void* __restrict__ O, size_t rows, size_t ld, unsigned Np,
                               const cplx<double>* __restrict__ v, cplx<double>* __restrict__ y) {
    const size_t r = (size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if(r >= rows) return;
    cplx<double> acc = mk(0.0, 0.0);
    for(unsigned k = lane; k < Np; k += 32) acc += ldO<T>(O, r * ld + k) * v[k];
    acc = warp_sum(acc);
    if(lane == 0) y[r] = acc;
}

// out_k -= conj(Obar_k) * (Obar . v)
__global__ void sdotv_final_kernel(cplx<double>* out, const cplx<double>* Obar, const cplx<double>* v, unsigned Np) {
    __shared__ double sh[32];
    double re = 0.0, im = 0.0;
    for(unsigned k = threadIdx.x; k < Np; k += blockDim.x) {
        const cplx<double> t = Obar[k] * v[k];
        re += t.re;
        im += t.im;
    }
    const double sre = block_sum(re, sh);
    __shared__ double tot[2];
    if(threadIdx.x == 0) tot[0] = sre;
    const double sim = block_sum(im, sh);
    if(threadIdx.x == 0) tot[1] = sim;
    __syncthreads();
    const cplx<double> d = mk(tot[0], tot[1]);
    for(unsigned k = threadIdx.x; k < Np; k += blockDim.x) out[k] = out[k] - conj(Obar[k]) * d;
}

}  // namespace

void row_stats(const Rows& rows, const double* wts, double w0, Stats* out, DevBuf& scratch, cudaStream_t st) {
    scratch.ensure((size_t)kRowBlocks * 6 * sizeof(double));
    row_stats_kernel<<<kRowBlocks, kRowThreads, 0, st>>>(rows.n, wts, w0, rows.eloc.as<cplx<double>>(),
                                                          rows.log_psi.as<cplx<double>>(), scratch.as<double>());
    check_launch("row_stats_kernel");
    row_stats_final<<<1, 32, 0, st>>>(scratch.as<double>(), kRowBlocks, out);
    check_launch("row_stats_final");
}

void col_stats(const void* O, int O_prec, size_t rows, size_t ld, unsigned Np, const double* wts, double w0,
               const cplx<double>* e, cplx<double>* Obar, cplx<double>* F, const Stats* center, cplx<double>* Osum,
               DevBuf& scratch, cudaStream_t st) {
    const unsigned cb = (Np + 255) / 256;
    // enough slabs to fill the GPU, each at least 64 rows (complex64: at most kSlab rows)
    unsigned slabs = (unsigned)((152u * 8u + cb - 1) / cb);
    const unsigned max_slabs = (unsigned)((rows + 63) / 64);
    if(slabs > max_slabs) slabs = max_slabs;
    if(slabs < 1) slabs = 1;
    int centred = 0;
    if(O_prec == 0) {
        unsigned per = (unsigned)((rows + slabs - 1) / slabs);
        if(per > (unsigned)kSlab) per = kSlab;
        if(per < 1) per = 1;
        // the autotuned slab for this shape, when there is one
        const int tuned = tuning_get(key_slab(rows, Np), 0);
        if(tuned > 0) per = (unsigned)std::min(std::max(tuned, 32), kSlab);
        slabs = (unsigned)((rows + per - 1) / per);
        if(slabs < 1) slabs = 1;
        scratch.ensure((size_t)slabs * Np * 3 * sizeof(cplx<double>));
        col_stats_f32_kernel<<<dim3(cb, slabs), 256, 0, st>>>(reinterpret_cast<const cplx<float>*>(O), rows, ld, Np,
                                                              wts, w0, e, center, scratch.as<cplx<double>>(),
                                                              Osum != nullptr, per);
        centred = center != nullptr && e != nullptr;
    } else {
        scratch.ensure((size_t)slabs * Np * 3 * sizeof(cplx<double>));
        col_stats_kernel<double><<<dim3(cb, slabs), 256, 0, st>>>(O, rows, ld, Np, wts, w0, e,
                                                                   scratch.as<cplx<double>>(), Osum != nullptr);
    }
    check_launch("col_stats_kernel");
    col_stats_final<<<cb, 256, 0, st>>>(scratch.as<cplx<double>>(), (int)slabs, Np, Obar, F, center, Osum, centred);
    check_launch("col_stats_final");
}

void row_dot(const void* O, int O_prec, size_t rows, size_t ld, unsigned Np, const cplx<double>* v,
             cplx<double>* y, cudaStream_t st) {
    const unsigned grid = (unsigned)((rows + 7) / 8);
    if(O_prec == 0) row_dot_kernel<float><<<grid, 256, 0, st>>>(O, rows, ld, Np, v, y);
    else row_dot_kernel<double><<<grid, 256, 0, st>>>(O, rows, ld, Np, v, y);
    check_launch("row_dot_kernel");
}

void finalize_sdotv(cplx<double>* out, const cplx<double>* Obar, const cplx<double>* v, unsigned Np, cudaStream_t st) {
    sdotv_final_kernel<<<1, 1024, 0, st>>>(out, Obar, v, Np);
    check_launch("sdotv_final_kernel");
}

}  // namespace ann
