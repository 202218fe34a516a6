// Plain-form S matrix: FP32 SIMT complex HERK over centred O rows.
//
//   S[k, l] = sum_s w_s conj(O_sk - mu_k) (O_sl - mu_l) + (1/W - 1) conj(Obar_k) Obar_l
//
// with Obar = sum_s w_s O_s, W = sum_s w_s and mu = Obar / W, which equals the
// reference's S = sum_s w_s conj(O_sk) O_sl - conj(Obar_k) Obar_l
// (source/network_functions/TDVP.cu.template:216-301) for any total weight W
// (W = 1 for Monte Carlo and for normalised states, where the correction vanishes).
// The reference adds N_s * Np^2 complex FP64 atomics; here each CTA owns one
// 64 x 64 output tile of the upper block triangle, accumulates in registers (FP32 for
// complex64 rows, FP64 for complex128 rows) and writes both triangles in FP64.
#include "ann_internal.hpp"

namespace ann {

namespace {

constexpr int TS = 64;   // output tile
constexpr int KC = 16;   // rows per smem stage

template<typename T>
__global__ void __launch_bounds__(256)
herk_simt_kernel(const cplx<T>* __restrict__ O, size_t rows, size_t ld, unsigned Np, const double* __restrict__ wts,
                 double w0, const cplx<double>* __restrict__ Obar, const Stats* __restrict__ stats,
                 cplx<double>* __restrict__ S, unsigned tiles) {
    __shared__ cplx<T> As[KC][TS];
    __shared__ cplx<T> Bs[KC][TS];
    __shared__ cplx<T> mA[TS], mB[TS];
    __shared__ T sw[KC];

    // upper-triangular tile (ti <= tj) from the linear block index
    unsigned b = blockIdx.x, ti = 0;
    while(b >= tiles - ti) { b -= tiles - ti; ti++; }
    const unsigned tj = ti + b;
    const unsigned k0 = ti * TS, l0 = tj * TS;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;

    const double invW = 1.0 / stats->W;
    if(threadIdx.x < TS) {
        const unsigned k = k0 + threadIdx.x, l = l0 + threadIdx.x;
        mA[threadIdx.x] = k < Np ? cvt<T>(invW * Obar[k]) : mk<T>(T(0), T(0));
        mB[threadIdx.x] = l < Np ? cvt<T>(invW * Obar[l]) : mk<T>(T(0), T(0));
    }
    cplx<T> acc[4][4];
#pragma unroll
    for(int i = 0; i < 4; i++)
#pragma unroll
        for(int j = 0; j < 4; j++) acc[i][j] = mk<T>(T(0), T(0));

    for(size_t s0 = 0; s0 < rows; s0 += KC) {
        __syncthreads();
        if(threadIdx.x < KC) {
            const size_t r = s0 + threadIdx.x;
            sw[threadIdx.x] = r < rows ? (T)sqrt(wts ? wts[r] : w0) : T(0);
        }
        __syncthreads();
#pragma unroll
        for(int q = 0; q < 4; q++) {
            const int idx = threadIdx.x + 256 * q;
            const int r = idx / TS, c = idx % TS;
            const size_t row = s0 + r;
            cplx<T> va = mk<T>(T(0), T(0)), vb = mk<T>(T(0), T(0));
            if(row < rows) {
                const unsigned k = k0 + c, l = l0 + c;
                if(k < Np) va = sw[r] * (cvt<T>(O[row * ld + k]) - mA[c]);
                if(l < Np) vb = sw[r] * (cvt<T>(O[row * ld + l]) - mB[c]);
            }
            As[r][c] = va;
            Bs[r][c] = vb;
        }
        __syncthreads();
#pragma unroll
        for(int s = 0; s < KC; s++) {
            cplx<T> a[4], bb[4];
#pragma unroll
            for(int i = 0; i < 4; i++) a[i] = As[s][ty + 16 * i];
#pragma unroll
            for(int j = 0; j < 4; j++) bb[j] = Bs[s][tx + 16 * j];
#pragma unroll
            for(int i = 0; i < 4; i++)
#pragma unroll
                for(int j = 0; j < 4; j++) cmac_conj(acc[i][j], a[i], bb[j]);  // += conj(a) b
        }
    }
    const double corr = invW - 1.0;
#pragma unroll
    for(int i = 0; i < 4; i++) {
        const unsigned k = k0 + ty + 16 * i;
        if(k >= Np) continue;
        const cplx<double> ok = conj(Obar[k]);
#pragma unroll
        for(int j = 0; j < 4; j++) {
            const unsigned l = l0 + tx + 16 * j;
            if(l >= Np) continue;
            const cplx<double> v = cvt<double>(acc[i][j]) + corr * (ok * Obar[l]);
            S[(size_t)k * Np + l] = v;
            if(ti != tj) S[(size_t)l * Np + k] = conj(v);
        }
    }
}

}  // namespace

void herk_simt(const void* O, int O_prec, size_t rows, size_t ld, unsigned Np, const double* wts, double w0,
               const cplx<double>* Obar, const Stats* stats, cplx<double>* S, cudaStream_t st) {
    const unsigned tiles = (Np + TS - 1) / TS;
    const unsigned nblk = tiles * (tiles + 1) / 2;
    if(O_prec == 0)
        herk_simt_kernel<float><<<nblk, 256, 0, st>>>(reinterpret_cast<const cplx<float>*>(O), rows, ld, Np, wts, w0,
                                                      Obar, stats, S, tiles);
    else
        herk_simt_kernel<double><<<nblk, 256, 0, st>>>(reinterpret_cast<const cplx<double>*>(O), rows, ld, Np, wts,
                                                       w0, Obar, stats, S, tiles);
    check_launch("herk_simt_kernel");
}

}  // namespace ann
