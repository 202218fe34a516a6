// Force vector and mean log-derivative without any device allocation.
//
// Some callers cannot allocate GPU memory at the moment they need this reduction:
// code that runs inside a host that owns the whole device memory pool (a framework
// that reserved nearly all HBM up front, so a raw cudaMalloc fails or fragments it),
// and latency-critical loops in which cudaMalloc/cudaFree are unacceptable because
// they can synchronise the device. For them, ann_force_vector_noalloc computes
//     E = sum_s w_s E_s,  Obar_k = sum_s w_s O_sk,  F_k = sum_s w_s E_s conj(O_sk) - E conj(Obar_k)
// from device arrays the caller owns (the same quantities ann_tdvp_eval_F stores),
// using only a fixed scratch area that is a file-scope device array of this library
// (every GPU that loads the library keeps its 4 MiB until the process exits). It calls
// no cudaMalloc, cudaFree or allocating library routine.
#include <algorithm>
#include <mutex>
#include <string>

#include "ann_internal.hpp"

namespace ann {

namespace {

// Fixed scratch, 4 MiB: row partials (kRows blocks x 4 doubles) at offset 0, then
// column partials (slabs x num_params x 2 complex128) from kColOff. At least one slab
// must fit, which caps num_params at kMaxParams (130,816).
constexpr size_t kScratchBytes = 4u << 20;
constexpr unsigned kRows = 256;
constexpr size_t kColOff = ((size_t)kRows * 4 * sizeof(double) + 255) & ~(size_t)255;
constexpr size_t kColBytes = kScratchBytes - kColOff;
constexpr size_t kSlabBytesPerParam = 2 * sizeof(cplx<double>);
constexpr size_t kMaxParams = kColBytes / kSlabBytesPerParam;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// In host code g_noalloc_scratch names a host-side shadow, not the device array: the
// device address is looked up once per device, with that device current, on the first
// call made on it (so the first call on a device should come before any stream capture).
std::mutex g_mu;
void* g_scratch_ptr[64] = {};

void* scratch_address() {
    int dev = 0;
    ANN_CUDA(cudaGetDevice(&dev));
    if(dev < 0 || dev >= 64) throw Error(ANN_ERR_INVALID, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_mu);
    if(!g_scratch_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if(e != cudaSuccess || !p)
            throw Error(ANN_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        g_scratch_ptr[dev] = p;
    }
    return g_scratch_ptr[dev];
}

__device__ __forceinline__ double bsum(double v, double* sh) {
    v = warp_sum(v);
    __syncthreads();
    if((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = 0.0;
    if(threadIdx.x < 32) r = warp_sum(threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0);
    return r;
}

// partial[b] = (sum w, sum w Re E, sum w Im E, unused) over block b's slab of rows
__global__ void __launch_bounds__(256) na_rows_kernel(size_t n, const double* __restrict__ w, double w0,
                                                      const cplx<double>* __restrict__ e, double* partial) {
    __shared__ double sh[32];
    const size_t per = (n + gridDim.x - 1) / gridDim.x;
    const size_t r0 = (size_t)blockIdx.x * per, r1 = min(n, r0 + per);
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    for(size_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        const double wr = w ? w[r] : w0;
        a0 += wr;
        a1 += wr * e[r].re;
        a2 += wr * e[r].im;
    }
    a0 = bsum(a0, sh);
    a1 = bsum(a1, sh);
    a2 = bsum(a2, sh);
    if(threadIdx.x == 0) {
        partial[4 * blockIdx.x] = a0;
        partial[4 * blockIdx.x + 1] = a1;
        partial[4 * blockIdx.x + 2] = a2;
        partial[4 * blockIdx.x + 3] = 0.0;
    }
}

// per column k and slab: sum w O, sum w E conj(O)
__global__ void __launch_bounds__(256) na_cols_kernel(const cplx<float>* __restrict__ O, size_t rows, size_t ld,
                                                      unsigned Np, const double* __restrict__ w, double w0,
                                                      const cplx<double>* __restrict__ e, cplx<double>* part) {
    const unsigned k = blockIdx.x * blockDim.x + threadIdx.x;
    if(k >= Np) return;
    const size_t per = (rows + gridDim.y - 1) / gridDim.y;
    const size_t r0 = (size_t)blockIdx.y * per, r1 = min(rows, r0 + per);
    cplx<double> ao = mk(0.0, 0.0), af = mk(0.0, 0.0);
    for(size_t r = r0; r < r1; r++) {
        const double wr = w ? w[r] : w0;
        const cplx<double> o = cvt<double>(O[r * ld + k]);
        ao.re += wr * o.re;
        ao.im += wr * o.im;
        cmac_conj(af, o, wr * e[r]);  // += w E conj(O)
    }
    cplx<double>* p = part + ((size_t)blockIdx.y * Np + k) * 2;
    p[0] = ao;
    p[1] = af;
}

__global__ void na_final_kernel(const double* __restrict__ rpart, unsigned nb, const cplx<double>* __restrict__ part,
                                unsigned slabs, unsigned Np, cplx<double>* Obar, cplx<double>* F, double* energy) {
    double E0 = 0.0, E1 = 0.0;
    for(unsigned b = 0; b < nb; b++) {
        E0 += rpart[4 * b + 1];
        E1 += rpart[4 * b + 2];
    }
    const unsigned k = blockIdx.x * blockDim.x + threadIdx.x;
    if(k == 0 && energy) {
        energy[0] = E0;
        energy[1] = E1;
    }
    if(k >= Np) return;
    cplx<double> ao = mk(0.0, 0.0), af = mk(0.0, 0.0);
    for(unsigned s = 0; s < slabs; s++) {
        ao += part[((size_t)s * Np + k) * 2];
        af += part[((size_t)s * Np + k) * 2 + 1];
    }
    Obar[k] = ao;
    F[k] = af - mk(E0, E1) * conj(ao);
}

}  // namespace

}  // namespace ann

using namespace ann;

extern "C" int ann_force_vector_noalloc(const void* O_rows, size_t n_rows, size_t ld, unsigned num_params,
                                        const double* weights, double uniform_weight, const double* local_energies,
                                        double* O_mean, double* F, double* energy, void* stream) {
    try {
        if(!O_rows || !local_energies || !O_mean || !F) throw Error(ANN_ERR_INVALID, "null argument");
        if(num_params == 0 || n_rows == 0 || ld < num_params) throw Error(ANN_ERR_INVALID, "bad sizes");
        if(num_params > kMaxParams)
            throw Error(ANN_ERR_INVALID, "ann_force_vector_noalloc: num_params " + std::to_string(num_params) +
                                             " exceeds the fixed scratch limit of " + std::to_string(kMaxParams));
        const size_t per_slab = (size_t)num_params * kSlabBytesPerParam;
        unsigned char* base = static_cast<unsigned char*>(scratch_address());
        double* rpart = reinterpret_cast<double*>(base);
        cplx<double>* cpart = reinterpret_cast<cplx<double>*>(base + kColOff);
        cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
        // The scratch keeps the previous call's partials; nothing needs clearing because
        // every partial read below is written earlier in the same call (all kRows row
        // blocks write theirs, empty slabs included, and the final pass reads exactly the
        // slabs the column pass wrote). Two calls in flight at once on the GPU (different
        // streams, or different host threads) share this scratch and race.
        na_rows_kernel<<<kRows, 256, 0, st>>>(n_rows, weights, uniform_weight,
                                              reinterpret_cast<const cplx<double>*>(local_energies), rpart);
        check_launch("na_rows_kernel");
        const unsigned cb = (num_params + 255) / 256;
        unsigned slabs = (unsigned)((152u * 8u + cb - 1) / cb);
        const unsigned by_rows = (unsigned)((n_rows + 63) / 64);
        const unsigned by_mem = (unsigned)(kColBytes / per_slab);
        slabs = std::max(1u, std::min(std::min(slabs, by_rows), by_mem));
        na_cols_kernel<<<dim3(cb, slabs), 256, 0, st>>>(static_cast<const cplx<float>*>(O_rows), n_rows, ld, num_params,
                                                        weights, uniform_weight,
                                                        reinterpret_cast<const cplx<double>*>(local_energies), cpart);
        check_launch("na_cols_kernel");
        na_final_kernel<<<cb, 256, 0, st>>>(rpart, kRows, cpart, slabs, num_params,
                                            reinterpret_cast<cplx<double>*>(O_mean), reinterpret_cast<cplx<double>*>(F),
                                            energy);
        check_launch("na_final_kernel");
        return ANN_OK;
    } catch(const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch(const std::exception& e) {
        set_last_error(e.what());
        return ANN_ERR_INVALID;
    }
}
