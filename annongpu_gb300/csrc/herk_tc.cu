// Precision-form S matrix on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// The complex HERK S = X^H X over centred, weight-scaled rows
// X_sk = sqrt(w_s) (O_sk - mu_k), mu = Obar / W (see herk_simt.cu for the
// identity with the reference's S, source/network_functions/TDVP.cu.template:216-301)
// is embedded in one real product. With A = Re X, B = Im X:
//   Re S = A^T A + B^T B,   Im S = A^T B - B^T A.
// herk_prep_kernel writes the operand XT in BF16, K-major (samples innermost),
// with the rows of parameter block I (128 parameters) stored as
// [Re of the block (128 rows) ; Im of the block (128 rows)]. One CTA computes the
// 128 x 128 complex tile (I, J <= I is mirrored): per K step of 64 samples TMA
// brings the 256 x 64 blocks of I and J into shared memory (128-byte swizzle) and
// one elected thread issues, per 16-sample slice,
//   D1 (TMEM cols   0..255) += Re_I  . [Re_J ; Im_J]^T   (M=128, N=256)
//   D2 (TMEM cols 256..511) += Im_I  . [Re_J ; Im_J]^T
// so Re S = D1[:, :128] + D2[:, 128:], Im S = D1[:, 128:] - D2[:, :128], read back
// by four warps with tcgen05.ld. FP32 accumulation; hi+lo splitting adds the
// products hi.lo and lo.hi as two more K segments.
//
// Every wait on an mbarrier is bounded (globaltimer deadline); a timeout sets
// kStatusTimeout, makes all roles leave their loops, waits (bounded) for the
// copies in flight and frees the tensor memory before returning.
#include <algorithm>

#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include "ann_internal.hpp"
#include "tcgen05.cuh"

namespace ann {

namespace {

using namespace tc;

constexpr int kBM = 128;                    // parameters per tile side
constexpr int kRowsPerBlock = 2 * kBM;      // Re + Im rows of one parameter block
constexpr int kBK = 64;                     // samples per K step (128 bytes of BF16)
constexpr int kStages = 3;
constexpr int kStageBytes = 2 * kRowsPerBlock * kBK * 2;  // A block + B block
constexpr int kTailBytes = 128 + kBM * 8;  // mbarriers, TMEM slot, abort flag | mu_J in FP32
constexpr int kSmemBytes = kStages * kStageBytes + 1024 + kTailBytes;
struct HerkArgs {
    unsigned Np;            // parameters
    unsigned nblk;          // parameter blocks of 128
    unsigned k_steps;       // K steps of 64 samples per segment
    unsigned segments;      // 1 (plain BF16) or 3 (hi.hi + hi.lo + lo.hi)
    unsigned lo_offset;     // column of the lo copy in XT
    const cplx<double>* Obar;
    const Stats* stats;
    cplx<double>* S;        // S in complex128 (integer-widened FP32 sums) ...
    cplx<float>* S32;       // ... or, when non-null, in complex64 (the mixed / FP32 solvers read it)
    unsigned* status;
};

__device__ __forceinline__ void store_widened(cplx<double>* p, float re, float im) {
    *reinterpret_cast<double2*>(p) = make_double2(widen(re), widen(im));
}

// lower block triangle (I >= J) from the linear CTA index
__device__ __forceinline__ void tile_of(unsigned b, unsigned& I, unsigned& J) {
    I = 0;
    while(b > I) { b -= I + 1; I++; }
    J = b;
}

__global__ void __launch_bounds__(128, 1)
herk_tc_kernel(const __grid_constant__ CUtensorMap tmap, HerkArgs a) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // 1024-byte aligned stage buffers (128-byte swizzle atoms)
    unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char* tail = base + kStages * kStageBytes;
    uint64_t* full = reinterpret_cast<uint64_t*>(tail);
    uint64_t* empty = full + kStages;
    uint64_t* done = empty + kStages;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    cplx<float>* obar_j = reinterpret_cast<cplx<float>*>(tail + 128);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned I, J;
    tile_of(blockIdx.x, I, J);

    if(threadIdx.x == 0) {
        for(int s = 0; s < kStages; s++) {
            mbar_init(smem_u32(&full[s]), 1);
            mbar_init(smem_u32(&empty[s]), 1);
        }
        mbar_init(smem_u32(done), 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    {
        // Obar of the tile's columns in FP32 for the epilogue (its only use there)
        const unsigned l = J * kBM + threadIdx.x;
        obar_j[threadIdx.x] = l < a.Np ? cvt<float>(a.Obar[l]) : mk(0.f, 0.f);
    }
    __syncwarp();
    if(warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(tmem_slot)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    const unsigned total = a.segments * a.k_steps;
    int issued = 0;  // TMA stages issued by the producer (for the drain on abort)
    if(warp == 0 && lane == 0) {
        // ---- TMA producer ----
        for(unsigned kt = 0; kt < total; kt++) {
            const int s = kt % kStages;
            const unsigned ph = (kt / kStages) & 1u;
            if(!mbar_wait(smem_u32(&empty[s]), ph ^ 1u, abort_flag, a.status)) break;
            const unsigned seg = kt / a.k_steps, k = kt % a.k_steps;
            const int xa = (int)(k * kBK + (seg == 2 ? a.lo_offset : 0u));
            const int xb = (int)(k * kBK + (seg == 1 ? a.lo_offset : 0u));
            unsigned char* sa = base + s * kStageBytes;
            unsigned char* sb = sa + kRowsPerBlock * kBK * 2;
            mbar_expect_tx(smem_u32(&full[s]), kStageBytes);
            tma_load_2d(smem_u32(sa), &tmap, xa, (int)(I * kRowsPerBlock), smem_u32(&full[s]));
            tma_load_2d(smem_u32(sb), &tmap, xb, (int)(J * kRowsPerBlock), smem_u32(&full[s]));
            issued++;
        }
    } else if(warp == 1 && lane == 0) {
        // ---- MMA issuer ----
        constexpr uint32_t idesc = idesc_bf16(128, 256);
        bool ok = true;
        for(unsigned kt = 0; kt < total && ok; kt++) {
            const int s = kt % kStages;
            const unsigned ph = (kt / kStages) & 1u;
            if(!mbar_wait(smem_u32(&full[s]), ph, abort_flag, a.status)) { ok = false; break; }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t sa = smem_u32(base + s * kStageBytes);
            const uint32_t sb = sa + kRowsPerBlock * kBK * 2;
#pragma unroll
            for(int kk = 0; kk < kBK / 16; kk++) {
                const int acc = (kt > 0 || kk > 0) ? 1 : 0;
                const uint64_t db = sw128_desc(sb + kk * 32);
                mma_bf16(tmem, sw128_desc(sa + kk * 32), db, idesc, acc);                        // Re_I rows
                mma_bf16(tmem + 256, sw128_desc(sa + kBM * 128 + kk * 32), db, idesc, acc);      // Im_I rows
            }
            mma_commit(smem_u32(&empty[s]));
        }
        mma_commit(smem_u32(done));
    }
    __syncwarp();

    // ---- epilogue: all four warps ----
    bool ok = mbar_wait(smem_u32(done), 0, abort_flag, a.status) && !*abort_flag;
    ok = __all_sync(0xffffffffu, ok);  // tcgen05.ld below is warp-collective
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if(ok) {
        // FP32 arithmetic and an integer widening to FP64: the FP64 pipe (1/64 of the FP32
        // rate on this GPU) would otherwise hold the SM for a third of the tile's time.
        // The accumulators are FP32 sums of K products, so rounding Re S = rr + ii once
        // more in FP32 is below their own rounding.
        const double W = a.stats->W;
        const double corr = 1.0 / W - 1.0;
        const unsigned i = warp * 32 + lane;  // TMEM lane = row of the tile
        const unsigned k = I * kBM + i;       // parameter of the row
        const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
        const bool row_ok = k < a.Np;
        const cplx<float> ok_c = row_ok ? cvt<float>(corr * conj(a.Obar[k])) : mk(0.f, 0.f);
        for(int c0 = 0; c0 < kBM; c0 += 16) {
            float rr[16], ri[16], ir[16], ii[16];
            tmem_ld16(lane_addr + c0, rr);
            tmem_ld16(lane_addr + kBM + c0, ri);
            tmem_ld16(lane_addr + 256 + c0, ir);
            tmem_ld16(lane_addr + 256 + kBM + c0, ii);
            if(!row_ok) continue;
#pragma unroll
            for(int q = 0; q < 16; q++) {
                const unsigned l = J * kBM + c0 + q;
                if(l >= a.Np) continue;
                const cplx<float> ob = obar_j[c0 + q];
                float vr = rr[q] + ii[q], vi = ri[q] - ir[q];
                vr = fmaf(ok_c.re, ob.re, vr);
                vr = fmaf(-ok_c.im, ob.im, vr);
                vi = fmaf(ok_c.re, ob.im, vi);
                vi = fmaf(ok_c.im, ob.re, vi);
                if(a.S32) {
                    a.S32[(size_t)k * a.Np + l] = mk(vr, vi);
                    if(I != J) a.S32[(size_t)l * a.Np + k] = mk(vr, -vi);
                } else {
                    store_widened(a.S + (size_t)k * a.Np + l, vr, vi);
                    if(I != J) store_widened(a.S + (size_t)l * a.Np + k, vr, -vi);
                }
            }
        }
    } else if(warp == 0 && lane == 0) {
        // drain: wait (bounded) for every issued copy before the buffers go away
        for(int q = issued > kStages ? issued - kStages : 0; q < issued; q++) {
            const int s = q % kStages;
            const unsigned long long t0 = gtime();
            while(!mbar_try(smem_u32(&full[s]), (q / kStages) & 1u) && gtime() - t0 < kWaitNs) {}
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if(warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem));
}

// Per-sample sqrt(w_s) and per-parameter mu_k = Obar_k / W, once per S in FP64 and rounded
// to FP32 (the values the operand prep used to form per CTA, where the FP64 square root and
// division, at 1/64 of the FP32 rate, cost more than the tile's loads). Entries past the
// samples / parameters are zero.
__global__ void herk_consts_kernel(size_t rows, size_t ns_pad, unsigned Np, unsigned np_pad,
                                   const double* __restrict__ wts, double w0, const cplx<double>* __restrict__ Obar,
                                   const Stats* __restrict__ stats, float* __restrict__ sw_all,
                                   cplx<float>* __restrict__ mu_all) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if(i < ns_pad) sw_all[i] = i < rows ? (float)sqrt(wts ? wts[i] : w0) : 0.f;
    if(i < np_pad) mu_all[i] = i < Np ? cvt<float>((1.0 / stats->W) * Obar[i]) : mk(0.f, 0.f);
}

// XT[row][col] (BF16): row = 256 * (k / 128) + (k % 128) for Re, + 128 for Im;
// col = sample (hi copy) and lo_offset + sample (lo copy, split mode).
template<typename T>
__global__ void __launch_bounds__(256)
herk_prep_kernel(const cplx<T>* __restrict__ O, size_t rows, size_t ld, unsigned Np, const float* __restrict__ sw_all,
                 const cplx<float>* __restrict__ mu_all, __nv_bfloat16* __restrict__ XT, size_t ldx,
                 unsigned lo_offset, int split) {
    __shared__ cplx<float> tile[64][65];
    __shared__ float sw[64];          // sqrt(w_s) of the tile's rows
    __shared__ cplx<float> mu[64];    // Obar_k / W of the tile's columns
    const size_t s0 = (size_t)blockIdx.y * 64;
    const unsigned k0 = blockIdx.x * 64;
    if(threadIdx.x < 64) sw[threadIdx.x] = sw_all[s0 + threadIdx.x];
    else if(threadIdx.x < 128) mu[threadIdx.x - 64] = mu_all[k0 + threadIdx.x - 64];
    __syncthreads();
    // per element in FP32: the centring and scaling feed BF16 operands
    for(int q = threadIdx.x; q < 64 * 64; q += 256) {
        const int r = q / 64, c = q % 64;
        const size_t s = s0 + r;
        const unsigned k = k0 + c;
        cplx<float> v = mk(0.f, 0.f);
        if(s < rows && k < Np) {
            const cplx<float> o = cvt<float>(O[s * ld + k]);
            v = mk(sw[r] * (o.re - mu[c].re), sw[r] * (o.im - mu[c].im));
        }
        tile[r][c] = v;
    }
    __syncthreads();
    // 128 output rows (64 params x Re/Im) of 64 samples = 32 bf16 pairs each
    for(int q = threadIdx.x; q < 128 * 32; q += 256) {
        const int orow = q / 32, pair = q % 32;
        const int c = orow >> 1, part = orow & 1;
        const unsigned k = k0 + c;
        const size_t row = (size_t)(k / kBM) * kRowsPerBlock + (k % kBM) + (part ? kBM : 0);
        const float x0 = part ? tile[2 * pair][c].im : tile[2 * pair][c].re;
        const float x1 = part ? tile[2 * pair + 1][c].im : tile[2 * pair + 1][c].re;
        const __nv_bfloat162 hi = __floats2bfloat162_rn(x0, x1);
        __nv_bfloat162* dst = reinterpret_cast<__nv_bfloat162*>(XT + row * ldx + s0) + pair;
        *dst = hi;
        if(split) {
            const float2 h = __bfloat1622float2(hi);
            *(reinterpret_cast<__nv_bfloat162*>(XT + row * ldx + lo_offset + s0) + pair) =
                __floats2bfloat162_rn(x0 - h.x, x1 - h.y);
        }
    }
}


}  // namespace

void herk_tc(ann_tdvp_impl& td, const double* wts, double w0, bool split, cudaStream_t st) {
    const unsigned Np = td.Np;
    const unsigned nblk = (Np + kBM - 1) / kBM;
    const size_t rows_x = (size_t)nblk * kRowsPerBlock;
    const size_t ns_pad = (td.n_rows + kBK - 1) / kBK * kBK;
    const size_t ldx = split ? 2 * ns_pad : ns_pad;
    // operand XT, then sqrt(w) per padded sample and mu per parameter slot (FP32)
    const size_t np_pad = (size_t)nblk * kBM;
    const size_t xt_bytes = rows_x * ldx * sizeof(__nv_bfloat16);  // a multiple of 128
    td.herk_in.ensure(xt_bytes + ns_pad * sizeof(float) + np_pad * sizeof(cplx<float>));
    auto* XT = td.herk_in.as<__nv_bfloat16>();
    float* sw_all = reinterpret_cast<float*>(td.herk_in.as<unsigned char>() + xt_bytes);
    auto* mu_all = reinterpret_cast<cplx<float>*>(sw_all + ns_pad);  // ns_pad is a multiple of 64
    if(td.O_precision != 0) throw Error(ANN_ERR_UNSUPPORTED, "tensor-core S takes complex64 rows");
    const size_t nc = std::max(ns_pad, np_pad);
    herk_consts_kernel<<<(unsigned)((nc + 255) / 256), 256, 0, st>>>(td.n_rows, ns_pad, Np, (unsigned)np_pad, wts, w0,
                                                                       td.Obar.as<cplx<double>>(),
                                                                       td.stats.as<Stats>(), sw_all, mu_all);
    check_launch("herk_consts_kernel");
    // the grid covers every parameter slot of the nblk blocks and every padded sample, so
    // the padding (parameters >= Np, samples >= rows) is written as zero by the kernel
    dim3 pg(2 * nblk, (unsigned)(ns_pad / 64));
    herk_prep_kernel<float><<<pg, 256, 0, st>>>(td.O.as<cplx<float>>(), td.n_rows, td.ldO, Np, sw_all, mu_all, XT,
                                                 ldx, (unsigned)ns_pad, split ? 1 : 0);
    check_launch("herk_prep_kernel");

    CUtensorMap map;
    const cuuint64_t dims[2] = {(cuuint64_t)ldx, (cuuint64_t)rows_x};
    const cuuint64_t strides[1] = {(cuuint64_t)(ldx * sizeof(__nv_bfloat16))};
    const cuuint32_t box[2] = {kBK, kRowsPerBlock};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = encode_fn()(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, td.herk_in.p, dims, strides, box, estr,
                                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if(r != CUDA_SUCCESS) throw Error(ANN_ERR_CUDA, "cuTensorMapEncodeTiled failed");

    HerkArgs a;
    a.Np = Np;
    a.nblk = nblk;
    a.k_steps = (unsigned)(ns_pad / kBK);
    a.segments = split ? 3 : 1;
    a.lo_offset = (unsigned)ns_pad;
    a.Obar = td.Obar.as<cplx<double>>();
    a.stats = td.stats.as<Stats>();
    a.S = td.S_in32 ? nullptr : td.S.as<cplx<double>>();
    a.S32 = td.S_in32 ? td.S32.as<cplx<float>>() : nullptr;
    a.status = status_word();
    static bool attr = false;
    if(!attr) {
        ANN_CUDA(cudaFuncSetAttribute(herk_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes));
        attr = true;
    }
    const unsigned tiles = nblk * (nblk + 1) / 2;
    herk_tc_kernel<<<tiles, 128, kSmemBytes, st>>>(map, a);
    check_launch("herk_tc_kernel");
}

}  // namespace ann
