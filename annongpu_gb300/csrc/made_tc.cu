// Tensor-core GEMMs of the MADE training step (tcgen05, kind::f16 with BF16 operands and
// FP32 accumulation in tensor memory).
//
//   C (M x N, FP32) = sum over segments s of  A[:, a_s : a_s + K] . B[:, b_s : b_s + K]^T
//
// A (M rows) and B (N rows) are BF16, row-major with K innermost (K-major), read by TMA in
// boxes of 64 K-values (128 bytes, 128-byte swizzle) x 128 rows (A) or x 64 rows (B); each
// CTA computes a 128 x 64 tile (small GEMMs of a few MFLOP: many CTAs share the epilogue). FP32
// activations and gradients enter as a BF16 pair hi + lo (hi = bf16(x), lo = bf16(x - hi),
// 16 significant bits): a product of two split operands is hi.hi + lo.hi + hi.lo, of a split
// operand and a BF16 weight (or the exact 0/1 inputs) hi.w + lo.w. The segments are those
// products, laid side by side along K in the operands ([hi | lo] columns), so one kernel
// covers every GEMM of the step:
//   pre = X W1^T + b1            A = X (0/1)       B = W1 (H x N)      1 segment
//   l   = relu(pre) W2^T + b2    A = [h | h_lo]    B = W2 (N x H)      2 segments
//   dh  = (dl W2) [pre > 0]      A = [dl | dl_lo]  B = W2^T (H x N)    2 segments
//   gW2 = dl^T h                 A = [dl^T | lo]   B = [h^T | lo]      3 segments, K = batch
//   gW1 = dh^T X                 A = [dh^T | lo]   B = X^T             2 segments, K = batch
// The weight gradients split K (the batch) over grid.z; partial tiles are summed in chunk
// order (deterministic).
//
// Warp roles per CTA (128 threads): warp 0 lane 0 issues the TMA loads into a 3-stage ring,
// warp 1 lane 0 issues the MMAs (M = 128, N = 64, K = 16 per instruction) and commits each
// stage back to the producer; then all four warps read the accumulator (TMEM lane = row of
// the tile) and apply the epilogue. Every mbarrier wait is bounded; on a timeout the CTA
// raises kStatusTimeout, drains its copies in flight and frees its tensor memory.
#include <algorithm>

#include "ann_internal.hpp"
#include "tcgen05.cuh"

namespace ann {

namespace {

using namespace tc;
using bf16 = __nv_bfloat16;

constexpr int kTM = 128;                 // tile rows (TMEM lanes)
constexpr int kTK = 64;                  // K values per stage (128 bytes of BF16)
constexpr int kStagesG = 3;

struct GemmArgs {
    unsigned M, N;          // output rows / columns
    unsigned ksteps;        // 64-wide K steps per segment
    unsigned kchunk;        // K steps of each segment per grid.z chunk
    unsigned nseg;          // 1 .. 3
    int aoff[3], boff[3];   // K offset (elements) of each segment in A and in B
    float* C;               // output, or partial tiles (grid.z chunks of M x N) when split
    size_t ldc;
    const float* bias;      // per column, or null
    const float* aux;       // C = 0 where aux[m * ldc + n] <= 0, or null
    unsigned* status;
};

template<int BN>
__host__ __device__ constexpr int stage_bytes() {
    return kTM * kTK * 2 + BN * kTK * 2;
}
template<int BN>
__host__ __device__ constexpr int gemm_smem() {
    return kStagesG * stage_bytes<BN>() + 1024 + 128;
}

template<int BN>
__global__ void __launch_bounds__(128, 1)
made_gemm_kernel(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, GemmArgs g) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char* tail = base + kStagesG * stage_bytes<BN>();
    uint64_t* full = reinterpret_cast<uint64_t*>(tail);
    uint64_t* empty = full + kStagesG;
    uint64_t* done = empty + kStagesG;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    constexpr uint32_t kCols = BN < 32 ? 32 : BN;  // TMEM columns: a power of two >= 32

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned n0 = blockIdx.x * BN, m0 = blockIdx.y * kTM;
    const unsigned k_lo = blockIdx.z * g.kchunk;
    const unsigned k_hi = min(g.ksteps, k_lo + g.kchunk);
    const unsigned steps = k_hi > k_lo ? k_hi - k_lo : 0u;

    if(threadIdx.x == 0) {
        for(int s = 0; s < kStagesG; s++) {
            mbar_init(smem_u32(&full[s]), 1);
            mbar_init(smem_u32(&empty[s]), 1);
        }
        mbar_init(smem_u32(done), 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if(warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(kCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    const unsigned total = g.nseg * steps;
    int issued = 0;
    if(warp == 0 && lane == 0) {
        // ---- TMA producer ----
        for(unsigned kt = 0; kt < total; kt++) {
            const int s = kt % kStagesG;
            const unsigned ph = (kt / kStagesG) & 1u;
            if(!mbar_wait(smem_u32(&empty[s]), ph ^ 1u, abort_flag, g.status)) break;
            const unsigned seg = kt / steps, k = k_lo + kt % steps;
            unsigned char* sa = base + s * stage_bytes<BN>();
            unsigned char* sb = sa + kTM * kTK * 2;
            mbar_expect_tx(smem_u32(&full[s]), stage_bytes<BN>());
            tma_load_2d(smem_u32(sa), &ta, g.aoff[seg] + (int)(k * kTK), (int)m0, smem_u32(&full[s]));
            tma_load_2d(smem_u32(sb), &tb, g.boff[seg] + (int)(k * kTK), (int)n0, smem_u32(&full[s]));
            issued++;
        }
    } else if(warp == 1 && lane == 0) {
        // ---- MMA issuer ----
        constexpr uint32_t idesc = idesc_bf16(kTM, BN);
        for(unsigned kt = 0; kt < total; kt++) {
            const int s = kt % kStagesG;
            const unsigned ph = (kt / kStagesG) & 1u;
            if(!mbar_wait(smem_u32(&full[s]), ph, abort_flag, g.status)) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t sa = smem_u32(base + s * stage_bytes<BN>());
            const uint32_t sb = sa + kTM * kTK * 2;
#pragma unroll
            for(int kk = 0; kk < kTK / 16; kk++)
                mma_bf16(tmem, sw128_desc(sa + kk * 32), sw128_desc(sb + kk * 32), idesc, (kt > 0 || kk > 0) ? 1 : 0);
            mma_commit(smem_u32(&empty[s]));
        }
        mma_commit(smem_u32(done));
    }
    __syncwarp();

    // ---- epilogue: all four warps (TMEM lane = row of the tile) ----
    bool ok = total == 0 || (mbar_wait(smem_u32(done), 0, abort_flag, g.status) && !*abort_flag);
    ok = __all_sync(0xffffffffu, ok);  // tcgen05.ld below is warp-collective
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if(ok) {
        const unsigned m = m0 + warp * 32 + lane;
        const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
        float* Crow = g.C + (size_t)blockIdx.z * g.M * g.ldc + (size_t)m * g.ldc;
        for(int c0 = 0; c0 < BN; c0 += 16) {
            float v[16];
            if(total) tmem_ld16(lane_addr + c0, v);
            else
#pragma unroll
                for(int q = 0; q < 16; q++) v[q] = 0.f;
            if(m >= g.M) continue;
            const unsigned nb = n0 + c0;
            if(nb + 16 <= g.N && (g.ldc & 3) == 0) {
                // whole 16-column group: four 16-byte loads and stores
#pragma unroll
                for(int q4 = 0; q4 < 4; q4++) {
                    float4 x = make_float4(v[4 * q4], v[4 * q4 + 1], v[4 * q4 + 2], v[4 * q4 + 3]);
                    if(g.bias) {
                        const float4 b = *reinterpret_cast<const float4*>(g.bias + nb + 4 * q4);
                        x.x += b.x; x.y += b.y; x.z += b.z; x.w += b.w;
                    }
                    if(g.aux) {
                        const float4 a = *reinterpret_cast<const float4*>(g.aux + (size_t)m * g.ldc + nb + 4 * q4);
                        if(!(a.x > 0.f)) x.x = 0.f;
                        if(!(a.y > 0.f)) x.y = 0.f;
                        if(!(a.z > 0.f)) x.z = 0.f;
                        if(!(a.w > 0.f)) x.w = 0.f;
                    }
                    *reinterpret_cast<float4*>(Crow + nb + 4 * q4) = x;
                }
                continue;
            }
#pragma unroll
            for(int q = 0; q < 16; q++) {
                const unsigned n = nb + q;
                if(n >= g.N) continue;
                float x = v[q];
                if(g.bias) x += g.bias[n];
                if(g.aux && !(g.aux[(size_t)m * g.ldc + n] > 0.f)) x = 0.f;
                Crow[n] = x;
            }
        }
    } else if(warp == 0 && lane == 0) {
        // drain: wait (bounded) for every issued copy before the buffers go away
        for(int q = issued > kStagesG ? issued - kStagesG : 0; q < issued; q++) {
            const int s = q % kStagesG;
            const unsigned long long t0 = gtime();
            while(!mbar_try(smem_u32(&full[s]), (q / kStagesG) & 1u) && gtime() - t0 < kWaitNs) {}
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if(warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols));
}

// BF16 hi / lo of FP32 values: dst[r][c] = hi, dst[r][lo_off + c] = lo (with_lo) for
// r < rows, c < cols; entries outside the R x C source (padding) are zero, so padded K
// contributes nothing and padded rows give zero output rows
__global__ void split_rows_kernel(const float* __restrict__ src, unsigned R, unsigned C, size_t lds,
                                  bf16* __restrict__ dst, size_t ldd, unsigned rows, unsigned cols, unsigned lo_off,
                                  int with_lo) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= (size_t)rows * cols) return;
    const unsigned r = (unsigned)(i / cols), c = (unsigned)(i % cols);
    const float x = (r < R && c < C) ? src[(size_t)r * lds + c] : 0.f;
    const bf16 h = __float2bfloat16_rn(x);
    dst[(size_t)r * ldd + c] = h;
    if(with_lo) dst[(size_t)r * ldd + lo_off + c] = __float2bfloat16_rn(x - __bfloat162float(h));
}

// the transposed split: dst[c][r] = hi, dst[c][lo_off + r] = lo for c < rows, r < cols,
// through a 32 x 32 tile; entries outside the source are zero
__global__ void split_cols_kernel(const float* __restrict__ src, unsigned R, unsigned C, size_t lds,
                                  bf16* __restrict__ dst, size_t ldd, unsigned rows, unsigned cols, unsigned lo_off,
                                  int with_lo) {
    __shared__ float t[32][33];
    const unsigned r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
    const unsigned tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads
    for(unsigned k = ty; k < 32; k += 8) {
        const unsigned r = r0 + k, c = c0 + tx;
        t[k][tx] = (r < R && c < C) ? src[(size_t)r * lds + c] : 0.f;
    }
    __syncthreads();
    for(unsigned k = ty; k < 32; k += 8) {
        const unsigned c = c0 + k, r = r0 + tx;
        if(c >= rows || r >= cols) continue;
        const float x = t[tx][k];
        const bf16 h = __float2bfloat16_rn(x);
        dst[(size_t)c * ldd + r] = h;
        if(with_lo) dst[(size_t)c * ldd + lo_off + r] = __float2bfloat16_rn(x - __bfloat162float(h));
    }
}

// partial tiles P[z] (M x N) summed in chunk order into C
__global__ void gemm_reduce_kernel(const float* __restrict__ P, unsigned splits, size_t mn, float* __restrict__ C) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= mn) return;
    float acc = 0.f;
    for(unsigned z = 0; z < splits; z++) acc += P[(size_t)z * mn + i];
    C[i] = acc;
}

CUtensorMap bf16_map(const void* p, unsigned cols, unsigned rows, unsigned box_rows) {
    CUtensorMap map;
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
    const cuuint32_t box[2] = {(cuuint32_t)kTK, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = encode_fn()(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(p), dims, strides, box,
                                   estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if(r != CUDA_SUCCESS) throw Error(ANN_ERR_CUDA, "cuTensorMapEncodeTiled failed (MADE GEMM operand)");
    return map;
}

template<int BN>
void launch_gemm(const MadeGemm& q, const CUtensorMap& ta, const CUtensorMap& tb, GemmArgs g, unsigned splits,
                 cudaStream_t st) {
    static bool attr = false;  // per process: the attribute is per function and device-independent
    if(!attr) {
        ANN_CUDA(cudaFuncSetAttribute(made_gemm_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      gemm_smem<BN>()));
        attr = true;
    }
    const dim3 grid((q.N + BN - 1) / BN, (q.M + kTM - 1) / kTM, splits);
    made_gemm_kernel<BN><<<grid, 128, gemm_smem<BN>(), st>>>(ta, tb, g);
    check_launch("made_gemm_kernel");
}

}  // namespace

void made_gemm(const MadeGemm& q, DevBuf& scratch, cudaStream_t st) {
    if(q.K == 0 || q.K % kTK || q.nseg < 1 || q.nseg > 3 || q.a_cols % 8 || q.b_cols % 8)
        throw Error(ANN_ERR_INVALID, "MADE GEMM: K must be a positive multiple of 64, rows 16-byte aligned");
    for(unsigned s = 0; s < q.nseg; s++)
        if(q.aoff[s] % kTK || q.boff[s] % kTK || (unsigned)q.aoff[s] + q.K > q.a_cols ||
           (unsigned)q.boff[s] + q.K > q.b_cols)
            throw Error(ANN_ERR_INVALID, "MADE GEMM: segment outside its operand");
    // 64-column tiles: the GEMMs are small (a few MFLOP), so more CTAs share the epilogue
    constexpr int BN = 64;
    const CUtensorMap ta = bf16_map(q.A, q.a_cols, q.a_rows, kTM);
    const CUtensorMap tb = bf16_map(q.B, q.b_cols, q.b_rows, BN);
    const unsigned ksteps = q.K / kTK;
    const unsigned splits = std::max(1u, std::min(q.splits, ksteps));
    GemmArgs g;
    g.M = q.M;
    g.N = q.N;
    g.ksteps = ksteps;
    g.kchunk = (ksteps + splits - 1) / splits;
    g.nseg = q.nseg;
    for(int s = 0; s < 3; s++) {
        g.aoff[s] = s < (int)q.nseg ? q.aoff[s] : 0;
        g.boff[s] = s < (int)q.nseg ? q.boff[s] : 0;
    }
    g.status = status_word();
    const size_t mn = (size_t)q.M * q.N;
    if(splits > 1) {
        if(q.bias || q.aux || q.ldc != q.N) throw Error(ANN_ERR_INVALID, "MADE GEMM: split K takes a plain output");
        scratch.ensure(splits * mn * sizeof(float));
        g.C = scratch.as<float>();
        g.ldc = q.N;
        g.bias = nullptr;
        g.aux = nullptr;
    } else {
        g.C = q.C;
        g.ldc = q.ldc;
        g.bias = q.bias;
        g.aux = q.aux;
    }
    launch_gemm<BN>(q, ta, tb, g, splits, st);
    if(splits > 1) {
        gemm_reduce_kernel<<<(unsigned)((mn + 255) / 256), 256, 0, st>>>(scratch.as<float>(), splits, mn, q.C);
        check_launch("gemm_reduce_kernel");
    }
}

void made_split_rows(const float* src, unsigned R, unsigned C, size_t lds, void* dst, size_t ldd, unsigned rows,
                     unsigned cols, unsigned lo_off, bool with_lo, cudaStream_t st) {
    if(rows < R || cols < C || (with_lo && lo_off < cols) || ldd < (with_lo ? lo_off + cols : cols))
        throw Error(ANN_ERR_INVALID, "MADE split: output smaller than its source");
    const size_t n = (size_t)rows * cols;
    split_rows_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(src, R, C, lds, static_cast<bf16*>(dst), ldd, rows,
                                                                   cols, lo_off, with_lo ? 1 : 0);
    check_launch("split_rows_kernel");
}

void made_split_cols(const float* src, unsigned R, unsigned C, size_t lds, void* dst, size_t ldd, unsigned rows,
                     unsigned cols, unsigned lo_off, bool with_lo, cudaStream_t st) {
    if(rows < C || cols < R || (with_lo && lo_off < cols) || ldd < (with_lo ? lo_off + cols : cols))
        throw Error(ANN_ERR_INVALID, "MADE split: output smaller than its source");
    const dim3 grid((rows + 31) / 32, (cols + 31) / 32);
    split_cols_kernel<<<grid, 256, 0, st>>>(src, R, C, lds, static_cast<bf16*>(dst), ldd, rows, cols, lo_off,
                                            with_lo ? 1 : 0);
    check_launch("split_cols_kernel");
}

}  // namespace ann
