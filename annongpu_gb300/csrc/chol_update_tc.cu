// Trailing update of the FP32 Cholesky on the tensor cores (tcgen05, kind::tf32):
//   A22 -= X X^H,  X = the factorised panel (rows below it, 64 complex columns).
//
// X is split into TF32 hi and lo parts (x = hi + lo + O(2^-22 |x|)); three products
// hi.hi + hi.lo + lo.hi restore FP32-level accuracy (the dropped lo.lo is below it),
// so the factor keeps the quality that the FP64 refinement of the mixed solver needs.
// The panel solve (trsm32_kernel) writes the operand PT, K-major: per 128-row block of
// the trailing rows, [Re rows (128) ; Im rows (128)], each row [hi (64) | lo (64)] floats.
// One CTA updates the 128 x 128 complex tile (I, J <= I) of the trailing matrix: per
// K step of 32 TF32 values TMA brings the 256 x 32 blocks of I and J (128-byte
// swizzle), one elected thread issues per 8-value slice
//   D1 (TMEM cols   0..255) += Re_I . [Re_J ; Im_J]^T   (M = 128, N = 256)
//   D2 (TMEM cols 256..511) += Im_I . [Re_J ; Im_J]^T
// and since (X X^H)_ij = sum_p x_ip conj(x_jp):
//   Re = D1[:, :128] + D2[:, 128:],  Im = D2[:, :128] - D1[:, 128:],
// which four warps read back with tcgen05.ld and subtract from A (FP32, row-major).
//
// Every mbarrier wait is bounded (globaltimer deadline): a timeout raises
// kStatusTimeout, all roles leave their loops, the producer waits (bounded) for its
// copies in flight and the tensor memory is freed before the CTA returns.
#include <algorithm>

#include "ann_internal.hpp"
#include "tcgen05.cuh"

namespace ann {

namespace {

using namespace tc;
using cf = cplx<float>;

constexpr int kBM = 128;                   // tile side (complex rows / columns)
constexpr int kRows = 2 * kBM;             // Re + Im rows of one 128-row block
constexpr int kPanel = 64;                 // panel width (complex columns = K)
constexpr int kRowFloats = 2 * kPanel;     // [hi | lo]
constexpr int kBK = 32;                    // TF32 values per K step (128 bytes)
constexpr int kStages = 3;
constexpr int kStageBytes = 2 * kRows * kBK * 4;  // A block + B block
constexpr int kSmemBytes = kStages * kStageBytes + 1024 + 256;
constexpr int kSegments = 3;               // hi.hi, hi.lo, lo.hi
constexpr int kStepsPerSeg = kPanel / kBK;

struct UpdArgs {
    cf* A;
    unsigned n;
    unsigned t0;        // first trailing row / column
    int col_only;       // tiles (I, 0) only; otherwise tiles (I, J) with 1 <= J <= I
    int tma_reduce;     // epilogue by TMA reduce-add through amap (n even), else row updates
    unsigned* status;
};

// bulk tensor reduce-add of a shared-memory box into global memory (L2 performs the adds)
__device__ __forceinline__ void tma_reduce_add_2d(const CUtensorMap* map, int x, int y, uint32_t src) {
    asm volatile("cp.reduce.async.bulk.tensor.2d.global.shared::cta.add.tile.bulk_group [%0, {%1, %2}], [%3];"
                 ::"l"((unsigned long long)map), "r"(x), "r"(y), "r"(src)
                 : "memory");
}

__global__ void __launch_bounds__(128, 1)
chol_update_tc_kernel(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ CUtensorMap amap, UpdArgs a) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char* tail = base + kStages * kStageBytes;
    uint64_t* full = reinterpret_cast<uint64_t*>(tail);
    uint64_t* empty = full + kStages;
    uint64_t* done = empty + kStages;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned I, J;
    if(a.col_only) {
        I = blockIdx.x;
        J = 0;
    } else {
        unsigned b = blockIdx.x;
        I = 0;
        while(b > I) { b -= I + 1; I++; }
        J = b + 1;
        I += 1;
    }

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
    __syncwarp();
    if(warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(tmem_slot)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    constexpr unsigned total = kSegments * kStepsPerSeg;
    int issued = 0;
    if(warp == 0 && lane == 0) {
        // ---- TMA producer ----
        for(unsigned kt = 0; kt < total; kt++) {
            const int s = kt % kStages;
            const unsigned ph = (kt / kStages) & 1u;
            if(!mbar_wait(smem_u32(&empty[s]), ph ^ 1u, abort_flag, a.status)) break;
            const unsigned seg = kt / kStepsPerSeg, k = kt % kStepsPerSeg;
            const int xa = (int)(k * kBK + (seg == 2 ? kPanel : 0u));  // lo of I in segment lo.hi
            const int xb = (int)(k * kBK + (seg == 1 ? kPanel : 0u));  // lo of J in segment hi.lo
            unsigned char* sa = base + s * kStageBytes;
            unsigned char* sb = sa + kRows * kBK * 4;
            mbar_expect_tx(smem_u32(&full[s]), kStageBytes);
            tma_load_2d(smem_u32(sa), &tmap, xa, (int)(I * kRows), smem_u32(&full[s]));
            tma_load_2d(smem_u32(sb), &tmap, xb, (int)(J * kRows), smem_u32(&full[s]));
            issued++;
        }
    } else if(warp == 1 && lane == 0) {
        // ---- MMA issuer ----
        constexpr uint32_t idesc = idesc_tf32(128, 256);
        bool ok = true;
        for(unsigned kt = 0; kt < total && ok; kt++) {
            const int s = kt % kStages;
            const unsigned ph = (kt / kStages) & 1u;
            if(!mbar_wait(smem_u32(&full[s]), ph, abort_flag, a.status)) { ok = false; break; }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t sa = smem_u32(base + s * kStageBytes);
            const uint32_t sb = sa + kRows * kBK * 4;
#pragma unroll
            for(int kk = 0; kk < kBK / 8; kk++) {
                const int acc = (kt > 0 || kk > 0) ? 1 : 0;
                const uint64_t db = sw128_desc(sb + kk * 32);
                mma_tf32(tmem, sw128_desc(sa + kk * 32), db, idesc, acc);                    // Re_I rows
                mma_tf32(tmem + 256, sw128_desc(sa + kBM * 128 + kk * 32), db, idesc, acc);  // Im_I rows
            }
            mma_commit(smem_u32(&empty[s]));
        }
        mma_commit(smem_u32(done));
    }
    __syncwarp();

    // ---- epilogue: all four warps. TMEM lane = row of the tile: the result goes to
    // shared memory (the drained stage buffers), then the warps update A row by row,
    // each lane 4 consecutive complex values (coalesced 1 KB rows, 16 loads in flight)
    bool ok = mbar_wait(smem_u32(done), 0, abort_flag, a.status) && !*abort_flag;
    ok = __all_sync(0xffffffffu, ok);  // tcgen05.ld below is warp-collective
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if(a.tma_reduce) {
        // -X X^H into shared memory as eight 128-row boxes of 16 complex (128 B rows,
        // 128-byte swizzle: 16-byte unit u of row r at u ^ (r % 8)), then eight bulk
        // tensor reduce-adds into A. Upper-triangle entries of a diagonal tile add 0.
        if(ok) {
            const unsigned i = warp * 32 + lane;
            const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
            const bool diag = I == J;
            for(int c = 0; c < kBM / 16; c++) {
                float rr[16], ri[16], ir[16], ii[16];
                tmem_ld16(lane_addr + c * 16, rr);
                tmem_ld16(lane_addr + kBM + c * 16, ri);
                tmem_ld16(lane_addr + 256 + c * 16, ir);
                tmem_ld16(lane_addr + 256 + kBM + c * 16, ii);
                unsigned char* box = base + (size_t)c * (kBM * 128) + (size_t)i * 128;
#pragma unroll
                for(int u = 0; u < 8; u++) {
                    float4 v;
                    const int q0 = 2 * u, q1 = 2 * u + 1;
                    const bool z0 = diag && (unsigned)(c * 16 + q0) > i, z1 = diag && (unsigned)(c * 16 + q1) > i;
                    v.x = z0 ? 0.f : -(rr[q0] + ii[q0]);
                    v.y = z0 ? 0.f : -(ir[q0] - ri[q0]);
                    v.z = z1 ? 0.f : -(rr[q1] + ii[q1]);
                    v.w = z1 ? 0.f : -(ir[q1] - ri[q1]);
                    *reinterpret_cast<float4*>(box + ((u ^ (i & 7u)) << 4)) = v;
                }
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        }
        if(__syncthreads_and(ok ? 1 : 0) && threadIdx.x == 0) {
            const int y = (int)(a.t0 + I * kBM);
            for(int c = 0; c < kBM / 16; c++)
                tma_reduce_add_2d(&amap, (int)(2 * (a.t0 + J * kBM) + 32 * c), y,
                                  smem_u32(base + (size_t)c * (kBM * 128)));
            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
            asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
        }
    }
    cf (*C)[kBM + 1] = reinterpret_cast<cf (*)[kBM + 1]>(base);  // 128 x 129 complex = 132 KB
    if(ok && !a.tma_reduce) {
        const unsigned i = warp * 32 + lane;
        const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
        for(int c0 = 0; c0 < kBM; c0 += 16) {
            float rr[16], ri[16], ir[16], ii[16];
            tmem_ld16(lane_addr + c0, rr);
            tmem_ld16(lane_addr + kBM + c0, ri);
            tmem_ld16(lane_addr + 256 + c0, ir);
            tmem_ld16(lane_addr + 256 + kBM + c0, ii);
#pragma unroll
            for(int q = 0; q < 16; q++) C[i][c0 + q] = mk(rr[q] + ii[q], ir[q] - ri[q]);
        }
    }
    __syncthreads();
    if(__syncthreads_and(ok && !a.tma_reduce ? 1 : 0)) {
        const size_t row0 = (size_t)a.t0 + (size_t)I * kBM, col0 = (size_t)a.t0 + (size_t)J * kBM;
        const unsigned jl0 = 4u * lane;
        const size_t gj0 = col0 + jl0;
        const bool diag = I == J;
        constexpr int kRowsPerPass = 8;
        for(unsigned r0 = warp * 32; r0 < warp * 32 + 32; r0 += kRowsPerPass) {
            float4 v[kRowsPerPass][2];
#pragma unroll
            for(int rr = 0; rr < kRowsPerPass; rr++) {
                const size_t gi = row0 + r0 + rr;
                const float4* src = reinterpret_cast<const float4*>(a.A + gi * a.n + gj0);
                if(gi < a.n && gj0 + 3 < a.n && (a.n & 1u) == 0) {
                    v[rr][0] = src[0];
                    v[rr][1] = src[1];
                } else {
                    v[rr][0] = make_float4(0.f, 0.f, 0.f, 0.f);
                    v[rr][1] = v[rr][0];
                    const cf* s1 = a.A + gi * a.n + gj0;
                    if(gi < a.n) {
                        if(gj0 < a.n) { v[rr][0].x = s1[0].re; v[rr][0].y = s1[0].im; }
                        if(gj0 + 1 < a.n) { v[rr][0].z = s1[1].re; v[rr][0].w = s1[1].im; }
                        if(gj0 + 2 < a.n) { v[rr][1].x = s1[2].re; v[rr][1].y = s1[2].im; }
                        if(gj0 + 3 < a.n) { v[rr][1].z = s1[3].re; v[rr][1].w = s1[3].im; }
                    }
                }
            }
#pragma unroll
            for(int rr = 0; rr < kRowsPerPass; rr++) {
                const unsigned il = r0 + rr;
                const size_t gi = row0 + il;
                if(gi >= a.n) continue;
                cf* dst = a.A + gi * a.n + gj0;
                float out[8] = {v[rr][0].x, v[rr][0].y, v[rr][0].z, v[rr][0].w,
                                v[rr][1].x, v[rr][1].y, v[rr][1].z, v[rr][1].w};
#pragma unroll
                for(int q = 0; q < 4; q++) {
                    const cf c = C[il][jl0 + q];
                    out[2 * q] -= c.re;
                    out[2 * q + 1] -= c.im;
                }
                const bool full = gj0 + 3 < a.n && (a.n & 1u) == 0 && !(diag && jl0 + 3 > il);
                if(full) {
                    float4* d4 = reinterpret_cast<float4*>(dst);
                    d4[0] = make_float4(out[0], out[1], out[2], out[3]);
                    d4[1] = make_float4(out[4], out[5], out[6], out[7]);
                } else {
#pragma unroll
                    for(int q = 0; q < 4; q++)
                        if(gj0 + q < a.n && !(diag && jl0 + q > il)) dst[q] = mk(out[2 * q], out[2 * q + 1]);
                }
            }
        }
    }
    if(!ok && warp == 0 && lane == 0) {
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

// The update with Re and Im of the tile accumulated directly (N = 128 MMAs, the
// negate-A bit giving -Re_I . Im_J^T), 256 TMEM columns per tile:
//   Re C (TMEM cols   0..127) += Re_I . Re_J^T + Im_I . Im_J^T
//   Im C (TMEM cols 128..255) += Im_I . Re_J^T - Re_I . Im_J^T
// The epilogue streams C in eight 16-column chunks through the swizzled buffer into bulk
// tensor reduce-adds (A's row pitch must be 16-byte aligned: n even).
constexpr int kStageBytesN = 2 * kRows * kBK * 4;  // one stage: A block + B block (64 KB)
constexpr int kChunkBytes = kBM * 128;             // 128 rows x 16 complex
// Persistent kernel: CTA g walks the tiles g, g + G, ... (one tile per CTA for launches of
// up to a wave) with the roles split over warps (warp 0: TMA producer, warp 1: MMA issuer,
// warps 4-7: epilogue, TMEM lane quarter = warp % 4). Two 256-column TMEM accumulators
// (Re | Im) let the MMAs of the next tile run while the epilogue drains the previous one;
// loads go through a two-stage ring of 64 KB, the epilogue through a double-buffered 16 KB
// chunk into bulk tensor reduce-adds.
// Barriers: full/empty (stage ring), acc_full (MMA -> epilogue), acc_empty (epilogue ->
// MMA), all waits bounded; a timeout raises kStatusTimeout and every role leaves.
constexpr int kStages3 = 2;
constexpr int kSmem3Bytes = kStages3 * kStageBytesN + 2 * kChunkBytes + 1024 + 256;
constexpr unsigned kEpiThreads = 128;

// P = K of the update: 64 (one panel) or 128 (two panels, rows [hi (128) | lo (128)])
template<int P>
__global__ void __launch_bounds__(256, 1)
chol_update_tc3_kernel(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ CUtensorMap amap, UpdArgs a,
                       unsigned n_tiles) {
    static_assert(P % kBK == 0, "K steps of 32 TF32 values");
    constexpr unsigned kSteps = P / kBK;  // K steps per segment
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char* chunks = base + kStages3 * kStageBytesN;
    uint64_t* full = reinterpret_cast<uint64_t*>(chunks + 2 * kChunkBytes);
    uint64_t* empty = full + kStages3;
    uint64_t* accf = empty + kStages3;
    uint64_t* acce = accf + 2;
    uint64_t* mdone = acce + 2;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mdone + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    auto tile_ij = [&](unsigned t, unsigned& I, unsigned& J) {
        if(a.col_only) {
            I = t;
            J = 0;
        } else {
            unsigned b = t;
            I = 0;
            while(b > I) { b -= I + 1; I++; }
            J = b + 1;
            I += 1;
        }
    };
    const unsigned my_tiles = n_tiles > blockIdx.x ? (n_tiles - blockIdx.x + gridDim.x - 1) / gridDim.x : 0u;

    if(threadIdx.x == 0) {
        for(int q = 0; q < kStages3; q++) {
            mbar_init(smem_u32(&full[q]), 1);
            mbar_init(smem_u32(&empty[q]), 1);
        }
        for(int q = 0; q < 2; q++) {
            mbar_init(smem_u32(&accf[q]), 1);
            mbar_init(smem_u32(&acce[q]), 1);
        }
        mbar_init(smem_u32(mdone), 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if(warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(tmem_slot)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    constexpr unsigned ksteps = kSegments * kSteps;

    if(warp == 0 && lane == 0) {
        // ---- TMA producer ----
        unsigned issued = 0;
        bool ok = true;
        for(unsigned lt = 0; lt < my_tiles && ok; lt++) {
            unsigned I, J;
            tile_ij(blockIdx.x + lt * gridDim.x, I, J);
            for(unsigned kt = 0; kt < ksteps; kt++) {
                const unsigned g = lt * ksteps + kt, s = g % kStages3, ph = (g / kStages3) & 1u;
                if(!mbar_wait(smem_u32(&empty[s]), ph ^ 1u, abort_flag, a.status)) { ok = false; break; }
                const unsigned seg = kt / kSteps, k = kt % kSteps;
                const int xa = (int)(k * kBK + (seg == 2 ? (unsigned)P : 0u));  // lo of I in segment lo.hi
                const int xb = (int)(k * kBK + (seg == 1 ? (unsigned)P : 0u));  // lo of J in segment hi.lo
                unsigned char* st = base + s * kStageBytesN;
                mbar_expect_tx(smem_u32(&full[s]), kStageBytesN);
                tma_load_2d(smem_u32(st), &tmap, xa, (int)(I * kRows), smem_u32(&full[s]));
                tma_load_2d(smem_u32(st + kRows * kBK * 4), &tmap, xb, (int)(J * kRows), smem_u32(&full[s]));
                issued++;
            }
        }
        if(!ok) {
            // wait (bounded) for the copies in flight before the buffers go away
            for(unsigned q = issued > (unsigned)kStages3 ? issued - kStages3 : 0u; q < issued; q++) {
                const unsigned long long t0 = gtime();
                while(!mbar_try(smem_u32(&full[q % kStages3]), (q / kStages3) & 1u) && gtime() - t0 < kWaitNs) {}
            }
        }
    } else if(warp == 1 && lane == 0) {
        // ---- MMA issuer ----
        constexpr uint32_t idesc = idesc_tf32(128, 128);
        constexpr uint32_t idesc_neg = idesc | (1u << 13);  // negate A
        bool ok = true;
        for(unsigned lt = 0; lt < my_tiles && ok; lt++) {
            const unsigned b = lt & 1u, aph = (lt >> 1) & 1u;
            if(!mbar_wait(smem_u32(&acce[b]), aph ^ 1u, abort_flag, a.status)) { ok = false; break; }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t d = tmem + b * 256u;
            for(unsigned kt = 0; kt < ksteps; kt++) {
                const unsigned g = lt * ksteps + kt, s = g % kStages3, ph = (g / kStages3) & 1u;
                if(!mbar_wait(smem_u32(&full[s]), ph, abort_flag, a.status)) { ok = false; break; }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t sa = smem_u32(base + s * kStageBytesN), sb = sa + kRows * kBK * 4;
#pragma unroll
                for(int kk = 0; kk < kBK / 8; kk++) {
                    const int acc = (kt > 0 || kk > 0) ? 1 : 0;
                    const uint64_t are = sw128_desc(sa + kk * 32), aim = sw128_desc(sa + kBM * 128 + kk * 32);
                    const uint64_t bre = sw128_desc(sb + kk * 32), bim = sw128_desc(sb + kBM * 128 + kk * 32);
                    mma_tf32(d, are, bre, idesc, acc);
                    mma_tf32(d, aim, bim, idesc, 1);
                    mma_tf32(d + 128, aim, bre, idesc, acc);
                    mma_tf32(d + 128, are, bim, idesc_neg, 1);
                }
                mma_commit(smem_u32(&empty[s]));
            }
            if(ok) mma_commit(smem_u32(&accf[b]));
        }
        // every MMA issued has retired before the tensor memory is freed
        mma_commit(smem_u32(mdone));
        const unsigned long long t0 = gtime();
        while(!mbar_try(smem_u32(mdone), 0) && gtime() - t0 < kWaitNs) {}
    } else if(warp >= 4) {
        // ---- epilogue ----
        const unsigned et = threadIdx.x - 128u;  // = TMEM lane = row of the tile
        const uint32_t lane_addr = tmem + ((uint32_t)((warp & 3) * 32) << 16);
        for(unsigned lt = 0; lt < my_tiles; lt++) {
            unsigned I, J;
            tile_ij(blockIdx.x + lt * gridDim.x, I, J);
            const unsigned b = lt & 1u, aph = (lt >> 1) & 1u;
            bool ok = mbar_wait(smem_u32(&accf[b]), aph, abort_flag, a.status) && !*abort_flag;
            if(!bar_and(1, kEpiThreads, ok)) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const bool diag = I == J;
            const int y = (int)(a.t0 + I * kBM);
            for(int c = 0; c < kBM / 16; c++) {
                const unsigned cc = lt * (kBM / 16) + c;
                unsigned char* buf = chunks + (cc & 1u) * kChunkBytes;
                if(cc >= 2) {
                    if(et == 0) asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
                    bar_sync(1, kEpiThreads);
                }
                float re[16], im[16];
                tmem_ld16(lane_addr + b * 256u + c * 16, re);
                tmem_ld16(lane_addr + b * 256u + 128 + c * 16, im);
                unsigned char* row = buf + (size_t)et * 128;
#pragma unroll
                for(int u = 0; u < 8; u++) {
                    const int q0 = 2 * u, q1 = 2 * u + 1;
                    const bool z0 = diag && (unsigned)(c * 16 + q0) > et, z1 = diag && (unsigned)(c * 16 + q1) > et;
                    float4 v;
                    v.x = z0 ? 0.f : -re[q0];
                    v.y = z0 ? 0.f : -im[q0];
                    v.z = z1 ? 0.f : -re[q1];
                    v.w = z1 ? 0.f : -im[q1];
                    *reinterpret_cast<float4*>(row + ((u ^ (et & 7u)) << 4)) = v;
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                bar_sync(1, kEpiThreads);
                if(et == 0) {
                    tma_reduce_add_2d(&amap, (int)(2 * (a.t0 + J * kBM) + 32 * c), y, smem_u32(buf));
                    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
                }
            }
            // accumulator b is drained (every tcgen05.ld above waited for its data)
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            bar_sync(1, kEpiThreads);
            if(et == 0) mbar_arrive(smem_u32(&acce[b]));
        }
        if(et == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if(warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem));
}

}  // namespace

// Operand buffers: two (panel k uses buffer k % 2), each with its TMA descriptor, in the
// layout of one panel (rows [hi (64) | lo (64)], chol_map) or of a panel pair (rows
// [hi (128) | lo (128)], chol_pmap); a factorisation uses one layout, so both views share
// the memory. Rows past the trailing matrix only reach outputs past n, never written.
size_t pt_bytes_w(unsigned n, unsigned P) {
    return (size_t)((n + kBM - 1) / kBM) * kRows * (2 * P) * sizeof(float);
}
size_t pt_bytes(unsigned n) { return pt_bytes_w(n, kPanel); }

static void encode_pt(unsigned char* map, unsigned char* base, size_t bytes, unsigned P) {
    const size_t rows = bytes / (2 * P * sizeof(float));
    const cuuint64_t dims[2] = {(cuuint64_t)(2 * P), (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)(2 * P * sizeof(float))};
    const cuuint32_t box[2] = {kBK, kRows};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = encode_fn()(reinterpret_cast<CUtensorMap*>(map), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims,
                                   strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if(r != CUDA_SUCCESS) throw Error(ANN_ERR_CUDA, "cuTensorMapEncodeTiled failed (Cholesky panel operand)");
}

// (the clear is ordered on the solve's stream: a plain cudaMemset goes to the legacy default
// stream, which does not order with the non-blocking streams the solves run on)
void chol_update_tc_prepare(ann_tdvp_impl& td, unsigned n, cudaStream_t st) {
    const size_t b1 = pt_bytes_w(n, kPanel), b2 = pt_bytes_w(n, 2 * kPanel);
    if(td.chol_pt.bytes >= 2 * b2 && td.chol_pt_n == n) return;
    td.chol_pt.ensure(2 * b2);
    ANN_CUDA(cudaMemsetAsync(td.chol_pt.p, 0, 2 * b2, st));
    td.chol_pt_n = n;
    for(int b = 0; b < 2; b++) {
        encode_pt(td.chol_map[b], td.chol_pt.as<unsigned char>() + b * b1, b1, kPanel);
        encode_pt(td.chol_pmap[b], td.chol_pt.as<unsigned char>() + b * b2, b2, 2 * kPanel);
    }
    static bool attr = false;
    if(!attr) {
        ANN_CUDA(cudaFuncSetAttribute(chol_update_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      kSmemBytes));
        ANN_CUDA(cudaFuncSetAttribute(chol_update_tc3_kernel<kPanel>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      kSmem3Bytes));
        ANN_CUDA(cudaFuncSetAttribute(chol_update_tc3_kernel<2 * kPanel>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem3Bytes));
        attr = true;
    }
}

// TMA descriptor of the FP32 factor A (n x n complex64 = n rows of 2n floats) for the
// reduce-add epilogue; needs 16-byte row pitch, i.e. n even
bool chol_update_tc_bind(ann_tdvp_impl& td, cplx<float>* A, unsigned n) {
    td.chol_reduce = 0;
    if(n & 1u) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)2 * n, (cuuint64_t)n};
    const cuuint64_t strides[1] = {(cuuint64_t)2 * n * sizeof(float)};
    const cuuint32_t box[2] = {32, kBM};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = encode_fn()(reinterpret_cast<CUtensorMap*>(td.chol_amap), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                                   A, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                   CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if(r != CUDA_SUCCESS) return false;
    td.chol_reduce = 1;
    return true;
}

float* chol_update_tc_operand(ann_tdvp_impl& td, unsigned buf) {
    return reinterpret_cast<float*>(td.chol_pt.as<unsigned char>() + buf * pt_bytes_w(td.chol_pt_n, kPanel));
}

float* chol_update_tc_pair_operand(ann_tdvp_impl& td, unsigned buf) {
    return reinterpret_cast<float*>(td.chol_pt.as<unsigned char>() + buf * pt_bytes_w(td.chol_pt_n, 2 * kPanel));
}

// Persistent launch of the reduce-add update (n even). More than a wave: persistent CTAs,
// the epilogue of one tile under the MMAs of the next; a few SMs stay free for the next
// panel (potrf32 / trsm32 on the side stream), which otherwise only gets the resources
// left beside the persistent CTAs and runs several times slower (the panel is the
// critical path of the factorisation). Up to a wave: one tile per CTA, still with the
// two-stage pipeline.
template<int P>
static void launch_tc3(const CUtensorMap& pmap, const CUtensorMap& amap, const UpdArgs& a, unsigned tiles, unsigned n,
                       cudaStream_t st) {
    static int sms = 0;
    if(!sms) {
        int dev = 0;
        ANN_CUDA(cudaGetDevice(&dev));
        ANN_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    }
    const int reserve = std::min(tuning_get(key_chol_reserve(n), 32), sms / 2);
    const unsigned grid = tiles > (unsigned)sms ? (unsigned)(sms - reserve) : tiles;
    chol_update_tc3_kernel<P><<<grid, 256, kSmem3Bytes, st>>>(pmap, amap, a, tiles);
    check_launch("chol_update_tc3_kernel");
}

// A22 -= X X^H on tiles (I, 0) (col_only) or (I, J >= 1) of the trailing matrix of panel kb
void chol_update_tc(ann_tdvp_impl& td, cplx<float>* A, unsigned n, unsigned kb, bool col_only, unsigned* status,
                    cudaStream_t st) {
    const unsigned t0 = kb + kPanel;
    const unsigned m = n - t0;
    const unsigned T = (m + kBM - 1) / kBM;
    const unsigned tiles = col_only ? T : T * (T - 1) / 2;
    if(tiles == 0) return;
    UpdArgs a{A, n, t0, col_only ? 1 : 0, td.chol_reduce, status};
    const CUtensorMap& pmap = *reinterpret_cast<const CUtensorMap*>(td.chol_map[(kb / kPanel) & 1u]);
    const CUtensorMap& amap = *reinterpret_cast<const CUtensorMap*>(td.chol_amap);
    if(td.chol_reduce) {
        launch_tc3<kPanel>(pmap, amap, a, tiles, n, st);
        return;
    }
    chol_update_tc_kernel<<<tiles, 128, kSmemBytes, st>>>(pmap, amap, a);
    check_launch("chol_update_tc_kernel");
}

// The same with K = 128 from the panel pair at columns pb .. pb + 127 (operand buffer
// (pb / 128) % 2); the reduce-add epilogue only (n even)
void chol_update_tc_pair(ann_tdvp_impl& td, cplx<float>* A, unsigned n, unsigned pb, bool col_only, unsigned* status,
                         cudaStream_t st) {
    if(!td.chol_reduce) throw Error(ANN_ERR_INVALID, "panel-pair update needs the reduce-add epilogue (n even)");
    const unsigned t0 = pb + 2 * kPanel;
    if(t0 >= n) return;
    const unsigned T = (n - t0 + kBM - 1) / kBM;
    const unsigned tiles = col_only ? T : T * (T - 1) / 2;
    if(tiles == 0) return;
    UpdArgs a{A, n, t0, col_only ? 1 : 0, 1, status};
    const CUtensorMap& pmap = *reinterpret_cast<const CUtensorMap*>(td.chol_pmap[(pb / (2 * kPanel)) & 1u]);
    const CUtensorMap& amap = *reinterpret_cast<const CUtensorMap*>(td.chol_amap);
    launch_tc3<2 * kPanel>(pmap, amap, a, tiles, n, st);
}

}  // namespace ann
