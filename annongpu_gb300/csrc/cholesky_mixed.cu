// Mixed-precision SR solve: (S + shift I) delta = F with the factorisation in
// FP32 and the answer refined against the FP64 matrix until its FP64 residual
// reaches a tolerance.
//
//   1. A32 = (complex64) (S + shift I), lower triangle.
//   2. Blocked right-looking complex Cholesky of A32 (panel width NB = 64, the
//      next panel factorised on a side stream while the trailing update runs).
//      Each diagonal block also stores its explicit inverse, so the panel solve
//      and every later triangular solve multiply by it instead of substituting.
//   3. x = 0, r = F; repeat: c = (L L^H)^{-1} r in FP32, x += c in FP64,
//      r = F - (S + shift I) x in FP64, until ||r|| / ||F|| <= tol or max_iter.
//      When S holds FP32 values in complex64 (the tensor-core HERK's sums), S x is
//      formed on the FP32 pipe in double-float arithmetic (below) until ||r|| / ||F||
//      falls to 1e-10, then in FP64 (whose 53 bits the last steps need).
//
// The iteration is classical mixed-precision iterative refinement (Wilkinson;
// Moler 1967; analysed by Higham, "Accuracy and Stability of Numerical
// Algorithms", ch. 12): it converges to the FP64 solution whenever
// cond(S + shift I) * u_fp32 < 1, and every step costs two FP32 triangular
// solves and one FP64 matrix-vector product. Convergence is decided on the
// device (a flag that later kernels of the same solve read), so the whole
// solve is a fixed launch sequence that a CUDA graph can hold.
//
// The reference has no solver (source/network_functions/TDVP.cu.template:181-302
// builds S and F; the caller solves). This file is the project's own.
#include <algorithm>
#include <cmath>

#include "ann_internal.hpp"

namespace ann {

namespace {

constexpr int NB = 64;     // panel / diagonal block width
constexpr int UT = 64;     // trailing-update tile (== NB: tile column 0 is the next panel)

using cf = cplx<float>;
using zc = cplx<double>;

// lower triangle of S + shift I in complex64, row-major n x n. CTA b converts rows b and
// n - 1 - b (n + 1 entries together, so every CTA has the same work).
__device__ __forceinline__ zc to_zc(zc v) { return v; }
__device__ __forceinline__ zc to_zc(cf v) { return mk(widen(v.re), widen(v.im)); }

template<typename TS>
__global__ void __launch_bounds__(256) cvt_shift_kernel(const TS* __restrict__ S, cf* __restrict__ A, unsigned n,
                                                        double shift) {
    const unsigned rows[2] = {blockIdx.x, n - 1u - blockIdx.x};
    for(int h = 0; h < 2; h++) {
        const unsigned i = rows[h];
        if(h == 1 && i == rows[0]) break;
        const TS* Si = S + (size_t)i * n;
        cf* Ai = A + (size_t)i * n;
        unsigned j = threadIdx.x;
        // four loads in flight per thread; off the diagonal a complex64 S is copied as is
        // (narrow(widen(v)) == v), the diagonal gets the shift in FP64 and one rounding
        for(; j + 768u <= i; j += 1024u) {
            TS v[4];
#pragma unroll
            for(int q = 0; q < 4; q++) v[q] = Si[j + 256u * q];
#pragma unroll
            for(int q = 0; q < 4; q++) {
                const unsigned jj = j + 256u * q;
                zc w = to_zc(v[q]);
                if(jj == i) w.re += shift;
                Ai[jj] = mk(narrow(w.re), narrow(w.im));
            }
        }
        for(; j <= i; j += 256u) {
            zc w = to_zc(Si[j]);
            if(j == i) w.re += shift;
            Ai[j] = mk(narrow(w.re), narrow(w.im));
        }
    }
}

// Cholesky of the nb x nb diagonal block at (kb, kb), factor only (the critical path of
// the factorisation; the inverses of the diagonal blocks are formed afterwards by
// diag_inv_kernel). Blocked in four 16-column panels on the block held in shared
// memory. A panel (rows kk.. of columns kk..kk+15) is factorised in registers with
// one row per lane: lanes 0-15 of every warp hold the 16 diagonal rows (each warp
// factorises them redundantly, so no warp waits on another) and lanes 16-31 hold 16 of
// the rows below. Column j of the panel is then
//   l_jj = a_jj rsqrt(a_jj), l_rj = a_rj rsqrt(a_jj), a_rc -= l_rj conj(l_cj) (c = j+1..15),
// with l_cj broadcast by shuffle from lane c. Every lane applies every column update
// (the entries above the diagonal of the panel block are never read back), so the
// updates of one column carry no branch and overlap; the chain per column is one
// shuffle, the reciprocal square root, one shuffle and one complex multiply-add. The
// 16-column trailing update of the rest of the block runs on all threads in 2 x 2
// register tiles; two barriers per panel.
constexpr int kPotrfThreads = 256;
constexpr int kPw = 16;  // panel width
constexpr unsigned kNoPrev = 0xFFFFFFFFu;
// dynamic shared memory of potrf32_kernel (two 64 x 65 complex blocks) and trsm32_kernel (one)
constexpr size_t kPotrfSmem = 2 * NB * (NB + 1) * sizeof(cf);
constexpr size_t kTrsmSmem = NB * (NB + 1) * sizeof(cf);

// The panel kernels run as programmatic dependent launches (sm_90+ griddepcontrol): a
// kernel launched with cudaLaunchAttributeProgrammaticStreamSerialization may start while
// the kernel before it on the stream still runs, and loads what does not depend on that
// kernel (its own rows, the pending update of the panel pair) in the meantime. pdl_wait()
// returns once the kernel before has completed and its writes are visible (at once for a
// kernel launched without the attribute); pdl_trigger() lets the next kernel start.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// With prev != kNoPrev the block first receives the rank-64 update of the panel at columns
// prev (the first panel of a pair: a_rc -= sum_k l_rk conj(l_ck) over its 64 columns),
// which the pair form applies here and in trsm32_kernel instead of a separate launch.
// The diagonal block is read before pdl_wait() (nothing before this kernel on its stream
// writes it: the panel at prev writes only its own columns); the rows at prev after it.
// The trigger follows the wait, so a kernel started by it finds the kernel before this
// one completed as well.
__global__ void __launch_bounds__(kPotrfThreads) potrf32_kernel(cf* __restrict__ A, unsigned n, unsigned kb,
                                                                unsigned* status, unsigned prev) {
    extern __shared__ float4 panel_smem[];
    cf (*a)[NB + 1] = reinterpret_cast<cf (*)[NB + 1]>(panel_smem);
    cf (*w)[NB + 1] = reinterpret_cast<cf (*)[NB + 1]>(reinterpret_cast<cf*>(panel_smem) + NB * (NB + 1));
    const unsigned nb = min((unsigned)NB, n - kb);
    const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    {
        cf v[NB * NB / kPotrfThreads];
#pragma unroll
        for(int q = 0; q < NB * NB / kPotrfThreads; q++) {
            const unsigned t = tid + q * kPotrfThreads, r = t / NB, c = t % NB;
            v[q] = (r < nb && c <= r) ? A[(size_t)(kb + r) * n + kb + c] : mk(r == c ? 1.f : 0.f, 0.f);
        }
#pragma unroll
        for(int q = 0; q < NB * NB / kPotrfThreads; q++) {
            const unsigned t = tid + q * kPotrfThreads;
            a[t / NB][t % NB] = v[q];
        }
        pdl_wait();
        pdl_trigger();
        if(prev != kNoPrev) {
#pragma unroll
            for(int q = 0; q < NB * NB / kPotrfThreads; q++) {
                const unsigned t = tid + q * kPotrfThreads, r = t / NB, k = t % NB;
                w[r][k] = r < nb ? A[(size_t)(kb + r) * n + prev + k] : mk(0.f, 0.f);
            }
        }
    }
    __syncthreads();
    if(prev != kNoPrev) {
        // a_rc -= sum_k w_rk conj(w_ck) on the lower triangle, in 4 x 4 register tiles
        // (rows 4 ty .. 4 ty + 3, columns 4 tx .. 4 tx + 3; tiles above the diagonal idle)
        const unsigned tx = tid & 15u, ty = tid >> 4;
        if(tx <= ty) {
            cf acc[4][4];
#pragma unroll
            for(int i = 0; i < 4; i++)
#pragma unroll
                for(int j = 0; j < 4; j++) acc[i][j] = mk(0.f, 0.f);
#pragma unroll 4
            for(int k = 0; k < NB; k++) {
                cf wr[4], wc[4];
#pragma unroll
                for(int i = 0; i < 4; i++) wr[i] = w[4 * ty + i][k];
#pragma unroll
                for(int j = 0; j < 4; j++) wc[j] = w[4 * tx + j][k];
#pragma unroll
                for(int i = 0; i < 4; i++)
#pragma unroll
                    for(int j = 0; j < 4; j++) cmac_conj(acc[i][j], wc[j], wr[i]);  // += w_rk conj(w_ck)
            }
#pragma unroll
            for(int i = 0; i < 4; i++)
#pragma unroll
                for(int j = 0; j < 4; j++) {
                    const unsigned r = 4 * ty + i, c = 4 * tx + j;
                    if(c <= r) a[r][c] = a[r][c] - acc[i][j];
                }
        }
        __syncthreads();
    }
#pragma unroll 1
    for(unsigned kk = 0; kk < NB; kk += kPw) {
        const unsigned below = NB - kk - kPw;                       // rows under the panel's diagonal block
        const unsigned nwp = below ? (below + kPw - 1) / kPw : 1u;  // warps on the panel
        // lane < 16: diagonal row kk + lane; lane >= 16: row kk + 16 + 16 warp + lane - 16
        const bool diag = lane < kPw;
        const unsigned r = diag ? kk + lane : kk + kPw + warp * kPw + (lane - kPw);
        const bool live = warp < nwp && r < NB;
        cf x[kPw];
#pragma unroll
        for(int c = 0; c < kPw; c++) x[c] = live ? a[r][kk + c] : mk(0.f, 0.f);
        // every warp holds its copy of the diagonal rows before warp 0 writes them back
        __syncthreads();
        if(warp < nwp) {
#pragma unroll
            for(int j = 0; j < kPw; j++) {
                float d = __shfl_sync(0xffffffffu, x[j].re, j);
                if(!(d > 0.f) || !isfinite(d)) {
                    if(tid == 0) atomicOr(status, kStatusNotPosDef);
                    d = 1.f;
                }
                const float inv = rsqrtf(d), s = d * inv;
                x[j] = (diag && lane == (unsigned)j) ? mk(s, 0.f) : inv * x[j];
                const cf nx = -x[j];
#pragma unroll
                for(int c = 1; c < kPw; c++) {  // constant bounds, so that both loops unroll
                    if(c <= j) continue;
                    cf l;
                    l.re = __shfl_sync(0xffffffffu, x[j].re, c);
                    l.im = __shfl_sync(0xffffffffu, x[j].im, c);
                    cmac_conj(x[c], l, nx);  // -= l_rj conj(l_cj)
                }
            }
            if(live && (!diag || warp == 0)) {
#pragma unroll
                for(int c = 0; c < kPw; c++)
                    if(!diag || (unsigned)c <= lane) a[r][kk + c] = x[c];
            }
        }
        __syncthreads();
        if(below) {
            // a_rc -= sum_p l_rp conj(l_cp) for kk + 16 <= c <= r < NB, in 2 x 2 tiles
            const unsigned t2 = below / 2, tiles = t2 * (t2 + 1) / 2, base = kk + kPw;
            for(unsigned q = tid; q < tiles; q += kPotrfThreads) {
                // tile q -> (ti, tj), tj <= ti, row-major over the lower triangle of tiles
                unsigned ti = (unsigned)((sqrtf(8.f * q + 1.f) - 1.f) * 0.5f);
                while(ti * (ti + 1) / 2 > q) ti--;
                while((ti + 1) * (ti + 2) / 2 <= q) ti++;
                const unsigned tj = q - ti * (ti + 1) / 2;
                const unsigned r0 = base + 2 * ti, c0 = base + 2 * tj;
                cf s00 = mk(0.f, 0.f), s01 = s00, s10 = s00, s11 = s00;
#pragma unroll
                for(int p = 0; p < kPw; p++) {
                    const cf xr0 = a[r0][kk + p], xr1 = a[r0 + 1][kk + p];
                    const cf xc0 = a[c0][kk + p], xc1 = a[c0 + 1][kk + p];
                    cmac_conj(s00, xc0, xr0);
                    cmac_conj(s01, xc1, xr0);
                    cmac_conj(s10, xc0, xr1);
                    cmac_conj(s11, xc1, xr1);
                }
                a[r0][c0] = a[r0][c0] - s00;
                if(ti != tj) a[r0][c0 + 1] = a[r0][c0 + 1] - s01;
                a[r0 + 1][c0] = a[r0 + 1][c0] - s10;
                a[r0 + 1][c0 + 1] = a[r0 + 1][c0 + 1] - s11;
            }
            __syncthreads();
        }
    }
    for(unsigned t = tid; t < NB * NB; t += kPotrfThreads) {
        const unsigned r = t / NB, c = t % NB;
        if(r < nb && c <= r) A[(size_t)(kb + r) * n + kb + c] = a[r][c];
    }
}

// inverse of every diagonal block of the factor (one CTA per block, 16 threads per
// column c): X[i][c] = (delta_ic - sum_{c <= p < i} L[i][p] X[p][c]) / L[i][i];
// Dinv[blk] = L_kk^{-1}, DinvH[blk] = L_kk^{-H} (row-major NB x NB, identity beyond nb)
__global__ void __launch_bounds__(1024) diag_inv_kernel(const cf* __restrict__ A, unsigned n, cf* __restrict__ Dinv,
                                                        cf* __restrict__ DinvH) {
    extern __shared__ float4 smem_raw[];
    cf (*Ls)[NB + 1] = reinterpret_cast<cf (*)[NB + 1]>(smem_raw);
    cf (*x)[NB + 1] = reinterpret_cast<cf (*)[NB + 1]>(reinterpret_cast<cf*>(smem_raw) + NB * (NB + 1));
    const unsigned kb = blockIdx.x * NB, nb = min((unsigned)NB, n - kb);
    const unsigned tid = threadIdx.x;
    for(unsigned t = tid; t < NB * NB; t += blockDim.x) {
        const unsigned r = t / NB, c = t % NB;
        Ls[r][c] = (r < nb && c <= r) ? A[(size_t)(kb + r) * n + kb + c] : mk(r == c ? 1.f : 0.f, 0.f);
        x[r][c] = mk(0.f, 0.f);
    }
    __syncthreads();
    {
        const unsigned c = tid >> 4, s = tid & 15u;
        const unsigned i0 = c & ~1u;  // both groups of a warp walk the same rows
        for(unsigned i = i0; i < NB; i++) {
            cf part = mk(0.f, 0.f);
            for(unsigned p = i0 + s; p < i; p += 16) cmac(part, Ls[i][p], x[p][c]);
#pragma unroll
            for(int o = 8; o > 0; o >>= 1) {
                part.re += __shfl_xor_sync(0xffffffffu, part.re, o, 16);
                part.im += __shfl_xor_sync(0xffffffffu, part.im, o, 16);
            }
            if(s == 0) {
                const float inv = 1.f / Ls[i][i].re;
                const float dre = (i == c) ? 1.f : 0.f;
                x[i][c] = mk(inv * (dre - part.re), -inv * part.im);
            }
            __syncwarp();
        }
    }
    __syncthreads();
    const size_t blk = blockIdx.x;
    for(unsigned t = tid; t < NB * NB; t += blockDim.x) {
        const unsigned r = t / NB, c = t % NB;
        Dinv[blk * NB * NB + t] = x[r][c];
        DinvH[blk * NB * NB + t] = conj(x[c][r]);
    }
}

constexpr unsigned kTrsmRows = 16;  // rows per CTA: many short CTAs, the panel is on the critical path

// rows below the diagonal block: X <- X L_kk^{-H} by substitution, one warp per two rows,
// lane owning columns lane and lane + 32: for c = 0..63 the owner finalises
//   x_c = (x_c - sum_{p<c} x_p conj(L_cp)) / L_cc,
// broadcasts it, and the lanes subtract x_c conj(L_qc) from their columns q > c.
// L_kk (just factorised) is staged transposed in shared memory: Lt[c][q] = L_qc.
__device__ __forceinline__ float tf32_round(float x) {
    uint32_t u;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(u) : "f"(x));
    return __uint_as_float(u);
}

// The panel rows are also the operand of the next tensor-core trailing update: with
// PT != null each row from global row pt_row0 on is written there as well, split into
// TF32 hi and lo (the layout of chol_update_tc.cu: per 128-row block of the rows from
// pt_row0, [Re rows ; Im rows], each row [hi (w/2) | lo (w/2)] floats; the panel's 64
// columns at pt_col0 of each half: w = 128 for one panel, 256 for a panel pair).
struct PtDst {
    float* PT;
    unsigned row0, col0, w;
};

__device__ __forceinline__ void put_tf32(const PtDst& d, size_t i, unsigned p, cf v) {
    const size_t blk = i / 128, r = i % 128;
    float* re = d.PT + (blk * 256 + r) * d.w + d.col0;
    float* im = d.PT + (blk * 256 + 128 + r) * d.w + d.col0;
    const unsigned lo = d.w / 2;
    const float hr = tf32_round(v.re), hi = tf32_round(v.im);
    re[p] = hr;
    re[lo + p] = tf32_round(v.re - hr);
    im[p] = hi;
    im[lo + p] = tf32_round(v.im - hi);
}

__global__ void __launch_bounds__(256) trsm32_kernel(cf* __restrict__ A, unsigned n, unsigned kb, PtDst pt,
                                                     unsigned prev) {
    // one 64 x 65 buffer: first W (the previous panel's factor rows of this block, for the
    // pending update), then L_kk transposed; 33 KB per CTA keeps six CTAs per SM
    extern __shared__ float4 panel_smem[];
    cf (*Lt)[NB + 1] = reinterpret_cast<cf (*)[NB + 1]>(panel_smem);
    cf (*W)[NB + 1] = Lt;
    __shared__ float inv_d[NB];
    // Started as a programmatic dependent launch after potrf32_kernel of this panel: the
    // rows and the pending update (the pair's first panel, completed before the potrf32
    // launch that started this kernel released it) are read before pdl_wait(), L_kk after.
    pdl_trigger();
    const unsigned nbk = min((unsigned)NB, n - kb);
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const size_t row0 = (size_t)kb + NB + (size_t)blockIdx.x * kTrsmRows;
    // each warp solves its two rows (warp, warp + 8) side by side: two independent chains
    static_assert(kTrsmRows == 16, "two rows per warp of eight");
    const size_t ra = row0 + warp, rb = row0 + warp + 8;
    const bool has_a = ra < n, has_b = rb < n;
    cf* Xa = A + (has_a ? ra : kb) * n + kb;
    cf* Xb = A + (has_b ? rb : (has_a ? ra : kb)) * n + kb;
    cf a0 = mk(0.f, 0.f), a1 = a0, b0 = a0, b1 = a0;
    if(has_a) {
        a0 = Xa[lane];
        a1 = Xa[lane + 32];
        b0 = Xb[lane];
        b1 = Xb[lane + 32];
    }
    if(prev != kNoPrev) {
        for(unsigned t = threadIdx.x; t < NB * NB; t += blockDim.x) {
            const unsigned q = t / NB, c = t % NB;
            W[q][c] = q < nbk ? A[(size_t)(kb + q) * n + prev + c] : mk(0.f, 0.f);
        }
        __syncthreads();
    }
    if(prev != kNoPrev && has_a) {
        // the previous panel's rank-64 update of these rows: x_q -= sum_k p_k conj(W[q][k]),
        // p = the row's factor entries in that panel, broadcast from lane k % 32
        const cf* Pa = A + ra * n + prev;
        const cf* Pb = A + (has_b ? rb : ra) * n + prev;
        const cf pa0 = Pa[lane], pa1 = Pa[lane + 32], pb0 = Pb[lane], pb1 = Pb[lane + 32];
#pragma unroll 8
        for(int k = 0; k < NB; k++) {
            const cf sa = k < 32 ? pa0 : pa1, sb = k < 32 ? pb0 : pb1;
            cf pa, pb;
            pa.re = __shfl_sync(0xffffffffu, sa.re, k & 31);
            pa.im = __shfl_sync(0xffffffffu, sa.im, k & 31);
            pb.re = __shfl_sync(0xffffffffu, sb.re, k & 31);
            pb.im = __shfl_sync(0xffffffffu, sb.im, k & 31);
            const cf w0 = W[lane][k], w1 = W[lane + 32][k];
            cmac_conj(a0, w0, -pa);  // -= p_k conj(W[q][k])
            cmac_conj(a1, w1, -pa);
            cmac_conj(b0, w0, -pb);
            cmac_conj(b1, w1, -pb);
        }
    }
    if(prev != kNoPrev) __syncthreads();  // W is read; the buffer takes L_kk next
    pdl_wait();
    for(unsigned t = threadIdx.x; t < NB * NB; t += blockDim.x) {
        const unsigned q = t / NB, c = t % NB;  // element (q, c) of L_kk
        Lt[c][q] = c <= q ? A[(size_t)(kb + q) * n + kb + c] : mk(0.f, 0.f);
    }
    __syncthreads();
    if(threadIdx.x < NB) inv_d[threadIdx.x] = 1.f / Lt[threadIdx.x][threadIdx.x].re;
    __syncthreads();
    if(!has_a) return;
#pragma unroll 8
    for(unsigned c = 0; c < 32; c++) {
        cf xa, xb;
        xa.re = __shfl_sync(0xffffffffu, a0.re, c);
        xa.im = __shfl_sync(0xffffffffu, a0.im, c);
        xb.re = __shfl_sync(0xffffffffu, b0.re, c);
        xb.im = __shfl_sync(0xffffffffu, b0.im, c);
        const float id = inv_d[c];
        xa = id * xa;
        xb = id * xb;
        const cf l0 = Lt[c][lane], l1 = Lt[c][lane + 32];
        // lane c takes x_c, lanes above subtract x_c conj(L_qc), lanes below keep their
        // finished values: selects, not branches, so consecutive columns overlap
        cf ua = a0, ub = b0;
        cmac_conj(ua, l0, -xa);
        cmac_conj(ub, l0, -xb);
        a0 = lane == c ? xa : (lane > c ? ua : a0);
        b0 = lane == c ? xb : (lane > c ? ub : b0);
        cmac_conj(a1, l1, -xa);
        cmac_conj(b1, l1, -xb);
    }
#pragma unroll 8
    for(unsigned c = 32; c < NB; c++) {
        cf xa, xb;
        xa.re = __shfl_sync(0xffffffffu, a1.re, c - 32);
        xa.im = __shfl_sync(0xffffffffu, a1.im, c - 32);
        xb.re = __shfl_sync(0xffffffffu, b1.re, c - 32);
        xb.im = __shfl_sync(0xffffffffu, b1.im, c - 32);
        const float id = inv_d[c];
        xa = id * xa;
        xb = id * xb;
        const cf l1 = Lt[c][lane + 32];
        cf ua = a1, ub = b1;
        cmac_conj(ua, l1, -xa);
        cmac_conj(ub, l1, -xb);
        a1 = lane + 32 == c ? xa : (lane + 32 > c ? ua : a1);
        b1 = lane + 32 == c ? xb : (lane + 32 > c ? ub : b1);
    }
    Xa[lane] = a0;
    Xa[lane + 32] = a1;
    if(pt.PT && ra >= pt.row0) {
        put_tf32(pt, ra - pt.row0, lane, a0);
        put_tf32(pt, ra - pt.row0, lane + 32, a1);
    }
    if(has_b) {
        Xb[lane] = b0;
        Xb[lane + 32] = b1;
        if(pt.PT && rb >= pt.row0) {
            put_tf32(pt, rb - pt.row0, lane, b0);
            put_tf32(pt, rb - pt.row0, lane + 32, b1);
        }
    }
}

// trailing lower triangle: A[i][j] -= sum_p X[i][p] conj(X[j][p]), i >= j >= kb + nb,
// X = A[:, kb : kb + nb]. 64 x 64 tiles, 256 threads with 4 x 4 complex each, the
// whole K = nb panel slice of both tile rows in shared memory (transposed).
// col_only: tile column 0 (it holds the next panel); otherwise tiles with column >= 1.
__global__ void __launch_bounds__(256) herk32_kernel(cf* __restrict__ A, unsigned n, unsigned kb, unsigned nb,
                                                     int col_only) {
    extern __shared__ float4 smem_raw[];
    cf (*Xi)[UT + 1] = reinterpret_cast<cf (*)[UT + 1]>(smem_raw);
    cf (*Xj)[UT + 1] = reinterpret_cast<cf (*)[UT + 1]>(reinterpret_cast<cf*>(smem_raw) + NB * (UT + 1));
    const unsigned t0 = kb + nb;
    unsigned ti, tj;
    if(col_only) {
        ti = blockIdx.x;
        tj = 0;
    } else {
        unsigned b = blockIdx.x;
        ti = 0;
        while(b > ti) { b -= ti + 1; ti++; }
        tj = b + 1;
        ti += 1;
    }
    const unsigned i0 = t0 + ti * UT, j0 = t0 + tj * UT;
    // load: thread q reads element p = q % 64 of row q / 64 (+4 rows per pass), coalesced
    for(unsigned q = threadIdx.x; q < UT * NB; q += 256) {
        const unsigned rr = q / NB, pp = q % NB;
        const unsigned gi = i0 + rr, gj = j0 + rr;
        Xi[pp][rr] = (gi < n && pp < nb) ? A[(size_t)gi * n + kb + pp] : mk(0.f, 0.f);
        Xj[pp][rr] = (gj < n && pp < nb) ? A[(size_t)gj * n + kb + pp] : mk(0.f, 0.f);
    }
    __syncthreads();
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    cf acc[4][4];
#pragma unroll
    for(int i = 0; i < 4; i++)
#pragma unroll
        for(int j = 0; j < 4; j++) acc[i][j] = mk(0.f, 0.f);
#pragma unroll 4
    for(int p = 0; p < NB; p++) {
        cf xa[4], xb[4];
#pragma unroll
        for(int i = 0; i < 4; i++) xa[i] = Xi[p][ty + 16 * i];
#pragma unroll
        for(int j = 0; j < 4; j++) xb[j] = Xj[p][tx + 16 * j];
#pragma unroll
        for(int i = 0; i < 4; i++)
#pragma unroll
            for(int j = 0; j < 4; j++) cmac_conj(acc[i][j], xb[j], xa[i]);  // += xa conj(xb)
    }
#pragma unroll
    for(int i = 0; i < 4; i++) {
        const unsigned gi = i0 + ty + 16 * i;
        if(gi >= n) continue;
#pragma unroll
        for(int j = 0; j < 4; j++) {
            const unsigned gj = j0 + tx + 16 * j;
            if(gj >= n || gj > gi) continue;
            cf& dst = A[(size_t)gi * n + gj];
            dst = dst - acc[i][j];
        }
    }
}

// ---- refinement ------------------------------------------------------------------
struct IrState {
    int done;        // set once ||r|| / ||F|| <= tol; later kernels of the solve return at once
    int iters;       // FP32 solves applied (the first one and the corrections)
    int stalled;     // max_iter reached above tol
    unsigned notpd;  // a pivot of the FP32 factorisation was <= 0 or not finite
    double first;    // ||r|| / ||F|| after the first solve
    double last;     // ... after the last one
};

__device__ __forceinline__ unsigned long long gtime() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

constexpr unsigned long long kWaitNs = 1000000000ull;  // 1 s per wait on a solution block
constexpr int kSolveThreads = 512;
constexpr size_t kSolveSyncHead = 16;  // abort flag, padded to the 16-byte alignment of the tagged blocks

// Solution blocks pass between the CTAs of a solve as self-validating words: one
// 64-bit word per float holds its bits in the low half and a ready tag in the high
// half (the "low-latency" protocol of NCCL's LL transport). A 64-bit access is
// single-copy atomic, so a reader that sees the tag also sees the value: a block
// reaches its consumers in one L2 round trip, with no fence and no separate flag
// to poll. The buffers are zeroed (tag 0) before every launch.
constexpr unsigned long long kReadyTag = 1ull << 32;

__device__ __forceinline__ void st_ll(ulonglong2* p, cf v) {
    const unsigned long long w0 = kReadyTag | __float_as_uint(v.re);
    const unsigned long long w1 = kReadyTag | __float_as_uint(v.im);
    asm volatile("st.relaxed.gpu.global.v2.u64 [%0], {%1, %2};" ::"l"(p), "l"(w0), "l"(w1) : "memory");
}

__device__ __forceinline__ bool ld_ll(const ulonglong2* p, cf& v) {
    unsigned long long w0, w1;
    asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(w0), "=l"(w1) : "l"(p) : "memory");
    v = mk(__uint_as_float((unsigned)w0), __uint_as_float((unsigned)w1));
    return (w0 >> 32) == 1ull && (w1 >> 32) == 1ull;
}

// Thread t < NB reads entry t of a published solution block into v[t], waiting until
// it carries the ready tag. Bounded: after kWaitNs the thread raises kStatusTimeout
// and the abort flag, and every CTA of the solve gives up at its next wait. Returns
// false, for the whole CTA, when the solve is being abandoned; on true, v is
// visible to every thread of the CTA.
__device__ bool wait_block(const ulonglong2* blk, cf* v, int* abort_flag, unsigned* status) {
    int bad = 0;
    const unsigned t = threadIdx.x;
    if(t < NB) {
        cf val;
        if(!ld_ll(blk + t, val)) {
            const unsigned long long t0 = gtime();
            for(unsigned it = 1;; it++) {
                if(ld_ll(blk + t, val)) break;
                if((it & 15u) == 0) {
                    if(*(volatile int*)abort_flag) { bad = 1; break; }
                    if(gtime() - t0 > kWaitNs) {
                        atomicExch(abort_flag, 1);
                        atomicOr(status, kStatusTimeout);
                        bad = 1;
                        break;
                    }
                }
            }
        }
        v[t] = val;
    }
    return __syncthreads_or(bad) == 0;
}

// y = D x for a diagonal block held in shared memory (D[c][p], rows padded to kDs):
// output c by eight threads (t = 8 c + part), part summing columns part, part + 8, ...,
// then three shuffle levels; 512 threads. The padding (kDs = NB + 8) puts the two rows a
// half-warp reads on different banks.
constexpr int kDs = NB + 8;
__device__ __forceinline__ void block_apply_sm(const cf (*D)[kDs], const cf* __restrict__ x, cf* y, unsigned nb) {
    const unsigned c = threadIdx.x >> 3, part = threadIdx.x & 7u;
    cf acc = mk(0.f, 0.f);
#pragma unroll
    for(int q = 0; q < NB / 8; q++) cmac(acc, D[c][part + 8 * q], x[part + 8 * q]);
#pragma unroll
    for(int o = 1; o < 8; o <<= 1) {
        acc.re += __shfl_xor_sync(0xffffffffu, acc.re, o);
        acc.im += __shfl_xor_sync(0xffffffffu, acc.im, o);
    }
    if(part == 0) y[c] = c < nb ? acc : mk(0.f, 0.f);
}

// b <- (L L^H)^{-1} b in one cooperative launch without grid barriers. CTA g owns the
// block rows j = g, g + G, ... (G CTAs, all resident). Forward: y_j = L_jj^{-1} (b_j -
// sum_{k<j} L_jk y_k), adding each y_k as soon as it is published. Backward:
// x_j = L_jj^{-H} (y_j - sum_{k>j} L_kj^H x_k), blocks taken from the last. Every
// thread adds its contributions in a fixed order, so the result is bit-reproducible.
// The critical path is the chain of published blocks, so everything that does not
// depend on the awaited block (the next L block, the inverted diagonal block) is
// loaded before the wait; the awaited block lands in one of two shared buffers in
// turn, so one barrier per block suffices.
// ll: [nblk * NB] forward blocks y, then [nblk * NB] backward blocks x, as tagged
// words; abort_flag: one int. All zero on entry. Entries past n are published as 0.
__global__ void __launch_bounds__(kSolveThreads) trsv_flags_kernel(const cf* __restrict__ A,
                                                                   const cf* __restrict__ Dinv,
                                                                   const cf* __restrict__ DinvH, unsigned n, cf* b,
                                                                   ulonglong2* ll, const IrState* irs,
                                                                   int* abort_flag, unsigned* status) {
    if(irs->done) return;
    __shared__ cf v[2][NB], w[NB], z[NB], red[8][NB];
    __shared__ cf D[NB][kDs];
    static_assert(kSolveThreads == 8 * NB, "block_apply_sm: eight threads per output");
    const unsigned nblk = (n + NB - 1) / NB;
    ulonglong2* yl = ll;
    ulonglong2* xl = ll + (size_t)nblk * NB;
    const unsigned t = threadIdx.x;
    // forward: thread t sums row r = t / 8 of the block, columns 8 (t % 8) .. + 7 of each L_jk
    for(unsigned j = blockIdx.x; j < nblk; j += gridDim.x) {
        const unsigned jb = j * NB, nbj = min((unsigned)NB, n - jb);
        const unsigned r = t >> 3, s8 = (t & 7u) * 8u;
        for(unsigned q = t; q < NB * NB; q += blockDim.x) D[q / NB][q % NB] = Dinv[(size_t)j * NB * NB + q];
        cf acc = mk(0.f, 0.f);
        cf Ln[8];
        const cf* Lrow = A + (size_t)(jb + min(r, nbj - 1)) * n + s8;
        if(j > 0) {
#pragma unroll
            for(int q = 0; q < 8; q++) Ln[q] = Lrow[q];
        }
        for(unsigned k = 0; k < j; k++) {
            cf Lc[8];
#pragma unroll
            for(int q = 0; q < 8; q++) Lc[q] = Ln[q];
            if(k + 1 < j) {
#pragma unroll
                for(int q = 0; q < 8; q++) Ln[q] = Lrow[(k + 1) * NB + q];
            }
            cf* vk = v[k & 1u];
            if(!wait_block(yl + (size_t)k * NB, vk, abort_flag, status)) return;
            if(r < nbj) {
#pragma unroll
                for(int q = 0; q < 8; q++) cmac(acc, Lc[q], vk[s8 + q]);
            }
        }
        // the 8 partial sums of row r are in lanes 8 (r % 4) .. + 7 of one warp
#pragma unroll
        for(int o = 4; o > 0; o >>= 1) {
            acc.re += __shfl_xor_sync(0xffffffffu, acc.re, o);
            acc.im += __shfl_xor_sync(0xffffffffu, acc.im, o);
        }
        if((t & 7u) == 0 && r < NB) w[r] = r < nbj ? b[jb + r] - acc : mk(0.f, 0.f);
        __syncthreads();
        block_apply_sm(D, w, z, nbj);
        __syncthreads();
        if(t < NB) st_ll(yl + jb + t, z[t]);
    }
    // backward: thread t sums column c = t % 64 of L_kj^H over rows q = 8 (t / 64) .. + 7
    for(int jj = (int)nblk - 1 - (int)blockIdx.x; jj >= 0; jj -= (int)gridDim.x) {
        const unsigned j = (unsigned)jj, jb = j * NB, nbj = min((unsigned)NB, n - jb);
        const unsigned c = t & 63u, q8 = (t >> 6) * 8u;
        __syncthreads();  // the previous block's reads of D, w and red are done
        for(unsigned q = t; q < NB * NB; q += blockDim.x) D[q / NB][q % NB] = DinvH[(size_t)j * NB * NB + q];
        cf acc = mk(0.f, 0.f);
        // L[kb + q8 + q][jb + c] of block k, rows past n read as zero
        auto load_col = [&](unsigned k, cf* out) {
            const unsigned kb = k * NB, nbk = min((unsigned)NB, n - kb);
#pragma unroll
            for(int q = 0; q < 8; q++)
                out[q] = (c < nbj && q8 + q < nbk) ? A[(size_t)(kb + q8 + q) * n + jb + c] : mk(0.f, 0.f);
        };
        cf Ln[8];
        if(j + 1 < nblk) load_col(nblk - 1, Ln);
        for(unsigned k = nblk - 1; k > j; k--) {
            cf Lc[8];
#pragma unroll
            for(int q = 0; q < 8; q++) Lc[q] = Ln[q];
            if(k - 1 > j) load_col(k - 1, Ln);
            cf* vk = v[k & 1u];
            if(!wait_block(xl + (size_t)k * NB, vk, abort_flag, status)) return;
#pragma unroll
            for(int q = 0; q < 8; q++) cmac_conj(acc, Lc[q], vk[q8 + q]);
        }
        red[t >> 6][c] = acc;
        // y_j, published by the forward pass (w as the landing buffer: its last reader,
        // the block_apply of the forward pass or of the previous block, is past a barrier)
        if(!wait_block(yl + jb, w, abort_flag, status)) return;
        if(t < NB) {
            cf sum = mk(0.f, 0.f);
#pragma unroll
            for(int g = 0; g < 8; g++) sum += red[g][t];
            z[t] = t < nbj ? w[t] - sum : mk(0.f, 0.f);
        }
        __syncthreads();
        block_apply_sm(D, z, w, nbj);
        __syncthreads();
        if(t < NB) {
            st_ll(xl + jb + t, w[t]);
            if(t < nbj) b[jb + t] = w[t];
        }
    }
}

__global__ void ir_init_kernel(const zc* __restrict__ F, zc* __restrict__ x, zc* __restrict__ r,
                               cf* __restrict__ c, unsigned n, IrState* st) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i == 0) *st = IrState{0, 0, 0, 0u, -1.0, -1.0};
    if(i < n) {
        x[i] = mk(0.0, 0.0);
        r[i] = F[i];
        c[i] = cvt<float>(F[i]);
    }
}

// x += c (FP64), then c is recomputed from the new residual by ir_residual_kernel. With
// xs, x is also split for the double-float residual: xs[i] = (hi, lo) of Re and Im, hi =
// fl32(x), lo = fl32(x - hi), so x = hi + lo to 2^-48 relative.
__global__ void ir_axpy_kernel(zc* __restrict__ x, const cf* __restrict__ c, unsigned n, const IrState* st,
                               float4* __restrict__ xs) {
    if(st->done) return;
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i < n) {
        const zc v = x[i] + cvt<double>(c[i]);
        x[i] = v;
        if(xs) {
            const float rh = narrow(v.re), ih = narrow(v.im);
            xs[i] = make_float4(rh, narrow(v.re - widen(rh)), ih, narrow(v.im - widen(ih)));
        }
    }
}

// r = F - (S + shift I) x in FP64 (one warp per row), c = (complex64) r, and per-CTA
// partial sums of |r|^2 and |F|^2 for the convergence test
// The refinement of a complex64 S switches residuals: double-float (ir_residual32_kernel)
// while ||r|| / ||F|| is above kFp64Below, FP64 (this kernel) from there on, where the
// double-float floor (about 2^-48 of sum |s x| per term, against 2^-53 in FP64) would
// otherwise decide whether the tolerance is reached. Both are launched every iteration;
// each reads the state and the one not due writes zero partials.
constexpr double kFp64Below = 1e-10;

__device__ __forceinline__ bool fp64_residual_due(const IrState* st, int always) {
    return always || (st->last >= 0.0 && st->last <= kFp64Below);
}

template<typename TS>
__global__ void __launch_bounds__(256) ir_residual_kernel(const TS* __restrict__ S, unsigned n, double shift,
                                                          const zc* __restrict__ x, const zc* __restrict__ F,
                                                          zc* __restrict__ r, cf* __restrict__ c,
                                                          double* __restrict__ part, const IrState* st,
                                                          int always) {
    __shared__ double sh[2][8];
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double rr = 0.0, ff = 0.0;
    if(!st->done && fp64_residual_due(st, always)) {
        const size_t i = (size_t)blockIdx.x * 8 + warp;
        if(i < n) {
            const TS* Si = S + i * n;
            // four independent accumulators: four loads in flight per lane
            zc a0 = mk(0.0, 0.0), a1 = a0, a2 = a0, a3 = a0;
            unsigned j = lane;
            for(; j + 96 < n; j += 128) {
                const zc s0 = to_zc(Si[j]), s1 = to_zc(Si[j + 32]), s2 = to_zc(Si[j + 64]), s3 = to_zc(Si[j + 96]);
                const zc x0 = x[j], x1 = x[j + 32], x2 = x[j + 64], x3 = x[j + 96];
                cmac(a0, s0, x0);
                cmac(a1, s1, x1);
                cmac(a2, s2, x2);
                cmac(a3, s3, x3);
            }
            for(; j < n; j += 32) cmac(a0, to_zc(Si[j]), x[j]);
            zc acc = (a0 + a1) + (a2 + a3);
            acc = warp_sum(acc);
            if(lane == 0) {
                const zc ri = F[i] - acc - shift * x[i];
                r[i] = ri;
                c[i] = cvt<float>(ri);
                rr = norm2(ri);
                ff = norm2(F[i]);
            }
        }
    }
    if(lane == 0) { sh[0][warp] = rr; sh[1][warp] = ff; }
    __syncthreads();
    if(threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for(int w = 0; w < 8; w++) { a += sh[0][w]; b += sh[1][w]; }
        part[2 * blockIdx.x] = a;
        part[2 * blockIdx.x + 1] = b;
    }
}

// ---- double-float arithmetic (pairs hi + lo of FP32 values; Dekker 1971, Knuth's
// TwoSum): S x for an S of FP32 entries on the FP32 pipe. Every operation is an explicit
// round-to-nearest intrinsic, so no multiply-add is contracted into the error terms.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// (h, l) += s (xh + xl): s xh exactly as p + pe (pe = fma(s, xh, -p)), s xl rounded once
__device__ __forceinline__ void df_mac(float& h, float& l, float s, float xh, float xl) {
    const float p = __fmul_rn(s, xh);
    const float pe = __fmaf_rn(s, xh, -p);
    float t, e;
    two_sum(h, p, t, e);
    h = t;
    l = __fadd_rn(l, __fadd_rn(e, __fmaf_rn(s, xl, pe)));
}
// back to |l| <= ulp(h) / 2 (Fast2Sum; |l| << |h| here)
__device__ __forceinline__ void df_norm(float& h, float& l) {
    const float s = __fadd_rn(h, l);
    l = __fsub_rn(l, __fsub_rn(s, h));
    h = s;
}
constexpr unsigned kRes32Rows = 16;  // rows per CTA of ir_residual32_kernel (two per warp)
constexpr unsigned kResBlock = 16;   // terms per lane in one double-float block of ir_residual32_kernel

// r = F - (S + shift I) x for S in complex64 holding FP32 values (the tensor-core HERK's
// sums): S x from x's split xs, each product s xh exact, s xl rounded once, summed by
// TwoSum with renormalisation after every term (about 2^-48 relative) over blocks of 16
// terms per lane; the block sums go into FP64 accumulators, so the error is 2^-48 of a
// block's partial sum plus FP64 rounding of the running sum, not 2^-48 of a running sum
// that cancellation may leave far larger than the residual; then F - S x - shift x in FP64.
// GB300's FP64 pipe (1/64 of the FP32 rate) would bound an FP64 product at ~0.5 ms for
// Np = 8384; here the FP64 work is two adds per 16 terms. One warp per two rows (each xs
// load serves both).
__global__ void __launch_bounds__(256) ir_residual32_kernel(const cf* __restrict__ S, unsigned n, double shift,
                                                            const zc* __restrict__ x, const float4* __restrict__ xs,
                                                            const zc* __restrict__ F, zc* __restrict__ r,
                                                            cf* __restrict__ c, double* __restrict__ part,
                                                            const IrState* st) {
    __shared__ double sh[2][8];
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double rr = 0.0, ff = 0.0;
    if(!st->done && !fp64_residual_due(st, 0)) {
        const size_t i0 = (size_t)blockIdx.x * kRes32Rows + 2 * warp;
        if(i0 < n) {
            const bool two = i0 + 1 < n;
            const cf* S0 = S + i0 * n;
            const cf* S1 = S + (two ? i0 + 1 : i0) * n;
            // [row][re, im]: double-float partials over blocks of kResBlock terms, each block
            // added to an FP64 accumulator (h + l is exact in FP64): the running sum keeps
            // FP64 precision whatever its size, the double-float error stays relative to one
            // block's partial
            double acc_d[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
            for(unsigned j0 = lane; j0 < n; j0 += 32 * kResBlock) {
                float h[2][2] = {{0.f, 0.f}, {0.f, 0.f}}, l[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
#pragma unroll 4
                for(unsigned jj = 0; jj < kResBlock; jj++) {
                    const unsigned j = j0 + 32 * jj;
                    if(j >= n) break;
                    const float4 xv = xs[j];
                    const cf s[2] = {S0[j], S1[j]};
#pragma unroll
                    for(int q = 0; q < 2; q++) {
                        df_mac(h[q][0], l[q][0], s[q].re, xv.x, xv.y);   // Re s Re x
                        df_mac(h[q][0], l[q][0], -s[q].im, xv.z, xv.w);  // - Im s Im x
                        df_mac(h[q][1], l[q][1], s[q].re, xv.z, xv.w);   // Re s Im x
                        df_mac(h[q][1], l[q][1], s[q].im, xv.x, xv.y);   // Im s Re x
                        df_norm(h[q][0], l[q][0]);
                        df_norm(h[q][1], l[q][1]);
                    }
                }
#pragma unroll
                for(int q = 0; q < 2; q++)
#pragma unroll
                    for(int k = 0; k < 2; k++) acc_d[q][k] += widen(h[q][k]) + widen(l[q][k]);
            }
#pragma unroll
            for(int q = 0; q < 2; q++) {
                acc_d[q][0] = warp_sum(acc_d[q][0]);
                acc_d[q][1] = warp_sum(acc_d[q][1]);
            }
            if(lane == 0) {
                for(int q = 0; q < (two ? 2 : 1); q++) {
                    const size_t i = i0 + q;
                    const zc acc = mk(acc_d[q][0], acc_d[q][1]);
                    const zc ri = F[i] - acc - shift * x[i];
                    r[i] = ri;
                    c[i] = cvt<float>(ri);
                    rr += norm2(ri);
                    ff += norm2(F[i]);
                }
            }
        }
    }
    if(lane == 0) { sh[0][warp] = rr; sh[1][warp] = ff; }
    __syncthreads();
    if(threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for(int w = 0; w < 8; w++) { a += sh[0][w]; b += sh[1][w]; }
        part[2 * blockIdx.x] = a;
        part[2 * blockIdx.x + 1] = b;
    }
}

// fixed-order sum of the partials; sets done when ||r|| / ||F|| <= tol. With
// `report` (no host-side fallback, e.g. inside a CUDA graph) a stall at the last
// iteration is raised in the device status word.
__global__ void ir_check_kernel(const double* __restrict__ part, unsigned n_part, double tol, int last_iter,
                                IrState* st, int report, unsigned* status) {
    if(st->done) return;
    __shared__ double sh[2][32];
    double a = 0.0, b = 0.0;
    for(unsigned k = threadIdx.x; k < n_part; k += blockDim.x) {  // the residual kernel not due wrote zeros
        a += part[2 * k];
        b += part[2 * k + 1];
    }
    a = warp_sum(a);
    b = warp_sum(b);
    if((threadIdx.x & 31) == 0) { sh[0][threadIdx.x >> 5] = a; sh[1][threadIdx.x >> 5] = b; }
    __syncthreads();
    if(threadIdx.x == 0) {
        double ta = 0.0, tb = 0.0;
        for(unsigned w = 0; w < (blockDim.x >> 5); w++) { ta += sh[0][w]; tb += sh[1][w]; }
        const double rel = tb > 0.0 ? sqrt(ta / tb) : sqrt(ta);
        st->iters += 1;
        if(st->first < 0.0) st->first = rel;
        st->last = rel;
        if(rel <= tol) st->done = 1;
        else if(last_iter) {
            st->stalled = 1;
            if(report) atomicOr(status, kStatusSolveStalled);
        }
    }
}

// Inside a CUDA graph there is no host-side FP64 fallback: a refinement that ends with a
// non-finite residual or one above kKeepBelow leaves delta = 0 (the SR update then changes
// nothing) instead of a step that would corrupt the parameters; ir_check_kernel has raised
// kStatusSolveStalled for it. The flags of the FP32 factorisation (a non-positive pivot, a
// wait that gave up), which an eager solve answers with the FP64 fallback, go to the status
// word as well.
constexpr double kKeepBelow = 1e-3;

__global__ void ir_guard_kernel(zc* __restrict__ x, unsigned n, const IrState* st, unsigned* status) {
    if(blockIdx.x == 0 && threadIdx.x == 0 && st->notpd) atomicOr(status, st->notpd);
    if(st->last <= kKeepBelow) return;  // also false for NaN
    for(unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] = mk(0.0, 0.0);
}

// diagonal block, then the rows below it (and, for the tensor-core update, its operand)
// (prev: a pending rank-64 update from the panel at those columns, applied first)
// a launch that may start before the kernel ahead of it on the stream has completed (the
// kernel waits for it with pdl_wait())
template<typename... P, typename... Args>
void launch_pdl(void (*kernel)(P...), unsigned grid, unsigned block, size_t smem, cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    ANN_CUDA(cudaLaunchKernelEx(&cfg, kernel, args...));
}

void panel32(cf* A, unsigned n, unsigned kb, unsigned* status, PtDst pt, cudaStream_t st, unsigned prev = kNoPrev) {
    // the first panel of a pair waits for the update before it in full (a plain launch);
    // the second starts under the first panel's row solve
    if(prev == kNoPrev) potrf32_kernel<<<1, kPotrfThreads, kPotrfSmem, st>>>(A, n, kb, status, prev);
    else launch_pdl(potrf32_kernel, 1, kPotrfThreads, kPotrfSmem, st, A, n, kb, status, prev);
    check_launch("potrf32_kernel");
    factor_mark(110, st, 2);
    const unsigned nb = min((unsigned)NB, n - kb);
    const unsigned below = n - kb - nb;
    if(below) {
        launch_pdl(trsm32_kernel, (below + kTrsmRows - 1) / kTrsmRows, 256, kTrsmSmem, st, A, n, kb, pt, prev);
        check_launch("trsm32_kernel");
    }
}

// the panel pair at columns pb .. pb + 127: panel pb, then the second panel, whose
// diagonal block (potrf32) and rows below (trsm32) first apply the first panel's rank-64
// update of the second panel's 64 columns. The rows from pb + 128 on of both panels go to
// PT (pair layout: K = 128, rows [hi | lo] of 256 floats) for the pair's tensor-core update
// of the rest.
void panel_pair32(cf* A, unsigned n, unsigned pb, unsigned* status, float* PT, cudaStream_t st) {
    factor_mark(100, st);
    panel32(A, n, pb, status, PtDst{PT, pb + 2 * NB, 0, 4 * NB}, st);
    factor_mark(101, st, 2);
    if(n - pb <= (unsigned)NB) return;
    panel32(A, n, pb + NB, status, PtDst{PT, pb + 2 * NB, NB, 4 * NB}, st, pb);
    factor_mark(103, st);
}

void set_smem_attrs() {
    static bool done = false;  // per process: the attribute is per function and device-independent
    if(done) return;
    ANN_CUDA(cudaFuncSetAttribute(diag_inv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  2 * NB * (NB + 1) * (int)sizeof(cf)));
    ANN_CUDA(cudaFuncSetAttribute(herk32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  2 * NB * (UT + 1) * (int)sizeof(cf)));
    ANN_CUDA(cudaFuncSetAttribute(potrf32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPotrfSmem));
    done = true;
}

// Right-looking blocked Cholesky with look-ahead (the FP32 twin of cholesky.cu's):
// after panel k the trailing update first covers the tile column holding panel k+1,
// which the high-priority side stream then factorises while the rest of the update
// runs. The update runs on the tensor cores (split TF32, 128 x 128 tiles) or on the
// FP32 SIMT cores (64 x 64 tiles), as td.chol_tc selects.
void cholesky32(ann_tdvp_impl& td, cf* A, unsigned n, cf* Dinv, cf* DinvH, unsigned* status, cudaStream_t st) {
    ensure_side_stream(td);
    // an explicit choice, else the autotuned one for this size, else the default
    const bool tc = td.chol_tc_set ? td.chol_tc != 0 : tuning_get(key_chol_update(n), td.chol_tc) != 0;
    if(tc) {
        chol_update_tc_prepare(td, n, st);
        chol_update_tc_bind(td, A, n);
    }
    const size_t herk_smem = 2 * NB * (UT + 1) * sizeof(cf);
    const bool pair = tc && td.chol_reduce && tuning_get(key_chol_pair(n), 1) != 0;
    factor_trace_reset();
    td.chol_form = pair ? ANN_CHOL_FORM_TC_PAIR : (tc ? ANN_CHOL_FORM_TC_PANEL : ANN_CHOL_FORM_SIMT);
    if(pair) {
        // Panel pairs (128 columns): the tensor-core update of the rest is one rank-128
        // update per pair, half the passes over the trailing matrix and half the launches
        // of one update per panel. Pair p's rows go to operand buffer p % 2: pair p+1 (side
        // stream, after the update of the tile column holding it) fills the other buffer
        // while the rest of update p still reads this one.
        auto ppt = [&](unsigned pb) { return chol_update_tc_pair_operand(td, (pb / (2 * NB)) & 1u); };
        panel_pair32(A, n, 0, status, ppt(0), st);
        for(unsigned pb = 0; pb + 2 * NB < n; pb += 2 * NB) {
            factor_mark(200, st);
            chol_update_tc_pair(td, A, n, pb, true, status, st);
            factor_mark(201, st);
            ANN_CUDA(cudaEventRecord(td.side_ev[0], st));
            ANN_CUDA(cudaStreamWaitEvent(td.side, td.side_ev[0], 0));
            panel_pair32(A, n, pb + 2 * NB, status, ppt(pb + 2 * NB), td.side);
            ANN_CUDA(cudaEventRecord(td.side_ev[1], td.side));
            chol_update_tc_pair(td, A, n, pb, false, status, st);
            factor_mark(202, st);
            ANN_CUDA(cudaStreamWaitEvent(st, td.side_ev[1], 0));
            factor_mark(203, st);
        }
        diag_inv_kernel<<<(n + NB - 1) / NB, 1024, 2 * NB * (NB + 1) * sizeof(cf), st>>>(A, n, Dinv, DinvH);
        check_launch("diag_inv_kernel");
        return;
    }
    // panel k's rows go to operand buffer k % 2: panel k+1 (side stream) fills the other
    // buffer while the rest of update k still reads this one
    auto pt = [&](unsigned kb) {
        return PtDst{tc ? chol_update_tc_operand(td, (kb / NB) & 1u) : nullptr, kb + NB, 0, 2 * NB};
    };
    panel32(A, n, 0, status, pt(0), st);
    for(unsigned kb = 0; kb < n; kb += NB) {
        const unsigned nb = min((unsigned)NB, n - kb);
        const unsigned below = n - kb - nb;
        if(below == 0) break;
        const unsigned tiles = (below + UT - 1) / UT;
        if(tc) {
            chol_update_tc(td, A, n, kb, true, status, st);
        } else {
            herk32_kernel<<<tiles, 256, herk_smem, st>>>(A, n, kb, nb, 1);
            check_launch("herk32_kernel");
        }
        ANN_CUDA(cudaEventRecord(td.side_ev[0], st));
        ANN_CUDA(cudaStreamWaitEvent(td.side, td.side_ev[0], 0));
        panel32(A, n, kb + nb, status, pt(kb + nb), td.side);
        ANN_CUDA(cudaEventRecord(td.side_ev[1], td.side));
        if(tc) {
            chol_update_tc(td, A, n, kb, false, status, st);
        } else if(tiles > 1) {
            herk32_kernel<<<(tiles - 1) * tiles / 2, 256, herk_smem, st>>>(A, n, kb, nb, 0);
            check_launch("herk32_kernel");
        }
        ANN_CUDA(cudaStreamWaitEvent(st, td.side_ev[1], 0));
    }
    // inverses of the diagonal blocks for the triangular solves, all blocks at once
    diag_inv_kernel<<<(n + NB - 1) / NB, 1024, 2 * NB * (NB + 1) * sizeof(cf), st>>>(A, n, Dinv, DinvH);
    check_launch("diag_inv_kernel");
}

// b <- (L L^H)^{-1} b; sync holds the abort flag (16 bytes) and the tagged solution
// blocks (2 nblk NB 16-byte entries), cleared before the launch
void solve32(const cf* A, const cf* Dinv, const cf* DinvH, unsigned n, cf* b, const IrState* irs, int* sync,
             unsigned* status, cudaStream_t st) {
    static int resident = 0;  // CTAs of trsv_flags_kernel that fit on the GPU at once
    if(!resident) {
        int dev = 0, sms = 0, per_sm = 0;
        ANN_CUDA(cudaGetDevice(&dev));
        ANN_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        ANN_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, trsv_flags_kernel, kSolveThreads, 0));
        if(per_sm < 1) throw Error(ANN_ERR_CUDA, "trsv_flags_kernel cannot be resident");
        resident = sms * per_sm;
    }
    const unsigned nblk = (n + NB - 1) / NB;
    const unsigned grid = std::min<unsigned>(nblk, (unsigned)resident);
    ANN_CUDA(cudaMemsetAsync(sync, 0, kSolveSyncHead + 2 * (size_t)nblk * NB * sizeof(ulonglong2), st));
    ulonglong2* ll = reinterpret_cast<ulonglong2*>(reinterpret_cast<char*>(sync) + kSolveSyncHead);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kSolveThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;  // every CTA resident: the waits can be met
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    ANN_CUDA(cudaLaunchKernelEx(&cfg, trsv_flags_kernel, A, Dinv, DinvH, n, b, ll, irs, sync, status));
    check_launch("trsv_flags_kernel");
}

}  // namespace

void sr_solve_mixed(ann_tdvp_impl& td, double shift, unsigned max_iter, double tol, bool pivots_to_status,
                    unsigned* status, cudaStream_t st) {
    const unsigned n = td.Np;
    const size_t nn = (size_t)n * n;
    const unsigned nblk = (n + NB - 1) / NB;
    set_smem_attrs();
    td.L32.ensure(nn * sizeof(cf));
    td.Dinv32.ensure(2 * (size_t)nblk * NB * NB * sizeof(cf));
    td.delta.ensure(n * sizeof(zc));
    td.resid.ensure(2 * n * sizeof(zc) + 2 * sizeof(double));
    td.c32.ensure((size_t)n * sizeof(cf));
    // S in complex64 (FP32 values): double-float residuals on the FP32 pipe until the
    // residual nears the tolerance, then FP64 ones; a complex128 S: FP64 residuals. The two
    // kernels keep their partial sums in separate ranges of `part` (FP64 first).
    const bool s32 = td.S_in32;
    if(s32) td.xs32.ensure((size_t)n * sizeof(float4));
    const unsigned res64 = (n + 7) / 8, res32 = s32 ? (n + kRes32Rows - 1) / kRes32Rows : 0u;
    const unsigned res_blocks = res64 + res32;
    static_assert(sizeof(IrState) % 16 == 0, "the solve's tagged blocks need 16-byte alignment");
    td.ir.ensure(sizeof(IrState) + 2 * (size_t)res_blocks * sizeof(double) + kSolveSyncHead +
                 2 * (size_t)nblk * NB * sizeof(ulonglong2));
    cf* A = td.L32.as<cf>();
    cf* Dinv = td.Dinv32.as<cf>();
    cf* DinvH = Dinv + (size_t)nblk * NB * NB;
    zc* x = td.delta.as<zc>();
    zc* r = td.resid.as<zc>();
    cf* c = td.c32.as<cf>();
    IrState* irs = td.ir.as<IrState>();
    double* part = reinterpret_cast<double*>(irs + 1);
    int* sync = reinterpret_cast<int*>(part + 2 * (size_t)res_blocks);
    const zc* S = s32 ? nullptr : td.S.as<zc>();
    const cf* S32 = s32 ? td.S32.as<cf>() : nullptr;
    float4* xs = s32 ? td.xs32.as<float4>() : nullptr;
    const zc* F = td.F.as<zc>();

    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    ANN_CUDA(cudaStreamIsCapturing(st, &cs));
    const int report = cs != cudaStreamCaptureStatusNone;
    ir_init_kernel<<<(n + 255) / 256, 256, 0, st>>>(F, x, r, c, n, irs);
    check_launch("ir_init_kernel");
    if(s32) cvt_shift_kernel<cf><<<(n + 1) / 2, 256, 0, st>>>(S32, A, n, shift);
    else cvt_shift_kernel<zc><<<(n + 1) / 2, 256, 0, st>>>(S, A, n, shift);
    check_launch("cvt_shift_kernel");
    // FP32 pivot failures are recorded in the refinement state (they end in a stall and
    // the FP64 fallback), or, with no refinement to fall back from, in the status word
    solve_mark(0, st);
    cholesky32(td, A, n, Dinv, DinvH, pivots_to_status ? status : &irs->notpd, st);
    solve_mark(1, st);
    for(unsigned it = 0; it < max_iter; it++) {
        solve32(A, Dinv, DinvH, n, c, irs, sync, status, st);
        ir_axpy_kernel<<<(n + 255) / 256, 256, 0, st>>>(x, c, n, irs, xs);
        check_launch("ir_axpy_kernel");
        if(s32) {
            ir_residual32_kernel<<<res32, 256, 0, st>>>(S32, n, shift, x, xs, F, r, c, part + 2 * (size_t)res64, irs);
            check_launch("ir_residual32_kernel");
            ir_residual_kernel<cf><<<res64, 256, 0, st>>>(S32, n, shift, x, F, r, c, part, irs, 0);
        } else {
            ir_residual_kernel<zc><<<res64, 256, 0, st>>>(S, n, shift, x, F, r, c, part, irs, 1);
        }
        check_launch("ir_residual_kernel");
        ir_check_kernel<<<1, 1024, 0, st>>>(part, res_blocks, tol, it + 1 == max_iter, irs, report, status);
        check_launch("ir_check_kernel");
    }
    if(report && !pivots_to_status) {
        ir_guard_kernel<<<(n + 255) / 256, 256, 0, st>>>(x, n, irs, status);
        check_launch("ir_guard_kernel");
    }
}

void mixed_solve_info(const ann_tdvp_impl& td, double* out4, cudaStream_t st) {
    IrState h{};
    ANN_CUDA(cudaMemcpyAsync(&h, td.ir.p, sizeof(IrState), cudaMemcpyDeviceToHost, st));
    ANN_CUDA(cudaStreamSynchronize(st));
    out4[0] = h.iters;
    out4[1] = h.first;
    out4[2] = h.last;
    out4[3] = (h.stalled || h.notpd) ? 1.0 : 0.0;
}

void sr_solve_any(ann_tdvp_impl& td, double shift, unsigned* status, cudaStream_t st) {
    td.fell_back = false;
    if(td.solver == ANN_SOLVER_FP64) {
        sr_solve(td, shift, status, st);
        return;
    }
    if(td.solver == ANN_SOLVER_FP32) {
        // one FP32 solve, no refinement, no tolerance (the plain FP32 form)
        sr_solve_mixed(td, shift, 1, HUGE_VAL, true, status, st);
        return;
    }
    sr_solve_mixed(td, shift, td.ir_max, td.ir_tol, false, status, st);
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    ANN_CUDA(cudaStreamIsCapturing(st, &cs));
    if(cs != cudaStreamCaptureStatusNone) return;  // no host decision inside a graph
    double info[4];
    mixed_solve_info(td, info, st);
    if(info[3] != 0.0) {
        // the FP32 factor was not good enough (cond(S + shift I) * u_fp32 >~ 1): FP64 solve
        sr_solve(td, shift, status, st);
        td.fell_back = true;
    }
}

}  // namespace ann
