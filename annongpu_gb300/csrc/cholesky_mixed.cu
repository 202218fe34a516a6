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
#include <cmath>

#include "ann_internal.hpp"

namespace ann {

namespace {

constexpr int NB = 64;     // panel / diagonal block width
constexpr int UT = 64;     // trailing-update tile (== NB: tile column 0 is the next panel)

using cf = cplx<float>;
using zc = cplx<double>;

// lower triangle of S + shift I in complex64, row-major n x n
__global__ void cvt_shift_kernel(const zc* __restrict__ S, cf* __restrict__ A, unsigned n, double shift) {
    const unsigned i = blockIdx.y;
    for(unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j <= i; j += gridDim.x * blockDim.x) {
        zc v = S[(size_t)i * n + j];
        if(i == j) v.re += shift;
        A[(size_t)i * n + j] = cvt<float>(v);
    }
}

// Cholesky of the nb x nb diagonal block at (kb, kb) in shared memory, then the
// inverse of the factor, column c by the 16 lanes of group c:
//   X[i][c] = (delta_ic - sum_{c <= p < i} L[i][p] X[p][c]) / L[i][i].
// Dinv[blk] = L_kk^{-1}, DinvH[blk] = L_kk^{-H} (row-major NB x NB, identity
// beyond nb).
__global__ void __launch_bounds__(1024) potrf32_kernel(cf* __restrict__ A, unsigned n, unsigned kb,
                                                       cf* __restrict__ Dinv, cf* __restrict__ DinvH,
                                                       unsigned* status) {
    extern __shared__ float4 smem_raw[];
    cf (*a)[NB + 1] = reinterpret_cast<cf (*)[NB + 1]>(smem_raw);
    cf (*x)[NB + 1] = reinterpret_cast<cf (*)[NB + 1]>(reinterpret_cast<cf*>(smem_raw) + NB * (NB + 1));
    const unsigned nb = min((unsigned)NB, n - kb);
    const unsigned tid = threadIdx.x;
    for(unsigned t = tid; t < NB * NB; t += blockDim.x) {
        const unsigned r = t / NB, c = t % NB;
        cf v = mk(0.f, 0.f);
        if(r < nb && c <= r) v = A[(size_t)(kb + r) * n + kb + c];
        else if(r == c) v = mk(1.f, 0.f);
        a[r][c] = v;
        x[r][c] = mk(0.f, 0.f);
    }
    __syncthreads();
    for(unsigned j = 0; j < NB; j++) {
        float d = a[j][j].re;
        if(!(d > 0.f) || !isfinite(d)) {
            if(tid == 0) atomicOr(status, kStatusNotPosDef);
            d = 1.f;
        }
        const float sd = sqrtf(d);
        __syncthreads();  // every thread has read the pivot before it changes
        if(tid == j) a[j][j] = mk(sd, 0.f);
        else if(tid > j && tid < NB) a[tid][j] = (1.f / sd) * a[tid][j];
        __syncthreads();
        for(unsigned t = tid; t < NB * NB; t += blockDim.x) {
            const unsigned r = t / NB, c = t % NB;
            if(c > j && c <= r) {
                cf v = a[r][c];
                cmac_conj(v, a[c][j], -a[r][j]);   // v -= a[r][j] conj(a[c][j])
                a[r][c] = v;
            }
        }
        __syncthreads();
    }
    // inverse: group g = tid / 16 owns column g (NB == 64 columns, 1024 threads)
    {
        const unsigned c = tid >> 4, s = tid & 15u;
        const unsigned i0 = c & ~1u;  // both groups of a warp walk the same rows
        for(unsigned i = i0; i < NB; i++) {
            cf part = mk(0.f, 0.f);
            for(unsigned p = i0 + s; p < i; p += 16) cmac(part, a[i][p], x[p][c]);
#pragma unroll
            for(int o = 8; o > 0; o >>= 1) {
                part.re += __shfl_xor_sync(0xffffffffu, part.re, o, 16);
                part.im += __shfl_xor_sync(0xffffffffu, part.im, o, 16);
            }
            if(s == 0) {
                const float inv = 1.f / a[i][i].re;
                const float dre = (i == c) ? 1.f : 0.f;
                x[i][c] = mk(inv * (dre - part.re), -inv * part.im);
            }
            __syncwarp();
        }
    }
    __syncthreads();
    const size_t blk = kb / NB;
    for(unsigned t = tid; t < NB * NB; t += blockDim.x) {
        const unsigned r = t / NB, c = t % NB;
        if(r < nb && c <= r) A[(size_t)(kb + r) * n + kb + c] = a[r][c];
        Dinv[blk * NB * NB + t] = x[r][c];
        DinvH[blk * NB * NB + t] = conj(x[c][r]);
    }
}

// rows below the diagonal block: X <- X L_kk^{-H}, out[c] = sum_{p <= c} X[p] conj(Dinv[c][p]).
// One warp per row, lane owns columns lane and lane + 32; DinvH staged in shared memory.
__global__ void __launch_bounds__(256) trsm32_kernel(cf* __restrict__ A, unsigned n, unsigned kb,
                                                     const cf* __restrict__ DinvH) {
    __shared__ cf D[NB][NB + 1];  // D[p][c] = DinvH[p][c] = conj(Dinv[c][p])
    const size_t blk = kb / NB;
    for(unsigned t = threadIdx.x; t < NB * NB; t += blockDim.x) D[t / NB][t % NB] = DinvH[blk * NB * NB + t];
    __syncthreads();
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned nb = min((unsigned)NB, n - kb);
    const size_t row0 = (size_t)kb + nb + (size_t)blockIdx.x * 64;
    for(unsigned rr = warp; rr < 64; rr += 8) {
        const size_t row = row0 + rr;
        if(row >= n) break;
        cf* X = A + row * n + kb;
        const cf x0 = lane < nb ? X[lane] : mk(0.f, 0.f);
        const cf x1 = lane + 32 < nb ? X[lane + 32] : mk(0.f, 0.f);
        cf o0 = mk(0.f, 0.f), o1 = mk(0.f, 0.f);
#pragma unroll 8
        for(unsigned p = 0; p < 32; p++) {
            cf xp;
            xp.re = __shfl_sync(0xffffffffu, x0.re, p);
            xp.im = __shfl_sync(0xffffffffu, x0.im, p);
            cmac(o0, xp, D[p][lane]);
            cmac(o1, xp, D[p][lane + 32]);
        }
#pragma unroll 8
        for(unsigned p = 0; p < 32; p++) {
            cf xp;
            xp.re = __shfl_sync(0xffffffffu, x1.re, p);
            xp.im = __shfl_sync(0xffffffffu, x1.im, p);
            cmac(o1, xp, D[p + 32][lane + 32]);
        }
        if(lane < nb) X[lane] = o0;
        if(lane + 32 < nb) X[lane + 32] = o1;
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

// y_k = Dk b_k for the diagonal block (Dk = Dinv or DinvH of block kb), by 8 warps,
// output c by one warp with the 64-term dot split over lanes
__device__ __forceinline__ void block_apply(const cf* __restrict__ Dk, const cf* __restrict__ bk, cf* y,
                                            unsigned nb) {
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for(unsigned c = warp; c < NB; c += 8) {
        cf acc = mk(0.f, 0.f);
        cmac(acc, Dk[c * NB + lane], bk[lane]);
        cmac(acc, Dk[c * NB + lane + 32], bk[lane + 32]);
        acc = warp_sum(acc);
        if(lane == 0) y[c] = c < nb ? acc : mk(0.f, 0.f);
    }
}

// forward step of L y = b for block kb: y_k = L_kk^{-1} b_k (every CTA, redundantly),
// CTA 0 stores it into y_out (b[kb:] is still read by CTAs that start later), all
// CTAs subtract L[i][kb:] y_k from the rows of b below (one warp per row)
__global__ void __launch_bounds__(256) fwd32_kernel(const cf* __restrict__ A, const cf* __restrict__ Dinv,
                                                    unsigned n, unsigned kb, cf* __restrict__ b,
                                                    cf* __restrict__ y_out, const IrState* st) {
    if(st->done) return;
    __shared__ cf bk[NB], y[NB];
    const unsigned nb = min((unsigned)NB, n - kb);
    if(threadIdx.x < NB) bk[threadIdx.x] = threadIdx.x < nb ? b[kb + threadIdx.x] : mk(0.f, 0.f);
    __syncthreads();
    block_apply(Dinv + (size_t)(kb / NB) * NB * NB, bk, y, nb);
    __syncthreads();
    if(blockIdx.x == 0 && threadIdx.x < nb) y_out[kb + threadIdx.x] = y[threadIdx.x];
    const unsigned lane = threadIdx.x & 31;
    const size_t warps = (size_t)gridDim.x * 8;
    for(size_t i = kb + nb + (size_t)blockIdx.x * 8 + (threadIdx.x >> 5); i < n; i += warps) {
        const cf* Li = A + i * n + kb;
        cf acc = mk(0.f, 0.f);
        if(lane < nb) cmac(acc, Li[lane], y[lane]);
        if(lane + 32 < nb) cmac(acc, Li[lane + 32], y[lane + 32]);
        acc = warp_sum(acc);
        if(lane == 0) b[i] = b[i] - acc;
    }
}

// backward step of L^H x = y for block kb: x_k = L_kk^{-H} y_k into x_out, then every
// row i < kb of b subtracts sum_p conj(L[kb + p][i]) x_p (thread per i, coalesced
// along the block rows)
__global__ void __launch_bounds__(256) bwd32_kernel(const cf* __restrict__ A, const cf* __restrict__ DinvH,
                                                    unsigned n, unsigned kb, cf* __restrict__ b,
                                                    cf* __restrict__ x_out, const IrState* st) {
    if(st->done) return;
    __shared__ cf bk[NB], x[NB];
    const unsigned nb = min((unsigned)NB, n - kb);
    if(threadIdx.x < NB) bk[threadIdx.x] = threadIdx.x < nb ? b[kb + threadIdx.x] : mk(0.f, 0.f);
    __syncthreads();
    block_apply(DinvH + (size_t)(kb / NB) * NB * NB, bk, x, nb);
    __syncthreads();
    if(blockIdx.x == 0 && threadIdx.x < nb) x_out[kb + threadIdx.x] = x[threadIdx.x];
    for(size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < kb; i += (size_t)gridDim.x * blockDim.x) {
        cf acc = mk(0.f, 0.f);
#pragma unroll 8
        for(unsigned q = 0; q < nb; q++) cmac_conj(acc, A[(size_t)(kb + q) * n + i], x[q]);
        b[i] = b[i] - acc;
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

// x += c (FP64), then c is recomputed from the new residual by ir_residual_kernel
__global__ void ir_axpy_kernel(zc* __restrict__ x, const cf* __restrict__ c, unsigned n, const IrState* st) {
    if(st->done) return;
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i < n) x[i] += cvt<double>(c[i]);
}

// r = F - (S + shift I) x in FP64 (one warp per row), c = (complex64) r, and per-CTA
// partial sums of |r|^2 and |F|^2 for the convergence test
__global__ void __launch_bounds__(256) ir_residual_kernel(const zc* __restrict__ S, unsigned n, double shift,
                                                          const zc* __restrict__ x, const zc* __restrict__ F,
                                                          zc* __restrict__ r, cf* __restrict__ c,
                                                          double* __restrict__ part, const IrState* st) {
    __shared__ double sh[2][8];
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double rr = 0.0, ff = 0.0;
    if(!st->done) {
        const size_t i = (size_t)blockIdx.x * 8 + warp;
        if(i < n) {
            const zc* Si = S + i * n;
            zc acc = mk(0.0, 0.0);
            for(unsigned j = lane; j < n; j += 32) cmac(acc, Si[j], x[j]);
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

// fixed-order sum of the partials; sets done when ||r|| / ||F|| <= tol. With
// `report` (no host-side fallback, e.g. inside a CUDA graph) a stall at the last
// iteration is raised in the device status word.
__global__ void ir_check_kernel(const double* __restrict__ part, unsigned n_part, double tol, int last_iter,
                                IrState* st, int report, unsigned* status) {
    if(st->done) return;
    __shared__ double sh[2][32];
    double a = 0.0, b = 0.0;
    for(unsigned k = threadIdx.x; k < n_part; k += blockDim.x) {
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

void panel32(cf* A, unsigned n, unsigned kb, cf* Dinv, cf* DinvH, unsigned* status, cudaStream_t st) {
    potrf32_kernel<<<1, 1024, 2 * NB * (NB + 1) * sizeof(cf), st>>>(A, n, kb, Dinv, DinvH, status);
    check_launch("potrf32_kernel");
    const unsigned nb = min((unsigned)NB, n - kb);
    const unsigned below = n - kb - nb;
    if(below) {
        trsm32_kernel<<<(below + 63) / 64, 256, 0, st>>>(A, n, kb, DinvH);
        check_launch("trsm32_kernel");
    }
}

void set_smem_attrs() {
    static bool done = false;  // per process: the attribute is per function and device-independent
    if(done) return;
    ANN_CUDA(cudaFuncSetAttribute(potrf32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  2 * NB * (NB + 1) * (int)sizeof(cf)));
    ANN_CUDA(cudaFuncSetAttribute(herk32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  2 * NB * (UT + 1) * (int)sizeof(cf)));
    done = true;
}

// right-looking blocked Cholesky with look-ahead (the FP32 twin of cholesky.cu's)
void cholesky32(ann_tdvp_impl& td, cf* A, unsigned n, cf* Dinv, cf* DinvH, unsigned* status, cudaStream_t st) {
    if(!td.side) {
        ANN_CUDA(cudaStreamCreateWithFlags(&td.side, cudaStreamNonBlocking));
        for(auto& e : td.side_ev) ANN_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    const size_t herk_smem = 2 * NB * (UT + 1) * sizeof(cf);
    panel32(A, n, 0, Dinv, DinvH, status, st);
    for(unsigned kb = 0; kb < n; kb += NB) {
        const unsigned nb = min((unsigned)NB, n - kb);
        const unsigned below = n - kb - nb;
        if(below == 0) break;
        const unsigned tiles = (below + UT - 1) / UT;
        herk32_kernel<<<tiles, 256, herk_smem, st>>>(A, n, kb, nb, 1);
        check_launch("herk32_kernel");
        ANN_CUDA(cudaEventRecord(td.side_ev[0], st));
        ANN_CUDA(cudaStreamWaitEvent(td.side, td.side_ev[0], 0));
        panel32(A, n, kb + nb, Dinv, DinvH, status, td.side);
        ANN_CUDA(cudaEventRecord(td.side_ev[1], td.side));
        if(tiles > 1) {
            herk32_kernel<<<(tiles - 1) * tiles / 2, 256, herk_smem, st>>>(A, n, kb, nb, 0);
            check_launch("herk32_kernel");
        }
        ANN_CUDA(cudaStreamWaitEvent(st, td.side_ev[1], 0));
    }
}

// b <- (L L^H)^{-1} b; tmp (n entries) holds y = L^{-1} b
void solve32(const cf* A, const cf* Dinv, const cf* DinvH, unsigned n, cf* b, cf* tmp, const IrState* irs,
             cudaStream_t st) {
    for(unsigned kb = 0; kb < n; kb += NB) {
        const unsigned below = n - kb - min((unsigned)NB, n - kb);
        const unsigned grid = below ? min(304u, (below + 7) / 8) : 1u;
        fwd32_kernel<<<grid, 256, 0, st>>>(A, Dinv, n, kb, b, tmp, irs);
        check_launch("fwd32_kernel");
    }
    const unsigned last = ((n - 1) / NB) * NB;
    for(int kb = (int)last; kb >= 0; kb -= NB) {
        const unsigned grid = kb ? min(304u, ((unsigned)kb + 255) / 256) : 1u;
        bwd32_kernel<<<grid, 256, 0, st>>>(A, DinvH, n, (unsigned)kb, tmp, b, irs);
        check_launch("bwd32_kernel");
    }
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
    td.c32.ensure(2 * (size_t)n * sizeof(cf));
    const unsigned res_blocks = (n + 7) / 8;
    td.ir.ensure(sizeof(IrState) + 2 * (size_t)res_blocks * sizeof(double));
    cf* A = td.L32.as<cf>();
    cf* Dinv = td.Dinv32.as<cf>();
    cf* DinvH = Dinv + (size_t)nblk * NB * NB;
    zc* x = td.delta.as<zc>();
    zc* r = td.resid.as<zc>();
    cf* c = td.c32.as<cf>();
    IrState* irs = td.ir.as<IrState>();
    double* part = reinterpret_cast<double*>(irs + 1);
    const zc* S = td.S.as<zc>();
    const zc* F = td.F.as<zc>();

    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    ANN_CUDA(cudaStreamIsCapturing(st, &cs));
    const int report = cs != cudaStreamCaptureStatusNone;
    ir_init_kernel<<<(n + 255) / 256, 256, 0, st>>>(F, x, r, c, n, irs);
    check_launch("ir_init_kernel");
    cvt_shift_kernel<<<dim3((n + 255) / 256, n), 256, 0, st>>>(S, A, n, shift);
    check_launch("cvt_shift_kernel");
    // FP32 pivot failures are recorded in the refinement state (they end in a stall and
    // the FP64 fallback), or, with no refinement to fall back from, in the status word
    cholesky32(td, A, n, Dinv, DinvH, pivots_to_status ? status : &irs->notpd, st);
    for(unsigned it = 0; it < max_iter; it++) {
        solve32(A, Dinv, DinvH, n, c, c + n, irs, st);
        ir_axpy_kernel<<<(n + 255) / 256, 256, 0, st>>>(x, c, n, irs);
        check_launch("ir_axpy_kernel");
        ir_residual_kernel<<<res_blocks, 256, 0, st>>>(S, n, shift, x, F, r, c, part, irs);
        check_launch("ir_residual_kernel");
        ir_check_kernel<<<1, 1024, 0, st>>>(part, res_blocks, tol, it + 1 == max_iter, irs, report, status);
        check_launch("ir_check_kernel");
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
