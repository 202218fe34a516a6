// FP64 SR solve on the GPU: (S + shift I) delta = F by a blocked right-looking
// complex Cholesky factorisation, two blocked triangular solves and one step of
// iterative refinement against the unfactored matrix.
//
// The reference has no solver: TDVP only builds S and F and the caller solves
// on the host (source/network_functions/TDVP.cu.template:181-302,
// pyANNonGPU/main.cpp.template:465-489). This file is the project's own.
//
// Matrices are row-major complex128, N x N; only the lower triangle of the
// factor is referenced. Failures never trap: a non-positive or non-finite pivot
// sets kStatusNotPosDef in the device status word, is replaced by 1 so the
// remaining kernels stay finite, and the host reports ANN_ERR_NUMERIC.
#include "ann_internal.hpp"

namespace ann {

namespace {

constexpr int NB = 32;   // panel width
constexpr int UT = 64;   // trailing-update tile

using zc = cplx<double>;

__global__ void copy_shift_kernel(const zc* __restrict__ S, zc* __restrict__ A, unsigned n, double shift) {
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t total = (size_t)n * n;
    if(idx >= total) return;
    zc v = S[idx];
    const size_t i = idx / n, j = idx % n;
    if(i == j) v.re += shift;
    A[idx] = v;
}

// unblocked Cholesky of the nb x nb diagonal block at (kb, kb)
__global__ void __launch_bounds__(NB * NB) potrf_diag_kernel(zc* __restrict__ A, unsigned n, unsigned kb,
                                                             unsigned* status) {
    __shared__ zc a[NB][NB + 1];
    const unsigned nb = min((unsigned)NB, n - kb);
    const unsigned r = threadIdx.x / NB, c = threadIdx.x % NB;
    if(r < nb && c < nb) a[r][c] = A[(size_t)(kb + r) * n + kb + c];
    __syncthreads();
    for(unsigned j = 0; j < nb; j++) {
        if(threadIdx.x == 0) {
            double d = a[j][j].re;
            if(!(d > 0.0) || !isfinite(d)) {
                atomicOr(status, kStatusNotPosDef);
                d = 1.0;
            }
            a[j][j] = mk(sqrt(d), 0.0);
        }
        __syncthreads();
        if(c == j && r > j && r < nb) {
            const double inv = 1.0 / a[j][j].re;
            a[r][j] = inv * a[r][j];
        }
        __syncthreads();
        if(r > j && c > j && c <= r && r < nb) a[r][c] = a[r][c] - a[r][j] * conj(a[c][j]);
        __syncthreads();
    }
    if(r < nb && c <= r) A[(size_t)(kb + r) * n + kb + c] = a[r][c];
}

// rows below the diagonal block: X <- X L_kk^{-H}, one warp per row, lane j owns
// column j: x_j = b_j / L_jj, then every later column p subtracts x_j conj(L_pj)
__global__ void __launch_bounds__(256) trsm_panel_kernel(zc* __restrict__ A, unsigned n, unsigned kb) {
    __shared__ zc L[NB][NB + 1];
    __shared__ double inv_d[NB];
    const unsigned nb = min((unsigned)NB, n - kb);
    for(unsigned t = threadIdx.x; t < nb * nb; t += blockDim.x) {
        const unsigned r = t / nb, c = t % nb;
        L[r][c] = r >= c ? A[(size_t)(kb + r) * n + kb + c] : mk(0.0, 0.0);
    }
    __syncthreads();
    if(threadIdx.x < nb) inv_d[threadIdx.x] = 1.0 / L[threadIdx.x][threadIdx.x].re;
    __syncthreads();
    const unsigned lane = threadIdx.x & 31;
    const size_t row = kb + nb + (size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if(row >= n) return;
    zc b = lane < nb ? A[row * n + kb + lane] : mk(0.0, 0.0);
    for(unsigned j = 0; j < nb; j++) {
        zc xj = inv_d[j] * b;
        xj.re = __shfl_sync(0xffffffffu, xj.re, j);
        xj.im = __shfl_sync(0xffffffffu, xj.im, j);
        if(lane == j) b = xj;
        else if(lane > j && lane < nb) b = b - xj * conj(L[lane][j]);
    }
    if(lane < nb) A[row * n + kb + lane] = b;
}

// trailing lower triangle: A[i][j] -= sum_p X[i][p] conj(X[j][p]), i >= j >= t0.
// col_only: the first tile column (the next panels, updated first for the
// look-ahead); otherwise the lower-triangular tiles with tile column >= 1.
__global__ void __launch_bounds__(256) herk_update_kernel(zc* __restrict__ A, unsigned n, unsigned kb, unsigned nb,
                                                          int col_only) {
    __shared__ zc Xi[16][UT];
    __shared__ zc Xj[16][UT];
    const unsigned t0 = kb + nb;
    unsigned ti, tj;
    if(col_only) {
        ti = blockIdx.x;
        tj = 0;
    } else {
        // lower-triangular tile (ti >= tj) of the sub-grid starting at tile (1, 1)
        unsigned b = blockIdx.x;
        ti = 0;
        while(b > ti) { b -= ti + 1; ti++; }
        tj = b + 1;
        ti += 1;
    }
    const unsigned i0 = t0 + ti * UT, j0 = t0 + tj * UT;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    zc acc[4][4];
#pragma unroll
    for(int i = 0; i < 4; i++)
#pragma unroll
        for(int j = 0; j < 4; j++) acc[i][j] = mk(0.0, 0.0);
    for(unsigned p0 = 0; p0 < nb; p0 += 16) {
        __syncthreads();
        for(int q = threadIdx.x; q < 16 * UT; q += 256) {
            const int rr = q / 16, pp = q % 16;
            const unsigned p = p0 + pp;
            const unsigned gi = i0 + rr, gj = j0 + rr;
            Xi[pp][rr] = (gi < n && p < nb) ? A[(size_t)gi * n + kb + p] : mk(0.0, 0.0);
            Xj[pp][rr] = (gj < n && p < nb) ? A[(size_t)gj * n + kb + p] : mk(0.0, 0.0);
        }
        __syncthreads();
#pragma unroll
        for(int p = 0; p < 16; p++) {
            zc xa[4], xb[4];
#pragma unroll
            for(int i = 0; i < 4; i++) xa[i] = Xi[p][ty + 16 * i];
#pragma unroll
            for(int j = 0; j < 4; j++) xb[j] = Xj[p][tx + 16 * j];
#pragma unroll
            for(int i = 0; i < 4; i++)
#pragma unroll
                for(int j = 0; j < 4; j++) cmac_conj(acc[i][j], xb[j], xa[i]);  // += xa conj(xb)
        }
    }
#pragma unroll
    for(int i = 0; i < 4; i++) {
        const unsigned gi = i0 + ty + 16 * i;
        if(gi >= n) continue;
#pragma unroll
        for(int j = 0; j < 4; j++) {
            const unsigned gj = j0 + tx + 16 * j;
            if(gj >= n || gj > gi) continue;
            zc& dst = A[(size_t)gi * n + gj];
            dst = dst - acc[i][j];
        }
    }
}

// forward substitution step for block kb: warp 0 of every CTA solves L_kk y_k = b_k
// (identically; lane j owns y_j), CTA 0 stores y_k into y_out (never into b, which
// CTAs that start later still read), and all CTAs update the rows of b below.
__global__ void __launch_bounds__(256) fwd_block_kernel(const zc* __restrict__ L, unsigned n, unsigned kb,
                                                        zc* __restrict__ b, zc* __restrict__ y_out) {
    __shared__ zc y[NB];
    const unsigned nb = min((unsigned)NB, n - kb);
    if(threadIdx.x < 32) {
        const unsigned lane = threadIdx.x;
        zc v = lane < nb ? b[kb + lane] : mk(0.0, 0.0);
        for(unsigned j = 0; j < nb; j++) {
            zc yj = (1.0 / L[(size_t)(kb + j) * n + kb + j].re) * v;
            yj.re = __shfl_sync(0xffffffffu, yj.re, j);
            yj.im = __shfl_sync(0xffffffffu, yj.im, j);
            if(lane == j) v = yj;
            else if(lane > j && lane < nb) v = v - L[(size_t)(kb + lane) * n + kb + j] * yj;
        }
        if(lane < nb) y[lane] = v;
    }
    __syncthreads();
    if(blockIdx.x == 0 && threadIdx.x < nb) y_out[kb + threadIdx.x] = y[threadIdx.x];
    for(size_t i = kb + nb + (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        zc acc = mk(0.0, 0.0);
        for(unsigned p = 0; p < nb; p++) cmac(acc, L[i * n + kb + p], y[p]);
        b[i] = b[i] - acc;
    }
}

// backward substitution step for block kb with L^H (lane j owns x_j, last first);
// x_k goes to x_out, the rows of b above the block are updated in place
__global__ void __launch_bounds__(256) bwd_block_kernel(const zc* __restrict__ L, unsigned n, unsigned kb,
                                                        zc* __restrict__ b, zc* __restrict__ x_out) {
    __shared__ zc x[NB];
    const unsigned nb = min((unsigned)NB, n - kb);
    if(threadIdx.x < 32) {
        const unsigned lane = threadIdx.x;
        zc v = lane < nb ? b[kb + lane] : mk(0.0, 0.0);
        for(int j = (int)nb - 1; j >= 0; j--) {
            zc xj = (1.0 / L[(size_t)(kb + j) * n + kb + j].re) * v;
            xj.re = __shfl_sync(0xffffffffu, xj.re, j);
            xj.im = __shfl_sync(0xffffffffu, xj.im, j);
            if((int)lane == j) v = xj;
            else if((int)lane < j) v = v - conj(L[(size_t)(kb + j) * n + kb + lane]) * xj;
        }
        if(lane < nb) x[lane] = v;
    }
    __syncthreads();
    if(blockIdx.x == 0 && threadIdx.x < nb) x_out[kb + threadIdx.x] = x[threadIdx.x];
    for(size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < kb; i += (size_t)gridDim.x * blockDim.x) {
        zc acc = mk(0.0, 0.0);
        for(unsigned q = 0; q < nb; q++) cmac_conj(acc, L[(size_t)(kb + q) * n + i], x[q]);
        b[i] = b[i] - acc;
    }
}

// r = F - (S + shift I) x, one warp per row
__global__ void residual_kernel(const zc* __restrict__ S, unsigned n, double shift, const zc* __restrict__ x,
                                const zc* __restrict__ F, zc* __restrict__ r) {
    const size_t i = (size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if(i >= n) return;
    zc acc = mk(0.0, 0.0);
    for(unsigned j = lane; j < n; j += 32) cmac(acc, S[i * n + j], x[j]);
    acc = warp_sum(acc);
    if(lane == 0) r[i] = F[i] - acc - shift * x[i];
}

__global__ void axpy_kernel(zc* __restrict__ x, const zc* __restrict__ c, unsigned n) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i < n) x[i] += c[i];
}

// info[0] = ||r|| / ||F|| before refinement, info[1] after
__global__ void norm_ratio_kernel(const zc* __restrict__ r, const zc* __restrict__ F, unsigned n, double* out) {
    __shared__ double sh[2][32];
    double a = 0.0, b = 0.0;
    for(unsigned i = threadIdx.x; i < n; i += blockDim.x) {
        a += norm2(r[i]);
        b += norm2(F[i]);
    }
    a = warp_sum(a);
    b = warp_sum(b);
    if((threadIdx.x & 31) == 0) { sh[0][threadIdx.x >> 5] = a; sh[1][threadIdx.x >> 5] = b; }
    __syncthreads();
    if(threadIdx.x == 0) {
        double ta = 0.0, tb = 0.0;
        for(unsigned w = 0; w < (blockDim.x >> 5); w++) { ta += sh[0][w]; tb += sh[1][w]; }
        *out = tb > 0.0 ? sqrt(ta / tb) : sqrt(ta);
    }
}

void panel(zc* A, unsigned n, unsigned kb, unsigned* status, cudaStream_t st) {
    potrf_diag_kernel<<<1, NB * NB, 0, st>>>(A, n, kb, status);
    check_launch("potrf_diag_kernel");
    const unsigned nb = min((unsigned)NB, n - kb);
    const unsigned below = n - kb - nb;
    if(below) {
        trsm_panel_kernel<<<(below + 7) / 8, 256, 0, st>>>(A, n, kb);
        check_launch("trsm_panel_kernel");
    }
}

// Right-looking blocked Cholesky with look-ahead: after panel k, the first tile
// column of the trailing matrix (it holds panels k+1, k+2) is updated first; panel
// k+1 is then factorised on a side stream while the rest of the trailing update of
// step k runs, hiding the serial diagonal factorisation and panel solve.
void cholesky(ann_tdvp_impl& td, zc* A, unsigned n, unsigned* status, cudaStream_t st) {
    ensure_side_stream(td);
    panel(A, n, 0, status, st);
    for(unsigned kb = 0; kb < n; kb += NB) {
        const unsigned nb = min((unsigned)NB, n - kb);
        const unsigned below = n - kb - nb;
        if(below == 0) break;
        const unsigned tiles = (below + UT - 1) / UT;
        herk_update_kernel<<<tiles, 256, 0, st>>>(A, n, kb, nb, 1);
        check_launch("herk_update_kernel");
        // panel k+1 on the side stream, after the first-column update
        ANN_CUDA(cudaEventRecord(td.side_ev[0], st));
        ANN_CUDA(cudaStreamWaitEvent(td.side, td.side_ev[0], 0));
        panel(A, n, kb + nb, status, td.side);
        ANN_CUDA(cudaEventRecord(td.side_ev[1], td.side));
        if(tiles > 1) {
            herk_update_kernel<<<(tiles - 1) * tiles / 2, 256, 0, st>>>(A, n, kb, nb, 0);
            check_launch("herk_update_kernel");
        }
        ANN_CUDA(cudaStreamWaitEvent(st, td.side_ev[1], 0));
    }
}

// b <- (L L^H)^{-1} b; tmp (n entries) holds the intermediate y = L^{-1} b
void solve_in_place(const zc* L, unsigned n, zc* b, zc* tmp, cudaStream_t st) {
    for(unsigned kb = 0; kb < n; kb += NB) {
        const unsigned below = n - kb - min((unsigned)NB, n - kb);
        const unsigned grid = below ? min(132u, (below + 255) / 256) : 1u;
        fwd_block_kernel<<<grid, 256, 0, st>>>(L, n, kb, b, tmp);
        check_launch("fwd_block_kernel");
    }
    const unsigned last = ((n - 1) / NB) * NB;
    for(int kb = (int)last; kb >= 0; kb -= NB) {
        const unsigned grid = kb ? min(132u, ((unsigned)kb + 255) / 256) : 1u;
        bwd_block_kernel<<<grid, 256, 0, st>>>(L, n, (unsigned)kb, tmp, b);
        check_launch("bwd_block_kernel");
    }
}

}  // namespace

// The panel work of the look-ahead runs at the highest stream priority: the CTA
// scheduler then starts it as soon as an SM frees up, ahead of the queued CTAs of
// the trailing update it overlaps with.
void ensure_side_stream(ann_tdvp_impl& td) {
    if(td.side) return;
    int lo = 0, hi = 0;
    ANN_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    ANN_CUDA(cudaStreamCreateWithPriority(&td.side, cudaStreamNonBlocking, hi));
    for(auto& e : td.side_ev) ANN_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
}

namespace {
__global__ void widen_S_kernel(const float2* __restrict__ s32, double2* __restrict__ s, size_t nn) {
    for(size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += (size_t)gridDim.x * blockDim.x) {
        const float2 v = s32[k];
        s[k] = make_double2(widen(v.x), widen(v.y));
    }
}
}  // namespace

const cplx<double>* S64(ann_tdvp_impl& td, cudaStream_t st) {
    if(td.S_in32 && !td.S64_fresh) {
        const size_t nn = (size_t)td.Np * td.Np;
        td.S.ensure(nn * 16);
        widen_S_kernel<<<152 * 8, 256, 0, st>>>(td.S32.as<float2>(), td.S.as<double2>(), nn);
        check_launch("widen_S_kernel");
        td.S64_fresh = true;
    }
    return td.S.as<cplx<double>>();
}

void sr_solve(ann_tdvp_impl& td, double shift, unsigned* status, cudaStream_t st) {
    const unsigned n = td.Np;
    const size_t nn = (size_t)n * n;
    td.L.ensure(nn * sizeof(zc));
    td.delta.ensure(n * sizeof(zc));
    td.resid.ensure(2 * n * sizeof(zc) + 2 * sizeof(double));
    td.tmp64.ensure(n * sizeof(zc));
    zc* A = td.L.as<zc>();
    zc* tmp = td.tmp64.as<zc>();
    zc* x = td.delta.as<zc>();
    zc* r = td.resid.as<zc>();
    double* info = reinterpret_cast<double*>(r + 2 * n);
    const zc* S = S64(td, st);
    const zc* F = td.F.as<zc>();
    copy_shift_kernel<<<(unsigned)((nn + 255) / 256), 256, 0, st>>>(S, A, n, shift);
    check_launch("copy_shift_kernel");
    cholesky(td, A, n, status, st);
    ANN_CUDA(cudaMemcpyAsync(x, F, n * sizeof(zc), cudaMemcpyDeviceToDevice, st));
    solve_in_place(A, n, x, tmp, st);
    // one step of iterative refinement against S + shift I
    residual_kernel<<<(n + 7) / 8, 256, 0, st>>>(S, n, shift, x, F, r);
    check_launch("residual_kernel");
    norm_ratio_kernel<<<1, 1024, 0, st>>>(r, F, n, info);
    check_launch("norm_ratio_kernel");
    solve_in_place(A, n, r, tmp, st);
    axpy_kernel<<<(n + 255) / 256, 256, 0, st>>>(x, r, n);
    check_launch("axpy_kernel");
    residual_kernel<<<(n + 7) / 8, 256, 0, st>>>(S, n, shift, x, F, r + n);
    check_launch("residual_kernel");
    norm_ratio_kernel<<<1, 1024, 0, st>>>(r + n, F, n, info + 1);
    check_launch("norm_ratio_kernel");
}

namespace {
__global__ void sr_update_kernel(zc* __restrict__ p, const zc* __restrict__ d, double lr, unsigned n) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i < n) p[i] = p[i] - lr * d[i];
}
}  // namespace

void sr_update(ann_psi_impl& psi, const cplx<double>* delta, double lr, cudaStream_t st) {
    sr_update_kernel<<<(psi.Np + 255) / 256, 256, 0, st>>>(psi.params.as<zc>(), delta, lr, psi.Np);
    check_launch("sr_update_kernel");
    psi_prepare(psi, st);
}

}  // namespace ann
