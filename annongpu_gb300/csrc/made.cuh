// Learned proposal: MADE (masked autoencoder for distribution estimation; Germain,
// Gregor, Murray, Larochelle, ICML 2015), one hidden layer of width H over N spins in
// the natural order. Hidden unit k has degree d_k in [1, N-1]: input i feeds it iff
// i < d_k and it feeds output j iff d_k <= j, so logit j depends on spins < j only.
//     pre = W1 x + b1,  h = relu(pre),  l = W2 h + b2,  x_j = 1 for spin up
//     q(s) = prod_j sigmoid(l_j)^{x_j} sigmoid(-l_j)^{1 - x_j}
// The kernels read BF16 copies of the weights (global: W1t[i][k], W2t[k][j]; staged in
// shared memory as W1t[i][k] and W2[j][k], so a warp reading one row with lanes over
// the hidden units k touches consecutive addresses) and accumulate in FP32. Masked weights are held at exactly zero, so the forward pass
// needs no mask.
//
// Used by the sampler as a Metropolis-Hastings independence proposal: s' ~ q,
// accepted with min(1, |psi(s')|^2 q(s) / (|psi(s)|^2 q(s'))), which keeps |psi|^2
// the stationary distribution exactly.
#pragma once

#include <cuda_bf16.h>

#include "ann_common.cuh"

namespace ann {

constexpr unsigned kMadeMaxN = 128;

// weights staged in shared memory by the calling CTA
struct MadeSm {
    unsigned N, H;
    const __nv_bfloat16* W1t;  // [i][k]
    const float* b1;
    const __nv_bfloat16* W2;   // [j][k]
    const float* b2;
};

__host__ __device__ inline size_t made_smem_bytes(unsigned N, unsigned H) {
    return ((size_t)2 * N * H * sizeof(__nv_bfloat16) + (size_t)(H + N) * sizeof(float) + 15) & ~(size_t)15;
}

__device__ inline MadeSm made_stage(const MadeDev& m, unsigned char* smem) {
    MadeSm s;
    s.N = m.N;
    s.H = m.H;
    __nv_bfloat16* w1 = reinterpret_cast<__nv_bfloat16*>(smem);
    __nv_bfloat16* w2 = w1 + (size_t)m.N * m.H;
    float* b1 = reinterpret_cast<float*>(w2 + (size_t)m.N * m.H);
    float* b2 = b1 + m.H;
    const size_t nw = (size_t)m.N * m.H;
    for(size_t k = threadIdx.x; k < nw; k += blockDim.x) {
        w1[k] = m.W1t[k];
        const size_t j = k / m.H, kk = k % m.H;
        w2[k] = m.W2t[kk * m.N + j];  // W2[j][kk]
    }
    for(unsigned k = threadIdx.x; k < m.H; k += blockDim.x) b1[k] = m.b1[k];
    for(unsigned k = threadIdx.x; k < m.N; k += blockDim.x) b2[k] = m.b2[k];
    s.W1t = w1;
    s.b1 = b1;
    s.W2 = w2;
    s.b2 = b2;
    return s;
}

// the weights as stored in global memory (read through L1: for samplers whose local
// sweeps outweigh the learned moves, so shared memory is left to occupancy)
__device__ __forceinline__ MadeSm made_global(const MadeDev& m) {
    return MadeSm{m.N, m.H, m.W1t, m.b1, m.W2, m.b2};
}

__device__ __forceinline__ float softplusf(float z) {
    return z > 0.f ? z + log1pf(expf(-z)) : log1pf(expf(z));
}

template<int NW>
__device__ __forceinline__ float xbit(const Conf<NW>& s, unsigned i) {
    return spin_bit(s, i) ? 1.f : 0.f;
}

// log q(s), cooperative over a team of TL lanes (lane: the lane within the team; the sums
// per virtual lane, as in the sampler, so any team gives the whole warp's value); h is a
// per-team scratch of H floats
template<int NW, int TL = 32>
__device__ float made_logq(const MadeSm& m, const Conf<NW>& s, float* h, int lane) {
    const unsigned mask = team_mask<TL>();
    for(unsigned k = lane; k < m.H; k += TL) {
        float pre = m.b1[k];
        for(unsigned i = 0; i < m.N; i++)
            if(spin_bit(s, i)) pre += __bfloat162float(m.W1t[i * m.H + k]);
        h[k] = fmaxf(pre, 0.f);
    }
    __syncwarp(mask);
    // logit j: lanes split the hidden units (consecutive W2[j][k]), butterfly sum
    float acc = 0.f;
    for(unsigned j = 0; j < m.N; j++) {
        float part[kVirt<TL>];
#pragma unroll
        for(int v = 0; v < kVirt<TL>; v++) {
            part[v] = 0.f;
            for(unsigned k = lane + v * TL; k < m.H; k += 32)
                part[v] = fmaf(__bfloat162float(m.W2[j * m.H + k]), h[k], part[v]);
        }
        const float l = m.b2[j] + team_total<TL>(part);
        acc -= spin_bit(s, j) ? softplusf(-l) : softplusf(l);
    }
    __syncwarp(mask);
    return acc;
}

// Draws s ~ q autoregressively; uniforms from Philox counters (c0, c1, c2, 3 + 4 b),
// word j % 4 of block b = j / 4, u_j = (word >> 8) 2^-24; x_j = 1 iff u_j < sigmoid(l_j).
// Team lane k keeps the pre-activations of hidden units k, k+TL, ... in registers; the
// team's lanes hold the uniforms of 4 TL spins (N <= 4 TL).
template<int NW, int HU, int TL = 32>
__device__ float made_sample(const MadeSm& m, uint32_t k0, uint32_t k1, uint32_t c0, uint32_t c1, uint32_t c2,
                             Conf<NW>& s, int lane) {
    const unsigned mask = team_mask<TL>();
    const u32x4 rr = philox4x32_10(k0, k1, u32x4{c0, c1, c2, 3u + 4u * (uint32_t)lane});
    float pre[HU];
#pragma unroll
    for(int u = 0; u < HU; u++) {
        const unsigned k = u * TL + lane;
        pre[u] = k < m.H ? m.b1[k] : 0.f;
    }
    for(int w = 0; w < NW; w++) s.w[w] = 0;
    float logq = 0.f;
    for(unsigned j = 0; j < m.N; j++) {
        float part[kVirt<TL>];
#pragma unroll
        for(int v = 0; v < kVirt<TL>; v++) part[v] = 0.f;
#pragma unroll
        for(int u = 0; u < HU; u++) {
            const unsigned k = u * TL + lane;
            if(k < m.H) part[u % kVirt<TL>] = fmaf(__bfloat162float(m.W2[j * m.H + k]), fmaxf(pre[u], 0.f), part[u % kVirt<TL>]);
        }
        const float l = m.b2[j] + team_total<TL>(part);
        const uint32_t word_src = (j & 3u) == 0 ? rr.x : (j & 3u) == 1 ? rr.y : (j & 3u) == 2 ? rr.z : rr.w;
        const uint32_t word = __shfl_sync(mask, word_src, j >> 2, TL);
        const float uj = __uint2float_rz(word >> 8) * 0x1.0p-24f;
        const float p = 1.f / (1.f + expf(-l));
        const bool up = uj < p;
        logq -= up ? softplusf(-l) : softplusf(l);
        if(up) {
            s.w[j >> 6] |= (uint64_t)1 << (j & 63u);
#pragma unroll
            for(int u = 0; u < HU; u++) {
                const unsigned k = u * TL + lane;
                if(k < m.H) pre[u] += __bfloat162float(m.W1t[j * m.H + k]);
            }
        }
    }
    return logq;
}

}  // namespace ann
