// MADE learned proposal: batched log q, sampling, and training (forward, backward,
// Adam) on configurations the chains generate. See made.cuh for the model.
//
// Training step on a batch of B configurations (loss = mean -log q):
//   pre = X W1^T + b1 (B x H), l = relu(pre) W2^T + b2 (B x N)          forward GEMMs
//   dl = (sigmoid(l) - X) / B
//   dW2 = dl^T relu(pre), db2 = sum dl, dh = (dl W2) * [pre > 0]           backward GEMMs
//   dW1 = dh^T X, db1 = sum dh
//   Adam (Kingma & Ba 2015) on the FP32 master weights, masked gradients, then the
//   BF16 transposed copies the samplers read are refreshed.
// The GEMMs run on the tensor cores (made_tc.cu: tcgen05 BF16 MMAs with FP32 accumulation
// in tensor memory); FP32 activations and gradients enter as BF16 hi + lo pairs, the
// weights as the BF16 copies the samplers read.
#include <algorithm>
#include <cmath>
#include <initializer_list>
#include <random>

#include "ann_internal.hpp"
#include "made.cuh"

namespace ann {

namespace {

// column sums over slabs of kSplitK rows; split_reduce_kernel adds the slabs in order
// (deterministic)
constexpr unsigned kSplitK = 128;

__global__ void split_reduce_kernel(const float* __restrict__ P, unsigned splits, size_t mn, float* __restrict__ C) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= mn) return;
    float acc = 0.f;
    for(unsigned z = 0; z < splits; z++) acc += P[(size_t)z * mn + i];
    C[i] = acc;
}

// GEMM operand extents: K (columns) padded to 64 values; rows to a whole number of tiles
// (128-row A tiles, B tiles of 64, 128 or 256 rows), the padding zero
__host__ __device__ inline unsigned pad64(unsigned x) { return (x + 63u) & ~63u; }
__host__ __device__ inline unsigned prow(unsigned x) { return x <= 128u ? 128u : (x + 255u) & ~255u; }

// BF16 operands of the training GEMMs: W1g[k][i] = W1[k][i] (prow(H) x N64),
// W2g[j][k] = W2[j][k] (prow(N) x H64), W2Tg[k][j] = W2[j][k] (prow(H) x N64)
__global__ void refresh_gemm_kernel(const float* __restrict__ W1, const float* __restrict__ W2, unsigned N, unsigned H,
                                    __nv_bfloat16* __restrict__ W1g, __nv_bfloat16* __restrict__ W2g,
                                    __nv_bfloat16* __restrict__ W2Tg) {
    const unsigned N64 = pad64(N), H64 = pad64(H);
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if(idx < (size_t)prow(H) * N64) {
        const unsigned k = (unsigned)(idx / N64), j = (unsigned)(idx % N64);
        const bool in = k < H && j < N;
        W1g[idx] = __float2bfloat16_rn(in ? W1[(size_t)k * N + j] : 0.f);
        W2Tg[idx] = __float2bfloat16_rn(in ? W2[(size_t)j * H + k] : 0.f);
    }
    if(idx < (size_t)prow(N) * H64) {
        const unsigned j = (unsigned)(idx / H64), k = (unsigned)(idx % H64);
        W2g[idx] = __float2bfloat16_rn(j < N && k < H ? W2[(size_t)j * H + k] : 0.f);
    }
}


__global__ void bits_kernel(const uint64_t* __restrict__ confs, unsigned B, unsigned N, float* __restrict__ X) {
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if(idx >= (size_t)B * N) return;
    const unsigned b = (unsigned)(idx / N), i = (unsigned)(idx % N);
    X[idx] = (float)((confs[(size_t)b * kMaxWords + (i >> 6)] >> (i & 63u)) & 1u);
}

// relu in place on a copy: h = max(pre, 0)
__global__ void relu_kernel(const float* __restrict__ pre, float* __restrict__ h, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if(i < n) h[i] = fmaxf(pre[i], 0.f);
}

// dl = (sigmoid(l) - x) / B ; loss partials of -log q per row
__global__ void dlogits_kernel(const float* __restrict__ l, const float* __restrict__ X, unsigned B, unsigned N,
                               float* __restrict__ dl, float* __restrict__ row_loss) {
    const unsigned b = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if(b >= B) return;
    float acc = 0.f;
    for(unsigned j = lane; j < N; j += 32) {
        const float z = l[(size_t)b * N + j], x = X[(size_t)b * N + j];
        dl[(size_t)b * N + j] = (1.f / (1.f + expf(-z)) - x) / (float)B;
        acc += x > 0.5f ? softplusf(-z) : softplusf(z);
    }
    acc = warp_sum(acc);
    if(lane == 0) row_loss[b] = acc;
}

// column sums: out[n] = sum_m X[m][n]
// partial column sums over slabs of kSplitK rows (blockIdx.y); split_reduce_kernel
// adds the slabs in order
__global__ void colsum_kernel(const float* __restrict__ X, unsigned M, unsigned Nn, float* __restrict__ part) {
    const unsigned n = blockIdx.x * blockDim.x + threadIdx.x;
    if(n >= Nn) return;
    const unsigned m0 = blockIdx.y * 128u, m1 = min(M, m0 + 128u);
    float s = 0.f;
    for(unsigned m = m0; m < m1; m++) s += X[(size_t)m * Nn + n];
    part[(size_t)blockIdx.y * Nn + n] = s;
}

struct AdamArgs {
    float lr, beta1, beta2, eps, c1, c2;  // c1 = 1 - beta1^t, c2 = 1 - beta2^t
};

// kind 0: W1 (H x N, mask i < d_k), 1: W2 (N x H, mask d_k <= j), 2: bias (no mask)
__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m1,
                            float* __restrict__ m2, size_t n, unsigned N, unsigned H, const uint16_t* __restrict__ deg,
                            int kind, AdamArgs a) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= n) return;
    bool live = true;
    if(kind == 0) live = (i % N) < deg[i / N];
    else if(kind == 1) live = deg[i % H] <= (i / H);
    if(!live) {
        p[i] = 0.f;
        return;
    }
    const float gi = g[i];
    const float mm = a.beta1 * m1[i] + (1.f - a.beta1) * gi;
    const float vv = a.beta2 * m2[i] + (1.f - a.beta2) * gi * gi;
    m1[i] = mm;
    m2[i] = vv;
    p[i] -= a.lr * (mm / a.c1) / (sqrtf(vv / a.c2) + a.eps);
}

// BF16 copies: W1t[i][k] = W1[k][i], W2t[k][j] = W2[j][k], W2b[j][k] = W2[j][k]
__global__ void refresh_bf16_kernel(const float* __restrict__ W1, const float* __restrict__ W2, unsigned N, unsigned H,
                                    __nv_bfloat16* __restrict__ W1t, __nv_bfloat16* __restrict__ W2t,
                                    __nv_bfloat16* __restrict__ W2b) {
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if(idx >= (size_t)N * H) return;
    const unsigned i = (unsigned)(idx / H), k = (unsigned)(idx % H);
    W1t[idx] = __float2bfloat16_rn(W1[(size_t)k * N + i]);
    const unsigned kk = (unsigned)(idx / N), j = (unsigned)(idx % N);
    W2t[idx] = __float2bfloat16_rn(W2[(size_t)j * H + kk]);
    W2b[idx] = __float2bfloat16_rn(W2[idx]);
}

__global__ void __launch_bounds__(256) made_logq_kernel(MadeDev m, const uint64_t* __restrict__ confs, size_t n,
                                                        double* __restrict__ out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const MadeSm ms = made_stage(m, smem_raw);
    float* h = reinterpret_cast<float*>(smem_raw + made_smem_bytes(m.N, m.H)) + (threadIdx.x >> 5) * m.H;
    __syncthreads();
    const size_t idx = (size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if(idx >= n) return;
    Conf<2> s;
    s.w[0] = confs[idx * kMaxWords];
    s.w[1] = confs[idx * kMaxWords + 1];
    const float lq = made_logq(ms, s, h, threadIdx.x & 31);
    if((threadIdx.x & 31) == 0) out[idx] = lq;
}

template<int HU>
__global__ void __launch_bounds__(256) made_sample_kernel(MadeDev m, uint32_t k0, uint32_t k1, uint64_t first,
                                                          size_t n, uint64_t* __restrict__ confs,
                                                          double* __restrict__ logq) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const MadeSm ms = made_stage(m, smem_raw);
    __syncthreads();
    const size_t idx = (size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if(idx >= n) return;
    const uint64_t q = first + idx;
    Conf<2> s;
    const float lq = made_sample<2, HU>(ms, k0, k1, (uint32_t)q, (uint32_t)(q >> 32), 0xFFFFFFFFu, s, threadIdx.x & 31);
    if((threadIdx.x & 31) == 0) {
        confs[idx * kMaxWords] = s.w[0];
        confs[idx * kMaxWords + 1] = s.w[1];
        logq[idx] = lq;
    }
}

__global__ void loss_sum_kernel(const float* __restrict__ row_loss, unsigned B, double* out) {
    __shared__ double sh[32];
    double acc = 0.0;
    for(unsigned b = threadIdx.x; b < B; b += blockDim.x) acc += row_loss[b];
    acc = warp_sum(acc);
    if((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if(threadIdx.x == 0) {
        double t = 0.0;
        for(unsigned w = 0; w < (blockDim.x >> 5); w++) t += sh[w];
        *out = t / B;
    }
}

}  // namespace

MadeDev made_view(const ann_made_impl& m) {
    MadeDev d;
    d.N = m.N;
    d.H = m.H;
    d.W1t = m.W1t.as<__nv_bfloat16>();
    d.b1 = m.b1.as<float>();
    d.W2t = m.W2t.as<__nv_bfloat16>();
    d.b2 = m.b2.as<float>();
    d.W2 = m.W2b.as<__nv_bfloat16>();
    return d;
}

void made_refresh(ann_made_impl& m, cudaStream_t st) {
    const size_t nh = (size_t)m.N * m.H;
    refresh_bf16_kernel<<<(unsigned)((nh + 255) / 256), 256, 0, st>>>(m.W1.as<float>(), m.W2.as<float>(), m.N, m.H,
                                                                        m.W1t.as<__nv_bfloat16>(),
                                                                        m.W2t.as<__nv_bfloat16>(),
                                                                        m.W2b.as<__nv_bfloat16>());
    check_launch("refresh_bf16_kernel");
    const size_t ng = std::max((size_t)prow(m.H) * pad64(m.N), (size_t)prow(m.N) * pad64(m.H));
    m.W1g.ensure((size_t)prow(m.H) * pad64(m.N) * 2);
    m.W2Tg.ensure((size_t)prow(m.H) * pad64(m.N) * 2);
    m.W2g.ensure((size_t)prow(m.N) * pad64(m.H) * 2);
    refresh_gemm_kernel<<<(unsigned)((ng + 255) / 256), 256, 0, st>>>(m.W1.as<float>(), m.W2.as<float>(), m.N, m.H,
                                                                        m.W1g.as<__nv_bfloat16>(),
                                                                        m.W2g.as<__nv_bfloat16>(),
                                                                        m.W2Tg.as<__nv_bfloat16>());
    check_launch("refresh_gemm_kernel");
}

void made_init(ann_made_impl& m, uint64_t seed) {
    const unsigned N = m.N, H = m.H;
    std::vector<uint16_t> deg(H);
    for(unsigned k = 0; k < H; k++) deg[k] = (uint16_t)((k % (N > 1 ? N - 1 : 1)) + 1);
    std::mt19937_64 gen(seed);
    std::uniform_real_distribution<float> U(-1.f, 1.f);
    std::vector<float> W1((size_t)H * N, 0.f), W2((size_t)N * H, 0.f), b1(H, 0.f), b2(N, 0.f);
    const float s1 = std::sqrt(6.f / (N + H)), s2 = std::sqrt(6.f / (N + H));
    for(unsigned k = 0; k < H; k++)
        for(unsigned i = 0; i < N; i++) W1[(size_t)k * N + i] = i < deg[k] ? s1 * U(gen) : 0.f;
    for(unsigned j = 0; j < N; j++)
        for(unsigned k = 0; k < H; k++) W2[(size_t)j * H + k] = deg[k] <= j ? 0.1f * s2 * U(gen) : 0.f;
    upload(m.deg, deg.data(), deg.size() * 2);
    upload(m.W1, W1.data(), W1.size() * 4);
    upload(m.W2, W2.data(), W2.size() * 4);
    upload(m.b1, b1.data(), b1.size() * 4);
    upload(m.b2, b2.data(), b2.size() * 4);
    const size_t nh = (size_t)N * H;
    for(DevBuf* b : {&m.mW1, &m.vW1, &m.mW2, &m.vW2, &m.gW1, &m.gW2}) {
        b->ensure(nh * 4);
        ANN_CUDA(cudaMemset(b->p, 0, nh * 4));
    }
    for(DevBuf* b : {&m.mb1, &m.vb1, &m.gb1}) {
        b->ensure(H * 4);
        ANN_CUDA(cudaMemset(b->p, 0, H * 4));
    }
    for(DevBuf* b : {&m.mb2, &m.vb2, &m.gb2}) {
        b->ensure(N * 4);
        ANN_CUDA(cudaMemset(b->p, 0, N * 4));
    }
    // the clears run on the legacy default stream, which does not order with the
    // non-blocking stream the training runs on: complete them here
    ANN_CUDA(cudaDeviceSynchronize());
    m.W1t.ensure(nh * 2);
    m.W2t.ensure(nh * 2);
    m.W2b.ensure(nh * 2);
    m.adam_t = 0;
    made_refresh(m, nullptr);
    ANN_CUDA(cudaDeviceSynchronize());
}

// gradient of the mean -log q over confs[0..B) into m.g*; loss to *loss_dev
void colsum(const float* X, unsigned M, unsigned Nn, float* out, DevBuf& scratch, cudaStream_t st) {
    const unsigned slabs = (M + kSplitK - 1) / kSplitK;
    scratch.ensure((size_t)slabs * Nn * sizeof(float));
    colsum_kernel<<<dim3((Nn + 127) / 128, slabs), 128, 0, st>>>(X, M, Nn, scratch.as<float>());
    check_launch("colsum_kernel");
    split_reduce_kernel<<<(Nn + 255) / 256, 256, 0, st>>>(scratch.as<float>(), slabs, Nn, out);
    check_launch("split_reduce_kernel");
}

void made_gradient(ann_made_impl& m, const uint64_t* confs, unsigned B, double* loss_dev, cudaStream_t st) {
    const unsigned N = m.N, H = m.H;
    const unsigned N64 = pad64(N), H64 = pad64(H), B64 = pad64(B);
    const unsigned Br = prow(B), Nr = prow(N), Hr = prow(H);
    m.X.ensure((size_t)B * N * 4);
    m.pre.ensure((size_t)B * H * 4);
    m.hbuf.ensure((size_t)B * H * 4);
    m.l.ensure((size_t)B * N * 4);
    m.dl.ensure((size_t)B * N * 4);
    m.dh.ensure((size_t)B * H * 4);
    m.row_loss.ensure((size_t)B * 4);
    m.Xg.ensure((size_t)Br * N64 * 2);
    m.XTg.ensure((size_t)Nr * B64 * 2);
    m.hs.ensure((size_t)Br * 2 * H64 * 2);
    m.hTs.ensure((size_t)Hr * 2 * B64 * 2);
    m.dls.ensure((size_t)Br * 2 * N64 * 2);
    m.dlTs.ensure((size_t)Nr * 2 * B64 * 2);
    m.dhTs.ensure((size_t)Hr * 2 * B64 * 2);
    float* X = m.X.as<float>();
    float* pre = m.pre.as<float>();
    float* h = m.hbuf.as<float>();
    float* l = m.l.as<float>();
    float* dl = m.dl.as<float>();
    float* dh = m.dh.as<float>();
    // weight gradients: K = the batch, split over CTAs in chunks of >= 4 K steps
    const unsigned splits = std::max(1u, std::min(16u, B64 / 256u));
    auto gemm = [&](const void* A, unsigned ar, unsigned ac, const void* Bm, unsigned br, unsigned bc, unsigned M,
                    unsigned Nn, unsigned K, std::initializer_list<int> ao, std::initializer_list<int> bo, float* C,
                    size_t ldc, const float* bias, const float* aux, unsigned sp) {
        MadeGemm g{};
        g.A = A;
        g.a_rows = ar;
        g.a_cols = ac;
        g.B = Bm;
        g.b_rows = br;
        g.b_cols = bc;
        g.M = M;
        g.N = Nn;
        g.K = K;
        g.nseg = (unsigned)ao.size();
        int s = 0;
        for(int v : ao) g.aoff[s++] = v;
        s = 0;
        for(int v : bo) g.boff[s++] = v;
        g.C = C;
        g.ldc = ldc;
        g.bias = bias;
        g.aux = aux;
        g.splits = sp;
        made_gemm(g, m.kpart, st);
    };
    bits_kernel<<<(unsigned)(((size_t)B * N + 255) / 256), 256, 0, st>>>(confs, B, N, X);
    check_launch("bits_kernel");
    made_split_rows(X, B, N, N, m.Xg.p, N64, Br, N64, 0, false, st);   // X (exact in BF16)
    made_split_cols(X, B, N, N, m.XTg.p, B64, Nr, B64, 0, false, st);  // X^T
    // pre[b][k] = sum_i X[b][i] W1[k][i] + b1[k]
    gemm(m.Xg.p, Br, N64, m.W1g.p, Hr, N64, B, H, N64, {0}, {0}, pre, H, m.b1.as<float>(), nullptr, 1);
    relu_kernel<<<(unsigned)(((size_t)B * H + 255) / 256), 256, 0, st>>>(pre, h, (size_t)B * H);
    check_launch("relu_kernel");
    made_split_rows(h, B, H, H, m.hs.p, 2 * H64, Br, H64, H64, true, st);   // [h | h_lo]
    made_split_cols(h, B, H, H, m.hTs.p, 2 * B64, Hr, B64, B64, true, st);  // [h^T | lo]
    // l[b][j] = sum_k h[b][k] W2[j][k] + b2[j]   (hi.W2 + lo.W2)
    gemm(m.hs.p, Br, 2 * H64, m.W2g.p, Nr, H64, B, N, H64, {0, (int)H64}, {0, 0}, l, N, m.b2.as<float>(), nullptr, 1);
    dlogits_kernel<<<(B + 7) / 8, 256, 0, st>>>(l, X, B, N, dl, m.row_loss.as<float>());
    check_launch("dlogits_kernel");
    loss_sum_kernel<<<1, 256, 0, st>>>(m.row_loss.as<float>(), B, loss_dev);
    check_launch("loss_sum_kernel");
    made_split_rows(dl, B, N, N, m.dls.p, 2 * N64, Br, N64, N64, true, st);   // [dl | lo]
    made_split_cols(dl, B, N, N, m.dlTs.p, 2 * B64, Nr, B64, B64, true, st);  // [dl^T | lo]
    // dW2[j][k] = sum_b dl[b][j] h[b][k]   (hi.hi + lo.hi + hi.lo)
    gemm(m.dlTs.p, Nr, 2 * B64, m.hTs.p, Hr, 2 * B64, N, H, B64, {0, (int)B64, 0}, {0, 0, (int)B64},
         m.gW2.as<float>(), H, nullptr, nullptr, splits);
    colsum(dl, B, N, m.gb2.as<float>(), m.kpart, st);
    // dh[b][k] = sum_j dl[b][j] W2[j][k] * [pre > 0]   (the weights the forward pass used)
    gemm(m.dls.p, Br, 2 * N64, m.W2Tg.p, Hr, N64, B, H, N64, {0, (int)N64}, {0, 0}, dh, H, nullptr, pre, 1);
    made_split_cols(dh, B, H, H, m.dhTs.p, 2 * B64, Hr, B64, B64, true, st);  // [dh^T | lo]
    // dW1[k][i] = sum_b dh[b][k] X[b][i]   (hi.X + lo.X)
    gemm(m.dhTs.p, Hr, 2 * B64, m.XTg.p, Nr, B64, H, N, B64, {0, (int)B64}, {0, 0}, m.gW1.as<float>(), N, nullptr,
         nullptr, splits);
    colsum(dh, B, H, m.gb1.as<float>(), m.kpart, st);
}

void made_adam(ann_made_impl& m, float lr, cudaStream_t st) {
    m.adam_t++;
    AdamArgs a;
    a.lr = lr;
    a.beta1 = 0.9f;
    a.beta2 = 0.999f;
    a.eps = 1e-8f;
    a.c1 = 1.f - std::pow(0.9f, (float)m.adam_t);
    a.c2 = 1.f - std::pow(0.999f, (float)m.adam_t);
    const size_t nh = (size_t)m.N * m.H;
    const uint16_t* deg = m.deg.as<uint16_t>();
    adam_kernel<<<(unsigned)((nh + 255) / 256), 256, 0, st>>>(m.W1.as<float>(), m.gW1.as<float>(), m.mW1.as<float>(),
                                                              m.vW1.as<float>(), nh, m.N, m.H, deg, 0, a);
    check_launch("adam_kernel");
    adam_kernel<<<(unsigned)((nh + 255) / 256), 256, 0, st>>>(m.W2.as<float>(), m.gW2.as<float>(), m.mW2.as<float>(),
                                                              m.vW2.as<float>(), nh, m.N, m.H, deg, 1, a);
    check_launch("adam_kernel");
    adam_kernel<<<(m.H + 255) / 256, 256, 0, st>>>(m.b1.as<float>(), m.gb1.as<float>(), m.mb1.as<float>(),
                                                   m.vb1.as<float>(), m.H, m.N, m.H, deg, 2, a);
    check_launch("adam_kernel");
    adam_kernel<<<(m.N + 255) / 256, 256, 0, st>>>(m.b2.as<float>(), m.gb2.as<float>(), m.mb2.as<float>(),
                                                   m.vb2.as<float>(), m.N, m.N, m.H, deg, 2, a);
    check_launch("adam_kernel");
    made_refresh(m, st);
}

void made_logq_batch(const ann_made_impl& m, const uint64_t* confs, size_t n, double* out, cudaStream_t st) {
    const size_t smem = made_smem_bytes(m.N, m.H) + 8 * m.H * sizeof(float);
    if(smem > 48 * 1024)
        ANN_CUDA(cudaFuncSetAttribute(made_logq_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    made_logq_kernel<<<(unsigned)((n + 7) / 8), 256, smem, st>>>(made_view(m), confs, n, out);
    check_launch("made_logq_kernel");
}

void made_sample_batch(ann_made_impl& m, uint64_t seed, uint64_t first, size_t n, uint64_t* confs, double* logq,
                       cudaStream_t st) {
    const size_t smem = made_smem_bytes(m.N, m.H);
    const unsigned hu = (m.H + 31) / 32;
    auto launch = [&](auto kernel) {
        if(smem > 48 * 1024)
            ANN_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kernel<<<(unsigned)((n + 7) / 8), 256, smem, st>>>(made_view(m), (uint32_t)seed, (uint32_t)(seed >> 32), first,
                                                            n, confs, logq);
    };
    if(hu <= 4) launch(made_sample_kernel<4>);
    else if(hu <= 8) launch(made_sample_kernel<8>);
    else if(hu <= 16) launch(made_sample_kernel<16>);
    else throw Error(ANN_ERR_INVALID, "MADE hidden width above 512");
    check_launch("made_sample_kernel");
}

}  // namespace ann

using namespace ann;

namespace {
template<typename F>
int mguard(F&& f) {
    try {
        f();
        return ANN_OK;
    } catch(const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch(const std::exception& e) {
        set_last_error(e.what());
        return ANN_ERR_INVALID;
    }
}
void mneed(bool ok, const char* msg) {
    if(!ok) throw Error(ANN_ERR_INVALID, msg);
}
}  // namespace

extern "C" {

int ann_made_create(unsigned N, unsigned H, uint64_t seed, ann_made** out) {
    return mguard([&] {
        mneed(out != nullptr, "null argument");
        mneed(N >= 2 && N <= kMadeMaxN, "MADE needs 2 <= N <= 128");
        mneed(H >= 32 && H <= 512, "MADE hidden width must be in [32, 512]");
        auto* m = new ann_made();
        try {
            m->N = N;
            m->H = H;
            m->seed = seed;
            made_init(*m, seed);
        } catch(...) {
            delete m;
            throw;
        }
        *out = m;
    });
}

int ann_made_destroy(ann_made* m) {
    return mguard([&] { delete m; });
}

int ann_made_get_params(const ann_made* m, float* W1, float* b1, float* W2, float* b2) {
    return mguard([&] {
        mneed(m != nullptr, "null argument");
        ANN_CUDA(cudaDeviceSynchronize());
        const size_t nh = (size_t)m->N * m->H;
        if(W1) ANN_CUDA(cudaMemcpy(W1, m->W1.p, nh * 4, cudaMemcpyDeviceToHost));
        if(b1) ANN_CUDA(cudaMemcpy(b1, m->b1.p, m->H * 4, cudaMemcpyDeviceToHost));
        if(W2) ANN_CUDA(cudaMemcpy(W2, m->W2.p, nh * 4, cudaMemcpyDeviceToHost));
        if(b2) ANN_CUDA(cudaMemcpy(b2, m->b2.p, m->N * 4, cudaMemcpyDeviceToHost));
    });
}

int ann_made_set_params(ann_made* m, const float* W1, const float* b1, const float* W2, const float* b2) {
    return mguard([&] {
        mneed(m && W1 && b1 && W2 && b2, "null argument");
        const size_t nh = (size_t)m->N * m->H;
        ANN_CUDA(cudaMemcpy(m->W1.p, W1, nh * 4, cudaMemcpyHostToDevice));
        ANN_CUDA(cudaMemcpy(m->b1.p, b1, m->H * 4, cudaMemcpyHostToDevice));
        ANN_CUDA(cudaMemcpy(m->W2.p, W2, nh * 4, cudaMemcpyHostToDevice));
        ANN_CUDA(cudaMemcpy(m->b2.p, b2, m->N * 4, cudaMemcpyHostToDevice));
        made_refresh(*m, nullptr);
        ANN_CUDA(cudaDeviceSynchronize());
    });
}

int ann_made_log_prob(ann_made* m, const uint64_t* confs, unsigned n, double* out) {
    return mguard([&] {
        mneed(m && confs && out, "null argument");
        DevBuf c, o;
        upload(c, confs, (size_t)n * kMaxWords * 8);
        o.ensure((size_t)n * 8);
        made_logq_batch(*m, c.as<uint64_t>(), n, o.as<double>(), nullptr);
        ANN_CUDA(cudaMemcpy(out, o.p, (size_t)n * 8, cudaMemcpyDeviceToHost));
    });
}

int ann_made_sample(ann_made* m, unsigned n, uint64_t seed, uint64_t first, uint64_t* confs, double* logq) {
    return mguard([&] {
        mneed(m && confs, "null argument");
        DevBuf c, o;
        c.ensure((size_t)n * kMaxWords * 8);
        o.ensure((size_t)n * 8);
        made_sample_batch(*m, seed, first, n, c.as<uint64_t>(), o.as<double>(), nullptr);
        ANN_CUDA(cudaMemcpy(confs, c.p, (size_t)n * kMaxWords * 8, cudaMemcpyDeviceToHost));
        if(logq) ANN_CUDA(cudaMemcpy(logq, o.p, (size_t)n * 8, cudaMemcpyDeviceToHost));
    });
}

int ann_made_gradient(ann_made* m, const uint64_t* confs, unsigned n, float* gW1, float* gb1, float* gW2, float* gb2,
                      double* loss) {
    return mguard([&] {
        mneed(m && confs && n > 0, "null argument");
        DevBuf c, L;
        upload(c, confs, (size_t)n * kMaxWords * 8);
        L.ensure(8);
        made_gradient(*m, c.as<uint64_t>(), n, L.as<double>(), nullptr);
        ANN_CUDA(cudaDeviceSynchronize());
        const size_t nh = (size_t)m->N * m->H;
        if(gW1) ANN_CUDA(cudaMemcpy(gW1, m->gW1.p, nh * 4, cudaMemcpyDeviceToHost));
        if(gb1) ANN_CUDA(cudaMemcpy(gb1, m->gb1.p, m->H * 4, cudaMemcpyDeviceToHost));
        if(gW2) ANN_CUDA(cudaMemcpy(gW2, m->gW2.p, nh * 4, cudaMemcpyDeviceToHost));
        if(gb2) ANN_CUDA(cudaMemcpy(gb2, m->gb2.p, m->N * 4, cudaMemcpyDeviceToHost));
        if(loss) ANN_CUDA(cudaMemcpy(loss, L.p, 8, cudaMemcpyDeviceToHost));
    });
}

// steps of Adam over batches drawn in order (wrapping) from device configurations
static void made_train_impl(ann_made* m, const uint64_t* confs_dev, size_t n, unsigned steps, unsigned batch,
                            double lr, cudaStream_t st, double* loss_out) {
    mneed(n > 0 && batch > 0, "empty training set");
    DevBuf L;
    L.ensure(8);
    size_t pos = 0;
    for(unsigned s = 0; s < steps; s++) {
        const unsigned b = (unsigned)std::min<size_t>(batch, n);
        if(pos + b > n) pos = 0;
        made_gradient(*m, confs_dev + pos * kMaxWords, b, L.as<double>(), st);
        made_adam(*m, (float)lr, st);
        pos += b;
    }
    if(loss_out) {
        ANN_CUDA(cudaMemcpyAsync(loss_out, L.p, 8, cudaMemcpyDeviceToHost, st));
        ANN_CUDA(cudaStreamSynchronize(st));
    }
}

int ann_made_train(ann_made* m, const uint64_t* confs, unsigned n, unsigned steps, unsigned batch, double lr,
                   void* stream, double* loss) {
    return mguard([&] {
        mneed(m && confs, "null argument");
        DevBuf c;
        upload(c, confs, (size_t)n * kMaxWords * 8);
        made_train_impl(m, c.as<uint64_t>(), n, steps, batch, lr, reinterpret_cast<cudaStream_t>(stream), loss);
    });
}

int ann_made_train_on_samples(ann_made* m, const ann_ens* ens, unsigned steps, unsigned batch, double lr, void* stream,
                              double* loss) {
    return mguard([&] {
        mneed(m && ens && ens->rows.n > 0, "the ensemble holds no samples yet");
        // the ring buffer of recent passes when the ensemble keeps one, else the last pass
        if(ens->hist_cap && ens->hist_len)
            made_train_impl(m, ens->hist.as<uint64_t>(), ens->hist_len, steps, batch, lr,
                            reinterpret_cast<cudaStream_t>(stream), loss);
        else
            made_train_impl(m, ens->rows.conf.as<uint64_t>(), ens->rows.n, steps, batch, lr,
                            reinterpret_cast<cudaStream_t>(stream), loss);
    });
}

}  // extern "C"
