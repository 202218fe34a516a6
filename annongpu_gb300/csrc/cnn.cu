// PsiCNN on the GPU (include/quantum_state/PsiCNN.hpp:97-266,
// include/quantum_state/detail/Convolve.hpp:110-173, source/quantum_state/PsiCNN.cpp:9-55).
//
// Periodic convolutions with forward-anchored windows on an e0 x e1 x e2 lattice,
// per-site symmetry classes selecting the kernel, one or two layers, sum pooling:
//   z^0_c(x) = sum_k w^0[0,c][cls(x), k] s(x + k)
//   a^0_c(x) = f_0(z^0_c(x))
//   z^1_d(x) = sum_c sum_k w^1[c,d][cls(x), k] a^0_c(x + k)
//   log psi  = log_prefactor + final_factor * sum_{d,x} f_1(z^1_d(x))
// (with one layer the sum runs over f_0(z^0)). Activations follow the reference
// layer semantics (layer 0: polynomial log cosh, deeper: odd polynomial) or
// log cosh on every layer.
//
// One warp per chain (or enumerated / explicit configuration); a persistent grid whose
// warps take chains in turn. Each warp keeps its chain's pre-activations z^0 and z^1 in a
// slab of global memory (L1 / L2 resident: one slab per resident warp). A move that
// flips one or two sites changes z^0 only on the sites whose layer-0 window holds a
// flipped site (3 x 3 = 9 sites per flip for 3 x 3 windows) and z^1 only on the sites
// whose layer-1 window holds one of those (the 5 x 5 cone): the proposal evaluates
// those entries alone, from lists of the changed sites in per-warp shared memory, and
// an accepted move writes them back. The reference recomputes the full forward pass for
// every proposal (PsiCNN.hpp:177-181); samples here recompute it once, which also
// removes the rounding the increments accumulate. Weights and neighbour tables
// (site x, window offset k) -> x + k and its inverse are shared by the CTA.
#include <algorithm>
#include <set>

#include "ann_internal.hpp"
#include "chain.cuh"

namespace ann {

namespace {

constexpr int kCnnMaxLayers = 2;
constexpr unsigned kCnnMaxSites = 128;   // site indices are stored as bytes
constexpr unsigned kCnnMaxMoveFlips = 2;  // moves and flip groups with more sites take a full forward pass

template<typename T>
struct CnnDev {
    unsigned N, L, ncls, Np;
    unsigned ch[kCnnMaxLayers], prev[kCnnMaxLayers], vol[kCnnMaxLayers], woff[kCnnMaxLayers];
    int act;
    double ff;
    cplx<T> lp;
    const cplx<T>* w;        // Np (global; staged in shared memory)
    const uint8_t* cls;      // N
    const uint16_t* nbr;     // [L][N][vol_l] input site of window offset k at site x (layer offsets nbr_off)
    const uint16_t* inv;     // [L][N][vol_l] site x whose window offset k lands on y
    unsigned nbr_off[kCnnMaxLayers];
    unsigned tab_len;        // entries of nbr (= inv)
    unsigned x0max, x1max;   // capacity of the changed-site lists (layer 0, layer 1)
    cplx<T>* slab;           // per resident warp: z0 [ch0 N] | z1 [ch1 N] | f0(z0) [ch0 N] | f1(z1) [ch1 N] |
                             // work A [ch0 N] | work B [ch1 N]
    size_t slab_len;         // complex entries per warp
};

template<typename T>
struct CnnCtx {
    const CnnDev<T>* p;
    const cplx<T>* w;
    const uint8_t* cls;
    const uint16_t* nbr;
    const uint16_t* inv;
    // this warp's slab (global)
    cplx<T>* z0;     // ch0 x N pre-activations of the current configuration
    cplx<T>* z1;     // ch1 x N (two layers)
    cplx<T>* a0;     // ch0 x N f0(z0), kept with z0 (each changed entry costs one activation)
    cplx<T>* f1;     // ch1 x N f1(z1)
    cplx<T>* bufA;   // ch0 x N work buffer (activations, deltas)
    cplx<T>* bufB;   // ch1 x N work buffer
    // this warp's move lists (shared)
    cplx<T>* da0;    // x0max x ch0: f0(z0 new) - f0(z0 old) on the changed layer-0 sites
    cplx<T>* z0n;    // x0max x ch0: new z0 there
    cplx<T>* z1n;    // x1max x ch1: new z1 on the changed layer-1 sites
    cplx<T>* df1;    // x1max x ch1: f1(z1 new) - f1(z1 old) there
    uint8_t* pos0;   // kCnnMaxSites: position of a site in list0, 0xFF if absent
    uint8_t* mark;   // kCnnMaxSites
    uint8_t* list0;  // x0max changed layer-0 sites
    uint8_t* list1;  // x1max changed layer-1 sites
    unsigned n0, n1;
};

template<typename T>
__device__ __forceinline__ cplx<T> wgt(const CnnCtx<T>& c, unsigned l, unsigned ci, unsigned cj, unsigned cl, unsigned k) {
    const CnnDev<T>& p = *c.p;
    return c.w[p.woff[l] + ((ci * p.ch[l] + cj) * p.ncls + cl) * p.vol[l] + k];
}

template<typename T>
__device__ __forceinline__ T spin_v(const Conf<2>& s, unsigned i) {
    return spin_bit(s, i) ? T(1) : T(-1);
}

// layer-0 pre-activation z^0_c(x) from the spins
template<typename T>
__device__ __forceinline__ cplx<T> z0_of(const CnnCtx<T>& c, const Conf<2>& s, unsigned ch, unsigned x) {
    const CnnDev<T>& p = *c.p;
    const uint16_t* nb = c.nbr + p.nbr_off[0] + x * p.vol[0];
    const cplx<T>* wr = c.w + p.woff[0] + (ch * p.ncls + c.cls[x]) * p.vol[0];
    cplx<T> z = mk<T>(T(0), T(0));
    for(unsigned k = 0; k < p.vol[0]; k++) {
        const T sv = spin_v<T>(s, nb[k]);
        z.re += sv * wr[k].re;
        z.im += sv * wr[k].im;
    }
    return z;
}

// layer-1 pre-activation z^1_d(x) from the layer-0 activations in a (ch0 x N)
template<typename T>
__device__ __forceinline__ cplx<T> z1_of(const CnnCtx<T>& c, const cplx<T>* a, unsigned d, unsigned x) {
    const CnnDev<T>& p = *c.p;
    const uint16_t* nb = c.nbr + p.nbr_off[1] + x * p.vol[1];
    cplx<T> z = mk<T>(T(0), T(0));
    for(unsigned ci = 0; ci < p.ch[0]; ci++) {
        const cplx<T>* wr = c.w + p.woff[1] + ((ci * p.ch[1] + d) * p.ncls + c.cls[x]) * p.vol[1];
        const cplx<T>* ac = a + ci * p.N;
        for(unsigned k = 0; k < p.vol[1]; k++) cmac(z, wr[k], ac[nb[k]]);
    }
    return z;
}

template<typename T>
__device__ __forceinline__ cplx<T> scaled_lp(const CnnDev<T>& p, cplx<T> acc) {
    return mk<T>((T)(p.ff * (double)acc.re) + p.lp.re, (T)(p.ff * (double)acc.im) + p.lp.im);
}

// Full forward pass of s into the warp's slab (pre-activations z0, z1 and activations f0, f1);
// returns log psi in every lane.
template<typename T>
__device__ cplx<T> cnn_forward_state(const CnnCtx<T>& c, const Conf<2>& s, int lane) {
    const CnnDev<T>& p = *c.p;
    cplx<T> acc = mk<T>(T(0), T(0));
    for(unsigned e = lane; e < p.ch[0] * p.N; e += 32) {
        const unsigned ch = e / p.N, x = e % p.N;
        const cplx<T> z = z0_of(c, s, ch, x);
        c.z0[e] = z;
        const cplx<T> f = act_f(z, p.act, 0);
        c.a0[e] = f;
        if(p.L == 1) acc += f;
    }
    __syncwarp();
    if(p.L > 1) {
        for(unsigned e = lane; e < p.ch[1] * p.N; e += 32) {
            const unsigned d = e / p.N, x = e % p.N;
            const cplx<T> z = z1_of(c, c.a0, d, x);
            c.z1[e] = z;
            const cplx<T> f = act_f(z, p.act, 1);
            c.f1[e] = f;
            acc += f;
        }
        __syncwarp();
    }
    return scaled_lp(p, warp_sum(acc));
}

// log psi of s without touching the slab's pre-activations (bufA as scratch)
template<typename T>
__device__ cplx<T> cnn_log_psi_scratch(const CnnCtx<T>& c, const Conf<2>& s, int lane) {
    const CnnDev<T>& p = *c.p;
    cplx<T> acc = mk<T>(T(0), T(0));
    for(unsigned e = lane; e < p.ch[0] * p.N; e += 32) {
        const unsigned ch = e / p.N, x = e % p.N;
        const cplx<T> f = act_f(z0_of(c, s, ch, x), p.act, 0);
        if(p.L == 1) acc += f;
        else c.bufA[e] = f;
    }
    __syncwarp();
    if(p.L > 1) {
        for(unsigned e = lane; e < p.ch[1] * p.N; e += 32) {
            const unsigned d = e / p.N, x = e % p.N;
            acc += act_f(z1_of(c, c.bufA, d, x), p.act, 1);
        }
        __syncwarp();
    }
    return scaled_lp(p, warp_sum(acc));
}

// Sites set in mark[] -> ascending list (and their positions in pos, when given); clears
// the marks. Returns the count; entries beyond cap are dropped and flagged.
__device__ unsigned compact_marks(uint8_t* mark, uint8_t* list, uint8_t* pos, unsigned N, unsigned cap, int lane,
                                  unsigned* status) {
    __syncwarp();
    unsigned n = 0;
    for(unsigned base = 0; base < N; base += 32) {
        const unsigned x = base + lane;
        const bool m = x < N && mark[x];
        const unsigned b = __ballot_sync(0xffffffffu, m);
        if(m) {
            const unsigned q = n + __popc(b & ((1u << lane) - 1u));
            if(q < cap) {
                list[q] = (uint8_t)x;
                if(pos) pos[x] = (uint8_t)q;
            } else {
                atomicOr(status, kStatusBadInput);
            }
            mark[x] = 0;
        }
        n += __popc(b);
    }
    __syncwarp();
    return n < cap ? n : cap;
}

// Change of log psi when the nF <= 2 sites F flip, from the changed pre-activations
// alone; leaves the new pre-activations in the move lists for cnn_commit.
template<typename T>
__device__ cplx<T> cnn_delta(CnnCtx<T>& c, const Conf<2>& s, const unsigned* F, unsigned nF, int lane,
                             unsigned* status) {
    const CnnDev<T>& p = *c.p;
    const unsigned N = p.N, C0 = p.ch[0], v0 = p.vol[0];
    // layer-0 sites whose window holds a flipped site
    for(unsigned q = lane; q < nF * v0; q += 32) c.mark[c.inv[p.nbr_off[0] + F[q / v0] * v0 + q % v0]] = 1;
    c.n0 = compact_marks(c.mark, c.list0, c.pos0, N, p.x0max, lane, status);
    const unsigned n0 = c.n0;
    const uint16_t* nb0 = c.nbr + p.nbr_off[0];
    const T m2s0 = spin_bit(s, F[0]) ? T(-2) : T(2);  // s' - s at the flipped sites
    const T m2s1 = nF > 1 ? (spin_bit(s, F[1]) ? T(-2) : T(2)) : T(0);
    const unsigned f1 = nF > 1 ? F[1] : 0xFFFFFFFFu;
    cplx<T> acc = mk<T>(T(0), T(0));
    for(unsigned e = lane; e < n0 * C0; e += 32) {
        const unsigned u = e / C0, ch = e % C0, x = c.list0[u];
        const cplx<T>* wr = c.w + p.woff[0] + (ch * p.ncls + c.cls[x]) * v0;
        cplx<T> dz = mk<T>(T(0), T(0));
        for(unsigned k = 0; k < v0; k++) {
            const unsigned y = nb0[x * v0 + k];
            const T m = y == F[0] ? m2s0 : (y == f1 ? m2s1 : T(0));
            dz.re += m * wr[k].re;
            dz.im += m * wr[k].im;
        }
        const cplx<T> zn = c.z0[ch * N + x] + dz;
        c.z0n[e] = zn;
        const cplx<T> df = act_f(zn, p.act, 0) - c.a0[ch * N + x];
        c.da0[e] = df;
        if(p.L == 1) acc += df;
    }
    c.n1 = 0;
    if(p.L > 1) {
        const unsigned C1 = p.ch[1], v1 = p.vol[1];
        // layer-1 sites whose window holds a changed layer-0 site
        for(unsigned q = lane; q < n0 * v1; q += 32)
            c.mark[c.inv[p.nbr_off[1] + c.list0[q / v1] * v1 + q % v1]] = 1;
        c.n1 = compact_marks(c.mark, c.list1, nullptr, N, p.x1max, lane, status);
        const uint16_t* nb1 = c.nbr + p.nbr_off[1];
        const unsigned cstride = C1 * p.ncls * v1;  // weight stride between input channels
        for(unsigned e = lane; e < c.n1 * C1; e += 32) {
            const unsigned v = e / C1, d = e % C1, x = c.list1[v];
            const cplx<T>* wr = c.w + p.woff[1] + (d * p.ncls + c.cls[x]) * v1;
            cplx<T> dz = mk<T>(T(0), T(0));
            for(unsigned k = 0; k < v1; k++) {
                const unsigned u = c.pos0[nb1[x * v1 + k]];
                if(u == 0xFFu) continue;
                const cplx<T>* da = c.da0 + u * C0;
                for(unsigned ci = 0; ci < C0; ci++) cmac(dz, wr[ci * cstride + k], da[ci]);
            }
            const cplx<T> zn = c.z1[d * N + x] + dz;
            c.z1n[e] = zn;
            const cplx<T> df = act_f(zn, p.act, 1) - c.f1[d * N + x];
            c.df1[e] = df;
            acc += df;
        }
    }
    __syncwarp();
    for(unsigned u = lane; u < n0; u += 32) c.pos0[c.list0[u]] = 0xFFu;
    __syncwarp();
    acc = warp_sum(acc);
    const T ff = (T)p.ff;
    return mk<T>(ff * acc.re, ff * acc.im);
}

// the accepted move: its new pre-activations into the slab
template<typename T>
__device__ void cnn_commit(const CnnCtx<T>& c, int lane) {
    const CnnDev<T>& p = *c.p;
    for(unsigned e = lane; e < c.n0 * p.ch[0]; e += 32) {
        const unsigned q = (e % p.ch[0]) * p.N + c.list0[e / p.ch[0]];
        c.z0[q] = c.z0n[e];
        c.a0[q] += c.da0[e];  // f0(z0 new) up to one rounding: samples recompute it exactly
    }
    if(p.L > 1)
        for(unsigned e = lane; e < c.n1 * p.ch[1]; e += 32) {
            const unsigned q = (e % p.ch[1]) * p.N + c.list1[e / p.ch[1]];
            c.z1[q] = c.z1n[e];
            c.f1[q] += c.df1[e];
        }
    __syncwarp();
}

// O_k row (back-propagation, PsiCNN.hpp:183-266) from the slab's pre-activations
template<typename T>
__device__ void cnn_O_row(const CnnCtx<T>& c, const Conf<2>& s, int lane, cplx<T>* O) {
    const CnnDev<T>& p = *c.p;
    const T ff = (T)p.ff;
    if(p.L == 1) {
        // dlogpsi/dz0 = ff f0'(z0); O[w0[0,c][cls,k]] = sum_{x in cls} ff f0'(z0_c(x)) s(x+k)
        for(unsigned e = lane; e < p.ch[0] * p.N; e += 32) c.bufA[e] = ff * act_df(c.z0[e], p.act, 0);
        __syncwarp();
    } else {
        for(unsigned e = lane; e < p.ch[1] * p.N; e += 32) c.bufB[e] = ff * act_df(c.z1[e], p.act, 1);
        __syncwarp();
        // layer-1 parameters: O[(ci, d), cls, k] = sum_{x: cls(x)=cls} delta1_d(x) a0_ci(x + k)
        const unsigned n1 = p.ch[0] * p.ch[1] * p.ncls * p.vol[1];
        const uint16_t* nb = c.nbr + p.nbr_off[1];
        for(unsigned q = lane; q < n1; q += 32) {
            const unsigned k = q % p.vol[1];
            const unsigned cl = (q / p.vol[1]) % p.ncls;
            const unsigned link = q / (p.vol[1] * p.ncls);
            const unsigned ci = link / p.ch[1], d = link % p.ch[1];
            cplx<T> o = mk<T>(T(0), T(0));
            const cplx<T>* dl = c.bufB + d * p.N;
            const cplx<T>* ac = c.a0 + ci * p.N;
            for(unsigned x = 0; x < p.N; x++) {
                if(c.cls[x] != cl) continue;
                cmac(o, dl[x], ac[nb[x * p.vol[1] + k]]);
            }
            O[p.woff[1] + q] = o;
        }
        __syncwarp();
        // delta0_ci(y) = f0'(z0_ci(y)) sum_d sum_k w1[ci,d][cls(x), k] delta1_d(x), x = inv(y, k)
        for(unsigned e = lane; e < p.ch[0] * p.N; e += 32) {
            const unsigned ci = e / p.N, y = e % p.N;
            cplx<T> g = mk<T>(T(0), T(0));
            const uint16_t* iv = c.inv + p.nbr_off[1] + y * p.vol[1];
            for(unsigned d = 0; d < p.ch[1]; d++)
                for(unsigned k = 0; k < p.vol[1]; k++) {
                    const unsigned x = iv[k];
                    cmac(g, wgt(c, 1, ci, d, c.cls[x], k), c.bufB[d * p.N + x]);
                }
            c.bufA[e] = g * act_df(c.z0[e], p.act, 0);
        }
        __syncwarp();
    }
    // layer-0 parameters: O[(0, c), cls, k] = sum_{x: cls(x)=cls} delta0_c(x) s(x + k)
    const unsigned n0 = p.ch[0] * p.ncls * p.vol[0];
    const uint16_t* nb = c.nbr + p.nbr_off[0];
    for(unsigned q = lane; q < n0; q += 32) {
        const unsigned k = q % p.vol[0];
        const unsigned cl = (q / p.vol[0]) % p.ncls;
        const unsigned ch = q / (p.vol[0] * p.ncls);
        cplx<T> o = mk<T>(T(0), T(0));
        const cplx<T>* dl = c.bufA + ch * p.N;
        for(unsigned x = 0; x < p.N; x++) {
            if(c.cls[x] != cl) continue;
            const T sv = spin_v<T>(s, nb[x * p.vol[0] + k]);
            o.re += sv * dl[x].re;
            o.im += sv * dl[x].im;
        }
        O[p.woff[0] + q] = o;
    }
    __syncwarp();
}

// local energy (Operator.hpp:36-121): one psi ratio per off-diagonal flip group, from the
// changed pre-activations for groups of one or two sites, a full forward pass otherwise
template<typename T>
__device__ cplx<double> cnn_local_energy(CnnCtx<T>& c, const OpDev& op, const Conf<2>& s, cplx<T> lpsi, int lane,
                                         unsigned* status) {
    T dre = T(0), dim = T(0);
    for(unsigned n = lane; n < op.n_diag; n += 32) {
        int neg = 0;
        for(int w = 0; w < 2; w++) neg += __popcll((~s.w[w]) & op.diag_mask[n * op.nw + w]);
        const T c_re = diag_coeff<T>(op)[2 * n], c_im = diag_coeff<T>(op)[2 * n + 1];
        dre += (neg & 1) ? -c_re : c_re;
        dim += (neg & 1) ? -c_im : c_im;
    }
    cplx<T> e = mk<T>(warp_sum(dre), warp_sum(dim));
    for(unsigned g = 0; g < op.n_groups; g++) {
        cplx<T> cg = mk<T>(T(0), T(0));
        for(unsigned k = op.grp_str_begin[g]; k < op.grp_str_begin[g + 1]; k++) {
            int neg = 0;
            for(int w = 0; w < 2; w++) neg += __popcll((~s.w[w]) & op.str_mask[k * op.nw + w]);
            const T c_re = str_coeff<T>(op)[2 * k], c_im = str_coeff<T>(op)[2 * k + 1];
            cg.re += (neg & 1) ? -c_re : c_re;
            cg.im += (neg & 1) ? -c_im : c_im;
        }
        if(cg.re == T(0) && cg.im == T(0)) continue;
        const unsigned sb = op.grp_site_begin[g], se = op.grp_site_begin[g + 1];
        cplx<T> d;
        if(se - sb <= kCnnMaxMoveFlips) {
            unsigned F[kCnnMaxMoveFlips];
            for(unsigned q = 0; q < se - sb; q++) F[q] = op.grp_sites[sb + q];
            d = cnn_delta(c, s, F, se - sb, lane, status);
        } else {
            Conf<2> s2 = s;
            for(unsigned q = sb; q < se; q++) flip(s2, op.grp_sites[q]);
            d = cnn_log_psi_scratch(c, s2, lane) - lpsi;
        }
        e += cg * cexp(d);
    }
    return cvt<double>(e);
}

template<typename T>
__device__ void cnn_process_sample(CnnCtx<T>& c, const OpDev* op, const Conf<2>& s, int lane, size_t row,
                                   const SampleOut& out, bool exact_weight) {
    const cplx<T> lpsi = cnn_forward_state(c, s, lane);
    cplx<double> e = mk(0.0, 0.0);
    if(op) e = cnn_local_energy(c, *op, s, lpsi, lane, out.status);
    if(lane == 0) {
        for(int w = 0; w < kMaxWords; w++) out.conf[row * kMaxWords + w] = s.w[w];
        const cplx<double> l = cvt<double>(lpsi);
        out.log_psi[row] = l;
        if(out.eloc) out.eloc[row] = e;
        if(exact_weight && out.weight) out.weight[row] = exp(2.0 * l.re);
        if(!(isfinite(l.re) && isfinite(l.im) && isfinite(e.re) && isfinite(e.im))) atomicOr(out.status, kStatusNonFinite);
    }
    if(out.O) cnn_O_row(c, s, lane, reinterpret_cast<cplx<T>*>(out.O) + row * out.ldO);
}

__host__ __device__ inline size_t cnn_warp_smem(unsigned x0max, unsigned x1max, unsigned ch0, unsigned ch1,
                                                size_t elem) {
    const size_t cplx_bytes = ((size_t)2 * x0max * ch0 + (size_t)2 * x1max * ch1) * elem;
    const size_t byte_bytes = 2 * kCnnMaxSites + x0max + x1max;
    return (cplx_bytes + byte_bytes + 15) & ~(size_t)15;
}

// stages weights and tables in shared memory, carves this warp's move lists and slab
template<typename T>
__device__ CnnCtx<T> cnn_stage(const CnnDev<T>& p, unsigned char* smem) {
    CnnCtx<T> c;
    c.p = &p;
    cplx<T>* w = reinterpret_cast<cplx<T>*>(smem);
    for(unsigned k = threadIdx.x; k < p.Np; k += blockDim.x) w[k] = p.w[k];
    unsigned char* q = smem + ((p.Np * sizeof(cplx<T>) + 15) & ~15u);
    uint16_t* nb = reinterpret_cast<uint16_t*>(q);
    uint16_t* iv = nb + p.tab_len;
    for(unsigned k = threadIdx.x; k < p.tab_len; k += blockDim.x) {
        nb[k] = p.nbr[k];
        iv[k] = p.inv[k];
    }
    q += ((2 * p.tab_len * sizeof(uint16_t) + 15) & ~15u);
    uint8_t* cl = q;
    for(unsigned k = threadIdx.x; k < p.N; k += blockDim.x) cl[k] = p.cls[k];
    q += (p.N + 15) & ~15u;
    const unsigned warp = threadIdx.x >> 5;
    const unsigned ch1 = p.L > 1 ? p.ch[1] : 0u;
    q += warp * cnn_warp_smem(p.x0max, p.x1max, p.ch[0], ch1, sizeof(cplx<T>));
    c.da0 = reinterpret_cast<cplx<T>*>(q);
    c.z0n = c.da0 + (size_t)p.x0max * p.ch[0];
    c.z1n = c.z0n + (size_t)p.x0max * p.ch[0];
    c.df1 = c.z1n + (size_t)p.x1max * ch1;
    uint8_t* b = reinterpret_cast<uint8_t*>(c.df1 + (size_t)p.x1max * ch1);
    c.pos0 = b;
    c.mark = b + kCnnMaxSites;
    c.list0 = b + 2 * kCnnMaxSites;
    c.list1 = c.list0 + p.x0max;
    const int lane = threadIdx.x & 31;
    for(unsigned k = lane; k < kCnnMaxSites; k += 32) {
        c.pos0[k] = 0xFFu;
        c.mark[k] = 0;
    }
    c.n0 = c.n1 = 0;
    cplx<T>* slab = p.slab + (size_t)(blockIdx.x * (blockDim.x >> 5) + warp) * p.slab_len;
    c.z0 = slab;
    c.z1 = c.z0 + (size_t)p.ch[0] * p.N;
    c.a0 = c.z1 + (size_t)ch1 * p.N;
    c.f1 = c.a0 + (size_t)p.ch[0] * p.N;
    c.bufA = c.f1 + (size_t)ch1 * p.N;
    c.bufB = c.bufA + (size_t)p.ch[0] * p.N;
    c.w = w;
    c.nbr = nb;
    c.inv = iv;
    c.cls = cl;
    __syncthreads();
    return c;
}

// Metropolis chains (MonteCarlo.hpp:55-177 with the sampler's Philox contract); each warp
// runs chains warp, warp + total warps, ...
template<typename T>
__global__ void __launch_bounds__(256) cnn_mc_kernel(CnnDev<T> p, OpDev op, int with_op, McArgs a, SampleOut out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CnnCtx<T> c = cnn_stage<T>(p, smem_raw);
    const int lane = threadIdx.x & 31;
    const unsigned warps = gridDim.x * (blockDim.x >> 5);
    const unsigned N = p.N;
    for(unsigned chain = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); chain < a.n_chains; chain += warps) {
        Conf<2> s;
        ChainDraw dr;
        chain_start(a, chain, N, s, dr.t);
        dr.t0 = dr.t;
        cnn_forward_state(c, s, lane);
        unsigned long long n_acc = 0, n_rej = 0;
        auto propose = [&]() {
            unsigned F[2];
            double u;
            float uf;
            dr.next(a, chain, N, lane, F[0], F[1], u, uf);
            unsigned nF = 1;
            if(F[1] != 0xFFFFFFFFu) {
                if(spin_bit(s, F[0]) == spin_bit(s, F[1])) { n_rej++; return; }
                nF = 2;
            }
            const cplx<T> d = cnn_delta(c, s, F, nF, lane, out.status);
            const T ratio = fexp(T(2) * d.re);
            const bool accept = sizeof(T) == 4 ? (uf <= (float)ratio) : (u <= (double)ratio);
            if(accept) {
                cnn_commit(c, lane);
                for(unsigned q = 0; q < nF; q++) flip(s, F[q]);
                n_acc++;
            } else {
                n_rej++;
            }
        };
        if(a.do_init || a.tape_site)
            for(unsigned k = 0; k < a.num_therm * N; k++) propose();
        for(unsigned st = 0; st < a.samples_per_chain; st++) {
            for(unsigned k = 0; k < a.num_sweeps * N; k++) propose();
            cnn_process_sample(c, with_op ? &op : nullptr, s, lane, (size_t)st * a.n_chains + chain, out, false);
        }
        if(lane == 0) {
            if(!a.tape_site) {
                for(int w = 0; w < kMaxWords; w++) a.chain_conf[(size_t)chain * kMaxWords + w] = s.w[w];
                a.chain_counter[chain] = dr.t;
            }
            atomicAdd(&a.acc_rej[0], n_acc);
            atomicAdd(&a.acc_rej[1], n_rej);
        }
    }
}

template<typename T>
__global__ void __launch_bounds__(256) cnn_exact_kernel(CnnDev<T> p, OpDev op, int with_op, uint64_t n_conf,
                                                         SampleOut out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CnnCtx<T> c = cnn_stage<T>(p, smem_raw);
    const int lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for(uint64_t idx = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); idx < n_conf; idx += warps) {
        Conf<2> s;
        s.w[0] = idx;
        s.w[1] = 0;
        cnn_process_sample(c, with_op ? &op : nullptr, s, lane, idx, out, true);
    }
}

template<typename T>
__global__ void __launch_bounds__(256) cnn_confs_kernel(CnnDev<T> p, OpDev op, int with_op, const uint64_t* confs,
                                                         uint64_t n, SampleOut out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CnnCtx<T> c = cnn_stage<T>(p, smem_raw);
    const int lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for(uint64_t idx = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); idx < n; idx += warps) {
        Conf<2> s;
        s.w[0] = confs[idx * kMaxWords];
        s.w[1] = confs[idx * kMaxWords + 1];
        cnn_process_sample(c, with_op ? &op : nullptr, s, lane, idx, out, true);
    }
}

template<typename T>
__global__ void cnn_prepare_kernel(const cplx<double>* __restrict__ params, cplx<T>* __restrict__ w, unsigned n) {
    const unsigned k = blockIdx.x * blockDim.x + threadIdx.x;
    if(k < n) w[k] = cvt<T>(params[k]);
}

// ----------------------------------------------------------------------------------
template<typename T>
CnnDev<T> cnn_view(const ann_psi_impl& psi) {
    CnnDev<T> p{};
    p.N = psi.N;
    p.L = (unsigned)psi.layers.size();
    p.ncls = psi.ncls;
    p.Np = psi.Np;
    unsigned tab = 0;
    for(unsigned l = 0; l < p.L; l++) {
        p.ch[l] = psi.layers[l].channels;
        p.prev[l] = psi.layers[l].prev_channels;
        p.vol[l] = psi.layers[l].vol;
        p.woff[l] = psi.layers[l].param_offset;
        p.nbr_off[l] = tab;
        tab += psi.N * p.vol[l];
    }
    p.tab_len = tab;
    p.act = psi.act;
    p.ff = psi.final_factor;
    p.lp = mk<T>((T)psi.lp.real(), (T)psi.lp.imag());
    p.w = psi.cnn_w.as<cplx<T>>();
    const unsigned char* meta = psi.cnn_meta.as<unsigned char>();
    p.nbr = reinterpret_cast<const uint16_t*>(meta);
    p.inv = p.nbr + tab;
    p.cls = meta + 4 * tab;
    p.x0max = psi.cnn_x0;
    p.x1max = p.L > 1 ? psi.cnn_x1 : 0u;
    p.slab_len = (size_t)3 * (p.ch[0] + (p.L > 1 ? p.ch[1] : 0u)) * p.N;
    return p;
}

template<typename T>
size_t cnn_smem(const CnnDev<T>& p, int warps) {
    const unsigned ch1 = p.L > 1 ? p.ch[1] : 0u;
    return ((p.Np * sizeof(cplx<T>) + 15) & ~(size_t)15) + ((2 * p.tab_len * 2 + 15) & ~(size_t)15) +
           ((p.N + 15) & ~(size_t)15) + warps * cnn_warp_smem(p.x0max, p.x1max, p.ch[0], ch1, sizeof(cplx<T>));
}

template<typename T>
int cnn_warps(const CnnDev<T>& p) {
    int w = 8;
    while(w > 1 && cnn_smem(p, w) > 112 * 1024) w >>= 1;
    if(cnn_smem(p, w) > 220 * 1024) throw Error(ANN_ERR_INVALID, "PsiCNN too large for shared memory");
    return w;
}

template<typename K>
void cnn_set_smem(K k, size_t bytes) {
    if(bytes > 48 * 1024) ANN_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
}

// Persistent grid: at most the CTAs resident at once (and no more than the work needs);
// binds one slab per warp of it.
template<typename T, typename K>
unsigned cnn_grid(K kernel, ann_psi_impl& psi, CnnDev<T>& p, int wpb, size_t smem, uint64_t work) {
    cnn_set_smem(kernel, smem);
    int dev = 0, sms = 0, per_sm = 0;
    ANN_CUDA(cudaGetDevice(&dev));
    ANN_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    ANN_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, wpb * 32, smem));
    if(per_sm < 1) throw Error(ANN_ERR_INVALID, "PsiCNN kernel does not fit on an SM");
    uint64_t grid = (uint64_t)sms * per_sm;
    const uint64_t need = (work + wpb - 1) / wpb;
    if(need < grid) grid = need;
    if(grid < 1) grid = 1;
    psi.cnn_scratch.ensure((size_t)grid * wpb * p.slab_len * sizeof(cplx<T>));
    p.slab = psi.cnn_scratch.as<cplx<T>>();
    return (unsigned)grid;
}

SampleOut cnn_out(Rows& rows, void* O, size_t ldO, bool want_eloc) {
    SampleOut o;
    o.conf = rows.conf.as<uint64_t>();
    o.log_psi = rows.log_psi.as<cplx<double>>();
    o.eloc = want_eloc ? rows.eloc.as<cplx<double>>() : nullptr;
    o.weight = rows.weight.as<double>();
    o.O = O;
    o.ldO = ldO;
    o.status = status_word();
    return o;
}

void cnn_rows(Rows& rows, size_t n) {
    rows.n = n;
    rows.conf.ensure(n * kMaxWords * sizeof(uint64_t));
    rows.log_psi.ensure(n * sizeof(cplx<double>));
    rows.eloc.ensure(n * sizeof(cplx<double>));
    rows.weight.ensure(n * sizeof(double));
}

template<typename T>
void cnn_run_T(ann_psi_impl& psi, const ann_op_impl* op, ann_ens_impl& ens, const SampleTargets& t, cudaStream_t st) {
    CnnDev<T> p = cnn_view<T>(psi);
    const int wpb = cnn_warps(p);
    const size_t smem = cnn_smem(p, wpb);
    OpDev ov{};
    if(op) ov = op->view();
    if(ens.kind == 0) {
        const uint64_t n_conf = 1ull << ens.N;
        cnn_rows(*t.rows, n_conf);
        SampleOut out = cnn_out(*t.rows, t.O, t.ldO, t.want_eloc && op);
        const unsigned grid = cnn_grid(cnn_exact_kernel<T>, psi, p, wpb, smem, n_conf);
        cnn_exact_kernel<T><<<grid, wpb * 32, smem, st>>>(p, ov, op ? 1 : 0, n_conf, out);
        check_launch("cnn_exact_kernel");
        return;
    }
    const unsigned spc = ens.num_samples / ens.n_chains;
    cnn_rows(*t.rows, (size_t)spc * ens.n_chains);
    McArgs a{};
    a.n_chains = ens.n_chains;
    a.samples_per_chain = spc;
    a.num_sweeps = ens.num_sweeps;
    a.num_therm = ens.num_therm;
    a.do_init = (!ens.persistent || !ens.chains_valid) ? 1 : 0;
    a.n_up = ens.n_up;
    a.move_kind = ens.move;
    a.bonds = ens.bonds_d.as<uint32_t>();
    a.n_bonds = (unsigned)(ens.bonds.size() / 2);
    a.k0 = (uint32_t)ens.seed;
    a.k1 = (uint32_t)(ens.seed >> 32);
    a.chain_conf = ens.chain_conf.as<uint64_t>();
    a.chain_counter = ens.chain_counter.as<uint64_t>();
    a.tape_site = ens.tape_len ? ens.tape_site.as<uint32_t>() : nullptr;
    a.tape_u = ens.tape_len ? ens.tape_u.as<double>() : nullptr;
    a.tape_len = ens.tape_len;
    a.acc_rej = ens.acc_rej.as<unsigned long long>();
    if(a.tape_site)
        ANN_CUDA(cudaMemcpyAsync(ens.chain_conf.p, ens.tape_init.p, (size_t)ens.n_chains * kMaxWords * 8,
                                 cudaMemcpyDeviceToDevice, st));
    ANN_CUDA(cudaMemsetAsync(ens.acc_rej.p, 0, 2 * sizeof(unsigned long long), st));
    SampleOut out = cnn_out(*t.rows, t.O, t.ldO, t.want_eloc && op);
    const unsigned grid = cnn_grid(cnn_mc_kernel<T>, psi, p, wpb, smem, ens.n_chains);
    cnn_mc_kernel<T><<<grid, wpb * 32, smem, st>>>(p, ov, op ? 1 : 0, a, out);
    check_launch("cnn_mc_kernel");
    ens.chains_valid = true;
}

template<typename T>
void cnn_confs_T(ann_psi_impl& psi, const ann_op_impl* op, const uint64_t* confs, size_t n, Rows& rows, void* O,
                 size_t ldO, cudaStream_t st) {
    CnnDev<T> p = cnn_view<T>(psi);
    const int wpb = cnn_warps(p);
    const size_t smem = cnn_smem(p, wpb);
    OpDev ov{};
    if(op) ov = op->view();
    cnn_rows(rows, n);
    SampleOut out = cnn_out(rows, O, ldO, op != nullptr);
    const unsigned grid = cnn_grid(cnn_confs_kernel<T>, psi, p, wpb, smem, n);
    cnn_confs_kernel<T><<<grid, wpb * 32, smem, st>>>(p, ov, op ? 1 : 0, confs, n, out);
    check_launch("cnn_confs_kernel");
}

}  // namespace

void cnn_prepare(ann_psi_impl& psi, cudaStream_t st) {
    const unsigned n = psi.Np;
    if(psi.precision == 0)
        cnn_prepare_kernel<float><<<(n + 255) / 256, 256, 0, st>>>(psi.params.as<cplx<double>>(),
                                                                   psi.cnn_w.as<cplx<float>>(), n);
    else
        cnn_prepare_kernel<double><<<(n + 255) / 256, 256, 0, st>>>(psi.params.as<cplx<double>>(),
                                                                    psi.cnn_w.as<cplx<double>>(), n);
    check_launch("cnn_prepare_kernel");
}

void cnn_run(ann_psi_impl& psi, const ann_op_impl* op, ann_ens_impl& ens, const SampleTargets& t, cudaStream_t st) {
    if(psi.precision == 0) cnn_run_T<float>(psi, op, ens, t, st);
    else cnn_run_T<double>(psi, op, ens, t, st);
}

void cnn_confs(ann_psi_impl& psi, const ann_op_impl* op, const uint64_t* confs, size_t n, Rows& rows, void* O,
               size_t ldO, cudaStream_t st) {
    if(psi.precision == 0) cnn_confs_T<float>(psi, op, confs, n, rows, O, ldO, st);
    else cnn_confs_T<double>(psi, op, confs, n, rows, O, ldO, st);
}

}  // namespace ann

using namespace ann;

extern "C" int ann_psi_create_cnn(const ann_cnn_desc* d, ann_psi** out) {
    try {
        if(!d || !out) throw Error(ANN_ERR_INVALID, "null argument");
        if(d->num_layers < 1 || d->num_layers > (unsigned)kCnnMaxLayers)
            throw Error(ANN_ERR_UNSUPPORTED, "PsiCNN supports one or two layers");
        const unsigned N = d->extent[0] * d->extent[1] * d->extent[2];
        if(N < 1 || N > 128) throw Error(ANN_ERR_INVALID, "PsiCNN needs 1 <= N <= 128 sites");
        if(d->precision != ANN_PREC_FP32 && d->precision != ANN_PREC_FP64) throw Error(ANN_ERR_INVALID, "precision");
        auto* p = new ann_psi();
        try {
            p->kind = 1;
            p->precision = d->precision;
            p->act = d->activation;
            p->N = N;
            p->NW = 2;
            for(int k = 0; k < 3; k++) p->extent[k] = d->extent[k];
            p->final_factor = d->final_factor;
            p->lp = zd(d->log_prefactor[0], d->log_prefactor[1]);
            p->sym.assign(d->symmetry_classes, d->symmetry_classes + N);
            std::vector<unsigned> cls_sorted = p->sym;
            std::sort(cls_sorted.begin(), cls_sorted.end());
            p->ncls = (unsigned)(std::unique(cls_sorted.begin(), cls_sorted.end()) - cls_sorted.begin());
            for(unsigned x = 0; x < N; x++)
                if(p->sym[x] >= p->ncls) throw Error(ANN_ERR_INVALID, "symmetry classes must be 0..n-1");
            if(p->ncls > 255) throw Error(ANN_ERR_INVALID, "at most 255 symmetry classes");
            unsigned off = 0;
            for(unsigned l = 0; l < d->num_layers; l++) {
                CnnLayerHost L{};
                L.channels = d->num_channels[l];
                L.prev_channels = l ? d->num_channels[l - 1] : 1u;
                L.vol = 1;
                for(int k = 0; k < 3; k++) {
                    L.conn[k] = d->connectivity[3 * l + k];
                    if(L.conn[k] < 1 || L.conn[k] > d->extent[k]) throw Error(ANN_ERR_INVALID, "connectivity > extent");
                    L.vol *= L.conn[k];
                }
                if(L.channels < 1 || L.channels > 64) throw Error(ANN_ERR_INVALID, "1..64 channels per layer");
                L.param_offset = off;
                off += L.channels * L.prev_channels * p->ncls * L.vol;
                p->layers.push_back(L);
            }
            if(off != d->num_params) throw Error(ANN_ERR_INVALID, "num_params does not match the layer structure");
            p->Np = off;
            // neighbour tables: forward-anchored periodic windows (Convolve<3>::foreach_connection)
            const unsigned e0 = d->extent[0], e1 = d->extent[1], e2 = d->extent[2];
            std::vector<uint16_t> nbr, inv;
            for(auto& L : p->layers) {
                std::vector<uint16_t> nb(N * L.vol), iv(N * L.vol);
                for(unsigned x = 0; x < N; x++) {
                    const unsigned pg = x / (e1 * e2), row = (x % (e1 * e2)) / e2, col = x % e2;
                    unsigned k = 0;
                    for(unsigned a = 0; a < L.conn[0]; a++)
                        for(unsigned b = 0; b < L.conn[1]; b++)
                            for(unsigned cc = 0; cc < L.conn[2]; cc++) {
                                const unsigned y = ((pg + a) % e0) * e1 * e2 + ((row + b) % e1) * e2 + (col + cc) % e2;
                                nb[x * L.vol + k] = (uint16_t)y;
                                iv[y * L.vol + k] = (uint16_t)x;
                                k++;
                            }
                }
                nbr.insert(nbr.end(), nb.begin(), nb.end());
                inv.insert(inv.end(), iv.begin(), iv.end());
            }
            std::vector<unsigned char> meta(4 * nbr.size() + N);
            std::memcpy(meta.data(), nbr.data(), 2 * nbr.size());
            std::memcpy(meta.data() + 2 * nbr.size(), inv.data(), 2 * inv.size());
            for(unsigned x = 0; x < N; x++) meta[4 * nbr.size() + x] = (unsigned char)p->sym[x];
            upload(p->cnn_meta, meta.data(), meta.size());
            // capacities of the move lists: the most layer-0 sites one flip reaches (its inverse
            // window) and the most layer-1 sites reached through those, times the flips of a move
            {
                const unsigned v0 = p->layers[0].vol;
                unsigned cone0 = 0, cone1 = 0;
                for(unsigned y = 0; y < N; y++) {
                    std::set<unsigned> s0, s1;
                    for(unsigned k = 0; k < v0; k++) s0.insert(inv[y * v0 + k]);
                    if(p->layers.size() > 1) {
                        const unsigned v1 = p->layers[1].vol;
                        for(unsigned x : s0)
                            for(unsigned k = 0; k < v1; k++) s1.insert(inv[N * v0 + x * v1 + k]);
                    }
                    cone0 = std::max<unsigned>(cone0, (unsigned)s0.size());
                    cone1 = std::max<unsigned>(cone1, (unsigned)s1.size());
                }
                p->cnn_x0 = std::min(N, 2 * cone0);
                p->cnn_x1 = std::min(N, 2 * cone1);
            }
            upload(p->params, d->params, (size_t)p->Np * 16);
            p->cnn_w.ensure((size_t)p->Np * p->elem_bytes());
            psi_prepare(*p, nullptr);
            ANN_CUDA(cudaDeviceSynchronize());
        } catch(...) {
            delete p;
            throw;
        }
        *out = p;
        return ANN_OK;
    } catch(const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch(const std::exception& e) {
        set_last_error(e.what());
        return ANN_ERR_INVALID;
    }
}
