// PsiDeep with several hidden layers on the GPU (include/quantum_state/PsiDeep.hpp:
// forward_pass :171-215, update_angles :268-343, foreach_O_k :345-445;
// source/quantum_state/PsiDeep.cu: parameter layout :142-183, rhs lists :213-242).
//
// Layer l (0-based) has M_l units; unit j reads C_l units of the layer below (the
// spins for l = 0) through its connection block conn_l[i][j]:
//   z_0,j = b_0,j + sum_i W_0[i,j] s[conn_0[i][j]]
//   z_l,j = b_l,j + sum_i W_l[i,j] f_{l-1}(z_{l-1})[conn_l[i][j]]
//   log psi = log_prefactor (+ a.s) + sum_j fw_j f_L(z_L,j)
// with f_0 the log-cosh polynomial and deeper f the odd polynomial (or log cosh on
// every layer). Parameters [a | b_0 | W_0 | b_1 | W_1 | ...], W_l entry (i, j) at i*M_l + j.
//
// Configurations are spins (bit i = input unit i) or, in the Pauli-string basis, strings of
// I, X, Y, Z over N/3 sites held as words (a, b) (include/basis/PauliString.hpp); site x
// feeds three input units, +1 for the one of X, Y, Z it holds and -1 otherwise
// (network_unit_at, :84-90). Operators act on Pauli strings by the product P x.
//
// One warp per chain (or enumerated / explicit configuration). A chain keeps its
// layer-0 pre-activations; a proposal adds the flipped sites' weight columns (the
// reference's update_angles, through per-site lists of (i, j) entries) and runs the
// deeper layers in full. O_k rows back-propagate through the same per-unit lists.
// Weights, connection blocks and lists sit in shared memory when they fit, the per-warp
// pre-activations Z and activations A (reused for the deltas) always do.
//
// The same kernels carry PsiClassical (include/quantum_state/PsiClassical.hpp:48-163): K
// classical features h_k(s) = fast_local_energy of operator k (Operator.hpp:122-133) enter
// log psi as sum_k theta_k h_k(s), their parameters first; the network above is its reference
// (order 2, with no layers when the reference is fully polarized).
#include <algorithm>

#include "ann_internal.hpp"
#include "chain.cuh"

namespace ann {

namespace {

constexpr unsigned kDeepMaxLayers = 4;
constexpr unsigned kNoSite = 0xFFFFFFFFu;

template<typename T>
struct DeepDev {
    unsigned N, L, Np, U;                     // U: hidden units of all layers
    unsigned size[kDeepMaxLayers], C[kDeepMaxLayers];
    unsigned b_off[kDeepMaxLayers], w_off[kDeepMaxLayers];   // parameter offsets
    unsigned uoff[kDeepMaxLayers];            // first unit of layer l in Z / A
    unsigned conn_off[kDeepMaxLayers];        // connection block of layer l in tab
    unsigned rbeg_off[kDeepMaxLayers];        // per input unit: first entry of its list (+1 end)
    unsigned rq_off[kDeepMaxLayers];          // list entries q = i*M_l + j
    unsigned tab_len;
    int act, a_in;
    int basis;      // 0 spins, 1 Pauli strings (N = 3 x sites input units)
    unsigned sites; // sites of a Pauli string
    int dup0;       // an input unit appears twice in one unit's window: layer 0 recomputed per move
    int stage_w;    // weights staged in shared memory
    cplx<T> lp;
    const cplx<T>* w;    // Np
    const cplx<T>* fw;   // M_{L-1}
    const uint16_t* tab; // tab_len
    unsigned a_off, na;  // input-unit parameters a: first index, count (0: none)
    unsigned K;                  // classical features; their parameters are w[0, K)
    const uint32_t* feat_beg;    // K + 1 offsets into the strings
    const uint64_t* feat_zy;     // [strings][2]: sites holding Z or Y
    const cplx<T>* feat_c;       // strings: coefficient x (-i)^{n_y}
};

template<typename T>
struct DeepCtx {
    const DeepDev<T>* p;
    const cplx<T>* w;
    const cplx<T>* fw;
    const uint16_t* tab;
    cplx<T>* th;   // M_0: the chain's layer-0 pre-activations
    cplx<T>* Z;    // U: pre-activations of the evaluated configuration
    cplx<T>* A;    // U: activations (deltas during back-propagation)
};

// Pauli type of site x: 0 I, 1 X, 2 Y, 3 Z (a bit | b bit << 1)
__device__ __forceinline__ unsigned ptype(const Conf<2>& s, unsigned x) {
    return (unsigned)((s.w[0] >> x) & 1u) | ((unsigned)((s.w[1] >> x) & 1u) << 1);
}

// input unit u is +1
template<typename T>
__device__ __forceinline__ int input_up(const DeepCtx<T>& c, const Conf<2>& s, unsigned u) {
    if(!c.p->basis) return spin_bit(s, u);
    const unsigned x = u / 3u;
    return ptype(s, x) == u - 3u * x + 1u;
}

// calls f(u) for every input unit whose value differs between s and s2 (warp-uniform)
template<typename T, typename F>
__device__ __forceinline__ void for_changed_units(const DeepCtx<T>& c, const Conf<2>& s, const Conf<2>& s2, F f) {
    if(!c.p->basis) {
        for(int w = 0; w < 2; w++) {
            uint64_t d = s.w[w] ^ s2.w[w];
            while(d) {
                f(64u * w + (unsigned)(__ffsll((long long)d) - 1));
                d &= d - 1;
            }
        }
        return;
    }
    uint64_t d = (s.w[0] ^ s2.w[0]) | (s.w[1] ^ s2.w[1]);
    while(d) {
        const unsigned x = (unsigned)(__ffsll((long long)d) - 1);
        d &= d - 1;
        const unsigned to = ptype(s, x), tn = ptype(s2, x);
        if(to) f(3u * x + to - 1u);
        if(tn) f(3u * x + tn - 1u);
    }
}

template<typename T>
__device__ __forceinline__ void add_spin(cplx<T>& z, cplx<T> w, int up) {
    if(up) { z.re += w.re; z.im += w.im; }
    else { z.re -= w.re; z.im -= w.im; }
}

// layer-0 pre-activations of s into dst (lanes over units)
template<typename T>
__device__ void deep_z0(const DeepCtx<T>& c, const Conf<2>& s, cplx<T>* dst, int lane) {
    const DeepDev<T>& p = *c.p;
    const unsigned M = p.size[0];
    const uint16_t* cn = c.tab + p.conn_off[0];
    for(unsigned j = lane; j < M; j += 32) {
        cplx<T> z = c.w[p.b_off[0] + j];
        for(unsigned i = 0; i < p.C[0]; i++) add_spin(z, c.w[p.w_off[0] + i * M + j], input_up(c, s, cn[i * M + j]));
        dst[j] = z;
    }
}

// a.s (every lane holds the sum)
template<typename T>
__device__ cplx<T> deep_as(const DeepCtx<T>& c, const Conf<2>& s, int lane) {
    cplx<T> acc = mk<T>(T(0), T(0));
    for(unsigned x = lane; x < c.p->na; x += 32) add_spin(acc, c.w[c.p->a_off + x], input_up(c, s, x));
    return warp_sum(acc);
}

// h_k(s) = sum over feature k's strings of c <s|P|P s> = c (-i)^{n_y} (-1)^{#(Z or Y on a down spin)}
template<typename T>
__device__ __forceinline__ cplx<T> feat_h(const DeepCtx<T>& c, const Conf<2>& s, unsigned k) {
    const DeepDev<T>& p = *c.p;
    cplx<T> r = mk<T>(T(0), T(0));
    for(unsigned q = p.feat_beg[k]; q < p.feat_beg[k + 1]; q++) {
        const int neg = (__popcll(~s.w[0] & p.feat_zy[2 * q]) + __popcll(~s.w[1] & p.feat_zy[2 * q + 1])) & 1;
        const cplx<T> cq = p.feat_c[q];
        r.re += neg ? -cq.re : cq.re;
        r.im += neg ? -cq.im : cq.im;
    }
    return r;
}

// sum_k theta_k h_k(s) (every lane holds the sum)
template<typename T>
__device__ cplx<T> classical_term(const DeepCtx<T>& c, const Conf<2>& s, int lane) {
    cplx<T> acc = mk<T>(T(0), T(0));
    for(unsigned k = lane; k < c.p->K; k += 32) cmac(acc, c.w[k], feat_h(c, s, k));
    return warp_sum(acc);
}

// Z[0, M_0) += the change of flipping input unit x of s (update_angles, PsiDeep.hpp:268-307).
// A unit's entries address distinct first-layer units (checked on the host), so lanes do not collide.
template<typename T>
__device__ void deep_flip0(const DeepCtx<T>& c, const Conf<2>& s, unsigned x, int lane) {
    const DeepDev<T>& p = *c.p;
    const uint16_t* rb = c.tab + p.rbeg_off[0];
    const uint16_t* rq = c.tab + p.rq_off[0];
    const unsigned M = p.size[0];
    const T d = input_up(c, s, x) ? T(-2) : T(2);
    for(unsigned e = rb[x] + lane; e < rb[x + 1]; e += 32) {
        const unsigned q = rq[e];
        const cplx<T> wv = c.w[p.w_off[0] + q];
        cplx<T>& z = c.Z[q % M];
        z.re += d * wv.re;
        z.im += d * wv.im;
    }
}

// deeper layers from Z[0, M_0); returns sum_j fw_j f(z_L,j) in every lane (forward_pass)
template<typename T>
__device__ cplx<T> deep_forward(const DeepCtx<T>& c, int lane) {
    const DeepDev<T>& p = *c.p;
    if(p.L == 0) return mk<T>(T(0), T(0));
    for(unsigned j = lane; j < p.size[0]; j += 32) c.A[j] = act_f(c.Z[j], p.act, 0);
    __syncwarp();
    for(unsigned l = 1; l < p.L; l++) {
        const unsigned M = p.size[l], C = p.C[l];
        const uint16_t* cn = c.tab + p.conn_off[l];
        const cplx<T>* in = c.A + p.uoff[l - 1];
        const cplx<T>* wl = c.w + p.w_off[l];
        for(unsigned j = lane; j < M; j += 32) {
            cplx<T> z = c.w[p.b_off[l] + j];
            for(unsigned i = 0; i < C; i++) cmac(z, wl[i * M + j], in[cn[i * M + j]]);
            c.Z[p.uoff[l] + j] = z;
            c.A[p.uoff[l] + j] = act_f(z, p.act, (int)l);
        }
        __syncwarp();
    }
    const unsigned top = p.uoff[p.L - 1];
    cplx<T> acc = mk<T>(T(0), T(0));
    for(unsigned j = lane; j < p.size[p.L - 1]; j += 32) cmac(acc, c.fw[j], c.A[top + j]);
    return warp_sum(acc);
}

// log psi of s2 from the chain's layer-0 pre-activations th of s (the units that differ are
// moved); Z / A hold s2 afterwards. `as` is a.s of s.
template<typename T>
__device__ cplx<T> deep_eval_moved(const DeepCtx<T>& c, const Conf<2>& s, const Conf<2>& s2, cplx<T> as, int lane) {
    const DeepDev<T>& p = *c.p;
    if(p.L && !p.dup0) {
        for(unsigned j = lane; j < p.size[0]; j += 32) c.Z[j] = c.th[j];
        __syncwarp();
        for_changed_units(c, s, s2, [&](unsigned u) {
            deep_flip0(c, s, u, lane);
            __syncwarp();
        });
    } else if(p.L) {
        deep_z0(c, s2, c.Z, lane);
        __syncwarp();
    }
    if(p.a_in && p.na)
        for_changed_units(c, s, s2, [&](unsigned u) {
            const T d = input_up(c, s, u) ? T(-2) : T(2);
            as.re += d * c.w[p.a_off + u].re;
            as.im += d * c.w[p.a_off + u].im;
        });
    cplx<T> f = deep_forward(c, lane);
    if(p.K) f += classical_term(c, s2, lane);
    return mk<T>(p.lp.re + as.re + f.re, p.lp.im + as.im + f.im);
}

// O_k row by back-propagation (foreach_O_k, PsiDeep.hpp:345-445); Z / A must hold s
template<typename T>
__device__ void deep_O_row(const DeepCtx<T>& c, const Conf<2>& s, int lane, cplx<T>* O) {
    const DeepDev<T>& p = *c.p;
    const unsigned L = p.L;
    for(unsigned k = lane; k < p.K; k += 32) O[k] = feat_h(c, s, k);
    if(L) {
        const unsigned top = p.uoff[L - 1];
        for(unsigned j = lane; j < p.size[L - 1]; j += 32)
            c.A[top + j] = c.fw[j] * act_df(c.Z[top + j], p.act, (int)(L - 1));
        __syncwarp();
    }
    for(int l = (int)L - 1; l >= 0; l--) {
        const unsigned M = p.size[l], C = p.C[l];
        const cplx<T>* dl = c.A + p.uoff[l];
        for(unsigned j = lane; j < M; j += 32) O[p.b_off[l] + j] = dl[j];
        const uint16_t* cn = c.tab + p.conn_off[l];
        for(unsigned q = lane; q < C * M; q += 32) {
            const unsigned j = q % M, u = cn[q];
            cplx<T> o;
            if(l == 0) o = input_up(c, s, u) ? dl[j] : -dl[j];
            else o = dl[j] * c.A[p.uoff[l - 1] + u];
            O[p.w_off[l] + q] = o;
        }
        __syncwarp();
        if(l > 0) {
            // delta of unit u below: f'(z_u) sum over its list of W_l[q] delta_l[j(q)]
            const uint16_t* rb = c.tab + p.rbeg_off[l];
            const uint16_t* rq = c.tab + p.rq_off[l];
            const cplx<T>* wl = c.w + p.w_off[l];
            const unsigned below = p.uoff[l - 1];
            for(unsigned u = lane; u < p.size[l - 1]; u += 32) {
                cplx<T> g = mk<T>(T(0), T(0));
                for(unsigned e = rb[u]; e < rb[u + 1]; e++) {
                    const unsigned q = rq[e];
                    cmac(g, wl[q], dl[q % M]);
                }
                c.A[below + u] = g * act_df(c.Z[below + u], p.act, l - 1);
            }
            __syncwarp();
        }
    }
    for(unsigned x = lane; x < p.na; x += 32) O[p.a_off + x] = mk<T>(input_up(c, s, x) ? T(1) : T(-1), T(0));
    __syncwarp();
}

// local energy (Operator.hpp:36-121): diagonal strings, then one evaluation per flip group
template<typename T>
__device__ cplx<double> deep_local_energy(const DeepCtx<T>& c, const OpDev& op, const Conf<2>& s, cplx<T> lpsi,
                                          cplx<T> as, int lane) {
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
        Conf<2> s2 = s;
        for(unsigned q = op.grp_site_begin[g]; q < op.grp_site_begin[g + 1]; q++) flip(s2, op.grp_sites[q]);
        const cplx<T> l2 = deep_eval_moved(c, s, s2, as, lane);
        e += cg * cexp(l2 - lpsi);
    }
    return cvt<double>(e);
}

// local energy over Pauli strings: sum_n c_n phase(P_n, x) psi(P_n x) / psi(x) with the product
// string P_n ^ x and phase (-1)^{#(XZ, YX, ZY) pairs} (-i)^{n_eps}, n_eps the sites where both
// are non-trivial and differ (PauliString::apply(PauliString), PauliString.hpp:256-276)
template<typename T>
__device__ cplx<double> deep_local_energy_paulis(const DeepCtx<T>& c, const OpDev& op, const Conf<2>& s,
                                                 cplx<T> lpsi, cplx<T> as, int lane) {
    const uint64_t xa = s.w[0], xb = s.w[1];
    const uint64_t xX = xa & ~xb, xY = ~xa & xb, xZ = xa & xb;
    cplx<T> e = mk<T>(T(0), T(0));
    for(unsigned n = 0; n < op.n_raw; n++) {
        const uint64_t pa = op.raw_a[n], pb = op.raw_b[n];
        const T c_re = raw_coeff<T>(op)[2 * n], c_im = raw_coeff<T>(op)[2 * n + 1];
        if(!(pa | pb)) {
            e.re += c_re;
            e.im += c_im;
            continue;
        }
        const uint64_t pX = pa & ~pb, pY = ~pa & pb, pZ = pa & pb;
        const int neg = __popcll((pX & xZ) | (pY & xX) | (pZ & xY)) & 1;
        const int ne = __popcll((pa | pb) & (xa | xb) & ((pa ^ xa) | (pb ^ xb)));
        // coefficient times (-1)^neg, times -1 if ne % 4 >= 2, times -i if ne is odd
        T f_re = c_re, f_im = c_im;
        if(neg ^ ((ne & 3) > 1)) { f_re = -f_re; f_im = -f_im; }
        if(ne & 1) { const T t = f_re; f_re = f_im; f_im = -t; }
        Conf<2> s2;
        s2.w[0] = xa ^ pa;
        s2.w[1] = xb ^ pb;
        const cplx<T> l2 = deep_eval_moved(c, s, s2, as, lane);
        e += mk<T>(f_re, f_im) * cexp(l2 - lpsi);
    }
    return cvt<double>(e);
}

// one sample row: refreshed layer-0 pre-activations, log psi, O_k row, local energy;
// the refreshed log psi and a.s are returned in every lane
template<typename T>
__device__ void deep_process_sample(const DeepCtx<T>& c, const OpDev* op, const Conf<2>& s, int lane, size_t row,
                                    const SampleOut& out, bool exact_weight, cplx<T>* lpsi_out = nullptr,
                                    cplx<T>* as_out = nullptr) {
    deep_z0(c, s, c.th, lane);
    __syncwarp();
    const cplx<T> as = c.p->a_in ? deep_as(c, s, lane) : mk<T>(T(0), T(0));
    const cplx<T> lpsi = deep_eval_moved(c, s, s, as, lane);
    if(lpsi_out) *lpsi_out = lpsi;
    if(as_out) *as_out = as;
    if(out.O) deep_O_row(c, s, lane, reinterpret_cast<cplx<T>*>(out.O) + row * out.ldO);
    cplx<double> e = mk(0.0, 0.0);
    if(op) e = c.p->basis ? deep_local_energy_paulis(c, *op, s, lpsi, as, lane)
                          : deep_local_energy(c, *op, s, lpsi, as, lane);
    if(lane == 0) {
        for(int w = 0; w < kMaxWords; w++) out.conf[row * kMaxWords + w] = s.w[w];
        const cplx<double> l = cvt<double>(lpsi);
        out.log_psi[row] = l;
        if(out.eloc) out.eloc[row] = e;
        if(exact_weight && out.weight) out.weight[row] = exp(2.0 * l.re);
        if(!(isfinite(l.re) && isfinite(l.im) && isfinite(e.re) && isfinite(e.im))) atomicOr(out.status, kStatusNonFinite);
    }
}

// units of the top layer (0 without layers)
template<typename T>
__host__ __device__ __forceinline__ unsigned deep_top(const DeepDev<T>& p) {
    return p.L ? p.size[p.L - 1] : 0u;
}

// shared-memory layout: [weights (if staged) | fw | tables | per-warp th, Z, A]
template<typename T>
__host__ __device__ size_t deep_fixed_bytes(const DeepDev<T>& p) {
    size_t b = 0;
    if(p.stage_w) b += ((size_t)p.Np * sizeof(cplx<T>) + 15) & ~(size_t)15;
    b += ((size_t)deep_top(p) * sizeof(cplx<T>) + 15) & ~(size_t)15;
    b += ((size_t)p.tab_len * sizeof(uint16_t) + 15) & ~(size_t)15;
    return b;
}
template<typename T>
__host__ __device__ size_t deep_warp_bytes(const DeepDev<T>& p) {
    return ((size_t)p.size[0] + 2 * (size_t)p.U) * sizeof(cplx<T>);
}

// the layer description is indexed by layer at run time: it is copied to shared memory
// (indexing the kernel parameter itself would copy it to the stack)
template<typename T>
__device__ DeepCtx<T> deep_stage(const DeepDev<T>& p, unsigned char* smem) {
    __shared__ DeepDev<T> sp;
    if(threadIdx.x == 0) sp = p;
    DeepCtx<T> c;
    c.p = &sp;
    unsigned char* q = smem;
    if(p.stage_w) {
        cplx<T>* w = reinterpret_cast<cplx<T>*>(q);
        for(unsigned k = threadIdx.x; k < p.Np; k += blockDim.x) w[k] = p.w[k];
        c.w = w;
        q += ((size_t)p.Np * sizeof(cplx<T>) + 15) & ~(size_t)15;
    } else {
        c.w = p.w;
    }
    cplx<T>* fw = reinterpret_cast<cplx<T>*>(q);
    for(unsigned k = threadIdx.x; k < deep_top(p); k += blockDim.x) fw[k] = p.fw[k];
    c.fw = fw;
    q += ((size_t)deep_top(p) * sizeof(cplx<T>) + 15) & ~(size_t)15;
    uint16_t* tab = reinterpret_cast<uint16_t*>(q);
    for(unsigned k = threadIdx.x; k < p.tab_len; k += blockDim.x) tab[k] = p.tab[k];
    c.tab = tab;
    q += ((size_t)p.tab_len * sizeof(uint16_t) + 15) & ~(size_t)15;
    cplx<T>* buf = reinterpret_cast<cplx<T>*>(q) + (size_t)(threadIdx.x >> 5) * (p.size[0] + 2 * p.U);
    c.th = buf;
    c.Z = buf + p.size[0];
    c.A = c.Z + p.U;
    __syncthreads();
    return c;
}

template<typename T>
__global__ void __launch_bounds__(256, 1) deep_mc_kernel(DeepDev<T> p, OpDev op, int with_op, McArgs a, SampleOut out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const DeepCtx<T> c = deep_stage<T>(p, smem_raw);
    const int lane = threadIdx.x & 31;
    const unsigned chain = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if(chain >= a.n_chains) return;
    const unsigned N = p.N;
    Conf<2> s;
    ChainDraw dr;
    if(p.basis) {
        // Pauli strings: a fresh string from counter (t, chain, 1), masked to the sites
        dr.t = a.chain_counter[chain];
        if(a.do_init) {
            const u32x4 r = philox4x32_10(a.k0, a.k1, u32x4{(uint32_t)dr.t, (uint32_t)(dr.t >> 32), chain, 1u});
            const uint64_t mask = p.sites >= 64u ? ~(uint64_t)0 : (((uint64_t)1 << p.sites) - 1u);
            s.w[0] = ((uint64_t)r.x | ((uint64_t)r.y << 32)) & mask;
            s.w[1] = ((uint64_t)r.z | ((uint64_t)r.w << 32)) & mask;
        } else {
            for(int w = 0; w < 2; w++) s.w[w] = a.chain_conf[(size_t)chain * kMaxWords + w];
        }
    } else {
        chain_start(a, chain, N, s, dr.t);
    }
    dr.t0 = dr.t;
    deep_z0(c, s, c.th, lane);
    __syncwarp();
    cplx<T> as = p.a_in ? deep_as(c, s, lane) : mk<T>(T(0), T(0));
    cplx<T> lpsi = deep_eval_moved(c, s, s, as, lane);
    unsigned long long n_acc = 0, n_rej = 0;
    auto propose = [&]() {
        double u;
        float uf;
        Conf<2> s2 = s;
        if(p.basis) {
            // site mulhi(r0, sites) set to type r1 >> 30 (Update_Policy.hpp:41-57 draws x % sites, x >> 30)
            uint32_t r0, r1, r2, r3;
            dr.words(a, chain, lane, r0, r1, r2, r3);
            const unsigned x = mulhi32(r0, p.sites), type = r1 >> 30;
            s2.w[0] = (s2.w[0] & ~((uint64_t)1 << x)) | ((uint64_t)(type & 1u) << x);
            s2.w[1] = (s2.w[1] & ~((uint64_t)1 << x)) | ((uint64_t)(type >> 1) << x);
            u = u53(r2, r3);
            uf = __uint2float_rz(r3 >> 8) * 0x1.0p-24f;
            if(s2.w[0] == s.w[0] && s2.w[1] == s.w[1]) { n_acc++; return; }  // ratio 1
        } else {
            unsigned i, j;
            dr.next(a, chain, N, lane, i, j, u, uf);
            flip(s2, i);
            if(j != kNoSite) {
                if(spin_bit(s, i) == spin_bit(s, j)) { n_rej++; return; }
                flip(s2, j);
            }
        }
        const cplx<T> l2 = deep_eval_moved(c, s, s2, as, lane);
        const T ratio = fexp(T(2) * (l2.re - lpsi.re));
        const bool accept = sizeof(T) == 4 ? (uf <= (float)ratio) : (u <= (double)ratio);
        if(accept) {
            // Z holds the moved configuration's layer-0 pre-activations
            for(unsigned q = lane; q < p.size[0]; q += 32) c.th[q] = c.Z[q];
            __syncwarp();
            if(p.a_in && p.na)
                for_changed_units(c, s, s2, [&](unsigned uu) {
                    const T d = input_up(c, s, uu) ? T(-2) : T(2);
                    as.re += d * c.w[p.a_off + uu].re;
                    as.im += d * c.w[p.a_off + uu].im;
                });
            s = s2;
            lpsi = l2;
            n_acc++;
        } else {
            n_rej++;
        }
    };
    if(a.do_init || a.tape_site)
        for(unsigned k = 0; k < a.num_therm * N; k++) propose();
    for(unsigned st = 0; st < a.samples_per_chain; st++) {
        for(unsigned k = 0; k < a.num_sweeps * N; k++) propose();
        // the sample refreshes th; the chain continues from the fresh sums
        deep_process_sample(c, with_op ? &op : nullptr, s, lane, (size_t)st * a.n_chains + chain, out, false, &lpsi,
                            &as);
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

template<typename T>
__global__ void __launch_bounds__(256, 1) deep_exact_kernel(DeepDev<T> p, OpDev op, int with_op, uint64_t n_conf,
                                                          SampleOut out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const DeepCtx<T> c = deep_stage<T>(p, smem_raw);
    const int lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for(uint64_t idx = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); idx < n_conf; idx += warps) {
        Conf<2> s;
        if(p.basis) {
            // base-4 digit x of idx is the type of site x (PauliString::enumerate, PauliString.hpp:30-35)
            s.w[0] = s.w[1] = 0;
            for(unsigned x = 0; x < p.sites; x++) {
                s.w[0] |= ((idx >> (2 * x)) & 1u) << x;
                s.w[1] |= ((idx >> (2 * x + 1)) & 1u) << x;
            }
        } else {
            s.w[0] = idx;
            s.w[1] = 0;
        }
        deep_process_sample(c, with_op ? &op : nullptr, s, lane, idx, out, true);
    }
}

template<typename T>
__global__ void __launch_bounds__(256, 1) deep_confs_kernel(DeepDev<T> p, OpDev op, int with_op, const uint64_t* confs,
                                                          uint64_t n, SampleOut out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const DeepCtx<T> c = deep_stage<T>(p, smem_raw);
    const int lane = threadIdx.x & 31;
    const uint64_t idx = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if(idx >= n) return;
    Conf<2> s;
    s.w[0] = confs[idx * kMaxWords];
    s.w[1] = confs[idx * kMaxWords + 1];
    deep_process_sample(c, with_op ? &op : nullptr, s, lane, idx, out, true);
}

template<typename T>
__global__ void deep_prepare_kernel(const cplx<double>* __restrict__ params, cplx<T>* __restrict__ w, unsigned n) {
    const unsigned k = blockIdx.x * blockDim.x + threadIdx.x;
    if(k < n) w[k] = cvt<T>(params[k]);
}

// ----------------------------------------------------------------------------------
constexpr size_t kDeepSmemCap = 200 * 1024;

template<typename T>
DeepDev<T> deep_view(const ann_psi_impl& psi, int basis) {
    DeepDev<T> p{};
    p.basis = basis;
    p.sites = basis ? psi.N / 3u : psi.N;
    const DeepHost& d = psi.deep;
    p.N = psi.N;
    p.L = (unsigned)d.sizes.size();
    p.Np = psi.Np;
    p.K = d.K;
    p.a_off = d.K;
    p.na = d.na;
    p.feat_beg = psi.feat_beg.as<uint32_t>();
    p.feat_zy = psi.feat_zy.as<uint64_t>();
    p.feat_c = psi.precision ? reinterpret_cast<const cplx<T>*>(psi.feat_c.p) : reinterpret_cast<const cplx<T>*>(psi.feat_cf.p);
    unsigned off = d.K + d.na, u = 0;
    for(unsigned l = 0; l < p.L; l++) {
        p.size[l] = d.sizes[l];
        p.C[l] = d.C[l];
        p.b_off[l] = off;
        off += p.size[l];
        p.w_off[l] = off;
        off += p.size[l] * p.C[l];
        p.uoff[l] = u;
        u += p.size[l];
        p.conn_off[l] = d.conn_off[l];
        p.rbeg_off[l] = d.rbeg_off[l];
        p.rq_off[l] = d.rq_off[l];
    }
    p.U = u;
    p.tab_len = d.tab_len;
    p.act = psi.act;
    p.a_in = psi.a_in;
    p.dup0 = d.dup0;
    p.lp = mk<T>((T)(psi.lp.real() + d.lp_ref.real()), (T)(psi.lp.imag() + d.lp_ref.imag()));
    p.w = psi.cnn_w.as<cplx<T>>();
    p.fw = psi.fwd.as<cplx<T>>();
    p.tab = psi.deep_tab.as<uint16_t>();
    p.stage_w = 1;
    if(deep_fixed_bytes(p) + deep_warp_bytes(p) > kDeepSmemCap) p.stage_w = 0;
    return p;
}

template<typename T>
int deep_warps(const DeepDev<T>& p) {
    int w = 8;
    while(w > 1 && deep_fixed_bytes(p) + w * deep_warp_bytes(p) > kDeepSmemCap) w >>= 1;
    if(deep_fixed_bytes(p) + deep_warp_bytes(p) > kDeepSmemCap)
        throw Error(ANN_ERR_UNSUPPORTED, "PsiDeep layers too wide for the per-warp shared-memory buffers");
    return w;
}

template<typename K>
void deep_set_smem(K k, size_t bytes) {
    if(bytes > 48 * 1024) ANN_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
}

SampleOut deep_out(Rows& rows, void* O, size_t ldO, bool want_eloc) {
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

void deep_rows(Rows& rows, size_t n) {
    rows.n = n;
    rows.conf.ensure(n * kMaxWords * sizeof(uint64_t));
    rows.log_psi.ensure(n * sizeof(cplx<double>));
    rows.eloc.ensure(n * sizeof(cplx<double>));
    rows.weight.ensure(n * sizeof(double));
}

template<typename T>
void deep_run_T(ann_psi_impl& psi, const ann_op_impl* op, ann_ens_impl& ens, const SampleTargets& t,
                cudaStream_t st) {
    const DeepDev<T> p = deep_view<T>(psi, ens.basis);
    const int wpb = deep_warps(p);
    const size_t smem = deep_fixed_bytes(p) + wpb * deep_warp_bytes(p);
    OpDev ov{};
    if(op) ov = op->view();
    if(ens.kind == 0) {
        const uint64_t n_conf = ens.num_steps();
        deep_rows(*t.rows, n_conf);
        SampleOut out = deep_out(*t.rows, t.O, t.ldO, t.want_eloc && op);
        uint64_t blocks = (n_conf + wpb - 1) / wpb;
        if(blocks > 152ull * 16) blocks = 152ull * 16;
        deep_set_smem(deep_exact_kernel<T>, smem);
        deep_exact_kernel<T><<<(unsigned)blocks, wpb * 32, smem, st>>>(p, ov, op ? 1 : 0, n_conf, out);
        check_launch("deep_exact_kernel");
        return;
    }
    const unsigned spc = ens.num_samples / ens.n_chains;
    deep_rows(*t.rows, (size_t)spc * ens.n_chains);
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
    SampleOut out = deep_out(*t.rows, t.O, t.ldO, t.want_eloc && op);
    deep_set_smem(deep_mc_kernel<T>, smem);
    deep_mc_kernel<T><<<(ens.n_chains + wpb - 1) / wpb, wpb * 32, smem, st>>>(p, ov, op ? 1 : 0, a, out);
    check_launch("deep_mc_kernel");
    ens.chains_valid = true;
}

template<typename T>
void deep_confs_T(ann_psi_impl& psi, const ann_op_impl* op, const uint64_t* confs, size_t n, Rows& rows, void* O,
                  size_t ldO, cudaStream_t st, int basis) {
    const DeepDev<T> p = deep_view<T>(psi, basis);
    const int wpb = deep_warps(p);
    const size_t smem = deep_fixed_bytes(p) + wpb * deep_warp_bytes(p);
    OpDev ov{};
    if(op) ov = op->view();
    deep_rows(rows, n);
    SampleOut out = deep_out(rows, O, ldO, op != nullptr);
    if(n == 0) return;
    deep_set_smem(deep_confs_kernel<T>, smem);
    deep_confs_kernel<T><<<(unsigned)((n + wpb - 1) / wpb), wpb * 32, smem, st>>>(p, ov, op ? 1 : 0, confs, n, out);
    check_launch("deep_confs_kernel");
}

// device table of a PsiDeep layer structure: connection blocks | per layer the lists of the
// units below (rbeg: units below + 1 offsets, rq: C x M entries). The lists follow the reference's
// compile_rhs_connections_and_weights order (PsiDeep.cu:213-242): units ascending, then
// connections ascending within a unit.
void deep_build_tables(ann_psi_impl& p) {
    DeepHost& h = p.deep;
    const unsigned L = (unsigned)h.sizes.size();
    // table: connection blocks | per layer (rbeg: in + 1 entries, rq: C x M entries)
    std::vector<uint16_t> tab;
    unsigned coff = 0;
    h.conn_off.assign(L, 0);
    h.rbeg_off.assign(L, 0);
    h.rq_off.assign(L, 0);
    for(unsigned l = 0; l < L; l++) {
        const unsigned in = l ? h.sizes[l - 1] : p.N, M = h.sizes[l], C = h.C[l];
        h.conn_off[l] = (unsigned)tab.size();
        for(unsigned k = 0; k < C * M; k++) {
            const unsigned u = h.conn[coff + k];
            if(u >= in) throw Error(ANN_ERR_INVALID, "connection index out of range");
            tab.push_back((uint16_t)u);
        }
        coff += C * M;
    }
    coff = 0;
    h.dup0 = 0;
    for(unsigned l = 0; l < L; l++) {
        const unsigned in = l ? h.sizes[l - 1] : p.N, M = h.sizes[l], C = h.C[l];
        std::vector<std::vector<uint16_t>> lists(in);
        for(unsigned j = 0; j < M; j++)
            for(unsigned i = 0; i < C; i++) lists[h.conn[coff + i * M + j]].push_back((uint16_t)(i * M + j));
        if(l == 0)
            for(const auto& li : lists) {
                std::vector<unsigned> js;
                for(uint16_t q : li) js.push_back(q % M);
                std::sort(js.begin(), js.end());
                if(std::adjacent_find(js.begin(), js.end()) != js.end()) h.dup0 = 1;
            }
        h.rbeg_off[l] = (unsigned)tab.size();
        unsigned acc = 0;
        for(unsigned u = 0; u <= in; u++) {
            tab.push_back((uint16_t)acc);
            if(u < in) acc += (unsigned)lists[u].size();
        }
        h.rq_off[l] = (unsigned)tab.size();
        for(const auto& li : lists) tab.insert(tab.end(), li.begin(), li.end());
        coff += C * M;
    }
    h.tab_len = (unsigned)tab.size();
    upload(p.deep_tab, tab.data(), tab.size() * sizeof(uint16_t));
}

}  // namespace

void deep_prepare(ann_psi_impl& psi, cudaStream_t st) {
    const unsigned n = psi.Np;
    if(psi.precision == 0)
        deep_prepare_kernel<float><<<(n + 255) / 256, 256, 0, st>>>(psi.params.as<cplx<double>>(),
                                                                    psi.cnn_w.as<cplx<float>>(), n);
    else
        deep_prepare_kernel<double><<<(n + 255) / 256, 256, 0, st>>>(psi.params.as<cplx<double>>(),
                                                                     psi.cnn_w.as<cplx<double>>(), n);
    check_launch("deep_prepare_kernel");
}

void deep_run(ann_psi_impl& psi, const ann_op_impl* op, ann_ens_impl& ens, const SampleTargets& t, cudaStream_t st) {
    if(psi.precision == 0) deep_run_T<float>(psi, op, ens, t, st);
    else deep_run_T<double>(psi, op, ens, t, st);
}

void deep_ensure(ann_psi_impl& psi) {
    if(psi.kind == 2 || psi.deep.tab_len) return;
    if(psi.kind != 0 || psi.layout != ANN_LAYOUT_DEEP)
        throw Error(ANN_ERR_UNSUPPORTED, "Pauli strings are built for PsiDeep (any depth)");
    psi.deep.sizes = {psi.M};
    psi.deep.C = {psi.C};
    psi.deep.conn = psi.conn;
    psi.deep.na = psi.N;
    deep_build_tables(psi);
    psi.cnn_w.ensure((size_t)psi.Np * psi.elem_bytes());
    deep_prepare(psi, nullptr);
    ANN_CUDA(cudaStreamSynchronize(nullptr));
}

void deep_confs(ann_psi_impl& psi, const ann_op_impl* op, const uint64_t* confs, size_t n, Rows& rows, void* O,
                size_t ldO, cudaStream_t st, int basis) {
    if(psi.precision == 0) deep_confs_T<float>(psi, op, confs, n, rows, O, ldO, st, basis);
    else deep_confs_T<double>(psi, op, confs, n, rows, O, ldO, st, basis);
}

}  // namespace ann

using namespace ann;

// PsiDeep(num_sites, a, b, connections, W, final_weights, log_prefactor, gpu) with any
// number of hidden layers (PsiDeep.hpp:488-560). The per-input-unit lists follow the
// reference's compile_rhs_connections_and_weights order (PsiDeep.cu:213-242): units
// ascending, then connections ascending within a unit.
extern "C" int ann_psi_create_deep(const ann_deep_desc* d, ann_psi** out) {
    try {
        if(!d || !out || !d->sizes || !d->connectivity || !d->connections || !d->params || !d->final_weights)
            throw Error(ANN_ERR_INVALID, "null argument");
        if(d->N < 1 || d->N > 128) throw Error(ANN_ERR_INVALID, "PsiDeep needs 1 <= N <= 128 input units");
        if(d->num_layers < 1 || d->num_layers > kDeepMaxLayers)
            throw Error(ANN_ERR_UNSUPPORTED, "PsiDeep supports 1 to 4 hidden layers");
        if(d->precision != ANN_PREC_FP32 && d->precision != ANN_PREC_FP64) throw Error(ANN_ERR_INVALID, "precision");
        if(d->activation != ANN_ACT_POLY && d->activation != ANN_ACT_LOGCOSH) throw Error(ANN_ERR_INVALID, "activation");
        auto* p = new ann_psi();
        try {
            p->kind = 2;
            p->precision = d->precision;
            p->act = d->activation;
            p->a_in = d->a_in_log_psi ? 1 : 0;
            p->N = d->N;
            p->NW = d->N > 64 ? 2 : 1;
            p->lp = zd(d->log_prefactor[0], d->log_prefactor[1]);
            DeepHost& h = p->deep;
            const unsigned L = d->num_layers;
            h.sizes.assign(d->sizes, d->sizes + L);
            h.C.assign(d->connectivity, d->connectivity + L);
            unsigned np = d->N, total = 0;
            for(unsigned l = 0; l < L; l++) {
                const unsigned in = l ? h.sizes[l - 1] : d->N;
                if(h.sizes[l] < 1 || h.sizes[l] > 1024) throw Error(ANN_ERR_INVALID, "1..1024 units per layer");
                if(h.C[l] < 1 || h.C[l] > in) throw Error(ANN_ERR_INVALID, "connectivity must be in [1, units below]");
                if((size_t)h.C[l] * h.sizes[l] > 65535) throw Error(ANN_ERR_UNSUPPORTED, "C x M above 65535 per layer");
                np += h.sizes[l] * (1 + h.C[l]);
                total += h.C[l] * h.sizes[l];
            }
            if(np != d->num_params) throw Error(ANN_ERR_INVALID, "num_params does not match the layer structure");
            p->Np = np;
            h.conn.assign(d->connections, d->connections + total);
            h.na = d->N;
            deep_build_tables(*p);
            const unsigned ML = h.sizes[L - 1];
            p->fw.assign(ML, zd(0, 0));
            const size_t es = p->elem_bytes();
            std::vector<unsigned char> fwb(ML * es, 0);
            for(unsigned j = 0; j < ML; j++) {
                p->fw[j] = zd(d->final_weights[2 * j], d->final_weights[2 * j + 1]);
                if(p->precision == 0) {
                    const float v[2] = {(float)p->fw[j].real(), (float)p->fw[j].imag()};
                    std::memcpy(&fwb[j * es], v, es);
                } else {
                    std::memcpy(&fwb[j * es], &d->final_weights[2 * j], es);
                }
            }
            upload(p->fwd, fwb.data(), fwb.size());
            upload(p->params, d->params, (size_t)p->Np * 16);
            p->cnn_w.ensure((size_t)p->Np * es);
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
