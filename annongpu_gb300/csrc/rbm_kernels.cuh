// RBM-family wavefunctions on the GPU: one warp or half-warp per Markov chain (one warp
// per enumerated configuration), hidden-unit angles held in registers and updated
// incrementally.
//
// Covers the reference's PsiRBM (include/quantum_state/PsiRBM.hpp:69-176) and
// PsiDeep with one hidden layer (include/quantum_state/PsiDeep.hpp:138-445): both
// are theta_j = b_j + sum_c W[c,j] s[conn(c,j)], log psi = log_pref + (a.s) +
// sum_j fw_j f(theta_j). The sampler follows MonteCarlo_t::kernel_foreach /
// mc_update (include/ensembles/MonteCarlo.hpp:55-177) and the local energy follows
// StandartOperator::local_energy (include/operator/Operator.hpp:36-121), restated
// with angle deltas instead of update / full recompute / revert.
#pragma once

#include "ann_common.cuh"
#include "made.cuh"

namespace ann {

constexpr int kWarpsPerBlock = 8;

// A team of TL lanes runs one chain: TL = 32 (a whole warp) or 16 (half a warp, two chains
// per warp: fewer shuffle levels per proposal and twice the independent units per lane).
// Below, `lane` is the lane within the team; unit j of the padded width lives in team lane
// j % TL, register slot j / TL. Slot u of a half-warp team belongs to virtual lane u % 2
// (unit u * 16 + l is unit (u / 2) * 32 + l + 16 (u % 2)), so every sum below, taken per
// virtual lane and combined by team_total, equals the whole-warp sum bit for bit: the
// choice of team changes speed, not chains.

// Wavefunction as the kernels see it. Unit j of the padded width Mpad lives in lane
// j % TL of the chain's team, register slot j / TL (Mpad = TL * U).
template<typename T>
struct RbmDev {
    unsigned N, M, Mpad, C, Np;
    unsigned Uact;       // register slots in use (Mpad / TL <= U)
    int layout;          // 0: params = W (PsiRBM), 1: params = [a | b | W] (PsiDeep)
    int a_in_log_psi;    // 1: log psi includes a.s
    int act;             // Activation
    const cplx<T>* Wd;   // N x Mpad, dense site -> unit weights (sum over connections)
    const cplx<T>* a;    // N
    const cplx<T>* b;    // Mpad (zero padded)
    const cplx<T>* fw;   // Mpad (zero padded)
    const uint16_t* conn;// C x M: input site of connection (c, j)
    cplx<T> lp;          // log prefactor
    int fw_real;         // every final weight is real: Re(fw f) = Re fw Re f
};

// Per lane: the angles of units lane, lane + TL, ... and the real parts of their
// log-psi terms. A Metropolis decision needs only Re(log psi' - log psi), so proposals
// evaluate the real part of the activation alone; the complex terms are formed when a
// sample is taken.
template<typename T, int U>
struct Lane {
    cplx<T> th[U];   // angles
    T fr[U];         // Re(fw_j f(theta_j))
    T fwr[U];        // Re fw_j (registers: read by every proposal when the final weights are real)
};

// Re f(z) of the first-layer activation: the polynomial's real part from z^2 and z^4
// (Re z^6 = Re z^4 Re z^2 - Im z^4 Im z^2), or Re log cosh z = Re w + log|1 + e^{-2w}| - log 2
template<typename T>
__device__ __forceinline__ T act_f_re(cplx<T> z, int act) {
    if(act == kPoly) {
        const T x2r = z.re * z.re - z.im * z.im, x2i = T(2) * z.re * z.im;
        const T x4r = x2r * x2r - x2i * x2i, x4i = T(2) * x2r * x2i;
        const T x6r = x4r * x2r - x4i * x2i;
        return T(0.5) * x2r - T(1.0 / 12.0) * x4r + T(1.0 / 45.0) * x6r;
    }
    const cplx<T> w = z.re >= T(0) ? z : -z;
    const cplx<T> e = cexp(T(-2) * w);
    return w.re + T(0.5) * flog(norm2(mk<T>(T(1) + e.re, e.im))) - T(0.69314718055994530942);
}

// Re(fw_j f(z)) of unit j = u * TL + lane (complex final weights are read from memory)
template<typename T, int U, int TL = 32>
__device__ __forceinline__ T fw_f_re(const RbmDev<T>& p, const Lane<T, U>& L, int u, int lane, cplx<T> z) {
    if(p.fw_real) return L.fwr[u] * act_f_re(z, p.act);
    const cplx<T> fw = p.fw[u * TL + lane];
    const cplx<T> f = act_f(z, p.act, 0);
    return fw.re * f.re - fw.im * f.im;
}

// ---- two-wide FP32 unit work (sm_100+ packed FP32 instructions) ----
// For complex64 chains with the polynomial activation and real final weights (PsiRBM),
// proposals and recompute() evaluate the units two values per instruction: angle changes
// and new angles as (re, im) of one unit, the activation's real part as (slot u, slot
// u + 1). Each component of a two-wide instruction rounds as the scalar instruction does,
// and every step below is an explicit round-to-nearest operation, so the results do not
// depend on the team width or on the compiler's contraction choices.
__device__ __forceinline__ float2 as_f2(cplx<float> c) { return make_float2(c.re, c.im); }
__device__ __forceinline__ float2 dup2(float v) { return make_float2(v, v); }

// a += b; a += s b with s = +-1 (exact product): one instruction for complex64
template<typename T>
__device__ __forceinline__ void add_to(cplx<T>& a, cplx<T> b) { a += b; }
__device__ __forceinline__ void add_to(cplx<float>& a, cplx<float> b) {
    const float2 r = __fadd2_rn(as_f2(a), as_f2(b));
    a = mk(r.x, r.y);
}
template<typename T>
__device__ __forceinline__ void add_signed(cplx<T>& a, T s, cplx<T> b) {
    a.re += s * b.re;
    a.im += s * b.im;
}
__device__ __forceinline__ void add_signed(cplx<float>& a, float s, cplx<float> b) {
    const float2 r = __ffma2_rn(dup2(s), as_f2(b), as_f2(a));
    a = mk(r.x, r.y);
}

// Re f(z) of the polynomial f = z^2/2 - z^4/12 + z^6/45 for two units, from P = Re z^2 =
// x^2 - y^2 and q = x y: Re z^4 = P^2 - 4 q^2, Re z^6 = P (P^2 - 12 q^2), so
// Re f = P/2 - P^2/12 + q^2/3 + (P/45) (P^2 - 12 q^2).
__device__ __forceinline__ float2 poly_re2(float2 z0, float2 z1) {
    const float2 s0 = __fmul2_rn(z0, z0), s1 = __fmul2_rn(z1, z1);
    const float2 P = make_float2(__fsub_rn(s0.x, s0.y), __fsub_rn(s1.x, s1.y));
    const float2 q = make_float2(__fmul_rn(z0.x, z0.y), __fmul_rn(z1.x, z1.y));
    const float2 A = __fmul2_rn(P, P), b = __fmul2_rn(q, q);
    const float2 c = __ffma2_rn(b, dup2(-12.f), A);
    const float2 t = __ffma2_rn(A, dup2(-1.f / 12.f), __fmul2_rn(b, dup2(1.f / 3.f)));
    const float2 h = __ffma2_rn(P, dup2(0.5f), t);
    return __ffma2_rn(__fmul2_rn(P, dup2(1.f / 45.f)), c, h);
}

// the packed path applies (complex64, polynomial activation, real final weights)
template<typename T>
__device__ __forceinline__ bool packed_units(const RbmDev<T>& p) {
    if constexpr(sizeof(T) == 4) return p.act == kPoly && p.fw_real;
    else return false;
}

// L.fr of every slot from L.th and L.fwr, two slots per step (slots past Uact hold
// th = 0 and fwr = 0, so their terms are 0)
template<int U>
__device__ __forceinline__ void lane_fr2(Lane<float, U>& L) {
#pragma unroll
    for(int u = 0; u < U; u += 2) {
        const float2 z1 = u + 1 < U ? as_f2(L.th[u + 1]) : make_float2(0.f, 0.f);
        const float2 fw = make_float2(L.fwr[u], u + 1 < U ? L.fwr[u + 1] : 0.f);
        const float2 f = __fmul2_rn(fw, poly_re2(as_f2(L.th[u]), z1));
        L.fr[u] = f.x;
        if(u + 1 < U) L.fr[u + 1] = f.y;
    }
}

// theta_j = b_j + sum_i s_i Wd[i][j] from scratch
template<typename T, int NW, int U, int TL = 32>
__device__ __forceinline__ void recompute(const RbmDev<T>& p, const cplx<T>* __restrict__ Wd,
                                          const Conf<NW>& s, Lane<T, U>& L, int lane) {
#pragma unroll
    for(int u = 0; u < U; u++) {
        const bool on = (unsigned)u < p.Uact;
        L.th[u] = on ? p.b[u * TL + lane] : mk<T>(T(0), T(0));
        L.fwr[u] = on ? p.fw[u * TL + lane].re : T(0);
    }
    for(unsigned i = 0; i < p.N; i++) {
        const T si = spin_bit(s, i) ? T(1) : T(-1);
        const cplx<T>* row = Wd + (size_t)i * p.Mpad + lane;
#pragma unroll
        for(int u = 0; u < U; u++) {
            if((unsigned)u >= p.Uact) break;
            add_signed(L.th[u], si, row[u * TL]);
        }
    }
    if constexpr(sizeof(T) == 4) {
        if(packed_units(p)) {
            lane_fr2<U>(L);
            return;
        }
    }
#pragma unroll
    for(int u = 0; u < U; u++) L.fr[u] = (unsigned)u < p.Uact ? fw_f_re<T, U, TL>(p, L, u, lane, L.th[u]) : T(0);
}

// complex terms fw_j f(theta_j) of the lane's units (sample time)
template<typename T, int U, int TL = 32>
__device__ __forceinline__ void lane_terms(const RbmDev<T>& p, const Lane<T, U>& L, int lane, cplx<T>* ft) {
#pragma unroll
    for(int u = 0; u < U; u++)
        ft[u] = (unsigned)u < p.Uact ? p.fw[u * TL + lane] * act_f(L.th[u], p.act, 0) : mk<T>(T(0), T(0));
}

// delta_re below on the two-wide path. The per-virtual-lane sums keep the scalar order:
// slot u of a half-warp team belongs to virtual lane u % 2, so the pair (u, u + 1) adds
// into (d[0], d[1]) in one instruction; a whole-warp team adds its slots one by one.
template<int NW, int U, int TL>
__device__ __forceinline__ float delta_re2(const RbmDev<float>& p, const cplx<float>* __restrict__ Wd,
                                           const Conf<NW>& s, const Lane<float, U>& L, int lane,
                                           const uint16_t* sites, unsigned nsites, cplx<float>* dth, float* fnew) {
    float2 dt[U];
#pragma unroll
    for(int u = 0; u < U; u++) dt[u] = make_float2(0.f, 0.f);
    float dvis = 0.f;
    for(unsigned q = 0; q < nsites; q++) {
        const unsigned i = sites[q];
        const float m2s = spin_bit(s, i) ? -2.f : 2.f;  // s'_i - s_i
        const float2 m2 = dup2(m2s);
        const cplx<float>* row = Wd + (size_t)i * p.Mpad + lane;
#pragma unroll
        for(int u = 0; u < U; u++) {
            if((unsigned)u >= p.Uact) break;
            dt[u] = __ffma2_rn(m2, as_f2(row[u * TL]), dt[u]);  // m2s w is exact
        }
        if(p.a_in_log_psi) dvis += m2s * p.a[i].re;
    }
    float d[kVirt<TL>];
    float2 dd = make_float2(0.f, 0.f);  // (d[0], d[1]) of a half-warp team
    d[0] = 0.f;
#pragma unroll
    for(int u = 0; u < U; u += 2) {
        if((unsigned)u >= p.Uact) {
            fnew[u] = 0.f;
            if(u + 1 < U) fnew[u + 1] = 0.f;
            continue;
        }
        // a slot past Uact has th = dt = 0 and fwr = fr = 0: its difference is +0
        const float2 z0 = __fadd2_rn(as_f2(L.th[u]), dt[u]);
        const float2 z1 = u + 1 < U ? __fadd2_rn(as_f2(L.th[u + 1]), dt[u + 1]) : make_float2(0.f, 0.f);
        const float2 fw = make_float2(L.fwr[u], u + 1 < U ? L.fwr[u + 1] : 0.f);
        const float2 f = __fmul2_rn(fw, poly_re2(z0, z1));
        const float2 fr = make_float2(L.fr[u], u + 1 < U ? L.fr[u + 1] : 0.f);
        const float2 df = __ffma2_rn(fr, dup2(-1.f), f);  // f - fr, rounded once
        fnew[u] = f.x;
        if(u + 1 < U) fnew[u + 1] = f.y;
        if constexpr(kVirt<TL> == 2) {
            dd = __fadd2_rn(dd, df);
        } else {
            d[0] += df.x;
            if(u + 1 < U) d[0] += df.y;
        }
    }
    if constexpr(kVirt<TL> == 2) {
        d[0] = dd.x;
        d[kVirt<TL> - 1] = dd.y;
    }
#pragma unroll
    for(int u = 0; u < U; u++) dth[u] = mk(dt[u].x, dt[u].y);
    return team_total<TL>(d) + dvis;
}

// Re(log psi(s') - log psi(s)) summed over the team for the flip of `sites`; leaves the
// angle changes in dth and the new real terms in fnew for an accepted move
template<typename T, int NW, int U, int TL = 32>
__device__ __forceinline__ T delta_re(const RbmDev<T>& p, const cplx<T>* __restrict__ Wd, const Conf<NW>& s,
                                      const Lane<T, U>& L, int lane, const uint16_t* sites, unsigned nsites,
                                      cplx<T>* dth, T* fnew) {
    if constexpr(sizeof(T) == 4) {
        if(packed_units(p)) return delta_re2<NW, U, TL>(p, Wd, s, L, lane, sites, nsites, dth, fnew);
    }
#pragma unroll
    for(int u = 0; u < U; u++) dth[u] = mk<T>(T(0), T(0));
    T dvis = T(0);
    for(unsigned q = 0; q < nsites; q++) {
        const unsigned i = sites[q];
        const T m2s = spin_bit(s, i) ? T(-2) : T(2);  // s'_i - s_i
        const cplx<T>* row = Wd + (size_t)i * p.Mpad + lane;
#pragma unroll
        for(int u = 0; u < U; u++) {
            if((unsigned)u >= p.Uact) break;
            const cplx<T> w = row[u * TL];
            dth[u].re += m2s * w.re;
            dth[u].im += m2s * w.im;
        }
        if(p.a_in_log_psi) dvis += m2s * p.a[i].re;
    }
    T d[kVirt<TL>];
#pragma unroll
    for(int k = 0; k < kVirt<TL>; k++) d[k] = T(0);
#pragma unroll
    for(int u = 0; u < U; u++) {
        if((unsigned)u >= p.Uact) {
            fnew[u] = T(0);
            continue;
        }
        fnew[u] = fw_f_re<T, U, TL>(p, L, u, lane, L.th[u] + dth[u]);
        d[u % kVirt<TL>] += fnew[u] - L.fr[u];
    }
    return team_total<TL>(d) + dvis;
}

// sum over the team of fw_j (f(theta_j + dtheta_j) - f(theta_j)) for the sites in `sites`
template<typename T, int NW, int U, int TL = 32>
__device__ __forceinline__ cplx<T> delta_log_psi(const RbmDev<T>& p, const cplx<T>* __restrict__ Wd,
                                                 const Conf<NW>& s, const Lane<T, U>& L, const cplx<T>* ft,
                                                 int lane, const uint16_t* sites, unsigned nsites,
                                                 cplx<T>* dth, cplx<T>* fnew) {
#pragma unroll
    for(int u = 0; u < U; u++) dth[u] = mk<T>(T(0), T(0));
    cplx<T> dvis = mk<T>(T(0), T(0));
    for(unsigned q = 0; q < nsites; q++) {
        const unsigned i = sites[q];
        const T m2s = spin_bit(s, i) ? T(-2) : T(2);  // s'_i - s_i
        const cplx<T>* row = Wd + (size_t)i * p.Mpad + lane;
#pragma unroll
        for(int u = 0; u < U; u++) {
            if((unsigned)u >= p.Uact) break;
            const cplx<T> w = row[u * TL];
            dth[u].re += m2s * w.re;
            dth[u].im += m2s * w.im;
        }
        if(p.a_in_log_psi) dvis += m2s * p.a[i];
    }
    cplx<T> d[kVirt<TL>];
#pragma unroll
    for(int k = 0; k < kVirt<TL>; k++) d[k] = mk<T>(T(0), T(0));
#pragma unroll
    for(int u = 0; u < U; u++) {
        if((unsigned)u >= p.Uact) {
            fnew[u] = mk<T>(T(0), T(0));
            continue;
        }
        fnew[u] = p.fw[u * TL + lane] * act_f(L.th[u] + dth[u], p.act, 0);
        d[u % kVirt<TL>] += fnew[u] - ft[u];
    }
    return team_total<TL>(d) + dvis;
}

// local energy of configuration s (Operator.hpp:86-121 semantics)
template<typename T, int NW, int U, int TL = 32>
__device__ cplx<double> local_energy(const RbmDev<T>& p, const cplx<T>* __restrict__ Wd, const OpDev& op,
                                     const Conf<NW>& s, const Lane<T, U>& L, const cplx<T>* ft, int lane) {
    // arithmetic in the kernel precision T (coefficients are stored in FP64 and
    // rounded once); the FP64 pipe is reserved for the final conversion
    // diagonal strings, split over lanes
    T dre[kVirt<TL>], dim[kVirt<TL>];
#pragma unroll
    for(int k = 0; k < kVirt<TL>; k++) {
        dre[k] = T(0);
        dim[k] = T(0);
        for(unsigned n = lane + k * TL; n < op.n_diag; n += 32) {
            int neg = 0;
#pragma unroll
            for(int w = 0; w < NW; w++) neg += __popcll((~s.w[w]) & op.diag_mask[n * op.nw + w]);
            const T c_re = diag_coeff<T>(op)[2 * n], c_im = diag_coeff<T>(op)[2 * n + 1];
            dre[k] += (neg & 1) ? -c_re : c_re;
            dim[k] += (neg & 1) ? -c_im : c_im;
        }
    }
    cplx<T> e = mk<T>(team_total<TL>(dre), team_total<TL>(dim));
    cplx<T> dth[U], fnew[U];
    for(unsigned g = 0; g < op.n_groups; g++) {
        // summed matrix element of the group first: when it vanishes (e.g. XX + YY on
        // aligned spins) the psi ratio is not needed
        cplx<T> cg = mk<T>(T(0), T(0));
        for(unsigned k = op.grp_str_begin[g]; k < op.grp_str_begin[g + 1]; k++) {
            int neg = 0;
#pragma unroll
            for(int w = 0; w < NW; w++) neg += __popcll((~s.w[w]) & op.str_mask[k * op.nw + w]);
            const T c_re = str_coeff<T>(op)[2 * k], c_im = str_coeff<T>(op)[2 * k + 1];
            cg.re += (neg & 1) ? -c_re : c_re;
            cg.im += (neg & 1) ? -c_im : c_im;
        }
        if(cg.re == T(0) && cg.im == T(0)) continue;
        const unsigned sb = op.grp_site_begin[g], se = op.grp_site_begin[g + 1];
        const cplx<T> d = delta_log_psi<T, NW, U, TL>(p, Wd, s, L, ft, lane, op.grp_sites + sb, se - sb, dth, fnew);
        e += cg * cexp(d);
    }
    return cvt<double>(e);
}

// log psi, local energy, O_k row and sample bookkeeping for one configuration
template<typename T, int NW, int U, int TL = 32>
__device__ void process_sample(const RbmDev<T>& p, const cplx<T>* __restrict__ Wd, const OpDev* op,
                               const Conf<NW>& s, const Lane<T, U>& L, int lane, size_t row,
                               const SampleOut& out, bool exact_weight) {
    cplx<T> ft[U];
    lane_terms<T, U, TL>(p, L, lane, ft);
    cplx<T> lpart[kVirt<TL>];
#pragma unroll
    for(int k = 0; k < kVirt<TL>; k++) lpart[k] = mk<T>(T(0), T(0));
#pragma unroll
    for(int u = 0; u < U; u++) lpart[u % kVirt<TL>] += ft[u];
    if(p.a_in_log_psi)
#pragma unroll
        for(int k = 0; k < kVirt<TL>; k++)
            for(unsigned i = lane + k * TL; i < p.N; i += 32) lpart[k] += (spin_bit(s, i) ? T(1) : T(-1)) * p.a[i];
    const cplx<T> lsum = team_total<TL>(lpart);
    const cplx<double> lpsi = cvt<double>(lsum) + cvt<double>(p.lp);
    cplx<double> e = mk<double>(0.0, 0.0);
    if(op) e = local_energy<T, NW, U, TL>(p, Wd, *op, s, L, ft, lane);
    if(lane == 0) {
        for(int w = 0; w < kMaxWords; w++) out.conf[row * kMaxWords + w] = w < NW ? s.w[w] : 0;
        out.log_psi[row] = lpsi;
        if(out.eloc) out.eloc[row] = e;
        if(exact_weight && out.weight) out.weight[row] = exp(2.0 * lpsi.re);
        if(!(isfinite(lpsi.re) && isfinite(lpsi.im) && isfinite(e.re) && isfinite(e.im)))
            atomicOr(out.status, kStatusNonFinite);
    }
    if(out.O) {
        cplx<T>* O = reinterpret_cast<cplx<T>*>(out.O) + row * out.ldO;
        cplx<T> g[U];
#pragma unroll
        for(int u = 0; u < U; u++)
            g[u] = (unsigned)u < p.Uact ? p.fw[u * TL + lane] * act_df(L.th[u], p.act, 0) : mk<T>(T(0), T(0));
        unsigned off = 0;
        if(p.layout == 1) {
            for(unsigned i = lane; i < p.N; i += TL) O[i] = mk<T>(spin_bit(s, i) ? T(1) : T(-1), T(0));
#pragma unroll
            for(int u = 0; u < U; u++) {
                const unsigned j = u * TL + lane;
                if(j < p.M) O[p.N + j] = g[u];
            }
            off = p.N + p.M;
        }
        for(unsigned c = 0; c < p.C; c++) {
            const uint16_t* cr = p.conn + (size_t)c * p.M;
            cplx<T>* orow = O + off + (size_t)c * p.M;
#pragma unroll
            for(int u = 0; u < U; u++) {
                const unsigned j = u * TL + lane;
                if(j < p.M) orow[j] = spin_bit(s, cr[j]) ? g[u] : -g[u];
            }
        }
    }
}

// Copies Wd to shared memory when it fits (w_smem != 0); returns the pointer to use.
template<typename T>
__device__ __forceinline__ const cplx<T>* stage_Wd(const RbmDev<T>& p, int w_smem, cplx<T>* smem) {
    if(!w_smem) return p.Wd;
    const size_t n = (size_t)p.N * p.Mpad;
    const float4* src = reinterpret_cast<const float4*>(p.Wd);
    float4* dst = reinterpret_cast<float4*>(smem);
    const size_t n4 = n * sizeof(cplx<T>) / sizeof(float4);
    for(size_t k = threadIdx.x; k < n4; k += blockDim.x) dst[k] = src[k];
    __syncthreads();
    return smem;
}

// One chain: thermalisation (when drawing fresh configurations), then per sample
// the local sweeps, the learned independence moves, and the sample bookkeeping.
template<typename T, int NW, int U, int TL = 32>
__device__ __forceinline__ void mc_chain(const RbmDev<T>& p, const cplx<T>* __restrict__ Wd, const OpDev& op, int with_op,
                         const McArgs& a, const SampleOut& out, unsigned chain, int lane, bool use_made,
                         const MadeSm& ms, float* mh) {
    const unsigned N = p.N;

    Conf<NW> s;
    uint64_t t;
    unsigned tape_pos = 0;
    const bool tape = a.tape_site != nullptr;
    if(tape) {
        for(int w = 0; w < NW; w++) s.w[w] = a.chain_conf[(size_t)chain * kMaxWords + w];
        t = 0;
    } else if(a.do_init) {
        t = a.chain_counter[chain];
        if(a.n_up < 0) {
            const u32x4 r = philox4x32_10(a.k0, a.k1, u32x4{(uint32_t)t, (uint32_t)(t >> 32), chain, 1u});
            s.w[0] = (uint64_t)r.x | ((uint64_t)r.y << 32);
            if(NW > 1) s.w[NW - 1] = (uint64_t)r.z | ((uint64_t)r.w << 32);
            for(int w = 0; w < NW; w++) {
                const unsigned lo = 64u * w;
                if(N <= lo) s.w[w] = 0;
                else if(N - lo < 64u) s.w[w] &= ((uint64_t)1 << (N - lo)) - 1u;
            }
        } else {
            for(int w = 0; w < NW; w++) s.w[w] = 0;
            for(int k = 0; k < a.n_up; k++) {
                const uint64_t tk = t + (uint64_t)k;
                const u32x4 r = philox4x32_10(a.k0, a.k1, u32x4{(uint32_t)tk, (uint32_t)(tk >> 32), chain, 2u});
                unsigned target = mulhi32(r.x, N - (unsigned)k);
                for(unsigned i = 0; i < N; i++) {
                    if(!spin_bit(s, i)) {
                        if(target == 0) { s.w[i >> 6] |= (uint64_t)1 << (i & 63u); break; }
                        target--;
                    }
                }
            }
        }
    } else {
        for(int w = 0; w < NW; w++) s.w[w] = a.chain_conf[(size_t)chain * kMaxWords + w];
        t = a.chain_counter[chain];
    }

    Lane<T, U> L;
    recompute<T, NW, U, TL>(p, Wd, s, L, lane);
    unsigned long long n_acc = 0, n_rej = 0, m_acc = 0, m_rej = 0;
    const unsigned mask = team_mask<TL>();
    // Philox words for the TL counters [rr_base, rr_base + TL), one per team lane
    uint64_t rr_base = 0;
    bool rr_valid = false;
    u32x4 rr = {0, 0, 0, 0};
    cplx<T> dth[U];
    T fnew[U];
    float lq_cur = 0.f;
    bool lq_stale = true;

    auto propose = [&]() {
        unsigned i, j = 0xFFFFFFFFu;
        double u = 0.0;
        float uf = 0.f;
        if(tape) {
            i = a.tape_site[(size_t)chain * a.tape_len + tape_pos];
            u = a.tape_u[(size_t)chain * a.tape_len + tape_pos];
            if(sizeof(T) == 4) uf = (float)u;
            tape_pos++;
        } else {
            if(!rr_valid || t - rr_base >= (unsigned)TL) {
                rr_valid = true;
                rr_base = t;
                const uint64_t tl = t + lane;
                rr = philox4x32_10(a.k0, a.k1, u32x4{(uint32_t)tl, (uint32_t)(tl >> 32), chain, 0u});
            }
            const unsigned k = (unsigned)(t - rr_base);
            const uint32_t r0 = __shfl_sync(mask, rr.x, k, TL);
            const uint32_t r1 = __shfl_sync(mask, rr.y, k, TL);
            const uint32_t r2 = __shfl_sync(mask, rr.z, k, TL);
            const uint32_t r3 = __shfl_sync(mask, rr.w, k, TL);
            t++;
            i = mulhi32(r0, N);
            if(a.move_kind == 1) {
                const unsigned bnd = mulhi32(r0, a.n_bonds);
                i = a.bonds[2 * bnd];
                j = a.bonds[2 * bnd + 1];
            } else if(a.move_kind == 2) {
                j = mulhi32(r1, N - 1u);
                j += (j >= i);
            }
            u = u53(r2, r3);
            if(sizeof(T) == 4) uf = __uint2float_rz(r3 >> 8) * 0x1.0p-24f;  // top 24 bits of u
        }
        uint16_t sites[2];
        unsigned ns = 1;
        sites[0] = (uint16_t)i;
        if(a.move_kind != 0 && !tape) {
            if(spin_bit(s, i) == spin_bit(s, j)) { n_rej++; return; }
            sites[1] = (uint16_t)j;
            ns = 2;
        }
        const T d = delta_re<T, NW, U, TL>(p, Wd, s, L, lane, sites, ns, dth, fnew);
        const T ratio = fexp(T(2) * d);
        // MonteCarlo.hpp:158-160: accept if ratio > 1 or u <= ratio; u < 1 makes
        // the first clause redundant.
        // complex64 chains compare in FP32 (GB300's FP64 rate is 1/64 of FP32):
        // decisions differ from the FP64 comparison only within 2^-24 of a tie
        const bool accept = sizeof(T) == 4 ? (uf <= (float)ratio) : (u <= (double)ratio);
        if(accept) {
#pragma unroll
            for(int q = 0; q < U; q++) { add_to(L.th[q], dth[q]); L.fr[q] = fnew[q]; }
            for(unsigned q = 0; q < ns; q++) flip(s, sites[q]);
            n_acc++;
            lq_stale = true;
        } else {
            n_rej++;
        }
    };

    // Metropolis-Hastings independence move with the learned proposal q:
    // accept s' ~ q with probability min(1, |psi(s')|^2 q(s) / (|psi(s)|^2 q(s')))
    auto propose_learned = [&]() {
        const uint64_t tq = t++;
        Conf<NW> s2;
        const float lq2 = made_sample<NW, 256 / TL, TL>(ms, a.k0, a.k1, (uint32_t)tq, (uint32_t)(tq >> 32), chain, s2,
                                                        lane);
        if(lq_stale) {
            lq_cur = made_logq<NW, TL>(ms, s, mh, lane);
            lq_stale = false;
        }
        Lane<T, U> L2;
        recompute<T, NW, U, TL>(p, Wd, s2, L2, lane);
        T dp[kVirt<TL>];
#pragma unroll
        for(int k = 0; k < kVirt<TL>; k++) dp[k] = T(0);
#pragma unroll
        for(int q = 0; q < U; q++) dp[q % kVirt<TL>] += L2.fr[q] - L.fr[q];
        if(p.a_in_log_psi)
#pragma unroll
            for(int k = 0; k < kVirt<TL>; k++)
                for(unsigned i = lane + k * TL; i < p.N; i += 32) {
                    const int b1 = spin_bit(s2, i), b0 = spin_bit(s, i);
                    if(b1 != b0) dp[k] += (b1 ? T(2) : T(-2)) * p.a[i].re;
                }
        const T d = team_total<TL>(dp);
        const u32x4 r = philox4x32_10(a.k0, a.k1, u32x4{(uint32_t)tq, (uint32_t)(tq >> 32), chain, 0u});
        const float lr = 2.f * (float)d + lq_cur - lq2;
        const float uf = __uint2float_rz(r.w >> 8) * 0x1.0p-24f;
        if(uf <= expf(lr)) {
            s = s2;
            L = L2;
            lq_cur = lq2;
            m_acc++;
        } else {
            m_rej++;
        }
    };

    if(a.do_init || tape)
        for(unsigned k = 0; k < a.num_therm * N; k++) propose();
    for(unsigned st = 0; st < a.samples_per_chain; st++) {
        for(unsigned k = 0; k < a.num_sweeps * N; k++) propose();
        if(use_made)
            for(unsigned k = 0; k < a.indep_per_sample; k++) propose_learned();
        recompute<T, NW, U, TL>(p, Wd, s, L, lane);  // removes accumulated rounding of the increments
        process_sample<T, NW, U, TL>(p, Wd, with_op ? &op : nullptr, s, L, lane,
                                     (size_t)st * a.n_chains + chain, out, false);
    }
    if(lane == 0) {
        if(!tape) {
            for(int w = 0; w < kMaxWords; w++) a.chain_conf[(size_t)chain * kMaxWords + w] = w < NW ? s.w[w] : 0;
            a.chain_counter[chain] = t;
        }
        atomicAdd(&a.acc_rej[0], n_acc);
        atomicAdd(&a.acc_rej[1], n_rej);
        if(use_made) {
            atomicAdd(&a.acc_rej[2], m_acc);
            atomicAdd(&a.acc_rej[3], m_rej);
        }
    }
}


// ---------------------------------------------------------------------------------
// Metropolis sampler: one team of TL lanes per chain (32 / TL chains per warp).
// complex64 chains with up to 128 hidden units: registers capped for three 8-warp CTAs per
// SM with whole-warp teams, two with half-warp teams (twice the units per lane; the
// sampler is latency-bound, the cap costs a few spilled words to L1)
template<typename T, int NW, int U, int TL>
__global__ void __launch_bounds__(256, (sizeof(T) == 4 && U * TL <= 128) ? (TL == 32 ? 3 : 2) : 1)
rbm_mc_kernel(RbmDev<T> p, OpDev op, int with_op, McArgs a, SampleOut out, int w_smem) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const cplx<T>* Wd = stage_Wd<T>(p, w_smem, reinterpret_cast<cplx<T>*>(smem_raw));
    // learned-proposal weights after Wd, then one H-float scratch per team; the drop rule
    // switches the moves off through a device flag (graph replays see it change)
    const bool use_made = a.made.N != 0 && (a.made_on == nullptr || *a.made_on != 0);
    MadeSm ms{};
    float* mh = nullptr;
    if(use_made) {
        unsigned char* mbase = smem_raw + (w_smem ? (((size_t)p.N * p.Mpad * sizeof(cplx<T>) + 15) & ~(size_t)15) : 0);
        if(a.made_smem) {
            ms = made_stage(a.made, mbase);
            mbase += made_smem_bytes(a.made.N, a.made.H);
        } else {
            ms = made_global(a.made);
        }
        mh = reinterpret_cast<float*>(mbase) + (threadIdx.x / TL) * a.made.H;  // one H-float scratch per team
        __syncthreads();
    }
    const int lane = threadIdx.x & (TL - 1);
    const unsigned chain = blockIdx.x * (blockDim.x / TL) + threadIdx.x / TL;
    if(chain >= a.n_chains) return;
    RbmDev<T> q = p;
    q.Uact = U;  // the padded width is exactly TL U here: the per-slot guards fold away
    mc_chain<T, NW, U, TL>(q, Wd, op, with_op, a, out, chain, lane, use_made, ms, mh);
}

// Drop rule of the learned proposal, on the device after each sampling pass: the flag
// goes to 0 when the pass's learned-move acceptance is below min_acceptance.
static __global__ void made_drop_rule_kernel(const unsigned long long* acc_rej, double min_acceptance, int* made_on) {
    const unsigned long long acc = acc_rej[2], tot = acc_rej[2] + acc_rej[3];
    if(tot > 0 && (double)acc < min_acceptance * (double)tot) *made_on = 0;
}

// ---------------------------------------------------------------------------------
// Exact summation: one warp per enumerated configuration (ExactSummation.hpp:33-72).
template<typename T, int NW, int U>
__global__ void __launch_bounds__(512)
rbm_exact_kernel(RbmDev<T> p, OpDev op, int with_op, uint64_t n_conf, SampleOut out, int w_smem) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const cplx<T>* Wd = stage_Wd<T>(p, w_smem, reinterpret_cast<cplx<T>*>(smem_raw));
    const int lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for(uint64_t idx = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); idx < n_conf; idx += warps) {
        Conf<NW> s;
        s.w[0] = idx;
        for(int w = 1; w < NW; w++) s.w[w] = 0;
        Lane<T, U> L;
        recompute<T, NW, U>(p, Wd, s, L, lane);
        process_sample<T, NW, U>(p, Wd, with_op ? &op : nullptr, s, L, lane, idx, out, true);
    }
}

// Explicit configurations (log_psi_s / psi_O_k of single configurations, batches).
template<typename T, int NW, int U>
__global__ void __launch_bounds__(512)
rbm_confs_kernel(RbmDev<T> p, OpDev op, int with_op, const uint64_t* confs, uint64_t n_conf, SampleOut out) {
    const int lane = threadIdx.x & 31;
    const uint64_t idx = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if(idx >= n_conf) return;
    Conf<NW> s;
    for(int w = 0; w < NW; w++) s.w[w] = confs[idx * kMaxWords + w];
    Lane<T, U> L;
    recompute<T, NW, U>(p, p.Wd, s, L, lane);
    process_sample<T, NW, U>(p, p.Wd, with_op ? &op : nullptr, s, L, lane, idx, out, true);
}

// params (FP64 master copy, layout 0 or 1) -> kernel-precision dense weights.
// One thread per hidden unit column; no two threads touch the same column.
template<typename T>
__global__ void rbm_prepare_kernel(RbmDev<T> p, const cplx<double>* __restrict__ params,
                                   cplx<T>* Wd, cplx<T>* a, cplx<T>* b) {
    const unsigned j = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned off = p.layout == 1 ? p.N + p.M : 0u;
    if(j < p.Mpad) {
        for(unsigned i = 0; i < p.N; i++) Wd[(size_t)i * p.Mpad + j] = mk<T>(T(0), T(0));
        if(j < p.M) {
            for(unsigned c = 0; c < p.C; c++) {
                const cplx<double> w = params[off + (size_t)c * p.M + j];
                cplx<T>& dst = Wd[(size_t)p.conn[(size_t)c * p.M + j] * p.Mpad + j];
                dst.re += (T)w.re;
                dst.im += (T)w.im;
            }
            b[j] = p.layout == 1 ? cvt<T>(params[p.N + j]) : mk<T>(T(0), T(0));
        } else {
            b[j] = mk<T>(T(0), T(0));
        }
    }
    if(j < p.N) a[j] = p.layout == 1 ? cvt<T>(params[j]) : mk<T>(T(0), T(0));
}

}  // namespace ann
