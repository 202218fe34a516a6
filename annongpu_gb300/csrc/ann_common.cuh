// Device-side building blocks shared by every kernel of the VMC inner loop:
// complex arithmetic, spin/Pauli bit algebra, activations, Philox4x32-10 and
// warp reductions. sm_103a only.
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace ann {

constexpr int kMaxWords = 2;  // spin configurations up to 128 sites (two 64-bit words)

// ---------------------------------------------------------------------------------
// complex numbers (interleaved re, im; 8 B for float, 16 B for double)
template<typename T>
struct alignas(2 * sizeof(T)) cplx {
    T re, im;
};

template<typename T> __host__ __device__ __forceinline__ cplx<T> mk(T r, T i) { return {r, i}; }
template<typename T> __host__ __device__ __forceinline__ cplx<T> operator+(cplx<T> a, cplx<T> b) { return {a.re + b.re, a.im + b.im}; }
template<typename T> __host__ __device__ __forceinline__ cplx<T> operator-(cplx<T> a, cplx<T> b) { return {a.re - b.re, a.im - b.im}; }
template<typename T> __host__ __device__ __forceinline__ cplx<T> operator-(cplx<T> a) { return {-a.re, -a.im}; }
template<typename T> __host__ __device__ __forceinline__ cplx<T> operator*(cplx<T> a, cplx<T> b) {
    return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template<typename T> __host__ __device__ __forceinline__ cplx<T> operator*(T s, cplx<T> a) { return {s * a.re, s * a.im}; }
template<typename T> __host__ __device__ __forceinline__ cplx<T>& operator+=(cplx<T>& a, cplx<T> b) { a.re += b.re; a.im += b.im; return a; }
template<typename T> __host__ __device__ __forceinline__ cplx<T> conj(cplx<T> a) { return {a.re, -a.im}; }
template<typename T> __host__ __device__ __forceinline__ T norm2(cplx<T> a) { return a.re * a.re + a.im * a.im; }
template<typename D, typename S> __host__ __device__ __forceinline__ cplx<D> cvt(cplx<S> a) { return {(D)a.re, (D)a.im}; }

// acc += a * b and acc += conj(a) * b as four fused multiply-adds (an expression such
// as acc.re += a.re*b.re - a.im*b.im compiles to a multiply, an FMA and an add)
template<typename T>
__host__ __device__ __forceinline__ void cmac(cplx<T>& acc, cplx<T> a, cplx<T> b) {
    acc.re = fma(a.re, b.re, acc.re);
    acc.re = fma(-a.im, b.im, acc.re);
    acc.im = fma(a.re, b.im, acc.im);
    acc.im = fma(a.im, b.re, acc.im);
}
template<typename T>
__host__ __device__ __forceinline__ void cmac_conj(cplx<T>& acc, cplx<T> a, cplx<T> b) {
    acc.re = fma(a.re, b.re, acc.re);
    acc.re = fma(a.im, b.im, acc.re);
    acc.im = fma(a.re, b.im, acc.im);
    acc.im = fma(-a.im, b.re, acc.im);
}

__device__ __forceinline__ float fexp(float x) { return expf(x); }
__device__ __forceinline__ double fexp(double x) { return exp(x); }
__device__ __forceinline__ void fsincos(float x, float* s, float* c) { sincosf(x, s, c); }
__device__ __forceinline__ void fsincos(double x, double* s, double* c) { sincos(x, s, c); }
__device__ __forceinline__ float flog1p(float x) { return log1pf(x); }
__device__ __forceinline__ double flog1p(double x) { return log1p(x); }
__device__ __forceinline__ float flog(float x) { return logf(x); }
__device__ __forceinline__ double flog(double x) { return log(x); }
__device__ __forceinline__ float fatan2(float y, float x) { return atan2f(y, x); }
__device__ __forceinline__ double fatan2(double y, double x) { return atan2(y, x); }

template<typename T>
__device__ __forceinline__ cplx<T> cexp(cplx<T> z) {
    T s, c;
    fsincos(z.im, &s, &c);
    const T e = fexp(z.re);
    return {e * c, e * s};
}
template<typename T>
__device__ __forceinline__ cplx<T> clog(cplx<T> z) {
    return {T(0.5) * flog(norm2(z)), fatan2(z.im, z.re)};
}
template<typename T>
__device__ __forceinline__ cplx<T> cdiv(cplx<T> a, cplx<T> b) {
    const T d = T(1) / norm2(b);
    return {(a.re * b.re + a.im * b.im) * d, (a.im * b.re - a.re * b.im) * d};
}

// ---------------------------------------------------------------------------------
// activations. Reference polynomial forms (include/quantum_state/psi_functions.hpp:
// my_logcosh :40-48, my_tanh :102-116); "exact" = log cosh / tanh.
enum Activation : int { kPoly = 0, kLogCosh = 1 };

template<typename T>
__device__ __forceinline__ cplx<T> poly_f(cplx<T> z, int layer) {
    const cplx<T> z2 = z * z, z4 = z2 * z2;
    if(layer == 0) return T(0.5) * z2 - T(1.0 / 12.0) * z4 + T(1.0 / 45.0) * (z4 * z2);
    return z - T(1.0 / 3.0) * (z2 * z) + T(2.0 / 15.0) * (z4 * z);
}
template<typename T>
__device__ __forceinline__ cplx<T> poly_df(cplx<T> z, int layer) {
    const cplx<T> z2 = z * z, z4 = z2 * z2;
    if(layer == 0) return z - T(1.0 / 3.0) * (z2 * z) + T(2.0 / 15.0) * (z4 * z);
    return mk<T>(T(1), T(0)) - z2 + T(2.0 / 3.0) * z4;
}
// log cosh z = w + log(1 + e^{-2w}) - log 2 with w = +-z, Re w >= 0 (cosh is even)
template<typename T>
__device__ __forceinline__ cplx<T> logcosh(cplx<T> z) {
    const cplx<T> w = z.re >= T(0) ? z : -z;
    const cplx<T> e = cexp(T(-2) * w);
    const cplx<T> l = clog(mk<T>(T(1) + e.re, e.im));
    return {w.re + l.re - T(0.69314718055994530942), w.im + l.im};
}
template<typename T>
__device__ __forceinline__ cplx<T> ctanh(cplx<T> z) {
    // tanh z = (1 - e^{-2w}) / (1 + e^{-2w}) * sign, w = +-z with Re w >= 0
    const bool neg = z.re < T(0);
    const cplx<T> w = neg ? -z : z;
    const cplx<T> e = cexp(T(-2) * w);
    const cplx<T> r = cdiv(mk<T>(T(1) - e.re, -e.im), mk<T>(T(1) + e.re, e.im));
    return neg ? -r : r;
}
template<typename T>
__device__ __forceinline__ cplx<T> act_f(cplx<T> z, int act, int layer) {
    return act == kPoly ? poly_f(z, layer) : logcosh(z);
}
template<typename T>
__device__ __forceinline__ cplx<T> act_df(cplx<T> z, int act, int layer) {
    return act == kPoly ? poly_df(z, layer) : ctanh(z);
}

// ---------------------------------------------------------------------------------
// spin configurations: bit i = 1 <-> sigma^z_i = +1 (include/basis/Spins.h:104-118)
template<int NW>
struct Conf {
    uint64_t w[NW];
};
template<int NW>
__device__ __forceinline__ int spin_bit(const Conf<NW>& s, unsigned i) {
    return (int)((s.w[i >> 6] >> (i & 63u)) & 1u);
}
template<int NW>
__device__ __forceinline__ void flip(Conf<NW>& s, unsigned i) {
    s.w[i >> 6] ^= (uint64_t)1 << (i & 63u);
}

// ---------------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw: "Parallel random numbers: as easy as
// 1, 2, 3", SC'11). Counter-based: every (key, counter) gives 4 independent words.
struct u32x4 {
    uint32_t x, y, z, w;
};
__host__ __device__ __forceinline__ u32x4 philox4x32_10(uint32_t k0, uint32_t k1, u32x4 c) {
#pragma unroll
    for(int r = 0; r < 10; r++) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c.x;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c.z;
        c = u32x4{(uint32_t)(p1 >> 32) ^ c.y ^ k0, (uint32_t)p1, (uint32_t)(p0 >> 32) ^ c.w ^ k1, (uint32_t)p0};
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}
__host__ __device__ __forceinline__ uint32_t mulhi32(uint32_t r, uint32_t n) {
    return (uint32_t)(((uint64_t)r * n) >> 32);
}
__host__ __device__ __forceinline__ double u53(uint32_t lo, uint32_t hi) {
    return (double)((((uint64_t)hi << 32) | lo) >> 11) * 0x1.0p-53;
}

// ---------------------------------------------------------------------------------
// FP32 <-> FP64 conversions off the FP64 pipe
// Exact FP32 -> FP64 widening in integer arithmetic (sign, exponent rebias 127 -> 1023,
// mantissa shifted to 52 bits; subnormals renormalised; infinities and NaNs kept).
__device__ __forceinline__ double widen(float f) {
    const uint32_t u = __float_as_uint(f);
    const uint64_t sign = (uint64_t)(u >> 31) << 63;
    const uint32_t e = (u >> 23) & 0xFFu, m = u & 0x7FFFFFu;
    uint64_t bits;
    if(e != 0u && e != 0xFFu) {
        bits = sign | ((uint64_t)(e + 896u) << 52) | ((uint64_t)m << 29);
    } else if(e == 0xFFu) {
        bits = sign | (0x7FFull << 52) | ((uint64_t)m << 29);
    } else if(m == 0u) {
        bits = sign;
    } else {
        const uint32_t p = 31u - __clz(m);  // top set bit: value = 1.f * 2^(p - 149)
        bits = sign | ((uint64_t)(p + 874u) << 52) | ((uint64_t)(m ^ (1u << p)) << (52u - p));
    }
    return __longlong_as_double((long long)bits);
}

// Round-to-nearest-even FP64 -> FP32 in integer arithmetic (subnormal results rounded
// at their own precision, overflow to infinity, NaN kept as NaN): the same value as
// cvt.rn.f32.f64, without the FP64 pipe, which runs at 1/64 of the FP32 rate on GB300.
__device__ __forceinline__ float narrow(double d) {
    const uint64_t b = (uint64_t)__double_as_longlong(d);
    const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
    const uint32_t E = (uint32_t)(b >> 52) & 0x7FFu;
    const uint64_t M = b & 0xFFFFFFFFFFFFFull;
    uint32_t r;
    if(E == 0x7FFu) {
        r = 0x7F800000u | (M ? (0x400000u | (uint32_t)(M >> 29)) : 0u);
    } else {
        const int e = (int)E - 1023;
        if(e > 127) {
            r = 0x7F800000u;
        } else if(e >= -126) {
            const uint32_t m23 = (uint32_t)(M >> 29), rem = (uint32_t)(M & 0x1FFFFFFFu);
            r = ((uint32_t)(e + 127) << 23) | m23;
            r += (rem > 0x10000000u || (rem == 0x10000000u && (m23 & 1u))) ? 1u : 0u;  // carries into the exponent
        } else {
            const int sh = -97 - e;  // bits of the 53-bit significand below the subnormal's last place
            if(sh > 54 || E == 0u) {
                r = 0u;
            } else {
                const uint64_t sig = M | (1ull << 52);
                const uint64_t q = sig >> sh, rm = sig & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
                r = (uint32_t)q + ((rm > half || (rm == half && (q & 1ull))) ? 1u : 0u);
            }
        }
    }
    return __uint_as_float(r | sign);
}

// ---------------------------------------------------------------------------------
// warp reductions (xor butterflies leave the bit-identical sum in every lane)
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for(int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for(int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
template<typename T>
__device__ __forceinline__ cplx<T> warp_sum(cplx<T> v) {
    return {warp_sum(v.re), warp_sum(v.im)};
}

// Teams of TL lanes (32: a whole warp; 16: half a warp) that run one Markov chain each.
// A half-warp team reproduces a whole-warp team's sums bit for bit: team lane l stands
// for the warp lanes l and l + 16 ("virtual lanes", kVirt<TL> = 32 / TL of them), keeps one
// partial per virtual lane in that warp lane's order of terms, and adds the two partials
// (the warp's first butterfly level, xor 16) before its own butterfly (xor 8 ... 1).
template<int TL>
constexpr int kVirt = 32 / TL;

template<int TL>
__device__ __forceinline__ unsigned team_mask() {
    static_assert(TL == 32 || TL == 16, "teams of 32 or 16 lanes");
    return TL == 32 ? 0xffffffffu : (0xffffu << ((threadIdx.x & 31u) & 16u));
}
template<int TL>
__device__ __forceinline__ float team_sum(float v) {
    const unsigned m = team_mask<TL>();
#pragma unroll
    for(int o = TL / 2; o > 0; o >>= 1) v += __shfl_xor_sync(m, v, o);
    return v;
}
template<int TL>
__device__ __forceinline__ double team_sum(double v) {
    const unsigned m = team_mask<TL>();
#pragma unroll
    for(int o = TL / 2; o > 0; o >>= 1) v += __shfl_xor_sync(m, v, o);
    return v;
}
template<int TL, typename T>
__device__ __forceinline__ cplx<T> team_sum(cplx<T> v) {
    return {team_sum<TL>(v.re), team_sum<TL>(v.im)};
}
// sum over the team of per-virtual-lane partials part[0 .. kVirt<TL>)
template<int TL, typename V>
__device__ __forceinline__ V team_total(const V* part) {
    V v = part[0];
    if constexpr(TL == 16) v += part[1];
    return team_sum<TL>(v);
}

// Pauli-sum operator grouped by flip mask. A string's matrix element on |s> is
// coeff * (-i)^{n_y} * (-1)^{popcount(~s & (Z|Y))} and it maps s -> s ^ (X|Y)
// (include/basis/PauliString.hpp:193-208, 242-254). Strings with no flips form
// the diagonal part; the others are grouped by their flip mask so one psi ratio
// serves the whole group.
struct OpDev {
    unsigned nw;
    unsigned n_diag;
    const uint64_t* diag_mask;    // [n_diag][nw]: sites with Z (the sign mask)
    const double* diag_coeff;     // [n_diag][2]
    unsigned n_groups;
    const unsigned* grp_site_begin;  // [n_groups + 1] into grp_sites
    const uint16_t* grp_sites;       // flipped sites of each group
    const unsigned* grp_str_begin;   // [n_groups + 1] into str_*
    const uint64_t* str_mask;        // [n_str][nw]: sites with Z or Y
    const double* str_coeff;         // [n_str][2]: coeff * (-i)^{n_y}
    const float* diag_coeff_f;       // FP32 copies for complex64 kernels
    const float* str_coeff_f;
    // every string as given (Pauli-string basis, first word; sites < 64)
    unsigned n_raw;
    const uint64_t* raw_a;
    const uint64_t* raw_b;
    const double* raw_coeff;         // [n_raw][2]
    const float* raw_coeff_f;
};

template<typename T> __device__ __forceinline__ const T* diag_coeff(const OpDev& op);
template<> __device__ __forceinline__ const float* diag_coeff<float>(const OpDev& op) { return op.diag_coeff_f; }
template<> __device__ __forceinline__ const double* diag_coeff<double>(const OpDev& op) { return op.diag_coeff; }
template<typename T> __device__ __forceinline__ const T* raw_coeff(const OpDev& op);
template<> __device__ __forceinline__ const float* raw_coeff<float>(const OpDev& op) { return op.raw_coeff_f; }
template<> __device__ __forceinline__ const double* raw_coeff<double>(const OpDev& op) { return op.raw_coeff; }
template<typename T> __device__ __forceinline__ const T* str_coeff(const OpDev& op);
template<> __device__ __forceinline__ const float* str_coeff<float>(const OpDev& op) { return op.str_coeff_f; }
template<> __device__ __forceinline__ const double* str_coeff<double>(const OpDev& op) { return op.str_coeff; }

// learned proposal weights as the kernels read them (see made.cuh)
struct MadeDev {
    unsigned N, H;             // N == 0: no learned proposal
    const __nv_bfloat16* W1t;  // N x H
    const float* b1;           // H
    const __nv_bfloat16* W2t;  // H x N
    const float* b2;           // N
    const __nv_bfloat16* W2;   // N x H (the sampler's layout, read through L1)
};

struct McArgs {
    unsigned n_chains;
    unsigned samples_per_chain;
    unsigned num_sweeps;
    unsigned num_therm;
    int do_init;              // draw fresh configurations (and thermalise) first
    int n_up;                 // < 0: unconstrained initial configurations
    int move_kind;            // 0 single flip, 1 exchange over bonds, 2 exchange over random pairs
    const uint32_t* bonds;    // [n_bonds][2]
    unsigned n_bonds;
    uint32_t k0, k1;          // Philox key
    uint64_t* chain_conf;     // [n_chains][kMaxWords], in/out
    uint64_t* chain_counter;  // [n_chains], in/out
    // proposal tape (parity replay): per chain, num_props sites and uniforms
    const uint32_t* tape_site;
    const double* tape_u;
    unsigned tape_len;
    unsigned long long* acc_rej;  // [4]: local accepted, rejected; learned accepted, rejected
    MadeDev made;                 // learned independence proposal (made.N == 0: none)
    unsigned indep_per_sample;    // independence proposals after the local sweeps of each sample
    const int* made_on;           // device flag: 0 while the drop rule holds the proposal off (null: on)
    int made_smem;                // 1: the weights are staged in shared memory; 0: read through L1
};

struct SampleOut {
    uint64_t* conf;           // [rows][kMaxWords]
    cplx<double>* log_psi;    // [rows]
    cplx<double>* eloc;       // [rows] (may be null)
    double* weight;           // [rows] (exact summation only)
    void* O;                  // [rows][ldO] cplx<T> (may be null)
    size_t ldO;
    unsigned* status;
};

// device status word bits (returned to the host as C-ABI status)
enum StatusBits : unsigned {
    kStatusNonFinite = 1u,    // NaN / Inf in log psi, E_loc or S
    kStatusNotPosDef = 2u,    // Cholesky pivot <= 0
    kStatusTimeout = 4u,      // a bounded device-side wait gave up
    kStatusBadInput = 8u,     // an index or size outside the checked bounds
    kStatusSolveStalled = 16u,  // mixed-precision SR solve did not reach its tolerance
};

}  // namespace ann
