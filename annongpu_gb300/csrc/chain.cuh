// Per-warp Metropolis chain plumbing shared by the full-forward samplers (PsiCNN and
// PsiDeep of any depth): initial configurations and proposal draws under the
// counter-based random-number contract of the RBM sampler (Philox4x32-10, key = seed,
// counter = (step, chain, stream)), or replayed from a proposal tape. The reference
// draws one site per update with curand (include/ensembles/policies/Update_Policy.hpp:20-33).
#pragma once

#include "ann_common.cuh"

namespace ann {

// The chain's starting configuration and counter: taken from the tape's initial
// configurations, drawn fresh (uniform, or exactly n_up up spins), or continued.
__device__ __forceinline__ void chain_start(const McArgs& a, unsigned chain, unsigned N, Conf<2>& s, uint64_t& t) {
    if(a.tape_site) {
        for(int w = 0; w < 2; w++) s.w[w] = a.chain_conf[(size_t)chain * kMaxWords + w];
        t = 0;
    } else if(a.do_init) {
        t = a.chain_counter[chain];
        if(a.n_up < 0) {
            const u32x4 r = philox4x32_10(a.k0, a.k1, u32x4{(uint32_t)t, (uint32_t)(t >> 32), chain, 1u});
            s.w[0] = (uint64_t)r.x | ((uint64_t)r.y << 32);
            s.w[1] = (uint64_t)r.z | ((uint64_t)r.w << 32);
            for(int w = 0; w < 2; w++) {
                const unsigned lo = 64u * w;
                if(N <= lo) s.w[w] = 0;
                else if(N - lo < 64u) s.w[w] &= ((uint64_t)1 << (N - lo)) - 1u;
            }
        } else {
            s.w[0] = s.w[1] = 0;
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
        for(int w = 0; w < 2; w++) s.w[w] = a.chain_conf[(size_t)chain * kMaxWords + w];
        t = a.chain_counter[chain];
    }
}

// One proposal: sites i (and j for exchange moves; 0xFFFFFFFF otherwise) and the
// uniform it is accepted against (u in FP64, uf in FP32 with 24 bits). Lanes draw
// 32 consecutive counters at once and broadcast one per step.
struct ChainDraw {
    uint64_t t, t0;
    unsigned tape_pos = 0;
    u32x4 rr = {0, 0, 0, 0};

    // the four words of proposal counter (t, chain, 0); t advances
    __device__ __forceinline__ void words(const McArgs& a, unsigned chain, int lane, uint32_t& r0, uint32_t& r1,
                                          uint32_t& r2, uint32_t& r3) {
        const unsigned k = (unsigned)(t - t0) & 31u;
        if(k == 0) {
            const uint64_t tl = t + lane;
            rr = philox4x32_10(a.k0, a.k1, u32x4{(uint32_t)tl, (uint32_t)(tl >> 32), chain, 0u});
        }
        r0 = __shfl_sync(0xffffffffu, rr.x, k);
        r1 = __shfl_sync(0xffffffffu, rr.y, k);
        r2 = __shfl_sync(0xffffffffu, rr.z, k);
        r3 = __shfl_sync(0xffffffffu, rr.w, k);
        t++;
    }

    __device__ __forceinline__ void next(const McArgs& a, unsigned chain, unsigned N, int lane, unsigned& i,
                                         unsigned& j, double& u, float& uf) {
        j = 0xFFFFFFFFu;
        if(a.tape_site) {
            i = a.tape_site[(size_t)chain * a.tape_len + tape_pos];
            u = a.tape_u[(size_t)chain * a.tape_len + tape_pos];
            uf = (float)u;
            tape_pos++;
            return;
        }
        uint32_t r0, r1, r2, r3;
        words(a, chain, lane, r0, r1, r2, r3);
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
        uf = __uint2float_rz(r3 >> 8) * 0x1.0p-24f;
    }
};

}  // namespace ann
