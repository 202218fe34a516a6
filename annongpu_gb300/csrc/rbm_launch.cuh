// Launchers of the RBM-family kernels for one arithmetic precision T. Included by
// rbm_f32.cu and rbm_f64.cu, which instantiate them (two translation units so the
// build compiles them in parallel).
#pragma once

#include "ann_internal.hpp"
#include "rbm_kernels.cuh"

namespace ann {

namespace {

template<typename T>
RbmDev<T> rbm_view(const ann_psi_impl& psi) {
    RbmDev<T> p;
    p.N = psi.N;
    p.M = psi.M;
    p.Mpad = psi.Mpad;
    p.Uact = psi.Mpad / 32;
    p.C = psi.C;
    p.Np = psi.Np;
    p.layout = psi.layout;
    p.a_in_log_psi = psi.a_in;
    p.act = psi.act;
    p.Wd = psi.Wd.as<cplx<T>>();
    p.a = psi.a.as<cplx<T>>();
    p.b = psi.b.as<cplx<T>>();
    p.fw = psi.fwd.as<cplx<T>>();
    p.conn = psi.connd.as<uint16_t>();
    p.lp = mk<T>((T)psi.lp.real(), (T)psi.lp.imag());
    p.fw_real = 1;
    for(const zd& f : psi.fw)
        if(f.imag() != 0.0) p.fw_real = 0;
    return p;
}

// largest Wd staged in shared memory; beyond it the kernels read Wd from global
// memory (L1/L2 resident)
constexpr size_t kMaxSmemWd = 200 * 1024;

template<typename T>
size_t wd_bytes(const ann_psi_impl& psi) {
    return (size_t)psi.N * psi.Mpad * sizeof(cplx<T>);
}

template<typename T>
int warps_per_block(size_t) {
    return 8;
}

SampleOut sample_out(Rows& rows, void* O, size_t ldO, bool want_eloc) {
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

void ensure_rows(Rows& rows, size_t n, unsigned NW) {
    rows.n = n;
    rows.conf.ensure(n * kMaxWords * sizeof(uint64_t));
    rows.log_psi.ensure(n * sizeof(cplx<double>));
    rows.eloc.ensure(n * sizeof(cplx<double>));
    rows.weight.ensure(n * sizeof(double));
}

template<typename K>
void set_smem(K kernel, size_t smem) {
    if(smem > 48 * 1024) ANN_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
}

#define ANN_DISPATCH_NW_U(NW_, U_, ...)                                                   \
    do {                                                                                  \
        if((NW_) == 1) {                                                                  \
            constexpr int NWc = 1;                                                        \
            switch(U_) {                                                                  \
                case 1: { constexpr int Uc = 1; __VA_ARGS__; } break;                     \
                case 2: { constexpr int Uc = 2; __VA_ARGS__; } break;                     \
                case 4: { constexpr int Uc = 4; __VA_ARGS__; } break;                     \
                case 8: { constexpr int Uc = 8; __VA_ARGS__; } break;                     \
                default: throw Error(ANN_ERR_INVALID, "unsupported hidden width");        \
            }                                                                             \
        } else {                                                                          \
            constexpr int NWc = 2;                                                        \
            switch(U_) {                                                                  \
                case 1: { constexpr int Uc = 1; __VA_ARGS__; } break;                     \
                case 2: { constexpr int Uc = 2; __VA_ARGS__; } break;                     \
                case 4: { constexpr int Uc = 4; __VA_ARGS__; } break;                     \
                case 8: { constexpr int Uc = 8; __VA_ARGS__; } break;                     \
                default: throw Error(ANN_ERR_INVALID, "unsupported hidden width");        \
            }                                                                             \
        }                                                                                 \
    } while(0)

}  // namespace

template<typename T>
void rbm_prepare_T(ann_psi_impl& psi, cudaStream_t st) {
    RbmDev<T> p = rbm_view<T>(psi);
    const unsigned threads = 128;
    const unsigned n = psi.Mpad > psi.N ? psi.Mpad : psi.N;
    rbm_prepare_kernel<T><<<(n + threads - 1) / threads, threads, 0, st>>>(
        p, psi.params.as<cplx<double>>(), psi.Wd.as<cplx<T>>(), psi.a.as<cplx<T>>(), psi.b.as<cplx<T>>());
    check_launch("rbm_prepare_kernel");
}

template<typename T>
void rbm_mc_T(ann_psi_impl& psi, const ann_op_impl* op, ann_ens_impl& ens, const SampleTargets& t,
              cudaStream_t st) {
    RbmDev<T> p = rbm_view<T>(psi);
    const unsigned spc = ens.num_samples / ens.n_chains;
    ensure_rows(*t.rows, (size_t)spc * ens.n_chains, psi.NW);
    McArgs a;
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
    a.made = MadeDev{};
    a.indep_per_sample = 0;
    a.made_on = nullptr;
    a.made_smem = 0;
    // the learned moves are launched whenever a proposal is set; the device flag (the drop
    // rule) decides in the kernel whether they run
    const bool learned = ens.made && ens.indep_per_sample > 0 && !a.tape_site;
    if(learned) {
        if(ens.made->N != psi.N) throw Error(ANN_ERR_INVALID, "learned proposal size differs from psi.N");
        if(ens.made->H > 256) throw Error(ANN_ERR_INVALID, "learned proposals in the sampler need H <= 256");
        if(ens.move != 0) throw Error(ANN_ERR_UNSUPPORTED, "learned proposals combine with single-flip moves");
        a.made = made_view(*ens.made);
        a.indep_per_sample = ens.indep_per_sample;
        a.made_on = ens.made_on.as<int>();
        // the proposal's weights in shared memory when its moves are a large part of the
        // work (each costs about one sweep); read through L1 when the local sweeps dominate,
        // so shared memory is left to occupancy
        a.made_smem = 4 * ens.indep_per_sample >= ens.num_sweeps ? 1 : 0;
    }
    if(a.tape_site) {
        // replay starts from the recorded initial configurations every call
        ANN_CUDA(cudaMemcpyAsync(ens.chain_conf.p, ens.tape_init.p, (size_t)ens.n_chains * kMaxWords * 8,
                                 cudaMemcpyDeviceToDevice, st));
    }
    ANN_CUDA(cudaMemsetAsync(ens.acc_rej.p, 0, 4 * sizeof(unsigned long long), st));
    SampleOut out = sample_out(*t.rows, t.O, t.ldO, t.want_eloc && op);
    OpDev ov{};
    if(op) ov = op->view();
    const size_t wb = wd_bytes<T>(psi);
    // warps per CTA: the autotuned choice for this shape, else the default
    int wpb = tuning_get(key_mc_wpb(psi, ens), warps_per_block<T>(0));
    if(wpb < 1 || wpb > 8) wpb = warps_per_block<T>(0);
    // lanes per chain: half-warp teams (two chains per warp, 2 U hidden units per lane)
    // for complex64 chains up to 128 hidden units, when the tuning table chose them; the
    // learned moves then draw their uniforms from 16 lanes (N <= 64)
    const bool team_ok = sizeof(T) == 4 && psi.Mpad <= 128 && (!learned || psi.N <= 64);
    const int team = team_ok && tuning_get(key_mc_team(psi, ens), 32) == 16 ? 16 : 32;
    const unsigned chains_per_cta = (unsigned)wpb * (32u / team);
    const size_t made_bytes = learned ? (a.made_smem ? made_smem_bytes(ens.made->N, ens.made->H) : 0) +
                                            (size_t)chains_per_cta * ens.made->H * 4
                                      : 0;
    // W staged in shared memory when it fits, unless the tuning table prefers reading it
    // through L1 (fewer bytes of shared memory per CTA, more CTAs per SM)
    const int w_smem = (wb + made_bytes <= kMaxSmemWd && tuning_get(key_mc_wsmem(psi, ens), 1)) ? 1 : 0;
    const size_t smem = (w_smem ? ((wb + 15) & ~(size_t)15) : 0) + made_bytes;
    if(smem > 220 * 1024) throw Error(ANN_ERR_INVALID, "learned proposal too large for shared memory");
    const unsigned grid = (ens.n_chains + chains_per_cta - 1) / chains_per_cta;
    if(team == 16) {
        if constexpr(sizeof(T) == 4) {
            // U of the half-warp kernel = Mpad / 16 (2, 4 or 8)
            auto go = [&](auto k) {
                set_smem(k, smem);
                k<<<grid, wpb * 32, smem, st>>>(p, ov, op ? 1 : 0, a, out, w_smem);
            };
            const int u16 = (int)psi.Mpad / 16;
            if(psi.NW == 1) {
                if(u16 == 2) go(rbm_mc_kernel<T, 1, 2, 16>);
                else if(u16 == 4) go(rbm_mc_kernel<T, 1, 4, 16>);
                else go(rbm_mc_kernel<T, 1, 8, 16>);
            } else {
                if(u16 == 2) go(rbm_mc_kernel<T, 2, 2, 16>);
                else if(u16 == 4) go(rbm_mc_kernel<T, 2, 4, 16>);
                else go(rbm_mc_kernel<T, 2, 8, 16>);
            }
        }
    } else {
        ANN_DISPATCH_NW_U(psi.NW, psi.U, {
            auto k = rbm_mc_kernel<T, NWc, Uc, 32>;
            set_smem(k, smem);
            k<<<grid, wpb * 32, smem, st>>>(p, ov, op ? 1 : 0, a, out, w_smem);
        });
    }
    check_launch("rbm_mc_kernel");
    if(learned) {
        made_drop_rule_kernel<<<1, 1, 0, st>>>(ens.acc_rej.as<unsigned long long>(), ens.made_min_acceptance,
                                               ens.made_on.as<int>());
        check_launch("made_drop_rule_kernel");
    }
    ens.chains_valid = true;
}

template<typename T>
void rbm_exact_T(ann_psi_impl& psi, const ann_op_impl* op, ann_ens_impl& ens, const SampleTargets& t,
                 cudaStream_t st) {
    RbmDev<T> p = rbm_view<T>(psi);
    const uint64_t n_conf = 1ull << ens.N;
    ensure_rows(*t.rows, n_conf, psi.NW);
    SampleOut out = sample_out(*t.rows, t.O, t.ldO, t.want_eloc && op);
    OpDev ov{};
    if(op) ov = op->view();
    const size_t wb = wd_bytes<T>(psi);
    const int w_smem = wb <= kMaxSmemWd ? 1 : 0;
    const size_t smem = w_smem ? wb : 0;
    const int wpb = warps_per_block<T>(smem);
    uint64_t blocks = (n_conf + wpb - 1) / wpb;
    const uint64_t cap = 152ull * 16;
    if(blocks > cap) blocks = cap;
    ANN_DISPATCH_NW_U(psi.NW, psi.U, {
        auto k = rbm_exact_kernel<T, NWc, Uc>;
        set_smem(k, smem);
        k<<<(unsigned)blocks, wpb * 32, smem, st>>>(p, ov, op ? 1 : 0, n_conf, out, w_smem);
    });
    check_launch("rbm_exact_kernel");
}

template<typename T>
void rbm_confs_T(ann_psi_impl& psi, const ann_op_impl* op, const uint64_t* confs, size_t n, Rows& rows, void* O,
                 size_t ldO, cudaStream_t st) {
    RbmDev<T> p = rbm_view<T>(psi);
    ensure_rows(rows, n, psi.NW);
    SampleOut out = sample_out(rows, O, ldO, op != nullptr);
    OpDev ov{};
    if(op) ov = op->view();
    const int wpb = 8;
    const unsigned grid = (unsigned)((n + wpb - 1) / wpb);
    ANN_DISPATCH_NW_U(psi.NW, psi.U, {
        rbm_confs_kernel<T, NWc, Uc><<<grid, wpb * 32, 0, st>>>(p, ov, op ? 1 : 0, confs, n, out);
    });
    check_launch("rbm_confs_kernel");
}

}  // namespace ann
