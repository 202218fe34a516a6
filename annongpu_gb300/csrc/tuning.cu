// Autotuner and tuning table.
//
// The launchers read launch and tile choices from a per-process table keyed by
// device, knob and problem shape ("dev0/rbm_mc.wpb/N64.M128.U4.NW1.made1" ...); an
// absent key means the built-in default. ann_autotune fills the table for one
// workload by timing every candidate of each knob on it with CUDA events (median of
// repeats) and keeping the fastest:
//   rbm_mc.wpb      warps (chains) per CTA of the Metropolis sampler: 2, 4, 8
//   rbm_mc.wsmem    sampler weights W staged in shared memory (1) or read through L1 (0)
//   rbm_mc.team     lanes per chain of the complex64 sampler: 32 (one chain per warp) or
//                   16 (two chains per warp, twice the hidden units per lane; Mpad <= 128)
//   stats.slab      rows per FP32 slab of the <O> / F reductions: 128, 256, 512
//   chol.update     trailing update of the FP32 Cholesky: 128 x 128 tcgen05 tiles
//                   (split TF32) or 64 x 64 FP32 SIMT tiles
//   chol.reserve    SMs the persistent tcgen05 update leaves free for the next panel: 0, 16, 32, 48, 64
//   chol.pair       tcgen05 trailing updates of rank 64 per panel (0) or rank 128 per panel pair (1)
// The sampler is timed on a copy of the ensemble, so the caller's chains do not move.
// The reference has no tuning layer (its launch shape is fixed: one CTA per chain,
// blockDim = hidden width, include/ensembles/MonteCarlo.hpp:223-228).
#include <algorithm>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "ann_internal.hpp"

namespace ann {

namespace {
std::mutex g_tune_mutex;
std::map<std::string, int> g_tune;

std::string dev_prefix() {
    int dev = 0;
    ANN_CUDA(cudaGetDevice(&dev));
    return "dev" + std::to_string(dev) + "/";
}

// median duration (ms) of `reps` runs of f on stream st, after one untimed run
template<typename Fn>
double time_ms(Fn&& f, int reps, cudaStream_t st) {
    cudaEvent_t e0, e1;
    ANN_CUDA(cudaEventCreate(&e0));
    ANN_CUDA(cudaEventCreate(&e1));
    std::vector<float> t;
    try {
        f();
        for(int r = 0; r < reps; r++) {
            ANN_CUDA(cudaEventRecord(e0, st));
            f();
            ANN_CUDA(cudaEventRecord(e1, st));
            ANN_CUDA(cudaEventSynchronize(e1));
            float ms = 0.f;
            ANN_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            t.push_back(ms);
        }
    } catch(...) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::sort(t.begin(), t.end());
    return t[t.size() / 2];
}
}  // namespace

int tuning_get(const std::string& key, int dflt) {
    const std::string k = dev_prefix() + key;
    std::lock_guard<std::mutex> lk(g_tune_mutex);
    auto it = g_tune.find(k);
    return it == g_tune.end() ? dflt : it->second;
}

void tuning_set(const std::string& key, int value) {
    const std::string k = dev_prefix() + key;
    std::lock_guard<std::mutex> lk(g_tune_mutex);
    g_tune[k] = value;
}

std::string key_mc_wpb(const ann_psi_impl& psi, const ann_ens_impl& ens) {
    std::ostringstream o;
    o << "rbm_mc.wpb/N" << psi.N << ".M" << psi.Mpad << ".U" << psi.U << ".P" << psi.precision << ".made"
      << (ens.made && !ens.made_dropped && ens.indep_per_sample ? 1 : 0);
    return o.str();
}

std::string key_mc_wsmem(const ann_psi_impl& psi, const ann_ens_impl& ens) {
    std::string k = key_mc_wpb(psi, ens);
    return "rbm_mc.wsmem" + k.substr(k.find('/'));
}

std::string key_mc_team(const ann_psi_impl& psi, const ann_ens_impl& ens) {
    std::string k = key_mc_wpb(psi, ens);
    return "rbm_mc.team" + k.substr(k.find('/'));
}

std::string key_slab(size_t rows, unsigned Np) {
    // rows rounded to a power of two: the choice depends on the shape class, not the count
    size_t r = 1;
    while(r < rows) r <<= 1;
    std::ostringstream o;
    o << "stats.slab/R" << r << ".Np" << ((Np + 1023) / 1024) * 1024;
    return o.str();
}

std::string key_chol_update(unsigned n) {
    std::ostringstream o;
    o << "chol.update/n" << ((n + 1023) / 1024) * 1024;
    return o.str();
}

std::string key_chol_reserve(unsigned n) {
    std::ostringstream o;
    o << "chol.reserve/n" << ((n + 1023) / 1024) * 1024;
    return o.str();
}

std::string key_chol_pair(unsigned n) {
    std::ostringstream o;
    o << "chol.pair/n" << ((n + 1023) / 1024) * 1024;
    return o.str();
}

}  // namespace ann

using namespace ann;

namespace {
template<typename F>
int tguard(F&& f) {
    try {
        f();
        return ANN_OK;
    } catch(const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch(const std::exception& e) {
        set_last_error(e.what());
        return ANN_ERR_CUDA;
    }
}
}  // namespace

extern "C" {

int ann_tuning_set(const char* key, int value) {
    return tguard([&] {
        if(!key || !*key) throw Error(ANN_ERR_INVALID, "empty tuning key");
        std::lock_guard<std::mutex> lk(g_tune_mutex);
        g_tune[key] = value;
    });
}

int ann_tuning_get(const char* key, int* value, int* found) {
    return tguard([&] {
        if(!key || !value || !found) throw Error(ANN_ERR_INVALID, "null argument");
        std::lock_guard<std::mutex> lk(g_tune_mutex);
        auto it = g_tune.find(key);
        *found = it != g_tune.end();
        if(*found) *value = it->second;
    });
}

int ann_tuning_dump(char* buf, size_t cap, size_t* len) {
    return tguard([&] {
        if(!len) throw Error(ANN_ERR_INVALID, "null argument");
        std::string s;
        {
            std::lock_guard<std::mutex> lk(g_tune_mutex);
            for(const auto& kv : g_tune) s += kv.first + " " + std::to_string(kv.second) + "\n";
        }
        *len = s.size();
        if(buf && cap) {
            const size_t n = std::min(cap - 1, s.size());
            std::copy(s.begin(), s.begin() + n, buf);
            buf[n] = 0;
        }
    });
}

int ann_tuning_clear(void) {
    return tguard([&] {
        std::lock_guard<std::mutex> lk(g_tune_mutex);
        g_tune.clear();
    });
}

int ann_autotune(ann_tdvp* t, ann_op* op, ann_psi* psi, ann_ens* ens, double diag_shift, void* stream,
                 double* report, unsigned cap, unsigned* n_report) {
    return tguard([&] {
        if(!t || !op || !psi || !ens) throw Error(ANN_ERR_INVALID, "null argument");
        if(t->Np != psi->Np) throw Error(ANN_ERR_INVALID, "TDVP num_params differs from psi.num_params");
        cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
        std::vector<double> rep;
        auto record = [&](int knob, int cand, double ms) {
            rep.push_back(knob);
            rep.push_back(cand);
            rep.push_back(ms);
        };
        ann_ens* e2 = ens_clone(*ens);
        try {
            // sampler launch shape (RBM family, Monte Carlo)
            if(psi->kind == 0 && e2->kind == 1) {
                // lanes per chain first (at the default CTA size), when the shape allows half warps
                if(psi->precision == 0 && psi->Mpad <= 128) {
                    const std::string kt = key_mc_team(*psi, *e2);
                    double best_t_ms = 1e300;
                    int best_t = 32;
                    for(int tl : {32, 16}) {
                        tuning_set(kt, tl);
                        const SampleTargets tg = tdvp_prepare(*t, *psi, *e2);
                        const double ms = time_ms([&] { run_ensemble(*psi, op, *e2, tg, st); }, 3, st);
                        record(6, tl, ms);
                        if(ms < best_t_ms) { best_t_ms = ms; best_t = tl; }
                    }
                    tuning_set(kt, best_t);
                }
                const std::string key = key_mc_wpb(*psi, *e2);
                double best = 1e300;
                int best_w = 8;
                for(int w : {2, 4, 8}) {
                    tuning_set(key, w);
                    const SampleTargets tg = tdvp_prepare(*t, *psi, *e2);
                    const double ms = time_ms([&] { run_ensemble(*psi, op, *e2, tg, st); }, 3, st);
                    record(0, w, ms);
                    if(ms < best) { best = ms; best_w = w; }
                }
                tuning_set(key, best_w);
                // W in shared memory or read through L1, at the chosen CTA size
                const std::string kw = key_mc_wsmem(*psi, *e2);
                double best_ws = 1e300;
                int best_s = 1;
                for(int ws : {1, 0}) {
                    tuning_set(kw, ws);
                    const SampleTargets tg = tdvp_prepare(*t, *psi, *e2);
                    const double ms = time_ms([&] { run_ensemble(*psi, op, *e2, tg, st); }, 3, st);
                    record(3, ws, ms);
                    if(ms < best_ws) { best_ws = ms; best_s = ws; }
                }
                tuning_set(kw, best_s);
            }
            // one evaluation on the copy: O rows and S for the remaining knobs
            {
                const SampleTargets tg = tdvp_prepare(*t, *psi, *e2);
                run_ensemble(*psi, op, *e2, tg, st);
                tdvp_post(*t, *psi, *e2, true, st);
                ANN_CUDA(cudaStreamSynchronize(st));
            }
            // slab rows of the FP32 reductions
            if(t->O_precision == 0) {
                const std::string key = key_slab(t->n_rows, t->Np);
                const double* w = t->wts_exact ? t->wts.as<double>() : nullptr;
                double best = 1e300;
                int best_s = 512;
                for(int sl : {128, 256, 512}) {
                    tuning_set(key, sl);
                    const double ms = time_ms(
                        [&] {
                            col_stats(t->O.p, 0, t->n_rows, t->ldO, t->Np, w, t->w0,
                                      e2->rows.eloc.as<cplx<double>>(), t->Obar.as<cplx<double>>(),
                                      t->F.as<cplx<double>>(), t->stats.as<Stats>(), nullptr, t->partial, st);
                        },
                        5, st);
                    record(1, sl, ms);
                    if(ms < best) { best = ms; best_s = sl; }
                }
                tuning_set(key, best_s);
            }
            // trailing update of the FP32 Cholesky (mixed / FP32 solvers)
            if(t->solver != ANN_SOLVER_FP64 && !t->chol_tc_set) {
                const std::string key = key_chol_update(t->Np);
                double best = 1e300;
                int best_m = 1;
                for(int m : {1, 0}) {
                    tuning_set(key, m);
                    const double ms = time_ms([&] { sr_solve_any(*t, diag_shift, status_word(), st); }, 2, st);
                    record(2, m, ms);
                    if(ms < best) { best = ms; best_m = m; }
                }
                tuning_set(key, best_m);
                // one rank-64 update per panel or one rank-128 update per panel pair (the
                // pair form needs the reduce-add epilogue: n even)
                if(best_m == 1 && t->Np % 2 == 0) {
                    const std::string kp = key_chol_pair(t->Np);
                    double best_p_ms = 1e300;
                    int best_p = 1;
                    for(int pr : {1, 0}) {
                        tuning_set(kp, pr);
                        const double ms = time_ms([&] { sr_solve_any(*t, diag_shift, status_word(), st); }, 2, st);
                        record(5, pr, ms);
                        if(ms < best_p_ms) { best_p_ms = ms; best_p = pr; }
                    }
                    tuning_set(kp, best_p);
                }
                // SMs left to the panel beside the persistent tensor-core update
                if(best_m == 1) {
                    const std::string kr = key_chol_reserve(t->Np);
                    double best_r_ms = 1e300;
                    int best_r = 32;
                    for(int r : {0, 16, 32, 48, 64}) {
                        tuning_set(kr, r);
                        const double ms = time_ms([&] { sr_solve_any(*t, diag_shift, status_word(), st); }, 2, st);
                        record(4, r, ms);
                        if(ms < best_r_ms) { best_r_ms = ms; best_r = r; }
                    }
                    tuning_set(kr, best_r);
                }
            }
        } catch(...) {
            ann_ens_destroy(e2);
            throw;
        }
        ann_ens_destroy(e2);
        const unsigned n = (unsigned)(rep.size() / 3);
        if(n_report) *n_report = n;
        if(report)
            for(unsigned k = 0; k < std::min(n, cap); k++)
                for(int q = 0; q < 3; q++) report[3 * k + q] = rep[3 * k + q];
    });
}

}  // extern "C"
