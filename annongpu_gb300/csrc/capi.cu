// C ABI (include/annongpu.h): handle management, argument checking, and the host
// logic of the reference's network functions on top of the device kernels.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_profiler_api.h>

#include "ann_internal.hpp"


namespace ann {

namespace {
thread_local std::string g_last_error;
// optional CUDA-event timing of the SR-step phases (sample, statistics, S, solve, update)
constexpr int kPhases = 5;
bool g_timing = false;
cudaEvent_t g_ev[kPhases + 1] = {};
bool g_ev_used[kPhases + 1] = {};
std::atomic<unsigned long long> g_launches{0};
std::mutex g_status_mutex;
std::map<int, unsigned*> g_status;  // device -> status word
}  // namespace

void cuda_check(cudaError_t e, const char* what) {
    if(e != cudaSuccess) throw Error(ANN_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
void count_launch(unsigned n) { g_launches += n; }
void set_last_error(const char* msg) { g_last_error = msg; }
void check_launch(const char* what) {
    count_launch();
    cudaError_t e = cudaGetLastError();
    if(e != cudaSuccess) throw Error(ANN_ERR_CUDA, std::string("launch of ") + what + ": " + cudaGetErrorString(e));
}

DevBuf::~DevBuf() { free_(); }
void DevBuf::free_() {
    if(p) cudaFree(p);
    p = nullptr;
    bytes = 0;
}
void DevBuf::ensure(size_t n) {
    if(n <= bytes && p) return;
    free_();
    if(n == 0) n = 16;
    ANN_CUDA(cudaMalloc(&p, n));
    bytes = n;
}
void upload(DevBuf& b, const void* src, size_t bytes) {
    b.ensure(bytes);
    if(bytes) ANN_CUDA(cudaMemcpy(b.p, src, bytes, cudaMemcpyHostToDevice));
}

namespace {
// ring buffer of sample configurations: row (pos + i) % cap <- row i of this pass
__global__ void hist_append_kernel(const uint64_t* __restrict__ conf, size_t n, uint64_t* __restrict__ hist,
                                   size_t cap, const unsigned long long* __restrict__ pos) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= n) return;
    const size_t r = (size_t)((*pos + i) % cap);
    for(int w = 0; w < kMaxWords; w++) hist[r * kMaxWords + w] = conf[i * kMaxWords + w];
}
__global__ void hist_advance_kernel(unsigned long long* pos, size_t n) { *pos += n; }
}  // namespace

unsigned* status_word() {
    int dev = 0;
    ANN_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_status_mutex);
    auto it = g_status.find(dev);
    if(it != g_status.end()) return it->second;
    unsigned* p = nullptr;
    ANN_CUDA(cudaMalloc(&p, sizeof(unsigned)));
    ANN_CUDA(cudaMemset(p, 0, sizeof(unsigned)));
    ANN_CUDA(cudaDeviceSynchronize());
    g_status[dev] = p;
    return p;
}

// copy of an ensemble: sizes, moves, chain state (configurations and Philox
// counters) and the learned proposal; not the sample rows, tape or history
::ann_ens* ens_clone(const ann_ens_impl& src) {
    auto* e = new ann_ens();
    try {
        e->kind = src.kind;
        e->basis = src.basis;
        e->N = src.N;
        e->num_samples = src.num_samples;
        e->num_sweeps = src.num_sweeps;
        e->num_therm = src.num_therm;
        e->n_chains = src.n_chains;
        e->move = src.move;
        e->n_up = src.n_up;
        e->persistent = src.persistent;
        e->seed = src.seed;
        e->bonds = src.bonds;
        e->chains_valid = src.chains_valid;
        e->made = src.made;
        e->indep_per_sample = src.indep_per_sample;
        e->made_min_acceptance = src.made_min_acceptance;
        e->made_dropped = src.made_dropped;
        auto clone = [](DevBuf& dst, const DevBuf& s) {
            if(!s.p) return;
            dst.ensure(s.bytes);
            ANN_CUDA(cudaMemcpy(dst.p, s.p, s.bytes, cudaMemcpyDeviceToDevice));
        };
        clone(e->bonds_d, src.bonds_d);
        clone(e->chain_conf, src.chain_conf);
        clone(e->chain_counter, src.chain_counter);
        clone(e->acc_rej, src.acc_rej);
        clone(e->made_on, src.made_on);
    } catch(...) {
        delete e;
        throw;
    }
    return e;
}

OpDev ann_op_impl::view() const {
    OpDev v;
    v.nw = nw;
    v.n_diag = n_diag;
    v.diag_mask = diag_mask.as<uint64_t>();
    v.diag_coeff = diag_coeff.as<double>();
    v.n_groups = n_groups;
    v.grp_site_begin = grp_site_begin.as<unsigned>();
    v.grp_sites = grp_sites.as<uint16_t>();
    v.grp_str_begin = grp_str_begin.as<unsigned>();
    v.str_mask = str_mask.as<uint64_t>();
    v.str_coeff = str_coeff.as<double>();
    v.diag_coeff_f = diag_coeff_f.as<float>();
    v.str_coeff_f = str_coeff_f.as<float>();
    v.n_raw = n_strings;
    v.raw_a = raw_a.as<uint64_t>();
    v.raw_b = raw_b.as<uint64_t>();
    v.raw_coeff = raw_c.as<double>();
    v.raw_coeff_f = raw_cf.as<float>();
    return v;
}

void psi_prepare(ann_psi_impl& psi, cudaStream_t st) {
    if(psi.kind == 0) {
        if(psi.precision == 0) rbm_prepare_T<float>(psi, st);
        else rbm_prepare_T<double>(psi, st);
        if(psi.deep.tab_len) deep_prepare(psi, st);  // also serves Pauli-string ensembles
    } else if(psi.kind == 1) {
        cnn_prepare(psi, st);
    } else {
        deep_prepare(psi, st);
    }
}

void run_ensemble(ann_psi_impl& psi, const ann_op_impl* op, ann_ens_impl& ens, const SampleTargets& t,
                  cudaStream_t st) {
    if(op && !ens.basis && op->max_site > psi.N)
        throw Error(ANN_ERR_INVALID, "operator acts on sites beyond the wavefunction");
    if(ens.kind == 0 && !ens.basis && ens.N != psi.N)
        throw Error(ANN_ERR_INVALID, "exact summation size differs from psi.N");
    if(ens.kind == 1 && ens.move == ANN_MOVE_EXCHANGE_BONDS)
        for(const uint32_t site : ens.bonds)
            if(site >= psi.N) throw Error(ANN_ERR_INVALID, "a bond names a site beyond the wavefunction");
    if((psi.kind != 0 || ens.basis) && ens.kind == 1 && ens.made && ens.indep_per_sample)
        throw Error(ANN_ERR_UNSUPPORTED, "the learned proposal is built for the RBM family over spins");
    if(ens.basis == ANN_BASIS_PAULIS) {
        if(psi.deep.K) throw Error(ANN_ERR_UNSUPPORTED, "classical networks are built over spins");
        const unsigned sites = ens.kind == 0 ? ens.N : psi.N / 3u;
        if(psi.N != 3u * sites)
            throw Error(ANN_ERR_INVALID, "a wavefunction over Pauli strings needs 3 input units per site");
        if(op && op->max_site > sites) throw Error(ANN_ERR_INVALID, "operator acts on sites beyond the strings");
        if(ens.kind == 1 && ens.tape_len) throw Error(ANN_ERR_UNSUPPORTED, "no proposal tape over Pauli strings");
        deep_ensure(psi);
        deep_run(psi, op, ens, t, st);
    } else if(psi.kind == 0) {
        if(ens.kind == 0) {
            if(psi.precision == 0) rbm_exact_T<float>(psi, op, ens, t, st);
            else rbm_exact_T<double>(psi, op, ens, t, st);
        } else {
            if(psi.precision == 0) rbm_mc_T<float>(psi, op, ens, t, st);
            else rbm_mc_T<double>(psi, op, ens, t, st);
        }
    } else if(psi.kind == 1) {
        cnn_run(psi, op, ens, t, st);
    } else {
        deep_run(psi, op, ens, t, st);
    }
    if(ens.hist_cap) hist_append(ens, t.rows->conf.as<uint64_t>(), t.rows->n, st);
}

// appends the configurations of a pass (n rows of conf) to the ring buffer; the write
// position is a device counter, so replays of a captured step keep advancing it
void hist_append(ann_ens_impl& ens, const uint64_t* conf, size_t n, cudaStream_t st) {
    hist_append_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
        conf, n, ens.hist.as<uint64_t>(), ens.hist_cap, ens.hist_posd.as<unsigned long long>());
    check_launch("hist_append_kernel");
    hist_advance_kernel<<<1, 1, 0, st>>>(ens.hist_posd.as<unsigned long long>(), n);
    check_launch("hist_advance_kernel");
    ens.hist_len = std::min(ens.hist_cap, ens.hist_len + n);  // rows valid once written (host bound)
}

void run_confs(ann_psi_impl& psi, const ann_op_impl* op, const uint64_t* confs, size_t n, Rows& rows, void* O,
               size_t ldO, cudaStream_t st, int basis) {
    if(basis == ANN_BASIS_PAULIS) {
        if(psi.deep.K) throw Error(ANN_ERR_UNSUPPORTED, "classical networks are built over spins");
        if(psi.N % 3u) throw Error(ANN_ERR_INVALID, "a wavefunction over Pauli strings needs 3 input units per site");
        if(op && op->max_site > psi.N / 3u) throw Error(ANN_ERR_INVALID, "operator acts on sites beyond the strings");
        deep_ensure(psi);
        deep_confs(psi, op, confs, n, rows, O, ldO, st, basis);
        return;
    }
    if(op && op->max_site > psi.N) throw Error(ANN_ERR_INVALID, "operator acts on sites beyond the wavefunction");
    if(psi.kind == 0) {
        if(psi.precision == 0) rbm_confs_T<float>(psi, op, confs, n, rows, O, ldO, st);
        else rbm_confs_T<double>(psi, op, confs, n, rows, O, ldO, st);
    } else if(psi.kind == 1) {
        cnn_confs(psi, op, confs, n, rows, O, ldO, st);
    } else {
        deep_confs(psi, op, confs, n, rows, O, ldO, st, basis);
    }
}

// sub-phases of the mixed solve: factorisation start / end (events 0, 1)
namespace {
cudaEvent_t g_sev[2] = {};
bool g_sev_used[2] = {};
}  // namespace

void solve_mark(int i, cudaStream_t st) {
    if(!g_timing) return;
    cudaStreamCaptureStatus cs;
    ANN_CUDA(cudaStreamIsCapturing(st, &cs));
    if(cs != cudaStreamCaptureStatusNone) return;
    if(!g_sev[i]) ANN_CUDA(cudaEventCreate(&g_sev[i]));
    ANN_CUDA(cudaEventRecord(g_sev[i], st));
    g_sev_used[i] = true;
}

// event timeline of the FP32 Cholesky (tagged events on its main and look-ahead streams)
namespace {
std::vector<std::pair<int, cudaEvent_t>> g_fev;
size_t g_fev_used = 0;
int g_ftrace = 0;  // 0 off, 1 panel-pair marks, 2 also the marks between the panel kernels
}  // namespace

void factor_trace_reset() { g_fev_used = 0; }

void factor_mark(int tag, cudaStream_t st, int level) {
    if(g_ftrace < level) return;
    cudaStreamCaptureStatus cs;
    ANN_CUDA(cudaStreamIsCapturing(st, &cs));
    if(cs != cudaStreamCaptureStatusNone) return;
    if(g_fev_used == g_fev.size()) {
        cudaEvent_t e;
        ANN_CUDA(cudaEventCreate(&e));
        g_fev.push_back({tag, e});
    }
    g_fev[g_fev_used].first = tag;
    ANN_CUDA(cudaEventRecord(g_fev[g_fev_used].second, st));
    g_fev_used++;
}

}  // namespace ann

using namespace ann;

namespace {

void mark(int i, cudaStream_t st) {
    if(!g_timing) return;
    cudaStreamCaptureStatus cs;
    ANN_CUDA(cudaStreamIsCapturing(st, &cs));
    if(cs != cudaStreamCaptureStatusNone) return;
    if(!g_ev[i]) ANN_CUDA(cudaEventCreate(&g_ev[i]));
    ANN_CUDA(cudaEventRecord(g_ev[i], st));
    g_ev_used[i] = true;
}

template<typename F>
int guard(F&& f) {
    try {
        f();
        return ANN_OK;
    } catch(const Error& e) {
        g_last_error = e.what();
        return e.code;
    } catch(const std::exception& e) {
        g_last_error = e.what();
        return ANN_ERR_INVALID;
    }
}

void need(bool ok, const char* msg) {
    if(!ok) throw Error(ANN_ERR_INVALID, msg);
}

cudaStream_t S(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// solves and residuals of the last SR solve (see ann_tdvp_solver_info)
void solver_info(const ann_tdvp_impl& t, double* out4, cudaStream_t st) {
    if(t.solver != ANN_SOLVER_FP64 && !t.fell_back && t.ir.p) {
        mixed_solve_info(t, out4, st);
        return;
    }
    double r[2] = {0.0, 0.0};
    ANN_CUDA(cudaMemcpyAsync(r, t.resid.as<cplx<double>>() + 2 * t.Np, sizeof(r), cudaMemcpyDeviceToHost, st));
    ANN_CUDA(cudaStreamSynchronize(st));
    out4[0] = 1.0;
    out4[1] = r[0];
    out4[2] = r[1];
    out4[3] = t.fell_back ? 1.0 : 0.0;
}

void sync(cudaStream_t st) { ANN_CUDA(cudaStreamSynchronize(st)); }

void check_status() {
    unsigned v = 0;
    unsigned* p = status_word();
    ANN_CUDA(cudaMemcpy(&v, p, sizeof(unsigned), cudaMemcpyDeviceToHost));
    if(v) {
        ANN_CUDA(cudaMemset(p, 0, sizeof(unsigned)));
        ANN_CUDA(cudaDeviceSynchronize());  // cleared before later kernels on other streams raise flags
        std::string m = "device status:";
        if(v & kStatusNonFinite) m += " non-finite value in log psi / local energy;";
        if(v & kStatusNotPosDef) m += " S + shift is not positive definite;";
        if(v & kStatusTimeout) m += " a bounded device wait timed out;";
        if(v & kStatusBadInput) m += " out-of-range index;";
        if(v & kStatusSolveStalled) m += " mixed-precision SR solve did not converge;";
        throw Error(ANN_ERR_NUMERIC, m);
    }
}

unsigned pow2_at_least(unsigned x) {
    unsigned p = 1;
    while(p < x) p <<= 1;
    return p;
}

size_t ld_for(unsigned Np) { return ((size_t)Np + 3) & ~(size_t)3; }

// weight pointer / constant of an ensemble's last rows
const double* row_weights(ann_ens_impl& ens) { return ens.kind == 0 ? ens.rows.weight.as<double>() : nullptr; }
double row_w0(const ann_ens_impl& ens) { return ens.kind == 0 ? 0.0 : ens.uniform_weight(); }

struct Scratch {
    DevBuf O, stats, partial, Obar, F, Osum, confs;
    Rows rows2;
};
Scratch& scratch() {
    static thread_local Scratch s;
    return s;
}

void mc_bookkeeping(ann_ens_impl& ens, cudaStream_t st) {
    if(ens.kind != 1) return;
    unsigned long long ar[4];
    ANN_CUDA(cudaMemcpyAsync(ar, ens.acc_rej.p, sizeof(ar), cudaMemcpyDeviceToHost, st));
    sync(st);
    ens.last_acc = ar[0];
    ens.last_rej = ar[1];
    ens.last_made_acc = ar[2];
    ens.last_made_rej = ar[3];
    // the learned proposal is dropped (local Metropolis continues alone) when its
    // acceptance falls below the set rate: the sampling pass's drop-rule kernel cleared the
    // device flag; the host copy follows it
    if(ens.made && ens.made_on.p) {
        int on = 1;
        ANN_CUDA(cudaMemcpyAsync(&on, ens.made_on.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        sync(st);
        ens.made_dropped = on == 0;
    }
}

Stats fetch_stats(const DevBuf& b, cudaStream_t st) {
    Stats s;
    ANN_CUDA(cudaMemcpyAsync(&s, b.p, sizeof(Stats), cudaMemcpyDeviceToHost, st));
    sync(st);
    return s;
}

}  // namespace

extern "C" {

const char* ann_last_error(void) { return g_last_error.c_str(); }
int ann_version(void) { return 10000; }

int ann_set_device(int device) {
    return guard([&] { ANN_CUDA(cudaSetDevice(device)); });
}
int ann_profiler_start(void) {
    return guard([&] { ANN_CUDA(cudaProfilerStart()); });
}
int ann_profiler_stop(void) {
    return guard([&] { ANN_CUDA(cudaProfilerStop()); });
}
unsigned long long ann_kernel_launch_count(void) { return g_launches.load(); }
int ann_status(unsigned* out) {
    return guard([&] {
        ANN_CUDA(cudaDeviceSynchronize());
        unsigned* p = status_word();
        ANN_CUDA(cudaMemcpy(out, p, sizeof(unsigned), cudaMemcpyDeviceToHost));
        ANN_CUDA(cudaMemset(p, 0, sizeof(unsigned)));
        ANN_CUDA(cudaDeviceSynchronize());
    });
}

// ---------------------------------------------------------------------------------
int ann_psi_create_rbm(const ann_rbm_desc* d, ann_psi** out) {
    return guard([&] {
        need(d && out, "null argument");
        need(d->N >= 1 && d->N <= 128, "N must be in [1, 128]");
        need(d->M >= 1 && d->M <= 256, "M must be in [1, 256]");
        need(d->C >= 1 && d->C <= d->N, "C must be in [1, N]");
        need(d->layout == ANN_LAYOUT_RBM || d->layout == ANN_LAYOUT_DEEP, "unknown layout");
        need(d->layout == ANN_LAYOUT_DEEP || d->C == d->N, "PsiRBM layout needs C == N");
        need(d->precision == ANN_PREC_FP32 || d->precision == ANN_PREC_FP64, "unknown precision");
        need(d->activation == ANN_ACT_POLY || d->activation == ANN_ACT_LOGCOSH, "unknown activation");
        need(d->params && d->final_weights, "params and final_weights are required");
        auto* p = new ann_psi();
        try {
            p->kind = 0;
            p->precision = d->precision;
            p->act = d->activation;
            p->N = d->N;
            p->NW = d->N > 64 ? 2 : 1;
            p->M = d->M;
            p->C = d->C;
            p->U = pow2_at_least((d->M + 31) / 32);
            p->Mpad = 32 * p->U;
            p->layout = d->layout;
            p->a_in = d->a_in_log_psi ? 1 : 0;
            p->Np = d->layout == ANN_LAYOUT_DEEP ? d->N + d->M + d->C * d->M : d->C * d->M;
            p->lp = zd(d->log_prefactor[0], d->log_prefactor[1]);
            p->conn.resize((size_t)d->C * d->M);
            std::vector<uint16_t> c16(p->conn.size());
            for(size_t k = 0; k < p->conn.size(); k++) {
                p->conn[k] = d->connections ? d->connections[k] : (unsigned)(k / d->M);
                need(p->conn[k] < d->N, "connection index out of range");
                c16[k] = (uint16_t)p->conn[k];
            }
            upload(p->connd, c16.data(), c16.size() * sizeof(uint16_t));
            upload(p->params, d->params, (size_t)p->Np * 16);
            p->fw.assign(d->M, zd(0, 0));
            const size_t es = p->elem_bytes();
            std::vector<unsigned char> fwb(p->Mpad * es, 0);
            for(unsigned j = 0; j < d->M; j++) {
                p->fw[j] = zd(d->final_weights[2 * j], d->final_weights[2 * j + 1]);
                if(p->precision == 0) {
                    float v[2] = {(float)p->fw[j].real(), (float)p->fw[j].imag()};
                    std::memcpy(&fwb[j * es], v, es);
                } else {
                    std::memcpy(&fwb[j * es], &d->final_weights[2 * j], es);
                }
            }
            upload(p->fwd, fwb.data(), fwb.size());
            p->Wd.ensure((size_t)p->N * p->Mpad * es);
            p->a.ensure((size_t)p->N * es);
            p->b.ensure((size_t)p->Mpad * es);
            psi_prepare(*p, nullptr);
            ANN_CUDA(cudaDeviceSynchronize());
        } catch(...) {
            delete p;
            throw;
        }
        *out = p;
    });
}

int ann_psi_copy(const ann_psi* src, ann_psi** out) {
    return guard([&] {
        need(src && out, "null argument");
        auto* p = new ann_psi();
        try {
            p->kind = src->kind;
            p->precision = src->precision;
            p->act = src->act;
            p->N = src->N;
            p->NW = src->NW;
            p->Np = src->Np;
            p->lp = src->lp;
            p->M = src->M;
            p->Mpad = src->Mpad;
            p->C = src->C;
            p->U = src->U;
            p->layout = src->layout;
            p->a_in = src->a_in;
            p->conn = src->conn;
            p->fw = src->fw;
            for(int d = 0; d < 3; d++) p->extent[d] = src->extent[d];
            p->layers = src->layers;
            p->sym = src->sym;
            p->ncls = src->ncls;
            p->final_factor = src->final_factor;
            p->deep = src->deep;
            auto clone = [](DevBuf& dst, const DevBuf& s) {
                if(!s.p) return;
                dst.ensure(s.bytes);
                ANN_CUDA(cudaMemcpy(dst.p, s.p, s.bytes, cudaMemcpyDeviceToDevice));
            };
            clone(p->params, src->params);
            clone(p->Wd, src->Wd);
            clone(p->a, src->a);
            clone(p->b, src->b);
            clone(p->fwd, src->fwd);
            clone(p->connd, src->connd);
            clone(p->cnn_w, src->cnn_w);
            clone(p->cnn_meta, src->cnn_meta);
            clone(p->deep_tab, src->deep_tab);
            clone(p->feat_beg, src->feat_beg);
            clone(p->feat_zy, src->feat_zy);
            clone(p->feat_c, src->feat_c);
            clone(p->feat_cf, src->feat_cf);
            p->feat_beg_h = src->feat_beg_h;
            p->feat_a_h = src->feat_a_h;
            p->feat_b_h = src->feat_b_h;
            p->feat_coeff_h = src->feat_coeff_h;
            p->order = src->order;
        } catch(...) {
            delete p;
            throw;
        }
        *out = p;
    });
}

int ann_psi_destroy(ann_psi* psi) {
    return guard([&] { delete psi; });
}
int ann_psi_num_params(const ann_psi* psi, unsigned* out) {
    return guard([&] {
        need(psi && out, "null argument");
        *out = psi->Np;
    });
}
int ann_psi_get_params(const ann_psi* psi, double* out) {
    return guard([&] {
        need(psi && out, "null argument");
        ANN_CUDA(cudaDeviceSynchronize());
        ANN_CUDA(cudaMemcpy(out, psi->params.p, (size_t)psi->Np * 16, cudaMemcpyDeviceToHost));
    });
}
int ann_psi_set_params(ann_psi* psi, const double* params) {
    return guard([&] {
        need(psi && params, "null argument");
        ANN_CUDA(cudaMemcpy(psi->params.p, params, (size_t)psi->Np * 16, cudaMemcpyHostToDevice));
        psi_prepare(*psi, nullptr);
    });
}
int ann_psi_set_params_async(ann_psi* psi, const double* params, void* stream) {
    return guard([&] {
        need(psi && params, "null argument");
        ANN_CUDA(cudaMemcpyAsync(psi->params.p, params, (size_t)psi->Np * 16, cudaMemcpyHostToDevice, S(stream)));
        psi_prepare(*psi, S(stream));
    });
}
int ann_psi_get_log_prefactor(const ann_psi* psi, double* out2) {
    return guard([&] {
        need(psi && out2, "null argument");
        out2[0] = psi->lp.real();
        out2[1] = psi->lp.imag();
    });
}
int ann_psi_set_log_prefactor(ann_psi* psi, double re, double im) {
    return guard([&] {
        need(psi, "null argument");
        psi->lp = zd(re, im);
    });
}
int ann_psi_params_device(ann_psi* psi, void** out) {
    return guard([&] {
        need(psi && out, "null argument");
        *out = psi->params.p;
    });
}
int ann_psi_sync_device_params(ann_psi* psi, void* stream) {
    return guard([&] {
        need(psi, "null argument");
        psi_prepare(*psi, S(stream));
    });
}

// ---------------------------------------------------------------------------------
int ann_op_create_pauli(unsigned n, unsigned nw_in, const uint64_t* a, const uint64_t* b, const double* coeff,
                        ann_op** out) {
    return guard([&] {
        need(out && (n == 0 || (a && b && coeff)), "null argument");
        need(nw_in >= 1 && nw_in <= (unsigned)kMaxWords, "num_words must be 1 or 2");
        auto* op = new ann_op();
        try {
            const unsigned nw = kMaxWords;
            op->nw = nw;
            op->n_strings = n;
            op->a.assign((size_t)n * nw, 0);
            op->b.assign((size_t)n * nw, 0);
            op->coeff.resize(n);
            for(unsigned k = 0; k < n; k++) {
                for(unsigned w = 0; w < nw_in; w++) {
                    op->a[k * nw + w] = a[k * nw_in + w];
                    op->b[k * nw + w] = b[k * nw_in + w];
                }
                op->coeff[k] = zd(coeff[2 * k], coeff[2 * k + 1]);
                for(unsigned w = 0; w < nw; w++) {
                    const uint64_t m = op->a[k * nw + w] | op->b[k * nw + w];
                    if(m) op->max_site = std::max(op->max_site, 64u * w + 64u - (unsigned)__builtin_clzll(m));
                }
            }
            // group: diagonal strings, then strings by flip mask in first-appearance order
            std::vector<uint64_t> dmask, smask;
            std::vector<double> dcoef, scoef;
            std::vector<unsigned> site_begin{0}, str_begin{0};
            std::vector<uint16_t> sites;
            std::vector<std::vector<uint64_t>> flips;
            std::vector<std::vector<unsigned>> members;
            for(unsigned k = 0; k < n; k++) {
                std::vector<uint64_t> f(nw);
                bool diag = true;
                for(unsigned w = 0; w < nw; w++) {
                    f[w] = op->a[k * nw + w] ^ op->b[k * nw + w];
                    diag = diag && f[w] == 0;
                }
                if(diag) {
                    for(unsigned w = 0; w < nw; w++) dmask.push_back(op->b[k * nw + w]);
                    dcoef.push_back(op->coeff[k].real());
                    dcoef.push_back(op->coeff[k].imag());
                    continue;
                }
                size_t g = 0;
                while(g < flips.size() && flips[g] != f) g++;
                if(g == flips.size()) {
                    flips.push_back(f);
                    members.push_back({});
                }
                members[g].push_back(k);
            }
            for(size_t g = 0; g < flips.size(); g++) {
                for(unsigned w = 0; w < nw; w++) {
                    uint64_t m = flips[g][w];
                    while(m) {
                        sites.push_back((uint16_t)(64u * w + __builtin_ctzll(m)));
                        m &= m - 1;
                    }
                }
                site_begin.push_back((unsigned)sites.size());
                for(unsigned k : members[g]) {
                    int ny = 0;
                    for(unsigned w = 0; w < nw; w++) {
                        smask.push_back(op->b[k * nw + w]);  // Z | Y sites are exactly the b bits
                        ny += __builtin_popcountll((~op->a[k * nw + w]) & op->b[k * nw + w]);
                    }
                    // (-i)^{n_y} (PauliString.hpp:193-208)
                    zd ph(1.0, 0.0);
                    for(int q = 0; q < (ny & 3); q++) ph *= zd(0.0, -1.0);
                    const zd c = op->coeff[k] * ph;
                    scoef.push_back(c.real());
                    scoef.push_back(c.imag());
                }
                str_begin.push_back((unsigned)(scoef.size() / 2));
            }
            op->n_diag = (unsigned)(dcoef.size() / 2);
            op->n_groups = (unsigned)flips.size();
            upload(op->diag_mask, dmask.data(), dmask.size() * 8);
            upload(op->diag_coeff, dcoef.data(), dcoef.size() * 8);
            upload(op->grp_site_begin, site_begin.data(), site_begin.size() * 4);
            upload(op->grp_sites, sites.data(), sites.size() * 2);
            upload(op->grp_str_begin, str_begin.data(), str_begin.size() * 4);
            upload(op->str_mask, smask.data(), smask.size() * 8);
            upload(op->str_coeff, scoef.data(), scoef.size() * 8);
            std::vector<float> df(dcoef.begin(), dcoef.end()), sf(scoef.begin(), scoef.end());
            upload(op->diag_coeff_f, df.data(), df.size() * 4);
            upload(op->str_coeff_f, sf.data(), sf.size() * 4);
            // the strings as given, for the Pauli-string basis (first word: sites < 64)
            std::vector<uint64_t> ra(n), rb(n);
            std::vector<double> rc(2 * (size_t)n);
            std::vector<float> rcf(2 * (size_t)n);
            for(unsigned k = 0; k < n; k++) {
                ra[k] = op->a[(size_t)k * nw];
                rb[k] = op->b[(size_t)k * nw];
                rc[2 * k] = op->coeff[k].real();
                rc[2 * k + 1] = op->coeff[k].imag();
                rcf[2 * k] = (float)rc[2 * k];
                rcf[2 * k + 1] = (float)rc[2 * k + 1];
            }
            upload(op->raw_a, ra.data(), ra.size() * 8);
            upload(op->raw_b, rb.data(), rb.size() * 8);
            upload(op->raw_c, rc.data(), rc.size() * 8);
            upload(op->raw_cf, rcf.data(), rcf.size() * 4);
        } catch(...) {
            delete op;
            throw;
        }
        *out = op;
    });
}
int ann_op_destroy(ann_op* op) {
    return guard([&] { delete op; });
}
int ann_op_num_strings(const ann_op* op, unsigned* out) {
    return guard([&] {
        need(op && out, "null argument");
        *out = op->n_strings;
    });
}

// ---------------------------------------------------------------------------------
int ann_ens_create_exact(unsigned num_sites, ann_ens** out) {
    return guard([&] {
        need(out, "null argument");
        need(num_sites >= 1 && num_sites <= 28, "exact summation supports 1..28 sites");
        auto* e = new ann_ens();
        e->kind = 0;
        e->N = num_sites;
        *out = e;
    });
}

int ann_ens_create_mc(const ann_mc_desc* d, ann_ens** out) {
    return guard([&] {
        need(d && out, "null argument");
        need(d->num_markov_chains >= 1, "num_markov_chains must be >= 1");
        need(d->num_samples >= d->num_markov_chains, "num_samples must be >= num_markov_chains");
        need(d->move >= ANN_MOVE_FLIP && d->move <= ANN_MOVE_EXCHANGE_PAIRS, "unknown move");
        need(d->move != ANN_MOVE_EXCHANGE_BONDS || (d->bonds && d->n_bonds > 0), "exchange moves need bonds");
        auto* e = new ann_ens();
        try {
            e->kind = 1;
            e->num_samples = d->num_samples;
            e->num_sweeps = d->num_sweeps;
            e->num_therm = d->num_thermalization_sweeps;
            e->n_chains = d->num_markov_chains;
            e->move = d->move;
            e->n_up = d->n_up;
            e->seed = d->seed;
            e->persistent = d->persistent;
            if(d->bonds && d->n_bonds) {
                e->bonds.assign(d->bonds, d->bonds + 2 * d->n_bonds);
                upload(e->bonds_d, e->bonds.data(), e->bonds.size() * 4);
            }
            e->chain_conf.ensure((size_t)e->n_chains * kMaxWords * 8);
            e->chain_counter.ensure((size_t)e->n_chains * 8);
            ANN_CUDA(cudaMemset(e->chain_conf.p, 0, e->chain_conf.bytes));
            ANN_CUDA(cudaMemset(e->chain_counter.p, 0, e->chain_counter.bytes));
            e->acc_rej.ensure(4 * sizeof(unsigned long long));
            ANN_CUDA(cudaMemset(e->acc_rej.p, 0, 4 * sizeof(unsigned long long)));
            // the clears run on the legacy default stream, which does not order with the
            // non-blocking streams the ensemble is used on: complete them here
            ANN_CUDA(cudaDeviceSynchronize());
        } catch(...) {
            delete e;
            throw;
        }
        *out = e;
    });
}

int ann_ens_copy(const ann_ens* src, ann_ens** out) {
    return guard([&] {
        need(src && out, "null argument");
        *out = ens_clone(*src);
    });
}

int ann_ens_destroy(ann_ens* e) {
    return guard([&] { delete e; });
}
int ann_ens_num_steps(const ann_ens* e, unsigned* out) {
    return guard([&] {
        need(e && out, "null argument");
        *out = e->kind == 0 ? e->num_steps() : e->num_samples;
    });
}
int ann_ens_set_basis(ann_ens* e, int basis) {
    return guard([&] {
        need(e, "null argument");
        need(basis == ANN_BASIS_SPINS || basis == ANN_BASIS_PAULIS, "unknown basis");
        if(basis == ANN_BASIS_PAULIS) {
            need(e->kind == 1 || e->N <= 14, "exact summation over Pauli strings supports 1..14 sites");
            need(e->kind == 0 || (e->move == ANN_MOVE_FLIP && e->n_up < 0 && e->tape_len == 0),
                 "Pauli-string chains take single-site moves only (no exchange, fixed Sz or tape)");
        }
        e->basis = basis;
        e->chains_valid = false;
    });
}
int ann_ens_refresh_stats(ann_ens* e, void* stream) {
    return guard([&] {
        need(e, "null argument");
        mc_bookkeeping(*e, S(stream));
    });
}

int ann_ens_acceptance_rate(const ann_ens* e, double* out) {
    return guard([&] {
        need(e && out, "null argument");
        const double tot = (double)(e->last_acc + e->last_rej);
        *out = tot > 0 ? (double)e->last_acc / tot : 0.0;
    });
}
int ann_ens_get_chains(const ann_ens* e, uint64_t* conf, uint64_t* counter) {
    return guard([&] {
        need(e && e->kind == 1, "not a Monte Carlo ensemble");
        ANN_CUDA(cudaDeviceSynchronize());
        if(conf) ANN_CUDA(cudaMemcpy(conf, e->chain_conf.p, (size_t)e->n_chains * kMaxWords * 8, cudaMemcpyDeviceToHost));
        if(counter) ANN_CUDA(cudaMemcpy(counter, e->chain_counter.p, (size_t)e->n_chains * 8, cudaMemcpyDeviceToHost));
    });
}
int ann_ens_set_chains(ann_ens* e, const uint64_t* conf, const uint64_t* counter) {
    return guard([&] {
        need(e && e->kind == 1 && conf && counter, "not a Monte Carlo ensemble / null argument");
        ANN_CUDA(cudaMemcpy(e->chain_conf.p, conf, (size_t)e->n_chains * kMaxWords * 8, cudaMemcpyHostToDevice));
        ANN_CUDA(cudaMemcpy(e->chain_counter.p, counter, (size_t)e->n_chains * 8, cudaMemcpyHostToDevice));
        e->chains_valid = true;
    });
}
int ann_ens_set_proposal(ann_ens* e, const ann_made* m, unsigned indep_per_sample, double min_acceptance) {
    return guard([&] {
        need(e && e->kind == 1, "not a Monte Carlo ensemble");
        e->made = m;
        e->indep_per_sample = m ? indep_per_sample : 0;
        e->made_min_acceptance = min_acceptance;
        e->made_dropped = false;
        const int on = 1;
        e->made_on.ensure(sizeof(int));
        ANN_CUDA(cudaMemcpy(e->made_on.p, &on, sizeof(int), cudaMemcpyHostToDevice));
    });
}
int ann_ens_proposal_stats(const ann_ens* e, double* acceptance, int* dropped) {
    return guard([&] {
        need(e && e->kind == 1, "not a Monte Carlo ensemble");
        const double tot = (double)(e->last_made_acc + e->last_made_rej);
        if(acceptance) *acceptance = tot > 0 ? (double)e->last_made_acc / tot : 0.0;
        if(dropped) *dropped = e->made_dropped ? 1 : 0;
    });
}
int ann_ens_set_history(ann_ens* e, unsigned capacity) {
    return guard([&] {
        need(e != nullptr, "null argument");
        e->hist_cap = capacity;
        e->hist_len = 0;
        if(capacity) {
            e->hist.ensure((size_t)capacity * kMaxWords * sizeof(uint64_t));
            e->hist_posd.ensure(sizeof(unsigned long long));
            ANN_CUDA(cudaMemset(e->hist_posd.p, 0, sizeof(unsigned long long)));
            ANN_CUDA(cudaDeviceSynchronize());  // before any non-blocking stream appends
        }
    });
}

int ann_ens_set_tape(ann_ens* e, const uint64_t* init, const uint32_t* sites, const double* u, unsigned len) {
    return guard([&] {
        need(e && e->kind == 1, "not a Monte Carlo ensemble");
        if(!sites) {
            e->tape_len = 0;
            return;
        }
        need(init && u && len > 0, "tape needs init, sites, u");
        need(e->move == ANN_MOVE_FLIP, "tape replay is defined for single flips");
        upload(e->tape_init, init, (size_t)e->n_chains * kMaxWords * 8);
        upload(e->tape_site, sites, (size_t)e->n_chains * len * 4);
        upload(e->tape_u, u, (size_t)e->n_chains * len * 8);
        e->tape_len = len;
    });
}
int ann_ens_get_samples(const ann_ens* e, uint64_t* conf, double* log_psi, double* eloc) {
    return guard([&] {
        need(e, "null argument");
        ANN_CUDA(cudaDeviceSynchronize());
        const size_t n = e->rows.n;
        if(conf) ANN_CUDA(cudaMemcpy(conf, e->rows.conf.p, n * kMaxWords * 8, cudaMemcpyDeviceToHost));
        if(log_psi) ANN_CUDA(cudaMemcpy(log_psi, e->rows.log_psi.p, n * 16, cudaMemcpyDeviceToHost));
        if(eloc) ANN_CUDA(cudaMemcpy(eloc, e->rows.eloc.p, n * 16, cudaMemcpyDeviceToHost));
    });
}

// ---------------------------------------------------------------------------------
int ann_expectation(ann_op* op, ann_psi* psi, ann_ens* ens, void* stream, double* out2) {
    return guard([&] {
        need(op && psi && ens && out2, "null argument");
        auto& sc = scratch();
        cudaStream_t st = S(stream);
        run_ensemble(*psi, op, *ens, SampleTargets{&ens->rows}, st);
        sc.stats.ensure(sizeof(Stats));
        row_stats(ens->rows, row_weights(*ens), row_w0(*ens), sc.stats.as<Stats>(), sc.partial, st);
        const Stats s = fetch_stats(sc.stats, st);
        mc_bookkeeping(*ens, st);
        check_status();
        out2[0] = s.E[0];
        out2[1] = s.E[1];
    });
}

int ann_expectation_list(ann_op** ops, unsigned n_ops, ann_psi* psi, ann_ens* ens, void* stream, double* out) {
    return guard([&] {
        need(ops && psi && ens && out, "null argument");
        auto& sc = scratch();
        cudaStream_t st = S(stream);
        // one sampling pass; every operator is evaluated on the same configurations
        // (ExpectationValue.cu.template:83-128)
        run_ensemble(*psi, nullptr, *ens, SampleTargets{&ens->rows, nullptr, 0, false}, st);
        sc.stats.ensure(sizeof(Stats));
        for(unsigned k = 0; k < n_ops; k++) {
            need(ops[k] != nullptr, "null operator");
            run_confs(*psi, ops[k], ens->rows.conf.as<uint64_t>(), ens->rows.n, sc.rows2, nullptr, 0, st);
            // weights of the sampling pass
            row_stats(sc.rows2, row_weights(*ens), row_w0(*ens), sc.stats.as<Stats>(), sc.partial, st);
            const Stats s = fetch_stats(sc.stats, st);
            out[2 * k] = s.E[0];
            out[2 * k + 1] = s.E[1];
        }
        mc_bookkeeping(*ens, st);
        check_status();
    });
}

int ann_fluctuation(ann_op* op, ann_psi* psi, ann_ens* ens, void* stream, double* out3) {
    return guard([&] {
        need(op && psi && ens && out3, "null argument");
        auto& sc = scratch();
        cudaStream_t st = S(stream);
        run_ensemble(*psi, op, *ens, SampleTargets{&ens->rows}, st);
        sc.stats.ensure(sizeof(Stats));
        row_stats(ens->rows, row_weights(*ens), row_w0(*ens), sc.stats.as<Stats>(), sc.partial, st);
        const Stats s = fetch_stats(sc.stats, st);
        mc_bookkeeping(*ens, st);
        check_status();
        out3[0] = std::sqrt(s.E2 - (s.E[0] * s.E[0] + s.E[1] * s.E[1]));
        out3[1] = s.E[0];
        out3[2] = s.E[1];
    });
}

int ann_gradient(ann_op* op, ann_psi* psi, ann_ens* ens, void* stream, double* grad, double* value2) {
    return guard([&] {
        need(op && psi && ens && grad, "null argument");
        auto& sc = scratch();
        cudaStream_t st = S(stream);
        const size_t rows = ens->num_steps();
        const size_t ld = ld_for(psi->Np);
        sc.O.ensure(rows * ld * psi->elem_bytes());
        run_ensemble(*psi, op, *ens, SampleTargets{&ens->rows, sc.O.p, ld, true}, st);
        sc.stats.ensure(sizeof(Stats));
        sc.F.ensure((size_t)psi->Np * 16);
        row_stats(ens->rows, row_weights(*ens), row_w0(*ens), sc.stats.as<Stats>(), sc.partial, st);
        // gradient_k = sum w conj(O_k) E_loc - <E> sum w conj(O_k) == F_k
        sc.Obar.ensure((size_t)psi->Np * 16);
        col_stats(sc.O.p, psi->precision, ens->rows.n, ld, psi->Np, row_weights(*ens), row_w0(*ens),
                  ens->rows.eloc.as<cplx<double>>(), sc.Obar.as<cplx<double>>(), sc.F.as<cplx<double>>(),
                  sc.stats.as<Stats>(), nullptr, sc.partial, st);
        ANN_CUDA(cudaMemcpyAsync(grad, sc.F.p, (size_t)psi->Np * 16, cudaMemcpyDeviceToHost, st));
        const Stats s = fetch_stats(sc.stats, st);
        mc_bookkeeping(*ens, st);
        check_status();
        if(value2) {
            value2[0] = s.E[0];
            value2[1] = s.E[1];
        }
    });
}

int ann_exp_sigma_z(ann_op* op, ann_psi* psi, ann_ens* ens, void* stream, double* out2) {
    return guard([&] {
        need(op && psi && ens && out2, "null argument");
        cudaStream_t st = S(stream);
        run_ensemble(*psi, nullptr, *ens, SampleTargets{&ens->rows, nullptr, 0, false}, st);
        exp_sigma_z_sum(*op, ens->rows, row_weights(*ens), row_w0(*ens), out2, st);
        mc_bookkeeping(*ens, st);
        check_status();
    });
}

int ann_log_psi_s(ann_psi* psi, const uint64_t* conf, double* out2) {
    return ann_log_psi_batch(psi, conf, 1, nullptr, out2);
}

int ann_log_psi_batch(ann_psi* psi, const uint64_t* confs, unsigned n, void* stream, double* out) {
    return guard([&] {
        need(psi && confs && out, "null argument");
        auto& sc = scratch();
        cudaStream_t st = S(stream);
        std::vector<uint64_t> c((size_t)n * kMaxWords, 0);
        for(unsigned k = 0; k < n; k++)
            for(unsigned w = 0; w < psi->NW; w++) c[(size_t)k * kMaxWords + w] = confs[(size_t)k * psi->NW + w];
        sc.confs.ensure(c.size() * 8);
        ANN_CUDA(cudaMemcpyAsync(sc.confs.p, c.data(), c.size() * 8, cudaMemcpyHostToDevice, st));
        run_confs(*psi, nullptr, sc.confs.as<uint64_t>(), n, sc.rows2, nullptr, 0, st);
        ANN_CUDA(cudaMemcpyAsync(out, sc.rows2.log_psi.p, (size_t)n * 16, cudaMemcpyDeviceToHost, st));
        sync(st);
        check_status();
    });
}

int ann_local_energies(ann_psi* psi, ann_op* op, const uint64_t* confs, unsigned n, void* stream, double* out) {
    return guard([&] {
        need(psi && op && confs && out, "null argument");
        auto& sc = scratch();
        cudaStream_t st = S(stream);
        std::vector<uint64_t> c((size_t)n * kMaxWords, 0);
        for(unsigned k = 0; k < n; k++)
            for(unsigned w = 0; w < psi->NW; w++) c[(size_t)k * kMaxWords + w] = confs[(size_t)k * psi->NW + w];
        sc.confs.ensure(c.size() * 8);
        ANN_CUDA(cudaMemcpyAsync(sc.confs.p, c.data(), c.size() * 8, cudaMemcpyHostToDevice, st));
        run_confs(*psi, op, sc.confs.as<uint64_t>(), n, sc.rows2, nullptr, 0, st);
        ANN_CUDA(cudaMemcpyAsync(out, sc.rows2.eloc.p, (size_t)n * 16, cudaMemcpyDeviceToHost, st));
        sync(st);
        check_status();
    });
}

namespace {
// (a, b) pairs -> device rows, then the explicit-configuration kernels in the Pauli basis
void paulis_to_rows(const uint64_t* ab, unsigned n, DevBuf& dst, cudaStream_t st) {
    dst.ensure((size_t)std::max(1u, n) * kMaxWords * 8);
    ANN_CUDA(cudaMemcpyAsync(dst.p, ab, (size_t)n * kMaxWords * 8, cudaMemcpyHostToDevice, st));
}
}  // namespace

int ann_log_psi_paulis(ann_psi* psi, const uint64_t* ab, unsigned n, void* stream, double* out) {
    return guard([&] {
        need(psi && ab && out, "null argument");
        auto& sc = scratch();
        cudaStream_t st = S(stream);
        paulis_to_rows(ab, n, sc.confs, st);
        run_confs(*psi, nullptr, sc.confs.as<uint64_t>(), n, sc.rows2, nullptr, 0, st, ANN_BASIS_PAULIS);
        ANN_CUDA(cudaMemcpyAsync(out, sc.rows2.log_psi.p, (size_t)n * 16, cudaMemcpyDeviceToHost, st));
        sync(st);
        check_status();
    });
}

int ann_local_energies_paulis(ann_psi* psi, ann_op* op, const uint64_t* ab, unsigned n, void* stream, double* out) {
    return guard([&] {
        need(psi && op && ab && out, "null argument");
        auto& sc = scratch();
        cudaStream_t st = S(stream);
        paulis_to_rows(ab, n, sc.confs, st);
        run_confs(*psi, op, sc.confs.as<uint64_t>(), n, sc.rows2, nullptr, 0, st, ANN_BASIS_PAULIS);
        ANN_CUDA(cudaMemcpyAsync(out, sc.rows2.eloc.p, (size_t)n * 16, cudaMemcpyDeviceToHost, st));
        sync(st);
        check_status();
    });
}

int ann_psi_O_k_paulis(ann_psi* psi, const uint64_t* ab, double* out) {
    return guard([&] {
        need(psi && ab && out, "null argument");
        auto& sc = scratch();
        paulis_to_rows(ab, 1, sc.confs, nullptr);
        const size_t ld = ld_for(psi->Np);
        sc.O.ensure(ld * psi->elem_bytes());
        run_confs(*psi, nullptr, sc.confs.as<uint64_t>(), 1, sc.rows2, sc.O.p, ld, nullptr, ANN_BASIS_PAULIS);
        ANN_CUDA(cudaDeviceSynchronize());
        if(psi->precision == 1) {
            ANN_CUDA(cudaMemcpy(out, sc.O.p, (size_t)psi->Np * 16, cudaMemcpyDeviceToHost));
        } else {
            std::vector<float> f((size_t)psi->Np * 2);
            ANN_CUDA(cudaMemcpy(f.data(), sc.O.p, f.size() * 4, cudaMemcpyDeviceToHost));
            for(size_t k = 0; k < f.size(); k++) out[k] = f[k];
        }
        check_status();
    });
}

int ann_psi_O_k(ann_psi* psi, const uint64_t* conf, double* out) {
    return guard([&] {
        need(psi && conf && out, "null argument");
        auto& sc = scratch();
        uint64_t c[kMaxWords] = {0, 0};
        for(unsigned w = 0; w < psi->NW; w++) c[w] = conf[w];
        sc.confs.ensure(sizeof(c));
        ANN_CUDA(cudaMemcpy(sc.confs.p, c, sizeof(c), cudaMemcpyHostToDevice));
        const size_t ld = ld_for(psi->Np);
        sc.O.ensure(ld * psi->elem_bytes());
        run_confs(*psi, nullptr, sc.confs.as<uint64_t>(), 1, sc.rows2, sc.O.p, ld, nullptr);
        ANN_CUDA(cudaDeviceSynchronize());
        if(psi->precision == 1) {
            ANN_CUDA(cudaMemcpy(out, sc.O.p, (size_t)psi->Np * 16, cudaMemcpyDeviceToHost));
        } else {
            std::vector<float> f((size_t)psi->Np * 2);
            ANN_CUDA(cudaMemcpy(f.data(), sc.O.p, f.size() * 4, cudaMemcpyDeviceToHost));
            for(size_t k = 0; k < f.size(); k++) out[k] = f[k];
        }
        check_status();
    });
}

int ann_psi_O_k_vector(ann_psi* psi, ann_ens* ens, void* stream, double* out) {
    return guard([&] {
        need(psi && ens && out, "null argument");
        auto& sc = scratch();
        cudaStream_t st = S(stream);
        const size_t rows = ens->num_steps();
        const size_t ld = ld_for(psi->Np);
        sc.O.ensure(rows * ld * psi->elem_bytes());
        run_ensemble(*psi, nullptr, *ens, SampleTargets{&ens->rows, sc.O.p, ld, false}, st);
        sc.Osum.ensure((size_t)psi->Np * 16);
        col_stats(sc.O.p, psi->precision, ens->rows.n, ld, psi->Np, nullptr, 1.0, nullptr, nullptr, nullptr, nullptr,
                  sc.Osum.as<cplx<double>>(), sc.partial, st);
        ANN_CUDA(cudaMemcpyAsync(out, sc.Osum.p, (size_t)psi->Np * 16, cudaMemcpyDeviceToHost, st));
        sync(st);
        mc_bookkeeping(*ens, st);
        check_status();
    });
}

int ann_log_psi(ann_psi* psi, ann_ens* ens, void* stream, double* out2) {
    return guard([&] {
        need(psi && ens && out2, "null argument");
        auto& sc = scratch();
        cudaStream_t st = S(stream);
        run_ensemble(*psi, nullptr, *ens, SampleTargets{&ens->rows, nullptr, 0, false}, st);
        sc.stats.ensure(sizeof(Stats));
        row_stats(ens->rows, row_weights(*ens), row_w0(*ens), sc.stats.as<Stats>(), sc.partial, st);
        const Stats s = fetch_stats(sc.stats, st);
        mc_bookkeeping(*ens, st);
        check_status();
        out2[0] = s.L[0];
        out2[1] = s.L[1];
    });
}

static int log_vec_impl(ann_psi* psi, ann_ens* ens, void* stream, double* out, bool expo) {
    return guard([&] {
        need(psi && ens && out, "null argument");
        cudaStream_t st = S(stream);
        run_ensemble(*psi, nullptr, *ens, SampleTargets{&ens->rows, nullptr, 0, false}, st);
        const size_t n = ens->rows.n;
        ANN_CUDA(cudaMemcpyAsync(out, ens->rows.log_psi.p, n * 16, cudaMemcpyDeviceToHost, st));
        sync(st);
        mc_bookkeeping(*ens, st);
        check_status();
        if(expo)
            for(size_t k = 0; k < n; k++) {
                const zd z = std::exp(zd(out[2 * k], out[2 * k + 1]));
                out[2 * k] = z.real();
                out[2 * k + 1] = z.imag();
            }
    });
}
int ann_psi_vector(ann_psi* psi, ann_ens* ens, void* stream, double* out) { return log_vec_impl(psi, ens, stream, out, true); }
int ann_log_psi_vector(ann_psi* psi, ann_ens* ens, void* stream, double* out) {
    return log_vec_impl(psi, ens, stream, out, false);
}

int ann_psi_norm(ann_psi* psi, ann_ens* ens, void* stream, double* out) {
    return guard([&] {
        need(psi && ens && out, "null argument");
        need(ens->kind == 0, "norm needs an exact-summation ensemble");
        auto& sc = scratch();
        cudaStream_t st = S(stream);
        run_ensemble(*psi, nullptr, *ens, SampleTargets{&ens->rows, nullptr, 0, false}, st);
        sc.stats.ensure(sizeof(Stats));
        row_stats(ens->rows, ens->rows.weight.as<double>(), 0.0, sc.stats.as<Stats>(), sc.partial, st);
        const Stats s = fetch_stats(sc.stats, st);
        check_status();
        *out = std::sqrt(s.W);
    });
}

int ann_apply_operator(ann_psi* psi, ann_op* op, ann_ens* ens, void* stream, double* out) {
    return guard([&] {
        need(psi && op && ens && out, "null argument");
        cudaStream_t st = S(stream);
        run_ensemble(*psi, op, *ens, SampleTargets{&ens->rows}, st);
        const size_t n = ens->rows.n;
        std::vector<double> lp(2 * n), el(2 * n);
        ANN_CUDA(cudaMemcpyAsync(lp.data(), ens->rows.log_psi.p, n * 16, cudaMemcpyDeviceToHost, st));
        ANN_CUDA(cudaMemcpyAsync(el.data(), ens->rows.eloc.p, n * 16, cudaMemcpyDeviceToHost, st));
        sync(st);
        mc_bookkeeping(*ens, st);
        check_status();
        for(size_t k = 0; k < n; k++) {
            const zd v = std::exp(zd(lp[2 * k], lp[2 * k + 1])) * zd(el[2 * k], el[2 * k + 1]);
            out[2 * k] = v.real();
            out[2 * k + 1] = v.imag();
        }
    });
}

int ann_activation_function(double re, double im, unsigned layer, int activation, double* out2) {
    return guard([&] {
        need(out2, "null argument");
        activation_host(re, im, layer, activation, out2);
    });
}

// ---------------------------------------------------------------------------------
int ann_tdvp_create(unsigned num_params, ann_tdvp** out) {
    return guard([&] {
        need(out && num_params >= 1, "bad argument");
        auto* t = new ann_tdvp();
        t->Np = num_params;
        *out = t;
    });
}
int ann_tdvp_destroy(ann_tdvp* t) {
    return guard([&] {
        if(t) {
            if(t->graph_exec) cudaGraphExecDestroy(t->graph_exec);
            if(t->graph) cudaGraphDestroy(t->graph);
            for(auto e : t->side_ev)
                if(e) cudaEventDestroy(e);
            if(t->side) cudaStreamDestroy(t->side);
        }
        delete t;
    });
}
int ann_tdvp_set_s_mode(ann_tdvp* t, int mode) {
    return guard([&] {
        need(t && mode >= ANN_S_FP32 && mode <= ANN_S_BF16_SPLIT, "bad S mode");
        t->s_mode = mode;
    });
}

}  // extern "C"

namespace ann {

SampleTargets tdvp_prepare(ann_tdvp_impl& t, ann_psi_impl& psi, ann_ens_impl& ens) {
    if(t.Np != psi.Np) throw Error(ANN_ERR_INVALID, "TDVP num_params differs from psi.num_params");
    const size_t rows = ens.num_steps();
    const size_t ld = ld_for(psi.Np);
    t.n_rows = rows;
    t.ldO = ld;
    t.O_precision = psi.precision;
    t.O.ensure(rows * ld * psi.elem_bytes());
    t.stats.ensure(sizeof(Stats));
    t.Obar.ensure((size_t)psi.Np * 16);
    t.F.ensure((size_t)psi.Np * 16);
    return SampleTargets{&ens.rows, t.O.p, ld, true};
}

void tdvp_post(ann_tdvp_impl& t, ann_psi_impl& psi, ann_ens_impl& ens, bool want_S, cudaStream_t st) {
    const size_t rows = t.n_rows, ld = t.ldO;
    const double* w = row_weights(ens);
    const double w0 = row_w0(ens);
    t.wts_exact = ens.kind == 0;
    t.w0 = w0;
    if(w) {
        t.wts.ensure(rows * sizeof(double));
        ANN_CUDA(cudaMemcpyAsync(t.wts.p, w, rows * sizeof(double), cudaMemcpyDeviceToDevice, st));
    }
    const double* tw = w ? t.wts.as<double>() : nullptr;
    row_stats(ens.rows, tw, w0, t.stats.as<Stats>(), t.partial, st);
    col_stats(t.O.p, psi.precision, rows, ld, psi.Np, tw, w0, ens.rows.eloc.as<cplx<double>>(),
              t.Obar.as<cplx<double>>(), t.F.as<cplx<double>>(), t.stats.as<Stats>(), nullptr, t.partial, st);
    mark(2, st);
    if(want_S) {
        const size_t nn = (size_t)psi.Np * psi.Np;
        if(t.s_mode == ANN_S_FP32 || psi.precision == 1) {
            t.S.ensure(nn * 16);
            t.S_in32 = false;
            herk_simt(t.O.p, psi.precision, rows, ld, psi.Np, tw, w0, t.Obar.as<cplx<double>>(),
                      t.stats.as<Stats>(), t.S.as<cplx<double>>(), st);
        } else {
            // FP32 sums: complex64 storage when the solver reads FP32
            t.S_in32 = t.solver != ANN_SOLVER_FP64;
            if(t.S_in32) t.S32.ensure(nn * 8);
            else t.S.ensure(nn * 16);
            herk_tc(t, tw, w0, t.s_mode == ANN_S_BF16_SPLIT, st);
        }
        t.S64_fresh = !t.S_in32;
        t.have_S = true;
    }
    mark(3, st);
}

}  // namespace ann

namespace {
void tdvp_eval_impl(ann_tdvp* t, ann_op* op, ann_psi* psi, ann_ens* ens, bool want_S, cudaStream_t st) {
    need(t && op && psi && ens, "null argument");
    const SampleTargets tg = tdvp_prepare(*t, *psi, *ens);
    mark(0, st);
    run_ensemble(*psi, op, *ens, tg, st);
    mark(1, st);
    tdvp_post(*t, *psi, *ens, want_S, st);
}
}  // namespace

extern "C" {

int ann_tdvp_eval(ann_tdvp* t, ann_op* op, ann_psi* psi, ann_ens* ens, void* stream) {
    return guard([&] { tdvp_eval_impl(t, op, psi, ens, true, S(stream)); });
}
int ann_tdvp_eval_F(ann_tdvp* t, ann_op* op, ann_psi* psi, ann_ens* ens, void* stream) {
    return guard([&] { tdvp_eval_impl(t, op, psi, ens, false, S(stream)); });
}

int ann_tdvp_get_S(ann_tdvp* t, double* out) {
    return guard([&] {
        need(t && out && t->have_S, "S not evaluated");
        ANN_CUDA(cudaDeviceSynchronize());
        check_status();
        const size_t nn = (size_t)t->Np * t->Np;
        if(t->S_in32 && !t->S64_fresh) {
            // complex64 values, widened exactly on the host
            std::vector<float> s32(2 * nn);
            ANN_CUDA(cudaMemcpy(s32.data(), t->S32.p, nn * 8, cudaMemcpyDeviceToHost));
            for(size_t k = 0; k < 2 * nn; k++) out[k] = (double)s32[k];
        } else {
            ANN_CUDA(cudaMemcpy(out, t->S.p, nn * 16, cudaMemcpyDeviceToHost));
        }
    });
}
int ann_tdvp_get_F(ann_tdvp* t, double* out) {
    return guard([&] {
        need(t && out && t->F.p, "F not evaluated");
        ANN_CUDA(cudaDeviceSynchronize());
        check_status();
        ANN_CUDA(cudaMemcpy(out, t->F.p, (size_t)t->Np * 16, cudaMemcpyDeviceToHost));
    });
}
int ann_tdvp_get_O(ann_tdvp* t, double* out) {
    return guard([&] {
        need(t && out && t->Obar.p, "O not evaluated");
        ANN_CUDA(cudaDeviceSynchronize());
        ANN_CUDA(cudaMemcpy(out, t->Obar.p, (size_t)t->Np * 16, cudaMemcpyDeviceToHost));
    });
}
int ann_tdvp_get_energy(ann_tdvp* t, double* E, double* E2) {
    return guard([&] {
        need(t && t->stats.p, "not evaluated");
        ANN_CUDA(cudaDeviceSynchronize());
        const Stats s = fetch_stats(t->stats, nullptr);
        if(E) { E[0] = s.E[0]; E[1] = s.E[1]; }
        if(E2) *E2 = s.E2;
    });
}
int ann_tdvp_get_total_weight(ann_tdvp* t, double* out) {
    return guard([&] {
        need(t && out && t->stats.p, "not evaluated");
        ANN_CUDA(cudaDeviceSynchronize());
        *out = fetch_stats(t->stats, nullptr).W;
    });
}
int ann_tdvp_get_O_samples(ann_tdvp* t, double* out) {
    return guard([&] {
        need(t && out && t->O.p, "not evaluated");
        ANN_CUDA(cudaDeviceSynchronize());
        const size_t es = t->O_precision ? 16 : 8;
        std::vector<unsigned char> buf(t->n_rows * t->ldO * es);
        ANN_CUDA(cudaMemcpy(buf.data(), t->O.p, buf.size(), cudaMemcpyDeviceToHost));
        for(size_t r = 0; r < t->n_rows; r++)
            for(size_t k = 0; k < t->Np; k++) {
                const size_t i = r * t->ldO + k;
                if(t->O_precision) {
                    std::memcpy(out + 2 * (r * t->Np + k), &buf[i * 16], 16);
                } else {
                    float f[2];
                    std::memcpy(f, &buf[i * 8], 8);
                    out[2 * (r * t->Np + k)] = f[0];
                    out[2 * (r * t->Np + k) + 1] = f[1];
                }
            }
    });
}
int ann_tdvp_S_dot_vector(ann_tdvp* t, const double* vec, void* stream, double* out) {
    return guard([&] {
        need(t && vec && out && t->O.p, "not evaluated");
        cudaStream_t st = S(stream);
        t->vec_in.ensure((size_t)t->Np * 16);
        t->vec_tmp.ensure(t->n_rows * 16);
        t->resid.ensure((size_t)t->Np * 16 * 2 + 16);
        ANN_CUDA(cudaMemcpyAsync(t->vec_in.p, vec, (size_t)t->Np * 16, cudaMemcpyHostToDevice, st));
        row_dot(t->O.p, t->O_precision, t->n_rows, t->ldO, t->Np, t->vec_in.as<cplx<double>>(),
                t->vec_tmp.as<cplx<double>>(), st);
        cplx<double>* res = t->resid.as<cplx<double>>();
        col_stats(t->O.p, t->O_precision, t->n_rows, t->ldO, t->Np, t->wts_exact ? t->wts.as<double>() : nullptr,
                  t->w0, t->vec_tmp.as<cplx<double>>(), nullptr, res, nullptr, nullptr, t->partial, st);
        finalize_sdotv(res, t->Obar.as<cplx<double>>(), t->vec_in.as<cplx<double>>(), t->Np, st);
        ANN_CUDA(cudaMemcpyAsync(out, res, (size_t)t->Np * 16, cudaMemcpyDeviceToHost, st));
        sync(st);
    });
}

int ann_tdvp_solve(ann_tdvp* t, double shift, void* stream, double* delta_out, double* info2) {
    return guard([&] {
        need(t && t->have_S, "S not evaluated");
        cudaStream_t st = S(stream);
        sr_solve_any(*t, shift, status_word(), st);
        if(delta_out) ANN_CUDA(cudaMemcpyAsync(delta_out, t->delta.p, (size_t)t->Np * 16, cudaMemcpyDeviceToHost, st));
        sync(st);
        check_status();
        if(info2) {
            double info[4];
            solver_info(*t, info, st);
            info2[0] = info[1];
            info2[1] = info[2];
        }
    });
}

int ann_tdvp_set_solver(ann_tdvp* t, int solver, unsigned max_iter, double tol) {
    return guard([&] {
        need(t, "null tdvp");
        need(solver == ANN_SOLVER_FP64 || solver == ANN_SOLVER_MIXED || solver == ANN_SOLVER_FP32,
             "unknown solver");
        need(max_iter >= 1 && max_iter <= 64, "max_iter must be in [1, 64]");
        need(tol > 0.0 && tol < 1.0, "tol must be in (0, 1)");
        t->solver = solver;
        t->ir_max = max_iter;
        t->ir_tol = tol;
    });
}

int ann_tdvp_set_chol_update(ann_tdvp* t, int mode) {
    return guard([&] {
        need(t, "null tdvp");
        need(mode == ANN_CHOL_UPDATE_SIMT || mode == ANN_CHOL_UPDATE_TC, "unknown Cholesky update mode");
        t->chol_tc = mode;
        t->chol_tc_set = true;
    });
}

int ann_tdvp_solver_info(ann_tdvp* t, double* out4) {
    return guard([&] {
        need(t && out4, "null argument");
        need(t->delta.p, "no solve yet");
        ANN_CUDA(cudaDeviceSynchronize());
        solver_info(*t, out4, nullptr);
    });
}

int ann_tdvp_solver_form(const ann_tdvp* t, int* form) {
    return guard([&] {
        need(t && form, "null argument");
        *form = t->solver == ANN_SOLVER_FP64 ? ANN_CHOL_FORM_NONE : t->chol_form;
    });
}

int ann_sr_update(ann_tdvp* t, ann_psi* psi, double lr, void* stream) {
    return guard([&] {
        need(t && psi && t->delta.p, "no solved delta");
        need(t->Np == psi->Np, "size mismatch");
        sr_update(*psi, t->delta.as<cplx<double>>(), lr, S(stream));
    });
}

int ann_sr_step(ann_tdvp* t, ann_op* op, ann_psi* psi, ann_ens* ens, double shift, double lr, void* stream) {
    return guard([&] {
        cudaStream_t st = S(stream);
        tdvp_eval_impl(t, op, psi, ens, true, st);
        sr_solve_any(*t, shift, status_word(), st);
        mark(4, st);
        sr_update(*psi, t->delta.as<cplx<double>>(), lr, st);
        mark(5, st);
    });
}

int ann_set_phase_timing(int enable) {
    return guard([&] {
        g_timing = enable != 0;
        for(auto& u : g_ev_used) u = false;
        for(auto& u : g_sev_used) u = false;
    });
}

int ann_get_solve_times(float* ms1) {
    return guard([&] {
        need(ms1, "null argument");
        ms1[0] = -1.f;
        if(g_sev_used[0] && g_sev_used[1]) {
            ANN_CUDA(cudaEventSynchronize(g_sev[1]));
            ANN_CUDA(cudaEventElapsedTime(&ms1[0], g_sev[0], g_sev[1]));
        }
    });
}

int ann_set_factor_trace(int enable) {
    return guard([&] {
        need(enable >= 0 && enable <= 2, "factor trace level 0, 1 or 2");
        g_ftrace = enable;
        g_fev_used = 0;
    });
}

int ann_get_factor_trace(double* out, unsigned cap, unsigned* n) {
    return guard([&] {
        need(n, "null argument");
        *n = (unsigned)g_fev_used;
        if(!g_fev_used || !out) return;
        ANN_CUDA(cudaEventSynchronize(g_fev[g_fev_used - 1].second));
        for(size_t k = 0; k < g_fev_used && k < cap; k++) {
            float ms = 0.f;
            ANN_CUDA(cudaEventSynchronize(g_fev[k].second));
            ANN_CUDA(cudaEventElapsedTime(&ms, g_fev[0].second, g_fev[k].second));
            out[2 * k] = g_fev[k].first;
            out[2 * k + 1] = ms;
        }
    });
}

int ann_get_phase_times(float* ms) {
    return guard([&] {
        need(ms, "null argument");
        for(int i = 0; i < kPhases; i++) {
            ms[i] = -1.f;
            if(g_ev_used[i] && g_ev_used[i + 1]) {
                ANN_CUDA(cudaEventSynchronize(g_ev[i + 1]));
                ANN_CUDA(cudaEventElapsedTime(&ms[i], g_ev[i], g_ev[i + 1]));
            }
        }
    });
}

int ann_sr_graph_capture(ann_tdvp* t, ann_op* op, ann_psi* psi, ann_ens* ens, double shift, double lr, void* stream) {
    return guard([&] {
        need(t && op && psi && ens, "null argument");
        need(stream != nullptr, "graph capture needs a non-default stream");
        need(ens->kind == 0 || ens->persistent, "graph replay needs persistent chains or exact summation");
        cudaStream_t st = S(stream);
        // one eager step sizes every buffer and validates the chains, so the
        // captured launches allocate nothing and bake in the steady-state arguments
        tdvp_eval_impl(t, op, psi, ens, true, st);
        sr_solve_any(*t, shift, status_word(), st);
        sr_update(*psi, t->delta.as<cplx<double>>(), lr, st);
        sync(st);
        if(t->graph_exec) { cudaGraphExecDestroy(t->graph_exec); t->graph_exec = nullptr; }
        if(t->graph) { cudaGraphDestroy(t->graph); t->graph = nullptr; }
        ANN_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        try {
            tdvp_eval_impl(t, op, psi, ens, true, st);
            sr_solve_any(*t, shift, status_word(), st);
            sr_update(*psi, t->delta.as<cplx<double>>(), lr, st);
        } catch(...) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(st, &g);
            if(g) cudaGraphDestroy(g);
            throw;
        }
        ANN_CUDA(cudaStreamEndCapture(st, &t->graph));
        ANN_CUDA(cudaGraphInstantiate(&t->graph_exec, t->graph, 0));
        size_t n_nodes = 0;
        ANN_CUDA(cudaGraphGetNodes(t->graph, nullptr, &n_nodes));
        std::vector<cudaGraphNode_t> nodes(n_nodes);
        ANN_CUDA(cudaGraphGetNodes(t->graph, nodes.data(), &n_nodes));
        unsigned kernels = 0;
        for(auto nd : nodes) {
            cudaGraphNodeType ty;
            ANN_CUDA(cudaGraphNodeGetType(nd, &ty));
            kernels += ty == cudaGraphNodeTypeKernel;
        }
        t->graph_kernels = kernels;
    });
}

int ann_sr_graph_launch(ann_tdvp* t, void* stream) {
    return guard([&] {
        need(t && t->graph_exec, "no captured graph");
        ANN_CUDA(cudaGraphLaunch(t->graph_exec, S(stream)));
        count_launch(t->graph_kernels);
    });
}

}  // extern "C"
