// Many Hamiltonian instances of uneven size in one persistent sampling launch.
//
// Each instance is a (PsiRBM/PsiDeep, Operator, MonteCarlo ensemble[, TDVP]) tuple.
// The sampling + local energy + O-row kernel runs once for all instances: a device
// work queue (one atomic counter) hands out items of eight chains of one instance,
// largest instances first; the CTA stages that instance's weights in shared memory and
// each warp runs one chain with the same per-chain code as the single-instance
// sampler (so a batched chain and the same chain sampled alone are identical). The
// per-instance reductions, S, FP64 Cholesky solve and update then run on a pool of
// streams; the whole step can be captured as one CUDA graph.
#include <algorithm>
#include <numeric>

#include "ann_internal.hpp"
#include "rbm_kernels.cuh"

namespace ann {

namespace {

constexpr int kBatchU = 8;       // register slots: hidden width up to 256
constexpr int kBatchWarps = 8;   // chains per work item
constexpr int kBatchStreams = 16;

struct BatchInst {
    RbmDev<float> p;
    OpDev op;
    McArgs a;
    SampleOut out;
    int with_op;
};

__global__ void __launch_bounds__(kBatchWarps * 32)
rbm_mc_batch_kernel(const BatchInst* __restrict__ insts, const uint2* __restrict__ items, unsigned n_items,
                    unsigned* __restrict__ next, size_t made_scratch_off) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ unsigned s_item;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for(;;) {
        if(threadIdx.x == 0) s_item = atomicAdd(next, 1u);
        __syncthreads();
        const unsigned it = s_item;
        if(it >= n_items) break;
        const uint2 w = items[it];
        const BatchInst& I = insts[w.x];
        const RbmDev<float> p = I.p;
        const cplx<float>* Wd = stage_Wd<float>(p, 1, reinterpret_cast<cplx<float>*>(smem_raw));
        const unsigned chain = w.y + warp;
        if(chain < I.a.n_chains) {
            // the instance's learned proposal (if any) read through L1; one H-float scratch
            // per warp after the largest instance's weights
            const bool use_made = I.a.made.N != 0 && (I.a.made_on == nullptr || *I.a.made_on != 0);
            const MadeSm ms = use_made ? made_global(I.a.made) : MadeSm{};
            float* mh = use_made ? reinterpret_cast<float*>(smem_raw + made_scratch_off) + warp * I.a.made.H : nullptr;
            mc_chain<float, 1, kBatchU>(p, Wd, I.op, I.with_op, I.a, I.out, chain, lane, use_made, ms, mh);
        }
        __syncthreads();  // before the next item restages the weights
    }
}

RbmDev<float> view_f32(const ann_psi_impl& psi) {
    RbmDev<float> p;
    p.N = psi.N;
    p.M = psi.M;
    p.Mpad = psi.Mpad;
    p.Uact = psi.Mpad / 32;
    p.C = psi.C;
    p.Np = psi.Np;
    p.layout = psi.layout;
    p.a_in_log_psi = psi.a_in;
    p.act = psi.act;
    p.Wd = psi.Wd.as<cplx<float>>();
    p.a = psi.a.as<cplx<float>>();
    p.b = psi.b.as<cplx<float>>();
    p.fw = psi.fwd.as<cplx<float>>();
    p.conn = psi.connd.as<uint16_t>();
    p.lp = mk<float>((float)psi.lp.real(), (float)psi.lp.imag());
    p.fw_real = 1;
    for(const zd& f : psi.fw)
        if(f.imag() != 0.0) p.fw_real = 0;
    return p;
}

}  // namespace

struct ann_batch_impl {
    std::vector<ann_psi*> psis;
    std::vector<ann_op*> ops;
    std::vector<ann_ens*> enss;
    std::vector<ann_tdvp*> tdvps;
    std::vector<BatchInst> host_insts;
    std::vector<uint2> host_items;
    DevBuf insts, items, counter;
    size_t smem = 0;
    size_t made_off = 0;   // byte offset of the per-warp learned-proposal scratch in shared memory
    bool table_valid = false;
    bool table_inits = false;  // the table draws fresh configurations (first call / non-persistent)
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> done;
    cudaEvent_t fork = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    unsigned graph_kernels = 0;
    ~ann_batch_impl() {
        if(exec) cudaGraphExecDestroy(exec);
        if(graph) cudaGraphDestroy(graph);
        for(auto s : streams) cudaStreamDestroy(s);
        for(auto e : done) cudaEventDestroy(e);
        if(fork) cudaEventDestroy(fork);
    }
};

namespace {

bool capturing(cudaStream_t st) {
    cudaStreamCaptureStatus cs;
    ANN_CUDA(cudaStreamIsCapturing(st, &cs));
    return cs != cudaStreamCaptureStatusNone;
}

// builds the per-instance table (McArgs like rbm_mc_T) and the work items
void batch_table(ann_batch_impl& b) {
    const size_t n = b.psis.size();
    b.table_inits = false;
    b.host_insts.assign(n, BatchInst{});
    std::vector<double> cost(n);
    size_t max_wd = 0;
    unsigned max_made_h = 0;
    for(size_t i = 0; i < n; i++) {
        ann_psi_impl& psi = *b.psis[i];
        ann_ens_impl& ens = *b.enss[i];
        BatchInst& I = b.host_insts[i];
        I.p = view_f32(psi);
        I.op = b.ops[i]->view();
        I.with_op = 1;
        McArgs& a = I.a;
        const unsigned spc = ens.num_samples / ens.n_chains;
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
        a.tape_site = nullptr;
        a.tape_u = nullptr;
        a.tape_len = 0;
        a.acc_rej = ens.acc_rej.as<unsigned long long>();
        a.made = MadeDev{};
        a.indep_per_sample = 0;
        a.made_on = nullptr;
        a.made_smem = 0;
        if(ens.made && ens.indep_per_sample > 0) {
            if(ens.made->N != psi.N) throw Error(ANN_ERR_INVALID, "learned proposal size differs from psi.N");
            if(ens.made->H > 256) throw Error(ANN_ERR_INVALID, "learned proposals in the sampler need H <= 256");
            a.made = made_view(*ens.made);
            a.indep_per_sample = ens.indep_per_sample;
            a.made_on = ens.made_on.as<int>();
            max_made_h = std::max(max_made_h, ens.made->H);
        }
        SampleTargets tg{&ens.rows, nullptr, 0, true};
        if(b.tdvps[i]) tg = tdvp_prepare(*b.tdvps[i], psi, ens);
        const size_t rows = (size_t)spc * ens.n_chains;
        ens.rows.n = rows;
        ens.rows.conf.ensure(rows * kMaxWords * sizeof(uint64_t));
        ens.rows.log_psi.ensure(rows * sizeof(cplx<double>));
        ens.rows.eloc.ensure(rows * sizeof(cplx<double>));
        ens.rows.weight.ensure(rows * sizeof(double));
        SampleOut& o = I.out;
        o.conf = ens.rows.conf.as<uint64_t>();
        o.log_psi = ens.rows.log_psi.as<cplx<double>>();
        o.eloc = ens.rows.eloc.as<cplx<double>>();
        o.weight = ens.rows.weight.as<double>();
        o.O = tg.O;
        o.ldO = tg.ldO;
        o.status = status_word();
        max_wd = std::max(max_wd, (size_t)psi.N * psi.Mpad * sizeof(cplx<float>));
        cost[i] = (double)ens.n_chains * (ens.num_sweeps + (a.do_init ? ens.num_therm : 0) + a.indep_per_sample) *
                  psi.N * psi.M;
        b.table_inits = b.table_inits || a.do_init;
    }
    std::vector<size_t> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](size_t x, size_t y) { return cost[x] > cost[y]; });
    b.host_items.clear();
    for(size_t i : order)
        for(unsigned c = 0; c < b.enss[i]->n_chains; c += kBatchWarps) b.host_items.push_back(uint2{(unsigned)i, c});
    upload(b.insts, b.host_insts.data(), b.host_insts.size() * sizeof(BatchInst));
    upload(b.items, b.host_items.data(), b.host_items.size() * sizeof(uint2));
    b.counter.ensure(sizeof(unsigned));
    b.made_off = (max_wd + 15) & ~(size_t)15;
    b.smem = b.made_off + (size_t)kBatchWarps * max_made_h * sizeof(float);
    if(b.smem > 200 * 1024) throw Error(ANN_ERR_INVALID, "instance weights exceed shared memory");
    ANN_CUDA(cudaFuncSetAttribute(rbm_mc_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)std::max<size_t>(b.smem, 1024)));
    b.table_valid = true;
}

void batch_sample(ann_batch_impl& b, cudaStream_t st) {
    if(!capturing(st)) {
        // arguments change only while chains are being (re)initialised
        bool stale = !b.table_valid;
        for(auto* e : b.enss) stale = stale || !e->persistent || !e->chains_valid;
        if(stale) batch_table(b);
    } else if(!b.table_valid) {
        throw Error(ANN_ERR_INVALID, "run one batched step before capturing it");
    }
    for(auto* e : b.enss) ANN_CUDA(cudaMemsetAsync(e->acc_rej.p, 0, 4 * sizeof(unsigned long long), st));
    ANN_CUDA(cudaMemsetAsync(b.counter.p, 0, sizeof(unsigned), st));
    int sms = 152;
    int dev = 0;
    ANN_CUDA(cudaGetDevice(&dev));
    ANN_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const unsigned n_items = (unsigned)b.host_items.size();
    const unsigned grid = std::min<unsigned>(n_items, (unsigned)sms * 2);
    rbm_mc_batch_kernel<<<grid, kBatchWarps * 32, std::max<size_t>(b.smem, 16), st>>>(
        b.insts.as<BatchInst>(), b.items.as<uint2>(), n_items, b.counter.as<unsigned>(), b.made_off);
    check_launch("rbm_mc_batch_kernel");
    for(size_t i = 0; i < b.enss.size(); i++) {
        ann_ens_impl& e = *b.enss[i];
        if(e.made && e.indep_per_sample > 0) {
            made_drop_rule_kernel<<<1, 1, 0, st>>>(e.acc_rej.as<unsigned long long>(), e.made_min_acceptance,
                                                   e.made_on.as<int>());
            check_launch("made_drop_rule_kernel");
        }
        if(e.hist_cap) hist_append(e, e.rows.conf.as<uint64_t>(), e.rows.n, st);  // the proposal's training data
    }
    for(auto* e : b.enss) e->chains_valid = true;
    if(b.table_inits && !capturing(st)) b.table_valid = false;  // next call continues the chains
}

void batch_streams(ann_batch_impl& b) {
    if(!b.streams.empty()) return;
    for(int k = 0; k < kBatchStreams; k++) {
        cudaStream_t s;
        cudaEvent_t e;
        ANN_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        ANN_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        b.streams.push_back(s);
        b.done.push_back(e);
    }
    ANN_CUDA(cudaEventCreateWithFlags(&b.fork, cudaEventDisableTiming));
}

// per-instance reductions, S, solve and update, spread over the stream pool
void batch_sr(ann_batch_impl& b, double shift, double lr, cudaStream_t st) {
    batch_streams(b);
    ANN_CUDA(cudaEventRecord(b.fork, st));
    for(auto s : b.streams) ANN_CUDA(cudaStreamWaitEvent(s, b.fork, 0));
    // longest first onto the least-loaded stream; the estimated cost (us) of an instance
    // is its solve: a latency-bound chain of Np / 64 panels plus the (4/3) Np^3 update
    // work, and the S product over its rows
    const size_t n = b.psis.size();
    std::vector<size_t> order(n);
    std::vector<double> cost(n), load(b.streams.size(), 0.0);
    for(size_t i = 0; i < n; i++) {
        const double np = b.psis[i]->Np, ns = (double)b.enss[i]->num_steps();
        cost[i] = np / 64.0 * 40.0 + (4.0 / 3.0) * np * np * np / 5e7 + 4.0 * np * np * ns / 1e9;
        order[i] = i;
    }
    std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) { return cost[x] > cost[y]; });
    for(size_t i : order) {
        const size_t k = (size_t)(std::min_element(load.begin(), load.end()) - load.begin());
        load[k] += cost[i];
        cudaStream_t s = b.streams[k];
        ann_tdvp_impl& t = *b.tdvps[i];
        tdvp_post(t, *b.psis[i], *b.enss[i], true, s);
        sr_solve_any(t, shift, status_word(), s);
        sr_update(*b.psis[i], t.delta.as<cplx<double>>(), lr, s);
    }
    for(size_t k = 0; k < b.streams.size(); k++) {
        ANN_CUDA(cudaEventRecord(b.done[k], b.streams[k]));
        ANN_CUDA(cudaStreamWaitEvent(st, b.done[k], 0));
    }
}

template<typename F>
int bguard(F&& f) {
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

void bneed(bool ok, const char* msg) {
    if(!ok) throw Error(ANN_ERR_INVALID, msg);
}

}  // namespace

}  // namespace ann

struct ann_batch : ann::ann_batch_impl {};

using namespace ann;

extern "C" {

int ann_batch_create(unsigned n, ann_psi** psis, ann_op** ops, ann_ens** enss, ann_tdvp** tdvps, ann_batch** out) {
    return bguard([&] {
        bneed(out && psis && ops && enss && n > 0, "null argument");
        auto* b = new ann_batch();
        try {
            for(unsigned i = 0; i < n; i++) {
                bneed(psis[i] && ops[i] && enss[i], "null instance member");
                const ann_psi_impl& p = *psis[i];
                bneed(p.kind == 0 && p.precision == 0 && p.NW == 1 && p.U <= kBatchU,
                      "batched instances are complex64 RBM-family wavefunctions with N <= 64, M <= 256");
                bneed(enss[i]->kind == 1 && enss[i]->move == 0 && enss[i]->tape_len == 0,
                      "batched instances use single-flip Monte Carlo ensembles");
                bneed(ops[i]->max_site <= p.N, "operator acts beyond the wavefunction");
                if(tdvps && tdvps[i]) bneed(tdvps[i]->Np == p.Np, "TDVP size differs from psi");
                b->psis.push_back(psis[i]);
                b->ops.push_back(ops[i]);
                b->enss.push_back(enss[i]);
                b->tdvps.push_back(tdvps ? tdvps[i] : nullptr);
            }
        } catch(...) {
            delete b;
            throw;
        }
        *out = b;
    });
}

int ann_batch_destroy(ann_batch* b) {
    return bguard([&] { delete b; });
}

int ann_batch_sample(ann_batch* b, void* stream) {
    return bguard([&] {
        bneed(b != nullptr, "null argument");
        batch_sample(*b, reinterpret_cast<cudaStream_t>(stream));
    });
}

int ann_batch_energies(ann_batch* b, double* out) {
    return bguard([&] {
        bneed(b && out, "null argument");
        ANN_CUDA(cudaDeviceSynchronize());
        DevBuf stats;
        stats.ensure(sizeof(Stats));
        DevBuf scratch;
        for(size_t i = 0; i < b->psis.size(); i++) {
            ann_ens_impl& e = *b->enss[i];
            row_stats(e.rows, nullptr, e.uniform_weight(), stats.as<Stats>(), scratch, nullptr);
            Stats s;
            ANN_CUDA(cudaMemcpy(&s, stats.p, sizeof(Stats), cudaMemcpyDeviceToHost));
            out[2 * i] = s.E[0];
            out[2 * i + 1] = s.E[1];
        }
    });
}

int ann_batch_sr_step(ann_batch* b, double shift, double lr, void* stream) {
    return bguard([&] {
        bneed(b != nullptr, "null argument");
        for(auto* t : b->tdvps) bneed(t != nullptr, "SR steps need a TDVP per instance");
        cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
        batch_sample(*b, st);
        batch_sr(*b, shift, lr, st);
    });
}

int ann_batch_graph_capture(ann_batch* b, double shift, double lr, void* stream) {
    return bguard([&] {
        bneed(b != nullptr && stream != nullptr, "graph capture needs a batch and a non-default stream");
        for(auto* e : b->enss) bneed(e->persistent, "graph replay needs persistent chains");
        for(auto* t : b->tdvps) bneed(t != nullptr, "SR steps need a TDVP per instance");
        cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
        batch_sample(*b, st);  // eager step: sizes every buffer, validates the chains
        batch_sr(*b, shift, lr, st);
        ANN_CUDA(cudaStreamSynchronize(st));
        batch_table(*b);  // steady-state arguments (no initialisation)
        if(b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
        if(b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
        ANN_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        try {
            batch_sample(*b, st);
            batch_sr(*b, shift, lr, st);
        } catch(...) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(st, &g);
            if(g) cudaGraphDestroy(g);
            throw;
        }
        ANN_CUDA(cudaStreamEndCapture(st, &b->graph));
        ANN_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
        size_t n_nodes = 0;
        ANN_CUDA(cudaGraphGetNodes(b->graph, nullptr, &n_nodes));
        std::vector<cudaGraphNode_t> nodes(n_nodes);
        ANN_CUDA(cudaGraphGetNodes(b->graph, nodes.data(), &n_nodes));
        unsigned k = 0;
        for(auto nd : nodes) {
            cudaGraphNodeType ty;
            ANN_CUDA(cudaGraphNodeGetType(nd, &ty));
            k += ty == cudaGraphNodeTypeKernel;
        }
        b->graph_kernels = k;
    });
}

int ann_batch_graph_launch(ann_batch* b, void* stream) {
    return bguard([&] {
        bneed(b && b->exec, "no captured graph");
        ANN_CUDA(cudaGraphLaunch(b->exec, reinterpret_cast<cudaStream_t>(stream)));
        count_launch(b->graph_kernels);
    });
}

}  // extern "C"
