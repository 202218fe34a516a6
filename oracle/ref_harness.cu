// Harness around the reference implementation's own CPU (host) code path.
//
// TEST INFRASTRUCTURE ONLY. Built by oracle/Makefile into oracle/_ref/ from the
// reference sources where they lie (never copied into this repository); used
// only to generate the golden fixtures under tests/golden/ and to pin the FP64
// restatement in oracle/oracle.cpp. Nothing in the product links or loads it.
//
// Every computation below runs the reference's templates with gpu=false:
//   * Operator / PauliString::apply / local_energy  include/operator/Operator.hpp:36-121
//   * PsiDeep (1 hidden layer, ENABLE_NETWORK_BASES) include/quantum_state/PsiDeep.hpp:138-445
//   * PsiDeep (several hidden layers)                the same kernel, layers assembled as
//                                                    the Python constructor does (PsiDeep.hpp:488-560)
//   * PsiRBM kernel                                 include/quantum_state/PsiRBM.hpp:69-176
//   * PsiCNN kernel                                 include/quantum_state/PsiCNN.hpp:97-266
//   * MonteCarlo_t::kernel_foreach / mc_update       include/ensembles/MonteCarlo.hpp:55-177
//   * ExactSummation_t::kernel_foreach               include/ensembles/ExactSummation.hpp:33-72
//   * PsiClassical kernel (order 1 with the fully polarized reference, order 2 with a
//     PsiDeep reference)                            include/quantum_state/PsiClassical.hpp:48-163
//   * KullbackLeibler value / gradient / gradient_with_noise
//                                                   source/network_functions/KullbackLeibler.cu.template
//   * HilbertSpaceDistance distance / gradient       source/network_functions/HilbertSpaceDistance.cu.template
//   * ExpectationValue / TDVP / PsiVector / PsiOkVector / PsiNorm bodies
//     (source/network_functions/*.cu.template, with the "//! begin template"
//     instantiation blocks stripped at build time by oracle/Makefile).
// The only harness-side logic is construction (the reference's constructors for
// these types exist only behind its Python binding) and a logging update policy
// that records every Metropolis proposal.

#include "bases.hpp"
#include "operators.hpp"
#include "quantum_states.hpp"
#include "ensembles.hpp"
#include "network_functions/ExpectationValue.hpp"
#include "network_functions/TDVP.hpp"
#include "network_functions/PsiVector.hpp"
#include "network_functions/PsiNorm.hpp"
#include "network_functions/PsiOkVector.hpp"
#include "network_functions/KullbackLeibler.hpp"
#include "network_functions/HilbertSpaceDistance.hpp"

#include <vector>
#include <cstdint>
#include <cstring>
#include <set>

namespace ann_on_gpu {

// A Pauli-sum expression as the three arrays that cross the reference's
// Operator constructor (source/operator/Operator.cpp:26-36).
struct HarnessExpr {
    const uint64_t* a;
    const uint64_t* b;
    const double* coeff;  // interleaved re, im
    unsigned int n;
};

template<>
template<>
StandartOperator<PauliString>::StandartOperator(const HarnessExpr& expr, const bool gpu)
    : gpu(gpu), coefficients(expr.n, gpu), quantum_strings(expr.n, gpu) {
    for(auto i = 0u; i < expr.n; i++) {
        this->coefficients[i] = complex_t(expr.coeff[2 * i], expr.coeff[2 * i + 1]);
        this->quantum_strings[i] = PauliString(expr.a[i], expr.b[i]);
    }
    this->kernel().num_strings = expr.n;
    this->kernel().coefficients = this->coefficients.data();
    this->kernel().quantum_strings = this->quantum_strings.data();
}

// PsiRBM: the reference's host constructor exists only under __PYTHONCC__
// (PsiRBM.hpp:225-243); this shim fills the same kernel fields.
struct HarnessRBM : public kernel::PsiRBM_t<complex_t, false> {
    using Kernel = kernel::PsiRBM_t<complex_t, false>;
    Array<complex_t> W_store;
    bool gpu;

    HarnessRBM(unsigned N_, unsigned M_, const double* W, const double* fw, const double* lp)
        : W_store(N_ * M_, false), gpu(false) {
        this->N = N_; this->num_sites = N_; this->M = M_; this->num_params = N_ * M_;
        for(auto k = 0u; k < N_ * M_; k++) this->W_store[k] = complex_t(W[2 * k], W[2 * k + 1]);
        this->final_weight = complex_t(fw[0], fw[1]);
        this->log_prefactor = complex_t(lp[0], lp[1]);
        this->kernel().W = this->W_store.data();
    }
    HarnessRBM(const HarnessRBM& o) : Kernel(o), W_store(o.W_store), gpu(false) {
        this->kernel().W = this->W_store.data();
    }
    Kernel& kernel() { return *this; }
    const Kernel& kernel() const { return *this; }
};

// PsiCNN: same situation (PsiCNN.hpp:347-373 is __PYTHONCC__-only); the layout
// assignment mirrors PsiCNN_t::init_kernel (source/quantum_state/PsiCNN.cpp:9-55).
struct HarnessCNN : public kernel::PsiCNN_t<3u, complex_t> {
    using Kernel = kernel::PsiCNN_t<3u, complex_t>;
    Array<complex_t> params;
    Array<complex_t> angles;
    bool gpu;
    unsigned extent_[3];
    std::vector<unsigned> channels_, connectivity_, classes_;

    HarnessCNN(const unsigned* extent, unsigned num_layers, const unsigned* num_channels,
               const unsigned* connectivity, const unsigned* sym_classes,
               const double* p, unsigned num_params_, double final_factor_, const double* lp)
        : params(num_params_, false), angles(false), gpu(false) {
        for(int d = 0; d < 3; d++) extent_[d] = extent[d];
        unsigned N_ = extent[0] * extent[1] * extent[2];
        channels_.assign(num_channels, num_channels + num_layers);
        connectivity_.assign(connectivity, connectivity + 3 * num_layers);
        classes_.assign(sym_classes, sym_classes + N_);
        for(auto k = 0u; k < num_params_; k++) this->params[k] = complex_t(p[2 * k], p[2 * k + 1]);
        this->N = N_; this->num_sites = N_;
        this->final_factor = final_factor_;
        this->log_prefactor = complex_t(lp[0], lp[1]);
        this->num_symmetry_classes = std::set<unsigned>(classes_.begin(), classes_.end()).size();
        this->init();
    }
    HarnessCNN(const HarnessCNN& o)
        : Kernel(o), params(o.params), angles(o.angles), gpu(false),
          channels_(o.channels_), connectivity_(o.connectivity_), classes_(o.classes_) {
        for(int d = 0; d < 3; d++) extent_[d] = o.extent_[d];
        this->init();
    }
    void init() {
        this->num_layers = channels_.size();
        this->num_params = this->params.size();
        this->num_angles = 0u;
        unsigned off = 0u;
        for(int d = 0; d < 3; d++) this->convolve.extent[d] = extent_[d];
        for(auto i = 0u; i < this->N; i++) this->convolve.symmetry_classes[i] = classes_[i];
        for(auto l = 0u; l < this->num_layers; l++) {
            auto& layer = this->layers[l];
            layer.num_channels = channels_[l];
            layer.num_channel_links = layer.num_channels * (l > 0 ? this->layers[l - 1].num_channels : 1u);
            layer.connectivity_vol = 1u;
            for(int d = 0; d < 3; d++) {
                layer.connectivity[d] = connectivity_[3 * l + d];
                layer.connectivity_vol *= layer.connectivity[d];
            }
            for(auto cl = 0u; cl < layer.num_channel_links; cl++) {
                layer.channel_links[cl].begin_params = off;
                layer.channel_links[cl].weights = this->params.data() + off;
                off += this->num_symmetry_classes * layer.connectivity_vol;
            }
            this->num_angles += layer.num_channels * this->N;
        }
        if(this->angles.size() < this->num_angles) this->angles.resize(this->num_angles);
        unsigned aoff = 0u;
        for(auto l = 0u; l < this->num_layers; l++)
            for(auto c = 0u; c < this->layers[l].num_channels; c++) {
                this->layers[l].channels[c].angles = this->angles.data() + aoff;
                aoff += this->N;
            }
    }
    void init_gradient(unsigned num_steps) {
        this->angles.resize(num_steps * this->num_angles);
        unsigned aoff = 0u;
        for(auto l = 0u; l < this->num_layers; l++)
            for(auto c = 0u; c < this->layers[l].num_channels; c++) {
                this->layers[l].channels[c].angles = this->angles.data() + aoff;
                aoff += this->N;
            }
    }
    Kernel& kernel() { return *this; }
    const Kernel& kernel() const { return *this; }
};

// Update policy that defers to the reference's single-flip policy
// (include/ensembles/policies/Update_Policy.hpp:20-33) and logs each
// proposal: the configuration it starts from and the flipped site.
std::vector<uint64_t> g_log_conf;
std::vector<uint32_t> g_log_site;

struct LoggingPolicyKernel {
    template<typename Psi_t>
    HDINLINE void operator()(Spins& next_spins, const Spins& spins, const Psi_t& psi, void* rng_state) const {
        const auto site = random_uint32(rng_state) % psi.num_sites;
        next_spins = spins.flip(site);
#ifndef __CUDA_ARCH__
        g_log_conf.push_back(spins.configuration());
        g_log_site.push_back(site);
#endif
    }
    LoggingPolicyKernel& kernel() { return *this; }
};
struct LoggingPolicy : public LoggingPolicyKernel {
    using kernel_t = LoggingPolicyKernel;
};

}  // namespace ann_on_gpu

// Reference bodies (stripped of their explicit-instantiation blocks).
#include "ExpectationValue.cu"
#include "TDVP.cu"
#include "PsiVector.cu"
#include "PsiNorm.cu"
#include "PsiOkVector.cu"
#include "ensembles/MonteCarlo.cu"
#include "KullbackLeibler.cu"
#include "HilbertSpaceDistance.cu"

using namespace ann_on_gpu;

using LoggingMC = MonteCarlo_t<Spins, Init_Policy<Spins>, LoggingPolicy>;

namespace {

struct DeepDesc {
    unsigned N, M, C;
    const unsigned* conn;     // C x M, entry (i, j) at i*M + j; may be null (identity, C == N)
    const double* params;     // [a(N) | b(M) | W(C*M)] interleaved complex
    const double* final_w;    // M complex
    const double* log_pref;   // 1 complex
};

PsiDeep make_deep(const DeepDesc& d) {
    PsiDeep psi(d.N, d.M, false);
    auto& layer0 = *psi.layers.begin();
    auto& layer1 = *std::next(psi.layers.begin());
    if(d.C != d.N) {
        layer1.lhs_connectivity = d.C;
        layer1.lhs_connections.resize(d.C * d.M);
        layer1.lhs_weights.resize(d.C * d.M);
    }
    if(d.conn) {
        for(auto k = 0u; k < d.C * d.M; k++) layer1.lhs_connections[k] = d.conn[k];
    }
    // the input layer's rhs (site -> hidden unit) lists follow the connections
    // (PsiDeep.cu:213-242); set_params only refreshes their weights.
    auto rhs = psi.compile_rhs_connections_and_weights(d.N, d.M, d.C, layer1.lhs_connections, layer1.lhs_weights);
    layer0.rhs_connections = std::move(rhs.first);
    layer0.rhs_weights = std::move(rhs.second);
    psi.init_kernel();
    const auto np = d.N + d.M + d.C * d.M;
    Array<complex_t> p(np, false);
    for(auto k = 0u; k < np; k++) p[k] = complex_t(d.params[2 * k], d.params[2 * k + 1]);
    for(auto j = 0u; j < d.M; j++) psi.final_weights[j] = complex_t(d.final_w[2 * j], d.final_w[2 * j + 1]);
    psi.log_prefactor = complex_t(d.log_pref[0], d.log_pref[1]);
    psi.set_params(p);
    return psi;
}

// Several hidden layers: the reference's multi-layer constructor is __PYTHONCC__-only
// (PsiDeep.hpp:488-560); this assembles the same layer list (input layer first, each
// layer's rhs lists compiled from the next layer's connections) and lets the
// reference's init_kernel / set_params fill offsets and weights.
struct DeepMLDesc {
    unsigned N, L;                 // N input units (3 per site for the Pauli-string basis)
    const unsigned* sizes;         // L
    const unsigned* connectivity;  // L
    const unsigned* conn;          // concatenated C_l x sizes[l] blocks
    const double* params;          // [a | b_0 | W_0 | ...] interleaved complex
    const double* final_w;         // sizes[L-1] complex
    const double* log_pref;
    unsigned num_sites = 0;        // 0: N
};

PsiDeep make_deep_ml(const DeepMLDesc& d) {
    PsiDeep psi(d.N, d.sizes[0], false);
    psi.layers.clear();
    psi.num_layers = d.L + 1u;
    psi.width = d.N;
    psi.num_units = 0u;
    std::vector<unsigned> coff(d.L, 0u);
    for(auto l = 1u; l < d.L; l++) coff[l] = coff[l - 1] + d.connectivity[l - 1] * d.sizes[l - 1];
    Array<unsigned int> rhs_c(0, false);
    Array<complex_t> rhs_w(0, false);
    for(int l = int(d.L) - 1; l >= 0; l--) {
        const unsigned size = d.sizes[l], C = d.connectivity[l];
        Array<unsigned int> lc(C * size, false);
        Array<complex_t> lw(C * size, false), bs(size, false);
        for(auto k = 0u; k < C * size; k++) {
            lc[k] = d.conn[coff[l] + k];
            lw[k] = complex_t(0.0, 0.0);
        }
        for(auto j = 0u; j < size; j++) bs[j] = complex_t(0.0, 0.0);
        if(size > psi.width) psi.width = size;
        psi.num_units += size;
        auto rhs = psi.compile_rhs_connections_and_weights(l > 0 ? d.sizes[l - 1] : d.N, size, C, lc, lw);
        psi.layers.push_front({size, C, std::move(lc), std::move(rhs_c), std::move(lw), std::move(rhs_w),
                               std::move(bs)});
        rhs_c = std::move(rhs.first);
        rhs_w = std::move(rhs.second);
    }
    psi.layers.push_front({d.N, 0u, Array<unsigned int>(1, false), std::move(rhs_c), Array<complex_t>(1, false),
                           std::move(rhs_w), Array<complex_t>(1, false)});
    const unsigned last = d.sizes[d.L - 1];
    psi.final_weights.resize(last);
    for(auto j = 0u; j < last; j++) psi.final_weights[j] = complex_t(d.final_w[2 * j], d.final_w[2 * j + 1]);
    psi.log_prefactor = complex_t(d.log_pref[0], d.log_pref[1]);
    psi.init_kernel();
    if(d.num_sites) psi.num_sites = d.num_sites;
    Array<complex_t> p(psi.num_params, false);
    for(auto k = 0u; k < psi.num_params; k++) p[k] = complex_t(d.params[2 * k], d.params[2 * k + 1]);
    psi.set_params(p);
    return psi;
}

// PsiClassical: the host constructor is __PYTHONCC__-only (PsiClassical.hpp:199-222); this
// shim fills the kernel fields as PsiClassical_t::init_kernel does (PsiClassical.cu:13-33),
// with one operator per feature built from HarnessExpr.
using OpKernel = kernel::StandartOperator<PauliString>;

template<unsigned order, typename RefKernel>
struct HarnessClassical : public kernel::PsiClassical_t<complex_t, OpKernel, order, false, RefKernel> {
    using Kernel = kernel::PsiClassical_t<complex_t, OpKernel, order, false, RefKernel>;
    std::vector<Operator> ops;
    Array<OpKernel> ops_kernel;
    Array<complex_t> prm;
    bool gpu;

    HarnessClassical(unsigned num_sites, const std::vector<HarnessExpr>& feats, const double* params,
                     const double* lp, const RefKernel& ref, unsigned ref_params)
        : ops_kernel(feats.size(), false), prm(feats.size(), false), gpu(false) {
        ops.reserve(feats.size());
        for(const auto& f : feats) ops.emplace_back(f, false);
        for(auto k = 0u; k < feats.size(); k++) {
            ops_kernel[k] = ops[k].kernel();
            prm[k] = complex_t(params[2 * k], params[2 * k + 1]);
        }
        this->params = prm.data();
        this->num_ops_H = feats.size();
        this->H_local = ops_kernel.data();
        this->num_sites = num_sites;
        this->log_prefactor = complex_t(lp[0], lp[1]);
        this->psi_ref = ref;
        this->num_params = feats.size() + (order > 1u ? ref_params : 0u);
    }
    HarnessClassical(const HarnessClassical& o)
        : Kernel(o), ops(), ops_kernel(o.ops_kernel.size(), false), prm(o.prm), gpu(false) {
        ops.reserve(o.ops.size());
        for(const auto& op : o.ops) ops.push_back(op);
        for(auto k = 0u; k < ops.size(); k++) ops_kernel[k] = ops[k].kernel();
        this->params = prm.data();
        this->H_local = ops_kernel.data();
    }
    Kernel& kernel() { return *this; }
    const Kernel& kernel() const { return *this; }
};

// a classical network: features (strings grouped per feature), parameters, order and an
// optional PsiDeep reference (order 2)
struct ClassicalDesc {
    unsigned num_sites, n_features;
    const unsigned* feat_begin;    // n_features + 1
    const uint64_t* a;             // strings (one word each)
    const uint64_t* b;
    const double* coeff;
    const double* params;          // n_features complex
    const double* log_pref;
    unsigned order;
    const DeepMLDesc* ref;         // order 2 (may be null: fully polarized)
};

std::vector<HarnessExpr> features_of(const ClassicalDesc& d) {
    std::vector<HarnessExpr> f;
    for(auto k = 0u; k < d.n_features; k++) {
        const unsigned b0 = d.feat_begin[k], b1 = d.feat_begin[k + 1];
        f.push_back(HarnessExpr{d.a + b0, d.b + b0, d.coeff + 2 * b0, b1 - b0});
    }
    return f;
}

kernel::PsiFullyPolarized_t<complex_t> fully_polarized(unsigned num_sites) {
    kernel::PsiFullyPolarized_t<complex_t> r;
    r.num_sites = num_sites;
    r.num_params = 0u;
    r.log_prefactor = complex_t(0.0, 0.0);
    r.gpu = false;
    return r;
}

void put(double* out, const complex_t& z) { out[0] = z.real(); out[1] = z.imag(); }
void put(double* out, const std::complex<double>& z) { out[0] = z.real(); out[1] = z.imag(); }

template<typename Psi>
void psi_log_psi_s(Psi& psi, uint64_t conf, double* out) {
    put(out, log_psi_s(psi, Spins(conf, psi.num_sites)));
}

template<typename Psi>
void psi_O_k(Psi& psi, uint64_t conf, double* out) {
    auto r = ann_on_gpu::psi_O_k(psi, Spins(conf, psi.num_sites));
    for(auto k = 0u; k < r.size(); k++) put(out + 2 * k, r[k]);
}

// Exact-summation quantities: <A> (unnormalised weights), fluctuation, gradient,
// TDVP E/E2/O/F/S, psi vector, norm, <log psi>.
template<typename Psi, typename Exact = ExactSummationSpins>
void exact_all(Psi& psi, const HarnessExpr& expr, double* E, double* fluct, double* grad,
               double* tdvp_E, double* tdvp_E2, double* tdvp_O, double* tdvp_F, double* tdvp_S,
               double* vec, double* norm, double* mean_log_psi, double* O_sum) {
    Operator op(expr, false);
    Exact es(psi.num_sites, false);
    ExpectationValue ev(false);
    put(E, ev(op, psi, es));
    auto fl = ev.fluctuation(op, psi, es);
    fluct[0] = fl.first; put(fluct + 1, fl.second);
    auto g = ev.gradient(op, psi, es);
    for(auto k = 0u; k < psi.num_params; k++) put(grad + 2 * k, g.first[k]);
    TDVP tdvp(psi.num_params, false);
    tdvp.eval(op, psi, es, false_t());
    put(tdvp_E, tdvp.E_local.front());
    tdvp_E2[0] = tdvp.E2_local.front();
    for(auto k = 0u; k < psi.num_params; k++) {
        put(tdvp_O + 2 * k, tdvp.O_k_ar[k]);
        put(tdvp_F + 2 * k, tdvp.F_vector[k]);
    }
    for(auto k = 0u; k < psi.num_params * psi.num_params; k++) put(tdvp_S + 2 * k, tdvp.S_matrix[k]);
    auto v = psi_vector(psi, es);
    for(auto k = 0u; k < v.size(); k++) put(vec + 2 * k, v[k]);
    norm[0] = psi_norm(psi, es);
    put(mean_log_psi, log_psi(psi, es));
    auto os = psi_O_k_vector(psi, es);
    for(auto k = 0u; k < os.size(); k++) put(O_sum + 2 * k, os[k]);
}

// One Markov chain on the host path (the host path always runs chain 0,
// MonteCarlo.hpp:69-71), recording every sample the functor sees and every
// proposal the update policy makes.
template<typename Psi>
unsigned mc_trace(Psi& psi, const HarnessExpr& expr, unsigned num_samples, unsigned num_sweeps,
                  unsigned num_therm, uint64_t* sample_conf, double* sample_log_psi, double* sample_eloc,
                  uint64_t* prop_conf, uint32_t* prop_site, unsigned max_props, double* mc_energy) {
    Operator op(expr, false);
    auto op_kernel = op.kernel();
    auto psi_kernel = psi.kernel();
    LoggingMC mc(num_samples, num_sweeps, num_therm, 1u, LoggingPolicy(), false);
    g_log_conf.clear();
    g_log_site.clear();
    mc.foreach(psi, [=] __host__ __device__ (const unsigned index, const Spins& conf, const complex_t& lp,
                        typename Psi::Payload& payload, const double) {
        complex_t eloc;
        op_kernel.local_energy(eloc, psi_kernel, conf, lp, payload);
        sample_conf[index] = conf.configuration();
        sample_log_psi[2 * index] = lp.real();
        sample_log_psi[2 * index + 1] = lp.imag();
        sample_eloc[2 * index] = eloc.real();
        sample_eloc[2 * index + 1] = eloc.imag();
    });
    const unsigned n = g_log_site.size();
    for(auto i = 0u; i < n && i < max_props; i++) {
        prop_conf[i] = g_log_conf[i];
        prop_site[i] = g_log_site[i];
    }
    // ExpectationValue through the reference's own MonteCarloSpins (1 chain).
    MonteCarloSpins mcs(num_samples, num_sweeps, num_therm, 1u, Update_Policy<Spins>(), false);
    ExpectationValue ev(false);
    put(mc_energy, ev(op, psi, mcs));
    return n;
}

}  // namespace

extern "C" {

// ---- PsiDeep (1 hidden layer) ----
void ref_deep_log_psi_s(unsigned N, unsigned M, unsigned C, const unsigned* conn, const double* params,
                        const double* fw, const double* lp, uint64_t conf, double* out) {
    auto psi = make_deep({N, M, C, conn, params, fw, lp});
    psi_log_psi_s(psi, conf, out);
}
void ref_deep_O_k(unsigned N, unsigned M, unsigned C, const unsigned* conn, const double* params,
                  const double* fw, const double* lp, uint64_t conf, double* out) {
    auto psi = make_deep({N, M, C, conn, params, fw, lp});
    psi_O_k(psi, conf, out);
}
void ref_deep_exact(unsigned N, unsigned M, unsigned C, const unsigned* conn, const double* params,
                    const double* fw, const double* lp,
                    const uint64_t* a, const uint64_t* b, const double* coeff, unsigned n_strings,
                    double* E, double* fluct, double* grad, double* tE, double* tE2, double* tO,
                    double* tF, double* tS, double* vec, double* norm, double* mlp, double* O_sum) {
    auto psi = make_deep({N, M, C, conn, params, fw, lp});
    exact_all(psi, {a, b, coeff, n_strings}, E, fluct, grad, tE, tE2, tO, tF, tS, vec, norm, mlp, O_sum);
}
unsigned ref_deep_mc(unsigned N, unsigned M, unsigned C, const unsigned* conn, const double* params,
                     const double* fw, const double* lp,
                     const uint64_t* a, const uint64_t* b, const double* coeff, unsigned n_strings,
                     unsigned num_samples, unsigned num_sweeps, unsigned num_therm,
                     uint64_t* sconf, double* slp, double* seloc, uint64_t* pconf, uint32_t* psite,
                     unsigned max_props, double* mc_energy) {
    auto psi = make_deep({N, M, C, conn, params, fw, lp});
    return mc_trace(psi, {a, b, coeff, n_strings}, num_samples, num_sweeps, num_therm,
                    sconf, slp, seloc, pconf, psite, max_props, mc_energy);
}

// HilbertSpaceDistance between psi_prime and U psi over ExactSummationSpins, both
// one-hidden-layer PsiDeep of the same shape: distance() and gradient(nu) with respect to
// psi_prime's parameters (HilbertSpaceDistance.cu.template:104-165); dist[0] from distance(),
// dist[1] from gradient()
void ref_deep_hsd_exact(unsigned N, unsigned M, unsigned C, const unsigned* conn,
                        const double* params, const double* fw, const double* lp,
                        const double* params_p, const double* fw_p, const double* lp_p,
                        const uint64_t* a, const uint64_t* b, const double* coeff, unsigned n_strings,
                        int unitary, double nu, double* dist, double* grad) {
    auto psi = make_deep({N, M, C, conn, params, fw, lp});
    auto psi_p = make_deep({N, M, C, conn, params_p, fw_p, lp_p});
    Operator op(HarnessExpr{a, b, coeff, n_strings}, false);
    ExactSummationSpins es(N, false);
    HilbertSpaceDistance hsd(psi_p.num_params, false);
    dist[0] = hsd.distance(psi, psi_p, op, unitary != 0, es);
    std::vector<std::complex<double>> g(psi_p.num_params);
    dist[1] = hsd.gradient(g.data(), psi, psi_p, op, unitary != 0, es, (float)nu);
    for(auto k = 0u; k < psi_p.num_params; k++) put(grad + 2 * k, g[k]);
}

// ---- PsiDeep (several hidden layers) ----
unsigned ref_deepml_num_params(unsigned N, unsigned L, const unsigned* sizes, const unsigned* connectivity,
                               const unsigned* conn, const double* params, const double* fw, const double* lp) {
    return make_deep_ml({N, L, sizes, connectivity, conn, params, fw, lp}).num_params;
}
void ref_deepml_log_psi_s(unsigned N, unsigned L, const unsigned* sizes, const unsigned* connectivity,
                          const unsigned* conn, const double* params, const double* fw, const double* lp,
                          uint64_t conf, double* out) {
    auto psi = make_deep_ml({N, L, sizes, connectivity, conn, params, fw, lp});
    psi_log_psi_s(psi, conf, out);
}
void ref_deepml_O_k(unsigned N, unsigned L, const unsigned* sizes, const unsigned* connectivity,
                    const unsigned* conn, const double* params, const double* fw, const double* lp,
                    uint64_t conf, double* out) {
    auto psi = make_deep_ml({N, L, sizes, connectivity, conn, params, fw, lp});
    psi_O_k(psi, conf, out);
}
void ref_deepml_exact(unsigned N, unsigned L, const unsigned* sizes, const unsigned* connectivity,
                      const unsigned* conn, const double* params, const double* fw, const double* lp,
                      const uint64_t* a, const uint64_t* b, const double* coeff, unsigned n_strings,
                      double* E, double* fluct, double* grad, double* tE, double* tE2, double* tO,
                      double* tF, double* tS, double* vec, double* norm, double* mlp, double* O_sum) {
    auto psi = make_deep_ml({N, L, sizes, connectivity, conn, params, fw, lp});
    exact_all(psi, {a, b, coeff, n_strings}, E, fluct, grad, tE, tE2, tO, tF, tS, vec, norm, mlp, O_sum);
}

// ---- PsiDeep over the Pauli-string basis: 3 input units per site (PauliString.hpp:84-90) ----
void ref_deepml_pauli_log_psi_s(unsigned N, unsigned L, const unsigned* sizes, const unsigned* connectivity,
                                const unsigned* conn, const double* params, const double* fw, const double* lp,
                                uint64_t a, uint64_t b, double* out) {
    auto psi = make_deep_ml({N, L, sizes, connectivity, conn, params, fw, lp, N / 3u});
    put(out, log_psi_s(psi, PauliString(a, b)));
}
void ref_deepml_pauli_O_k(unsigned N, unsigned L, const unsigned* sizes, const unsigned* connectivity,
                          const unsigned* conn, const double* params, const double* fw, const double* lp,
                          uint64_t a, uint64_t b, double* out) {
    auto psi = make_deep_ml({N, L, sizes, connectivity, conn, params, fw, lp, N / 3u});
    auto r = ann_on_gpu::psi_O_k(psi, PauliString(a, b));
    for(auto k = 0u; k < r.size(); k++) put(out + 2 * k, r[k]);
}
void ref_deepml_pauli_exact(unsigned N, unsigned L, const unsigned* sizes, const unsigned* connectivity,
                            const unsigned* conn, const double* params, const double* fw, const double* lp,
                            const uint64_t* a, const uint64_t* b, const double* coeff, unsigned n_strings,
                            double* E, double* fluct, double* grad, double* tE, double* tE2, double* tO,
                            double* tF, double* tS, double* vec, double* norm, double* mlp, double* O_sum) {
    auto psi = make_deep_ml({N, L, sizes, connectivity, conn, params, fw, lp, N / 3u});
    exact_all<PsiDeep, ExactSummationPaulis>(psi, {a, b, coeff, n_strings}, E, fluct, grad, tE, tE2, tO, tF, tS,
                                             vec, norm, mlp, O_sum);
}

// ---- PsiClassical and KullbackLeibler ----
// (descriptors arrive as void pointers: their types have internal linkage)
void ref_classical_log_psi_s(const void* dv, uint64_t conf, double* out) {
    const ClassicalDesc* d = static_cast<const ClassicalDesc*>(dv);
    if(d->ref) {
        auto ref = make_deep_ml(*d->ref);
        HarnessClassical<2u, PsiDeep::Kernel> psi(d->num_sites, features_of(*d), d->params, d->log_pref, ref.kernel(),
                                                  ref.num_params);
        psi_log_psi_s(psi, conf, out);
    } else {
        HarnessClassical<1u, kernel::PsiFullyPolarized_t<complex_t>> psi(
            d->num_sites, features_of(*d), d->params, d->log_pref, fully_polarized(d->num_sites), 0u);
        psi_log_psi_s(psi, conf, out);
    }
}
void ref_classical_O_k(const void* dv, uint64_t conf, double* out) {
    const ClassicalDesc* d = static_cast<const ClassicalDesc*>(dv);
    if(d->ref) {
        auto ref = make_deep_ml(*d->ref);
        HarnessClassical<2u, PsiDeep::Kernel> psi(d->num_sites, features_of(*d), d->params, d->log_pref, ref.kernel(),
                                                  ref.num_params);
        psi_O_k(psi, conf, out);
    } else {
        HarnessClassical<1u, kernel::PsiFullyPolarized_t<complex_t>> psi(
            d->num_sites, features_of(*d), d->params, d->log_pref, fully_polarized(d->num_sites), 0u);
        psi_O_k(psi, conf, out);
    }
}
void ref_classical_exact(const void* dv, const uint64_t* a, const uint64_t* b, const double* coeff,
                         unsigned n_strings, double* E, double* fluct, double* grad, double* tE, double* tE2,
                         double* tO, double* tF, double* tS, double* vec, double* norm, double* mlp, double* O_sum) {
    const ClassicalDesc* d = static_cast<const ClassicalDesc*>(dv);
    if(d->ref) {
        auto ref = make_deep_ml(*d->ref);
        HarnessClassical<2u, PsiDeep::Kernel> psi(d->num_sites, features_of(*d), d->params, d->log_pref, ref.kernel(),
                                                  ref.num_params);
        exact_all(psi, {a, b, coeff, n_strings}, E, fluct, grad, tE, tE2, tO, tF, tS, vec, norm, mlp, O_sum);
    } else {
        HarnessClassical<1u, kernel::PsiFullyPolarized_t<complex_t>> psi(
            d->num_sites, features_of(*d), d->params, d->log_pref, fully_polarized(d->num_sites), 0u);
        exact_all(psi, {a, b, coeff, n_strings}, E, fluct, grad, tE, tE2, tO, tF, tS, vec, norm, mlp, O_sum);
    }
}
// KL of the classical network against psi_prime over ExactSummationSpins: two consecutive
// value calls (the second subtracts the first's mean deviation), then gradient and
// gradient_with_noise; out4 = total weight, mean deviation (re, im), second value
void ref_kl_exact(const void* dv, const void* primev, double threshold, double nu, double* value,
                  double* grad, double* grad2, double* noise, double* out4) {
    const ClassicalDesc* d = static_cast<const ClassicalDesc*>(dv);
    auto pp = make_deep_ml(*static_cast<const DeepMLDesc*>(primev));
    ExactSummationSpins es(d->num_sites, false);
    KullbackLeibler kl(pp.num_params, false);
    auto run = [&](auto& psi) {
        value[0] = kl.value(psi, pp, es, threshold);
        out4[0] = kl.total_weight.front();
        out4[1] = kl.mean_deviation.front().real();
        out4[2] = kl.mean_deviation.front().imag();
        out4[3] = kl.value(psi, pp, es, threshold);
        std::vector<std::complex<double>> g(pp.num_params);
        value[1] = kl.gradient(g.data(), psi, pp, es, nu, threshold);
        for(auto k = 0u; k < pp.num_params; k++) put(grad + 2 * k, g[k]);
        auto r = kl.gradient_with_noise(psi, pp, es, nu, threshold);
        for(auto k = 0u; k < pp.num_params; k++) {
            put(grad2 + 2 * k, std::get<0>(r)[k]);
            noise[k] = std::get<1>(r)[k];
        }
        value[2] = std::get<2>(r);
    };
    if(d->ref) {
        auto ref = make_deep_ml(*d->ref);
        HarnessClassical<2u, PsiDeep::Kernel> psi(d->num_sites, features_of(*d), d->params, d->log_pref, ref.kernel(),
                                                  ref.num_params);
        run(psi);
    } else {
        HarnessClassical<1u, kernel::PsiFullyPolarized_t<complex_t>> psi(
            d->num_sites, features_of(*d), d->params, d->log_pref, fully_polarized(d->num_sites), 0u);
        run(psi);
    }
}

// ---- PsiRBM (no biases) ----
void ref_rbm_log_psi_s(unsigned N, unsigned M, const double* W, const double* fw, const double* lp,
                       uint64_t conf, double* out) {
    HarnessRBM psi(N, M, W, fw, lp);
    psi_log_psi_s(psi, conf, out);
}
void ref_rbm_O_k(unsigned N, unsigned M, const double* W, const double* fw, const double* lp,
                 uint64_t conf, double* out) {
    HarnessRBM psi(N, M, W, fw, lp);
    psi_O_k(psi, conf, out);
}
void ref_rbm_exact(unsigned N, unsigned M, const double* W, const double* fw, const double* lp,
                   const uint64_t* a, const uint64_t* b, const double* coeff, unsigned n_strings,
                   double* E, double* fluct, double* grad, double* tE, double* tE2, double* tO,
                   double* tF, double* tS, double* vec, double* norm, double* mlp, double* O_sum) {
    HarnessRBM psi(N, M, W, fw, lp);
    exact_all(psi, {a, b, coeff, n_strings}, E, fluct, grad, tE, tE2, tO, tF, tS, vec, norm, mlp, O_sum);
}
unsigned ref_rbm_mc(unsigned N, unsigned M, const double* W, const double* fw, const double* lp,
                    const uint64_t* a, const uint64_t* b, const double* coeff, unsigned n_strings,
                    unsigned num_samples, unsigned num_sweeps, unsigned num_therm,
                    uint64_t* sconf, double* slp, double* seloc, uint64_t* pconf, uint32_t* psite,
                    unsigned max_props, double* mc_energy) {
    HarnessRBM psi(N, M, W, fw, lp);
    return mc_trace(psi, {a, b, coeff, n_strings}, num_samples, num_sweeps, num_therm,
                    sconf, slp, seloc, pconf, psite, max_props, mc_energy);
}

// TDVP (E, E2, <O>, F, S) over the reference's own host Monte Carlo with one chain (the
// host path runs chain 0 alone, MonteCarlo.hpp:69-71): TDVP::eval, TDVP.cu.template:181-302.
// Used to time the reference's CPU path against the oracle's restatement of it.
void ref_rbm_tdvp_mc(unsigned N, unsigned M, const double* W, const double* fw, const double* lp,
                     const uint64_t* a, const uint64_t* b, const double* coeff, unsigned n_strings,
                     unsigned num_samples, unsigned num_sweeps, unsigned num_therm, double* tE) {
    HarnessRBM psi(N, M, W, fw, lp);
    Operator op(HarnessExpr{a, b, coeff, n_strings}, false);
    MonteCarloSpins mc(num_samples, num_sweeps, num_therm, 1u, Update_Policy<Spins>(), false);
    TDVP tdvp(psi.num_params, false);
    tdvp.eval(op, psi, mc, false_t());
    put(tE, tdvp.E_local.front());
}

// ---- PsiCNN ----
void ref_cnn_log_psi_s(const unsigned* extent, unsigned L, const unsigned* ch, const unsigned* conn,
                       const unsigned* cls, const double* p, unsigned np, double ff, const double* lp,
                       uint64_t conf, double* out) {
    HarnessCNN psi(extent, L, ch, conn, cls, p, np, ff, lp);
    psi_log_psi_s(psi, conf, out);
}
void ref_cnn_O_k(const unsigned* extent, unsigned L, const unsigned* ch, const unsigned* conn,
                 const unsigned* cls, const double* p, unsigned np, double ff, const double* lp,
                 uint64_t conf, double* out) {
    HarnessCNN psi(extent, L, ch, conn, cls, p, np, ff, lp);
    psi.init_gradient(1u);
    psi_O_k(psi, conf, out);
}
void ref_cnn_exact_energy(const unsigned* extent, unsigned L, const unsigned* ch, const unsigned* conn,
                          const unsigned* cls, const double* p, unsigned np, double ff, const double* lp,
                          const uint64_t* a, const uint64_t* b, const double* coeff, unsigned n_strings,
                          double* E, double* norm) {
    HarnessCNN psi(extent, L, ch, conn, cls, p, np, ff, lp);
    Operator op(HarnessExpr{a, b, coeff, n_strings}, false);
    ExactSummationSpins es(psi.num_sites, false);
    ExpectationValue ev(false);
    put(E, ev(op, psi, es));
    norm[0] = psi_norm(psi, es);
}

// ---- activation ----
void ref_activation(double re, double im, unsigned layer, double* out, double* dout) {
    put(out, my_logcosh(complex_t(re, im), layer));
    put(dout, my_tanh(complex_t(re, im), layer));
}

// ---- Pauli string application (PauliString.hpp:242-254) ----
void ref_pauli_apply(uint64_t a, uint64_t b, uint64_t conf, unsigned N, double* factor, uint64_t* out_conf) {
    auto me = PauliString(a, b).apply(Spins(conf, N));
    put(factor, me.coefficient);
    out_conf[0] = me.vector.configuration();
}

}  // extern "C"
