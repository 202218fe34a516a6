// Host-side objects behind the C ABI handles, and the launchers each .cu file provides.
#pragma once

#include <complex>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "annongpu.h"
#include "ann_common.cuh"

namespace ann {

using zd = std::complex<double>;

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void cuda_check(cudaError_t e, const char* what);
void set_last_error(const char* msg);
#define ANN_CUDA(x) ::ann::cuda_check((x), #x)
void count_launch(unsigned n = 1);
void check_launch(const char* what);

// device allocation that only grows
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf();
    void ensure(size_t n);
    void free_();
    template<typename X> X* as() const { return reinterpret_cast<X*>(p); }
};

void upload(DevBuf& b, const void* src, size_t bytes);

struct ann_made_impl;

// ---------------------------------------------------------------------------------
struct CnnLayerHost {
    unsigned channels, prev_channels, vol, conn[3], param_offset;
};

// PsiDeep with several hidden layers: layer structure and the offsets of its tables
struct DeepHost {
    std::vector<unsigned> sizes, C, conn;          // units, connections per unit, connection blocks
    std::vector<unsigned> conn_off, rbeg_off, rq_off;  // offsets into the device table (u16 entries)
    unsigned tab_len = 0;
    int dup0 = 0;   // a site appears twice in one first-layer window
    unsigned na = 0;        // input-unit parameters a (N; 0 for a classical network without reference)
    unsigned K = 0;         // classical features (PsiClassical), parameters [theta | network]
    zd lp_ref{0.0, 0.0};    // log prefactor of the reference network (PsiClassical)
};

struct ann_psi_impl {
    int kind = 0;       // 0 RBM family, 1 CNN, 2 PsiDeep with several hidden layers
    int precision = 0;  // 0 fp32, 1 fp64
    int act = 0;
    unsigned N = 0, NW = 1, Np = 0;
    zd lp{0.0, 0.0};
    DevBuf params;      // FP64 master copy (Np complex128)
    // RBM family
    unsigned M = 0, Mpad = 0, C = 0, U = 1;
    int layout = 0, a_in = 1;
    std::vector<unsigned> conn;
    std::vector<zd> fw;
    DevBuf Wd, a, b, fwd, connd;
    // CNN
    unsigned extent[3] = {1, 1, 1};
    std::vector<CnnLayerHost> layers;
    std::vector<unsigned> sym;
    unsigned ncls = 1;
    double final_factor = 1.0;
    DevBuf cnn_w, cnn_meta;  // kernel-precision weights (CNN, multi-layer PsiDeep); packed CNN metadata
    DevBuf cnn_scratch;      // CNN: per resident warp, pre-activations of both layers and two work buffers
    unsigned cnn_x0 = 0, cnn_x1 = 0;  // CNN: most layer-0 / layer-1 sites a move of one or two flips changes
    // multi-layer PsiDeep (final weights in fw / fwd)
    DeepHost deep;
    DevBuf deep_tab;
    DevBuf feat_beg, feat_zy, feat_c, feat_cf;   // classical features (u32 offsets, Z|Y masks, FP64 / FP32 coefficients)
    std::vector<unsigned> feat_beg_h;
    std::vector<uint64_t> feat_a_h, feat_b_h;     // feature strings as given (one word each)
    std::vector<zd> feat_coeff_h;
    int order = 0;                                 // PsiClassical order (0: not a classical network)
    size_t elem_bytes() const { return precision ? 16 : 8; }
};

struct ann_op_impl {
    unsigned n_strings = 0, nw = 2, max_site = 0;
    std::vector<uint64_t> a, b;   // n x nw
    std::vector<zd> coeff;
    // grouped device form
    unsigned n_diag = 0, n_groups = 0;
    DevBuf diag_mask, diag_coeff, grp_site_begin, grp_sites, grp_str_begin, str_mask, str_coeff, diag_coeff_f,
        str_coeff_f;
    DevBuf raw_a, raw_b, raw_c, raw_cf;   // strings as given (Pauli-string basis)
    OpDev view() const;
};

// per-call sample rows written by the sampling / enumeration kernels
struct Rows {
    size_t n = 0;
    DevBuf conf, log_psi, eloc, weight;
};

struct ann_ens_impl {
    int kind = 0;  // 0 exact, 1 Monte Carlo
    int basis = 0; // ANN_BASIS_SPINS or ANN_BASIS_PAULIS
    unsigned N = 0;
    // Monte Carlo
    unsigned num_samples = 0, num_sweeps = 0, num_therm = 0, n_chains = 0;
    int move = 0, n_up = -1, persistent = 0;
    uint64_t seed = 0;
    std::vector<uint32_t> bonds;
    DevBuf bonds_d, chain_conf, chain_counter, acc_rej;
    bool chains_valid = false;  // chain state holds equilibrated chains
    unsigned long long last_acc = 0, last_rej = 0;
    // learned proposal (Metropolis-Hastings independence moves)
    const ann_made_impl* made = nullptr;
    unsigned indep_per_sample = 0;
    double made_min_acceptance = 0.0;
    bool made_dropped = false;     // host copy of the device flag, read back by the bookkeeping
    DevBuf made_on;                // int on the device: the sampler runs the learned moves while 1
    unsigned long long last_made_acc = 0, last_made_rej = 0;
    // ring buffer of recent sample configurations (training data for the proposal)
    DevBuf hist, hist_posd;        // rows; device write position (advanced by every pass)
    size_t hist_cap = 0, hist_len = 0;
    // tape replay
    DevBuf tape_site, tape_u, tape_init;
    unsigned tape_len = 0;
    Rows rows;
    unsigned num_steps() const {
        return kind == 0 ? (unsigned)(1ull << (basis ? 2 * N : N)) : (num_samples / n_chains) * n_chains;
    }
    double uniform_weight() const { return 1.0 / (double)num_samples; }
};

struct ann_made_impl {
    unsigned N = 0, H = 0, adam_t = 0;
    uint64_t seed = 0;
    DevBuf W1, b1, W2, b2;            // FP32 master weights (W1: H x N, W2: N x H)
    DevBuf W1t, W2t;                  // BF16 transposed copies read by the kernels
    DevBuf W2b;                       // BF16 copy of W2 as stored (N x H): read through L1 by the samplers
    // BF16 operands of the tensor-core training GEMMs (rows zero-padded to 64-value multiples):
    // W1 as stored (H x N64), W2 as stored (N x H64), W2^T (H x N64)
    DevBuf W1g, W2g, W2Tg;
    DevBuf deg;                       // hidden-unit degrees (u16)
    DevBuf mW1, vW1, mb1, vb1, mW2, vW2, mb2, vb2;  // Adam moments
    DevBuf gW1, gb1, gW2, gb2;        // gradients
    DevBuf X, pre, hbuf, l, dl, dh, row_loss;       // training scratch
    // BF16 hi / lo splits of the training step's activations and gradients (GEMM operands)
    DevBuf Xg, XTg, hs, hTs, dls, dlTs, dhTs;
    DevBuf kpart;                                   // split-K partial tiles of the weight gradients
};

struct ann_tdvp_impl {
    unsigned Np = 0;
    int s_mode = 0;
    size_t n_rows = 0, ldO = 0;
    int O_precision = 0;
    DevBuf O;                   // n_rows x ldO, kernel precision complex
    DevBuf stats;               // Stats
    DevBuf Obar, F, Osum;       // Np complex128
    DevBuf partial;             // reduction scratch
    DevBuf S;                   // Np x Np complex128
    // S from the tensor-core HERK holds FP32 sums: with the mixed or FP32 solver it is kept
    // in complex64 (half the bytes for the HERK's stores, the FP32 copy and every residual
    // of the refinement); the complex128 copy is formed only when something reads it
    DevBuf S32;                 // Np x Np complex64
    bool S_in32 = false;        // the last S is in S32
    bool S64_fresh = false;     // S (complex128) holds the last S
    DevBuf L;                   // Cholesky factor (lower), Np x Np complex128
    DevBuf rhs, delta, resid;   // Np complex128
    DevBuf tmp64;               // Np complex128: intermediate of the FP64 triangular solves
    // SR solver: ANN_SOLVER_FP64 (FP64 Cholesky + one refinement step), ANN_SOLVER_MIXED
    // (FP32 Cholesky + FP64 refinement to ir_tol, at most ir_max solves) or
    // ANN_SOLVER_FP32 (one FP32 Cholesky solve, no refinement)
    int solver = ANN_SOLVER_FP64;
    unsigned ir_max = 10;
    double ir_tol = 1e-12;
    bool fell_back = false;     // the last mixed solve stalled and the FP64 solve replaced it
    DevBuf L32, Dinv32, c32, ir;  // FP32 factor, inverted diagonal blocks, FP32 vectors, refinement state
    DevBuf xs32;                // double-float split of the iterate (residual from a complex64 S)
    int chol_tc = 1;            // FP32 Cholesky trailing update: 1 tcgen05 (split TF32), 0 FP32 SIMT
    int chol_form = 0;          // ANN_CHOL_FORM_* of the last FP32 factorisation
    bool chol_tc_set = false;   // chosen explicitly (ann_tdvp_set_chol_update): the tuning table is not read
    DevBuf chol_pt;             // TF32 hi/lo panel operands (two buffers) of the tensor-core update
    unsigned chol_pt_n = 0;
    alignas(64) unsigned char chol_map[2][128];  // TMA descriptors of its two buffers (CUtensorMap)
    alignas(64) unsigned char chol_pmap[2][128]; // the same buffers in the panel-pair layout (K = 128)
    alignas(64) unsigned char chol_amap[128]; // TMA descriptor of the FP32 factor (reduce-add epilogue)
    int chol_reduce = 0;                      // chol_amap is bound (n even)
    DevBuf herk_in;             // BF16 operand for the tensor-core HERK
    DevBuf vec_in, vec_tmp;
    DevBuf wts;                 // per-row weights of the last eval (exact summation)
    bool wts_exact = false;
    double w0 = 0.0;            // uniform row weight (Monte Carlo)
    bool have_S = false;
    unsigned graph_kernels = 0;
    cudaStream_t side = nullptr;          // look-ahead panel stream of the Cholesky
    cudaEvent_t side_ev[2] = {nullptr, nullptr};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
};

struct Stats {
    double W;       // total weight
    double E[2];    // sum w E_loc
    double E2;      // sum w |E_loc|^2
    double L[2];    // sum w log psi
};

// ---- launchers ------------------------------------------------------------------
struct SampleTargets {
    Rows* rows;
    void* O = nullptr;     // rows x ldO (kernel precision) or null
    size_t ldO = 0;
    bool want_eloc = true;
};

void psi_prepare(ann_psi_impl& psi, cudaStream_t st);
// runs the ensemble (MC sampling or exact enumeration) over psi
void run_ensemble(ann_psi_impl& psi, const ann_op_impl* op, ann_ens_impl& ens, const SampleTargets& t,
                  cudaStream_t st);
// appends n sample configurations (rows of conf) to the ensemble's history ring (capi.cu)
void hist_append(ann_ens_impl& ens, const uint64_t* conf, size_t n, cudaStream_t st);
void run_confs(ann_psi_impl& psi, const ann_op_impl* op, const uint64_t* confs_dev, size_t n, Rows& rows,
               void* O, size_t ldO, cudaStream_t st, int basis = ANN_BASIS_SPINS);

// per-precision RBM launchers (rbm_f32.cu / rbm_f64.cu)
template<typename T> void rbm_prepare_T(ann_psi_impl& psi, cudaStream_t st);
template<typename T> void rbm_mc_T(ann_psi_impl& psi, const ann_op_impl* op, ann_ens_impl& ens,
                                   const SampleTargets& t, cudaStream_t st);
template<typename T> void rbm_exact_T(ann_psi_impl& psi, const ann_op_impl* op, ann_ens_impl& ens,
                                      const SampleTargets& t, cudaStream_t st);
template<typename T> void rbm_confs_T(ann_psi_impl& psi, const ann_op_impl* op, const uint64_t* confs, size_t n,
                                      Rows& rows, void* O, size_t ldO, cudaStream_t st);

// statistics (stats.cu)
void row_stats(const Rows& rows, const double* weight_or_null, double w0, Stats* out_dev, DevBuf& scratch,
               cudaStream_t st);
// acc_O[k] = sum_s w_s O_sk ; acc_F[k] = sum_s w_s e_s conj(O_sk); then
// F[k] = acc_F[k] - E conj(acc_O[k]) when `center_with` != null
void col_stats(const void* O, int O_prec, size_t rows, size_t ld, unsigned Np, const double* weight_or_null,
               double w0, const cplx<double>* e, cplx<double>* Obar, cplx<double>* F, const Stats* center_with,
               cplx<double>* Osum, DevBuf& scratch, cudaStream_t st);
void row_dot(const void* O, int O_prec, size_t rows, size_t ld, unsigned Np, const cplx<double>* v,
             cplx<double>* y, cudaStream_t st);
void finalize_sdotv(cplx<double>* out, const cplx<double>* Obar, const cplx<double>* v, unsigned Np,
                    cudaStream_t st);

// S = sum_s w_s conj(O_s - Obar) (O_s - Obar) + (1 - W) conj(Obar) Obar^T (herk_simt.cu / herk_tc.cu)
void herk_simt(const void* O, int O_prec, size_t rows, size_t ld, unsigned Np, const double* weight_or_null,
               double w0, const cplx<double>* Obar, const Stats* stats, cplx<double>* S, cudaStream_t st);
void herk_tc(ann_tdvp_impl& td, const double* weight_or_null, double w0, bool split, cudaStream_t st);

// TDVP evaluation split for the batched path (capi.cu): buffers and sample targets,
// then reductions and S from the sampled rows
SampleTargets tdvp_prepare(ann_tdvp_impl& t, ann_psi_impl& psi, ann_ens_impl& ens);
void tdvp_post(ann_tdvp_impl& t, ann_psi_impl& psi, ann_ens_impl& ens, bool want_S, cudaStream_t st);

// FP64 Cholesky SR solve (cholesky.cu)
// BF16 tensor-core GEMM of the MADE training step (made_tc.cu):
//   C (M x N, FP32) = sum over segments s of A[:, aoff_s : aoff_s + K] . B[:, boff_s : boff_s + K]^T
// A (a_rows x a_cols) and B (b_rows x b_cols) BF16 row-major; K and the offsets multiples of 64;
// with splits > 1 the K range is split over CTAs and the partial tiles summed in order.
struct MadeGemm {
    const void* A;
    unsigned a_rows, a_cols;
    const void* B;
    unsigned b_rows, b_cols;
    unsigned M, N, K, nseg;
    int aoff[3], boff[3];
    float* C;
    size_t ldc;
    const float* bias;     // per output column, or null
    const float* aux;      // C = 0 where aux[m * ldc + n] <= 0, or null
    unsigned splits;
};
void made_gemm(const MadeGemm& g, DevBuf& scratch, cudaStream_t st);
// BF16 hi (and lo) of an FP32 R x C matrix into a zero-padded rows x cols block: row-major
// (dst[r][c], lo at column lo_off + c) or transposed (dst[c][r], lo at lo_off + r)
void made_split_rows(const float* src, unsigned R, unsigned C, size_t lds, void* dst, size_t ldd, unsigned rows,
                     unsigned cols, unsigned lo_off, bool with_lo, cudaStream_t st);
void made_split_cols(const float* src, unsigned R, unsigned C, size_t lds, void* dst, size_t ldd, unsigned rows,
                     unsigned cols, unsigned lo_off, bool with_lo, cudaStream_t st);
void sr_solve(ann_tdvp_impl& td, double shift, unsigned* status_dev, cudaStream_t st);
// the last S in complex128 (widened from S32 on first use after an evaluation that kept it there)
const cplx<double>* S64(ann_tdvp_impl& td, cudaStream_t st);
// mixed-precision SR solve (cholesky_mixed.cu); out4 = {solves, first and last
// relative FP64 residual, stalled}
void sr_solve_mixed(ann_tdvp_impl& td, double shift, unsigned max_iter, double tol, bool pivots_to_status,
                    unsigned* status_dev, cudaStream_t st);
void mixed_solve_info(const ann_tdvp_impl& td, double* out4, cudaStream_t st);
// tensor-core trailing update of the FP32 Cholesky (chol_update_tc.cu)
void chol_update_tc_prepare(ann_tdvp_impl& td, unsigned n, cudaStream_t st);
bool chol_update_tc_bind(ann_tdvp_impl& td, cplx<float>* A, unsigned n);
// operand buffer 0 / 1 (panel k uses k % 2), written by the panel solve
float* chol_update_tc_operand(ann_tdvp_impl& td, unsigned buf);
float* chol_update_tc_pair_operand(ann_tdvp_impl& td, unsigned buf);
void chol_update_tc_pair(ann_tdvp_impl& td, cplx<float>* A, unsigned n, unsigned pb, bool col_only, unsigned* status,
                         cudaStream_t st);
void chol_update_tc(ann_tdvp_impl& td, cplx<float>* A, unsigned n, unsigned kb, bool col_only, unsigned* status,
                    cudaStream_t st);
// the look-ahead side stream of the Cholesky factorisations (high priority)
void ensure_side_stream(ann_tdvp_impl& td);
// the configured solver; an eager mixed solve that stalls is redone in FP64
void sr_solve_any(ann_tdvp_impl& td, double shift, unsigned* status_dev, cudaStream_t st);
// CUDA-event marks around the FP32 factorisation when phase timing is on (capi.cu)
void solve_mark(int i, cudaStream_t st);
// tagged events of the FP32 Cholesky's timeline (ann_set_factor_trace); reset per factorisation.
// A mark of level 2 sits between two panel kernels and turns their programmatic launch
// into a plain one, so it is recorded only at trace level 2
void factor_mark(int tag, cudaStream_t st, int level = 1);
void factor_trace_reset();
void sr_update(ann_psi_impl& psi, const cplx<double>* delta, double lr, cudaStream_t st);

unsigned* status_word();
::ann_ens* ens_clone(const ann_ens_impl& src);  // capi.cu (release with ann_ens_destroy)

// ---- tuning table (tuning.cu): launch and tile choices per device and shape ----
// key: "<knob>/<shape>"; absent keys fall back to the built-in default
int tuning_get(const std::string& key, int dflt);
void tuning_set(const std::string& key, int value);
std::string key_mc_wpb(const ann_psi_impl& psi, const ann_ens_impl& ens);
std::string key_mc_wsmem(const ann_psi_impl& psi, const ann_ens_impl& ens);
std::string key_mc_team(const ann_psi_impl& psi, const ann_ens_impl& ens);
std::string key_slab(size_t rows, unsigned Np);
std::string key_chol_update(unsigned n);
std::string key_chol_reserve(unsigned n);
std::string key_chol_pair(unsigned n);

// PsiCNN (cnn.cu)
void deep_prepare(ann_psi_impl& psi, cudaStream_t st);
// builds the layer tables of the multi-layer kernels for a one-layer PsiDeep (RBM family,
// [a | b | W] parameters) the first time a Pauli-string ensemble or configuration meets it
void deep_ensure(ann_psi_impl& psi);
void deep_run(ann_psi_impl& psi, const ann_op_impl* op, ann_ens_impl& ens, const SampleTargets& t, cudaStream_t st);
void deep_confs(ann_psi_impl& psi, const ann_op_impl* op, const uint64_t* confs, size_t n, Rows& rows, void* O,
                size_t ldO, cudaStream_t st, int basis);
void cnn_prepare(ann_psi_impl& psi, cudaStream_t st);
void cnn_run(ann_psi_impl& psi, const ann_op_impl* op, ann_ens_impl& ens, const SampleTargets& t, cudaStream_t st);
void cnn_confs(ann_psi_impl& psi, const ann_op_impl* op, const uint64_t* confs, size_t n, Rows& rows, void* O,
               size_t ldO, cudaStream_t st);

// sum_s w_s exp(sum_n c_n <s|P_n|s'>) over the rows (ExpectationValue.cu.template:52-81)
void exp_sigma_z_sum(const ann_op_impl& op, const Rows& rows, const double* wts, double w0, double* out2,
                     cudaStream_t st);
// MADE (made.cu)
struct MadeDev;
MadeDev made_view(const ann_made_impl& m);
void made_logq_batch(const ann_made_impl& m, const uint64_t* confs, size_t n, double* out, cudaStream_t st);

// activation_function(z, layer) evaluated by the device code path
void activation_host(double re, double im, unsigned layer, int activation, double* out2);

}  // namespace ann

// the opaque handle types of include/annongpu.h
struct ann_psi : ann::ann_psi_impl {};
struct ann_op : ann::ann_op_impl {};
struct ann_ens : ann::ann_ens_impl {};
struct ann_tdvp : ann::ann_tdvp_impl {};
struct ann_made : ann::ann_made_impl {};
