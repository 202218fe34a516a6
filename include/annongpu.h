/*
 * annongpu.h -- C ABI of the GB300-native VMC inner loop (libannongpu.so).
 *
 * Drop-in boundary for the reference's pybind11 module _pyANNonGPU
 * (pyANNonGPU/main.cpp.template:65-541): every entry point below replaces one
 * binding of that module, cited beside it. Plain pointers and sizes only; complex
 * numbers are interleaved (re, im) doubles; spin configurations are arrays of
 * 64-bit words (bit i = 1 <-> sigma^z_i = +1, include/basis/Spins.h:104-118).
 *
 * Conventions
 *   - Every function returns ANN_OK (0) or an error code; ann_last_error() gives
 *     the message of the last failure on the calling thread. The reference turns
 *     CUDA errors into std::runtime_error (include/types.h:139-147); the Python
 *     layer turns these codes into RuntimeError.
 *   - `stream` is a cudaStream_t passed as void* (NULL = the legacy default
 *     stream). Functions that return host data synchronise that stream.
 *   - Handles are not thread-safe; use one handle per thread.
 *   - There is no CPU fallback: a call without a usable CUDA device fails.
 */
#ifndef ANNONGPU_H
#define ANNONGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ANN_OK 0
#define ANN_ERR_INVALID 1      /* bad argument or size beyond a documented limit */
#define ANN_ERR_CUDA 2         /* a CUDA runtime call failed */
#define ANN_ERR_NUMERIC 3      /* non-finite value or non-positive-definite matrix */
#define ANN_ERR_UNSUPPORTED 4  /* combination not implemented */

typedef struct ann_psi ann_psi;
typedef struct ann_op ann_op;
typedef struct ann_ens ann_ens;
typedef struct ann_tdvp ann_tdvp;
typedef struct ann_made ann_made;
typedef struct ann_batch ann_batch;
typedef struct ann_kl ann_kl;

const char* ann_last_error(void);
int ann_version(void);

/* setDevice (pyANNonGPU/main.cpp.template:538, source/ANNonGPU.cu:7-9) */
int ann_set_device(int device);
/* start_profiling / stop_profiling (main.cpp.template:539-540, source/ANNonGPU.cu:11-17) */
int ann_profiler_start(void);
int ann_profiler_stop(void);

/* ---------------------------------------------------------------------------------
 * Wavefunctions
 * ------------------------------------------------------------------------------ */
#define ANN_LAYOUT_RBM 0    /* params = W (N x M)          -- PsiRBM (include/quantum_state/PsiRBM.hpp:251-257) */
#define ANN_LAYOUT_DEEP 1   /* params = [a | b | W (C x M)] -- PsiDeep (source/quantum_state/PsiDeep.cu:245-270) */
#define ANN_ACT_POLY 0      /* reference polynomial log cosh (include/quantum_state/psi_functions.hpp:40-48) */
#define ANN_ACT_LOGCOSH 1   /* exact log cosh / tanh */
#define ANN_PREC_FP32 0     /* complex64 arithmetic in the kernels */
#define ANN_PREC_FP64 1     /* complex128 arithmetic in the kernels */

typedef struct {
    unsigned N;                   /* input sites (<= 128) */
    unsigned M;                   /* hidden units (<= 256) */
    unsigned C;                   /* connections per hidden unit (<= N) */
    const unsigned* connections;  /* C x M, entry (c, j) = input site; NULL = identity (C == N) */
    const double* params;         /* interleaved complex, laid out as `layout` says */
    const double* final_weights;  /* M complex */
    double log_prefactor[2];
    int layout;                   /* ANN_LAYOUT_* */
    int a_in_log_psi;             /* 1: log psi includes a.s (standard RBM); 0: reference PsiDeep */
    int activation;               /* ANN_ACT_* */
    int precision;                /* ANN_PREC_* */
} ann_rbm_desc;

/* PsiDeep(...) ctor (main.cpp.template:71-81) and PsiRBM(...) ctor (:120-126) */
int ann_psi_create_rbm(const ann_rbm_desc* desc, ann_psi** out);

typedef struct {
    unsigned extent[3];               /* lattice extent (N = product <= 128) */
    unsigned num_layers;              /* <= 4 */
    const unsigned* num_channels;     /* num_layers */
    const unsigned* connectivity;     /* num_layers x 3 (forward-anchored periodic windows) */
    const unsigned* symmetry_classes; /* N */
    const double* params;             /* interleaved complex */
    unsigned num_params;
    double final_factor;
    double log_prefactor[2];
    int activation;                   /* ANN_ACT_POLY: reference layer semantics; ANN_ACT_LOGCOSH: log cosh on every layer */
    int precision;
} ann_cnn_desc;

/* PsiCNN(...) ctor (main.cpp.template:160-170) */
int ann_psi_create_cnn(const ann_cnn_desc* desc, ann_psi** out);
typedef struct {
    unsigned N;                     /* input units (spins), <= 128 */
    unsigned num_layers;            /* hidden layers, 1..4 (the reference allows 3, PsiDeep.hpp:88) */
    const unsigned* sizes;          /* num_layers: units per layer, <= 1024 */
    const unsigned* connectivity;   /* num_layers: connections per unit C_l (<= units of the layer below) */
    const unsigned* connections;    /* concatenated C_l x sizes[l] blocks; entry (i, j) at i*sizes[l] + j is the
                                       unit of the layer below (spin for l = 0) read by unit j */
    const double* params;           /* [a(N) | b_0 | W_0 | b_1 | W_1 | ...] interleaved complex */
    unsigned num_params;            /* N + sum_l sizes[l] * (1 + connectivity[l]) */
    const double* final_weights;    /* sizes[num_layers-1] complex (fixed, not variational) */
    double log_prefactor[2];
    int a_in_log_psi;               /* 0 reproduces the reference, whose log psi omits a.s (PsiDeep.hpp:260-264) */
    int activation;                 /* ANN_ACT_POLY: log-cosh polynomial on layer 0, odd polynomial deeper;
                                       ANN_ACT_LOGCOSH: log cosh on every layer */
    int precision;
} ann_deep_desc;

/* PsiDeep(num_sites, a, b, connections, W, final_weights, log_prefactor, gpu) with several
   hidden layers (main.cpp.template:71-81, include/quantum_state/PsiDeep.hpp:488-560) */
int ann_psi_create_deep(const ann_deep_desc* desc, ann_psi** out);

/* copy() (main.cpp.template:82, 127, 171) */
int ann_psi_copy(const ann_psi* psi, ann_psi** out);
int ann_psi_destroy(ann_psi* psi);
/* num_params (main.cpp.template:93, 138, 191) */
int ann_psi_num_params(const ann_psi* psi, unsigned* out);
/* params getter / setter (main.cpp.template:94-101, 139-145, 192-198); 2*num_params doubles */
int ann_psi_get_params(const ann_psi* psi, double* out);
int ann_psi_set_params(ann_psi* psi, const double* params);
/* asynchronous variant: copies from (pinned) host memory on `stream` and re-derives
   the kernel-precision weights there */
int ann_psi_set_params_async(ann_psi* psi, const double* params, void* stream);
/* log_prefactor getter / setter (main.cpp.template:85-89) */
int ann_psi_get_log_prefactor(const ann_psi* psi, double* out2);
int ann_psi_set_log_prefactor(ann_psi* psi, double re, double im);
/* device pointer of the FP64 master parameters (num_params complex128) */
int ann_psi_params_device(ann_psi* psi, void** out);
/* re-derive the kernel-precision weights from the device master parameters */
int ann_psi_sync_device_params(ann_psi* psi, void* stream);

/* ---------------------------------------------------------------------------------
 * Operators: Operator(PauliExpression, gpu) (main.cpp.template:321-333,
 * source/operator/Operator.cpp:18-39). String n uses words [n*num_words,
 * (n+1)*num_words) of a and b; per site (a,b) = (0,0) I, (1,0) X, (0,1) Y, (1,1) Z.
 * ------------------------------------------------------------------------------ */
int ann_op_create_pauli(unsigned n_strings, unsigned num_words, const uint64_t* a, const uint64_t* b,
                        const double* coeff, ann_op** out);
int ann_op_destroy(ann_op* op);
/* num_strings (main.cpp.template:332) */
int ann_op_num_strings(const ann_op* op, unsigned* out);

/* ---------------------------------------------------------------------------------
 * Ensembles
 * ------------------------------------------------------------------------------ */
/* ExactSummationSpins(num_sites, gpu) (main.cpp.template:395-399, include/ensembles/ExactSummation.hpp:33-72) */
int ann_ens_create_exact(unsigned num_sites, ann_ens** out);

#define ANN_MOVE_FLIP 0            /* single spin flip (include/ensembles/policies/Update_Policy.hpp:20-33) */
#define ANN_MOVE_EXCHANGE_BONDS 1  /* swap the spins of a random bond (Sz conserving) */
#define ANN_MOVE_EXCHANGE_PAIRS 2  /* swap the spins of a random site pair (Sz conserving) */

typedef struct {
    unsigned num_samples;               /* total samples; per chain num_samples / num_markov_chains */
    unsigned num_sweeps;                /* sweeps (N proposals each) between samples */
    unsigned num_thermalization_sweeps;
    unsigned num_markov_chains;
    int move;                           /* ANN_MOVE_* */
    const uint32_t* bonds;              /* n_bonds x 2 site pairs for ANN_MOVE_EXCHANGE_BONDS */
    unsigned n_bonds;
    int n_up;                           /* < 0: free; >= 0: initial configurations with exactly n_up up spins */
    uint64_t seed;                      /* Philox key */
    int persistent;                     /* 0: every call re-draws and re-thermalises the chains
                                           (MonteCarlo.hpp:79, 89-93); 1: chains continue across calls */
} ann_mc_desc;

/* MonteCarloSpins(num_samples, num_sweeps, num_thermalization_sweeps, num_markov_chains, gpu)
   (main.cpp.template:358-366, include/ensembles/MonteCarlo.hpp:249-259); also MonteCarloLoop */
int ann_ens_create_mc(const ann_mc_desc* desc, ann_ens** out);
/* copy constructor MonteCarloSpins(MonteCarloSpins&) (main.cpp.template:360) */
int ann_ens_copy(const ann_ens* ens, ann_ens** out);
int ann_ens_destroy(ann_ens* ens);
/* num_steps (main.cpp.template:363, 398) */
int ann_ens_num_steps(const ann_ens* ens, unsigned* out);

#define ANN_BASIS_SPINS 0   /* configurations are spins, bit i = input unit i */
#define ANN_BASIS_PAULIS 1  /* configurations are Pauli strings (words a, b; include/basis/PauliString.hpp) */
/* ExactSummationPaulis(num_sites) (main.cpp.template:402-406) = an exact ensemble over num_sites
   sites switched to ANN_BASIS_PAULIS (4^num_sites strings, PauliString.hpp:26-35);
   MonteCarloPaulis (main.cpp.template:369-380) = a Monte Carlo ensemble switched to it (moves set
   one random site to a random Pauli type, Update_Policy.hpp:41-57; single-flip moves only, no
   tape, no learned proposal). The wavefunction sees 3 input units per site
   (PauliString::network_unit_at, :84-90): PsiDeep of any depth. */
int ann_ens_set_basis(ann_ens* ens, int basis);
/* acceptance_rate of the last sampling call (main.cpp.template:364-366) */
int ann_ens_acceptance_rate(const ann_ens* ens, double* out);
/* reads the acceptance counters of the last sampling pass (synchronising `stream`) and
   applies the learned proposal's drop rule; the ExpectationValue family does this after
   every call, TDVP eval / SR steps leave it to the caller (no per-step host round trip) */
int ann_ens_refresh_stats(ann_ens* ens, void* stream);
/* chain state (configurations num_markov_chains x num_words, Philox counters) */
int ann_ens_get_chains(const ann_ens* ens, uint64_t* conf, uint64_t* counter);
int ann_ens_set_chains(ann_ens* ens, const uint64_t* conf, const uint64_t* counter);
/* Learned proposal: after the local sweeps of each sample, `indep_per_sample`
   Metropolis-Hastings independence moves draw s' from the MADE `m` (NULL disables).
   When the acceptance of these moves in a call falls below `min_acceptance`, the
   proposal is dropped and local Metropolis continues alone. */
int ann_ens_set_proposal(ann_ens* ens, const ann_made* m, unsigned indep_per_sample, double min_acceptance);
/* acceptance of the learned moves in the last call, and whether the proposal was dropped */
int ann_ens_proposal_stats(const ann_ens* ens, double* acceptance, int* dropped);
/* keep the configurations of the last `capacity` samples (ring buffer) as training data */
int ann_ens_set_history(ann_ens* ens, unsigned capacity);
/* Proposal replay (parity checking): per chain, the initial configuration and
   `len` (site, uniform) pairs consumed in order instead of Philox draws; u = 0
   marks a proposal the reference accepted without drawing. NULL sites disables. */
int ann_ens_set_tape(ann_ens* ens, const uint64_t* init_conf, const uint32_t* sites, const double* u,
                     unsigned len);
/* configurations of the last sampling call, num_steps x num_words */
int ann_ens_get_samples(const ann_ens* ens, uint64_t* conf, double* log_psi, double* local_energy);

/* ---------------------------------------------------------------------------------
 * Network functions (source/network_functions/*.cu.template)
 * ------------------------------------------------------------------------------ */
/* ExpectationValue.__call__(op, psi, ens) (ExpectationValue.cu.template:19-50) */
int ann_expectation(ann_op* op, ann_psi* psi, ann_ens* ens, void* stream, double* out2);
/* ExpectationValue.__call__(list[op], psi, ens) (ExpectationValue.cu.template:83-128) */
int ann_expectation_list(ann_op** ops, unsigned n_ops, ann_psi* psi, ann_ens* ens, void* stream, double* out);
/* ExpectationValue.fluctuation -> (sigma, <A>) (ExpectationValue.cu.template:175-216); out3 = sigma, re, im */
int ann_fluctuation(ann_op* op, ann_psi* psi, ann_ens* ens, void* stream, double* out3);
/* ExpectationValue.gradient -> (G, <A>) (ExpectationValue.cu.template:219-275) */
int ann_gradient(ann_op* op, ann_psi* psi, ann_ens* ens, void* stream, double* grad, double* value2);
/* ExpectationValue.exp_sigma_z (ExpectationValue.cu.template:52-81) */
int ann_exp_sigma_z(ann_op* op, ann_psi* psi, ann_ens* ens, void* stream, double* out2);
/* log_psi_s(psi, Spins) (PsiVector.cu.template:101-133) */
int ann_log_psi_s(ann_psi* psi, const uint64_t* conf, double* out2);
/* batched log psi of explicit configurations (n x num_words) */
int ann_log_psi_batch(ann_psi* psi, const uint64_t* confs, unsigned n, void* stream, double* out);
/* local energies E_loc(s) = sum_n c_n <s|P_n|s'> psi(s')/psi(s) of explicit configurations
   (n x num_words), the per-sample quantity of ExpectationValue (Operator.hpp:86-121) */
int ann_local_energies(ann_psi* psi, ann_op* op, const uint64_t* confs, unsigned n, void* stream, double* out);
/* psi_O_k(psi, Spins) (PsiOkVector.cu.template:40-74) */
int ann_psi_O_k(ann_psi* psi, const uint64_t* conf, double* out);
/* the same over Pauli strings (log_psi_s / psi_O_k with a PauliString, PsiVector.cu.template:191-197):
   `ab` holds (a, b) word pairs, one per string */
int ann_log_psi_paulis(ann_psi* psi, const uint64_t* ab, unsigned n, void* stream, double* out);
int ann_psi_O_k_paulis(ann_psi* psi, const uint64_t* ab, double* out);
int ann_local_energies_paulis(ann_psi* psi, ann_op* op, const uint64_t* ab, unsigned n, void* stream, double* out);
/* psi_O_k_vector(psi, esum): sum_s O_k(s), unweighted (PsiOkVector.cu.template:8-38) */
int ann_psi_O_k_vector(ann_psi* psi, ann_ens* ens, void* stream, double* out);
/* log_psi(psi, ens): sum_s w(s) log psi(s) (PsiVector.cu.template:73-99) */
int ann_log_psi(ann_psi* psi, ann_ens* ens, void* stream, double* out2);
/* psi_vector / log_psi_vector (PsiVector.cu.template:14-71); 2 * num_steps doubles */
int ann_psi_vector(ann_psi* psi, ann_ens* ens, void* stream, double* out);
int ann_log_psi_vector(ann_psi* psi, ann_ens* ens, void* stream, double* out);
/* norm(esum) = sqrt(sum_s |psi(s)|^2) (PsiNorm.cu.template:13-42) */
int ann_psi_norm(ann_psi* psi, ann_ens* ens, void* stream, double* out);
/* apply_operator(psi, op, ens): psi(s) E_loc(s) (ApplyOperator.cu.template:9-44) */
int ann_apply_operator(ann_psi* psi, ann_op* op, ann_ens* ens, void* stream, double* out);
/* activation_function(z, layer) (main.cpp.template:534-536) */
int ann_activation_function(double re, double im, unsigned layer, int activation, double* out2);

/* ---------------------------------------------------------------------------------
 * TDVP / SR (include/network_functions/TDVP.hpp, source/network_functions/TDVP.cu.template)
 * ------------------------------------------------------------------------------ */
#define ANN_S_FP32 0         /* centred O, FP32 SIMT complex HERK (the plain form) */
#define ANN_S_BF16 1         /* centred O, BF16 tcgen05 real-embedded HERK, FP32 accumulation */
#define ANN_S_BF16_SPLIT 2   /* as ANN_S_BF16 with hi+lo split products (three BF16 products) */

/* TDVP(num_params, gpu) (main.cpp.template:465-466) */
int ann_tdvp_create(unsigned num_params, ann_tdvp** out);
int ann_tdvp_destroy(ann_tdvp* tdvp);
int ann_tdvp_set_s_mode(ann_tdvp* tdvp, int mode);
/* eval(op, psi, ens): E, E2, <O>, F and S on the device (TDVP.cu.template:181-302) */
int ann_tdvp_eval(ann_tdvp* tdvp, ann_op* op, ann_psi* psi, ann_ens* ens, void* stream);
/* eval_F: E, E2, <O>, F only (TDVP.cu.template:305-334) */
int ann_tdvp_eval_F(ann_tdvp* tdvp, ann_op* op, ann_psi* psi, ann_ens* ens, void* stream);
/* results (S_matrix, F_vector, O_k_vector, var_H, total_weight: main.cpp.template:467-472) */
int ann_tdvp_get_S(ann_tdvp* tdvp, double* out);       /* num_params^2 complex, row-major */
int ann_tdvp_get_F(ann_tdvp* tdvp, double* out);
int ann_tdvp_get_O(ann_tdvp* tdvp, double* out);
int ann_tdvp_get_energy(ann_tdvp* tdvp, double* E2re_im, double* E2);
int ann_tdvp_get_total_weight(ann_tdvp* tdvp, double* out);
/* O_k_samples (main.cpp.template:472): num_steps x num_params complex */
int ann_tdvp_get_O_samples(ann_tdvp* tdvp, double* out);
/* S_dot_vector(vec, ens) (TDVP.cu.template:336-443), from the stored O samples */
int ann_tdvp_S_dot_vector(ann_tdvp* tdvp, const double* vec, void* stream, double* out);
/* E, <O> and F from caller-owned device arrays, allocating nothing. No counterpart in
   the reference. It exists for callers that cannot call cudaMalloc at this point:
   hosts whose allocator already owns the device memory (a raw cudaMalloc would fail or
   fragment their pool), and latency-critical loops where an allocation could
   synchronise the device. It computes what ann_tdvp_eval_F stores, with the same
   definitions: E = sum_s w_s E_s, <O>_k = sum_s w_s O_sk,
   F_k = sum_s w_s E_s conj(O_sk) - E conj(<O>_k).
   Inputs (device pointers): O_rows n_rows x ld complex64 (row-major, ld >= num_params),
   local_energies n_rows complex128, weights n_rows doubles or NULL for uniform_weight.
   Outputs (device pointers): O_mean and F num_params complex128, energy 1 complex128
   (may be NULL). Work is queued on `stream` (NULL = legacy default stream).
   Scratch is a fixed 4 MiB device array inside the library, held on every GPU that
   loads it until exit; num_params above 130,816 is rejected with ANN_ERR_INVALID.
   The first call on a device looks up that array's address with the device current,
   so make it before any stream capture. Every call shares the scratch: calls that
   overlap on the GPU (other streams or host threads) race. */
int ann_force_vector_noalloc(const void* O_rows, size_t n_rows, size_t ld, unsigned num_params,
                             const double* weights, double uniform_weight, const double* local_energies,
                             double* O_mean, double* F, double* energy, void* stream);
/* SR solver selection (no counterpart in the reference, which has no solver;
   TDVP.cu.template:181-302 leaves the solve to the caller).
   ANN_SOLVER_FP64: FP64 Cholesky of S + shift I on the GPU, two triangular solves and
     one step of iterative refinement (the default).
   ANN_SOLVER_MIXED: FP32 Cholesky of S + shift I, then iterative refinement with the
     residual F - (S + shift I) x formed against S (FP64 arithmetic, or double-float
     arithmetic with FP64 accumulation when S is held in complex64), until
     ||r|| / ||F|| <= tol or max_iter FP32 solves (default 10); converges to the FP64 answer when
     cond(S + shift I) * 6e-8 < 1. An eager solve that does not converge (or whose FP32
     factorisation meets a non-positive pivot) is redone with ANN_SOLVER_FP64; inside a
     captured graph it raises ANN_ERR_NUMERIC at the next status check instead, and a
     solution whose final ||r|| / ||F|| is not finite or above 1e-3 is replaced by zero, so
     the graph's SR update leaves the parameters unchanged.
   ANN_SOLVER_FP32: the FP32 factorisation and one FP32 solve, no refinement; its FP64
     residual is still measured and reported by ann_tdvp_solver_info.
   max_iter and tol apply to ANN_SOLVER_MIXED. */
#define ANN_SOLVER_FP64 0
#define ANN_SOLVER_MIXED 1
#define ANN_SOLVER_FP32 2  /* one FP32 Cholesky solve, no refinement (the plain FP32 form) */
int ann_tdvp_set_solver(ann_tdvp* tdvp, int solver, unsigned max_iter, double tol);
/* trailing update of the FP32 Cholesky of ANN_SOLVER_MIXED / ANN_SOLVER_FP32:
   ANN_CHOL_UPDATE_TC (default) on the tensor cores with split-TF32 products (tcgen05),
   ANN_CHOL_UPDATE_SIMT on the FP32 SIMT cores */
#define ANN_CHOL_UPDATE_SIMT 0
#define ANN_CHOL_UPDATE_TC 1
int ann_tdvp_set_chol_update(ann_tdvp* tdvp, int mode);

/* ---------------------------------------------------------------------------------
 * HilbertSpaceDistance (HilbertSpaceDistance(num_params, gpu), main.cpp.template:436-442;
 * source/network_functions/HilbertSpaceDistance.cu.template:16-168): distance between
 * psi_prime and U psi with U = op (is_unitary: U a unitary-like sum; otherwise exp of the
 * local energy), sampled from psi's ensemble; the gradient is with respect to the
 * parameters of psi_prime (num_params(psi_prime) complex values), scaled by 1 / distance^nu.
 * ------------------------------------------------------------------------------ */
int ann_hsd_distance(ann_psi* psi, ann_psi* psi_prime, ann_op* op, int is_unitary, ann_ens* ens, void* stream,
                     double* distance);
int ann_hsd_gradient(ann_psi* psi, ann_psi* psi_prime, ann_op* op, int is_unitary, ann_ens* ens, double nu,
                     void* stream, double* grad, double* distance);

/* ---------------------------------------------------------------------------------
 * PsiClassical, the variational classical network (PsiClassicalFP_1/_2, PsiClassicalANN_1/_2;
 * include/quantum_state/PsiClassical.hpp:48-260, main.cpp.template:207-268):
 * log psi(s) = log_prefactor + sum_k params_k h_k(s) (+ log psi_ref(s) for order 2), with
 * h_k(s) = sum over the strings of operator k of coeff <s|P|P s> (Operator::fast_local_energy,
 * Operator.hpp:122-133) and O_k = (h_k(s), O_ref(s)); params = [params_k | reference params].
 * The reference network (a PsiDeep of any depth) is copied; NULL = fully polarized (log psi_ref = 0).
 * ------------------------------------------------------------------------------ */
typedef struct {
    unsigned num_sites;              /* spins, <= 128 */
    unsigned n_features;             /* operators H_local, one feature each */
    const unsigned* feature_begin;   /* n_features + 1 offsets into the strings */
    unsigned num_words;              /* words per string, 1 or 2 */
    const uint64_t* a;               /* strings x num_words, Pauli (a, b) encoding as ann_op_create_pauli */
    const uint64_t* b;
    const double* coeff;             /* strings, interleaved complex */
    const double* params;            /* n_features complex */
    double log_prefactor[2];
    unsigned order;                  /* 1 or 2 */
    const ann_psi* ref;              /* order 2: reference PsiDeep (copied), or NULL */
    int precision;                   /* ANN_PREC_* without a reference (with one: the reference's) */
} ann_classical_desc;
int ann_psi_create_classical(const ann_classical_desc* desc, ann_psi** out);
/* log_prefactor of the reference part (ref_log_prefactor, main.cpp.template:224-231); either pointer may be NULL */
int ann_psi_ref_log_prefactor(ann_psi* psi, const double* set2, double* get2);

/* ---------------------------------------------------------------------------------
 * KullbackLeibler (KullbackLeibler(num_params, gpu), main.cpp.template:445-461;
 * source/network_functions/KullbackLeibler.cu.template:17-329) of psi (classical) against
 * psi_prime over psi_prime's ensemble: w = |psi/psi'|^2 w', d = log psi' - log psi - the mean
 * deviation of the previous call; deviations with |d|^2 <= threshold^2 are left out of the
 * deviation sums. value = sqrt(max(1e-8, <|d|^2> - |<d>|^2)); gradient (psi_prime's parameters)
 * = (<d conj(O)> - <d> conj(<O>)) / value^nu; noise as gradient_with_noise.
 * ------------------------------------------------------------------------------ */
int ann_kl_create(unsigned num_params, ann_kl** out);
int ann_kl_destroy(ann_kl* kl);
/* log_psi_scale (read / write property): log psi is scaled by it; either pointer may be NULL */
int ann_kl_log_psi_scale(ann_kl* kl, const double* set, double* get);
int ann_kl_value(ann_kl* kl, ann_psi* psi, ann_psi* psi_prime, ann_ens* ens, double threshold, void* stream,
                 double* value);
/* grad: num_params(psi_prime) complex; noise (num_params doubles) may be NULL */
int ann_kl_gradient(ann_kl* kl, ann_psi* psi, ann_psi* psi_prime, ann_ens* ens, double nu, double threshold,
                    void* stream, double* grad, double* noise, double* value);
/* total_weight and mean_deviation (2 doubles) of the last call */
int ann_kl_stats(const ann_kl* kl, double* total_weight, double* mean_deviation2);

/* ---------------------------------------------------------------------------------
 * Autotuner (no counterpart in the reference, whose launch shape is fixed: one CTA
 * per chain with blockDim = hidden width, include/ensembles/MonteCarlo.hpp:223-228).
 * ann_autotune times every candidate of each knob on the given workload (CUDA events,
 * median of repeats; the sampler runs on a copy of the ensemble) and stores the
 * fastest in the per-process tuning table that the launchers read:
 *   knob 0  sampler warps (chains) per CTA: 2, 4, 8
 *   knob 1  rows per FP32 slab of the <O> / F reductions: 128, 256, 512
 *   knob 2  FP32 Cholesky trailing update: 1 = 128 x 128 tcgen05 tiles, 0 = 64 x 64 SIMT
 *           (mixed / FP32 solvers without an explicit ann_tdvp_set_chol_update)
 *   knob 3  sampler weights W staged in shared memory (1) or read through L1 (0)
 *   knob 4  SMs the persistent tcgen05 trailing update leaves to the next panel: 0, 16, 32, 48, 64
 *   knob 5  tcgen05 trailing updates of rank 64 per panel (0) or rank 128 per pair of panels (1;
 *           n even)
 * report (3 doubles per timed candidate: knob, candidate, median ms) may be NULL;
 * n_report receives the number of rows. Table keys are "dev<ordinal>/<knob>/<shape>". */
int ann_autotune(ann_tdvp* tdvp, ann_op* op, ann_psi* psi, ann_ens* ens, double diag_shift, void* stream,
                 double* report, unsigned report_cap, unsigned* n_report);
int ann_tuning_set(const char* key, int value);
int ann_tuning_get(const char* key, int* value, int* found);
/* "key value" lines; len receives the full length (call with buf NULL to size it) */
int ann_tuning_dump(char* buf, size_t cap, size_t* len);
int ann_tuning_clear(void);
/* after a solve: out4 = {FP32 solves used, relative FP64 residual after the first and
   after the last solve, 1 if the FP64 solve replaced a stalled mixed solve}
   (ANN_SOLVER_FP64: {1, residual before refinement, after, 0}) */
int ann_tdvp_solver_info(ann_tdvp* tdvp, double* out4);
/* the factorisation form of the last FP32 Cholesky: 0 none (ANN_SOLVER_FP64 or no solve
   yet), 1 FP32 SIMT trailing updates, 2 tensor-core trailing update per 64-column panel,
   3 tensor-core trailing update per pair of panels (rank 128). No counterpart in the
   reference, which has no solver (source/network_functions/TDVP.cu.template:181-302). */
#define ANN_CHOL_FORM_NONE 0
#define ANN_CHOL_FORM_SIMT 1
#define ANN_CHOL_FORM_TC_PANEL 2
#define ANN_CHOL_FORM_TC_PAIR 3
int ann_tdvp_solver_form(const ann_tdvp* tdvp, int* form);
/* SR solve: (S + shift I) delta = F on the GPU with the configured solver; writes delta
   (num_params complex) if out != NULL and the relative residuals ||F - (S + shift I) x|| /
   ||F|| of the first and the final solution to info2 if info2 != NULL. */
int ann_tdvp_solve(ann_tdvp* tdvp, double diag_shift, void* stream, double* delta_out, double* info2);
/* SR update: params <- params - lr * delta (device resident; re-derives kernel weights) */
int ann_sr_update(ann_tdvp* tdvp, ann_psi* psi, double lr, void* stream);
/* one full SR step = eval + solve + update, on the device */
int ann_sr_step(ann_tdvp* tdvp, ann_op* op, ann_psi* psi, ann_ens* ens, double diag_shift, double lr,
                void* stream);

/* ---------------------------------------------------------------------------------
 * Learned proposal: masked autoregressive MLP (MADE, one hidden layer of width H,
 * BF16 weights in the kernels, FP32 master weights, accumulation and Adam moments).
 * Not in the reference; this project's own component.
 * Weight layouts: W1 H x N, b1 H, W2 N x H, b2 N (float). Configurations as
 * 2-word rows (uint64 x 2, bit i = spin up at site i).
 * ------------------------------------------------------------------------------ */
int ann_made_create(unsigned N, unsigned H, uint64_t seed, ann_made** out);
int ann_made_destroy(ann_made* m);
int ann_made_get_params(const ann_made* m, float* W1, float* b1, float* W2, float* b2);
int ann_made_set_params(ann_made* m, const float* W1, const float* b1, const float* W2, const float* b2);
/* log q(s) of n configurations */
int ann_made_log_prob(ann_made* m, const uint64_t* confs, unsigned n, double* out);
/* n samples s ~ q with Philox key `seed`, sample indices first .. first + n - 1 */
int ann_made_sample(ann_made* m, unsigned n, uint64_t seed, uint64_t first, uint64_t* confs, double* logq);
/* gradient of the mean -log q over n configurations (unmasked entries), and the loss */
int ann_made_gradient(ann_made* m, const uint64_t* confs, unsigned n, float* gW1, float* gb1, float* gW2,
                      float* gb2, double* loss);
/* `steps` Adam steps (learning rate lr) over batches of `batch` configurations */
int ann_made_train(ann_made* m, const uint64_t* confs, unsigned n, unsigned steps, unsigned batch, double lr,
                   void* stream, double* loss);
/* same, on the configurations the ensemble's chains produced (its history buffer if set) */
int ann_made_train_on_samples(ann_made* m, const ann_ens* ens, unsigned steps, unsigned batch, double lr,
                              void* stream, double* loss);

/* ---------------------------------------------------------------------------------
 * Batched uneven instances (no counterpart in the reference, which runs one
 * Hamiltonian per call): n (psi, op, Monte Carlo ensemble, TDVP) tuples; complex64
 * RBM-family wavefunctions with N <= 64 and M <= 256, single-flip ensembles. One
 * persistent launch samples every instance (device work queue, largest first);
 * the per-instance S, Cholesky solves and updates run on a stream pool.
 * ------------------------------------------------------------------------------ */
int ann_batch_create(unsigned n, ann_psi** psis, ann_op** ops, ann_ens** enss, ann_tdvp** tdvps, ann_batch** out);
int ann_batch_destroy(ann_batch* b);
/* sampling + local energies (+ O rows for instances with a TDVP) of every instance */
int ann_batch_sample(ann_batch* b, void* stream);
/* <H> of every instance from its last samples (2 n doubles) */
int ann_batch_energies(ann_batch* b, double* out);
/* one SR step of every instance (sample, S, F, FP64 Cholesky solve, update) */
int ann_batch_sr_step(ann_batch* b, double diag_shift, double lr, void* stream);
/* capture the batched SR step as one CUDA graph (runs one eager step first); replay */
int ann_batch_graph_capture(ann_batch* b, double diag_shift, double lr, void* stream);
int ann_batch_graph_launch(ann_batch* b, void* stream);

/* ---------------------------------------------------------------------------------
 * CUDA graph of a whole SR step (capture once, replay many)
 * ------------------------------------------------------------------------------ */
int ann_sr_graph_capture(ann_tdvp* tdvp, ann_op* op, ann_psi* psi, ann_ens* ens, double diag_shift, double lr,
                         void* stream);
int ann_sr_graph_launch(ann_tdvp* tdvp, void* stream);

/* CUDA-event timing of the SR-step phases on the calling stream (not inside graph
   capture): ms[0] sampling + local energy + O rows, ms[1] reductions (E, <O>, F),
   ms[2] S matrix, ms[3] SR solve, ms[4] update; -1 where a phase did not run */
int ann_set_phase_timing(int enable);
int ann_get_phase_times(float* ms5);
/* with phase timing on: duration (ms) of the FP32 Cholesky factorisation inside the
   last mixed / FP32 SR solve (-1 if none was timed) */
int ann_get_solve_times(float* ms1);
/* event timeline of the FP32 Cholesky factorisation (this project's diagnostic): with the
   trace on (enable 1 or 2), every mixed / FP32 factorisation outside graph capture records
   tagged CUDA events; ann_get_factor_trace writes (tag, ms since the first event) pairs of
   the last one. Tags: 200 / 201 tile-column update of the next panel pair start / end, 202
   rest of the trailing update done, 203 main stream joined with the look-ahead stream (main
   stream); 100 panel pair start, 103 panel pair done (look-ahead stream). Level 2 adds 110
   after each diagonal-block factorisation and 101 after the first panel of a pair; those
   events sit between panel kernels that otherwise start early as programmatic dependent
   launches, so level 2 times the panel kernels one after the other. */
int ann_set_factor_trace(int enable);
int ann_get_factor_trace(double* out, unsigned cap, unsigned* n);

/* kernels this library launched so far (monotonic counter of its own launches) */
unsigned long long ann_kernel_launch_count(void);
/* device status word of the last computation (ANN bit flags; 0 = clean) */
int ann_status(unsigned* out);

#ifdef __cplusplus
}
#endif

#endif /* ANNONGPU_H */
