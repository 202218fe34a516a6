// FP64 CPU restatement of the reference's VMC inner loop -- TEST INFRASTRUCTURE.
//
// This library is the checker: only tests/, __graft_entry__.smoke() and the
// cpu_baseline / --impl reference legs of bench.py may load it. The product
// (annongpu_gb300/) never links, loads or calls it.
//
// Parity anchors (reference file:line):
//   Pauli string apply ............ include/basis/PauliString.hpp:193-208, 242-254
//   local energy .................. include/operator/Operator.hpp:36-121
//   polynomial log cosh / tanh .... include/quantum_state/psi_functions.hpp:40-48, 102-116
//   PsiRBM ........................ include/quantum_state/PsiRBM.hpp:69-176
//   PsiDeep (1 hidden layer) ...... include/quantum_state/PsiDeep.hpp:138-445,
//                                   source/quantum_state/PsiDeep.cu:142-305
//   PsiDeep (any depth) ........... include/quantum_state/PsiDeep.hpp:171-215 (forward),
//                                   :345-445 (O_k back-propagation),
//                                   source/quantum_state/PsiDeep.cu:142-183 (parameter layout)
//   PsiCNN ........................ include/quantum_state/PsiCNN.hpp:97-266,
//                                   include/quantum_state/detail/Convolve.hpp:15-173
//   MonteCarlo host path .......... include/ensembles/MonteCarlo.hpp:55-177,
//                                   include/random.h:21-54, source/RNGStates.cu:47-51
//   ExactSummation ................ include/ensembles/ExactSummation.hpp:33-72
//   ExpectationValue .............. source/network_functions/ExpectationValue.cu.template:19-50,175-275
//   TDVP .......................... source/network_functions/TDVP.cu.template:77-126,181-302,336-443
//   psi_norm / log_psi / vectors .. source/network_functions/PsiNorm.cu.template:13-42,
//                                   PsiVector.cu.template:14-133, PsiOkVector.cu.template:8-74
// Parity is pinned against the reference's own host code (oracle/ref_harness.cu)
// through the fixtures in tests/golden/.
#pragma once
#include <cstdint>

extern "C" {

// Pauli-sum operator. String n occupies words [n*nw, n*nw + nw) of a and b.
// Encoding per site (PauliString.hpp:37-56): (a,b) = (0,0) I, (1,0) X, (0,1) Y, (1,1) Z.
struct or_op {
    unsigned n;
    unsigned nw;
    const uint64_t* a;
    const uint64_t* b;
    const double* coeff;  // interleaved re, im
};

// RBM family: the reference PsiRBM (params = W) and PsiDeep with one hidden layer
// (params = [a | b | W]).
struct or_rbm {
    unsigned N, M, C;
    const unsigned* conn;  // C x M, entry (c, j) -> input site; NULL = identity (C == N)
    const double* a;       // N complex (may be NULL: zero)
    const double* b;       // M complex (may be NULL: zero)
    const double* W;       // C*M complex, entry (c, j) at c*M + j
    const double* fw;      // M complex final weights
    double lp_re, lp_im;   // log prefactor
    int a_in_log_psi;      // 1: log psi includes a.s ; 0: reference PsiDeep (PsiDeep.hpp:260-264)
    int activation;        // 0: reference polynomial ; 1: exact log cosh
    int layout;            // 0: params = W only (PsiRBM) ; 1: params = [a | b | W] (PsiDeep)
};

// Convolutional network (PsiCNN): periodic 3-d convolutions, forward-anchored windows.
struct or_cnn {
    unsigned extent[3];
    unsigned num_layers;
    const unsigned* channels;      // num_layers
    const unsigned* connectivity;  // num_layers x 3
    const unsigned* sym_classes;   // N
    const double* params;          // interleaved complex
    unsigned num_params;
    double final_factor;
    double lp_re, lp_im;
    int activation;                // 0: reference layer polynomials ; 1: log cosh on every layer
};

// PsiDeep with any number of hidden layers. Layer l (0-based) has sizes[l] units;
// unit j of layer l reads connectivity[l] units of the layer below (the spins for
// l = 0): entry (i, j) of its connection block is the index of the i-th of them.
// params = [a(N) | b_0 | W_0 | b_1 | W_1 | ...], W_l entry (i, j) at i*sizes[l] + j.
// log psi = lp (+ a.s) + sum_j fw_j f_L(z_L,j); f on layer 0 is the log-cosh
// polynomial, on deeper layers the odd (tanh-like) polynomial.
struct or_deep {
    unsigned N;
    unsigned num_layers;
    const unsigned* sizes;         // num_layers
    const unsigned* connectivity;  // num_layers
    const unsigned* connections;   // concatenated blocks, connectivity[l] x sizes[l] each
    const double* params;          // interleaved complex
    const double* fw;              // sizes[num_layers - 1] complex final weights
    double lp_re, lp_im;
    int a_in_log_psi;              // 0 reproduces the reference (PsiDeep.hpp:260-264)
    int activation;                // 0: reference layer polynomials ; 1: log cosh on every layer
    int basis;                     // 0 spins (conf = bits); 1 Pauli strings (conf = words a, b; N = 3 x sites)
};

unsigned or_rbm_num_params(const or_rbm* p);
void or_rbm_log_psi(const or_rbm* p, const uint64_t* conf, double* out);
void or_rbm_O_k(const or_rbm* p, const uint64_t* conf, double* out);
void or_rbm_local_energy(const or_rbm* p, const or_op* op, const uint64_t* conf, double* out);

// Exact summation over all 2^N configurations; any output pointer may be NULL.
void or_rbm_exact(const or_rbm* p, const or_op* op,
                  double* E, double* fluct, double* grad,
                  double* tE, double* tE2, double* tO, double* tF, double* tS,
                  double* vec, double* log_vec, double* norm, double* mean_log_psi, double* O_sum,
                  double* eloc_vec);

// The reference host Monte Carlo, including its std::mt19937 draws, for one chain
// seeded with `seed`. Returns the number of proposals recorded.
unsigned or_rbm_mc_reference(const or_rbm* p, const or_op* op, unsigned num_samples, unsigned num_sweeps,
                             unsigned num_therm, unsigned seed,
                             uint64_t* sconf, double* slp, double* seloc,
                             uint64_t* pconf, uint32_t* psite, double* pu, uint8_t* pacc,
                             unsigned max_props, double* mc_energy);

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).
void or_philox4x32_10(uint32_t k0, uint32_t k1, const uint32_t* ctr, uint32_t* out);

// Counter-based Metropolis chains as this project's sampler defines them
// (move_kind 0 = single flip, 1 = exchange over bonds, 2 = exchange over random pairs).
// Chain state in/out: conf[n_chains*nw], counter[n_chains]. If init != 0 the
// configurations are drawn first (n_up < 0: uniform; n_up >= 0: exactly n_up up spins)
// and num_therm sweeps run before the first sample.
void or_rbm_mc_philox(const or_rbm* p, const or_op* op, unsigned n_chains, uint64_t seed,
                      unsigned samples_per_chain, unsigned num_sweeps, unsigned num_therm,
                      int move_kind, const uint32_t* bonds, unsigned n_bonds, int init, int n_up,
                      uint64_t* conf, uint64_t* counter,
                      uint64_t* sconf, double* slp, double* seloc,
                      uint64_t* n_accept, uint64_t* n_reject, double* min_tie);

// The reference's TDVP accumulation (TDVP.cu.template:77-126, 216-301) over given
// configurations with a uniform weight: E, E2, <O>, F and (if tS != NULL) S.
void or_rbm_tdvp_samples(const or_rbm* p, const or_op* op, const uint64_t* confs, unsigned n, double weight,
                         double* E, double* tE2, double* tO, double* tF, double* tS);

// PsiCNN (reference activation semantics: layer 0 poly log cosh, deeper layers odd poly)
void or_cnn_log_psi(const or_cnn* p, const uint64_t* conf, double* out);
void or_cnn_O_k(const or_cnn* p, const uint64_t* conf, double* out);
void or_cnn_local_energy(const or_cnn* p, const or_op* op, const uint64_t* conf, double* out);
void or_cnn_exact(const or_cnn* p, const or_op* op, double* E, double* norm,
                  double* tE, double* tE2, double* tO, double* tF, double* tS);
// counter-based chains (same contract as or_rbm_mc_philox); dlogpsi from full forward passes
void or_cnn_mc_philox(const or_cnn* p, const or_op* op, unsigned n_chains, uint64_t seed,
                      unsigned samples_per_chain, unsigned num_sweeps, unsigned num_therm,
                      int move_kind, const uint32_t* bonds, unsigned n_bonds, int init, int n_up,
                      uint64_t* conf, uint64_t* counter,
                      uint64_t* sconf, double* slp, double* seloc,
                      uint64_t* n_accept, uint64_t* n_reject, double* min_tie);

unsigned or_deep_num_params(const or_deep* p);
void or_deep_log_psi(const or_deep* p, const uint64_t* conf, double* out);
void or_deep_O_k(const or_deep* p, const uint64_t* conf, double* out);
void or_deep_local_energy(const or_deep* p, const or_op* op, const uint64_t* conf, double* out);
void or_deep_exact(const or_deep* p, const or_op* op, double* E, double* norm,
                   double* tE, double* tE2, double* tO, double* tF, double* tS);
// counter-based chains (same contract as or_rbm_mc_philox); dlogpsi from full forward passes.
// Pauli-string basis (basis = 1; move_kind, bonds and n_up unused): initial string at counter
// (t, chain, 1): a = r0 | r1 << 32, b = r2 | r3 << 32 masked to N/3 sites; proposal t at
// (t, chain, 0): site mulhi(r0, N/3) set to type r1 >> 30 (the reference draws x % sites and
// x >> 30 from one word, Update_Policy.hpp:41-57), u from (r2, r3); a sweep is N proposals.
void or_deep_mc_philox(const or_deep* p, const or_op* op, unsigned n_chains, uint64_t seed,
                       unsigned samples_per_chain, unsigned num_sweeps, unsigned num_therm,
                       int move_kind, const uint32_t* bonds, unsigned n_bonds, int init, int n_up,
                       uint64_t* conf, uint64_t* counter,
                       uint64_t* sconf, double* slp, double* seloc,
                       uint64_t* n_accept, uint64_t* n_reject, double* min_tie);

// PsiClassical (vCN, include/quantum_state/PsiClassical.hpp:48-163): features h_k(s) =
// fast_local_energy of operator k = sum of its strings' c <s|P|s'> (Operator.hpp:122-133);
// log psi = lp + sum_k params_k h_k(s) (+ log psi_ref(s) for order 2), O_k = (h_k(s), O_ref).
// params = [params_k | ref params] (PsiClassical.cu:37-60). ref NULL: fully polarized (log psi_ref = 0).
struct or_classical {
    unsigned num_sites;
    unsigned n_features;
    const unsigned* feat_begin;    // n_features + 1 offsets into the strings
    unsigned nw;                   // words per string
    const uint64_t* a;             // strings x nw
    const uint64_t* b;
    const double* coeff;           // strings complex
    const double* params;          // n_features complex
    double lp_re, lp_im;
    int order;                     // 1 or 2
    const or_deep* ref;            // reference network (order 2), or NULL
};
unsigned or_classical_num_params(const or_classical* p);
void or_classical_log_psi(const or_classical* p, const uint64_t* conf, double* out);
void or_classical_O_k(const or_classical* p, const uint64_t* conf, double* out);
void or_classical_local_energy(const or_classical* p, const or_op* op, const uint64_t* conf, double* out);
void or_classical_exact(const or_classical* p, const or_op* op, double* E, double* norm,
                        double* tE, double* tE2, double* tO, double* tF, double* tS);

// KullbackLeibler (source/network_functions/KullbackLeibler.cu.template:17-329) of psi
// (classical) against psi_prime over psi_prime's ensemble: rows (conf, w') given, or all 2^N
// configurations with w' = |psi'(s)|^2 when confs is NULL. w = |psi/psi'|^2 w',
// d = log psi' - log psi - last_mean (deviations with |d|^2 <= threshold^2 skipped in the
// deviation sums). Outputs value, gradient (psi_prime's parameters), noise (if non-NULL),
// total weight and the new mean deviation.
void or_kl(const or_classical* psi, const or_deep* psi_prime, const uint64_t* confs, const double* wprime,
           unsigned n, double threshold, const double* last_mean, double log_psi_scale, double nu,
           double* value, double* grad, double* noise, double* total_weight, double* mean_deviation);

// Pauli application, single string (for KATs).
void or_pauli_apply(const uint64_t* a, const uint64_t* b, unsigned nw, const uint64_t* conf,
                    double* factor, uint64_t* out_conf);

// activations (layer semantics as psi_functions.hpp)
void or_activation(double re, double im, unsigned layer, int exact, double* f, double* df);

}  // extern "C"
