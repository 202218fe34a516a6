// FP64 CPU restatement of the reference's VMC inner loop -- TEST INFRASTRUCTURE.
// See oracle.hpp for the reference file:line anchors and the usage rule: only
// tests/, __graft_entry__.smoke() and bench.py's CPU legs load this library.
#include "oracle.hpp"

#include <algorithm>
#include <array>
#include <cmath>
#include <complex>
#include <cstring>
#include <memory>
#include <random>
#include <vector>

namespace {

using cd = std::complex<double>;
using Conf = std::array<uint64_t, 2>;

inline cd cx(const double* p, size_t k) { return p ? cd(p[2 * k], p[2 * k + 1]) : cd(0.0, 0.0); }
inline void put(double* out, cd z) { out[0] = z.real(); out[1] = z.imag(); }
inline int popc(uint64_t x) { return __builtin_popcountll(x); }
inline unsigned nwords(unsigned N) { return (N + 63u) / 64u; }

inline double spin(const Conf& s, unsigned i) { return ((s[i >> 6] >> (i & 63u)) & 1u) ? 1.0 : -1.0; }
inline Conf load_conf(const uint64_t* c, unsigned nw) {
    Conf s{0, 0};
    for(unsigned w = 0; w < nw; w++) s[w] = c[w];
    return s;
}
inline Conf enumerate(uint64_t idx) { return Conf{idx, 0}; }

// ---- activations: psi_functions.hpp:40-48 (my_logcosh) and :102-116 (my_tanh) ----
inline cd poly_f(cd z, unsigned layer) {
    const cd z2 = z * z, z4 = z2 * z2;
    if(layer == 0u) return 0.5 * z2 - (1.0 / 12.0) * z4 + (1.0 / 45.0) * z4 * z2;
    return z - (1.0 / 3.0) * z2 * z + (2.0 / 15.0) * z4 * z;
}
inline cd poly_df(cd z, unsigned layer) {
    const cd z2 = z * z, z4 = z2 * z2;
    if(layer == 0u) return z - (1.0 / 3.0) * z2 * z + (2.0 / 15.0) * z4 * z;
    return 1.0 - z2 + (2.0 / 3.0) * z4;
}
// log cosh z, evaluated as |Re z| + log1p(exp(-2|z|')) - log 2 with the branch
// chosen by the sign of Re z (cosh is even).
inline cd exact_logcosh(cd z) {
    const cd w = z.real() >= 0.0 ? z : -z;
    return w + std::log(1.0 + std::exp(-2.0 * w)) - std::log(2.0);
}
inline cd act_f(cd z, unsigned layer, int exact) { return exact ? exact_logcosh(z) : poly_f(z, layer); }
inline cd act_df(cd z, unsigned layer, int exact) { return exact ? std::tanh(z) : poly_df(z, layer); }

// ---- Pauli strings: PauliString.hpp:193-208 (prefactor) and :242-254 (apply) ----
struct ME {
    cd factor;
    Conf conf;
};
inline ME pauli_apply(const uint64_t* a, const uint64_t* b, unsigned nw, const Conf& s) {
    int ny = 0, neg = 0;
    Conf out = s;
    for(unsigned w = 0; w < nw; w++) {
        const uint64_t y = (~a[w]) & b[w];
        const uint64_t z = a[w] & b[w];
        ny += popc(y);
        neg += popc((~s[w]) & (z | y));
        out[w] ^= (a[w] ^ b[w]);
    }
    cd f(1.0, 0.0);
    if((ny & 3) > 1) f *= -1.0;
    if(ny & 1) f *= cd(0.0, -1.0);
    if(neg & 1) f *= -1.0;
    return {f, out};
}

// ---- RBM family ----
struct Rbm {
    const or_rbm* p;
    unsigned N, M, C;
    std::vector<unsigned> conn;
    std::vector<cd> a, b, W, fw;
    cd lp;
    // input-site -> (unit, weight) lists in the order the reference compiles them
    // (PsiDeep.cu:213-242): units ascending, connections ascending within a unit.
    std::vector<std::vector<std::pair<unsigned, cd>>> rhs;

    explicit Rbm(const or_rbm* p_) : p(p_), N(p_->N), M(p_->M), C(p_->C) {
        conn.resize(C * M);
        for(unsigned k = 0; k < C * M; k++) conn[k] = p->conn ? p->conn[k] : k / M;
        a.resize(N); b.resize(M); W.resize(C * M); fw.resize(M);
        for(unsigned i = 0; i < N; i++) a[i] = C_(p->a, i);
        for(unsigned j = 0; j < M; j++) { b[j] = C_(p->b, j); fw[j] = C_(p->fw, j); }
        for(unsigned k = 0; k < C * M; k++) W[k] = C_(p->W, k);
        lp = cd(p->lp_re, p->lp_im);
        rhs.assign(N, {});
        for(unsigned j = 0; j < M; j++)
            for(unsigned c = 0; c < C; c++) rhs[conn[c * M + j]].push_back({j, W[c * M + j]});
    }
    static cd C_(const double* x, size_t k) { return cx(x, k); }
    bool is_deep() const { return p->layout == 1; }
    unsigned num_params() const { return is_deep() ? N + M + C * M : C * M; }

    // PsiRBM.hpp:69-80 / PsiDeep.hpp:138-157
    void angles(const Conf& s, std::vector<cd>& th) const {
        th.assign(M, cd(0.0));
        for(unsigned j = 0; j < M; j++) {
            cd acc(0.0);
            for(unsigned c = 0; c < C; c++) acc += W[c * M + j] * spin(s, conn[c * M + j]);
            if(is_deep()) acc += b[j];
            th[j] = acc;
        }
    }
    // PsiRBM.hpp:90-119 / PsiDeep.hpp:171-266 (+ a.s when a_in_log_psi)
    cd log_psi(const Conf& s, const std::vector<cd>& th) const {
        cd r = lp;
        for(unsigned j = 0; j < M; j++) r += act_f(th[j], 0, p->activation) * fw[j];
        if(p->a_in_log_psi)
            for(unsigned i = 0; i < N; i++) r += a[i] * spin(s, i);
        return r;
    }
    // PsiRBM.hpp:121-157 / PsiDeep.hpp:268-343: one update per differing site, ascending
    void update(std::vector<cd>& th, const Conf& from, const Conf& to) const {
        for(unsigned w = 0; w < 2; w++) {
            uint64_t d = from[w] ^ to[w];
            while(d) {
                const unsigned pos = 64u * w + __builtin_ctzll(d);
                d &= d - 1;
                const double ds = spin(to, pos) - spin(from, pos);
                for(const auto& e : rhs[pos]) th[e.first] += ds * e.second;
            }
        }
    }
    // PsiRBM.hpp:159-176 / PsiDeep.hpp:345-445 (one hidden layer)
    void O_k(const Conf& s, std::vector<cd>& out) const {
        std::vector<cd> th;
        angles(s, th);
        out.assign(num_params(), cd(0.0));
        const unsigned off = is_deep() ? N + M : 0u;
        if(is_deep()) {
            for(unsigned i = 0; i < N; i++) out[i] = spin(s, i);
        }
        for(unsigned j = 0; j < M; j++) {
            const cd g = fw[j] * act_df(th[j], 0, p->activation);
            if(is_deep()) out[N + j] = g;
            for(unsigned c = 0; c < C; c++) out[off + c * M + j] += g * spin(s, conn[c * M + j]);
        }
    }
};

// Operator::local_energy (Operator.hpp:36-121): update, full log psi, revert.
template<typename Psi, typename Payload>
cd local_energy_incremental(const Psi& psi, const or_op* op, const Conf& s, cd log_psi, Payload& th) {
    cd r(0.0);
    for(unsigned n = 0; n < op->n; n++) {
        ME me = pauli_apply(op->a + n * op->nw, op->b + n * op->nw, op->nw, s);
        me.factor *= cx(op->coeff, n);
        if(me.conf != s) {
            psi.update(th, s, me.conf);
            const cd lpp = psi.log_psi(me.conf, th);
            r += me.factor * std::exp(lpp - log_psi);
            psi.update(th, me.conf, s);
        } else {
            r += me.factor;
        }
    }
    return r;
}

struct Accum {
    unsigned np;
    cd E{0.0}, A2{0.0};
    double E2 = 0.0;
    std::vector<cd> O, F, S, gO, gF, Osum;
    explicit Accum(unsigned np_) : np(np_), O(np_), F(np_), S((size_t)np_ * np_), gO(np_), gF(np_), Osum(np_) {}
    void add(double w, cd eloc, const std::vector<cd>& Ok, bool want_S) {
        E += w * eloc;
        E2 += w * std::norm(eloc);
        for(unsigned k = 0; k < np; k++) {
            O[k] += w * Ok[k];
            F[k] += w * eloc * std::conj(Ok[k]);
            gO[k] += w * std::conj(Ok[k]);
            gF[k] += w * std::conj(Ok[k]) * eloc;
            Osum[k] += Ok[k];
        }
        if(want_S)
            for(unsigned k = 0; k < np; k++) {
                const cd ck = w * std::conj(Ok[k]);
                cd* row = &S[(size_t)k * np];
                for(unsigned l = 0; l < np; l++) row[l] += ck * Ok[l];
            }
    }
    void finish(double* fluct, double* grad, double* tE, double* tE2, double* tO, double* tF, double* tS) {
        if(fluct) { fluct[0] = std::sqrt(E2 - std::norm(E)); put(fluct + 1, E); }
        if(grad) for(unsigned k = 0; k < np; k++) put(grad + 2 * k, gF[k] - E * gO[k]);
        if(tE) put(tE, E);
        if(tE2) tE2[0] = E2;
        if(tO) for(unsigned k = 0; k < np; k++) put(tO + 2 * k, O[k]);
        if(tF) for(unsigned k = 0; k < np; k++) put(tF + 2 * k, F[k] - E * std::conj(O[k]));
        if(tS)
            for(unsigned k = 0; k < np; k++)
                for(unsigned l = 0; l < np; l++)
                    put(tS + 2 * ((size_t)k * np + l), S[(size_t)k * np + l] - std::conj(O[k]) * O[l]);
    }
};

// ---- Philox4x32-10 ----
inline void philox(uint32_t k0, uint32_t k1, const uint32_t* ctr, uint32_t* out) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    for(int r = 0; r < 10; r++) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        const uint32_t n1 = (uint32_t)p1;
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        const uint32_t n3 = (uint32_t)p0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}
inline uint32_t mulhi(uint32_t r, uint32_t n) { return (uint32_t)(((uint64_t)r * n) >> 32); }
inline double u53(uint32_t lo, uint32_t hi) { return (double)((((uint64_t)hi << 32) | lo) >> 11) * 0x1.0p-53; }

inline Conf mask_conf(Conf s, unsigned N) {
    for(unsigned w = 0; w < 2; w++) {
        const unsigned lo = 64u * w;
        if(N <= lo) s[w] = 0;
        else if(N - lo < 64u) s[w] &= ((uint64_t)1 << (N - lo)) - 1u;
    }
    return s;
}

// Sampler random-number contract (shared with the CUDA sampler):
//   key = (seed & 0xffffffff, seed >> 32)
//   initial configuration at chain counter t: counter (t_lo, t_hi, chain, 1) ->
//       words (r0 | r1 << 32, r2 | r3 << 32), masked to N sites
//   fixed-magnetisation init: draw k uses counter (t + k, chain, 2): set the
//       mulhi(r0, N - k)-th down spin up
//   proposal t: counter (t_lo, t_hi, chain, 0): r0 -> first site, r1 -> partner,
//       (r2, r3) -> uniform u in [0, 1) with 53 bits; accept iff u <= exp(2 Re dlogpsi)
Conf draw_initial(uint32_t k0, uint32_t k1, unsigned chain, unsigned N, int n_up, uint64_t t) {
    if(n_up < 0) {
        uint32_t ctr[4] = {(uint32_t)t, (uint32_t)(t >> 32), chain, 1u}, r[4];
        philox(k0, k1, ctr, r);
        Conf s{(uint64_t)r[0] | ((uint64_t)r[1] << 32), (uint64_t)r[2] | ((uint64_t)r[3] << 32)};
        return mask_conf(s, N);
    }
    Conf s{0, 0};
    for(int k = 0; k < n_up; k++) {
        const uint64_t tk = t + (uint64_t)k;
        uint32_t ctr[4] = {(uint32_t)tk, (uint32_t)(tk >> 32), chain, 2u}, r[4];
        philox(k0, k1, ctr, r);
        unsigned target = mulhi(r[0], N - (unsigned)k);
        for(unsigned i = 0; i < N; i++) {
            if(!((s[i >> 6] >> (i & 63u)) & 1u)) {
                if(target == 0) { s[i >> 6] |= (uint64_t)1 << (i & 63u); break; }
                target--;
            }
        }
    }
    return s;
}


// ---- PsiCNN: PsiCNN.hpp:97-266, Convolve.hpp:110-173, PsiCNN.cpp:9-55 ----
struct Cnn {
    const or_cnn* p;
    unsigned N, L, e[3];
    std::vector<unsigned> ch, vol, link_off;  // link_off[l] = first param of layer l
    unsigned ncls;
    std::vector<cd> w;
    cd lp;
    explicit Cnn(const or_cnn* p_) : p(p_) {
        for(int d = 0; d < 3; d++) e[d] = p->extent[d];
        N = e[0] * e[1] * e[2];
        L = p->num_layers;
        std::vector<unsigned> cls(p->sym_classes, p->sym_classes + N);
        std::sort(cls.begin(), cls.end());
        ncls = (unsigned)(std::unique(cls.begin(), cls.end()) - cls.begin());
        unsigned off = 0;
        for(unsigned l = 0; l < L; l++) {
            ch.push_back(p->channels[l]);
            unsigned v = 1;
            for(int d = 0; d < 3; d++) v *= p->connectivity[3 * l + d];
            vol.push_back(v);
            link_off.push_back(off);
            off += ch[l] * (l ? ch[l - 1] : 1u) * ncls * v;
        }
        w.resize(p->num_params);
        for(unsigned k = 0; k < p->num_params; k++) w[k] = cx(p->params, k);
        lp = cd(p->lp_re, p->lp_im);
    }
    unsigned prev(unsigned l) const { return l ? ch[l - 1] : 1u; }
    unsigned link_begin(unsigned l, unsigned ci, unsigned cj) const {
        return link_off[l] + (ci * ch[l] + cj) * ncls * vol[l];
    }
    // forward-anchored periodic window (Convolve<3>::foreach_connection)
    template<typename F>
    void window(unsigned l, unsigned x, F f) const {
        const unsigned* cn = p->connectivity + 3 * l;
        const unsigned page_size = e[1] * e[2];
        const unsigned pg = x / page_size, row = (x % page_size) / e[2], col = (x % page_size) % e[2];
        unsigned c = 0;
        for(unsigned k = 0; k < cn[0]; k++)
            for(unsigned i = 0; i < cn[1]; i++)
                for(unsigned j = 0; j < cn[2]; j++) {
                    f(c, ((pg + k) % e[0]) * page_size + ((row + i) % e[1]) * e[2] + ((col + j) % e[2]));
                    c++;
                }
    }
    cd f(cd z, unsigned l) const { return p->activation ? exact_logcosh(z) : poly_f(z, l); }
    cd df(cd z, unsigned l) const { return p->activation ? std::tanh(z) : poly_df(z, l); }
    // returns log psi; angles[l][c*N + x] recorded
    cd forward(const Conf& s, std::vector<std::vector<cd>>& ang) const {
        std::vector<cd> in(N);
        for(unsigned x = 0; x < N; x++) in[x] = spin(s, x);
        ang.assign(L, {});
        cd r = lp;
        for(unsigned l = 0; l < L; l++) {
            ang[l].assign(ch[l] * N, cd(0.0));
            std::vector<cd> out(ch[l] * N);
            for(unsigned cj = 0; cj < ch[l]; cj++) {
                for(unsigned ci = 0; ci < prev(l); ci++) {
                    const unsigned lb = link_begin(l, ci, cj);
                    for(unsigned x = 0; x < N; x++) {
                        cd acc(0.0);
                        window(l, x, [&](unsigned c, unsigned y) {
                            acc += w[lb + p->sym_classes[x] * vol[l] + c] * in[ci * N + y];
                        });
                        ang[l][cj * N + x] += acc;
                    }
                }
                for(unsigned x = 0; x < N; x++) out[cj * N + x] = f(ang[l][cj * N + x], l);
            }
            if(l + 1 < L) in = out;
            else for(unsigned k = 0; k < ch[l] * N; k++) r += out[k] * p->final_factor;
        }
        return r;
    }
    cd log_psi(const Conf& s) const {
        std::vector<std::vector<cd>> ang;
        return forward(s, ang);
    }
    void O_k(const Conf& s, std::vector<cd>& O) const {
        std::vector<std::vector<cd>> ang;
        forward(s, ang);
        O.assign(p->num_params, cd(0.0));
        std::vector<cd> out(ch[L - 1] * N, cd(p->final_factor));
        for(int l = (int)L - 1; l >= 0; l--) {
            std::vector<cd> delta(ch[l] * N);
            for(unsigned k = 0; k < ch[l] * N; k++) delta[k] = out[k] * df(ang[l][k], l);
            std::vector<cd> nout(prev(l) * N, cd(0.0));
            for(unsigned ci = 0; ci < prev(l); ci++)
                for(unsigned cj = 0; cj < ch[l]; cj++) {
                    const unsigned lb = link_begin(l, ci, cj);
                    for(unsigned x = 0; x < N; x++) {
                        window(l, x, [&](unsigned c, unsigned y) {
                            const unsigned k = lb + p->sym_classes[x] * vol[l] + c;
                            const cd inp = l == 0 ? cd(spin(s, y)) : f(ang[l - 1][ci * N + y], l - 1);
                            O[k] += delta[cj * N + x] * inp;
                            if(l > 0) nout[ci * N + y] += w[k] * delta[cj * N + x];
                        });
                    }
                }
            out = nout;
        }
    }
    // local energy with full recomputation (PsiCNN has no incremental update, PsiCNN.hpp:177-181)
    cd local_energy(const or_op* op, const Conf& s, cd lpsi) const {
        cd r(0.0);
        for(unsigned n = 0; n < op->n; n++) {
            ME me = pauli_apply(op->a + n * op->nw, op->b + n * op->nw, op->nw, s);
            me.factor *= cx(op->coeff, n);
            if(me.conf != s) r += me.factor * std::exp(log_psi(me.conf) - lpsi);
            else r += me.factor;
        }
        return r;
    }
};


// ---- PsiDeep of any depth: PsiDeep.hpp:171-215 (forward_pass), :345-445 (foreach_O_k),
//      PsiDeep.cu:142-183 (init_kernel: parameter offsets) ----
struct Deep {
    const or_deep* p;
    unsigned N, L, np;
    std::vector<unsigned> size, C, conn_off, b_off, w_off;
    std::vector<cd> prm, fw;
    cd lp;
    explicit Deep(const or_deep* p_) : p(p_), N(p_->N), L(p_->num_layers) {
        unsigned off = N, coff = 0;
        for(unsigned l = 0; l < L; l++) {
            size.push_back(p->sizes[l]);
            C.push_back(p->connectivity[l]);
            conn_off.push_back(coff);
            coff += C[l] * size[l];
            b_off.push_back(off);
            off += size[l];
            w_off.push_back(off);
            off += C[l] * size[l];
        }
        np = off;
        prm.resize(np);
        for(unsigned k = 0; k < np; k++) prm[k] = cx(p->params, k);
        fw.resize(size[L - 1]);
        for(unsigned j = 0; j < size[L - 1]; j++) fw[j] = cx(p->fw, j);
        lp = cd(p->lp_re, p->lp_im);
    }
    bool paulis() const { return p->basis == 1; }
    unsigned sites() const { return paulis() ? N / 3u : N; }
    // input unit u: a spin, or for Pauli strings +1 iff site u/3 holds X, Y, Z for u%3 = 0, 1, 2
    // (PauliString.hpp:84-90: type = a_bit | b_bit << 1)
    double in_val(const Conf& s, unsigned u) const {
        if(!paulis()) return spin(s, u);
        const unsigned x = u / 3u;
        const unsigned t = (unsigned)((s[0] >> x) & 1u) | ((unsigned)((s[1] >> x) & 1u) << 1);
        return t == u % 3u + 1u ? 1.0 : -1.0;
    }
    unsigned conn(unsigned l, unsigned i, unsigned j) const { return p->connections[conn_off[l] + i * size[l] + j]; }
    cd W(unsigned l, unsigned i, unsigned j) const { return prm[w_off[l] + i * size[l] + j]; }
    // layer 0 uses my_logcosh(., 0) / my_tanh(., 0); deeper layers index >= 1 (PsiDeep.hpp:182, 207, 369-377)
    cd f(cd z, unsigned l) const { return act_f(z, l, p->activation); }
    cd df(cd z, unsigned l) const { return act_df(z, l, p->activation); }
    // pre-activations z[l][j]; returns log psi
    cd forward(const Conf& s, std::vector<std::vector<cd>>& z) const {
        std::vector<cd> in(N);
        for(unsigned x = 0; x < N; x++) in[x] = in_val(s, x);
        z.assign(L, {});
        for(unsigned l = 0; l < L; l++) {
            z[l].assign(size[l], cd(0.0));
            std::vector<cd> out(size[l]);
            for(unsigned j = 0; j < size[l]; j++) {
                cd acc(0.0);
                for(unsigned i = 0; i < C[l]; i++) acc += W(l, i, j) * in[conn(l, i, j)];
                acc += prm[b_off[l] + j];
                z[l][j] = acc;
                out[j] = f(acc, l);
            }
            in = out;
        }
        cd r = lp;
        for(unsigned j = 0; j < size[L - 1]; j++) r += in[j] * fw[j];
        if(p->a_in_log_psi)
            for(unsigned x = 0; x < N; x++) r += prm[x] * in_val(s, x);
        return r;
    }
    cd log_psi(const Conf& s) const {
        std::vector<std::vector<cd>> z;
        return forward(s, z);
    }
    // configuration index of the exact sum: bits (spins) or base-4 digits per site
    // (PauliString::enumerate, PauliString.hpp:30-35)
    Conf enumerate_conf(uint64_t idx) const {
        if(!paulis()) return enumerate(idx);
        Conf c{0, 0};
        for(unsigned x = 0; x < sites(); x++) {
            c[0] |= ((idx >> (2 * x)) & 1u) << x;
            c[1] |= ((idx >> (2 * x + 1)) & 1u) << x;
        }
        return c;
    }
    uint64_t num_confs() const { return (uint64_t)1 << (paulis() ? 2 * sites() : N); }
    void O_k(const Conf& s, std::vector<cd>& O) const {
        std::vector<std::vector<cd>> z;
        forward(s, z);
        O.assign(np, cd(0.0));
        for(unsigned x = 0; x < N; x++) O[x] = in_val(s, x);
        // dlogpsi / dz for the top layer, then down through the rhs connections
        std::vector<cd> delta(size[L - 1]);
        for(unsigned j = 0; j < size[L - 1]; j++) delta[j] = fw[j] * df(z[L - 1][j], L - 1);
        for(int l = (int)L - 1; l >= 0; l--) {
            const unsigned in_size = l ? size[l - 1] : N;
            std::vector<cd> up(in_size, cd(0.0));
            for(unsigned j = 0; j < size[l]; j++) {
                O[b_off[l] + j] = delta[j];
                for(unsigned i = 0; i < C[l]; i++) {
                    const unsigned u = conn(l, i, j);
                    const cd inp = l == 0 ? cd(in_val(s, u)) : f(z[l - 1][u], l - 1);
                    O[w_off[l] + i * size[l] + j] = delta[j] * inp;
                    up[u] += W(l, i, j) * delta[j];
                }
            }
            if(l > 0) {
                delta.assign(in_size, cd(0.0));
                for(unsigned u = 0; u < in_size; u++) delta[u] = up[u] * df(z[l - 1][u], l - 1);
            }
        }
    }
    cd local_energy(const or_op* op, const Conf& s, cd lpsi) const {
        cd r(0.0);
        for(unsigned n = 0; n < op->n; n++) {
            ME me = paulis() ? pauli_times_string(op->a[n * op->nw], op->b[n * op->nw], s)
                             : pauli_apply(op->a + n * op->nw, op->b + n * op->nw, op->nw, s);
            me.factor *= cx(op->coeff, n);
            if(me.conf != s) r += me.factor * std::exp(log_psi(me.conf) - lpsi);
            else r += me.factor;
        }
        return r;
    }
    // P x for Pauli strings P = (pa, pb) and x = (s[0], s[1]) (PauliString.hpp:256-276):
    // the product string P ^ x with phase (-1)^{#(XZ, YX, ZY) pairs} (-i)^{n_eps}, n_eps = sites
    // where both are non-trivial and differ
    static ME pauli_times_string(uint64_t pa, uint64_t pb, const Conf& s) {
        const uint64_t xa = s[0], xb = s[1];
        const uint64_t pX = pa & ~pb, pY = ~pa & pb, pZ = pa & pb;
        const uint64_t xX = xa & ~xb, xY = ~xa & xb, xZ = xa & xb;
        cd f(1.0, 0.0);
        if(popc((pX & xZ) | (pY & xX) | (pZ & xY)) & 1) f *= -1.0;
        const int ne = popc((pa | pb) & (xa | xb) & ((pa ^ xa) | (pb ^ xb)));
        if((ne & 3) > 1) f *= -1.0;
        if(ne & 1) f *= cd(0.0, -1.0);
        return {f, Conf{pa ^ xa, pb ^ xb}};
    }
};

// Counter-based Metropolis chains (the sampler contract above). The model supplies
//   reset(s)              state for configuration s
//   dre(s, nx)            Re dlogpsi of the move s -> nx, keeping the proposed state
//   accept()              the proposed state becomes current
//   sample(s, op, eloc)   log psi of s from a fresh state; local energy into *eloc
template<typename Model>
void philox_chains(Model& m, unsigned N, const or_op* op, unsigned n_chains, uint64_t seed,
                   unsigned samples_per_chain, unsigned num_sweeps, unsigned num_therm,
                   int move_kind, const uint32_t* bonds, unsigned n_bonds, int init, int n_up,
                   uint64_t* conf, uint64_t* counter, uint64_t* sconf, double* slp, double* seloc,
                   uint64_t* n_accept, uint64_t* n_reject, double* min_tie) {
    const unsigned nw = nwords(N);
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    uint64_t acc_total = 0, rej_total = 0;
    double tie = 1e300;
    for(unsigned c = 0; c < n_chains; c++) {
        uint64_t t = counter[c];
        Conf s = init ? draw_initial(k0, k1, c, N, n_up, t) : load_conf(conf + (size_t)c * nw, nw);
        m.reset(s);
        auto propose = [&]() {
            uint32_t ctr[4] = {(uint32_t)t, (uint32_t)(t >> 32), c, 0u}, r[4];
            philox(k0, k1, ctr, r);
            t++;
            unsigned i = mulhi(r[0], N), j = i;
            if(move_kind == 1) {
                const unsigned bnd = mulhi(r[0], n_bonds);
                i = bonds[2 * bnd];
                j = bonds[2 * bnd + 1];
            } else if(move_kind == 2) {
                j = mulhi(r[1], N - 1u);
                j += (j >= i);
            }
            Conf nx = s;
            if(move_kind == 0) {
                nx[i >> 6] ^= (uint64_t)1 << (i & 63u);
            } else {
                if(spin(s, i) == spin(s, j)) { rej_total++; return; }
                nx[i >> 6] ^= (uint64_t)1 << (i & 63u);
                nx[j >> 6] ^= (uint64_t)1 << (j & 63u);
            }
            const double ratio = std::exp(2.0 * m.dre(s, nx));
            const double u = u53(r[2], r[3]);
            tie = std::min(tie, std::fabs(ratio - u));
            if(u <= ratio) { s = nx; m.accept(); acc_total++; }
            else rej_total++;
        };
        if(init)
            for(unsigned k = 0; k < num_therm * N; k++) propose();
        for(unsigned st = 0; st < samples_per_chain; st++) {
            for(unsigned k = 0; k < num_sweeps * N; k++) propose();
            cd el(0.0);
            const cd lp = m.sample(s, op, seloc ? &el : nullptr);
            const size_t row = (size_t)st * n_chains + c;
            if(sconf) for(unsigned w = 0; w < nw; w++) sconf[row * nw + w] = s[w];
            if(slp) put(slp + 2 * row, lp);
            if(seloc && op) put(seloc + 2 * row, el);
        }
        for(unsigned w = 0; w < nw; w++) conf[(size_t)c * nw + w] = s[w];
        counter[c] = t;
    }
    if(n_accept) *n_accept = acc_total;
    if(n_reject) *n_reject = rej_total;
    if(min_tie) *min_tie = tie;
}

// RBM family: dlogpsi from the angle deltas (the sampler's incremental form);
// samples recompute the angles
struct RbmChain {
    const Rbm& psi;
    std::vector<cd> th, th2;
    explicit RbmChain(const Rbm& p) : psi(p) {}
    void reset(const Conf& s) { psi.angles(s, th); }
    double dre(const Conf& s, const Conf& nx) {
        th2 = th;
        psi.update(th2, s, nx);
        const int act = psi.p->activation;
        cd d(0.0);
        for(unsigned q = 0; q < psi.M; q++) d += (act_f(th2[q], 0, act) - act_f(th[q], 0, act)) * psi.fw[q];
        if(psi.p->a_in_log_psi)
            for(unsigned w = 0; w < 2; w++) {
                uint64_t dm = s[w] ^ nx[w];
                while(dm) {
                    const unsigned pos = 64u * w + __builtin_ctzll(dm);
                    dm &= dm - 1;
                    d += psi.a[pos] * (spin(nx, pos) - spin(s, pos));
                }
            }
        return d.real();
    }
    void accept() { th = th2; }
    cd sample(const Conf& s, const or_op* op, cd* eloc) {
        psi.angles(s, th);
        const cd lp = psi.log_psi(s, th);
        if(op && eloc) {
            std::vector<cd> th3 = th;
            *eloc = local_energy_incremental(psi, op, s, lp, th3);
        }
        return lp;
    }
};

// PsiDeep: full forward passes
struct DeepChain {
    const Deep& psi;
    cd lp{0.0}, lp2{0.0};
    explicit DeepChain(const Deep& p) : psi(p) {}
    void reset(const Conf& s) { lp = psi.log_psi(s); }
    double dre(const Conf&, const Conf& nx) {
        lp2 = psi.log_psi(nx);
        return lp2.real() - lp.real();
    }
    void accept() { lp = lp2; }
    cd sample(const Conf& s, const or_op* op, cd* eloc) {
        lp = psi.log_psi(s);
        if(op && eloc) *eloc = psi.local_energy(op, s, lp);
        return lp;
    }
};


// PsiCNN: full forward passes (the reference recomputes fully, PsiCNN.hpp:177-181)
struct CnnChain {
    const Cnn& psi;
    cd lp{0.0}, lp2{0.0};
    explicit CnnChain(const Cnn& p) : psi(p) {}
    void reset(const Conf& s) { lp = psi.log_psi(s); }
    double dre(const Conf&, const Conf& nx) {
        lp2 = psi.log_psi(nx);
        return lp2.real() - lp.real();
    }
    void accept() { lp = lp2; }
    cd sample(const Conf& s, const or_op* op, cd* eloc) {
        lp = psi.log_psi(s);
        if(op && eloc) *eloc = psi.local_energy(op, s, lp);
        return lp;
    }
};


// ---- PsiClassical: PsiClassical.hpp:75-133, Operator.hpp:122-133 ----
struct Classical {
    const or_classical* p;
    unsigned K;
    std::vector<cd> theta;
    const Deep* ref;
    cd lp;
    Classical(const or_classical* p_, const Deep* ref_) : p(p_), K(p_->n_features), ref(ref_) {
        theta.resize(K);
        for(unsigned k = 0; k < K; k++) theta[k] = cx(p->params, k);
        lp = cd(p->lp_re, p->lp_im);
    }
    bool with_ref() const { return p->order > 1 && ref; }
    unsigned np() const { return K + (with_ref() ? ref->np : 0u); }
    // h_k(s) = sum over the feature's strings of coefficient x <s|P|P s> (Operator::fast_local_energy)
    cd h(unsigned k, const Conf& s) const {
        cd r(0.0);
        for(unsigned q = p->feat_begin[k]; q < p->feat_begin[k + 1]; q++)
            r += cx(p->coeff, q) * pauli_apply(p->a + (size_t)q * p->nw, p->b + (size_t)q * p->nw, p->nw, s).factor;
        return r;
    }
    cd log_psi(const Conf& s) const {
        cd r = lp;
        for(unsigned k = 0; k < K; k++) r += theta[k] * h(k, s);
        if(with_ref()) r += ref->log_psi(s);
        return r;
    }
    void O_k(const Conf& s, std::vector<cd>& O) const {
        O.assign(np(), cd(0.0));
        for(unsigned k = 0; k < K; k++) O[k] = h(k, s);
        if(with_ref()) {
            std::vector<cd> Or;
            ref->O_k(s, Or);
            for(size_t k = 0; k < Or.size(); k++) O[K + k] = Or[k];
        }
    }
    cd local_energy(const or_op* op, const Conf& s, cd lpsi) const {
        cd r(0.0);
        for(unsigned n = 0; n < op->n; n++) {
            ME me = pauli_apply(op->a + n * op->nw, op->b + n * op->nw, op->nw, s);
            me.factor *= cx(op->coeff, n);
            if(me.conf != s) r += me.factor * std::exp(log_psi(me.conf) - lpsi);
            else r += me.factor;
        }
        return r;
    }
};

}  // namespace

extern "C" {

unsigned or_rbm_num_params(const or_rbm* p) { return Rbm(p).num_params(); }

void or_rbm_log_psi(const or_rbm* p, const uint64_t* conf, double* out) {
    Rbm psi(p);
    const Conf s = load_conf(conf, nwords(p->N));
    std::vector<cd> th;
    psi.angles(s, th);
    put(out, psi.log_psi(s, th));
}

void or_rbm_O_k(const or_rbm* p, const uint64_t* conf, double* out) {
    Rbm psi(p);
    std::vector<cd> O;
    psi.O_k(load_conf(conf, nwords(p->N)), O);
    for(size_t k = 0; k < O.size(); k++) put(out + 2 * k, O[k]);
}

void or_rbm_local_energy(const or_rbm* p, const or_op* op, const uint64_t* conf, double* out) {
    Rbm psi(p);
    const Conf s = load_conf(conf, nwords(p->N));
    std::vector<cd> th;
    psi.angles(s, th);
    put(out, local_energy_incremental(psi, op, s, psi.log_psi(s, th), th));
}

void or_rbm_exact(const or_rbm* p, const or_op* op, double* E, double* fluct, double* grad,
                  double* tE, double* tE2, double* tO, double* tF, double* tS,
                  double* vec, double* log_vec, double* norm, double* mean_log_psi, double* O_sum,
                  double* eloc_vec) {
    Rbm psi(p);
    const unsigned np = psi.num_params();
    const uint64_t nconf = (uint64_t)1 << p->N;
    Accum acc(np);
    double nrm = 0.0;
    cd mlp(0.0);
    std::vector<cd> th, Ok;
    for(uint64_t idx = 0; idx < nconf; idx++) {
        const Conf s = enumerate(idx);
        psi.angles(s, th);
        const cd lp = psi.log_psi(s, th);
        const double w = std::exp(2.0 * lp.real());
        cd eloc(0.0);
        if(op) eloc = local_energy_incremental(psi, op, s, lp, th);
        psi.O_k(s, Ok);
        acc.add(w, eloc, Ok, tS != nullptr);
        nrm += w;
        mlp += w * lp;
        if(vec) put(vec + 2 * idx, std::exp(lp));
        if(log_vec) put(log_vec + 2 * idx, lp);
        if(eloc_vec) put(eloc_vec + 2 * idx, eloc);
    }
    if(E) put(E, acc.E);
    acc.finish(fluct, grad, tE, tE2, tO, tF, tS);
    if(norm) norm[0] = std::sqrt(nrm);
    if(mean_log_psi) put(mean_log_psi, mlp);
    if(O_sum) for(unsigned k = 0; k < np; k++) put(O_sum + 2 * k, acc.Osum[k]);
}

unsigned or_rbm_mc_reference(const or_rbm* p, const or_op* op, unsigned num_samples, unsigned num_sweeps,
                             unsigned num_therm, unsigned seed,
                             uint64_t* sconf, double* slp, double* seloc,
                             uint64_t* pconf, uint32_t* psite, double* pu, uint8_t* pacc,
                             unsigned max_props, double* mc_energy) {
    Rbm psi(p);
    const unsigned N = p->N;
    std::mt19937 rng(seed);  // RNGStates.cu:47-51
    auto u32 = [&]() { return (uint32_t)std::uniform_int_distribution<uint64_t>(0, UINT32_MAX)(rng); };
    auto real = [&]() { return std::uniform_real_distribution<double>(0.0, 1.0)(rng); };
    // Spins_t::set_randomly (Spins.h:90-102): one 64-bit word from two 32-bit draws
    Conf s{0, 0};
    for(unsigned w = 0; w < nwords(N); w++) {
        uint64_t lo = u32();
        uint64_t hi = u32();
        s[w] = lo | (hi << 32);
    }
    if(N < 64u * nwords(N)) s[N / 64u] &= ((uint64_t)1 << (N % 64u)) - 1u;
    std::vector<cd> th;
    psi.angles(s, th);
    cd lp = psi.log_psi(s, th);
    unsigned nprop = 0;
    auto mc_update = [&]() {  // MonteCarlo.hpp:133-177
        const unsigned site = u32() % N;
        Conf nx = s;
        nx[site >> 6] ^= (uint64_t)1 << (site & 63u);
        psi.update(th, s, nx);
        const cd nlp = psi.log_psi(nx, th);
        const double ratio = std::exp(2.0 * (nlp.real() - lp.real()));
        double u = 0.0;
        bool acc;
        if(ratio > 1.0) acc = true;
        else { u = real(); acc = u <= ratio; }
        if(nprop < max_props) {
            if(pconf) pconf[nprop] = s[0];
            if(psite) psite[nprop] = site;
            if(pu) pu[nprop] = u;
            if(pacc) pacc[nprop] = acc;
        }
        nprop++;
        if(acc) { lp = nlp; s = nx; }
        else psi.update(th, nx, s);
    };
    for(unsigned i = 0; i < num_therm * N; i++) mc_update();
    const unsigned steps = num_samples;  // one chain: num_mc_steps_per_chain = num_samples
    cd e(0.0);
    const double weight = 1.0 / num_samples;
    for(unsigned st = 0; st < steps; st++) {
        for(unsigned i = 0; i < num_sweeps * N; i++) mc_update();
        const cd eloc = local_energy_incremental(psi, op, s, lp, th);
        if(sconf) sconf[st] = s[0];
        if(slp) put(slp + 2 * st, lp);
        if(seloc) put(seloc + 2 * st, eloc);
        e += weight * eloc;
    }
    if(mc_energy) put(mc_energy, e);
    return nprop;
}

void or_philox4x32_10(uint32_t k0, uint32_t k1, const uint32_t* ctr, uint32_t* out) { philox(k0, k1, ctr, out); }

void or_rbm_mc_philox(const or_rbm* p, const or_op* op, unsigned n_chains, uint64_t seed,
                      unsigned samples_per_chain, unsigned num_sweeps, unsigned num_therm,
                      int move_kind, const uint32_t* bonds, unsigned n_bonds, int init, int n_up,
                      uint64_t* conf, uint64_t* counter,
                      uint64_t* sconf, double* slp, double* seloc,
                      uint64_t* n_accept, uint64_t* n_reject, double* min_tie) {
    Rbm psi(p);
    RbmChain m(psi);
    philox_chains(m, p->N, op, n_chains, seed, samples_per_chain, num_sweeps, num_therm, move_kind, bonds, n_bonds,
                  init, n_up, conf, counter, sconf, slp, seloc, n_accept, n_reject, min_tie);
}

void or_cnn_log_psi(const or_cnn* p, const uint64_t* conf, double* out) {
    Cnn psi(p);
    put(out, psi.log_psi(load_conf(conf, nwords(psi.N))));
}

void or_cnn_O_k(const or_cnn* p, const uint64_t* conf, double* out) {
    Cnn psi(p);
    std::vector<cd> O;
    psi.O_k(load_conf(conf, nwords(psi.N)), O);
    for(size_t k = 0; k < O.size(); k++) put(out + 2 * k, O[k]);
}

void or_cnn_local_energy(const or_cnn* p, const or_op* op, const uint64_t* conf, double* out) {
    Cnn psi(p);
    const Conf s = load_conf(conf, nwords(psi.N));
    put(out, psi.local_energy(op, s, psi.log_psi(s)));
}

void or_cnn_exact(const or_cnn* p, const or_op* op, double* E, double* norm,
                  double* tE, double* tE2, double* tO, double* tF, double* tS) {
    Cnn psi(p);
    const unsigned np = p->num_params;
    Accum acc(np);
    double nrm = 0.0;
    std::vector<cd> Ok;
    for(uint64_t idx = 0; idx < ((uint64_t)1 << psi.N); idx++) {
        const Conf s = enumerate(idx);
        const cd lp = psi.log_psi(s);
        const double w = std::exp(2.0 * lp.real());
        const cd eloc = op ? psi.local_energy(op, s, lp) : cd(0.0);
        if(tO || tF || tS) psi.O_k(s, Ok);
        else Ok.assign(np, cd(0.0));
        acc.add(w, eloc, Ok, tS != nullptr);
        nrm += w;
    }
    if(E) put(E, acc.E);
    if(norm) norm[0] = std::sqrt(nrm);
    acc.finish(nullptr, nullptr, tE, tE2, tO, tF, tS);
}

void or_cnn_mc_philox(const or_cnn* p, const or_op* op, unsigned n_chains, uint64_t seed,
                      unsigned samples_per_chain, unsigned num_sweeps, unsigned num_therm,
                      int move_kind, const uint32_t* bonds, unsigned n_bonds, int init, int n_up,
                      uint64_t* conf, uint64_t* counter,
                      uint64_t* sconf, double* slp, double* seloc,
                      uint64_t* n_accept, uint64_t* n_reject, double* min_tie) {
    Cnn psi(p);
    CnnChain m(psi);
    philox_chains(m, psi.N, op, n_chains, seed, samples_per_chain, num_sweeps, num_therm, move_kind, bonds, n_bonds,
                  init, n_up, conf, counter, sconf, slp, seloc, n_accept, n_reject, min_tie);
}

void or_rbm_tdvp_samples(const or_rbm* p, const or_op* op, const uint64_t* confs, unsigned n, double weight,
                         double* E, double* tE2, double* tO, double* tF, double* tS) {
    Rbm psi(p);
    const unsigned np = psi.num_params(), nw = nwords(p->N);
    Accum acc(np);
    std::vector<cd> th, Ok;
    for(unsigned r = 0; r < n; r++) {
        const Conf s = load_conf(confs + (size_t)r * nw, nw);
        psi.angles(s, th);
        const cd lp = psi.log_psi(s, th);
        const cd eloc = local_energy_incremental(psi, op, s, lp, th);
        psi.O_k(s, Ok);
        acc.add(weight, eloc, Ok, tS != nullptr);
    }
    acc.finish(nullptr, nullptr, E, tE2, tO, tF, tS);
}

unsigned or_deep_num_params(const or_deep* p) { return Deep(p).np; }

void or_deep_log_psi(const or_deep* p, const uint64_t* conf, double* out) {
    Deep psi(p);
    put(out, psi.log_psi(load_conf(conf, psi.paulis() ? 2u : nwords(p->N))));
}

void or_deep_O_k(const or_deep* p, const uint64_t* conf, double* out) {
    Deep psi(p);
    std::vector<cd> O;
    psi.O_k(load_conf(conf, psi.paulis() ? 2u : nwords(p->N)), O);
    for(size_t k = 0; k < O.size(); k++) put(out + 2 * k, O[k]);
}

void or_deep_local_energy(const or_deep* p, const or_op* op, const uint64_t* conf, double* out) {
    Deep psi(p);
    const Conf s = load_conf(conf, psi.paulis() ? 2u : nwords(p->N));
    put(out, psi.local_energy(op, s, psi.log_psi(s)));
}

void or_deep_exact(const or_deep* p, const or_op* op, double* E, double* norm,
                   double* tE, double* tE2, double* tO, double* tF, double* tS) {
    Deep psi(p);
    Accum acc(psi.np);
    double nrm = 0.0;
    std::vector<cd> Ok;
    for(uint64_t idx = 0; idx < psi.num_confs(); idx++) {
        const Conf s = psi.enumerate_conf(idx);
        const cd lp = psi.log_psi(s);
        const double w = std::exp(2.0 * lp.real());
        const cd eloc = op ? psi.local_energy(op, s, lp) : cd(0.0);
        if(tO || tF || tS) psi.O_k(s, Ok);
        else Ok.assign(psi.np, cd(0.0));
        acc.add(w, eloc, Ok, tS != nullptr);
        nrm += w;
    }
    if(E) put(E, acc.E);
    if(norm) norm[0] = std::sqrt(nrm);
    acc.finish(nullptr, nullptr, tE, tE2, tO, tF, tS);
}

void or_deep_mc_philox(const or_deep* p, const or_op* op, unsigned n_chains, uint64_t seed,
                       unsigned samples_per_chain, unsigned num_sweeps, unsigned num_therm,
                       int move_kind, const uint32_t* bonds, unsigned n_bonds, int init, int n_up,
                       uint64_t* conf, uint64_t* counter,
                       uint64_t* sconf, double* slp, double* seloc,
                       uint64_t* n_accept, uint64_t* n_reject, double* min_tie) {
    Deep psi(p);
    if(!psi.paulis()) {
        DeepChain m(psi);
        philox_chains(m, p->N, op, n_chains, seed, samples_per_chain, num_sweeps, num_therm, move_kind, bonds,
                      n_bonds, init, n_up, conf, counter, sconf, slp, seloc, n_accept, n_reject, min_tie);
        return;
    }
    // Pauli-string chains: one sweep = N proposals, N the input units (MonteCarlo.hpp:89-100
    // counts sweeps in get_num_input_units())
    const unsigned S = psi.sites();
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    uint64_t acc_total = 0, rej_total = 0;
    double tie = 1e300;
    for(unsigned c = 0; c < n_chains; c++) {
        uint64_t t = counter[c];
        Conf s;
        if(init) {
            uint32_t ctr[4] = {(uint32_t)t, (uint32_t)(t >> 32), c, 1u}, r[4];
            philox(k0, k1, ctr, r);
            const uint64_t mask = S >= 64 ? ~(uint64_t)0 : (((uint64_t)1 << S) - 1u);
            s = Conf{((uint64_t)r[0] | ((uint64_t)r[1] << 32)) & mask, ((uint64_t)r[2] | ((uint64_t)r[3] << 32)) & mask};
        } else {
            s = Conf{conf[(size_t)c * 2], conf[(size_t)c * 2 + 1]};
        }
        cd lp = psi.log_psi(s);
        auto propose = [&]() {
            uint32_t ctr[4] = {(uint32_t)t, (uint32_t)(t >> 32), c, 0u}, r[4];
            philox(k0, k1, ctr, r);
            t++;
            const unsigned x = mulhi(r[0], S), type = r[1] >> 30;
            Conf nx = s;
            nx[0] = (nx[0] & ~((uint64_t)1 << x)) | ((uint64_t)(type & 1u) << x);
            nx[1] = (nx[1] & ~((uint64_t)1 << x)) | ((uint64_t)(type >> 1) << x);
            const cd lp2 = psi.log_psi(nx);
            const double ratio = std::exp(2.0 * (lp2.real() - lp.real()));
            const double u = u53(r[2], r[3]);
            tie = std::min(tie, std::fabs(ratio - u));
            if(u <= ratio) { s = nx; lp = lp2; acc_total++; }
            else rej_total++;
        };
        if(init)
            for(unsigned k = 0; k < num_therm * psi.N; k++) propose();
        for(unsigned st = 0; st < samples_per_chain; st++) {
            for(unsigned k = 0; k < num_sweeps * psi.N; k++) propose();
            lp = psi.log_psi(s);
            const size_t row = (size_t)st * n_chains + c;
            if(sconf) { sconf[row * 2] = s[0]; sconf[row * 2 + 1] = s[1]; }
            if(slp) put(slp + 2 * row, lp);
            if(seloc && op) put(seloc + 2 * row, psi.local_energy(op, s, lp));
        }
        conf[(size_t)c * 2] = s[0];
        conf[(size_t)c * 2 + 1] = s[1];
        counter[c] = t;
    }
    if(n_accept) *n_accept = acc_total;
    if(n_reject) *n_reject = rej_total;
    if(min_tie) *min_tie = tie;
}

unsigned or_classical_num_params(const or_classical* p) {
    if(p->order > 1 && p->ref) return p->n_features + Deep(p->ref).np;
    return p->n_features;
}

void or_classical_log_psi(const or_classical* p, const uint64_t* conf, double* out) {
    std::unique_ptr<Deep> ref(p->ref ? new Deep(p->ref) : nullptr);
    Classical psi(p, ref.get());
    put(out, psi.log_psi(load_conf(conf, nwords(p->num_sites))));
}

void or_classical_O_k(const or_classical* p, const uint64_t* conf, double* out) {
    std::unique_ptr<Deep> ref(p->ref ? new Deep(p->ref) : nullptr);
    Classical psi(p, ref.get());
    std::vector<cd> O;
    psi.O_k(load_conf(conf, nwords(p->num_sites)), O);
    for(size_t k = 0; k < O.size(); k++) put(out + 2 * k, O[k]);
}

void or_classical_local_energy(const or_classical* p, const or_op* op, const uint64_t* conf, double* out) {
    std::unique_ptr<Deep> ref(p->ref ? new Deep(p->ref) : nullptr);
    Classical psi(p, ref.get());
    const Conf s = load_conf(conf, nwords(p->num_sites));
    put(out, psi.local_energy(op, s, psi.log_psi(s)));
}

void or_classical_exact(const or_classical* p, const or_op* op, double* E, double* norm,
                        double* tE, double* tE2, double* tO, double* tF, double* tS) {
    std::unique_ptr<Deep> ref(p->ref ? new Deep(p->ref) : nullptr);
    Classical psi(p, ref.get());
    Accum acc(psi.np());
    double nrm = 0.0;
    std::vector<cd> Ok;
    for(uint64_t idx = 0; idx < ((uint64_t)1 << p->num_sites); idx++) {
        const Conf s = enumerate(idx);
        const cd lp = psi.log_psi(s);
        const double w = std::exp(2.0 * lp.real());
        const cd eloc = op ? psi.local_energy(op, s, lp) : cd(0.0);
        psi.O_k(s, Ok);
        acc.add(w, eloc, Ok, tS != nullptr);
        nrm += w;
    }
    if(E) put(E, acc.E);
    if(norm) norm[0] = std::sqrt(nrm);
    acc.finish(nullptr, nullptr, tE, tE2, tO, tF, tS);
}

void or_kl(const or_classical* pc, const or_deep* pp, const uint64_t* confs, const double* wprime, unsigned n,
           double threshold, const double* last_mean, double log_psi_scale, double nu,
           double* value, double* grad, double* noise, double* total_weight, double* mean_deviation) {
    std::unique_ptr<Deep> ref(pc->ref ? new Deep(pc->ref) : nullptr);
    Classical psi(pc, ref.get());
    Deep prime(pp);
    const unsigned np = prime.np;
    const cd last(last_mean ? last_mean[0] : 0.0, last_mean ? last_mean[1] : 0.0);
    const double th2 = threshold * threshold;
    double W = 0.0, d2 = 0.0;
    cd mean(0.0), d(0.0);
    std::vector<cd> Ok(np, 0.0), dOc(np, 0.0), dO(np, 0.0), d2O(np, 0.0), dOk2(np, 0.0);
    std::vector<double> d2Ok2(np, 0.0), Ok2(np, 0.0);
    const bool exact = confs == nullptr;
    const uint64_t rows = exact ? ((uint64_t)1 << prime.N) : n;
    std::vector<cd> O;
    for(uint64_t r = 0; r < rows; r++) {
        const Conf s = exact ? enumerate(r) : load_conf(confs + r * 2, 2);
        const cd lpp = prime.log_psi(s);
        const double wp = exact ? std::exp(2.0 * lpp.real()) : wprime[r];
        const cd lps = log_psi_scale * psi.log_psi(s);
        const double w = std::exp(2.0 * (lps.real() - lpp.real())) * wp;
        W += w;
        mean += w * (lpp - lps);
        const cd dev = lpp - lps - last;
        const double dev2 = std::norm(dev);
        const bool in = dev2 > th2;
        if(in) { d += w * dev; d2 += w * dev2; }
        if(!grad) continue;
        prime.O_k(s, O);
        for(unsigned k = 0; k < np; k++) {
            Ok[k] += w * O[k];
            if(in) dOc[k] += w * dev * std::conj(O[k]);
            if(noise) {
                const double o2 = std::norm(O[k]);
                if(in) {
                    d2Ok2[k] += w * dev2 * o2;
                    dO[k] += w * dev * O[k];
                    dOk2[k] += w * dev * o2;
                    d2O[k] += w * dev2 * O[k];
                }
                Ok2[k] += w * o2;
            }
        }
    }
    d /= W;
    d2 /= W;
    const double val = std::sqrt(std::max(1e-8, d2 - std::norm(d)));
    if(value) *value = val;
    if(total_weight) *total_weight = W;
    if(mean_deviation) put(mean_deviation, mean / W);
    if(!grad) return;
    const double factor = std::pow(val, nu);
    for(unsigned k = 0; k < np; k++) {
        const cd o = Ok[k] / W, doc = dOc[k] / W;
        put(grad + 2 * k, (doc - d * std::conj(o)) / factor);
        if(noise) {
            const double a = d2Ok2[k] / W, o2 = Ok2[k] / W;
            const cd b = dO[k] / W, c = dOk2[k] / W, e = d2O[k] / W;
            const double var = a - std::norm(doc) +
                2.0 * (b * std::conj(d) * std::conj(o) + 2.0 * std::conj(doc) * d * std::conj(o) - e * std::conj(o) -
                       c * std::conj(d)).real() +
                d2 * std::norm(o) + std::norm(d) * o2 - 4.0 * std::norm(d) * std::norm(o);
            noise[k] = std::sqrt(var / (double)rows) / factor;
        }
    }
}

void or_pauli_apply(const uint64_t* a, const uint64_t* b, unsigned nw, const uint64_t* conf,
                    double* factor, uint64_t* out_conf) {
    const ME me = pauli_apply(a, b, nw, load_conf(conf, nw));
    put(factor, me.factor);
    for(unsigned w = 0; w < nw; w++) out_conf[w] = me.conf[w];
}

void or_activation(double re, double im, unsigned layer, int exact, double* f, double* df) {
    put(f, act_f(cd(re, im), layer, exact));
    put(df, act_df(cd(re, im), layer, exact));
}

}  // extern "C"
