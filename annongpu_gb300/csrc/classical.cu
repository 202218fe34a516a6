// PsiClassical (the variational classical network) and KullbackLeibler.
//
// A classical network is a PsiDeep-family wavefunction whose log psi carries K classical
// features in front of an optional reference network (include/quantum_state/PsiClassical.hpp:
// log_psi_s :75-101, foreach_O_k :113-133; source/quantum_state/PsiClassical.cu:13-60): the
// sampling, local-energy and O_k kernels are the PsiDeep ones (deep.cu).
//
// KullbackLeibler (source/network_functions/KullbackLeibler.cu.template:17-329): psi_prime's
// ensemble supplies rows (configuration, log psi', weight w'); the explicit-configuration
// kernels give log psi of the classical network on the same rows. Per row
//   w = exp(2 (Re log psi - Re log psi')) w',  d = log psi' - log psi - last mean deviation,
// deviation sums only where |d|^2 > threshold^2. The O_k columns of psi_prime are reduced in
// one pass over the O rows (FP64 accumulation, fixed row slabs: deterministic), the few
// scalars by a two-pass block reduction; the value, gradient and noise formulas run on the host.
#include <cmath>

#include "ann_internal.hpp"

namespace ann {

namespace {

constexpr int kKlThreads = 256;
constexpr int kKlBlocks = 256;
constexpr unsigned kKlSlab = 512;   // rows per column partial

__device__ double kl_block_sum(double v, double* sh) {
    v = warp_sum(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if(l == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if(w == 0) {
        r = (l < (int)(blockDim.x >> 5)) ? sh[l] : 0.0;
        r = warp_sum(r);
    }
    return r;
}

// per row: w, w d (complex, 0 below the threshold), w |d|^2 (0 below); per block:
// sum w, sum w (log psi' - log psi) (complex), sum w d (complex), sum w |d|^2
__global__ void __launch_bounds__(kKlThreads)
kl_rows_kernel(size_t n, const double* __restrict__ wprime, double w0, const cplx<double>* __restrict__ lpp,
               const cplx<double>* __restrict__ lps, double scale, double last_re, double last_im, double th2,
               double* __restrict__ rw, cplx<double>* __restrict__ rdw, double* __restrict__ rd2w,
               double* __restrict__ partial) {
    __shared__ double sh[32];
    const size_t per = (n + gridDim.x - 1) / gridDim.x;
    const size_t r0 = (size_t)blockIdx.x * per, r1 = min(n, r0 + per);
    double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for(size_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        const cplx<double> lp = mk(scale * lps[r].re, scale * lps[r].im);
        const cplx<double> lq = lpp[r];
        const double wp = wprime ? wprime[r] : w0;
        const double w = exp(2.0 * (lp.re - lq.re)) * wp;
        const cplx<double> dev = mk(lq.re - lp.re - last_re, lq.im - lp.im - last_im);
        const double dev2 = norm2(dev);
        const bool in = dev2 > th2;
        rw[r] = w;
        rdw[r] = in ? mk(w * dev.re, w * dev.im) : mk(0.0, 0.0);
        rd2w[r] = in ? w * dev2 : 0.0;
        acc[0] += w;
        acc[1] += w * (lq.re - lp.re);
        acc[2] += w * (lq.im - lp.im);
        if(in) {
            acc[3] += w * dev.re;
            acc[4] += w * dev.im;
            acc[5] += w * dev2;
        }
    }
    for(int k = 0; k < 6; k++) {
        const double s = kl_block_sum(acc[k], sh);
        if(threadIdx.x == 0) partial[(size_t)blockIdx.x * 6 + k] = s;
    }
}

__global__ void kl_final_kernel(const double* __restrict__ partial, int nb, double* __restrict__ out6) {
    if(threadIdx.x < 6) {
        double a = 0.0;
        for(int b = 0; b < nb; b++) a += partial[(size_t)b * 6 + threadIdx.x];
        out6[threadIdx.x] = a;
    }
}

// Column sums over a slab of rows (one thread per parameter k, rows read coalesced):
// [0] sum w O, [1] sum w d conj(O), and with noise [2] sum w d O, [3] sum w d |O|^2,
// [4] sum w |d|^2 O (complex), [5] sum w |d|^2 |O|^2, sum w |O|^2 (real, in one complex slot)
constexpr int kKlCols = 6;

template<typename T>
__global__ void __launch_bounds__(kKlThreads)
kl_cols_kernel(const cplx<T>* __restrict__ O, size_t ld, size_t n, unsigned np, const double* __restrict__ rw,
               const cplx<double>* __restrict__ rdw, const double* __restrict__ rd2w, int noise,
               cplx<double>* __restrict__ part) {
    const unsigned k = blockIdx.x * blockDim.x + threadIdx.x;
    if(k >= np) return;
    const size_t r0 = (size_t)blockIdx.y * kKlSlab, r1 = min(n, r0 + kKlSlab);
    cplx<double> s[kKlCols];
    for(int q = 0; q < kKlCols; q++) s[q] = mk(0.0, 0.0);
    for(size_t r = r0; r < r1; r++) {
        const cplx<double> o = cvt<double>(O[r * ld + k]);
        const double w = rw[r];
        const cplx<double> dw = rdw[r];
        s[0].re += w * o.re;
        s[0].im += w * o.im;
        cmac_conj(s[1], o, dw);  // dw conj(o)
        if(noise) {
            const double o2 = norm2(o), d2w = rd2w[r];
            s[2] += dw * o;
            s[3].re += dw.re * o2;
            s[3].im += dw.im * o2;
            s[4].re += d2w * o.re;
            s[4].im += d2w * o.im;
            s[5].re += d2w * o2;
            s[5].im += w * o2;
        }
    }
    for(int q = 0; q < kKlCols; q++) part[((size_t)blockIdx.y * kKlCols + q) * np + k] = s[q];
}

__global__ void kl_cols_final_kernel(const cplx<double>* __restrict__ part, unsigned slabs, unsigned np,
                                     cplx<double>* __restrict__ out) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= np * kKlCols) return;
    cplx<double> a = mk(0.0, 0.0);
    for(unsigned b = 0; b < slabs; b++) a += part[(size_t)b * np * kKlCols + i];
    out[i] = a;
}

template<typename F>
int kguard(F&& f) {
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

void kl_check_status() {
    unsigned v = 0;
    unsigned* p = status_word();
    ANN_CUDA(cudaMemcpy(&v, p, sizeof(unsigned), cudaMemcpyDeviceToHost));
    if(v) {
        ANN_CUDA(cudaMemset(p, 0, sizeof(unsigned)));
        throw Error(ANN_ERR_NUMERIC, "device status: non-finite value in log psi");
    }
}

}  // namespace

struct ann_kl_impl {
    unsigned Np = 0;
    double log_psi_scale = 1.0;
    zd last_mean{0.0, 0.0};
    double W = 0.0;
    zd mean{0.0, 0.0};
    DevBuf O, rw, rdw, rd2w, partial, sums, cpart, csum;
    Rows rows2;
};

namespace {

struct KlResult {
    double W, D2, value;
    zd mean, D;
    std::vector<zd> cols;   // np x kKlCols, column q of parameter k at q * np + k
};

KlResult kl_pass(ann_kl_impl& kl, ann_psi_impl& psi, ann_psi_impl& pp, ann_ens_impl& ens, double threshold,
                 bool grad, bool noise, cudaStream_t st) {
    if(psi.N != pp.N) throw Error(ANN_ERR_INVALID, "psi and psi_prime act on different numbers of sites");
    if(grad && pp.Np != kl.Np) throw Error(ANN_ERR_INVALID, "KullbackLeibler num_params differs from psi_prime");
    const size_t ld = ((size_t)pp.Np + 3) & ~(size_t)3;
    SampleTargets tg{&ens.rows};
    tg.want_eloc = false;
    if(grad) {
        kl.O.ensure((size_t)ens.num_steps() * ld * pp.elem_bytes());
        tg.O = kl.O.p;
        tg.ldO = ld;
    }
    run_ensemble(pp, nullptr, ens, tg, st);
    const size_t n = ens.rows.n;
    run_confs(psi, nullptr, ens.rows.conf.as<uint64_t>(), n, kl.rows2, nullptr, 0, st);
    kl.rw.ensure(n * sizeof(double));
    kl.rdw.ensure(n * sizeof(cplx<double>));
    kl.rd2w.ensure(n * sizeof(double));
    kl.partial.ensure((size_t)kKlBlocks * 6 * sizeof(double));
    kl.sums.ensure(6 * sizeof(double));
    const double* w = ens.kind == 0 ? ens.rows.weight.as<double>() : nullptr;
    const double w0 = ens.kind == 0 ? 0.0 : ens.uniform_weight();
    kl_rows_kernel<<<kKlBlocks, kKlThreads, 0, st>>>(n, w, w0, ens.rows.log_psi.as<cplx<double>>(),
                                                     kl.rows2.log_psi.as<cplx<double>>(), kl.log_psi_scale,
                                                     kl.last_mean.real(), kl.last_mean.imag(), threshold * threshold,
                                                     kl.rw.as<double>(), kl.rdw.as<cplx<double>>(),
                                                     kl.rd2w.as<double>(), kl.partial.as<double>());
    check_launch("kl_rows_kernel");
    kl_final_kernel<<<1, 32, 0, st>>>(kl.partial.as<double>(), kKlBlocks, kl.sums.as<double>());
    check_launch("kl_final_kernel");
    KlResult r{};
    const unsigned np = pp.Np;
    if(grad) {
        const unsigned slabs = (unsigned)((n + kKlSlab - 1) / kKlSlab);
        kl.cpart.ensure((size_t)std::max(1u, slabs) * kKlCols * np * sizeof(cplx<double>));
        kl.csum.ensure((size_t)kKlCols * np * sizeof(cplx<double>));
        const dim3 grid((np + kKlThreads - 1) / kKlThreads, std::max(1u, slabs));
        if(pp.precision == 0)
            kl_cols_kernel<float><<<grid, kKlThreads, 0, st>>>(kl.O.as<cplx<float>>(), ld, n, np, kl.rw.as<double>(),
                                                               kl.rdw.as<cplx<double>>(), kl.rd2w.as<double>(),
                                                               noise ? 1 : 0, kl.cpart.as<cplx<double>>());
        else
            kl_cols_kernel<double><<<grid, kKlThreads, 0, st>>>(kl.O.as<cplx<double>>(), ld, n, np,
                                                                kl.rw.as<double>(), kl.rdw.as<cplx<double>>(),
                                                                kl.rd2w.as<double>(), noise ? 1 : 0,
                                                                kl.cpart.as<cplx<double>>());
        check_launch("kl_cols_kernel");
        kl_cols_final_kernel<<<(np * kKlCols + 255) / 256, 256, 0, st>>>(kl.cpart.as<cplx<double>>(), slabs, np,
                                                                         kl.csum.as<cplx<double>>());
        check_launch("kl_cols_final_kernel");
        r.cols.resize((size_t)np * kKlCols);
        ANN_CUDA(cudaMemcpyAsync(r.cols.data(), kl.csum.p, r.cols.size() * sizeof(zd), cudaMemcpyDeviceToHost, st));
    }
    double h[6];
    ANN_CUDA(cudaMemcpyAsync(h, kl.sums.p, sizeof(h), cudaMemcpyDeviceToHost, st));
    ANN_CUDA(cudaStreamSynchronize(st));
    kl_check_status();
    r.W = h[0];
    r.mean = zd(h[1], h[2]) / r.W;
    r.D = zd(h[3], h[4]) / r.W;
    r.D2 = h[5] / r.W;
    r.value = std::sqrt(std::max(1e-8, r.D2 - std::norm(r.D)));
    // update_last_mean_deviation (KullbackLeibler.cu.template:175-181)
    kl.W = r.W;
    kl.mean = r.mean;
    kl.last_mean = r.mean;
    return r;
}

}  // namespace

}  // namespace ann

using namespace ann;

struct ann_kl : ann::ann_kl_impl {};

extern "C" {

int ann_psi_create_classical(const ann_classical_desc* d, ann_psi** out) {
    return kguard([&] {
        if(!d || !out || (d->n_features && (!d->feature_begin || !d->params))) throw Error(ANN_ERR_INVALID, "null argument");
        if(d->num_sites < 1 || d->num_sites > 128) throw Error(ANN_ERR_INVALID, "num_sites must be in [1, 128]");
        if(d->order != 1 && d->order != 2) throw Error(ANN_ERR_INVALID, "order must be 1 or 2");
        if(d->num_words < 1 || d->num_words > (unsigned)kMaxWords) throw Error(ANN_ERR_INVALID, "num_words must be 1 or 2");
        const unsigned K = d->n_features;
        const unsigned n_str = K ? d->feature_begin[K] : 0u;
        if(n_str && (!d->a || !d->b || !d->coeff)) throw Error(ANN_ERR_INVALID, "null feature strings");
        for(unsigned k = 0; k < K; k++)
            if(d->feature_begin[k + 1] < d->feature_begin[k]) throw Error(ANN_ERR_INVALID, "feature_begin must ascend");
        const ann_psi* ref = d->order > 1 ? d->ref : nullptr;
        auto* p = new ann_psi();
        try {
            p->kind = 2;
            p->order = (int)d->order;
            p->N = d->num_sites;
            p->NW = d->num_sites > 64 ? 2 : 1;
            p->lp = zd(d->log_prefactor[0], d->log_prefactor[1]);
            std::vector<zd> params(K);
            for(unsigned k = 0; k < K; k++) params[k] = zd(d->params[2 * k], d->params[2 * k + 1]);
            if(ref) {
                ann_psi* r = const_cast<ann_psi*>(ref);
                if(r->N != d->num_sites) throw Error(ANN_ERR_INVALID, "the reference acts on a different number of sites");
                if(r->kind == 2 && r->deep.K) throw Error(ANN_ERR_UNSUPPORTED, "the reference is itself a classical network");
                deep_ensure(*r);  // PsiDeep of any depth (a one-layer PsiDeep gets the layer tables)
                p->precision = r->precision;
                p->act = r->act;
                p->a_in = r->a_in;
                p->deep = r->deep;
                p->deep.lp_ref = r->lp;
                p->fw = r->fw;
                p->deep_tab.ensure(r->deep_tab.bytes);
                if(r->deep_tab.bytes)
                    ANN_CUDA(cudaMemcpy(p->deep_tab.p, r->deep_tab.p, r->deep_tab.bytes, cudaMemcpyDeviceToDevice));
                std::vector<zd> rp(r->Np);
                ANN_CUDA(cudaMemcpy(rp.data(), r->params.p, (size_t)r->Np * 16, cudaMemcpyDeviceToHost));
                params.insert(params.end(), rp.begin(), rp.end());
            } else {
                if(d->precision != ANN_PREC_FP32 && d->precision != ANN_PREC_FP64) throw Error(ANN_ERR_INVALID, "precision");
                p->precision = d->precision;
                p->a_in = 0;
                p->deep = DeepHost{};   // no layers, no input-unit parameters
            }
            p->deep.K = K;
            p->Np = (unsigned)params.size();
            // final weights in kernel precision (the reference's top layer)
            const size_t es = p->elem_bytes();
            std::vector<unsigned char> fwb(std::max<size_t>(1, p->fw.size()) * es, 0);
            for(size_t j = 0; j < p->fw.size(); j++) {
                if(p->precision == 0) {
                    const float v[2] = {(float)p->fw[j].real(), (float)p->fw[j].imag()};
                    std::memcpy(&fwb[j * es], v, es);
                } else {
                    const double v[2] = {p->fw[j].real(), p->fw[j].imag()};
                    std::memcpy(&fwb[j * es], v, es);
                }
            }
            upload(p->fwd, fwb.data(), fwb.size());
            // features: the Z|Y mask of a string is its b word; the coefficient carries
            // (-i)^{n_y} (PauliString::complex_prefactor, PauliString.hpp:193-208)
            p->feat_beg_h.assign(d->feature_begin, d->feature_begin + K + 1);
            if(!K) p->feat_beg_h.assign(1, 0u);
            std::vector<uint64_t> zy(2 * (size_t)std::max(1u, n_str), 0);
            std::vector<double> fc(2 * (size_t)std::max(1u, n_str), 0.0);
            std::vector<float> fcf(fc.size(), 0.f);
            for(unsigned q = 0; q < n_str; q++) {
                int ny = 0;
                for(unsigned w = 0; w < d->num_words; w++) {
                    const uint64_t a = d->a[(size_t)q * d->num_words + w], b = d->b[(size_t)q * d->num_words + w];
                    zy[2 * q + w] = b;
                    ny += __builtin_popcountll(~a & b);
                    p->feat_a_h.push_back(a);
                    p->feat_b_h.push_back(b);
                }
                zd c(d->coeff[2 * q], d->coeff[2 * q + 1]);
                p->feat_coeff_h.push_back(c);
                if((ny & 3) > 1) c = -c;
                if(ny & 1) c *= zd(0.0, -1.0);
                fc[2 * q] = c.real();
                fc[2 * q + 1] = c.imag();
                fcf[2 * q] = (float)c.real();
                fcf[2 * q + 1] = (float)c.imag();
            }
            upload(p->feat_beg, p->feat_beg_h.data(), p->feat_beg_h.size() * sizeof(unsigned));
            upload(p->feat_zy, zy.data(), zy.size() * 8);
            upload(p->feat_c, fc.data(), fc.size() * 8);
            upload(p->feat_cf, fcf.data(), fcf.size() * 4);
            upload(p->params, params.data(), params.size() * 16);
            p->cnn_w.ensure(std::max<size_t>(1, p->Np) * es);
            psi_prepare(*p, nullptr);
            ANN_CUDA(cudaDeviceSynchronize());
        } catch(...) {
            delete p;
            throw;
        }
        *out = p;
    });
}

int ann_psi_ref_log_prefactor(ann_psi* psi, const double* set2, double* get2) {
    return kguard([&] {
        if(!psi) throw Error(ANN_ERR_INVALID, "null argument");
        if(psi->order == 0) throw Error(ANN_ERR_INVALID, "not a classical network");
        if(get2) {
            get2[0] = psi->deep.lp_ref.real();
            get2[1] = psi->deep.lp_ref.imag();
        }
        if(set2) psi->deep.lp_ref = zd(set2[0], set2[1]);
    });
}

int ann_kl_create(unsigned num_params, ann_kl** out) {
    return kguard([&] {
        if(!out) throw Error(ANN_ERR_INVALID, "null argument");
        auto* k = new ann_kl();
        k->Np = num_params;
        *out = k;
    });
}

int ann_kl_destroy(ann_kl* kl) {
    return kguard([&] { delete kl; });
}

int ann_kl_log_psi_scale(ann_kl* kl, const double* set, double* get) {
    return kguard([&] {
        if(!kl) throw Error(ANN_ERR_INVALID, "null argument");
        if(get) *get = kl->log_psi_scale;
        if(set) kl->log_psi_scale = *set;
    });
}

int ann_kl_value(ann_kl* kl, ann_psi* psi, ann_psi* psi_prime, ann_ens* ens, double threshold, void* stream,
                 double* value) {
    return kguard([&] {
        if(!kl || !psi || !psi_prime || !ens || !value) throw Error(ANN_ERR_INVALID, "null argument");
        *value = kl_pass(*kl, *psi, *psi_prime, *ens, threshold, false, false,
                         reinterpret_cast<cudaStream_t>(stream)).value;
    });
}

int ann_kl_gradient(ann_kl* kl, ann_psi* psi, ann_psi* psi_prime, ann_ens* ens, double nu, double threshold,
                    void* stream, double* grad, double* noise, double* value) {
    return kguard([&] {
        if(!kl || !psi || !psi_prime || !ens || !grad) throw Error(ANN_ERR_INVALID, "null argument");
        const KlResult r = kl_pass(*kl, *psi, *psi_prime, *ens, threshold, true, noise != nullptr,
                                   reinterpret_cast<cudaStream_t>(stream));
        const unsigned np = psi_prime->Np;
        const double factor = std::pow(r.value, nu);
        const zd d = r.D;
        const double d2 = r.D2, W = r.W;
        for(unsigned k = 0; k < np; k++) {
            const zd o = r.cols[0 * (size_t)np + k] / W, doc = r.cols[1 * (size_t)np + k] / W;
            const zd g = (doc - d * std::conj(o)) / factor;
            grad[2 * k] = g.real();
            grad[2 * k + 1] = g.imag();
            if(noise) {
                // gradient_with_noise (KullbackLeibler.cu.template:289-300)
                const zd dO = r.cols[2 * (size_t)np + k] / W, dOk2 = r.cols[3 * (size_t)np + k] / W;
                const zd d2O = r.cols[4 * (size_t)np + k] / W;
                const double d2Ok2 = r.cols[5 * (size_t)np + k].real() / W, Ok2 = r.cols[5 * (size_t)np + k].imag() / W;
                const double var = d2Ok2 - std::norm(doc) +
                                   2.0 * (dO * std::conj(d) * std::conj(o) + 2.0 * std::conj(doc) * d * std::conj(o) -
                                          d2O * std::conj(o) - dOk2 * std::conj(d)).real() +
                                   d2 * std::norm(o) + std::norm(d) * Ok2 - 4.0 * std::norm(d) * std::norm(o);
                noise[k] = std::sqrt(var / (double)ens->num_steps()) / factor;
            }
        }
        if(value) *value = r.value;
    });
}

int ann_kl_stats(const ann_kl* kl, double* total_weight, double* mean_deviation2) {
    return kguard([&] {
        if(!kl) throw Error(ANN_ERR_INVALID, "null argument");
        if(total_weight) *total_weight = kl->W;
        if(mean_deviation2) {
            mean_deviation2[0] = kl->mean.real();
            mean_deviation2[1] = kl->mean.imag();
        }
    });
}

}  // extern "C"
