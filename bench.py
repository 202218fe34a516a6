"""Benchmark of the SR step of the VMC inner loop on the 2-D TFIM 8x8 workload,
plain FP32 form against the precision form on the same GPU in the same run.

Workload (square lattice 8 x 8, periodic, J = 1, h = 3.04): complex RBM with
visible bias a(64), hidden bias b(128) and W(64 x 128), Np = 8384, entries
iid N(0, 0.01^2) in real and imaginary parts (seeded). 16384 Markov chains,
one sample per chain per SR step (N_s = 16384), diagonal shift 1e-3, lr 0.01.
One step = sampling + local energies + O rows + <O>, F + S + solve + update.

  plain:     64 single-flip sweeps between samples; S in FP32 (SIMT); one FP32
             Cholesky solve with FP32 SIMT trailing updates.
  precision: learned MADE independence moves between samples (N -> 256 -> N,
             retrained every 10 SR steps on the last 65536 chain configurations,
             Adam lr 1e-3, batch 4096; dropped below 10 % acceptance); S from centred
             O in BF16 on tcgen05 with FP32 accumulation; FP32 Cholesky refined with
             FP64 residuals against the FP64 S to ||r|| / ||F|| <= 1e-12; launch and
             tile shapes from the autotuner, run on this workload before timing.

metric: effective samples/s with E_loc = N_s / tau_int / (seconds per SR step),
tau_int from the Sokal automatic-window estimator (c = 5) on per-chain local
energy series of a separate sampling run with the same moves and parameters.
`value` is the precision form's; `forms` and `vs_plain` carry both forms.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                       [--form both|precision|plain]
"""

import argparse
import json
import os
import subprocess
import sys
import threading
import time

# the CPU legs are single-threaded unless stated otherwise
for _v in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS"):
    os.environ.setdefault(_v, "1")

import numpy as np  # noqa: E402

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "effective samples/s (with E_loc) and SR steps/s vs plain form at matched energy"
UNIT = "samples/s"
L, H_FIELD, ALPHA = 8, 3.04, 2
N_SITES = L * L
M_HIDDEN = ALPHA * N_SITES
N_CHAINS = 16384
SWEEPS = 64
THERM = 64
SHIFT = 1e-3
LR = 0.01
SEED = 1234
# learned proposal of the precision form: MADE N -> 256 -> N, Adam lr 1e-3, batch 4096,
# retrained every 10 SR steps on the last 65536 chain configurations
MADE_H = 256
MADE_LR = 1e-3
MADE_BATCH = 4096
HISTORY = 65536
RETRAIN_EVERY = 10
MADE_FIRST_EPOCHS = 4
LEARNED_SWEEPS = 1       # local sweeps between samples with the learned proposal on
LEARNED_INDEP = 2        # learned independence moves per sample
MIN_ACCEPT = 0.1         # the proposal is dropped below this acceptance
TUNING_FILE = None       # --tuning: load the tuning table instead of autotuning
# DRAM bytes (read + written) of this workload from a one-pass ncu capture of two precision-form
# SR steps (dram__bytes_read.sum + dram__bytes_write.sum per kernel, profile window, Np = 8384,
# 16384 samples): the FP32 factorisation's kernels (trailing updates, panels, inverses, shift
# conversion) 20.9 GB per factorisation with one rank-64 trailing update per panel (the
# panel-pair form was not captured); herk_tc_kernel 7.0 GB per launch
WORKLOAD_NP_NS = (N_SITES + M_HIDDEN + N_SITES * M_HIDDEN, N_CHAINS)
FACTOR_DRAM_BYTES = 20.9e9
HERK_DRAM_BYTES = 7.0e9


def init_params(rng):
    s = 0.01
    a = s * (rng.standard_normal(N_SITES) + 1j * rng.standard_normal(N_SITES))
    b = s * (rng.standard_normal(M_HIDDEN) + 1j * rng.standard_normal(M_HIDDEN))
    W = s * (rng.standard_normal((N_SITES, M_HIDDEN)) + 1j * rng.standard_normal((N_SITES, M_HIDDEN)))
    return a, b, W


def config_dict(form, extra=None):
    d = {"workload": f"2D TFIM {L}x{L} PBC h={H_FIELD}, complex RBM alpha={ALPHA} (Np=8384), "
                     f"{N_CHAINS} chains, {SWEEPS} sweeps between samples, 1 sample/chain/SR step",
         "form": form, "N": N_SITES, "M": M_HIDDEN, "num_params": N_SITES + M_HIDDEN + N_SITES * M_HIDDEN,
         "chains": N_CHAINS, "sweeps_between_samples": SWEEPS, "samples_per_step": N_CHAINS,
         "diag_shift": SHIFT, "lr": LR,
         "l2": "inputs larger than L2 (O rows 1.1 GB, S 1.1 GB per step)"}
    if extra:
        d.update(extra)
    return d


# ----------------------------------------------------------------------------------
def tau_int_sokal(series, c=5.0):
    """Integrated autocorrelation time tau = 1 + 2 sum_t rho(t) with the automatic
    window W = min{W : W >= c tau(W)}; rho averaged over chains. series: (T, chains)."""
    x = np.asarray(series, float)
    x = x - x.mean(axis=0, keepdims=True)
    T = x.shape[0]
    var = (x * x).mean()
    if var <= 0:
        return 1.0
    tau = 1.0
    for t in range(1, T):
        rho = (x[:-t] * x[t:]).mean() / var
        tau += 2.0 * rho
        if t >= c * tau:
            break
    return max(tau, 1.0)


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self):
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([s.strip() for s in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        rows = [r for r in self.rows if len(r) >= 9]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


# ----------------------------------------------------------------------------------
class Form:
    """One form of the SR step on the 8x8 workload.

    plain:     complex64 sampling with single-flip Metropolis (64 sweeps between
               samples), S in FP32 on SIMT cores, one FP32 Cholesky solve.
    precision: complex64 sampling with learned MADE independence moves (retrained every
               10 SR steps on the last 65536 chain configurations), S from centred O in
               BF16 on tcgen05 (FP32 accumulation), FP32 Cholesky + refinement against
               the FP64 S to ||r||/||F|| <= 1e-12 (FP64 Cholesky when it stalls)."""

    def __init__(self, ann, name, rank):
        self.ann, self.name = ann, name
        rng = np.random.default_rng(SEED)
        a, b, W = init_params(rng)
        self.H = ann.transverse_field_ising_2d(L, L, h=H_FIELD)
        self.op = ann.Operator(self.H)
        self.psi = ann.PsiRBM(W, 1.0, 0.0, True, a=a, b=b, precision="fp32")
        self.Np = self.psi.num_params
        self.rank = rank
        self.made = None
        self.retrain_ms = []
        self.n_steps = 0
        self.tuning = None
        self.t_factor_ms = None
        if name == "plain":
            self.sweeps, self.indep = SWEEPS, 0
            self.tdvp = ann.TDVP(self.Np, s_mode="fp32", solver="fp32")
            self.tdvp.chol_update = "simt"  # FP32 SIMT arithmetic throughout
        else:
            self.sweeps, self.indep = LEARNED_SWEEPS, LEARNED_INDEP
            self.tdvp = ann.TDVP(self.Np, s_mode="bf16", solver="mixed", max_iter=6, tol=1e-12)
            self.made = ann.MADE(N_SITES, MADE_H, seed=SEED + rank)
        self.mc = self._ensemble(N_CHAINS, SEED + 17 * rank)

    def _ensemble(self, n_samples, seed):
        mc = self.ann.MonteCarloLoop(n_samples, self.sweeps, THERM, N_CHAINS, True, seed=seed, persistent=True)
        if self.made is not None:
            mc.set_history(HISTORY)
        return mc

    def prepare(self, stream):
        """Thermalises the chains; the precision form fills its history with chain
        configurations (local moves), trains the proposal and switches it on."""
        self.tdvp.stream = stream
        if self.made is None:
            return
        # first training set: 65536 configurations of thermalised chains, one local sweep apart
        prep = self.ann.MonteCarloLoop(N_CHAINS, 1, THERM, N_CHAINS, True, seed=SEED + 5 + 17 * self.rank,
                                       persistent=True)
        prep.set_history(HISTORY)
        ev = self.ann.ExpectationValue(stream=stream)
        for _ in range((HISTORY + N_CHAINS - 1) // N_CHAINS):
            ev(self.op, self.psi, prep)
        self.made.train_on_samples(prep, steps=MADE_FIRST_EPOCHS * HISTORY // MADE_BATCH, batch=MADE_BATCH,
                                   lr=MADE_LR, stream=stream)
        self.mc.set_chains(*prep.get_chains())
        self.mc.set_proposal(self.made, indep_per_sample=self.indep, min_acceptance=MIN_ACCEPT)
        # launch and tile shapes for this workload (outside the timed region), or a table
        # saved by an earlier run (profiling runs: ncu serialises and slows every launch)
        if TUNING_FILE:
            if not self.ann.load_tuning(TUNING_FILE):
                raise RuntimeError(f"{TUNING_FILE} was tuned on another GPU model")
        else:
            self.tuning = self.ann.autotune(self.op, self.psi, self.mc, self.tdvp, SHIFT, stream)

    def retrain(self, stream):
        import torch
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        self.made.train_on_samples(self.mc, steps=HISTORY // MADE_BATCH, batch=MADE_BATCH, lr=MADE_LR,
                                   stream=stream)
        e1.record(stream)
        e1.synchronize()
        self.retrain_ms.append(e0.elapsed_time(e1))
        self.mc.refresh_stats(stream)  # the drop rule for the learned proposal

    def step(self, stream):
        # the proposal is retrained every RETRAIN_EVERY SR steps after its first training
        if self.made is not None and self.n_steps > 0 and self.n_steps % RETRAIN_EVERY == 0:
            self.retrain(stream)
        self.tdvp.sr_step(self.op, self.psi, self.mc, SHIFT, LR)
        self.n_steps += 1

    def capture(self, stream):
        """Captures the SR step as one CUDA graph (the capture call runs one eager step)."""
        self.tdvp.capture_sr_step(self.op, self.psi, self.mc, SHIFT, LR, stream)
        self.n_steps += 1

    def graph_step(self, stream):
        if self.made is not None and self.n_steps > 0 and self.n_steps % RETRAIN_EVERY == 0:
            self.retrain(stream)
        self.tdvp.launch_sr_step(stream)
        self.n_steps += 1

    def tau(self, sweeps=None, indep=None):
        """tau_int of the local energy from T samples per chain of a separate run with
        the same moves (fresh chains, thermalised with local sweeps)."""
        T = 24
        sweeps = self.sweeps if sweeps is None else sweeps
        indep = self.indep if indep is None else indep
        mc = self.ann.MonteCarloLoop(N_CHAINS * T, sweeps, THERM, N_CHAINS, True, seed=SEED + 99,
                                     persistent=True)
        if self.made is not None and indep:
            mc.set_proposal(self.made, indep_per_sample=indep, min_acceptance=0.0)
        self.ann.ExpectationValue()(self.op, self.psi, mc)
        _, _, el = mc.samples()
        acc = {"local": mc.acceptance_rate}
        if self.made is not None and indep:
            acc["learned"] = mc.proposal_acceptance
        return tau_int_sokal(el.real.reshape(T, N_CHAINS)), acc

    def tau_ablation(self):
        """tau_int with the learned moves alone, the local sweeps alone, and both."""
        out = {}
        for name, sw, ind in (("learned_only", 0, self.indep), ("local_only", self.sweeps, 0),
                              ("local_and_learned", self.sweeps, self.indep)):
            t, a = self.tau(sw, ind)
            out[name] = {"sweeps": sw, "learned_moves": ind, "tau_int": t, "acceptance": a}
        return out

    def energy_check(self):
        """Per-site energy of the last step's 16384 sample configurations with the current
        parameters from the complex64 kernels of the step against the FP64 kernels (which
        match the FP64 oracle to 1e-10) on the same configurations."""
        conf, _, _ = self.mc.samples()
        el32 = self.ann.local_energies(self.psi, self.op, conf)
        psi64 = self.ann.PsiRBM(self.psi.W, 1.0, 0.0, True, a=self.psi.a, b=self.psi.b, precision="fp64")
        psi64.params = self.psi.params
        el64 = self.ann.local_energies(psi64, self.op, conf)
        return {"energy_per_site": float(el32.real.mean() / N_SITES),
                "abs_diff_per_site_vs_fp64": float(abs(el32.mean() - el64.mean()) / N_SITES),
                "max_abs_diff_per_sample_per_site": float(np.abs(el32 - el64).max() / N_SITES)}


def eager_phases(form, stream, n=3):
    """CUDA-event phase times (sampling, reductions, S, solve, update) and the time of the
    FP32 factorisation, averaged over n eager SR steps (diagnostics next to the headline)."""
    import annongpu_gb300 as ann
    ann._lib.call("ann_set_phase_timing", 1)
    phase = np.zeros(5)
    t_factor, ms_eager = [], []
    import torch
    for _ in range(n):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        form.step(stream)
        e1.record(stream)
        e1.synchronize()
        ms_eager.append(e0.elapsed_time(e1))
        ph = np.zeros(5, np.float32)
        ann._lib.call("ann_get_phase_times", ann._lib.ptr(ph))
        phase += ph
        sf = np.zeros(1, np.float32)
        ann._lib.call("ann_get_solve_times", ann._lib.ptr(sf))
        if sf[0] > 0:
            t_factor.append(float(sf[0]))
    ann._lib.call("ann_set_phase_timing", 0)
    form.t_factor_ms = float(np.mean(t_factor)) if t_factor else None
    form.ms_eager = float(np.mean(ms_eager))
    return phase / n


def timed_steps(form, args, stream, dist):
    """K SR steps as replays of the captured step (the proposal retrained between replays
    every RETRAIN_EVERY steps), CUDA events on the launching stream, max over ranks."""
    import torch
    import annongpu_gb300 as ann
    phase = eager_phases(form, stream)
    form.capture(stream)
    form.graph_step(stream)  # one replay before the timed region
    stream.synchronize()
    if args.profile_window:
        ann.start_profiling()  # ncu --profile-from-start off captures the timed steps only
    lc0 = ann.launch_count()
    if dist:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for i in range(args.steps):
        form.graph_step(stream)
    ev1.record(stream)
    torch.cuda.synchronize()
    if dist:
        torch.distributed.barrier()
    if args.profile_window:
        ann.stop_profiling()
    ms = ev0.elapsed_time(ev1) / args.steps
    if dist:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    launches = ann.launch_count() - lc0
    return ms, phase, launches


def whole_job(ms, ms_e2e, samples, tau, dist):
    """Whole-job figures over the ranks (independent replicas, weak scaling): the step
    times are the maximum over ranks, the effective samples per step the sum of each
    rank's samples / tau_int. Returns (ms, ms_e2e, value, e2e_value)."""
    eff = samples / tau
    if dist:
        import torch
        import torch.distributed as td
        dev = "cuda" if td.get_backend() == "nccl" else "cpu"
        t = torch.tensor([ms, ms_e2e], dtype=torch.float64, device=dev)
        td.all_reduce(t, op=td.ReduceOp.MAX)
        e = torch.tensor([eff], dtype=torch.float64, device=dev)
        td.all_reduce(e, op=td.ReduceOp.SUM)
        ms, ms_e2e, eff = float(t[0].item()), float(t[1].item()), float(e[0].item())
    return ms, ms_e2e, eff / (ms * 1e-3), eff / (ms_e2e * 1e-3)


def form_summary(form, ms, phase, tau, acc):
    Ns = N_CHAINS
    d = {"ms_per_step": ms, "ms_per_step_eager": getattr(form, "ms_eager", None), "sr_steps_per_s": 1e3 / ms,
         "effective_samples_per_s": Ns / tau / (ms * 1e-3),
         "sampler_effective_samples_per_s": Ns / tau / (phase[0] * 1e-3),
         "tau_int": tau, "acceptance": acc,
         "phase_ms": {"sample_eloc_O": phase[0], "reductions": phase[1], "S": phase[2], "solve": phase[3],
                      "update": phase[4]},
         "sweeps_between_samples": form.sweeps, "learned_moves_per_sample": form.indep}
    if form.retrain_ms:
        d["proposal_retrain_ms"] = float(np.mean(form.retrain_ms))
    if form.tuning:
        d["autotune_ms"] = {k: {str(c): round(ms, 4) for c, ms in v.items()} for k, v in form.tuning.items()}
    return d


# ----------------------------------------------------------------------------------
# Batched uneven instances (BASELINE config 5): 96 1-D TFIM chains, L uniform on
# {12, 16, ..., 48}, h uniform on [0.5, 1.5], J = 1, complex RBM with alpha from
# {1, 2, 4} and a per-instance seed; chains 512 .. 8192 in proportion to Np.
N_INST = 96
BATCH_SWEEPS = 4


def batched_instances(ann, st, steps):
    """One persistent sampling + E_loc launch for all instances, per-instance S (BF16
    tcgen05) and mixed solves on a stream pool, the whole step one CUDA graph; against the
    same instances stepped one after another (one CUDA graph each). Energies of the
    instances with L <= 20 against exact summation."""
    import torch
    rng = np.random.default_rng(SEED + 5)
    specs = [(int(rng.choice(np.arange(12, 49, 4))), float(rng.uniform(0.5, 1.5)), int(rng.choice([1, 2, 4])))
             for _ in range(N_INST)]
    nps = [L + al * L + al * L * L for L, _, al in specs]
    lo, hi = min(nps), max(nps)
    chains = [int(round((512 + (8192 - 512) * (n - lo) / max(hi - lo, 1)) / 64)) * 64 for n in nps]

    def make(k):
        L, h, al = specs[k]
        r = np.random.default_rng(SEED + 1000 + k)
        c = lambda *sh: 0.01 * (r.standard_normal(sh) + 1j * r.standard_normal(sh))  # noqa: E731
        psi = ann.PsiRBM(c(L, al * L), 1.0, 0.0, True, a=c(L), b=c(al * L), precision="fp32")
        op = ann.Operator(ann.transverse_field_ising_1d(L, h))
        mc = ann.MonteCarloLoop(chains[k], BATCH_SWEEPS, 16, chains[k], True, seed=SEED + 2000 + k, persistent=True)
        td = ann.TDVP(psi.num_params, s_mode="bf16", solver="mixed", stream=st)
        return psi, op, mc, td

    def timed(fn, n):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(st)
        for _ in range(n):
            fn()
        e1.record(st)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n

    # batched: one graph per step
    inst = [make(k) for k in range(N_INST)]
    batch = ann.Batch(*[list(x) for x in zip(*inst)], stream=st)
    batch.capture_sr_step(SHIFT, LR, st)  # runs one eager step (thermalises) first
    batch.launch_sr_step(st)
    ms_batched = timed(lambda: batch.launch_sr_step(st), steps)
    # energies after the timed steps (persistent, equilibrated chains)
    batch.sample()
    E = batch.energies()
    checks = []
    for k, (L, h, al) in enumerate(specs):
        if L <= 20:
            psi, op, mc, td = inst[k]
            es = ann.ExactSummationSpins(L)
            psi.normalize(es)
            e_ex = ann.ExpectationValue()(op, psi, es).real
            _, _, el = mc.samples()
            se = el.real.std() / np.sqrt(len(el))
            checks.append({"L": L, "alpha": al, "h": round(h, 4), "E_mc": float(E[k].real), "E_exact": float(e_ex),
                           "abs_diff_per_site": float(abs(E[k].real - e_ex) / L),
                           "diff_in_se": float(abs(E[k].real - e_ex) / se)})
    del batch, inst
    torch.cuda.empty_cache()
    # one instance after another: a captured SR step per instance, launched in turn
    seq = [make(k) for k in range(N_INST)]
    for psi, op, mc, td in seq:
        td.capture_sr_step(op, psi, mc, SHIFT, LR, st)
    ms_seq = timed(lambda: [td.launch_sr_step(st) for (_, _, _, td) in seq], steps)
    samples = sum(chains)
    return {"instances": N_INST, "samples_per_step": samples, "num_params_range": [lo, hi],
            "chains_range": [min(chains), max(chains)], "sweeps_between_samples": BATCH_SWEEPS,
            "ms_per_step_batched": ms_batched, "ms_per_step_one_by_one": ms_seq,
            "speedup": ms_seq / ms_batched, "samples_per_s_batched": samples / (ms_batched * 1e-3),
            "exact_summation_checks": checks,
            "max_diff_in_standard_errors": max(c["diff_in_se"] for c in checks) if checks else None}


def hsd_timing(ann, f, st):
    """HilbertSpaceDistance gradient on the 8x8 workload: psi' = the current psi, U = 1 + i H t
    (t = 0.01), 16384 Monte Carlo samples from psi's persistent chains (one sampling pass with
    E_loc, log psi' and O' rows, the reductions) per call."""
    import torch
    psi_p = +f.psi
    op = ann.Operator(ann.identity() + 0.01j * f.H)
    hsd = ann.HilbertSpaceDistance(psi_p.num_params, stream=st)
    hsd.gradient(f.psi, psi_p, op, True, f.mc, 1.0)
    reps = 5
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        _, d = hsd.gradient(f.psi, psi_p, op, True, f.mc, 1.0)
    ms = (time.perf_counter() - t0) * 1e3 / reps
    return {"ms_per_gradient_call": ms, "samples": N_CHAINS, "distance": d,
            "note": "host-synchronous calls (the gradient returns to the host), sampling included"}


def run_ours(args):
    import torch
    import annongpu_gb300 as ann

    dist = int(os.environ.get("WORLD_SIZE", "1")) > 1
    rank = int(os.environ.get("RANK", "0"))
    if dist:
        import torch.distributed as td
        td.init_process_group("nccl")
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        ann.setDevice(torch.cuda.current_device())
    st = torch.cuda.Stream()
    results = {}
    clocks = ClockSampler()
    clk = None
    forms = ["plain", "precision"] if args.form == "both" else [args.form]
    for name in forms:
        f = Form(ann, name, rank)
        f.prepare(st)
        for _ in range(args.warmup):
            f.step(st)
        st.synchronize()
        if name == "precision" or len(forms) == 1:
            clocks.start()
        ms, phase, launches = timed_steps(f, args, st, dist)
        if name == "precision" or len(forms) == 1:
            clk = clocks.stop()
        f.mc.refresh_stats(st)
        info = f.tdvp.solver_info
        tau, acc = f.tau()
        results[name] = (f, ms, phase, launches, tau, acc, info)

    main = results["precision"] if "precision" in results else results[forms[0]]
    f, ms, phase, launches, tau, acc, info = main
    Np, Ns = f.Np, N_CHAINS
    energy = f.energy_check()
    ablation = f.tau_ablation() if f.made is not None else None

    # the same step with the FP64 Cholesky solver (and the solve error of the mixed solver)
    fp64 = {}
    if f.name == "precision":
        d_mixed = f.tdvp.solve(SHIFT)
        f.tdvp.set_solver("fp64")
        d_fp64 = f.tdvp.solve(SHIFT)  # same S and F
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        f.step(st)
        e1.record(st)
        e1.synchronize()
        f.tdvp.set_solver("mixed", 6, 1e-12)
        fp64 = {"ms_per_step_fp64_cholesky": e0.elapsed_time(e1),
                "solve_rel_err_vs_fp64_cholesky": float(np.linalg.norm(d_mixed - d_fp64) / np.linalg.norm(d_fp64))}

    # end to end through the public API: parameters from pinned host memory in, the
    # step's energy out, every step
    host_params = torch.from_numpy(f.psi.params.view(np.float64).copy()).pin_memory()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    f.capture(st)  # the parameters may have changed: recapture, then replay
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(args.steps):
        f.psi.set_params_async(host_params, st)
        f.graph_step(st)
        _ = f.tdvp.E_local  # device -> host read of the step's energy (synchronising)
    st.synchronize()
    ms_e2e = (time.perf_counter() - t0) * 1e3 / args.steps

    pk, pk_kind = peaks()
    flops_S = 4.0 * Np * (Np + 1) * Ns  # algorithmic HERK count per step
    s_tflops = flops_S / (phase[2] * 1e-3) / 1e12
    summary = form_summary(f, ms, phase, tau, acc)
    ms, ms_e2e, value, e2e_value = whole_job(ms, ms_e2e, Ns, tau, dist)
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": ("c64 sampling + learned proposal / bf16 S (fp32 acc) / fp32 Cholesky + f64 refinement"
                  if f.name == "precision" else "c64 sampling / fp32 S / fp32 Cholesky"),
        "data": "synthetic (seeded random-init RBM, 2D TFIM)",
        "config": config_dict(f.name),
        "sr_steps_per_s": 1e3 / ms, "ms_per_step_eager": f.ms_eager, "tau_int": tau, "acceptance": acc,
        "energy_per_site": energy["energy_per_site"], "energy_check": energy,
        "phase_ms": summary["phase_ms"], "phase_note": "CUDA-event phases of eager steps (the headline times graph replays)",
        "solver": info,
        "roofline_herk": {"bound": "tensor", "kernel": "herk_tc_kernel (S = O_c^H O_c, tcgen05 BF16)",
                          "achieved": s_tflops, "peak": pk.get("bf16_tflops", 1900.0) if f.name == "precision" else None,
                          "unit": "TFLOP/s", "peak_kind": pk_kind + " bf16 burst",
                          "traffic": HERK_DRAM_BYTES if (Np, Ns) == WORKLOAD_NP_NS and f.name == "precision"
                          else None,
                          "work": "4*Np*(Np+1)*Ns real flops per step (over the S phase: operand prep + kernel)"},
        "clocks": clk,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": Np * 16,
                "d2h_bytes_per_step": 16, "ms_per_step": ms_e2e},
        "gpu_launches": int(launches),
    }
    if out["roofline_herk"]["peak"]:
        out["roofline_herk"]["frac"] = s_tflops / out["roofline_herk"]["peak"]
    if getattr(f, "t_factor_ms", None):
        # FP32 Cholesky: (4/3) Np^3 real flops of complex factorisation; its trailing
        # updates run as three TF32 products on tcgen05 (TF32 rate = half the BF16 rate)
        chol_tflops = (4.0 / 3.0) * Np ** 3 / (f.t_factor_ms * 1e-3) / 1e12
        tf32x3_peak = pk.get("bf16_tflops", 1900.0) / 2 / 3
        # the autotuned form of the trailing updates; the DRAM capture is of the per-panel form
        pair = any("/chol.pair/" in k and v == 1 for k, v in ann.tuning_table().items())
        # the dominant kernel group of the step: trailing updates + panel path are about half
        # of the launch list (the S kernel 14 %)
        out["roofline"] = {"bound": "tensor",
                           "kernel": "FP32 Cholesky factorisation (chol_update_tc3 tcgen05 split-TF32 trailing "
                                     "updates + potrf32/trsm32 panel path)",
                           "achieved": chol_tflops, "peak": tf32x3_peak, "unit": "TFLOP/s",
                           "frac": chol_tflops / tf32x3_peak, "ms": f.t_factor_ms,
                           "traffic": FACTOR_DRAM_BYTES
                           if (Np, Ns) == WORKLOAD_NP_NS and f.name == "precision" and not pair else None,
                           "update_form": "rank 128 per panel pair" if pair else "rank 64 per panel",
                           "peak_kind": pk_kind + " bf16 burst / 2 (TF32) / 3 (split products)",
                           "work": "(4/3)*Np^3 real flops per factorisation (CUDA events around it)"}
    else:
        out["roofline"] = out["roofline_herk"]
    out.update(fp64)
    if ablation:
        out["tau_ablation"] = ablation
    out["forms"] = {name: form_summary(r[0], r[1], r[2], r[4], r[5]) for name, r in results.items()}
    if "plain" in results and "precision" in results:
        p, q = out["forms"]["plain"], out["forms"]["precision"]
        out["vs_plain"] = {k: q[k] / p[k] for k in ("sr_steps_per_s", "effective_samples_per_s",
                                                    "sampler_effective_samples_per_s")}
        out["forms"]["plain"]["energy_check"] = results["plain"][0].energy_check()
    if f.name == "precision":
        out["hilbert_space_distance"] = hsd_timing(ann, f, st)
    if not args.no_batched and f.name == "precision":
        out["batched_instances"] = batched_instances(ann, st, max(2, args.steps // 5))
    if rank == 0 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(*init_params(np.random.default_rng(SEED)), f.H, tau, cores=1)
    if rank == 0:
        print(json.dumps(out))
    if dist:
        torch.distributed.destroy_process_group()


# ----------------------------------------------------------------------------------
def cpu_step_seconds(a, b, W, H, n_samples=4, chains=None):
    """Time the FP64 oracle (a restatement of the reference's host path) on a
    bounded sample of one SR step and scale to the full step: per-sample work
    (64 sweeps of single-flip Metropolis, local energy, O_k, S accumulation)
    times N_s, plus a Cholesky solve timed at n = 2048 and scaled by (Np/2048)^3."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from pyoracle import Oracle, RbmDesc
    o = Oracle()
    psi = RbmDesc(N_SITES, M_HIDDEN, W, a=a, b=b, layout=1)
    t0 = time.perf_counter()
    r = o.mc_philox(psi, H, n_samples, SEED, 1, SWEEPS, 0, init=True)
    t_mc = (time.perf_counter() - t0) / n_samples
    t0 = time.perf_counter()
    o.tdvp_samples(psi, H, r["sconf"], 1.0 / n_samples, want_S=True)
    t_tdvp = (time.perf_counter() - t0) / n_samples
    n = 2048
    A = np.random.default_rng(0).standard_normal((n, n)) + 1j * np.random.default_rng(1).standard_normal((n, n))
    A = A @ A.conj().T + n * np.eye(n)
    t0 = time.perf_counter()
    np.linalg.cholesky(A)
    t_chol = (time.perf_counter() - t0) * ((N_SITES + M_HIDDEN + N_SITES * M_HIDDEN) / n) ** 3
    return N_CHAINS * (t_mc + t_tdvp) + t_chol, t_mc, t_tdvp, t_chol


def cpu_baseline(a, b, W, H, tau, cores=1):
    step_s, t_mc, t_tdvp, t_chol = cpu_step_seconds(a, b, W, H)
    return {"value": N_CHAINS / tau / step_s, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"4 chains x 1 sample (64 sweeps, E_loc, O_k, S rows) timed and scaled to {N_CHAINS} "
                      f"samples; Cholesky timed at n=2048 and scaled by n^3 to Np=8384; tau_int from the GPU run",
            "seconds_per_step": step_s, "s_per_sample_mc": t_mc, "s_per_sample_tdvp": t_tdvp,
            "s_cholesky": t_chol}


def _expression_module():
    # the Hamiltonian builder alone (pure Python); the CPU legs never load the CUDA library
    import importlib.util
    spec = importlib.util.spec_from_file_location("_ann_expression",
                                                  os.path.join(ROOT, "annongpu_gb300", "expression.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _cpu_worker(q):
    rng = np.random.default_rng(SEED)
    a, b, W = init_params(rng)
    H = _expression_module().transverse_field_ising_2d(L, L, h=H_FIELD)
    q.put(cpu_step_seconds(a, b, W, H, n_samples=2)[0])


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import multiprocessing as mp
    P = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    times = []
    t_start = time.perf_counter()
    for _ in range(max(1, args.steps)):
        q = ctx.Queue()
        procs = [ctx.Process(target=_cpu_worker, args=(q,)) for _ in range(P)]
        for p in procs:
            p.start()
        vals = [q.get() for _ in procs]
        for p in procs:
            p.join()
        # P independent processes split the samples of one step
        times.append(float(np.median(vals)) / P)
    step_s = float(np.median(times))
    tau = 1.0  # not measured on the CPU: taking 1 makes this an upper bound of the CPU effective rate
    value = N_CHAINS / tau / step_s
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "c128", "data": "synthetic (seeded random-init RBM, 2D TFIM)",
           "config": config_dict("precision" if args.form == "both" else args.form), "impl": "reference",
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": P, "kind": "port",
                            "sample": f"{P} processes x 2 chains x 1 sample timed per step and scaled to "
                                      f"{N_CHAINS} samples; Cholesky scaled from n=2048; tau_int = 1 assumed"},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "wall_s": time.perf_counter() - t_start}
    print(json.dumps(out))


def run_profile_case(solver="fp64"):
    """Small case for ncu captures (a few GB at most, one SR step after one warm-up):
    N=32, M=64 complex RBM (Np = 2144), 1-D TFIM, 16384 chains, 4 sweeps between
    samples, BF16 tensor-core S, SR solve by `solver` (fp64 / mixed / fp32)."""
    import annongpu_gb300 as ann
    rng = np.random.default_rng(0)
    N, M = 32, 64
    a = 0.01 * (rng.standard_normal(N) + 1j * rng.standard_normal(N))
    b = 0.01 * (rng.standard_normal(M) + 1j * rng.standard_normal(M))
    W = 0.01 * (rng.standard_normal((N, M)) + 1j * rng.standard_normal((N, M)))
    psi = ann.PsiRBM(W, 1.0, 0.0, True, a=a, b=b, precision="fp32")
    op = ann.Operator(ann.transverse_field_ising_1d(N, 1.0))
    mc = ann.MonteCarloLoop(16384, 4, 8, 16384, True, seed=1, persistent=True)
    td = ann.TDVP(psi.num_params, s_mode="bf16", solver=solver)
    for _ in range(2):
        td.sr_step(op, psi, mc, 1e-3, 0.01)
    print("profile case: E/N =", td.E_local / N)


def run_profile_case_learned():
    """Small case for ncu captures of the sampler with learned moves: the 8x8 workload's
    shapes (N = 64, M = 128, h = 3.04) with 4096 chains (O rows 275 MB), one local sweep
    and two learned independence moves per sample, the proposal trained on 16384
    configurations first; two SR steps (BF16 tensor-core S, mixed solver)."""
    import annongpu_gb300 as ann
    rng = np.random.default_rng(SEED)
    a, b, W = init_params(rng)
    op = ann.Operator(ann.transverse_field_ising_2d(L, L, h=H_FIELD))
    psi = ann.PsiRBM(W, 1.0, 0.0, True, a=a, b=b, precision="fp32")
    chains = 4096
    prep = ann.MonteCarloLoop(chains, 1, THERM, chains, True, seed=5, persistent=True)
    prep.set_history(4 * chains)
    for _ in range(4):
        ann.ExpectationValue()(op, psi, prep)
    made = ann.MADE(N_SITES, MADE_H, seed=1)
    made.train_on_samples(prep, steps=16, batch=MADE_BATCH, lr=MADE_LR)
    mc = ann.MonteCarloLoop(chains, LEARNED_SWEEPS, THERM, chains, True, seed=6, persistent=True)
    mc.set_chains(*prep.get_chains())
    mc.set_proposal(made, indep_per_sample=LEARNED_INDEP, min_acceptance=0.0)
    td = ann.TDVP(psi.num_params, s_mode="bf16", solver="mixed")
    for _ in range(2):
        td.sr_step(op, psi, mc, SHIFT, LR)
    print("profile case (learned): E/N =", td.E_local / N_SITES)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--form", default="both", choices=["both", "precision", "plain"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-instances measurement")
    ap.add_argument("--profile-case", action="store_true", help="run the small ncu capture case and exit")
    ap.add_argument("--profile-solver", default="fp64", choices=["fp64", "mixed", "fp32", "learned"],
                    help="SR solver of the small profile case; 'learned': the learned-proposal sampler case")
    ap.add_argument("--tuning", default=None, help="load this tuning table (from --save-tuning) instead of autotuning")
    ap.add_argument("--save-tuning", default=None, help="save the tuning table after the run")
    ap.add_argument("--profile-window", action="store_true",
                    help="bracket the timed steps with cudaProfilerStart/Stop (for ncu --profile-from-start off)")
    args = ap.parse_args()
    if args.profile_case:
        if args.profile_solver == "learned":
            run_profile_case_learned()
        else:
            run_profile_case(args.profile_solver)
        return
    global TUNING_FILE
    TUNING_FILE = args.tuning
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)
        if args.save_tuning:
            import annongpu_gb300 as ann
            ann.save_tuning(args.save_tuning)


if __name__ == "__main__":
    main()
