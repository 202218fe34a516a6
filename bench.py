"""Benchmark of the VMC inner loop's SR step on the 2-D TFIM 8x8 workload (the headline),
plain FP32 form against the precision form on the same GPU in the same run, plus the
other workloads of the path (learned proposal at alpha = 4, CNN on the 10x10 J1-J2
model, batched uneven instances) as legs of the same JSON line.

Headline workload (square lattice 8 x 8, periodic, J = 1, h = 3.04): complex RBM with
visible bias a(64), hidden bias b(128) and W(64 x 128), Np = 8384, entries iid
N(0, 0.01^2) in real and imaginary parts (seeded). 16384 Markov chains, 64 single-flip
sweeps between samples in both forms, one sample per chain per SR step (N_s = 16384),
diagonal shift 1e-3, lr 0.01. One step = sampling + local energies + O rows + <O>, F +
S + solve + update. Both forms first run 300 SR steps from the same initial parameters;
the timed steps continue from there.

  plain:     S in FP32 (SIMT); one FP32 Cholesky solve with FP32 SIMT trailing updates.
  precision: two learned MADE independence moves per sample after the 64 sweeps
             (N -> 256 -> N, retrained every 10 SR steps on the last 65536 chain
             configurations, Adam lr 1e-3, batch 4096; dropped below 10 % acceptance and
             re-armed after each retraining); S from centred O in BF16 on tcgen05 with
             FP32 accumulation; FP32 Cholesky refined with FP64 residuals against the
             FP64 S to ||r|| / ||F|| <= 1e-12; launch and tile shapes from the autotuner,
             run on this workload before timing.

metric: effective samples/s with E_loc = N_s / tau_int / (seconds per SR step), tau_int
from the Sokal automatic-window estimator (c = 5) on per-chain local-energy series of
200 samples per chain (4096 chains) with each form's own moves at the trained psi.
`value` is the precision form's; `forms` and `vs_plain` carry both forms.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                       [--form both|precision|plain] [--train-steps T] [--no-legs]
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
NP_C2 = N_SITES + M_HIDDEN + N_SITES * M_HIDDEN
N_CHAINS = 16384
SWEEPS = 64
THERM = 64
SHIFT = 1e-3
LR = 0.01
SEED = 1234
TRAIN_STEPS = 300
# learned proposal of the precision form: MADE N -> 256 -> N, Adam lr 1e-3, batch 4096,
# retrained every 10 SR steps on the last 65536 chain configurations
MADE_H = 256
MADE_LR = 1e-3
MADE_BATCH = 4096
HISTORY = 65536
RETRAIN_EVERY = 10
MADE_FIRST_EPOCHS = 4
LEARNED_INDEP = 2        # learned independence moves per sample
MIN_ACCEPT = 0.1         # the proposal is dropped below this acceptance (re-armed after retraining)
TAU_T, TAU_CHAINS = 200, 4096
TUNING_FILE = None       # --tuning: load the tuning table instead of autotuning


def init_rbm(rng, N, M, s=0.01):
    c = lambda *sh: s * (rng.standard_normal(sh) + 1j * rng.standard_normal(sh))  # noqa: E731
    return c(N), c(M), c(N, M)


def init_params(rng):
    return init_rbm(rng, N_SITES, M_HIDDEN)


def config_dict(form, extra=None):
    d = {"workload": f"2D TFIM {L}x{L} PBC h={H_FIELD}, complex RBM alpha={ALPHA} (Np={NP_C2}), "
                     f"{N_CHAINS} chains, {SWEEPS} sweeps between samples, 1 sample/chain/SR step",
         "form": form, "N": N_SITES, "M": M_HIDDEN, "num_params": NP_C2,
         "chains": N_CHAINS, "sweeps_between_samples": SWEEPS,
         "learned_moves_per_sample": LEARNED_INDEP if form == "precision" else 0,
         "samples_per_step": N_CHAINS, "diag_shift": SHIFT, "lr": LR, "train_steps_before_timing": TRAIN_STEPS,
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


def fp32_simt_peak_tflops():
    """FP32 FMA peak of the SIMT pipes (128 lanes x 2 flops per SM per clock) at the SM
    clock the device reports; MEASURED_PEAKS.json has no SIMT figure."""
    import torch
    p = torch.cuda.get_device_properties(0)
    mhz = 2070.0
    try:
        out = subprocess.run(["nvidia-smi", "--query-gpu=clocks.max.sm", "--format=csv,noheader,nounits"],
                             capture_output=True, text=True, timeout=10).stdout.split()
        mhz = float(out[0])
    except (OSError, ValueError, IndexError, subprocess.TimeoutExpired):
        pass
    return p.multi_processor_count * 128 * 2 * mhz * 1e6 / 1e12


def cuda_ms(fn, stream):
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1)


# ----------------------------------------------------------------------------------
class Form:
    """One form of the SR step on the 8x8 workload (see the module docstring)."""

    def __init__(self, ann, name, rank):
        self.ann, self.name = ann, name
        a, b, W = init_params(np.random.default_rng(SEED))
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
        self.energy = []
        self.drops = 0
        self.sweeps = SWEEPS
        if name == "plain":
            self.indep = 0
            self.tdvp = ann.TDVP(self.Np, s_mode="fp32", solver="fp32")
            self.tdvp.chol_update = "simt"  # FP32 SIMT arithmetic throughout
        else:
            self.indep = LEARNED_INDEP
            self.tdvp = ann.TDVP(self.Np, s_mode="bf16", solver="mixed", max_iter=10, tol=1e-12)
            self.made = ann.MADE(N_SITES, MADE_H, seed=SEED + rank)
        self.mc = ann.MonteCarloLoop(N_CHAINS, self.sweeps, THERM, N_CHAINS, True, seed=SEED + 17 * rank,
                                     persistent=True)
        if self.made is not None:
            self.mc.set_history(HISTORY)

    def prepare(self, stream):
        """Thermalises the chains; the precision form fills its history with chain
        configurations, trains the proposal, switches it on and autotunes."""
        self.tdvp.stream = stream
        ev = self.ann.ExpectationValue(stream=stream)
        if self.made is None:
            ev(self.op, self.psi, self.mc)
            return
        for _ in range((HISTORY + N_CHAINS - 1) // N_CHAINS):
            ev(self.op, self.psi, self.mc)
        self.made.train_on_samples(self.mc, steps=MADE_FIRST_EPOCHS * HISTORY // MADE_BATCH, batch=MADE_BATCH,
                                   lr=MADE_LR, stream=stream)
        self.mc.set_proposal(self.made, indep_per_sample=self.indep, min_acceptance=MIN_ACCEPT)
        # launch and tile shapes for this workload (outside the timed region), or a table
        # saved by an earlier run (profiling runs: ncu serialises and slows every launch)
        if TUNING_FILE:
            if not self.ann.load_tuning(TUNING_FILE):
                raise RuntimeError(f"{TUNING_FILE} was tuned on another GPU model")
        else:
            self.tuning = self.ann.autotune(self.op, self.psi, self.mc, self.tdvp, SHIFT, stream)

    def retrain(self, stream):
        """Retrains the proposal on the history ring and re-arms it (the drop rule decides
        again on the next sampling pass)."""
        self.mc.refresh_stats(stream)
        self.drops += int(self.mc.proposal_dropped)
        self.retrain_ms.append(cuda_ms(lambda: self.made.train_on_samples(
            self.mc, steps=HISTORY // MADE_BATCH, batch=MADE_BATCH, lr=MADE_LR, stream=stream), stream))
        self.mc.set_proposal(self.made, indep_per_sample=self.indep, min_acceptance=MIN_ACCEPT)

    def step(self, stream):
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

    def train(self, n, stream):
        """n SR steps as graph replays, recording the energy per site of every step."""
        self.capture(stream)
        self.energy.append(self.tdvp.E_local.real / N_SITES)
        for _ in range(n - 1):
            self.graph_step(stream)
            self.energy.append(self.tdvp.E_local.real / N_SITES)

    def tau_run(self, sweeps, indep, T=TAU_T, chains=TAU_CHAINS):
        """tau_int, acceptance and cost per sample of chains with `sweeps` local sweeps and
        `indep` learned moves per sample, continuing from the form's chains at the current
        psi; T samples per chain."""
        import torch
        conf, ctr = self.mc.get_chains()
        mc = self.ann.MonteCarloLoop(chains * T, sweeps, 0, chains, True, seed=SEED + 99, persistent=True)
        mc.set_chains(conf[:chains], ctr[:chains])
        if self.made is not None and indep:
            mc.set_proposal(self.made, indep_per_sample=indep, min_acceptance=0.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        self.ann.ExpectationValue()(self.op, self.psi, mc)
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t0) * 1e3
        _, _, el = mc.samples()
        x = el.real.reshape(T, chains)
        tau = tau_int_sokal(x)
        acc = {"local": mc.acceptance_rate}
        if self.made is not None and indep:
            acc["learned"] = mc.proposal_acceptance
        se = float(x.std() * np.sqrt(tau / x.size) / N_SITES)
        return {"sweeps": sweeps, "learned_moves": indep, "tau_int": tau, "acceptance": acc,
                "ms_per_sample_pass": ms / T, "energy_per_site": float(x.mean() / N_SITES), "se_per_site": se,
                "effective_samples_per_s_sampler": chains / tau / (ms / T * 1e-3)}

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

    def fp64_errors(self, stream):
        """E, F, S and the SR update delta of one eager evaluation of this form against a
        full FP64 evaluation on the same 16384 sample configurations: complex128 log psi,
        local energies and O rows, S from FP64 HERK, delta from the FP64 Cholesky solve of
        (S + shift) delta = F. Relative Frobenius / 2-norm errors."""
        ann = self.ann
        self.tdvp.eval(self.op, self.psi, self.mc)
        stream.synchronize()
        S, F, E = self.tdvp.S_matrix, self.tdvp.F_vector, self.tdvp.E_local
        d = self.tdvp.solve(SHIFT)
        conf, _, _ = self.mc.samples()
        psi64 = ann.PsiRBM(self.psi.W, 1.0, 0.0, True, a=self.psi.a, b=self.psi.b, precision="fp64")
        psi64.params = self.psi.params
        n = len(conf)
        replay = ann.MonteCarloLoop(n, 0, 0, n, True, persistent=True)
        replay.set_tape(conf[:, 0], np.zeros((n, 1), np.uint32), np.zeros((n, 1)))
        td64 = ann.TDVP(self.Np, s_mode="fp32", solver="fp64", stream=stream)
        td64.eval(self.op, psi64, replay)
        c64, _, _ = replay.samples()
        assert (c64[:, 0] == conf[:, 0]).all()
        S64, F64, E64 = td64.S_matrix, td64.F_vector, td64.E_local
        d64 = td64.solve(SHIFT)
        rel = lambda x, y: float(np.linalg.norm(x - y) / np.linalg.norm(y))  # noqa: E731
        out = {"energy_abs_diff_per_site": float(abs(E - E64) / N_SITES), "F_rel_err": rel(F, F64),
               "S_rel_err_fro": rel(S, S64), "delta_rel_err": rel(d, d64),
               "S_max_abs_err_rel_to_max": float(np.abs(S - S64).max() / np.abs(S64).max()),
               "samples": n, "reference": "complex128 kernels + FP64 HERK + FP64 Cholesky on the same samples"}
        del S, S64
        return out


def eager_phases(form, stream, n=3):
    """CUDA-event phase times (sampling, reductions, S, solve, update) and the time of the
    FP32 factorisation, averaged over n eager SR steps (diagnostics next to the headline)."""
    import annongpu_gb300 as ann
    ann._lib.call("ann_set_phase_timing", 1)
    phase = np.zeros(5)
    t_factor, ms_eager = [], []
    for _ in range(n):
        ms_eager.append(cuda_ms(lambda: form.step(stream), stream))
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
    for _ in range(args.warmup):
        form.graph_step(stream)
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


def form_summary(form, ms, phase, tau_rec):
    Ns = N_CHAINS
    tau = tau_rec["tau_int"]
    e = np.asarray(form.energy[-20:])
    d = {"ms_per_step": ms, "ms_per_step_eager": getattr(form, "ms_eager", None), "sr_steps_per_s": 1e3 / ms,
         "effective_samples_per_s": Ns / tau / (ms * 1e-3),
         "sampler_effective_samples_per_s": Ns / tau / (phase[0] * 1e-3),
         "tau_int": tau, "tau_samples_per_chain": TAU_T, "acceptance": tau_rec["acceptance"],
         "phase_ms": {"sample_eloc_O": phase[0], "reductions": phase[1], "S": phase[2], "solve": phase[3],
                      "update": phase[4]},
         "sweeps_between_samples": form.sweeps, "learned_moves_per_sample": form.indep,
         "energy_per_site_after_training": {"steps": len(form.energy), "mean_last_20": float(e.mean()),
                                            "se_last_20": float(e.std(ddof=1) / np.sqrt(len(e))) if len(e) > 1
                                            else None,
                                            "trajectory_every_50": [round(float(x), 6) for x in form.energy[::50]]},
         "energy_per_site_trained_psi": {"value": tau_rec["energy_per_site"], "se": tau_rec["se_per_site"],
                                         "samples": TAU_T * TAU_CHAINS}}
    if form.retrain_ms:
        d["proposal_retrain_ms"] = float(np.mean(form.retrain_ms))
        d["proposal_dropped_at_retrains"] = form.drops
    if form.tuning:
        d["autotune_ms"] = {k: {str(c): round(ms, 4) for c, ms in v.items()} for k, v in form.tuning.items()}
    return d


# ----------------------------------------------------------------------------------
# Learned proposal at alpha = 4: 1-D TFIM N = 64, h = 1.0 and 2-D TFIM 8 x 8, h = 3.04,
# complex RBM alpha = 4 (M = 256, Np = 16704), 16384 chains; the psi is trained by SR with
# the learned moves on, then local Metropolis and the learned moves are compared there.
C4_TRAIN = 200
C4_SWEEP_SETS = [(1, 0), (2, 0), (4, 0), (8, 0), (0, 2), (0, 4), (1, 2), (1, 4)]
C4_RETRAIN_EPOCHS = 4    # passes over the 65536 configurations per retraining (every 10 SR steps)
C4_FINAL_EPOCHS = 16     # before the move sets are compared at the trained psi


def run_leg(ann, fn):
    """Runs one leg of the line (another workload, after the headline): an exception or a
    device status word raised during it is recorded in the leg's entry instead of ending the
    run, and the status word is read (and cleared) before and after it."""
    import ctypes as ct
    w = ct.c_uint(0)
    ann._lib.call("ann_status", ct.byref(w))
    before = w.value
    try:
        out = fn()
    except Exception as e:  # noqa: BLE001 (recorded in the line)
        out = {"error": f"{type(e).__name__}: {e}"}
    ann._lib.call("ann_status", ct.byref(w))
    if isinstance(out, dict) and (w.value or before):
        out["device_status"] = {"before": hex(before), "after": hex(w.value)}
    return out


def learned_proposal_leg(ann, st, name, H, train_steps=C4_TRAIN):
    import torch
    a, b, W = init_rbm(np.random.default_rng(SEED + 4), 64, 256)
    psi = ann.PsiRBM(W, 1.0, 0.0, True, a=a, b=b, precision="fp32")
    op = ann.Operator(H)
    td = ann.TDVP(psi.num_params, s_mode="bf16", solver="mixed", max_iter=10, tol=1e-12, stream=st)
    made = ann.MADE(64, MADE_H, seed=SEED + 5)
    mc = ann.MonteCarloLoop(N_CHAINS, 1, THERM, N_CHAINS, True, seed=SEED + 6, persistent=True)
    mc.set_history(HISTORY)
    ev = ann.ExpectationValue(stream=st)
    for _ in range(HISTORY // N_CHAINS):
        ev(op, psi, mc)
    made.train_on_samples(mc, steps=MADE_FIRST_EPOCHS * HISTORY // MADE_BATCH, batch=MADE_BATCH, lr=MADE_LR,
                          stream=st)
    mc.set_proposal(made, indep_per_sample=LEARNED_INDEP, min_acceptance=MIN_ACCEPT)
    energy, acc_hist, drops, retrain = [], [], 0, []
    td.capture_sr_step(op, psi, mc, SHIFT, LR, st)
    t0 = time.perf_counter()
    for k in range(1, train_steps):
        if k % RETRAIN_EVERY == 0:
            mc.refresh_stats(st)
            drops += int(mc.proposal_dropped)
            acc_hist.append(round(mc.proposal_acceptance, 4))
            retrain.append(cuda_ms(lambda: made.train_on_samples(mc, steps=C4_RETRAIN_EPOCHS * HISTORY // MADE_BATCH,
                                                                 batch=MADE_BATCH, lr=MADE_LR, stream=st), st))
            mc.set_proposal(made, indep_per_sample=LEARNED_INDEP, min_acceptance=MIN_ACCEPT)
        td.launch_sr_step(st)
        energy.append(td.E_local.real / 64)
    torch.cuda.synchronize()
    ms_step = (time.perf_counter() - t0) * 1e3 / max(train_steps - 1, 1)
    # the proposal retrained at the trained psi, then each move set from the same chains
    made.train_on_samples(mc, steps=C4_FINAL_EPOCHS * HISTORY // MADE_BATCH, batch=MADE_BATCH, lr=MADE_LR, stream=st)
    conf, ctr = mc.get_chains()
    rows = []
    for sw, ind in C4_SWEEP_SETS:
        m = ann.MonteCarloLoop(TAU_CHAINS * TAU_T, sw, 0, TAU_CHAINS, True, seed=SEED + 99, persistent=True)
        m.set_chains(conf[:TAU_CHAINS], ctr[:TAU_CHAINS])
        if ind:
            m.set_proposal(made, indep_per_sample=ind, min_acceptance=0.0)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        ann.ExpectationValue()(op, psi, m)
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t1) * 1e3 / TAU_T
        _, _, el = m.samples()
        x = el.real.reshape(TAU_T, TAU_CHAINS)
        tau = tau_int_sokal(x)
        acc = {"local": round(m.acceptance_rate, 4)}
        if ind:
            acc["learned"] = round(m.proposal_acceptance, 4)
        rows.append({"sweeps": sw, "learned_moves": ind, "tau_int": tau, "acceptance": acc,
                     "ms_per_sample_pass": ms, "effective_samples_per_s_sampler": TAU_CHAINS / tau / (ms * 1e-3),
                     "energy_per_site": float(x.mean() / 64), "se_per_site": float(x.std() * np.sqrt(tau / x.size) / 64)})
    best_local = max((r for r in rows if r["learned_moves"] == 0), key=lambda r: r["effective_samples_per_s_sampler"])
    best_learned = max((r for r in rows if r["learned_moves"] > 0), key=lambda r: r["effective_samples_per_s_sampler"])
    e = np.asarray(energy[-20:])
    return {"workload": name, "num_params": psi.num_params, "chains": N_CHAINS, "train_steps": train_steps,
            "ms_per_sr_step": ms_step, "sr_step": "1 local sweep + 2 learned moves per sample, BF16 tcgen05 S, "
                                                  "mixed solve, graph replays (retraining included)",
            "energy_per_site_last_20": float(e.mean()) if len(e) else None,
            "energy_trajectory_every_20": [round(float(x), 6) for x in energy[::20]],
            "proposal": {"acceptance_at_retrains": acc_hist, "dropped_at_retrains": drops,
                         "retrain_ms": float(np.mean(retrain)) if retrain else None,
                         "retrain_epochs": C4_RETRAIN_EPOCHS, "final_epochs": C4_FINAL_EPOCHS,
                         "note": "acceptance of the last pass before each retraining (0 after a drop: the "
                                 "learned moves are off until re-armed by the retraining)"},
            "move_sets_at_trained_psi": rows,
            "learned_gain_effective_samples_per_s": best_learned["effective_samples_per_s_sampler"] /
            best_local["effective_samples_per_s_sampler"],
            "best_local": [best_local["sweeps"], 0], "best_learned": [best_learned["sweeps"],
                                                                     best_learned["learned_moves"]]}


# ----------------------------------------------------------------------------------
# CNN on the 2-D J1-J2 Heisenberg model: 10 x 10 periodic, J1 = 1, J2 = 0.5, Sz = 0
# (50 up spins), two periodic 3 x 3 conv layers (16 then 8 channels), log cosh, sum
# pooling, kernels N(0, 0.02^2), 32768 chains with exchange moves over the J1 and J2
# bonds (one sweep of 100 proposals between samples), S from centred O with split hi+lo
# BF16 products, FP64 Cholesky solve with diagonal shift 1e-4.
C3_CHAINS, C3_SWEEPS, C3_SHIFT = 32768, 1, 1e-4


def cnn_leg(ann, st, steps=3, warm=2):
    import torch
    rng = np.random.default_rng(SEED + 3)
    np_ = 16 * 9 + 16 * 8 * 9
    params = 0.02 * (rng.standard_normal(np_) + 1j * rng.standard_normal(np_))
    psi = ann.PsiCNN([1, 10, 10], [16, 8], [[1, 3, 3], [1, 3, 3]], np.zeros(100, np.uint32), params, 1.0, 0.0,
                     True, activation="logcosh", precision="fp32")
    op = ann.Operator(ann.heisenberg_j1j2_2d(10, 10, 1.0, 0.5))
    nn, nnn = ann.square_lattice_bonds(10, 10, diagonal=True)
    mc = ann.MonteCarloSpins(C3_CHAINS, C3_SWEEPS, 8, C3_CHAINS, True, move="exchange",
                             bonds=np.array(nn + nnn, np.uint32), n_up=50, seed=SEED + 7, persistent=True)
    td = ann.TDVP(np_, s_mode="bf16_split", solver="fp64", stream=st)
    for _ in range(warm):
        td.sr_step(op, psi, mc, C3_SHIFT, LR)
    ann._lib.call("ann_set_phase_timing", 1)
    phase = np.zeros(5)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        td.sr_step(op, psi, mc, C3_SHIFT, LR)
        ph = np.zeros(5, np.float32)
        ann._lib.call("ann_get_phase_times", ann._lib.ptr(ph))
        phase += ph
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) * 1e3 / steps
    ann._lib.call("ann_set_phase_timing", 0)
    phase /= steps
    mc.refresh_stats(st)
    conf, _, _ = mc.samples()
    pop = np.array([bin(int(x)).count("1") + bin(int(y)).count("1") for x, y in conf[:256]])
    o_bytes = 8.0 * np_ * C3_CHAINS
    return {"workload": "2D J1-J2 10x10 PBC J2=0.5, Sz=0, PsiCNN 3x3 16 -> 8 channels log cosh (Np=1296), "
                        f"{C3_CHAINS} chains, exchange moves over J1+J2 bonds, {C3_SWEEPS} sweep (100 proposals) "
                        "between samples, hi+lo BF16 S, FP64 Cholesky, shift 1e-4",
            "ms_per_sr_step": ms, "sr_steps_per_s": 1e3 / ms,
            "phase_ms": {"sample_eloc_O": phase[0], "reductions": phase[1], "S": phase[2], "solve": phase[3],
                         "update": phase[4]},
            "samples_per_s": C3_CHAINS / (ms * 1e-3), "acceptance": mc.acceptance_rate,
            "sz_sector_kept": bool((pop == 50).all()), "energy_per_site": td.E_local.real / 100,
            "O_rows_hbm_gbs": o_bytes / (phase[0] * 1e-3) / 1e9,
            "note": "synchronous eager steps; the sampler phase is SIMT-bound (psi ratios of 400 bond "
                    "pairs per sample from the 3x3 / 5x5 cones), O rows are 8 * Np bytes per sample"}


def cnn_cpu_seconds_per_sample():
    """The FP64 oracle's restatement (not the reference: it caps N at 64 and channels at
    6) on one 10x10 sample: one exchange sweep of full forward passes, the J1-J2 local
    energy and the O_k row."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from pyoracle import CnnDesc, Oracle
    ex = _expression_module()
    rng = np.random.default_rng(SEED + 3)
    np_ = 16 * 9 + 16 * 8 * 9
    params = 0.02 * (rng.standard_normal(np_) + 1j * rng.standard_normal(np_))
    ref = CnnDesc([1, 10, 10], [16, 8], [[1, 3, 3], [1, 3, 3]], np.zeros(100, np.uint32), params, 1.0,
                  activation=1)
    o = Oracle()
    nn, nnn = ex.square_lattice_bonds(10, 10, diagonal=True)
    H = ex.heisenberg_j1j2_2d(10, 10, 1.0, 0.5)
    t0 = time.perf_counter()
    r = o.cnn_mc_philox(ref, H, 1, SEED, 1, 1, 0, move_kind=1, bonds=np.array(nn + nnn, np.uint32), n_up=50)
    o.cnn_O_k(ref, int(r["sconf"][0]) | (int(r["sconf"][1]) << 64))
    return time.perf_counter() - t0


# ----------------------------------------------------------------------------------
# Batched uneven instances: 96 1-D TFIM chains, L uniform on {12, 16, ..., 48}, h uniform
# on [0.5, 1.5], J = 1, complex RBM with alpha from {1, 2, 4} and a per-instance seed;
# chains 512 .. 8192 in proportion to Np; per-instance FP64 Cholesky SR solves.
N_INST = 96
BATCH_SWEEPS = 4
BATCH_MADE_H = 64
BATCH_HISTORY_PASSES = 4
BATCH_MADE_STEPS = 64


def batched_instances(ann, st, steps):
    """One persistent sampling + E_loc launch for all instances (local sweeps and each
    instance's learned proposal), per-instance S (BF16 tcgen05) and FP64 Cholesky solves on
    a stream pool, the whole step one CUDA graph; against the same instances stepped one
    after another (one CUDA graph each). Energies of the instances with L <= 20 against
    exact summation."""
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
        mc.set_history(BATCH_HISTORY_PASSES * chains[k])
        td = ann.TDVP(psi.num_params, s_mode="bf16", solver="fp64", stream=st)
        return psi, op, mc, td

    def arm_proposals(inst, batch=None):
        """Fills each instance's history with BATCH_HISTORY_PASSES sampling passes, trains its
        MADE (L -> 64 -> L) on them and switches the learned moves on."""
        for _ in range(BATCH_HISTORY_PASSES):
            if batch is not None:
                batch.sample()
            else:
                for psi, op, mc, _ in inst:
                    ann.ExpectationValue(stream=st)(op, psi, mc)
        mades = []
        for k, (psi, op, mc, _) in enumerate(inst):
            made = ann.MADE(psi.N, BATCH_MADE_H, seed=SEED + 3000 + k)
            made.train_on_samples(mc, steps=BATCH_MADE_STEPS, batch=1024, lr=MADE_LR, stream=st)
            mc.set_proposal(made, indep_per_sample=LEARNED_INDEP, min_acceptance=MIN_ACCEPT)
            mades.append(made)
        return mades

    def timed(fn, n):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(st)
        for _ in range(n):
            fn()
        e1.record(st)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n

    inst = [make(k) for k in range(N_INST)]
    batch = ann.Batch(*[list(x) for x in zip(*inst)], stream=st)
    mades = arm_proposals(inst, batch)  # noqa: F841 (kept alive with the ensembles)
    batch.capture_sr_step(SHIFT, LR, st)  # runs one eager step first
    batch.launch_sr_step(st)
    ms_batched = timed(lambda: batch.launch_sr_step(st), steps)
    batch.sample()
    E = batch.energies()
    acc = []
    for _, _, mc, _ in inst:
        mc.refresh_stats(st)
        acc.append(mc.proposal_acceptance)
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
    # the same step with the mixed-precision solve per instance (FP32 Cholesky on the tensor
    # cores + FP64 refinement to ||r|| / ||F|| <= 1e-12), for comparison. Inside the graph a
    # refinement that fails (an instance whose S + shift is too ill-conditioned for the FP32
    # factor) has no FP64 fallback: it raises the stall flag and leaves that instance's step
    # at zero; the comparison then records the instances instead of a time.
    import ctypes as ct
    for _, _, _, td in inst:
        td.set_solver("mixed", 10, 1e-12)
    try:
        batch.capture_sr_step(SHIFT, LR, st)
        ms_batched_mixed = timed(lambda: batch.launch_sr_step(st), steps)
        word = ct.c_uint(0)
        ann._lib.call("ann_status", ct.byref(word))  # reads and clears the device status word
        if word.value:
            raise RuntimeError(f"device status 0x{word.value:x} after the mixed-solver graph steps")
    except Exception as e:  # noqa: BLE001 (the status word names the failure)
        failed = [{"instance": k, "L": specs[k][0], "alpha": specs[k][2], "num_params": nps[k],
                   "chains": chains[k], **td.solver_info}
                  for k, (_, _, _, td) in enumerate(inst) if td.solver_info["fell_back"]]
        ms_batched_mixed = {"error": f"{type(e).__name__}: {e}", "instances_not_converged": failed}
        ann._lib.lib.ann_status(ct.byref(ct.c_uint(0)))  # clear what is left of the status word
    del batch, inst, mades
    torch.cuda.empty_cache()
    seq = [make(k) for k in range(N_INST)]
    mades = arm_proposals(seq)  # noqa: F841
    for psi, op, mc, td in seq:
        td.capture_sr_step(op, psi, mc, SHIFT, LR, st)
    ms_seq = timed(lambda: [td.launch_sr_step(st) for (_, _, _, td) in seq], steps)
    samples = sum(chains)
    return {"instances": N_INST, "samples_per_step": samples, "num_params_range": [lo, hi],
            "chains_range": [min(chains), max(chains)], "sweeps_between_samples": BATCH_SWEEPS,
            "solver": "per-instance FP64 Cholesky + 1 refinement step",
            "learned_proposal": {"made": f"L -> {BATCH_MADE_H} -> L per instance, trained on "
                                         f"{BATCH_HISTORY_PASSES} sampling passes", "moves_per_sample": LEARNED_INDEP,
                                 "acceptance_mean": float(np.mean(acc)), "acceptance_min": float(np.min(acc)),
                                 "dropped": int(sum(a < MIN_ACCEPT for a in acc))},
            "form": "BF16 tcgen05 S + learned proposal + one batched sampling launch (the combined form)",
            "ms_per_step_batched": ms_batched, "ms_per_step_one_by_one": ms_seq,
            "ms_per_step_batched_mixed_solver": ms_batched_mixed,
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
    reps = 3
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        _, d = hsd.gradient(f.psi, psi_p, op, True, f.mc, 1.0)
    ms = (time.perf_counter() - t0) * 1e3 / reps
    return {"ms_per_gradient_call": ms, "samples": N_CHAINS, "distance": d,
            "note": "host-synchronous calls (the gradient returns to the host), 64-sweep sampling included"}


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of the precision step's kernels
# from one capture of this workload at full size with those one-pass metrics:
#   python bench.py --form precision --steps 1 --warmup 1 --train-steps 3 --no-cpu --no-legs \
#       --save-tuning tuning.json
#   ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum \
#       --clock-control none --profile-from-start off --csv --log-file traffic.csv \
#       python bench.py --form precision --steps 1 --warmup 1 --train-steps 3 --no-cpu --no-legs \
#       --tuning tuning.json --profile-window
# sampler: one launch (half-warp chains, O rows 1.10 GB written); S: one herk_tc launch
# (complex64 S); factorisation: its 129 tcgen05 update launches (10.37 GB) and the panel
# kernels potrf32 / trsm32 (0.44 GB), per factorisation.
TRAFFIC_BYTES = {"sampler": 1.0583e9, "herk_tc": 6.4523e9, "factorisation": 1.0811e10}
TRAFFIC_SRC = "DRAM bytes per launch from one full-size ncu capture of this workload (one-pass metrics)"


def sampler_kernel_name(ann):
    """The sampler instance the tuning table selects for the 8x8 shape (whole- or
    half-warp chains)."""
    team = next((v for k, v in ann.tuning_table().items()
                 if f"/rbm_mc.team/N{N_SITES}.M{M_HIDDEN}." in k and k.endswith("made1")), 32)
    return ("rbm_mc_kernel<float,1,8,16> (half-warp chains; sampling + E_loc + O rows)" if team == 16 else
            "rbm_mc_kernel<float,1,4,32> (sampling + E_loc + O rows)")


def roofline_objects(f, ms, phase, pk, pk_kind):
    """The dominant kernel of the precision step (the sampler at 64 sweeps) and the other
    two large kernel groups, each with its algorithmic work per launch."""
    Np, Ns = f.Np, N_CHAINS
    props = Ns * (SWEEPS * N_SITES)
    simt_peak = fp32_simt_peak_tflops()
    flops_sampler = 34.0 * M_HIDDEN * props  # 34 M flops per proposal (the 64-sweep part alone)
    sampler = {"bound": "fp32_simt", "kernel": sampler_kernel_name(f.ann),
               "achieved": flops_sampler / (phase[0] * 1e-3) / 1e12, "peak": simt_peak, "unit": "TFLOP/s",
               "frac": flops_sampler / (phase[0] * 1e-3) / 1e12 / simt_peak, "ms": phase[0],
               "traffic": TRAFFIC_BYTES["sampler"],
               "dram_gbs": TRAFFIC_BYTES["sampler"] / (phase[0] * 1e-3) / 1e9,
               "traffic_source": TRAFFIC_SRC,
               "work": f"34*M flops per single-flip proposal x {props} proposals per step (16384 chains x 64 "
                       "sweeps x 64 sites); E_loc and the O-row writes (1.1 GB) are not credited",
               "peak_kind": "nominal FP32 FMA rate (SMs x 128 lanes x 2 flops x max SM clock): "
                            "MEASURED_PEAKS.json holds no SIMT figure"}
    flops_S = 4.0 * Np * (Np + 1) * Ns
    herk = {"bound": "tensor", "kernel": "herk_tc_kernel (S = O_c^H O_c, tcgen05 BF16)",
            "achieved": flops_S / (phase[2] * 1e-3) / 1e12, "peak": pk.get("bf16_tflops", 1900.0),
            "unit": "TFLOP/s", "peak_kind": pk_kind + " bf16 burst", "ms": phase[2],
            "traffic": TRAFFIC_BYTES["herk_tc"], "traffic_source": TRAFFIC_SRC,
            "work": "4*Np*(Np+1)*Ns real flops per step (over the S phase: operand prep + kernel)"}
    herk["frac"] = herk["achieved"] / herk["peak"]
    out = {"roofline": sampler, "roofline_herk": herk}
    if f.t_factor_ms:
        chol = (4.0 / 3.0) * Np ** 3 / (f.t_factor_ms * 1e-3) / 1e12
        peak = pk.get("bf16_tflops", 1900.0)
        out["roofline_factorisation"] = {
            "bound": "tensor", "kernel": "FP32 Cholesky factorisation (tcgen05 split-TF32 trailing updates + "
                                        "potrf32/trsm32 panel path)",
            "achieved": chol, "peak": peak, "unit": "TFLOP/s", "frac": chol / peak, "ms": f.t_factor_ms,
            "traffic": TRAFFIC_BYTES["factorisation"],
            "traffic_source": "DRAM bytes per factorisation (all its launches) from one full-size ncu capture",
            "update_form": f.tdvp.solver_info.get("update_form"),
            "peak_kind": pk_kind + " bf16 burst (no credit for the three split products)",
            "work": "(4/3)*Np^3 real flops per factorisation (CUDA events around it)"}
    return out


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
    t_train = {}
    for name in forms:
        f = Form(ann, name, rank)
        f.prepare(st)
        t0 = time.perf_counter()
        f.train(args.train_steps, st)
        torch.cuda.synchronize()
        t_train[name] = time.perf_counter() - t0
        if name == "precision" or len(forms) == 1:
            clocks.start()
        ms, phase, launches = timed_steps(f, args, st, dist)
        if name == "precision" or len(forms) == 1:
            clk = clocks.stop()
        f.mc.refresh_stats(st)
        info = f.tdvp.solver_info
        tau_rec = f.tau_run(f.sweeps, f.indep)
        results[name] = (f, ms, phase, launches, tau_rec, info)

    main = results["precision"] if "precision" in results else results[forms[0]]
    f, ms, phase, launches, tau_rec, info = main
    tau = tau_rec["tau_int"]
    Np, Ns = f.Np, N_CHAINS
    energy = f.energy_check()
    summary = {name: form_summary(r[0], r[1], r[2], r[4]) for name, r in results.items()}
    timeline = None
    if f.tdvp.solver_info.get("update_form") == "tensor core, rank 128 per panel pair":
        timeline = factor_timeline(ann, f.tdvp)  # one more solve of the last S, outside the timed steps

    # end to end through the public API: parameters from pinned host memory in, the
    # step's energy out, every step
    host_params = torch.from_numpy(f.psi.params.view(np.float64).copy()).pin_memory()
    f.capture(st)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(args.steps):
        f.psi.set_params_async(host_params, st)
        f.graph_step(st)
        _ = f.tdvp.E_local  # device -> host read of the step's energy (synchronising)
    st.synchronize()
    ms_e2e = (time.perf_counter() - t0) * 1e3 / args.steps

    pk, pk_kind = peaks()
    ms_w, ms_e2e_w, value, e2e_value = whole_job(ms, ms_e2e, Ns, tau, dist)
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_w, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": ("c64 sampling + learned proposal / bf16 S (fp32 acc) / fp32 Cholesky + f64 refinement"
                  if f.name == "precision" else "c64 sampling / fp32 S / fp32 Cholesky"),
        "data": "synthetic (seeded random-init RBM trained by SR, 2D TFIM)",
        "config": config_dict(f.name),
        "sr_steps_per_s": 1e3 / ms_w, "ms_per_step_eager": f.ms_eager, "tau_int": tau,
        "tau_samples_per_chain": TAU_T, "acceptance": tau_rec["acceptance"],
        "energy_per_site": energy["energy_per_site"], "energy_check": energy,
        "phase_ms": summary[f.name]["phase_ms"],
        "phase_note": "CUDA-event phases of eager steps (the headline times graph replays)",
        "solver": info, "factorisation_timeline": timeline, "train_seconds": t_train,
        "clocks": clk,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": Np * 16,
                "d2h_bytes_per_step": 16, "ms_per_step": ms_e2e_w},
        "gpu_launches": int(launches),
    }
    out.update(roofline_objects(f, ms, phase, pk, pk_kind))
    out["forms"] = summary
    if "plain" in results and "precision" in results:
        p, q = summary["plain"], summary["precision"]
        out["vs_plain"] = {k: q[k] / p[k] for k in ("sr_steps_per_s", "effective_samples_per_s",
                                                    "sampler_effective_samples_per_s")}
        ep, eq = p["energy_per_site_trained_psi"], q["energy_per_site_trained_psi"]
        out["matched_energy"] = {"plain": ep["value"], "precision": eq["value"],
                                 "abs_diff_per_site": abs(ep["value"] - eq["value"]),
                                 "combined_se_per_site": float(np.hypot(ep["se"], eq["se"])),
                                 "note": "each form's psi after the same 300 SR steps from the same initial "
                                         "parameters, sampled with its own moves (200 x 4096 samples)"}
        out["forms"]["plain"]["energy_check"] = results["plain"][0].energy_check()
    if not args.no_legs:
        # error against FP64 of each result (same samples), then the ablation of the moves
        out["fp64_errors"] = {name: r[0].fp64_errors(st) for name, r in results.items()}
        if f.made is not None:
            out["tau_ablation_trained_psi"] = [f.tau_run(sw, ind) for sw, ind in
                                               ((1, 0), (4, 0), (16, 0), (64, 0), (0, 2), (1, 2), (64, 2))]
        if f.name == "precision":
            d_mixed = f.tdvp.solve(SHIFT)
            f.tdvp.set_solver("fp64")
            d_fp64 = f.tdvp.solve(SHIFT)
            out["ms_per_step_fp64_cholesky"] = cuda_ms(lambda: f.step(st), st)
            f.tdvp.set_solver("mixed", 10, 1e-12)
            out["solve_rel_err_vs_fp64_cholesky"] = float(np.linalg.norm(d_mixed - d_fp64) / np.linalg.norm(d_fp64))
            out["hilbert_space_distance"] = hsd_timing(ann, f, st)
        del results
        torch.cuda.empty_cache()
        c4_train = min(C4_TRAIN, max(args.train_steps, 2))
        out["learned_proposal_alpha4"] = [
            run_leg(ann, lambda: learned_proposal_leg(ann, st, "1D TFIM N=64 PBC h=1.0, complex RBM alpha=4 (M=256)",
                                                      ann.transverse_field_ising_1d(64, 1.0), c4_train)),
            run_leg(ann, lambda: learned_proposal_leg(ann, st, "2D TFIM 8x8 PBC h=3.04, complex RBM alpha=4 (M=256)",
                                                      ann.transverse_field_ising_2d(8, 8, h=3.04), c4_train))]
        torch.cuda.empty_cache()
        out["cnn_j1j2_10x10"] = run_leg(ann, lambda: cnn_leg(ann, st))
        if rank == 0 and not args.no_cpu and "error" not in out["cnn_j1j2_10x10"]:
            t_cpu = cnn_cpu_seconds_per_sample()
            out["cnn_j1j2_10x10"]["cpu_oracle"] = {"seconds_per_sample": t_cpu, "cores": 1,
                                                   "kind": "port (not the reference: it caps N at 64, channels at 6)",
                                                   "samples_per_s": 1.0 / t_cpu}
        torch.cuda.empty_cache()
        out["batched_instances"] = run_leg(ann, lambda: batched_instances(ann, st, 2))
    if rank == 0 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(*init_params(np.random.default_rng(SEED)),
                                           _expression_module().transverse_field_ising_2d(L, L, h=H_FIELD), tau)
    if rank == 0:
        print(json.dumps(out))
    if dist:
        torch.distributed.destroy_process_group()


# ----------------------------------------------------------------------------------
def cpu_step_seconds(a, b, W, H, n_samples=4, with_chol=True):
    """The FP64 oracle (a restatement of the reference's host path, which runs one chain on
    one core) on a bounded sample of one SR step: per sample 64 sweeps of single-flip
    Metropolis, the local energy, the O_k row and its S/F accumulation; plus a complex
    Cholesky solve timed at n = 2048. Returns (seconds per sample of MC, of TDVP, seconds
    of the n = 2048 Cholesky or None)."""
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
    if not with_chol:
        return t_mc, t_tdvp, None
    n = 2048
    A = np.random.default_rng(0).standard_normal((n, n)) + 1j * np.random.default_rng(1).standard_normal((n, n))
    A = A @ A.conj().T + n * np.eye(n)
    t0 = time.perf_counter()
    np.linalg.cholesky(A)
    t_chol = time.perf_counter() - t0
    return t_mc, t_tdvp, t_chol


def cpu_baseline(a, b, W, H, tau, cores=1):
    t_mc, t_tdvp, t_chol = cpu_step_seconds(a, b, W, H)
    t_chol_full = t_chol * (NP_C2 / 2048) ** 3
    step_s = N_CHAINS * (t_mc + t_tdvp) + t_chol_full
    return {"value": N_CHAINS / tau / step_s, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"4 samples (64 sweeps, E_loc, O_k, S rows) timed; the SR step's time = {N_CHAINS} x that "
                      f"per-sample time + the Cholesky of n=8384 (timed at n=2048, scaled by n^3); tau_int from the "
                      "GPU run",
            "seconds_per_step": step_s, "s_per_sample_mc": t_mc, "s_per_sample_tdvp": t_tdvp,
            "s_cholesky_n2048": t_chol}


def _expression_module():
    # the Hamiltonian builder alone (pure Python); the CPU legs never load the CUDA library
    import importlib.util
    spec = importlib.util.spec_from_file_location("_ann_expression",
                                                  os.path.join(ROOT, "annongpu_gb300", "expression.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


REF_SAMPLES_PER_PROC = 2


def _cpu_worker(_):
    a, b, W = init_params(np.random.default_rng(SEED))
    H = _expression_module().transverse_field_ising_2d(L, L, h=H_FIELD)
    t_mc, t_tdvp, _ = cpu_step_seconds(a, b, W, H, n_samples=REF_SAMPLES_PER_PROC, with_chol=False)
    return t_mc, t_tdvp


def run_reference(args):
    """The reference's CPU path for this workload, restated in the FP64 oracle (the
    reference's own host build is x86-only here and is not on the GPU machine): each step is a
    bounded sample of the SR step, timed in full: P worker processes (all host cores) each
    run REF_SAMPLES_PER_PROC samples (64 sweeps, E_loc, O_k row, S/F accumulation), plus
    the samples' share of the n = 8384 Cholesky (a numpy solve timed at n = 1024 once,
    scaled by n^3). value = samples / seconds of the bounded step (tau_int = 1)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import multiprocessing as mp
    P = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    t_start = time.perf_counter()
    n = 1024
    A = np.random.default_rng(0).standard_normal((n, n)) + 1j * np.random.default_rng(1).standard_normal((n, n))
    A = A @ A.conj().T + n * np.eye(n)
    t0 = time.perf_counter()
    np.linalg.cholesky(A)
    t_chol_full = (time.perf_counter() - t0) * (NP_C2 / n) ** 3
    steps = []
    with ctx.Pool(P) as pool:
        for k in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            vals = pool.map(_cpu_worker, range(P), chunksize=1)
            wall = time.perf_counter() - t0
            samples = P * REF_SAMPLES_PER_PROC
            # the Cholesky share of these samples (one solve per 16384 samples)
            step_s = wall + t_chol_full * samples / N_CHAINS
            if k >= args.warmup:
                steps.append((step_s, samples, vals))
    step_s = float(np.mean([s for s, _, _ in steps]))
    samples = steps[0][1]
    value = samples / step_s
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "c128", "data": "synthetic (seeded random-init RBM, 2D TFIM)",
           "config": config_dict("precision" if args.form == "both" else args.form), "impl": "reference",
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": P, "kind": "port",
                            "sample": f"per step {P} worker processes (one pool, started before the warm-up "
                                      f"steps) x {REF_SAMPLES_PER_PROC} samples of the SR step (64 sweeps, E_loc, "
                                      "O_k, S/F rows), the step's wall time measured in full, plus the samples' "
                                      f"share of the n=8384 Cholesky (timed at n={n}, scaled by n^3); tau_int = 1 "
                                      "assumed",
                            "seconds_per_sample_per_core": float(np.mean([sum(v) for _, _, vs in steps for v in vs]))},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "wall_s": time.perf_counter() - t_start}
    print(json.dumps(out))


def run_profile_case(solver="fp64"):
    """Small case for ncu captures (a few GB at most, one SR step after one warm-up):
    N=32, M=64 complex RBM (Np = 2144), 1-D TFIM, 16384 chains, 4 sweeps between
    samples, BF16 tensor-core S, SR solve by `solver` (fp64 / mixed / fp32)."""
    import annongpu_gb300 as ann
    rng = np.random.default_rng(0)
    a, b, W = init_rbm(rng, 32, 64)
    psi = ann.PsiRBM(W, 1.0, 0.0, True, a=a, b=b, precision="fp32")
    op = ann.Operator(ann.transverse_field_ising_1d(32, 1.0))
    mc = ann.MonteCarloLoop(16384, 4, 8, 16384, True, seed=1, persistent=True)
    td = ann.TDVP(psi.num_params, s_mode="bf16", solver=solver)
    for _ in range(2):
        td.sr_step(op, psi, mc, 1e-3, 0.01)
    print("profile case: E/N =", td.E_local / 32)


def run_profile_case_sampler(team=32):
    """Small case for ncu captures of the sampler: the 8x8 workload's shapes (N = 64,
    M = 128, h = 3.04) with 4096 chains (O rows 275 MB), 8 sweeps between samples, two
    sampling passes with E_loc and O rows (TDVP evaluations, BF16 S); chains of `team`
    lanes (32: one per warp, 16: two per warp)."""
    import torch
    import annongpu_gb300 as ann
    ann.set_tuning({f"dev{torch.cuda.current_device()}/rbm_mc.team/N{N_SITES}.M{M_HIDDEN}.U4.P0.made0": team})
    a, b, W = init_params(np.random.default_rng(SEED))
    op = ann.Operator(ann.transverse_field_ising_2d(L, L, h=H_FIELD))
    psi = ann.PsiRBM(W, 1.0, 0.0, True, a=a, b=b, precision="fp32")
    mc = ann.MonteCarloLoop(4096, 8, 8, 4096, True, seed=6, persistent=True)
    td = ann.TDVP(psi.num_params, s_mode="bf16", solver="mixed")
    for _ in range(2):
        td.eval(op, psi, mc)
    print("profile case (sampler): E/N =", td.E_local / N_SITES)


def factor_timeline(ann, td, shift=SHIFT, level=1):
    """Event timeline of one FP32 factorisation (pair form): per panel pair the tile-column
    update that precedes it, the look-ahead stream's panel kernels and the rest of the
    tensor-core update beside them, in microseconds. Level 2 also splits the panel pair into
    its four kernels; its extra events make those kernels run one after the other instead of
    as programmatic dependent launches."""
    import ctypes as ct
    ann._lib.call("ann_set_factor_trace", level)
    td.solve(shift)
    out = np.zeros(2 * 8192)
    n = ct.c_uint(0)
    ann._lib.call("ann_get_factor_trace", ann._lib.ptr(out), 8192, ct.byref(n))
    ann._lib.call("ann_set_factor_trace", 0)
    ev = out[: 2 * n.value].reshape(-1, 2)
    tags, t = ev[:, 0].astype(int), ev[:, 1] * 1e3
    starts = [i for i, g in enumerate(tags) if g == 200]
    rows = []
    for k, i0 in enumerate(starts):
        seg = list(zip(tags[i0: starts[k + 1] if k + 1 < len(starts) else len(tags)],
                       t[i0: starts[k + 1] if k + 1 < len(starts) else len(tags)]))
        d, p110 = {}, []
        for g, tt in seg:
            (p110.append(tt) if g == 110 else d.__setitem__(g, tt))
        if 103 not in d or (level == 2 and len(p110) < 2):
            continue
        row = {"tile_column_update": d[201] - d[200], "stream_hand_off": d[100] - d[201]}
        if level == 2:
            row.update({"potrf_1": p110[0] - d[100], "trsm_1": d[101] - p110[0], "potrf_2": p110[1] - d[101],
                        "trsm_2": d[103] - p110[1]})
        row.update({"panel_pair": d[103] - d[100], "rest_of_update": d[202] - d[201], "iteration": d[203] - d[200]})
        rows.append(row)
    keys = list(rows[0]) if rows else []
    return {"pairs": len(rows), "total_ms": float(t.max() / 1e3) if len(t) else None,
            "sum_us": {k: float(sum(r[k] for r in rows)) for k in keys},
            "first_pair_us": {k: round(rows[0][k], 1) for k in keys} if rows else None,
            "last_pair_us": {k: round(rows[-1][k], 1) for k in keys} if rows else None,
            "panel_bound_pairs": int(sum(r["panel_pair"] + r["stream_hand_off"] > r["rest_of_update"] for r in rows))}


def run_profile_case_factor():
    """The 8x8 workload's S (Np = 8384, BF16, 16384 samples of the random-init RBM), the
    mixed solve autotuned, then the event timeline of one FP32 factorisation."""
    import annongpu_gb300 as ann
    a, b, W = init_params(np.random.default_rng(SEED))
    op = ann.Operator(ann.transverse_field_ising_2d(L, L, h=H_FIELD))
    psi = ann.PsiRBM(W, 1.0, 0.0, True, a=a, b=b, precision="fp32")
    mc = ann.MonteCarloLoop(N_CHAINS, 8, THERM, N_CHAINS, True, seed=3, persistent=True)
    td = ann.TDVP(psi.num_params, s_mode="bf16", solver="mixed")
    td.eval(op, psi, mc)
    ann.autotune(op, psi, mc, td, SHIFT)
    td.eval(op, psi, mc)
    for _ in range(3):
        td.solve(SHIFT)
    print(json.dumps({"factorisation_timeline": factor_timeline(ann, td),
                      "factorisation_timeline_kernels": factor_timeline(ann, td, level=2),
                      "tuning": {k: v for k, v in ann.tuning_table().items() if "chol" in k},
                      "solver": td.solver_info}))


def run_profile_case_made():
    """Small case for ncu captures of the proposal's training GEMMs: N = 64, H = 256 (the
    alpha = 4 workload's proposal), batches of 4096 configurations, 8 Adam steps (each one
    forward and backward pass: five tcgen05 GEMMs)."""
    import torch
    import annongpu_gb300 as ann
    rng = np.random.default_rng(SEED)
    m = ann.MADE(64, 256, seed=SEED)
    confs = rng.integers(0, 2 ** 63, size=(8192, 2), dtype=np.uint64)
    confs[:, 1] = 0
    m.train(confs, steps=2, batch=4096, lr=1e-3)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    loss = m.train(confs, steps=8, batch=4096, lr=1e-3)
    torch.cuda.synchronize()
    print(f"profile case (proposal training): 8 steps in {1e3 * (time.perf_counter() - t0):.2f} ms, loss {loss:.4f}")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--train-steps", type=int, default=TRAIN_STEPS,
                    help="SR steps of each form before the timed steps (the workload's 300)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--form", default="both", choices=["both", "precision", "plain"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-legs", action="store_true", help="headline only: skip the FP64 checks and other workloads")
    ap.add_argument("--profile-case", action="store_true", help="run the small ncu capture case and exit")
    ap.add_argument("--profile-solver", default="fp64",
                    choices=["fp64", "mixed", "fp32", "sampler", "sampler16", "made", "factor-trace"],
                    help="SR solver of the small profile case; 'sampler' / 'sampler16': the sampler case "
                         "(whole- / half-warp chains); 'made': the "
                         "proposal's training; 'factor-trace': event timeline of the 8x8 factorisation")
    ap.add_argument("--tuning", default=None, help="load this tuning table (from --save-tuning) instead of autotuning")
    ap.add_argument("--save-tuning", default=None, help="save the tuning table after the run")
    ap.add_argument("--profile-window", action="store_true",
                    help="bracket the timed steps with cudaProfilerStart/Stop (for ncu --profile-from-start off)")
    args = ap.parse_args()
    if args.warmup < 1 or args.steps < 1:
        ap.error("--steps and --warmup must be at least 1")
    if args.profile_case:
        if args.profile_solver in ("sampler", "sampler16"):
            run_profile_case_sampler(16 if args.profile_solver == "sampler16" else 32)
        elif args.profile_solver == "made":
            run_profile_case_made()
        elif args.profile_solver == "factor-trace":
            run_profile_case_factor()
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
