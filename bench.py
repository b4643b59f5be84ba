#!/usr/bin/env python3
"""Walker-steps/s of the phaseless AFQMC step on one GB300 (one JSON line).

Workload (default, the metric's configuration): norb=120, nalpha=nbeta=20,
nchol=600 synthetic Hamiltonian (vmc_gb300/synthetic.py: Cholesky variance
sigma_g^2 / norb, see `config.generator`), UHF trial and UHF walkers, 2048
walkers, dt=0.005.  One step = force bias, fields, VHS, propagator, overlap and
weights of every live walker, the walkers orthonormalised every 5 steps, an
energy estimate every step, and the reference's comb reconfiguration every 50
steps (its measurement cadence), which keeps the population alive.

`value` counts live walker-steps only (walkers with weight > 1e-8 when a step
begins; dead walkers are not propagated), from the library's device counter,
over the device time of the timed steps.

Forms, all on the same GPU:
  headline ("value"): mixed precision + control variate, an energy estimate
      every step (network for every walker, exact local energy of 1 walker in
      8, Horvitz-Thompson correction);
  mixed_fp64_lu_qr: the same with the overlap inverse / log-determinant and the
      walker QR in FP64 (block Gauss-Jordan, Householder);
  fp64_every_step: the plain FP64 form, exact local energy of every walker
      every step (the metric's comparison);
  mixed_every50 / fp64_every50: both forms at the reference's cadence;
  cfg1 / cfg3 / cfg4 / cfg5: the other workloads (see `forms`; cfg5 with its
      energy error against the FP64 form).
energy_check: over 100 steps with identical fields, the headline estimator and
the mixed form's exact energy against the FP64 form's exact energy.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the C++ restatement of the reference's walker step
(oracle/cpu_step.cpp; the reference's own C++ needs Boost, HDF5 and MPI, absent
here) on all host cores, same workload and metric.  Under torchrun every rank
runs an independent replica; rank 0 prints value = walker-steps of all ranks /
max time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "AFQMC walker-steps/s, mixed vs FP64 on same GB300, at ≤0.1 mEh energy error"
ORTHO_EVERY = 5
REF_CADENCE = 50
STAGES = ["fb", "fields", "vhs", "prop", "overlap", "weights", "ortho", "energy"]
# the reference's published per-core rate at its rhf_rhf regression size
# (N=13, 5/5 electrons, 64 Cholesky vectors; 20 walkers x 2499 steps in
# 1.34078 s of propagation on a Xeon Gold 6254, tests/DQMC/rhf_rhf/afqmc.ref)
REF_PUBLISHED_PER_CORE = 20 * 2499 / 1.34078
GENERATOR = ("Cholesky entries N(0, sigma_g^2 / norb), sigma_g = 0.5 exp(-g/20): the workload text's variance "
             "divided by norb, which keeps sum_g ||L_g||^2 near 10 (as the reference's H2O fixture) instead of "
             "growing with norb; the FLOP count is unchanged")
DTYPE = ("split-BF16 (3 passes, FP32 accumulation) force bias, VHS, propagator and exchange on tcgen05; overlap "
         "matrix from exact BF16 slices (FP64-grade); double-FP32 (~48-bit) LU, FP32 theta; Cholesky-QR with FP32 "
         "Gram/Cholesky/R^-1 and a compensated double-FP32 Q; FP64 weights, phases and determinant products")


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=50)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="cfg2")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--quick", action="store_true", help="headline form only")
    p.add_argument("--profile", action="store_true",
                   help="for ncu: headline form only, short training, no e2e / CPU legs (numbers not reported)")
    a = p.parse_args()
    if a.profile:
        a.quick = True
        a.no_cpu_baseline = True
    return a


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def fp32_nominal_tflops(sm_mhz=2070.0):
    """GB300 CUDA-core FP32: 152 SMs x 128 lanes x 2 FLOPs (FMA) per clock."""
    return 152 * 128 * 2 * sm_mhz * 1e6 / 1e12


# executed cost per algorithmic multiply-add of the mixed form's emulated arithmetic
SPLIT_BF16_PASSES = 3   # hi*hi + lo*hi + hi*lo tensor-core products per FP32-accurate product
OZAKI_PAIRS = 28        # slice pairs of levels 0..6 (7 slices per operand) per FP64-accurate product
DF32_LU_OPS = 14        # FP32 instructions per double-FP32 complex-part multiply-add in the LU
DF32_DOT_OPS = 11       # FP32 instructions per multiply-add of the compensated (Dot2) product Q = psi X


def mixed_stage_pipes(N, na, nb, G):
    """Work per walker of each stage of the mixed form: for each part, its
    algorithmic FLOPs (complex multiply-add = 8, real x complex = 4), the pipe
    that executes it and the executed instructions per algorithmic multiply-add
    (the bound of the part is FLOPs x cost / the pipe's peak):
      vhs      packed-triangle VHS: split-BF16 tensor-core products;
      prop     B exp-Taylor B products: split-BF16 tensor-core products;
      overlap  M = Phi^T psi by exact BF16 slices on the tensor cores, the LU in
               double-FP32, the inverse rows and theta = psi M^-1 in FP32;
      ortho    Cholesky-QR: Gram, Cholesky and R^-1 in FP32, Q = psi R^-1 as a
               compensated double-FP32 product.
    The force bias of the control-variate form runs inside its measurement."""
    T = N * (N + 1) // 2
    ns = [na, nb]
    return {
        "vhs": [("bf16x3", 4 * T * G, "tensor", SPLIT_BF16_PASSES)],
        "prop": [("bf16x3", sum(48 * N * N * n for n in ns), "tensor", SPLIT_BF16_PASSES)],
        "overlap": [("ozaki bf16 slices", sum(4 * n * n * N for n in ns), "tensor", OZAKI_PAIRS),
                    ("double-fp32 LU", sum(8 * n ** 3 / 3 for n in ns), "fp32", DF32_LU_OPS),
                    ("fp32 inverse rows + theta", sum(8 * n ** 3 + 8 * N * n * n for n in ns), "fp32", 1)],
        "ortho": [("fp32 Gram + Cholesky + R^-1", sum(4 * N * n * n + 8 * n ** 3 / 3 for n in ns), "fp32", 1),
                  ("double-fp32 Q = psi R^-1", sum(4 * N * n * n for n in ns), "fp32", DF32_DOT_OPS)],
    }


def flops_model(N, na, nb, G, ortho_every=ORTHO_EVERY):
    """Algorithmic FLOPs per walker: force bias, VHS, propagator with
    a real exp(-dt/2 h1') (2 real x complex + 5 complex x complex products per
    spin), overlap, QR amortised, and one exact local energy."""
    T = N * (N + 1) // 2
    ns = [na, nb]
    fb = sum(4 * n * n * N + 16 * n ** 3 + 8 * N * n * n + 4 * n * N * G for n in ns)
    vhs = 4 * T * G
    prop = sum(48 * N * N * n for n in ns)
    ovl = sum(4 * n * n * N + 5.3 * n ** 3 for n in ns)
    qr = sum(32 * N * n * n for n in ns) / ortho_every
    el = sum(4 * G * n * n * N + 8 * G * n * n + 4 * n * N for n in ns)
    return dict(fb=fb, vhs=vhs, prop=prop, overlap=ovl, ortho=qr, energy=el, step=fb + vhs + prop + ovl + qr)


class Clocks:
    """nvidia-smi samples during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(index), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], [], set()
        for line in self.f.read().splitlines():
            c = [x.strip() for x in line.split(",")]
            if len(c) < 9:
                continue
            try:
                sm.append(float(c[1]))
                mx.append(float(c[2]))
            except ValueError:
                continue
            for name, v in zip(["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"], c[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.f.name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return json.load(open(p)), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_port_rate(sysd, nchol_ene, threads, walkers_per_thread=8, steps=10, energy_every=1):
    """The C++ restatement of the reference's walker step (oracle/cpu_step.cpp:
    the reference's FP32 VHS, FP64 elsewhere) on `threads` host threads, one
    OpenMP thread per core standing in for one MPI rank per core, each with
    `walkers_per_thread` walkers: (walker-steps/s with an exact energy every
    `energy_every` steps, the same without energies, seconds, sample text)."""
    from oracle import afqmc_oracle as O
    from oracle import cpu_port as C
    N, na, nb = sysd["norb"], sysd["nalpha"], sysd["nbeta"]
    oh = O.Hamiltonian(N, na, nb, sysd["ecore"], sysd["h1"], sysd["h1mod"], sysd["chol"])
    ot = O.Trial(oh, sysd["trial"], sysd["phi_a"], sysd["phi_b"])
    rw = sysd["trial"] == "rhf"
    prop = O.Propagator(oh, ot.phi, 0.005, mode="ref")
    W = walkers_per_thread * threads
    cw = C.CpuWalkers(oh, ot, prop, rw, W, nthreads=threads, nchol_ene=nchol_ene)
    cw.set_walkers(np.repeat(O._ref_dets(oh, ot.phi, rw)[None], W, axis=0))
    e0 = O.hf_energy(ot, oh, ot.phi, rw).real
    t_step, t_qr, t_e, ws = cw.run_timed(steps, ORTHO_EVERY, energy_every, e0, max(100.0, W / 10.0))
    cw.close()
    total = t_step + t_qr + t_e
    return (ws / total, ws / (t_step + t_qr), total,
            "%d walkers (%d per thread) x %d steps of the same workload, QR every %d, exact local energy "
            "(%d Cholesky vectors) every %d step(s)" % (W, walkers_per_thread, steps, ORTHO_EVERY, nchol_ene,
                                                         energy_every))


def cpu_calibration():
    """The same C++ step at the reference's rhf_rhf regression size (its own
    fixture: N=13, 5/5, 64 Cholesky vectors, RHF walkers, 20 walkers, one
    thread), timed as the reference times its propagation (the step loop only),
    beside the reference's published per-core rate."""
    from oracle import afqmc_oracle as O
    from oracle import cpu_port as C
    from tests import refcases
    c = refcases.load("rhf_rhf")
    oh, ot, rw = c["ham"], c["trial"], c["rhf_walker"]
    prop = O.Propagator(oh, c["ref_phi"], float(c["cfg"]["sampling"]["dt"]), mode="ref")
    cw = C.CpuWalkers(oh, ot, prop, rw, 20, nthreads=1)
    cw.set_walkers(np.repeat(O._ref_dets(oh, c["ref_phi"], rw)[None], 20, axis=0))
    t_step, _, _, ws = cw.run_timed(1500, 20, 50, O.hf_energy(ot, oh, c["ref_phi"], rw).real)
    cw.close()
    rate = ws / t_step
    return {"fixture": "rhf_rhf (N=13, 5/5, 64 Cholesky vectors, RHF walkers)", "port_per_core": rate,
            "reference_published_per_core": REF_PUBLISHED_PER_CORE,
            "reference_hardware": "Xeon Gold 6254 @ 3.10 GHz (tests/DQMC/rhf_rhf/afqmc.ref)",
            "port_over_reference": rate / REF_PUBLISHED_PER_CORE,
            "representative": bool(rate * 3.0 >= REF_PUBLISHED_PER_CORE)}


def cpu_baseline(sysd, nchol_ene, threads=None):
    threads = threads or host_threads()
    v, v_noe, secs, sample = cpu_port_rate(sysd, nchol_ene, threads)
    cal = cpu_calibration()
    return {"value": v, "unit": "walker-steps/s", "cores": threads, "kind": "port", "sample": sample,
            "every50_value": 1.0 / (1.0 / v_noe + (1.0 / v - 1.0 / v_noe) / REF_CADENCE),
            "seconds": secs,
            "code": "oracle/cpu_step.cpp: C++ restatement of the reference's walker step (FP32 VHS as the "
                    "reference, FP64 elsewhere), g++ -O3 -fopenmp, one thread per core",
            "calibration": cal}


def make_walkers(A, sysd, form, device, nwalk=None, seed=20261203):
    N, na, nb = sysd["norb"], sysd["nalpha"], sysd["nbeta"]
    gh = A.Hamiltonian(N, na, nb, sysd["ecore"], sysd["h1"], sysd["h1mod"], sysd["chol"])
    gt = A.UHF(gh, sysd["phi_a"], sysd["phi_b"]) if sysd["trial"] == "uhf" else A.RHF(gh, sysd["phi_a"])
    return A.DQMCWalkers(gh, gt, nwalk or sysd["walkers"], sysd["trial"] == "rhf", 0.005, precision=form,
                         device=device, seed=seed)


def cholesky_truncation(wk, G, threshold=1e-3):
    """Cholesky vectors for the energy, the reference's rule (MixedEstimator.cpp:363-384):
    the first of 0.3 .. 0.7 G whose trial-state energy is within the threshold."""
    e_full = wk.ham_and_overlap().real.mean()
    for frac in (0.3, 0.4, 0.5, 0.6, 0.7):
        n = int(frac * G)
        wk.set_nchol_ene(n)
        if abs(e_full - wk.ham_and_overlap().real.mean()) < threshold:
            return n
    wk.set_nchol_ene(G)
    return G


def energy_all(A, wk):
    wk._check(A.lib().afqmc_local_energy(wk.h, None))


class Comb:
    """The reference's comb every REF_CADENCE steps (MixedEstimator.cpp:559-635),
    on the device, with zetas from a seeded host generator."""

    def __init__(self, seed=99):
        self.rng = np.random.default_rng(seed)

    def __call__(self, wk):
        wk.comb(float(self.rng.random()))


def timed(A, wk, k0, K, energy, cv=None, comb=None):
    """K steps on the device; energy in {"cv", "every", "every50"}; the comb
    every REF_CADENCE steps when given.  Returns (ms, launches, stage ms, live
    walker-steps)."""
    wk.sync()
    wk.enable_timing(True)
    l0 = wk.launch_count()
    n0 = wk.walker_steps()
    wk.timer_start()
    for k in range(k0, k0 + K):
        wk.propagate_phaseless(None)
        if (k + 1) % ORTHO_EVERY == 0:
            wk.orthogonalize()
        if energy == "cv":
            cv.measure(tag=k, slot=k % 4096)
        elif energy == "every" or (k + 1) % REF_CADENCE == 0:
            energy_all(A, wk)
        if comb is not None and (k + 1) % REF_CADENCE == 0:
            comb(wk)
    ms = wk.timer_stop()
    launches = wk.launch_count() - l0
    stage = {s: wk.stage_time(s) for s in STAGES}
    wk.enable_timing(False)
    live = wk.walker_steps() - n0
    return ms, launches, stage, live


def energy_check(A, sysd, device, wm, cv, nchol_ene, steps=100):
    """The energy error of the headline form, on the headline handle itself
    (its equilibrated walkers, the trained network attached).  Its walkers are
    copied into an FP64 handle; both then run `steps` steps with identical host
    fields and a fixed eshift (QR every 5), at the production cadence: every
    REF_CADENCE steps the comb reconfigures the mixed handle's walkers and the
    FP64 handle restarts from them (a precision error accumulates over at most
    REF_CADENCE steps, as between the reference's combs).  Per step: the FP64 form's exact
    mixed energy sum_w w E_L / sum_w w, the mixed form's exact one, the mixed
    form's control-variate estimate (Horvitz-Thompson and ratio corrections)
    and the plain 1/8 subsample estimate.  Reported: the precision error of
    the mixed form (mixed exact - FP64 exact; the mean over the steps, which
    the time-averaged AFQMC energy sees, and the largest single step), and the
    estimator's statistics against the mixed form's own exact energy (mean with
    its standard error: no bias is expected; noise per step; the variance gain
    over the plain subsample)."""
    from vmc_gb300 import cv as CV
    nw = wm.nwalk
    rng = np.random.default_rng(11)
    d, o, w = wm.get_det()
    wf = make_walkers(A, sysd, "fp64", device, nw)
    wf.set_nchol_ene(nchol_ene)
    wf.set_det(d, overlaps=o, weights=w)
    e0 = float((w * wm.ham_and_overlap().real).sum() / w.sum())
    ef, em = [], []
    zeta = np.random.default_rng(12)
    for k in range(steps):
        xi = rng.standard_normal((nw, sysd["nchol"]))
        for h in (wm, wf):
            h.propagate_phaseless(xi, e0)
            if (k + 1) % ORTHO_EVERY == 0:
                h.orthogonalize()
        CV.measure(wm, tag=70000 + k, slot=k)
        out = []
        for h in (wf, wm):
            wt = h.weights()
            el = h.ham_and_overlap().real
            out.append((wt * el).sum() / wt.sum())
        ef.append(out[0])
        em.append(out[1])
        if (k + 1) % REF_CADENCE == 0:
            wm.comb(float(zeta.random()))
            d, o, w = wm.get_det()
            wf.set_det(d, overlaps=o, weights=w)
    r = CV.results(wm, steps)
    wf.close()
    ef, em = np.array(ef), np.array(em)
    d_prec = (em - ef) * 1e3
    d_ht = (r[:, 1] - em) * 1e3
    d_ratio = (r[:, 0] - em) * 1e3
    d_sub = (r[:, 2] - em) * 1e3
    se = lambda x: float(x.std(ddof=1) / np.sqrt(len(x)))  # noqa: E731
    return {"walkers": nw, "steps": steps, "nchol_energy": nchol_ene,
            "precision_error_mEh": float(abs(d_prec.mean())),
            "precision_error_mEh_max_step": float(abs(d_prec).max()),
            "cv_minus_exact_mEh_mean": float(d_ht.mean()), "cv_minus_exact_mEh_stderr": se(d_ht),
            "cv_noise_mEh_per_step": float(d_ht.std(ddof=1)),
            "ratio_form_minus_exact_mEh_mean": float(d_ratio.mean()), "ratio_form_stderr": se(d_ratio),
            "plain_subsample_noise_mEh_per_step": float(d_sub.std(ddof=1)),
            "variance_gain_over_plain_subsample": float(d_sub.var(ddof=1) / max(d_ht.var(ddof=1), 1e-300)),
            "within_0p1_mEh": bool(abs(d_prec.mean()) <= 0.1),
            "estimator": "E_cv = [sum_w w f_w + sum_S pi_w^-1 w (E_w - f_w)] / sum_w w (Horvitz-Thompson, "
                         "exactly unbiased given the walkers)"}


def train_cv(A, wk, hidden=256, n_eq=120, n_skip=20, epochs=20, seed=3):
    """Equilibrate the walkers (device fields, QR every 5) collecting features
    and exact energies of a stratified 1/8 subsample after step n_skip, then
    train the network and attach it."""
    from vmc_gb300.cv import ControlVariate
    cv = ControlVariate(wk, hidden=hidden, den=8, seed=seed)
    for k in range(n_eq):
        wk.propagate_phaseless(None)
        if (k + 1) % ORTHO_EVERY == 0:
            wk.orthogonalize()
        if k >= n_skip:
            cv.collect()
    loss, n = cv.train(epochs=epochs, batch=512, lr=1e-3)
    return cv, loss, n


def tune_cache():
    cache = os.environ.get("AFQMC_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "vmc_gb300",
                                                            "autotune.txt"))
    os.makedirs(os.path.dirname(cache), exist_ok=True)
    return cache


def form_single(A, sysd, device, precision, steps, energy, cv_train=None, nchol_ene=None):
    """A workload's own timed line (autotuned kernels, device fields, QR every
    5, the comb every 50): value over live walker-steps."""
    W, G = sysd["walkers"], sysd["nchol"]
    wk = make_walkers(A, sysd, precision, device)
    tuned = None
    if precision == "mixed":
        tuned, _ = A.autotune(wk, tune_cache())
    n_ene = nchol_ene or cholesky_truncation(wk, G)
    wk.set_nchol_ene(n_ene)
    e0 = wk.ham_and_overlap().real.mean()
    wk.set_energy_estimate(e0, e0)
    cv, info = None, {}
    if energy == "cv":
        n_eq, n_skip = cv_train
        cv, loss, n = train_cv(A, wk, n_eq=n_eq, n_skip=n_skip)
        info = {"cv_train_steps": n_eq, "cv_train_samples": n, "cv_train_mse_std_units": loss}
    for k in range(3):
        wk.propagate_phaseless(None)
        if cv is not None:
            cv.measure(tag=k, slot=k)
    comb = Comb()
    ms, launches, stage, live = timed(A, wk, 3, steps, energy, cv, comb)
    wk.close()
    N, na = sysd["norb"], sysd["nalpha"]
    fl = flops_model(N, na, sysd["nbeta"], G)
    out = {"workload": "norb=%d nalpha=nbeta=%d nchol=%d walkers=%d %s" % (N, na, G, W, sysd["trial"].upper()),
           "form": precision + (" + control variate" if energy == "cv" else ""), "energy": energy,
           "value": live / (ms / 1e3), "live_fraction": live / (W * steps), "ms_per_step": ms / steps,
           "steps": steps, "nchol_energy": n_ene, "tuning": tuned, "gpu_launches": launches,
           "achieved_tflops_algorithmic": fl["step"] * live / (ms / 1e3) / 1e12,
           "stage_ms_per_step": {k: v / steps for k, v in stage.items()}}
    out.update(info)
    return out


def form_large(A, device, steps=50, nw_check=16, check_steps=10):
    """The large-system workload (norb=400, nalpha=nbeta=60, nchol=2400, 1024
    walkers): the mixed form timed at the reference's cadence (exact energy of
    every walker and the comb every 50 steps), and its energy error against the
    FP64 form on nw_check walkers after check_steps steps with identical host
    fields (QR every 5), both from the same perturbed trial determinants."""
    from vmc_gb300 import synthetic as S
    sysd = S.workload("cfg5")
    out = form_single(A, sysd, device, "mixed", steps, "every50")
    rng = np.random.default_rng(21)
    base = np.concatenate([sysd["phi_a"], sysd["phi_b"]], axis=1).astype(np.complex128)
    d0 = base[None] + 0.02 * (rng.standard_normal((nw_check,) + base.shape)
                              + 1j * rng.standard_normal((nw_check,) + base.shape))
    xs = [rng.standard_normal((nw_check, sysd["nchol"])) for _ in range(check_steps)]
    res = {}
    for form in ("mixed", "fp64"):
        wk = make_walkers(A, sysd, form, device, nw_check)
        if form == "mixed":
            A.set_tuning(wk, **(out["tuning"] or {}))
        wk.set_nchol_ene(out["nchol_energy"])
        wk.set_det(d0)
        e0 = float(wk.ham_and_overlap().real.mean())
        for k in range(check_steps):
            wk.propagate_phaseless(xs[k], e0)
            if (k + 1) % ORTHO_EVERY == 0:
                wk.orthogonalize()
        w = wk.weights()
        el = wk.ham_and_overlap().real
        res[form] = ((w * el).sum() / w.sum(), el)
        wk.close()
    out["energy_error_mEh"] = abs(res["mixed"][0] - res["fp64"][0]) * 1e3
    out["energy_check"] = {"walkers": nw_check, "steps": check_steps, "e_fp64": res["fp64"][0],
                           "e_mixed": res["mixed"][0],
                           "max_walker_el_diff_mEh": float(np.abs(res["mixed"][1] - res["fp64"][1]).max() * 1e3)}
    return out


def form_multisystem(A, device, reps=3):
    """Uneven multi-system batch: 16 synthetic systems, norb ~ U[40, 200],
    nocc = round(norb / 6), nchol = 5 norb, 256 walkers each, mixed form, each
    system autotuned for its size class, all advanced by one CUDA graph per
    replay (10 steps + QR every 5; no energy in the timed region)."""
    from vmc_gb300 import synthetic as S
    systems = S.multi_system_batch()
    hs, flops = [], 0.0
    for sd in systems:
        n = sd["nalpha"]
        gh = A.Hamiltonian(sd["norb"], n, n, sd["ecore"], sd["h1"], sd["h1mod"], sd["chol"])
        gt = A.UHF(gh, sd["phi_a"], sd["phi_b"])
        wk = A.DQMCWalkers(gh, gt, sd["walkers"], False, 0.005, precision="mixed", device=device, seed=7 + len(hs))
        A.autotune(wk, tune_cache())
        e0 = wk.ham_and_overlap().real.mean()
        wk.set_energy_estimate(e0, e0)
        hs.append(wk)
        flops += flops_model(sd["norb"], n, n, sd["nchol"])["step"] * sd["walkers"]
    g = A.StepGraph(hs, 10, ortho_every=5)
    g.launch()
    for h in hs:
        h.sync()
    n0 = sum(h.walker_steps() for h in hs)
    hs[0].timer_start()
    for _ in range(reps):
        g.launch()
    ms = hs[0].timer_stop()
    for h in hs:
        h.sync()
    live = sum(h.walker_steps() for h in hs) - n0
    W = sum(sd["walkers"] for sd in systems)
    out = {"workload": "16 systems, norb %s, 256 walkers each, UHF, mixed form, one CUDA graph"
                       % sorted(sd["norb"] for sd in systems),
           "value": live / (ms / 1e3), "live_fraction": live / (W * 10 * reps), "ms_per_step": ms / (10 * reps),
           "graph_nodes": g.nodes(), "energy": "none in the timed region",
           "achieved_tflops_algorithmic": flops * 10 * reps / (ms / 1e3) / 1e12}
    g.close()
    for h in hs:
        h.close()
    return out


# DRAM bytes of one launch of the tensor-core propagator on this workload
# (dram__bytes_read.sum + dram__bytes_write.sum of one ncu capture, 2048 walkers
# x 2 spins): k_prop_tc2 197.8 + 179.6 MB, k_prop_tc 198 + 179 MB; a recorded
# constant, refreshed with each capture
PROP_TC_DRAM_BYTES = {"cfg2": 197.8e6 + 179.6e6}


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        return main_reference(args, rank, world)
    from vmc_gb300 import afqmc as A
    from vmc_gb300 import synthetic as S
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    sysd = S.workload(args.workload)
    W, N, na, nb, G = sysd["walkers"], sysd["norb"], sysd["nalpha"], sysd["nbeta"], sysd["nchol"]
    A.lib()
    A._bind_cv(A.lib())

    # --- headline: mixed + control variate, energy estimate every step, comb every 50 ---
    wk = make_walkers(A, sysd, "mixed", local)
    tuned, tune_report = A.autotune(wk, tune_cache())
    nchol_ene = cholesky_truncation(wk, G)
    e0 = wk.ham_and_overlap().real.mean()
    wk.set_energy_estimate(e0, e0)
    n_eq, n_skip = (25, 20) if args.profile else (120, 20)
    cv, cv_loss, cv_n = train_cv(A, wk, n_eq=n_eq, n_skip=n_skip, epochs=1 if args.profile else 20)
    k0 = n_eq
    comb = Comb()
    for k in range(k0, k0 + args.warmup):
        wk.propagate_phaseless(None)
        cv.measure(tag=k, slot=k % 4096)
    k0 += args.warmup
    if world > 1:
        dist.barrier()
    clk = Clocks(local)
    ms, launches, stage, live = timed(A, wk, k0, args.steps, "cv", cv, comb)
    clocks = clk.stop()
    if world > 1:
        import torch
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        t = torch.tensor([live], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        live = float(t.item())
    value = live / (ms / 1e3)
    live_fraction = live / (W * args.steps * world)
    k0 += args.steps

    if args.profile:
        print(json.dumps({"profile_run": True, "ms_per_step": ms / args.steps, "launches": launches,
                          "stage_ms_per_step": {k: v / args.steps for k, v in stage.items()}}))
        return
    # the headline estimator against FP64, from the walkers the timed region left
    err = None
    if not args.quick:
        err = energy_check(A, sysd, local, wk, cv, nchol_ene)
        k0 += 100
    # end to end through the public API with host buffers: the step's fields H2D,
    # the weights and the step's energy estimate D2H, every step
    rng = np.random.default_rng(1)
    import torch
    # each step's own fields, drawn beforehand into page-locked host memory
    # (one buffer per step up to 64, then reused in turn): the walkers take
    # the random walk that the device-drawn fields give them
    nbuf = max(1, min(args.steps, 64))
    xis = []
    for _ in range(nbuf):
        t = torch.empty((W, G), dtype=torch.float64, pin_memory=True)
        t.numpy()[:] = rng.standard_normal((W, G))
        xis.append(t)
    from vmc_gb300 import cv as CVM
    ebuf = np.zeros(6)
    wk.sync()
    n0 = wk.walker_steps()
    t0 = time.perf_counter()
    # pipelined as a caller would: step k + 1 is issued (its fields copied on
    # the handle's copy stream while step k runs) before step k's estimate is
    # taken from the result queue
    for k in range(args.steps):
        wk.propagate_phaseless(xis[k % nbuf].numpy())
        if (k + 1) % ORTHO_EVERY == 0:
            wk.orthogonalize()
        cv.measure(tag=k0 + k, slot=k % 2)
        if (k + 1) % REF_CADENCE == 0:
            comb(wk)
        CVM.result_post(wk, k % 2)
        if k > 0:
            CVM.result_take(wk, ebuf)
    CVM.result_take(wk, ebuf)
    wk.sync()
    e2e_s = time.perf_counter() - t0
    e2e_live = wk.walker_steps() - n0
    e2e = {"value": e2e_live * world / e2e_s, "unit": "walker-steps/s",
           "h2d_bytes_per_step": W * G * 8, "d2h_bytes_per_step": 48, "host_fields": "page-locked",
           "result": "each step's control-variate estimate (6 doubles) read back; step k + 1 issued before "
                     "step k's estimate is taken",
           "live_fraction": e2e_live / (W * args.steps)}
    k0 += args.steps

    forms = {}
    if not args.quick:
        # mixed at the reference cadence (exact energy of every walker every 50 steps)
        ms_m50, _, _, live_m50 = timed(A, wk, k0, REF_CADENCE, "every50", comb=comb)
        forms["mixed_every50"] = {"value": live_m50 / (ms_m50 / 1e3), "ms_per_step": ms_m50 / REF_CADENCE,
                                  "live_fraction": live_m50 / (W * REF_CADENCE)}
        k0 += REF_CADENCE
        # the mixed form with the overlap inverse / log-det and the QR in FP64
        A.set_tuning(wk, ovl=2, qr="householder")
        ms_f64, _, st_f64, live_f64 = timed(A, wk, k0, args.steps, "cv", cv, comb)
        forms["mixed_fp64_lu_qr"] = {
            "value": live_f64 / (ms_f64 / 1e3), "ms_per_step": ms_f64 / args.steps,
            "live_fraction": live_f64 / (W * args.steps),
            "precision": "as the headline, with the n x n overlap inverse and log-determinant by FP64 block "
                         "Gauss-Jordan and the walker QR by FP64 Householder",
            "stage_ms_per_step": {s: v / args.steps for s, v in st_f64.items()}}
        wk.close()
        # the plain FP64 form: warm-up 1 step, time 3 steps with an exact energy every step
        wf = make_walkers(A, sysd, "fp64", local)
        wf.set_nchol_ene(nchol_ene)
        ef = wf.ham_and_overlap().real.mean()
        wf.set_energy_estimate(ef, ef)
        wf.propagate_phaseless(None)
        kf = 3
        ms_f, _, stage_f, live_f = timed(A, wf, 1, kf, "every")
        forms["fp64_every_step"] = {"value": live_f / (ms_f / 1e3), "ms_per_step": ms_f / kf,
                                    "live_fraction": live_f / (W * kf),
                                    "stage_ms_per_step": {s: v / kf for s, v in stage_f.items()}}
        step_ms = (ms_f - stage_f["energy"]) / kf
        lf = live_f / (W * kf)
        forms["fp64_every50"] = {"value": W * lf / ((step_ms + stage_f["energy"] / kf / REF_CADENCE) / 1e3),
                                 "ms_per_step": step_ms + stage_f["energy"] / kf / REF_CADENCE}
        wf.close()
        # the other workloads, each on its own line of `forms`
        forms["cfg1"] = {"fp64": form_single(A, S.workload("cfg1"), local, "fp64", 200, "every50"),
                         "mixed": form_single(A, S.workload("cfg1"), local, "mixed", 200, "every50")}
        forms["cfg3"] = form_multisystem(A, local)
        forms["cfg4"] = form_single(A, S.workload("cfg4"), local, "mixed", args.steps, "cv", cv_train=(200, 0))
        forms["cfg5"] = form_large(A, local)
    else:
        wk.close()

    fl = flops_model(N, na, nb, G)
    pk, src = peaks()
    per_launch = {"fb": fl["fb"] * W, "vhs": fl["vhs"] * W, "prop": fl["prop"] * W, "overlap": fl["overlap"] * W,
                  "ortho": fl["ortho"] * ORTHO_EVERY * W, "energy": fl["energy"] * W / 8}
    launches_of = {s: args.steps for s in per_launch}
    launches_of["ortho"] = max(1, args.steps // ORTHO_EVERY)
    peak = pk["bf16_tflops_sustained"] if "bf16_tflops_sustained" in pk else pk["bf16_tflops"]
    # every stage against the pipes that execute it: its bound is the sum over its
    # parts of (algorithmic FLOPs x executed instructions per multiply-add / the
    # pipe's peak) -- tensor cores at the measured bf16 peak, the FP32 CUDA cores
    # at their nominal rate (no measured FP32 peak exists for this GPU pool) --
    # and frac = bound time / measured time
    pipe_peak = {"tensor": peak, "fp32": fp32_nominal_tflops()}
    pipes = mixed_stage_pipes(N, na, nb, G)
    stage_roof = {}
    for s in pipes:
        if launches_of[s] == 0 or stage[s] <= 0:
            continue
        t = stage[s] / launches_of[s]
        parts = {name: {"gflop": f * W / 1e9, "pipe": pp, "cost": c} for name, f, pp, c in pipes[s]}
        bound_ms = sum(f * W * c / (pipe_peak[pp] * 1e12) for _, f, pp, c in pipes[s]) * 1e3
        stage_roof[s] = {"ms_per_launch": t, "parts": parts,
                         "achieved_tflops": sum(f * W for _, f, _, _ in pipes[s]) / (t / 1e3) / 1e12,
                         "bound_ms": bound_ms, "frac": bound_ms / t}
    dom = max(("vhs", "prop"), key=lambda s: stage[s])
    achieved = per_launch[dom] / (stage_roof[dom]["ms_per_launch"] / 1e3) / 1e12
    traffic = PROP_TC_DRAM_BYTES.get(args.workload) if dom == "prop" else None
    roof = {"bound": "tensor", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "traffic": traffic,
            "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum per launch of the tensor-core "
                              "propagator (k_prop_tc2), one ncu capture of this workload (recorded constant)"
                              if traffic else None,
            "peak_source": "%s bf16 sustained (MEASURED_PEAKS.json); algorithmic FLOPs of the stage per launch "
                           "/ its CUDA-event time; the largest tensor-core stage (every stage against the executed "
                           "cost of its parts in stage_roofline; FP32 peak nominal)" % src,
            "stage_roofline": stage_roof}
    out = {"metric": METRIC, "value": value, "unit": "walker-steps/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": DTYPE, "data": "synthetic (seeded generator, vmc_gb300/synthetic.py)",
           "config": {"workload": "%s: norb=%d nalpha=nbeta=%d nchol=%d walkers=%d %s trial and walkers dt=0.005; "
                                  "generator: Cholesky variance sigma_g^2/norb"
                                  % (args.workload, N, na, G, W, sysd["trial"].upper()),
                      "generator": GENERATOR,
                      "form": "mixed + control variate (energy estimate every step: network for every walker, "
                              "exact on 1/8, Horvitz-Thompson correction), comb every %d steps" % REF_CADENCE,
                      "counted": "live walker-steps (weight > 1e-8 when the step begins), device counter",
                      "live_fraction": live_fraction,
                      "ortho_every": ORTHO_EVERY, "fields": "device Philox",
                      "nchol_energy": nchol_ene, "autotune": tuned, "autotune_report": tune_report,
                      "l2": "inputs larger than L2 (walker state + split operands + VHS %.0f MB per step)"
                            % ((W * 40 * 120 * 16 + W * 2 * 14400 * 2 + W * 2 * 7260 * 4) / 1e6),
                      "parallelism": "replicas" if world > 1 else "single GPU",
                      "cv": {"train_samples": cv_n, "train_mse_std_units": cv_loss}},
           "forms": forms,
           "speedup_vs_fp64": (value / forms["fp64_every_step"]["value"]) if forms else None,
           "energy_check": err,
           "energy_error_mEh": err["precision_error_mEh"] if err else None,
           "stage_ms_per_step": {k: v / args.steps for k, v in stage.items()},
           "roofline": roof, "e2e": e2e, "gpu_launches": launches, "clocks": clocks}
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(sysd, nchol_ene)
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        dist.destroy_process_group()


def reference_truncation(sysd, threshold=1e-3):
    """The reference's energy Cholesky truncation (MixedEstimator.cpp:363-384), on the oracle."""
    from oracle import afqmc_oracle as O
    N, na, nb = sysd["norb"], sysd["nalpha"], sysd["nbeta"]
    oh = O.Hamiltonian(N, na, nb, sysd["ecore"], sysd["h1"], sysd["h1mod"], sysd["chol"])
    ot = O.Trial(oh, sysd["trial"], sysd["phi_a"], sysd["phi_b"])
    return O.truncate_cholesky(ot, oh, ot.phi, sysd["trial"] == "rhf", threshold)[0]


def main_reference(args, rank, world):
    """The reference's path on the host cores: the C++ restatement of its walker
    step with all host threads, each step a bounded sample of the workload."""
    if rank != 0:
        return
    from vmc_gb300 import synthetic as S
    sysd = S.workload(args.workload)
    nchol_ene = reference_truncation(sysd)
    cb = cpu_baseline(sysd, nchol_ene)
    N, na, G, W = sysd["norb"], sysd["nalpha"], sysd["nchol"], sysd["walkers"]
    out = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "walker-steps/s",
           "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64 (FP32 VHS as the reference)", "data": "synthetic",
           "config": {"workload": "%s: norb=%d nalpha=nbeta=%d nchol=%d walkers=%d %s trial and walkers dt=0.005; "
                                  "generator: Cholesky variance sigma_g^2/norb"
                                  % (args.workload, N, na, G, W, sysd["trial"].upper()),
                      "generator": GENERATOR,
                      "ortho_every": ORTHO_EVERY, "energy": "exact local energy every step",
                      "nchol_energy": nchol_ene},
           "cpu_baseline": cb,
           "e2e": {"value": cb["value"], "unit": "walker-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "note": "the reference's own C++ (DQMC/*.cpp) needs Boost, HDF5 and MPI, absent here; this arm times "
                   "the C++ restatement of the same path (oracle/cpu_step.cpp) on all host cores, calibrated "
                   "against the reference's published per-core rate at its rhf_rhf size (cpu_baseline.calibration)"}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
