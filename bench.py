#!/usr/bin/env python3
"""Walker-steps/s of the phaseless AFQMC step on one GB300 (one JSON line).

Workload (default): norb=120, nalpha=nbeta=20, nchol=600 synthetic Hamiltonian
(vmc_gb300/synthetic.py), UHF trial and UHF walkers, 2048 walkers, dt=0.005.
One step = force bias, fields, VHS, propagator, overlap and weights of every
walker, the walkers orthonormalised every 5 steps, and an energy estimate.

Forms, all on the same GPU and workload:
  headline ("value"): mixed precision + control variate, an energy estimate
      every step (MLP for every walker + exact local energy of 1 walker in 8);
  fp64_every_step: the plain FP64 form, exact local energy of every walker every
      step (the metric's comparison);
  mixed_every50 / fp64_every50: both forms at the reference's own measurement
      cadence (every sampling.nsteps = 50 steps, exact energies).
energy_error_mEh: |mixed-estimator energy of the mixed form - that of the FP64
form| after 40 steps from the same walkers with identical fields (the FP64 form
equals the FP64 oracle to 1e-10).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the CPU restatement of the reference's path (the
oracle port: the reference's own C++ needs Boost, HDF5 and MPI, absent here)
on all host cores, same workload and metric.  Under torchrun every rank runs
an independent replica; rank 0 prints value = walker-steps of all ranks / max
time.
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


def cpu_baseline(sysd, nwalk_sample=32, steps=4, seconds_cap=30.0, nchol_ene=None):
    """The oracle port (numpy complex128 + the reference's FP32 VHS) on the host cores;
    local energies with the same Cholesky truncation as the GPU run."""
    from oracle import afqmc_oracle as O
    N, na, nb = sysd["norb"], sysd["nalpha"], sysd["nbeta"]
    oh = O.Hamiltonian(N, na, nb, sysd["ecore"], sysd["h1"], sysd["h1mod"], sysd["chol"])
    ot = O.Trial(oh, sysd["trial"], sysd["phi_a"], sysd["phi_b"])
    prop = O.Propagator(oh, ot.phi, 0.005, mode="ref")
    wk = O.Walkers(oh, False, np.repeat(O._ref_dets(oh, ot.phi, False)[None], nwalk_sample, axis=0))
    wk.overlaps = O.overlap(ot, wk)
    rng = np.random.default_rng(0)
    e0 = O.hf_energy(ot, oh, ot.phi, False).real
    t0 = time.perf_counter()
    done = 0
    for st in range(1, steps + 1):
        O.step(ot, oh, prop, wk, rng.standard_normal((nwalk_sample, oh.nchol)), e0, 100.0)
        if st % ORTHO_EVERY == 0:
            O.orthogonalize(wk)
        done += nwalk_sample
        if time.perf_counter() - t0 > seconds_cap:
            break
    t_step = (time.perf_counter() - t0) / done
    te = time.perf_counter()
    O.local_energy(ot, wk, oh, nchol_ene)
    t_el = (time.perf_counter() - te) / nwalk_sample
    per_ws = t_step + t_el  # energy every step, as the headline form
    return {"value": 1.0 / per_ws, "unit": "walker-steps/s", "cores": os.cpu_count(), "kind": "port",
            "sample": "%d walkers x %d steps of the same workload + one exact local energy per walker-step "
                      "(oracle port: numpy complex128 with the reference's FP32 VHS, all BLAS threads)"
                      % (nwalk_sample, done // nwalk_sample),
            "every50_value": 1.0 / (t_step + t_el / REF_CADENCE)}


def make_walkers(A, sysd, form, device, nwalk=None):
    N, na, nb = sysd["norb"], sysd["nalpha"], sysd["nbeta"]
    gh = A.Hamiltonian(N, na, nb, sysd["ecore"], sysd["h1"], sysd["h1mod"], sysd["chol"])
    gt = A.UHF(gh, sysd["phi_a"], sysd["phi_b"]) if sysd["trial"] == "uhf" else A.RHF(gh, sysd["phi_a"])
    return A.DQMCWalkers(gh, gt, nwalk or sysd["walkers"], sysd["trial"] == "rhf", 0.005, precision=form,
                         device=device, seed=20261203)


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


def timed(A, wk, k0, K, energy, cv=None):
    """K steps on the device; energy in {"cv", "every", "every50"}; returns (ms, launches, stage ms)."""
    wk.sync()
    wk.enable_timing(True)
    l0 = wk.launch_count()
    wk.timer_start()
    for k in range(k0, k0 + K):
        wk.propagate_phaseless(None)
        if (k + 1) % ORTHO_EVERY == 0:
            wk.orthogonalize()
        if energy == "cv":
            cv.measure(tag=k, slot=k % 4096)
        elif energy == "every" or (k + 1) % REF_CADENCE == 0:
            energy_all(A, wk)
    ms = wk.timer_stop()
    launches = wk.launch_count() - l0
    stage = {s: wk.stage_time(s) for s in STAGES}
    wk.enable_timing(False)
    return ms, launches, stage


def energy_error(A, sysd, device, tuned, nw=256, steps=40):
    """Mixed vs FP64 form from the same walkers with identical host fields; the
    mixed form runs the kernel variants the timed run uses (`tuned`)."""
    rng = np.random.default_rng(11)
    xs = [rng.standard_normal((nw, sysd["nchol"])) for _ in range(steps)]
    out = {}
    for form in ("mixed", "fp64"):
        wk = make_walkers(A, sysd, form, device, nw)
        if form == "mixed":
            A.set_tuning(wk, **tuned)
        e0 = wk.ham_and_overlap().real.mean()
        for k in range(steps):
            wk.propagate_phaseless(xs[k], e0)
            if (k + 1) % ORTHO_EVERY == 0:
                wk.orthogonalize()
        _, _, w = wk.get_det()
        el = wk.ham_and_overlap().real
        out[form] = (w * el).sum() / w.sum()
        wk.close()
    return abs(out["mixed"] - out["fp64"]) * 1e3, out


def main_multisystem(args, local):
    """Uneven multi-system batch: 16 synthetic systems, norb ~ U[40, 200],
    nocc = round(norb / 6), nchol = 5 norb, 256 walkers each, mixed form,
    each system autotuned for its size class, all advanced by one CUDA graph
    (10 steps + QR every 5 per replay)."""
    from vmc_gb300 import afqmc as A
    from vmc_gb300 import synthetic as S
    systems = S.multi_system_batch()
    cache = os.environ.get("AFQMC_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "vmc_gb300",
                                                            "autotune.txt"))
    os.makedirs(os.path.dirname(cache), exist_ok=True)
    hs, flops = [], 0.0
    for sd in systems:
        n = sd["nalpha"]
        gh = A.Hamiltonian(sd["norb"], n, n, sd["ecore"], sd["h1"], sd["h1mod"], sd["chol"])
        gt = A.UHF(gh, sd["phi_a"], sd["phi_b"])
        wk = A.DQMCWalkers(gh, gt, sd["walkers"], False, 0.005, precision="mixed", device=local, seed=7 + len(hs))
        A.autotune(wk, cache)
        e0 = wk.ham_and_overlap().real.mean()
        wk.set_energy_estimate(e0, e0)
        hs.append(wk)
        flops += flops_model(sd["norb"], n, n, sd["nchol"])["step"] * sd["walkers"]
    g = A.StepGraph(hs, 10, ortho_every=5)
    for _ in range(max(1, args.warmup // 10 + 1)):
        g.launch()
    reps = max(1, args.steps // 10)
    for h in hs:
        h.sync()
    t0 = time.perf_counter()
    hs[0].timer_start()
    for _ in range(reps):
        g.launch()
    ms = hs[0].timer_stop()
    for h in hs:
        h.sync()
    wall = time.perf_counter() - t0
    W = sum(sd["walkers"] for sd in systems)
    out = {"metric": METRIC, "value": W * 10 * reps / (ms / 1e3), "unit": "walker-steps/s", "n_gpus": 1,
           "steps": 10 * reps, "warmup": args.warmup, "ms_per_step": ms / (10 * reps), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "bf16x3 / f32 / f64", "data": "synthetic",
           "config": {"workload": "cfg3: 16 systems, norb %s, 256 walkers each, UHF, mixed form, one CUDA graph"
                                  % sorted(sd["norb"] for sd in systems),
                      "graph_nodes": g.nodes(), "ortho_every": 5, "energy": "none in the timed region"},
           "achieved_tflops_algorithmic": flops * 10 * reps / (ms / 1e3) / 1e12, "wall_s": wall}
    print(json.dumps(out))


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        return main_reference(args, rank, world)
    if args.workload == "cfg3":
        return main_multisystem(args, local)
    from vmc_gb300 import afqmc as A
    from vmc_gb300 import synthetic as S
    from vmc_gb300.cv import ControlVariate
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    sysd = S.workload(args.workload)
    W, N, na, nb, G = sysd["walkers"], sysd["norb"], sysd["nalpha"], sysd["nbeta"], sysd["nchol"]
    A.lib()
    A._bind_cv(A.lib())

    # --- headline: mixed + control variate, energy estimate every step ---
    wk = make_walkers(A, sysd, "mixed", local)
    cache = os.environ.get("AFQMC_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "vmc_gb300",
                                                            "autotune.txt"))
    os.makedirs(os.path.dirname(cache), exist_ok=True)
    tuned, tune_report = A.autotune(wk, cache)
    nchol_ene = cholesky_truncation(wk, G)
    e0 = wk.ham_and_overlap().real.mean()
    wk.set_energy_estimate(e0, e0)
    cv = ControlVariate(wk, hidden=256, den=8, seed=3)
    n_eq, n_skip = (25, 20) if args.profile else (120, 20)
    for k in range(n_eq):  # equilibration; training data from steps 20.. (untimed)
        wk.propagate_phaseless(None)
        if (k + 1) % ORTHO_EVERY == 0:
            wk.orthogonalize()
        if k >= n_skip:
            cv.collect()
    cv_loss, cv_n = cv.train(epochs=1 if args.profile else 20, batch=512, lr=1e-3)
    k0 = n_eq
    for k in range(k0, k0 + args.warmup):
        wk.propagate_phaseless(None)
        cv.measure(tag=k, slot=k % 4096)
    k0 += args.warmup
    if world > 1:
        dist.barrier()
    clk = Clocks(local)
    ms, launches, stage = timed(A, wk, k0, args.steps, "cv", cv)
    clocks = clk.stop()
    if world > 1:
        import torch
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = W * args.steps * world / (ms / 1e3)
    k0 += args.steps

    if args.profile:
        print(json.dumps({"profile_run": True, "ms_per_step": ms / args.steps, "launches": launches,
                          "stage_ms_per_step": {k: v / args.steps for k, v in stage.items()}}))
        return
    # end to end through the public API with host buffers: fields H2D, weights and the
    # step's energy estimate D2H every step
    rng = np.random.default_rng(1)
    import torch
    xis = []
    for _ in range(2):  # the step's fields in page-locked host memory
        t = torch.empty((W, G), dtype=torch.float64, pin_memory=True)
        t.numpy()[:] = rng.standard_normal((W, G))
        xis.append(t.numpy())
    wbuf = np.zeros(W)
    ebuf = np.zeros(4)
    wk.sync()
    t0 = time.perf_counter()
    for k in range(args.steps):
        wk.propagate_phaseless(xis[k % 2])
        if (k + 1) % ORTHO_EVERY == 0:
            wk.orthogonalize()
        cv.measure(tag=k0 + k, slot=0)
        A.lib().afqmc_get_walkers(wk.h, None, None, wbuf.ctypes.data)
        A.lib().afqmc_cv_results(wk.h, ebuf.ctypes.data, 1)
    wk.sync()
    e2e_s = time.perf_counter() - t0
    e2e = {"value": W * args.steps * world / e2e_s, "unit": "walker-steps/s",
           "h2d_bytes_per_step": W * G * 8, "d2h_bytes_per_step": W * 8 + 32, "host_fields": "page-locked"}

    forms = {}
    if not args.quick:
        # mixed at the reference cadence (energy every 50 steps)
        ms_m50, _, _ = timed(A, wk, k0, REF_CADENCE, "every50")
        forms["mixed_every50"] = {"value": W * REF_CADENCE / (ms_m50 / 1e3), "ms_per_step": ms_m50 / REF_CADENCE}
        wk.close()
        # the plain FP64 form: warm-up 1 step, time 3 steps with an exact energy every step
        wf = make_walkers(A, sysd, "fp64", local)
        wf.set_nchol_ene(nchol_ene)
        ef = wf.ham_and_overlap().real.mean()
        wf.set_energy_estimate(ef, ef)
        wf.propagate_phaseless(None)
        kf = 3
        ms_f, _, stage_f = timed(A, wf, 1, kf, "every")
        forms["fp64_every_step"] = {"value": W * kf / (ms_f / 1e3), "ms_per_step": ms_f / kf,
                                    "stage_ms_per_step": {s: v / kf for s, v in stage_f.items()}}
        step_ms = (ms_f - stage_f["energy"]) / kf
        forms["fp64_every50"] = {"value": W / ((step_ms + stage_f["energy"] / kf / REF_CADENCE) / 1e3),
                                 "ms_per_step": step_ms + stage_f["energy"] / kf / REF_CADENCE}
        wf.close()
        err_meh, err_e = energy_error(A, sysd, local, tuned)
    else:
        wk.close()
        err_meh, err_e = None, None

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
    # DRAM bytes per launch of the dominant kernel from one ncu capture of this workload
    # (dram__bytes_read.sum + dram__bytes_write.sum; profiles/k_prop_tc_cfg2.md)
    traffic = {"prop": 198.0e6 + 179.0e6}.get(dom) if args.workload == "cfg2" else None
    roof = {"bound": "tensor", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "traffic": traffic, "traffic_unit": "bytes per launch (ncu capture)",
            "peak_source": "%s bf16 sustained (MEASURED_PEAKS.json); algorithmic FLOPs of the stage per launch "
                           "/ its CUDA-event time; the largest tensor-core stage (every stage against the executed "
                           "cost of its parts in stage_roofline; FP32 peak nominal)"
                           % src,
            "stage_roofline": stage_roof}
    out = {"metric": METRIC, "value": value, "unit": "walker-steps/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "bf16x3 contractions / f32 propagator / f64 inverse, det, QR, weights",
           "data": "synthetic (seeded generator, vmc_gb300/synthetic.py)",
           "config": {"workload": "%s: norb=%d nalpha=nbeta=%d nchol=%d walkers=%d UHF trial and walkers dt=0.005"
                                  % (args.workload, N, na, G, W),
                      "form": "mixed + control variate (energy estimate every step, exact on 1/8)",
                      "ortho_every": ORTHO_EVERY, "fields": "device Philox",
                      "nchol_energy": nchol_ene, "autotune": tuned, "autotune_report": tune_report,
                      "l2": "inputs larger than L2 (walker state + split operands + VHS %.0f MB per step)"
                            % ((W * 40 * 120 * 16 + W * 2 * 14400 * 2 + W * 2 * 7260 * 4) / 1e6),
                      "parallelism": "replicas" if world > 1 else "single GPU",
                      "cv": {"train_samples": cv_n, "train_mse_std_units": cv_loss}},
           "forms": forms,
           "speedup_vs_fp64": (value / forms["fp64_every_step"]["value"]) if forms else None,
           "energy_error_mEh": err_meh, "energy_check": err_e,
           "stage_ms_per_step": {k: v / args.steps for k, v in stage.items()},
           "roofline": roof, "e2e": e2e, "gpu_launches": launches, "clocks": clocks}
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(sysd, nchol_ene=nchol_ene)
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
    if rank != 0:
        return
    from vmc_gb300 import synthetic as S
    sysd = S.workload(args.workload)
    cb = cpu_baseline(sysd, nwalk_sample=32, steps=max(2, min(args.steps, 6)), nchol_ene=reference_truncation(sysd))
    N, na, G, W = sysd["norb"], sysd["nalpha"], sysd["nchol"], sysd["walkers"]
    out = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "walker-steps/s",
           "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64 (FP32 VHS as the reference)", "data": "synthetic",
           "config": {"workload": "%s: norb=%d nalpha=nbeta=%d nchol=%d walkers=%d UHF trial and walkers dt=0.005"
                                  % (args.workload, N, na, G, W),
                      "ortho_every": ORTHO_EVERY, "energy": "exact local energy every step"},
           "cpu_baseline": cb,
           "e2e": {"value": cb["value"], "unit": "walker-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "note": "the reference's own C++ (DQMC/*.cpp) needs Boost, HDF5 and MPI, absent here; this arm times "
                   "the oracle port of the same path on all host cores"}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
