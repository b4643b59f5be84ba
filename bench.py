#!/usr/bin/env python3
"""Walker-steps/s of the phaseless AFQMC step on one GB300 (one JSON line).

Workload (default): norb=120, nalpha=nbeta=20, nchol=600 synthetic Hamiltonian,
UHF trial and UHF walkers, 2048 walkers, dt=0.005; one step = force bias,
fields, VHS, propagator, overlap and weights of every walker; walkers are
orthonormalised every 5 steps and measured (local energy of every walker)
every 50 steps, the reference's measurement cadence (sampling.nsteps = 50).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--form fp64|mixed] [--impl reference]

--impl reference times the CPU restatement of the reference's path (the oracle
port; the reference's own C++ needs Boost, HDF5 and MPI, which are absent) on
all host cores on the same workload.  Under torchrun every rank runs an
independent replica (the path has no data-path collective at this scale);
rank 0 prints the line with value = walker-steps of all ranks / max time.
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
ENERGY_EVERY = 50


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=50)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--form", default="fp64", choices=["fp64", "mixed"])
    p.add_argument("--workload", default="cfg2")
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# --------------------------------------------------------------------------
# algorithmic FLOPs (count of the algorithm, not of what a kernel executes)
# --------------------------------------------------------------------------
def flops_model(N, na, nb, G, spins=2, ortho_every=ORTHO_EVERY):
    """Per walker: force bias (theta + contraction), VHS, propagator with a real
    exp(-dt/2 h1') (2 real x complex + 5 complex x complex products per spin),
    overlap (Phi^T psi and LU), QR amortised, and one exact local energy."""
    T = N * (N + 1) // 2
    ns = [na, nb][:spins]
    fb = sum(4 * n * n * N + 16 * n ** 3 + 8 * N * n * n + 4 * n * N * G for n in ns)
    vhs = 4 * T * G
    prop = sum(48 * N * N * n for n in ns)
    ovl = sum(4 * n * n * N + 5.3 * n ** 3 for n in ns)
    qr = sum(32 * N * n * n for n in ns) / ortho_every
    el = sum(4 * G * n * n * N + 8 * G * n * n + 4 * n * N for n in ns)
    return dict(fb=fb, vhs=vhs, prop=prop, overlap=ovl, ortho=qr, energy=el,
                step=fb + vhs + prop + ovl + qr)


# --------------------------------------------------------------------------
# clocks sampled during the timed region
# --------------------------------------------------------------------------
class Clocks:
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
        d = json.load(open(p))
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


# --------------------------------------------------------------------------
# CPU baseline: the oracle port on the host cores
# --------------------------------------------------------------------------
def cpu_baseline(sysd, nwalk_sample=32, steps=4, seconds_cap=30.0):
    from oracle import afqmc_oracle as O
    N, na, nb = sysd["norb"], sysd["nalpha"], sysd["nbeta"]
    oh = O.Hamiltonian(N, na, nb, sysd["ecore"], sysd["h1"], sysd["h1mod"], sysd["chol"])
    ot = O.Trial(oh, sysd["trial"], sysd["phi_a"], sysd["phi_b"])
    rw = False
    prop = O.Propagator(oh, ot.phi, 0.005, mode="ref")
    wk = O.Walkers(oh, rw, np.repeat(O._ref_dets(oh, ot.phi, rw)[None], nwalk_sample, axis=0))
    wk.overlaps = O.overlap(ot, wk)
    rng = np.random.default_rng(0)
    e0 = O.hf_energy(ot, oh, ot.phi, rw).real
    t0 = time.perf_counter()
    done = 0
    for st in range(1, steps + 1):
        O.step(ot, oh, prop, wk, rng.standard_normal((nwalk_sample, oh.nchol)), e0, 100.0)
        if st % ORTHO_EVERY == 0:
            O.orthogonalize(wk)
        done += nwalk_sample
        if time.perf_counter() - t0 > seconds_cap:
            break
    # one local-energy evaluation per ENERGY_EVERY steps, timed on a small sample
    te = time.perf_counter()
    O.local_energy(ot, wk, oh)
    t_el = (time.perf_counter() - te) / nwalk_sample
    dt = time.perf_counter() - t0 - t_el * nwalk_sample
    per_ws = dt / done + t_el / ENERGY_EVERY
    return {"value": 1.0 / per_ws, "unit": "walker-steps/s", "cores": os.cpu_count(), "kind": "port",
            "sample": "%d walkers x %d steps of the same workload (oracle, numpy complex128 + FP32 VHS, "
                      "all BLAS threads) + one local energy per %d steps" % (nwalk_sample, done // nwalk_sample,
                                                                             ENERGY_EVERY)}


# --------------------------------------------------------------------------
def make_walkers(sysd, form, device):
    from vmc_gb300 import afqmc as A
    N, na, nb = sysd["norb"], sysd["nalpha"], sysd["nbeta"]
    gh = A.Hamiltonian(N, na, nb, sysd["ecore"], sysd["h1"], sysd["h1mod"], sysd["chol"])
    gt = A.UHF(gh, sysd["phi_a"], sysd["phi_b"]) if sysd["trial"] == "uhf" else A.RHF(gh, sysd["phi_a"])
    wk = A.DQMCWalkers(gh, gt, sysd["walkers"], sysd["trial"] == "rhf", 0.005, precision=form,
                       device=device, seed=20261203)
    return wk


def run_steps(wk, k0, K, e_every=ENERGY_EVERY):
    for k in range(k0, k0 + K):
        wk.propagate_phaseless(None)
        if (k + 1) % ORTHO_EVERY == 0:
            wk.orthogonalize()
        if (k + 1) % e_every == 0:
            wk.lib_energy()


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        return main_reference(args, rank, world)
    from vmc_gb300 import synthetic as S
    from vmc_gb300 import afqmc as A
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    sysd = S.workload(args.workload)
    W = sysd["walkers"]
    N, na, nb, G = sysd["norb"], sysd["nalpha"], sysd["nbeta"], sysd["nchol"]
    wk = make_walkers(sysd, args.form, local)
    e0 = wk.ham_and_overlap().real.mean()
    wk.set_energy_estimate(e0, e0)
    A.DQMCWalkers.lib_energy = lambda self: A.lib().afqmc_local_energy(self.h, None)

    # warm-up
    run_steps(wk, 0, args.warmup)
    wk.sync()
    # timed region (device events on the handle's stream)
    if world > 1:
        dist.barrier()
    wk.sync()
    clk = Clocks(local)
    wk.enable_timing(True)
    l0 = wk.launch_count()
    wk.timer_start()
    run_steps(wk, args.warmup, args.steps)
    ms = wk.timer_stop()
    launches = wk.launch_count() - l0
    clocks = clk.stop()
    stage = {s: wk.stage_time(s) for s in ["fb", "fields", "vhs", "prop", "overlap", "weights", "ortho", "energy"]}
    wk.enable_timing(False)
    if world > 1:
        import torch
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    walker_steps = W * args.steps * world
    value = walker_steps / (ms / 1e3)

    # end to end through the public API with host buffers: H2D fields, D2H weights
    rng = np.random.default_rng(1)
    xis = [np.ascontiguousarray(rng.standard_normal((W, G))) for _ in range(2)]
    import ctypes
    wbuf = np.zeros(W)
    wk.sync()
    t0 = time.perf_counter()
    for k in range(args.steps):
        wk.propagate_phaseless(xis[k % 2])
        if (k + 1) % ORTHO_EVERY == 0:
            wk.orthogonalize()
        if (k + 1) % ENERGY_EVERY == 0:
            wk.lib_energy()
        A.lib().afqmc_get_walkers(wk.h, None, None, wbuf.ctypes.data)
    wk.sync()
    e2e_s = time.perf_counter() - t0
    e2e = {"value": W * args.steps * world / e2e_s, "unit": "walker-steps/s",
           "h2d_bytes_per_step": W * G * 8, "d2h_bytes_per_step": W * 8}

    fl = flops_model(N, na, nb, G)
    pk, src = peaks()
    nsteps_e = args.steps // ENERGY_EVERY
    per_launch = {"fb": fl["fb"] * W, "vhs": fl["vhs"] * W, "prop": fl["prop"] * W,
                  "overlap": fl["overlap"] * W, "energy": fl["energy"] * W}
    launches_of = {"fb": args.steps, "vhs": args.steps, "prop": args.steps, "overlap": args.steps,
                   "energy": max(nsteps_e, 1)}
    dom = max(per_launch, key=lambda s: stage[s] if launches_of[s] else 0)
    avg_ms = stage[dom] / launches_of[dom]
    achieved = per_launch[dom] / (avg_ms / 1e3) / 1e12
    if args.form == "fp64":
        roof = {"bound": "tensor", "kernel": dom, "achieved": achieved, "peak": pk["bf16_tflops"],
                "unit": "TFLOP/s", "frac": achieved / pk["bf16_tflops"], "traffic": None,
                "peak_source": src + " bf16 burst; the FP64 form runs on the FP64 pipe"}
    else:
        roof = {"bound": "tensor", "kernel": dom, "achieved": achieved, "peak": pk["bf16_tflops"],
                "unit": "TFLOP/s", "frac": achieved / pk["bf16_tflops"], "traffic": None,
                "peak_source": src + " bf16 burst"}

    out = {"metric": METRIC, "value": value, "unit": "walker-steps/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64" if args.form == "fp64" else "bf16x3/f32/f64",
           "data": "synthetic (seeded generator, vmc_gb300/synthetic.py)",
           "config": {"workload": "%s: norb=%d nalpha=nbeta=%d nchol=%d walkers=%d UHF trial+walkers dt=0.005"
                                  % (args.workload, N, na, G, W),
                      "form": args.form, "ortho_every": ORTHO_EVERY, "energy_every": ENERGY_EVERY,
                      "fields": "device Philox", "l2": "inputs larger than L2 (VHS matrices %.0f MB)" %
                                                      (W * 2 * 2 * N * N * 8 / 1e6 if args.form == "fp64" else 0),
                      "parallelism": "replicas" if world > 1 else "single GPU"},
           "stage_ms_per_step": {k: v / max(launches_of.get(k, args.steps), 1) for k, v in stage.items()},
           "roofline": roof, "e2e": e2e, "gpu_launches": launches, "clocks": clocks}
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(sysd)
    if rank == 0:
        print(json.dumps(out))
    wk.close()
    if world > 1:
        dist.destroy_process_group()


def main_reference(args, rank, world):
    if rank != 0:
        return
    from vmc_gb300 import synthetic as S
    sysd = S.workload(args.workload)
    cb = cpu_baseline(sysd, nwalk_sample=32, steps=max(2, min(args.steps, 6)))
    N, na, G, W = sysd["norb"], sysd["nalpha"], sysd["nchol"], sysd["walkers"]
    out = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "walker-steps/s",
           "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": "%s: norb=%d nalpha=nbeta=%d nchol=%d walkers=%d UHF trial+walkers dt=0.005"
                                  % (args.workload, N, na, G, W),
                      "ortho_every": ORTHO_EVERY, "energy_every": ENERGY_EVERY},
           "cpu_baseline": cb,
           "e2e": {"value": cb["value"], "unit": "walker-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "note": "the reference's own C++ (DQMC/*.cpp) needs Boost, HDF5 and MPI, absent here; "
                   "this arm times the oracle port of the same path on all host cores"}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
