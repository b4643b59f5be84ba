"""Mixed one-body RDM estimator on the GPU against the oracle.

* Direct: walkers with mixed weights (some zero) accumulated twice through the
  C ABI equal the oracle's walker-by-walker running weighted mean
  (DQMC/MixedEstimator.cpp:488-510 with RHF.cpp:64-67 / UHF.cpp:68-72):
  FP64 form <= 1e-12 relative, mixed form (FP32 theta) <= 1e-6; restricted
  walkers with an RHF trial, UHF walkers with a UHF trial, and unrestricted
  integrals (the reference's uhf_uhf_ui fixture), which give up / down blocks.
* A run: afqmc_run with the reference's field order in the FP64 form
  accumulates the measurements after equilibration (step dt > 10) exactly as
  the oracle's run does (<= 1e-9).
* Device blocks: the gate evaluated on the device gives the host loop's RDM.
"""
import numpy as np
import pytest

from oracle import afqmc_oracle as O
from tests import refcases
from vmc_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def A():
    from vmc_gb300 import afqmc
    afqmc.lib()
    return afqmc


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())


def case(kind):
    if kind == "uhf_uhf":
        s = S.make_system(26, 5, 70, 3131, "uhf")
        na, nb, rw, tk = 5, 4, False, "uhf"
    elif kind == "rhf_rhf":
        s = S.make_system(24, 5, 60, 3232, "rhf")
        na, nb, rw, tk = 5, 5, True, "rhf"
    else:
        raise ValueError(kind)
    N = s["norb"]
    oh = O.Hamiltonian(N, na, nb, s["ecore"], s["h1"], s["h1mod"], s["chol"])
    ot = O.Trial(oh, tk, s["phi_a"][:, :na], s["phi_b"][:, :nb])
    return oh, ot, rw


def gpu_handle(A, oh, ot, rw, W, precision, dt=0.005, **kw):
    it = oh.int_type
    if it == "r":
        gh = A.Hamiltonian(oh.norb, oh.nalpha, oh.nbeta, oh.ecore, oh.h1, oh.h1mod, oh.chol)
    else:
        gh = A.Hamiltonian(oh.norb, oh.nalpha, oh.nbeta, oh.ecore, oh.h1s, oh.h1mods, oh.chols, int_type="u")
    gt = A.RHF(gh, ot.phi[0]) if ot.kind == "rhf" else A.UHF(gh, ot.phi[0], ot.phi[1])
    return A.DQMCWalkers(gh, gt, W, rw, dt, precision=precision, **kw)


def walker_set(oh, ot, rw, W, seed):
    rng = np.random.default_rng(seed)
    base = O._ref_dets(oh, ot.phi, rw)
    d = base[None] + 0.2 * (rng.standard_normal((W,) + base.shape) + 1j * rng.standard_normal((W,) + base.shape))
    w = rng.random(W) + 0.5
    w[rng.random(W) < 0.2] = 0.0
    return d, w


@pytest.mark.parametrize("kind,precision", [("uhf_uhf", "fp64"), ("rhf_rhf", "fp64"), ("uhf_uhf", "mixed"),
                                            ("rhf_rhf", "mixed"), ("ui", "fp64")])
def test_rdm_accumulation_matches_oracle(A, kind, precision):
    if kind == "ui":
        c = refcases.load("uhf_uhf_ui")
        oh, ot, rw = c["ham"], c["trial"], c["rhf_walker"]
    else:
        oh, ot, rw = case(kind)
    W = 40
    wk = gpu_handle(A, oh, ot, rw, W, precision)
    wk.rdm_enable(True)
    acc = O.OneRDM(oh.norb, oh.int_type)
    for seed in (1, 2):
        d, w = walker_set(oh, ot, rw, W, seed)
        wk.set_det(d, weights=w)
        wk.rdm_accumulate()
        ow = O.Walkers(oh, rw, d, weights=w)
        acc.add(ot, ow)
    r, cw = wk.rdm()
    wk.close()
    assert r.shape == acc.rdm.shape
    assert abs(cw - acc.cum) <= 1e-12 * acc.cum
    tol = 1e-12 if precision == "fp64" else 1e-6
    assert rel(r, acc.rdm) < tol, rel(r, acc.rdm)


def test_rdm_of_a_run_matches_oracle_run(A):
    """FP64 form, the reference's field order, dt = 0.05 so that measurements
    after step 200 (step dt > 10) count: steps 210 .. 290."""
    oh, ot, rw = case("uhf_uhf")
    W, dt, nsteps, nsweeps = 24, 0.05, 10, 30
    tw_o, te_o, info = O.run(oh, ot, ot.phi, rw, seed=77, nprocs=1, nwalk=W, dt=dt, nsteps=nsteps,
                             nsweeps=nsweeps, ortho_steps=5, cholesky_threshold=1e-3, mode="fp64", one_rdm=True)
    gh = A.Hamiltonian(oh.norb, oh.nalpha, oh.nbeta, oh.ecore, oh.h1, oh.h1mod, oh.chol)
    gt = A.UHF(gh, ot.phi[0], ot.phi[1])
    wk = A.DQMCWalkers(gh, gt, W, rw, dt, precision="fp64", ref=(ot.phi[0], ot.phi[1]), pop_target=W)
    wk.set_det(np.repeat(O._ref_dets(oh, ot.phi, rw)[None], W, axis=0))
    wk.rdm_enable(True)
    tw, te, st = wk.run(nsteps=nsteps, nsweeps=nsweeps, ortho_steps=5, seed=77, nprocs=1,
                        cholesky_threshold=1e-3)
    r, cw = wk.rdm()
    wk.close()
    assert rel(te, te_o) < 1e-10
    assert info["rdm_weight"] > 0 and abs(cw - info["rdm_weight"]) <= 1e-9 * info["rdm_weight"]
    assert rel(r, info["one_rdm"]) < 1e-9, rel(r, info["one_rdm"])
    # the spin-summed 1-RDM of a normalised mixed estimate has trace nalpha + nbeta
    assert abs(np.trace(r[0]) - (oh.nalpha + oh.nbeta)) < 1e-8


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_rdm_device_blocks_equal_host_loop(A, precision):
    """dt = 0.1: the measurements at steps 110, 120, 130 pass the gate (step dt
    > 10), those before do not; on the device the gate reads the step counter."""
    oh, ot, rw = case("uhf_uhf")
    W = 32
    out = []
    for dev in (False, True):
        wk = gpu_handle(A, oh, ot, rw, W, precision, dt=0.1, ref=(ot.phi[0], ot.phi[1]), pop_target=W)
        wk.set_det(np.repeat(O._ref_dets(oh, ot.phi, rw)[None], W, axis=0))
        wk.rdm_enable(True)
        tw, te, _ = wk.run(nsteps=10, nsweeps=14, ortho_steps=5, seed=5, nprocs=1, field_source="device",
                           cholesky_threshold=1e-3, device_blocks=dev)
        out.append((wk.rdm(), tw))
        wk.close()
    ((r0, c0), tw0), ((r1, c1), tw1) = out
    # three measurements of the whole population's weight (the comb keeps it)
    assert c0 > 0 and abs(c0 - tw0[11:14].sum()) <= 1e-9 * c0
    assert abs(c1 - c0) <= 1e-10 * c0
    assert rel(r1, r0) < 1e-10
