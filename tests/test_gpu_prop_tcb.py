"""Tensor-core propagator for 128 < N <= 512 (streamed tile images of V and
B - I, every row tile's accumulators in TMEM) against the FP64 oracle and the
FP32 column-chunked propagator it replaces.

One step with identical fields: walker determinants and weights within 5e-5
relative of the FP64 oracle and of the FP32 propagator (the same split-BF16
products as the N <= 128 kernel).  Shapes: two row tiles with three and with
four K panels (N = 136, 200), three row tiles (N = 300), four (N = 392); RHF
walkers (one column pass); more columns than one pass holds at four row
tiles (two passes); several walkers per CTA (more walkers than SMs) with dead
walkers among them.
"""
import numpy as np
import pytest

from oracle import afqmc_oracle as O
from vmc_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

SYSTEMS = {
    # name: N, nalpha, nbeta, nchol, seed, trial, rhf walker, walkers
    "n136": (136, 8, 7, 60, 5151, "uhf", False, 12),
    "n200": (200, 12, 12, 80, 5252, "uhf", False, 10),
    "n200_rhf": (200, 10, 10, 70, 5353, "rhf", True, 10),
    "n300": (300, 10, 9, 60, 5454, "uhf", False, 6),
    "n392_wide": (392, 20, 18, 60, 5555, "uhf", False, 4),   # 38 columns: passes of 32 and 6
    "n136_many": (136, 4, 4, 40, 5656, "uhf", False, 400),   # several walkers per CTA, some dead
}


@pytest.fixture(scope="module")
def A():
    from vmc_gb300 import afqmc
    afqmc.lib()
    return afqmc


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())


@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_prop_tcb_one_step(A, name):
    N, na, nb, G, seed, kind, rw, W = SYSTEMS[name]
    s = S.make_system(N, max(na, nb), G, seed, kind)
    oh = O.Hamiltonian(N, na, nb, s["ecore"], s["h1"], s["h1mod"], s["chol"])
    ot = O.Trial(oh, s["trial"], s["phi_a"][:, :na], s["phi_b"][:, :nb])
    rng = np.random.default_rng(seed + 1)
    base = O._ref_dets(oh, ot.phi, rw)
    dets = base[None] + 0.1 * (rng.standard_normal((W,) + base.shape) + 1j * rng.standard_normal((W,) + base.shape))
    w0 = np.ones(W)
    if W > 100:
        w0[::7] = 0.0  # dead walkers are skipped by the persistent CTAs
    xi = rng.standard_normal((W, G))
    e0 = O.hf_energy(ot, oh, ot.phi, rw).real
    out = {}
    for prop in ("tensor", "chunked"):
        gh = A.Hamiltonian(N, na, nb, oh.ecore, oh.h1, oh.h1mod, oh.chol)
        gt = A.RHF(gh, ot.phi[0]) if kind == "rhf" else A.UHF(gh, ot.phi[0], ot.phi[1])
        wk = A.DQMCWalkers(gh, gt, W, rw, 0.005, precision="mixed")
        A.set_tuning(wk, prop=prop)
        wk.set_det(dets, weights=w0)
        wk.propagate_phaseless(xi, e0)
        out[prop] = wk.get_det()
        wk.close()
    live = w0 > 0
    ow = O.Walkers(oh, rw, dets[live].copy(), weights=w0[live].copy())
    ow.overlaps = O.overlap(ot, ow)
    prop_o = O.Propagator(oh, ot.phi, 0.005, mode="fp64")
    O.step(ot, oh, prop_o, ow, xi[live], e0, 1e9)
    d, o, w = out["tensor"]
    dc, oc, wc = out["chunked"]
    errs = dict(dets=rel(d[live], ow.dets), w=rel(w[live], ow.weights),
                dets_vs_fp32=rel(d[live], dc[live]), w_vs_fp32=rel(w[live], wc[live]))
    print(name, errs)
    assert errs["dets"] < 5e-5 and errs["w"] < 5e-5, errs
    assert errs["dets_vs_fp32"] < 5e-5 and errs["w_vs_fp32"] < 5e-5, errs
    # dead walkers are not touched
    assert np.array_equal(d[~live], dets[~live]) and np.all(w[~live] == 0.0)
