"""Device-resident blocks: the comb reconfiguration and the end-of-block
measurement on the device, and whole blocks as graph replays.

* The device comb moves exactly the walkers the reference's comb picks
  (MixedEstimator.cpp:583-621: cumulative weights in walker order,
  z = (w + zeta) / nwalk / P, lower_bound), restated here in numpy.
* A run whose blocks are graph replays with the block end on the device
  reproduces the host-loop run with the same device fields and comb zetas:
  samples.dat columns within 1e-10 relative, the same count of clamped energies.
* One block as a graph replay equals the same launches made one by one, bit
  for bit.
* Host fields from page-locked and from pageable memory give the same steps.
"""
import numpy as np
import pytest

from vmc_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def A():
    from vmc_gb300 import afqmc
    afqmc.lib()
    return afqmc


def make(A, s, W, precision="mixed", seed=7, rw=False):
    n = s["nalpha"]
    gh = A.Hamiltonian(s["norb"], n, n, 0.0, s["h1"], s["h1mod"], s["chol"])
    gt = A.UHF(gh, s["phi_a"], s["phi_b"])
    return A.DQMCWalkers(gh, gt, W, rw, 0.005, precision=precision, seed=seed)


def test_device_comb_matches_reference_rule(A):
    s = S.make_system(24, 4, 60, 77, "uhf")
    W, P = 64, 4
    wk = make(A, s, W)
    rng = np.random.default_rng(0)
    d0, _, _ = wk.get_det()
    d0 = d0 + 0.05 * (rng.standard_normal(d0.shape) + 1j * rng.standard_normal(d0.shape))
    w0 = rng.uniform(0.2, 2.0, W)
    w0[[3, 17, 40]] = 0.0
    wk.set_det(d0, weights=w0)
    d1, o1, _ = wk.get_det()
    for zeta in (0.0, 0.37, 0.999):
        wk.set_det(d1, overlaps=o1, weights=w0)
        wk.comb(zeta, nprocs=P)
        d2, o2, w2 = wk.get_det()
        cum = np.cumsum(w0)
        tot = cum[-1]
        z = (np.arange(W) + zeta) / (W // P) / P
        idx = np.minimum(np.searchsorted(cum, z * tot, side="left"), W - 1)
        assert np.array_equal(d2, d1[idx])
        assert np.array_equal(o2, o1[idx])
        assert np.all(w2 == tot / P / (W // P))


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_device_blocks_reproduce_host_loop(A, precision):
    s = S.make_system(24, 4, 60, 78, "uhf")
    W = 64
    out = []
    for dev in (False, True):
        wk = make(A, s, W, precision)
        tw, te, st = wk.run(nsteps=10, nsweeps=6, ortho_steps=5, seed=11, nprocs=4, field_source="device",
                            cholesky_threshold=1e-3, device_blocks=dev, block_info=True)
        out.append((tw, te, st, wk.get_det()))
    (tw0, te0, st0, g0), (tw1, te1, st1, g1) = out
    assert np.abs(tw1 - tw0).max() <= 1e-10 * np.abs(tw0).max()
    assert np.abs(te1 - te0).max() <= 1e-10 * np.abs(te0).max()
    assert st1["n_large_deviations"] == st0["n_large_deviations"]
    assert np.abs(g1[0] - g0[0]).max() <= 1e-8 * np.abs(g0[0]).max()
    # afqmc.dat's eshift column: read from the device in the host loop,
    # reconstructed from the block ring with device blocks; the same numbers
    assert np.abs(st1["eshift"] - st0["eshift"]).max() <= 1e-9 * np.abs(st0["eshift"]).max()
    assert np.all(np.diff(st0["walltime"]) >= 0) and np.all(np.diff(st1["walltime"]) >= 0)


def test_block_graph_equals_calls(A):
    s = S.make_system(30, 5, 90, 79, "uhf")
    W = 96
    a, b = make(A, s, W, seed=3), make(A, s, W, seed=3)
    e0 = a.ham_and_overlap().real.mean()
    for wk in (a, b):
        wk.set_energy_estimate(e0, e0)
        wk.block_setup(10, e0, zetas=[0.25, 0.5])
    for blk in range(3):
        for k in range(10):
            a.propagate_phaseless(None)
            if (k + 1) % 5 == 0:
                a.orthogonalize()
        a.block_end(comb=True)
    g = A.StepGraph([b], 10, ortho_every=5, block_end="comb")
    for blk in range(3):
        g.launch()
    ra, rb = a.block_results(3), b.block_results(3)
    assert np.array_equal(ra[0], rb[0]) and np.array_equal(ra[1], rb[1]) and ra[2] == rb[2]
    da, oa, wa = a.get_det()
    db, ob, wb = b.get_det()
    assert np.array_equal(da, db) and np.array_equal(oa, ob) and np.array_equal(wa, wb)
    # after the comb every weight is the mean weight
    assert np.allclose(wa, wa[0])
    g.close()


def test_host_fields_pinned_and_pageable_give_the_same_step(A):
    """afqmc_step takes a page-locked field buffer by direct transfer and a
    pageable one through its two staging buffers: the same fields give the
    same walkers bit for bit, over several steps (the staging buffers are
    reused in turn)."""
    torch = pytest.importorskip("torch")
    s = S.make_system(40, 7, 150, 77, "uhf")
    W, G = 64, s["nchol"]
    rng = np.random.default_rng(11)
    fields = [rng.standard_normal((W, G)) for _ in range(3)]
    a = make(A, s, W)
    b = make(A, s, W)
    pinned = torch.empty((W, G), dtype=torch.float64, pin_memory=True)
    for f in fields:
        a.propagate_phaseless(np.array(f))
        pinned.numpy()[:] = f
        b.propagate_phaseless(pinned.numpy())
    da, oa, wa = a.get_det()
    db, ob, wb = b.get_det()
    assert np.array_equal(da, db) and np.array_equal(oa, ob) and np.array_equal(wa, wb)
