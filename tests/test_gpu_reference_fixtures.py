"""The GPU path against the reference's own regression outputs.

``afqmc_run`` (the calcMixedEstimatorLongProp restatement over the C ABI) runs
the reference's DQMC fixtures with 4 emulated ranks, the reference's field
order and its FP32 VHS (precision "ref32").  samples.ref is reproduced to the
printed precision of the energies and weights: the only difference from the
reference's arithmetic is the summation order of FP32 products.
"""
import numpy as np
import pytest

from tests import refcases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def A():
    from vmc_gb300 import afqmc
    afqmc.lib()
    return afqmc


def trials_of(c):
    raw, N = c["raw"], c["ham"].norb
    out = {}
    if "rhf_txt" in raw:
        out["rhf"] = ("rhf", raw["rhf_txt"].reshape(N, N)[:, :c["ham"].nalpha])
    if "uhf_txt" in raw:
        m = raw["uhf_txt"].reshape(N, 2 * N)
        out["uhf"] = ("uhf", m[:, :c["ham"].nalpha], m[:, N:N + c["ham"].nbeta])
    return out


def ham_arrays(c):
    h = c["ham"]
    d = dict(norb=h.norb, nalpha=h.nalpha, nbeta=h.nbeta, ecore=h.ecore)
    if h.int_type == "r":
        d.update(h1=h.h1, h1mod=h.h1mod, chol=h.chol)
    else:
        d.update(h1u=h.h1s, h1umod=h.h1mods, cholu=h.chols)
    return d


@pytest.mark.parametrize("name", refcases.FIXTURES)
def test_samples_ref_on_gpu(A, name):
    c = refcases.load(name)
    s = c["cfg"]["sampling"]
    wk = A.from_reference_inputs(ham_arrays(c), trials_of(c), c["cfg"], nprocs=4, precision="ref32")
    tw, te, st = wk.run(nsteps=int(s["nsteps"]), nsweeps=int(s["stochasticIter"]), ortho_steps=int(s["orthoSteps"]),
                        seed=int(s["seed"]), nprocs=4, cholesky_threshold=float(s["choleskyThreshold"]))
    ref = c["samples"]
    scale_e = 10 ** np.floor(np.log10(np.abs(ref[:, 1]).max()))
    scale_w = 10 ** np.floor(np.log10(ref[:, 0].max()))
    # first block: deterministic (energy at the trial); afterwards FP32 order
    assert abs(te[0] - ref[0, 1]) <= 0.5e-10 * scale_e + 1e-11
    assert np.abs(te - ref[:, 1]).max() <= 2e-9 * scale_e, np.abs(te - ref[:, 1]).max()
    assert np.abs(tw - ref[:, 0]).max() <= 2e-6 * scale_w, np.abs(tw - ref[:, 0]).max()
