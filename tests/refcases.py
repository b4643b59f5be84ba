"""Load the reference's DQMC regression fixtures from tests/golden/ref_<name>.npz.

The npz files are made by tests/golden/make_reference_fixtures.py from the
reference's tests/DQMC/<name>/ directory.  Walker and trial choices follow
executables/DQMC.cpp:74-82, :96-100, :147-153 and the reference-determinant
choice of DQMC/MixedEstimator.cpp:338-350.
"""
import json
import os

import numpy as np

from oracle import afqmc_oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURES = ["rhf_rhf", "rhf_uhf", "uhf_rhf", "uhf_uhf", "uhf_uhf_ui"]


def load(name):
    z = np.load(os.path.join(GOLDEN, "ref_%s.npz" % name))
    cfg = json.loads(str(z["afqmc_json"]))
    it = cfg["system"].get("intType", "r")
    d = {k: z[k] for k in z.files}
    for k in ("nelec", "norb", "ms", "nchol", "nalpha", "nbeta"):
        d[k] = int(d[k])
    d["ecore"] = float(d["ecore"])
    ham = O.Hamiltonian.from_fcidump(d, it)
    N = ham.norb

    def trial(kind):
        if kind == "rhf":
            m = d["rhf_txt"].reshape(N, N)
            return O.Trial(ham, "rhf", m[:, :ham.nalpha])
        m = d["uhf_txt"].reshape(N, 2 * N)
        return O.Trial(ham, "uhf", m[:, :ham.nalpha], m[:, N:N + ham.nbeta])

    left, right = cfg["wavefunction"]["left"], cfg["wavefunction"]["right"]
    rhf_walker = (ham.nalpha == ham.nbeta) and right != "uhf"
    return dict(cfg=cfg, ham=ham, trial=trial(left), ref_phi=trial("rhf" if rhf_walker else "uhf").phi,
                right_phi=trial(right).phi, rhf_walker=rhf_walker, samples=d["samples_ref"],
                int_type=it, raw=d)
