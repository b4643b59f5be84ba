"""Convert the reference's DQMC regression fixtures into small .npz files.

Reads, for each hot-path fixture directory of the reference checkout
(tests/DQMC/{rhf_rhf,rhf_uhf,uhf_rhf,uhf_uhf,uhf_uhf_ui}), the integral file
``FCIDUMP_chol`` (HDF5, via vmc_gb300/hdf5.py), the trial files ``rhf.txt`` /
``uhf.txt``, ``afqmc.json`` and the pinned series ``samples.ref`` (weight and
energy of each 50-step block of a 4-rank run, checked by the reference's
tests/testEnergy.py:108-121), and writes ``tests/golden/ref_<name>.npz``.

Usage: python tests/golden/make_reference_fixtures.py [REFERENCE_ROOT]
(default: $VMC_REFERENCE_ROOT, else /root/reference)
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from vmc_gb300.hdf5 import read_fcidump_chol  # noqa: E402

FIXTURES = ["rhf_rhf", "rhf_uhf", "uhf_rhf", "uhf_uhf", "uhf_uhf_ui"]


def convert(ref_root, name):
    d = os.path.join(ref_root, "tests", "DQMC", name)
    cfg = json.load(open(os.path.join(d, "afqmc.json")))
    ints = read_fcidump_chol(os.path.join(d, "FCIDUMP_chol"))
    out = {"afqmc_json": np.array(json.dumps(cfg)),
           "samples_ref": np.loadtxt(os.path.join(d, "samples.ref"))}
    for k in ("nelec", "norb", "ms", "nchol", "nalpha", "nbeta", "ecore"):
        out[k] = np.array(ints[k])
    for k in ("h1", "h1mod", "chol", "h1u", "h1umod", "cholu"):
        if k in ints:
            out[k] = ints[k]  # exactly as stored in the HDF5 datasets
    for t in ("rhf.txt", "uhf.txt"):
        p = os.path.join(d, t)
        if os.path.exists(p):
            out[t.replace(".txt", "_txt")] = np.loadtxt(p)
    path = os.path.join(HERE, "ref_%s.npz" % name)
    np.savez_compressed(path, **out)
    return path


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("VMC_REFERENCE_ROOT", "/root/reference")
    for n in FIXTURES:
        print(convert(root, n))
