"""Learned control variate for the mixed local-energy estimate (no counterpart
in the reference).

During equilibration the walkers' features and the exact local energies of a
random 1/den subsample are collected (``collect``); the MLP is trained on them
on the GPU (``train``); afterwards every measurement predicts all walkers'
energies and corrects their weighted mean with the exact subsample's mean
residual (``afqmc_cv_measure``), so the estimate follows the exact energies
whatever the network predicts.
"""
import numpy as np

from . import afqmc as A


class ControlVariate:
    def __init__(self, walkers, hidden=256, den=8, seed=7):
        self.wk = walkers
        self.den = den
        self.seed = seed
        self.rng = np.random.default_rng(seed)
        self.X, self.Y = [], []
        self.mlp = A.MLP(A.CV_NF, hidden, max_batch=max(4096, walkers.nwalk), seed=seed)

    def stratified(self):
        W, d = self.wk.nwalk, self.den
        starts = np.arange(0, W, d)
        sizes = np.minimum(d, W - starts)
        return starts + (self.rng.random(len(starts)) * sizes).astype(np.int64).clip(max=sizes - 1)

    def collect(self):
        """Features of the current walkers and exact E_L of a subsample (training data)."""
        feats = A.cv_features(self.wk)
        w = self.wk.weights()
        idx = self.stratified()
        idx = idx[w[idx] > 0]
        if len(idx) == 0:
            return
        e = A.local_energy_subset(self.wk, idx).real
        self.X.append(feats[idx])
        self.Y.append(e)

    def train(self, epochs=30, batch=256, lr=1e-3):
        X = np.concatenate(self.X).astype(np.float64)
        Y = np.concatenate(self.Y)
        self.xmean = X.mean(0).astype(np.float32)
        self.xstd = (X.std(0) + 1e-6).astype(np.float32)
        self.ymean = float(Y.mean())
        self.ystd = float(Y.std() + 1e-12)
        Xs = ((X - self.xmean) / self.xstd).astype(np.float32)
        Ys = ((Y - self.ymean) / self.ystd).astype(np.float32)
        loss = self.mlp.train(Xs, Ys, epochs=epochs, batch=min(batch, len(Ys)), lr=lr, seed=self.seed)
        L = A.lib()
        self.wk._check(L.afqmc_cv_attach(self.wk.h, self.mlp.h, self.xmean.ctypes.data, self.xstd.ctypes.data,
                                         self.ymean, self.ystd, self.den))
        return loss, len(Ys)

    def attach(self, walkers):
        """Use the trained network, with its training set's scalings, on another
        handle of the same system (mixed form, nwalk <= the network's batch)."""
        L = A.lib()
        walkers._check(L.afqmc_cv_attach(walkers.h, self.mlp.h, self.xmean.ctypes.data, self.xstd.ctypes.data,
                                         self.ymean, self.ystd, self.den))

    def measure(self, tag, slot):
        self.wk._check(A.lib().afqmc_cv_measure(self.wk.h, int(tag), int(slot)))

    def results(self, nslots):
        """(nslots, 6): E_cv, E_cv (HT), E_sub (HT), E_sub (ratio), sum_w, sum_w (subsample)."""
        return results(self.wk, nslots)


def measure(walkers, tag, slot):
    """Control-variate measurement on a handle the network is attached to."""
    walkers._check(A.lib().afqmc_cv_measure(walkers.h, int(tag), int(slot)))


def result_post(walkers, slot):
    """Enqueue an asynchronous read of result slot `slot` (first in first out, at most 8)."""
    walkers._check(A.lib().afqmc_cv_result_post(walkers.h, int(slot)))


def result_take(walkers, out=None):
    """The oldest posted result (6 values), waiting for its copy only."""
    out = np.zeros(6) if out is None else out
    walkers._check(A.lib().afqmc_cv_result_take(walkers.h, out.ctypes.data))
    return out


def results(walkers, nslots):
    """(nslots, 6) control-variate results of a handle: E_cv (ratio correction),
    E_cv (Horvitz-Thompson correction, exactly unbiased), E_sub (HT), E_sub
    (ratio), sum of weights, sum of subsample weights."""
    out = np.zeros((nslots, 6))
    walkers._check(A.lib().afqmc_cv_results(walkers.h, out.ctypes.data, int(nslots)))
    return out
