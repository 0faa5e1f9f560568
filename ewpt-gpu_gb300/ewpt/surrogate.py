"""Learned surrogate for parameter sweeps.

A 3-layer BF16 MLP (width 256, GELU, FP32 accumulate; ewpt_mlp_* in
include/ewpt.h, trained on the GPU by the library's own tensor-core forward
and backward kernels and AdamW) maps the early-time spectra of a run (B and
Higgs, `nshell` log shells each) plus its parameters (lambda, g, g', bubble
count) to the late-time log B spectrum.  Training data come from the
library's batched ensemble engine (seeded uniform parameter draws, device
bubble or thermal ICs); the plain evolution is the fallback and the yardstick of
the surrogate's error, and the surrogate never replaces the evolution path.
"""
from __future__ import annotations

import ctypes as C
import math
import time

import numpy as np

from . import _lib, ic
from .ensemble import Ensemble
from .params import baseline_couplings

FP = C.POINTER(C.c_float)


def _fp(a: np.ndarray):
    return a.ctypes.data_as(FP)


class MLP:
    """ctypes handle of one ewpt_mlp (n_in -> width -> width -> n_out)."""

    def __init__(self, n_in: int, width: int, n_out: int, max_batch: int, device: int = 0, seed: int = 0):
        self.L = _lib.load()
        self.n_in, self.width, self.n_out, self.max_batch = n_in, width, n_out, max_batch
        h = C.c_void_p()
        _lib.check(self.L.ewpt_mlp_create(n_in, width, n_out, max_batch, device, C.byref(h)))
        self.h = h
        self.set_params(self.init_params(seed))

    def _chk(self, rc):
        if rc != _lib.OK:
            raise _lib.EwptError(rc, self.L.ewpt_mlp_last_error(self.h).decode())

    def close(self):
        if self.h:
            self.L.ewpt_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_wait_limit(self, polls: int):
        """Limit of the GEMM's tensor-core waits in polls (< 0: default)."""
        self._chk(self.L.ewpt_mlp_set_wait_limit(self.h, int(polls)))

    @property
    def num_params(self) -> int:
        return int(self.L.ewpt_mlp_num_params(self.h))

    def init_params(self, seed: int = 0) -> np.ndarray:
        """Uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights and biases."""
        rng = np.random.default_rng(seed)
        parts = []
        for fan_in, shape in [(self.n_in, (self.width, self.n_in)), (self.n_in, (self.width,)),
                              (self.width, (self.width, self.width)), (self.width, (self.width,)),
                              (self.width, (self.n_out, self.width)), (self.width, (self.n_out,))]:
            b = 1.0 / math.sqrt(fan_in)
            parts.append(rng.uniform(-b, b, size=shape).ravel())
        return np.concatenate(parts).astype(np.float32)

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.num_params
        self._chk(self.L.ewpt_mlp_set_params(self.h, _fp(p)))

    def get_params(self) -> np.ndarray:
        p = np.empty(self.num_params, dtype=np.float32)
        self._chk(self.L.ewpt_mlp_get_params(self.h, _fp(p)))
        return p

    def forward(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32)
        out = np.empty((x.shape[0], self.n_out), dtype=np.float32)
        for s in range(0, x.shape[0], self.max_batch):
            xb = np.ascontiguousarray(x[s:s + self.max_batch])
            yb = np.empty((xb.shape[0], self.n_out), dtype=np.float32)
            self._chk(self.L.ewpt_mlp_forward(self.h, _fp(xb), xb.shape[0], _fp(yb)))
            out[s:s + self.max_batch] = yb
        return out

    def gradients(self, x: np.ndarray, y: np.ndarray):
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        g = np.empty(self.num_params, dtype=np.float32)
        loss = C.c_float()
        self._chk(self.L.ewpt_mlp_gradients(self.h, _fp(x), _fp(y), x.shape[0], _fp(g), C.byref(loss)))
        return g, float(loss.value)

    def train_step(self, x: np.ndarray, y: np.ndarray, lr: float, wd: float = 0.0) -> float:
        loss = C.c_float()
        self._chk(self.L.ewpt_mlp_train_step(self.h, _fp(x), _fp(y), x.shape[0], float(lr), float(wd),
                                             C.byref(loss)))
        return float(loss.value)


def log_spectrum(mean: np.ndarray, floor: float = 1e-30) -> np.ndarray:
    return np.log10(np.maximum(mean, 0.0) + floor)


def draw_members(n: int, N, seed: int, thermal_fraction: float = 0.0):
    """Seeded uniform draws of (lambda, g, g', bubble count) and the member
    params.  N is one lattice size or a sequence of sizes drawn uniformly per
    member; with several sizes log2(N) joins the parameter features.  With
    thermal_fraction > 0 that share of the runs starts from the thermal IC
    at T in [1, 2] vev instead of bubbles (bubble count 0), and T joins the
    features (0 for bubble runs)."""
    rng = np.random.default_rng(seed)
    lam = rng.uniform(0.11, 0.15, n)
    gw = rng.uniform(0.60, 0.70, n)
    gy = rng.uniform(0.32, 0.38, n)
    nb = rng.integers(4, 17, n)
    sizes = [int(N)] if np.isscalar(N) else [int(v) for v in N]
    Ns = rng.choice(sizes, n) if len(sizes) > 1 else np.full(n, sizes[0])
    ps = [baseline_couplings(N=int(Ns[i]), dx=0.25, dt=0.025, lam=float(lam[i]), gw=float(gw[i]),
                             gy=float(gy[i]), precision=_lib.FP32) for i in range(n)]
    cols = [lam, gw, gy]
    if thermal_fraction > 0:
        Ts = np.where(rng.random(n) < thermal_fraction, rng.uniform(1.0, 2.0, n), 0.0)
        nb = np.where(Ts > 0, 0, nb)
        cols += [nb.astype(np.float64), Ts]
    else:
        cols += [nb.astype(np.float64)]
    cols += [np.log2(Ns.astype(np.float64))] if len(sizes) > 1 else []
    return ps, np.stack(cols, axis=1), nb


def generate_dataset(n_runs: int, N=64, nshell: int = 40, t_early: int = 50, t_late: int = 500,
                     seed: int = 0, chunk: int = 96, verbose: bool = False, thermal_fraction: float = 0.0) -> dict:
    """Evolve n_runs seeded bubble-nucleation runs with the ensemble engine and
    record X = [log B spectrum, log Higgs spectrum at t_early, params] and
    Y = log B spectrum at t_late (nshell log shells each over [1, N/2] in
    index units).  N: one size or a sequence of sizes (draw_members)."""
    X, Y, P, E = [], [], [], []
    t0 = time.perf_counter()
    gpu_s = 0.0
    for c0 in range(0, n_runs, chunk):
        n = min(chunk, n_runs - c0)
        ps, prm, nb = draw_members(n, N, seed * 100003 + c0, thermal_fraction)
        with Ensemble(ps) as ens:
            for m, p in enumerate(ps):
                if nb[m] > 0:
                    R, w = ic.tanh_profile_params(p.lam, p.vev)
                    bl = ic.tanh_bubble_list(p.dims, p.dx, int(nb[m]), seed=seed * 7919 + c0 + m)
                    ens.init_bubbles(m, bl, "tanh", R, w)
                else:  # thermal run: T is the feature after the bubble count
                    ens.init_thermal(m, float(prm[m, 4]) * p.vev, seed=seed * 7919 + c0 + m)
            ts = time.perf_counter()
            ens.step(t_early)
            ens.sync()
            gpu_s += time.perf_counter() - ts
            early = [(ens.spectrum(m, "B", "log", nshell)["mean"], ens.spectrum(m, "higgs", "log", nshell)["mean"])
                     for m in range(n)]
            e_early = [ens.diagnostics(m)[13] for m in range(n)]
            ts = time.perf_counter()
            ens.step(t_late - t_early)
            ens.sync()
            gpu_s += time.perf_counter() - ts
            late = [ens.spectrum(m, "B", "log", nshell)["mean"] for m in range(n)]
        for m in range(n):
            X.append(np.concatenate([log_spectrum(early[m][0]), log_spectrum(early[m][1]), prm[m]]))
            Y.append(log_spectrum(late[m]))
            P.append(prm[m])
            E.append(e_early[m])
        if verbose:
            print(f"runs {c0 + n}/{n_runs}  {time.perf_counter() - t0:.1f}s", flush=True)
    return dict(X=np.array(X, dtype=np.float32), Y=np.array(Y, dtype=np.float32), params=np.array(P),
                evolve_seconds=gpu_s, runs=n_runs, N=N if np.isscalar(N) else list(N), t_early=t_early,
                t_late=t_late, nshell=nshell)


class Surrogate:
    """Standardised-feature MLP regressor of the late-time log B spectrum."""

    def __init__(self, n_in: int, n_out: int, width: int = 256, max_batch: int = 512, device: int = 0,
                 seed: int = 0):
        self.net = MLP(n_in, width, n_out, max_batch, device, seed)
        self.mx = self.sx = self.my = self.sy = None

    def _norm(self, X, Y=None):
        if self.mx is None:
            self.mx, self.sx = X.mean(0), np.maximum(X.std(0), 1e-6)
            if Y is not None:
                self.my, self.sy = Y.mean(0), np.maximum(Y.std(0), 1e-6)
        xs = ((X - self.mx) / self.sx).astype(np.float32)
        ys = None if Y is None else ((Y - self.my) / self.sy).astype(np.float32)
        return xs, ys

    def fit(self, X, Y, epochs: int = 300, batch: int = 128, lr: float = 2e-3, wd: float = 1e-4, seed: int = 0):
        xs, ys = self._norm(X, Y)
        rng = np.random.default_rng(seed)
        n = xs.shape[0]
        hist = []
        for ep in range(epochs):
            order = rng.permutation(n)
            lr_ep = lr * 0.5 * (1 + math.cos(math.pi * ep / epochs))
            tot = 0.0
            for s in range(0, n, batch):
                idx = order[s:s + batch]
                tot += self.net.train_step(np.ascontiguousarray(xs[idx]), np.ascontiguousarray(ys[idx]), lr_ep,
                                           wd) * len(idx)
            hist.append(tot / n)
        return hist

    def predict(self, X):
        xs, _ = self._norm(X)
        return self.net.forward(xs) * self.sy + self.my


def train_and_evaluate(n_runs: int = 1024, N=48, nshell: int = 40, t_early: int = 50, t_late: int = 500,
                       holdout: float = 0.1, epochs: int = 300, seed: int = 0, verbose: bool = True,
                       thermal_fraction: float = 0.0) -> dict:
    """Generate a dataset with the ensemble engine, train the surrogate on the
    growth of the log B spectrum over persistence, and report held-out errors
    against the evolved spectra (the reference answer) and the cost of both paths.
    holdout: a fraction of the runs (< 1) or a number of runs (>= 1)."""
    t_gen = time.perf_counter()
    data = generate_dataset(n_runs, N=N, nshell=nshell, t_early=t_early, t_late=t_late, seed=seed,
                            verbose=verbose, thermal_fraction=thermal_fraction)
    t_gen = time.perf_counter() - t_gen
    X, Y = data["X"], data["Y"]
    n_te = int(holdout) if holdout >= 1 else max(1, int(round(holdout * n_runs)))
    ntr = n_runs - n_te
    early = X[:, :nshell]
    sur = Surrogate(X.shape[1], nshell, width=256, max_batch=512, seed=seed)
    t0 = time.perf_counter()
    hist = sur.fit(X[:ntr], Y[:ntr] - early[:ntr], epochs=epochs, batch=128)
    t_train = time.perf_counter() - t0
    t0 = time.perf_counter()
    pred = sur.predict(X[ntr:]) + early[ntr:]
    t_inf = time.perf_counter() - t0
    live = Y[:ntr].std(0) > 1e-3
    Yt = Y[ntr:]
    mse = lambda P: float(np.mean((P - Yt)[:, live] ** 2))
    report = dict(runs=n_runs, train=ntr, held_out=n_te, N=data["N"], nshell=nshell, t_early=t_early,
                  t_late=t_late, thermal_fraction=thermal_fraction, dataset_seconds=t_gen,
                  mse_surrogate=mse(pred), mse_mean_baseline=mse(np.broadcast_to(Y[:ntr].mean(0), Yt.shape)),
                  mse_persistence=mse(early[ntr:] + (Y[:ntr] - early[:ntr]).mean(0)),
                  train_seconds=t_train, final_train_loss=hist[-1],
                  inference_us_per_run=t_inf / n_te * 1e6,
                  evolution_ms_per_run=data["evolve_seconds"] / n_runs * 1e3,
                  params=sur.net.num_params)
    return dict(report=report, surrogate=sur, data=data)


if __name__ == "__main__":
    import argparse
    import json

    ap = argparse.ArgumentParser(description="train and evaluate the spectrum surrogate")
    ap.add_argument("--runs", type=int, default=1024)
    ap.add_argument("--N", default="48", help="lattice size, or sizes drawn per run: 64,96,128")
    ap.add_argument("--held-out", type=float, default=0.1, help="fraction (< 1) or number of held-out runs")
    ap.add_argument("--thermal-fraction", type=float, default=0.0, help="share of thermal-IC runs (T in [1, 2])")
    ap.add_argument("--nshell", type=int, default=40)
    ap.add_argument("--t-early", type=int, default=50)
    ap.add_argument("--t-late", type=int, default=500)
    ap.add_argument("--epochs", type=int, default=300)
    ap.add_argument("--out", default=None, help="write the report JSON here")
    a = ap.parse_args()
    sizes = [int(v) for v in a.N.split(",")]
    r = train_and_evaluate(a.runs, sizes[0] if len(sizes) == 1 else sizes, a.nshell, a.t_early, a.t_late,
                           holdout=a.held_out, epochs=a.epochs, thermal_fraction=a.thermal_fraction)["report"]
    print(json.dumps(r, indent=1))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(r, f, indent=1)
