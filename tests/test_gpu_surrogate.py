"""What the trained surrogate gains over the method without it: on held-out
seeds it predicts the late-time log B spectrum far better than the
input-blind baseline (the training-set mean spectrum) and than persistence
(the early spectrum shifted by the mean growth), at a small fraction of the
cost of evolving the run.  The evolution remains the reference answer: the errors are
measured against evolved spectra."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def data():
    import build_lib

    build_lib.build()
    from ewpt import surrogate

    return surrogate.generate_dataset(640, N=24, nshell=12, t_early=60, t_late=240, seed=11, chunk=128)


def test_surrogate_beats_baselines(data):
    from ewpt import surrogate

    X, Y = data["X"], data["Y"]
    ntr = 512
    nsh = Y.shape[1]
    early_B = X[:, :nsh]
    live = Y[:ntr].std(0) > 1e-3  # shells with power (empty shells are constant)
    # the network learns the growth of the spectrum over persistence
    sur = surrogate.Surrogate(X.shape[1], nsh, width=256, max_batch=256, seed=2)
    hist = sur.fit(X[:ntr], Y[:ntr] - early_B[:ntr], epochs=300, batch=64, lr=2e-3, wd=1e-3)
    assert hist[-1] < 0.5 * hist[0]
    t0 = time.perf_counter()
    pred = sur.predict(X[ntr:]) + early_B[ntr:]
    t_inf = time.perf_counter() - t0
    Yt = Y[ntr:]
    mse_sur = np.mean((pred - Yt)[:, live] ** 2)
    mse_mean = np.mean((Y[:ntr].mean(0) - Yt)[:, live] ** 2)
    shift = (Y[:ntr] - early_B[:ntr]).mean(0)
    mse_persist = np.mean((early_B[ntr:] + shift - Yt)[:, live] ** 2)
    per_run_inf = t_inf / len(Yt)
    per_run_evolve = data["evolve_seconds"] / data["runs"]
    print(f"held-out MSE (log10 spectrum): surrogate {mse_sur:.4g}, mean baseline {mse_mean:.4g}, "
          f"persistence {mse_persist:.4g}; inference {per_run_inf * 1e6:.1f} us/run vs "
          f"evolution {per_run_evolve * 1e3:.2f} ms/run")
    assert mse_sur < 0.85 * min(mse_mean, mse_persist)
    assert per_run_inf * 100 < per_run_evolve
