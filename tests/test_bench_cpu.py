"""bench.py's host-side pieces (no GPU): the roofline traffic taken from the
committed pair-kernel profile, the peaks, the drift fit and the argument
defaults of the measurement contract."""
import importlib.util
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_traffic_comes_from_the_committed_profile():
    b = _bench()
    t = b.profile_traffic()
    assert t is not None and 1e8 < t < 1e9
    with open(b.PROFILE) as f:
        txt = f.read()
    assert re.search(rf"traffic_bytes_per_launch:\s*{int(t)}\b", txt)


def test_peaks_measured_or_fallback():
    b = _bench()
    peaks, kind = b.load_peaks()
    assert kind in ("measured", "fallback")
    assert float(peaks["hbm_gbs"]) > 1000.0


def test_drift_fit_recovers_a_known_slope():
    b = _bench()

    class S:
        dt = 0.0005
        T = 300.0
        n = 3000

    t = np.arange(2001) * S.dt
    rec = np.zeros((t.size, 5))
    rec[:, 0] = 1000.0 + 3.0 * t  # kinetic part grows 3 kJ/mol/ps
    d = b.nve_drift(rec, S)
    kT = 1.380662e-23 * 6.022045e23 * S.T * 1e-3
    assert abs(d["kT_per_ns_per_dof"] - 3.0 * 1000.0 / (kT * (3 * S.n - 3))) < 1e-9
    assert d["steps"] == t.size


def test_defaults_keep_the_contract():
    src = open(os.path.join(ROOT, "bench.py")).read()
    steps = int(re.search(r'"--steps", type=int, default=(\d+)', src).group(1))
    warm = int(re.search(r'"--warmup", type=int, default=(\d+)', src).group(1))
    gpus = int(re.search(r'"--gpus", type=int, default=(\d+)', src).group(1))
    assert gpus == 1 and warm >= 3 and 100 <= steps <= 10000
