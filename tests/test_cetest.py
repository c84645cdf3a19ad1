"""The circular-explosion convergence harness (sim_circularexplosiontest) at
a reduced size: reference solution 400x400, runs at 50 and 100 cells."""
import os

import numpy as np
import pytest

import gfm_gb300 as g


def test_bilinear_matches_oracle_definition():
    """The harness's vectorised interpolation against the scalar definition."""
    import cetest
    d = cetest._desc(12, 2, False)
    nr, nc = d.shape
    f = np.random.default_rng(3).standard_normal((nr, nc))
    xs = np.array([0.01, 0.5, 1.33, 1.99, -0.2, 2.3])
    ys = np.array([0.2, 1.0, 0.07, 1.5, 0.9, -0.4])
    got = cetest.bilinear(d, f, xs, ys)
    for k in range(len(xs)):
        s = (xs[k] - d.x0) * (1.0 / d.dx) + d.numGC - 0.5
        t = (ys[k] - d.y0) * (1.0 / d.dy) + d.numGC - 0.5
        j0 = min(max(int(np.floor(s)), 0), nc - 2)
        i0 = min(max(int(np.floor(t)), 0), nr - 2)
        a, b = s - j0, t - i0
        v = (((1.0 - a) * (1.0 - b)) * f[i0, j0] + (a * (1.0 - b)) * f[i0, j0 + 1] +
             ((1.0 - a) * b) * f[i0 + 1, j0] + (a * b) * f[i0 + 1, j0 + 1])
        assert got[k] == v


@pytest.mark.gpu
def test_convergence_harness(tmp_path):
    import cetest
    out = cetest.run(str(tmp_path), N_ref=400, res=(50, 100))
    for name in ("singlemat",) + cetest.GFMS:
        rows = out[name]
        assert rows[1][1] < rows[0][1], (name, rows)     # l1 falls with resolution
        assert all(np.isfinite(r[1:4]).all() for r in [np.array(r) for r in rows])
    for name in cetest.GFMS:
        assert os.path.exists(tmp_path / ("CEtesterror-%s.dat" % name))
        assert os.path.exists(tmp_path / ("CEtestconservation-%s.dat" % name))
        assert all(np.isfinite(r[4]) and r[4] < 1.0 for r in out[name])   # a relative mass change
    with open(tmp_path / "CEtesterror-singlemat.dat") as f:
        assert len(f.read().split("\n")) == 3
