"""Host side of radiativeTransferGradient on CPU: the library calls are replaced by the
event oracle (same paths, same score restatement), so the set-up, misfit, target floor,
adjoint weights, bias correction and exact Q derivative are checked without a GPU."""
import math

import numpy as np
import pytest

from oracle import oracle as O
from radiativetransfermontecarlo_gb300 import MaterialClass, colon, normalise
from radiativetransfermontecarlo_gb300 import adjoint as A
from radiativetransfermontecarlo_gb300 import radiative_transfer as RT
from radiativetransfermontecarlo_gb300 import workloads as W


class _OracleContext:
    def forward(self, prob, tables, out=None):
        h, st, _ = O.run(prob, O.table_knots(tables), scheme="event", ufloat=False)
        return h, st

    def gradient(self, prob, tables, dls, dlS, adjoint):
        return O.gradient(prob, O.table_knots(tables), dls, dlS, adjoint, ufloat=False)


@pytest.fixture
def oracle_backend(monkeypatch):
    monkeypatch.setattr(RT.TransportProblem, "to_ctypes", lambda self: (self, []))
    monkeypatch.setattr(A, "get_context", lambda device=0: _OracleContext())


def _case():
    geo, src, mat, obs, opts = W.c1_acoustic3d()
    obs = dict(obs, time=colon(0, 0.1, 2.0))
    tgt = MaterialClass(geo, 10, True, 1, [0.06, 0.04], 0, "exp", 0.12)
    tgt.Q = 300
    mat = MaterialClass(geo, 10, True, 1, [0.05, 0.05], 0, "exp", 0.1)
    mat.Q = 400
    o = dict(opts, exact_count=True, precision="fp64")
    return geo, dict(src, numberParticles=20000), mat, tgt, obs, o


def test_gradient_host_pipeline(oracle_backend):
    geo, src, mat, tgt, obs, o = _case()
    Et = A.forward_weighted(geo, src, tgt, obs, dict(o, seed=77))[0]
    params = ("lc", "cv_kappa", "cv_rho", "Q", "mfp")
    res = A.radiativeTransferGradient(geo, src, mat, obs, Et, params, dict(o, seed=3, min_target_count=20))
    # the same quantities by hand
    E, prob, grid, N, counts, _ = A.forward_weighted(geo, src, mat, obs, dict(o, seed=3))
    one = normalise(np.ones(grid.hist_len), grid, 1)[0]
    keep = (Et > 0) & (Et * N / one >= 20 - 1e-9)
    assert res["bins"] == int(keep.sum()) and 0 < res["bins"] < int((Et > 0).sum())
    T = np.where(keep, Et, 0.0)
    L = float(np.sum(((E - T) ** 2 / np.where(keep, T, 1.0))[keep]))
    assert math.isclose(res["L"], L, rel_tol=1e-12)
    w = np.exp(-2 * math.pi * 10 * grid.t / 400)
    unit = normalise(np.ones(prob.hist_len), grid, N)[0] * w[None, None, :, None]
    r = np.where(keep, 2 * (E - T) / np.where(keep, T, 1.0) - unit / np.where(keep, T, 1.0), 0.0)
    adj = r * unit
    # centring: every particle is in the grid at every instant here (weight mode, full box),
    # so the count-weighted mean weight of each instant is taken off that instant
    c = counts.reshape(E.shape, order="F").astype(np.float64) / float(1 << prob.hist_shift)
    assert res["centred"] and np.all(c.sum(axis=(0, 1, 3))[1:] == N)
    adj = adj - ((adj * c).sum(axis=(0, 1, 3)) / N)[None, None, :, None]
    scat = ["lc", "cv_kappa", "cv_rho", "mfp"]
    dls, dlS = A.score_tables(mat, 3, scat)
    g, _ = O.gradient(prob, O.table_knots(prob.tables), dls, dlS, adj.ravel(order="F"), ufloat=False)
    for q, p in enumerate(scat):
        assert math.isclose(res["grad"][p], g[q], rel_tol=1e-9, abs_tol=1e-12)
    # Q: exact, equal to central differences of the weight-mode misfit
    fdq = A.finite_difference(geo, src, mat, obs, Et, "Q", 1e-4, dict(o, seed=3, min_target_count=20))
    assert math.isclose(res["grad"]["Q"], fdq, rel_tol=1e-6)


def _trapz(y, x):
    return float(np.sum((y[1:] + y[:-1]) * np.diff(x)) / 2)


def test_score_tables_match_closed_form():
    """3D acoustic 'exp' medium: sigma ~ zeta^3 (cv_k^2 + cv_r^2 cos^2) / (1 + zeta^2 s^2 / a^2)^2,
    s^2 = 2 (1 - cos theta), a^3 = 6, zeta = omega lc / v (MaterialClass.m:479-517)."""
    geo = {"dimension": 3}
    mat = MaterialClass(geo, 10, True, 1, [0.05, 0.03], 0, "exp", 0.1)
    dls, dlS = A.score_tables(mat, 3, ["lc", "cv_kappa", "cv_rho", "mfp"])
    th = np.linspace(0, math.pi, dls.shape[1])
    c = np.cos(th)
    zeta, a2 = 2 * math.pi * 10 * 0.1, 6 ** (2 / 3)
    s2 = 2 * (1 - c)
    lc_ = 3 / 0.1 - 4 * zeta ** 2 * s2 / (0.1 * (a2 + zeta ** 2 * s2))
    poly = 0.05 ** 2 + 0.03 ** 2 * c ** 2
    assert np.allclose(dls[0], lc_, rtol=1e-6, atol=1e-6)
    assert np.allclose(dls[1], 2 * 0.05 / poly, rtol=1e-6)
    assert np.allclose(dls[2], 2 * 0.03 * c ** 2 / poly, rtol=1e-6, atol=1e-6)
    # d log Sigma = E[d log sigma] under the angular law sigma sin(theta) / Sigma
    pdf = np.sin(th) * (poly / (1 + zeta ** 2 * s2 / a2) ** 2)
    for q in range(3):
        assert math.isclose(_trapz(dls[q] * pdf, th) / _trapz(pdf, th), dlS[q], rel_tol=1e-5)
    assert np.allclose(dls[3], dlS[3]) and dlS[3] < 0


def test_gradient_without_centring(oracle_backend):
    geo, src, mat, tgt, obs, o = _case()
    Et = A.forward_weighted(geo, src, tgt, obs, dict(o, seed=77))[0]
    res = A.radiativeTransferGradient(geo, src, mat, obs, Et, ("lc", "mfp"),
                                      dict(o, seed=3, min_target_count=20, centre_weights=False))
    assert not res["centred"]
    E, prob, grid, N, counts, _ = A.forward_weighted(geo, src, mat, obs, dict(o, seed=3))
    one = normalise(np.ones(grid.hist_len), grid, 1)[0]
    keep = (Et > 0) & (Et * N / one >= 20 - 1e-9)
    T = np.where(keep, Et, 1.0)
    w = np.exp(-2 * math.pi * 10 * grid.t / 400)
    unit = normalise(np.ones(prob.hist_len), grid, N)[0] * w[None, None, :, None]
    r = np.where(keep, 2 * (E - T) / T - unit / T, 0.0)
    dls, dlS = A.score_tables(mat, 3, ["lc", "mfp"])
    g, _ = O.gradient(prob, O.table_knots(prob.tables), dls, dlS, (r * unit).ravel(order="F"), ufloat=False)
    for q, p in enumerate(("lc", "mfp")):
        assert math.isclose(res["grad"][p], g[q], rel_tol=1e-9, abs_tol=1e-12)
