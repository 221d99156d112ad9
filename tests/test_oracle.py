"""The CPU oracle: the event (snap) scheme against the reference's sub-step order, and
the known answers that pin both (energy conservation, Q-kill survival, equipartition,
the elastic boundary energy partition of Examples/BoundaryReflectionEnergyTests.m)."""
import math

import numpy as np
import pytest

from oracle import oracle as O
from radiativetransfermontecarlo_gb300 import MaterialClass, build_problem, colon
from radiativetransfermontecarlo_gb300 import workloads as W


def _both(geo, src, mat, obs, opts, n):
    prob, grid, N = build_problem(geo, dict(src, numberParticles=n), mat, obs,
                                  dict(opts, exact_count=True, precision="fp64"))
    kn = O.table_knots(prob.tables)
    he, se, _ = O.run(prob, kn, scheme="event")
    hs, ss, _ = O.run(prob, kn, scheme="substep")
    return prob, grid, N, he.reshape(grid.shape, order="F"), hs.reshape(grid.shape, order="F"), se, ss


def _chi2_per_dof(a, b, floor=20):
    a, b = a.astype(float).ravel(), b.astype(float).ravel()
    m = (a + b) > floor
    return float(np.mean((a[m] - b[m]) ** 2 / (a[m] + b[m])))


def test_event_scheme_equals_substep_scheme_acoustic():
    geo, src, mat, obs, opts = W.c1_acoustic3d()
    prob, grid, N, he, hs, se, ss = _both(geo, src, mat, obs, opts, 20000)
    assert _chi2_per_dof(he, hs) < 1.3
    assert abs(se["scatter_events"] - ss["scatter_events"]) < 4 * math.sqrt(se["scatter_events"])
    # energy is conserved exactly at Q = Inf in an unbounded medium (radiativeTransfer.m:191)
    for h in (he, hs):
        energy = h.sum(axis=(0, 1))[:, 0] / N
        assert energy[0] == 0.0 and np.all(energy[1:] == 1.0)


def test_event_scheme_equals_substep_scheme_elastic_boundary_q():
    geo, src, mat, obs, opts = W.c3_halfspace2d(t_end=1.5)
    with pytest.warns(UserWarning):
        prob, grid, N, he, hs, se, ss = _both(geo, src, mat, obs, opts, 3000)
    assert _chi2_per_dof(he, hs) < 1.3
    for k in ("scatter_events", "boundary_hits", "kills", "conversions"):
        assert abs(se[k] - ss[k]) < 5 * math.sqrt(max(se[k], 1)) + 5, k


def test_q_kill_survival_is_exp_minus_omega_t_over_q():
    geo = {"dimension": 3}
    mat = MaterialClass(geo, 2, True, 1, [0.05, 0.05], 0, "exp", 0.3)
    mat.Q = 50
    src = {"lambda": 0.05}
    obs = {"x": colon(0, 1, 50), "time": colon(0, 0.05, 5)}
    prob, grid, N = build_problem(geo, dict(src, numberParticles=100_000), mat, obs,
                                  {"exact_count": True, "precision": "fp64"})
    h, st, _ = O.run(prob, O.table_knots(prob.tables), scheme="event")
    alive = h.reshape(grid.shape, order="F").sum(axis=(0, 1))[:, 0] / N
    want = np.exp(-2 * math.pi * 2 * grid.t / 50)
    sd = np.sqrt(want * (1 - want) / N) + 1e-12
    assert np.max(np.abs(alive[1:] - want[1:]) / sd[1:]) < 4.5


def test_equipartition_elastic_3d():
    """P/S energy ratio tends to (vs/vp)^d / (d-1) (plotEnergies.m:39); isotropic cross-sections
    of Examples/IsotropicElastic3D.m:24-30 on MaterialClass.preset(3)."""
    geo = {"dimension": 3}
    mat = MaterialClass.preset(3)
    d, K = 3, mat.vp / mat.vs
    spp = sps = 0.2 * mat.vp
    ssp = sps / ((d - 1) * K ** d)
    sss = spp + sps - ssp
    mat.sigma = [[spp / (4 * math.pi), sps / (4 * math.pi)], [ssp / (4 * math.pi), sss / (4 * math.pi)]]
    src = {"lambda": 0.002, "polarization": "P"}
    obs = {"x": colon(0, 1, 100), "time": colon(0, 0.1, 6)}
    prob, grid, N = build_problem(geo, dict(src, numberParticles=40_000), mat, obs,
                                  {"exact_count": True, "precision": "fp64"})
    h, st, _ = O.run(prob, O.table_knots(prob.tables), scheme="event")
    e = h.reshape(grid.shape, order="F").sum(axis=(0, 1)) / N
    late = grid.t >= 4.0
    ratio = e[late, 0].sum() / e[late, 1].sum()
    want = (mat.vs / mat.vp) ** d / (d - 1)
    assert abs(ratio - want) / want < 0.05


@pytest.mark.parametrize("mode,angle", [("P", 15), ("P", 30), ("P", 45), ("P", 60), ("SV", 10), ("SV", 20),
                                        ("SV", 30), ("SV", 45), ("SH", 15), ("SH", 60)])
def test_boundary_energy_partition(mode, angle):
    """Examples/BoundaryReflectionEnergyTests.m:384-440: a pure incident packet on z = 0
    ends as P with probability E_Rpp (P in), 1 - E_Rsvsv (SV in, below the critical
    angle), never (SV above it: the conversion falls back to SV), never (SH in)."""
    vp, vs, rho = 2500.0, 2500.0 / math.sqrt(3), 2000.0
    mat = MaterialClass.preset(3)
    mat.vp, mat.vs, mat.rho = vp, vs, rho
    z = MaterialClass.Zoeppritz(mat)
    n = 200_000
    a = math.radians(angle)
    d = np.tile([math.sin(a), 0.0, -math.cos(a)], (n, 1))
    eSH = np.array([0.0, 1.0, 0.0])  # d x n with n = e_z, normalised
    eSV = np.cross(eSH, d[0])
    q = np.tile(eSV if mode == "SV" else eSH, (n, 1))
    m = np.full(n, 0 if mode == "P" else 1)
    u = np.random.default_rng(angle).random(2 * n)
    d2, q2, m2 = O.reflect(z["E_Rpp"], z["E_Rsvsv"], vp, vs, 2, d, q, m, u)
    frac_p = np.mean(m2 == 0)
    crit = math.degrees(math.asin(vs / vp))
    if mode == "P":
        want = np.interp(angle, z["j1_deg"], z["E_Rpp"])
    elif mode == "SV":
        want = 1 - np.interp(angle, z["j1_deg"], z["E_Rsvsv"]) if angle < crit else 0.0
    else:
        want = 0.0
    assert abs(frac_p - want) < 5 * math.sqrt(max(want * (1 - want), 1e-6) / n) + 1e-12
    assert np.all(d2[:, 2] > 0)  # every particle leaves the boundary upwards
    conv = (m == 0) & (m2 == 1)  # P -> SV obeys Snell's law
    if conv.any():
        s_out = np.hypot(d2[conv, 0], d2[conv, 1])
        assert np.allclose(s_out, math.sin(a) * vs / vp, atol=1e-12)
