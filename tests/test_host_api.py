"""Host-side mirror of the reference: observation grid (initializeObservation.m), problem
set-up (radiativeTransfer.m:4-38, propagateParticleSmallDt.m:3-82) and the FP64
normalisation (radiativeTransfer.m:160-191).  CPU only."""
import math

import numpy as np
import pytest

from radiativetransfermontecarlo_gb300 import MaterialClass, build_problem, colon, initialize_observation, normalise
from radiativetransfermontecarlo_gb300 import workloads as W
from radiativetransfermontecarlo_gb300.replicas import shard


def test_colon_like_matlab():
    e = colon(0, 0.05, 6)
    assert e.size == 121 and e[0] == 0.0 and e[-1] == 6.0
    e = colon(-5, 1 / 6, 5)
    assert e.size == 61 and e[0] == -5.0 and e[-1] == 5.0
    assert np.allclose(np.diff(e), 1 / 6)


def test_c1_observation_grid():
    geo, src, mat, obs, opts = W.c1_acoustic3d()
    g = initialize_observation(dict(geo), True, obs, 10 ** 6)
    assert g.Nt == 251 and g.t[0] == 0.0 and math.isclose(g.t[-1], 5.0)
    assert g.ibins == [1, 2] and g.shape == (120, 1, 251, 1)
    r, dr = g.obs["x"], np.diff(obs["x"])
    # spherical volume weights r^2 dr + dr^3/12 at the bin centres (initializeObservation.m:173-186;
    # the dr^3/24 special case applies only to a centre at r = 0)
    assert np.allclose(g.obs["dx"], r ** 2 * dr + dr ** 3 / 12)
    assert np.allclose(g.obs["binZ"], [-1.0, 1.0])                  # sin of the elevation edges
    assert np.allclose(g.obs["binPsi"], [-1.0, 1.0])                # cos of the reversed direction edges
    assert g.axis_mode == [2, 2, 1, 1] and g.time_stride == 120 and g.hist_len == 120 * 251


def test_extended_grid_and_two_axis_limit():
    geo, src, mat, obs, opts = W.c2_elastic3d()
    with pytest.raises(ValueError, match="two directions"):
        initialize_observation(dict(geo), False, obs, 10)
    g = initialize_observation(dict(geo), False, obs, 10, extended=True)
    assert g.shape == (60, 60, 60, 8, 251, 2) and g.hist_len == 867_456_000
    assert np.allclose(g.obs["binPsi"], np.cos(colon(0, math.pi / 8, math.pi)[::-1]))


def test_2d_never_checks_the_z_axis():
    g = initialize_observation({"dimension": 2, "frame": "cylindrical"}, False, {"x": colon(0, 0.05, 10),
                                                                             "time": colon(0, 0.025, 1)}, 10)
    assert g.axis_mode[2] == 0 and g.ibins == [1, 2]


def test_problem_set_up_substeps_q_and_rounding():
    geo, src, mat, obs, opts = W.c1_acoustic3d(n=123_456)
    prob, grid, N = build_problem(geo, src, mat, obs, opts)
    assert N == 200_000  # rounded up to whole packets of 1e5 (radiativeTransfer.m:23-24)
    assert prob.n_sub == 1 and math.isclose(prob.h, 0.02)
    assert prob.axis_mode == [2, 0, 0, 0]  # y, z and direction ranges cover everything: skipped
    geo, src, mat, obs, opts = W.c2_elastic3d()
    prob, grid, N = build_problem(geo, src, mat, obs, dict(opts, exact_count=True))
    assert prob.n_sub == 3 and math.isclose(prob.h, 0.02 / 3) and N == 10 ** 7
    geo, src, mat, obs, opts = W.c3_halfspace2d()
    with pytest.warns(UserWarning, match="Only one quality factor"):
        prob, grid, N = build_problem(geo, src, mat, obs, opts)
    assert prob.n_sub == 76 and math.isclose(prob.h, 0.025 / 76)
    assert math.isclose(prob.qrate[0], 2 * math.pi * 8 * prob.h / 200) and prob.qrate[0] == prob.qrate[1]
    assert prob.bnd == [(2, 0.0, False)] and prob.zoe_rpp is not None


def test_problem_set_up_errors_like_the_reference():
    geo, src, mat, obs, opts = W.c1_acoustic3d()
    with pytest.raises(ValueError, match="Unknown boundary type"):
        build_problem(dict(geo, bnd=[{"dir": 3, "val": 0, "type": "sticky"}]), src, mat, obs, opts)
    m = MaterialClass.preset(1)
    m.Q = 100  # finite Q needs a frequency (propagateParticleSmallDt.m:59-62)
    with pytest.raises(ValueError, match="Frequency"):
        build_problem(geo, src, m, obs, opts)
    with pytest.raises(ValueError, match="boundary dir"):
        build_problem(dict(geo, bnd=[{"dir": 5, "val": 1}]), src, mat, obs, opts)
    with pytest.raises(ValueError, match="plane sources are 3D only"):
        g2, s2, m2, o2, p2 = W.c3_halfspace2d()
        build_problem(g2, dict(s2, type="plane", direction=1, extent=1), m2, o2, p2)
    with pytest.raises(ValueError, match="use \\+-1"):
        build_problem(geo, dict(src, type="plane", direction=4, extent=1), mat, obs, opts)
    with pytest.raises(ValueError, match="scalar radius"):
        build_problem(geo, dict(src, type="plane", direction=3, aperture="circle", extent=[1, 2]), mat, obs, opts)
    with pytest.raises(ValueError, match="Unknown plane-wave aperture"):
        build_problem(geo, dict(src, type="plane", direction=3, aperture="hexagon", extent=1), mat, obs, opts)
    with pytest.raises(ValueError, match="density"):
        geo3, src3, mat3, obs3, opts3 = W.c3_halfspace2d()
        mat3.rho = None
        build_problem(geo3, src3, mat3, obs3, opts3)


def test_normalise_matches_radiativeTransfer_formulas():
    rng = np.random.default_rng(0)
    # 3D spherical, ibins [1 4]: E ./ (d1' * (d2*N)) .* dpsi / (dy*dz)
    obs = {"x": colon(0, 0.5, 3), "directions": colon(0, math.pi / 4, math.pi), "time": [0, 1, 2]}
    g = initialize_observation({"dimension": 3, "frame": "spherical"}, True, obs, 1000)
    assert g.ibins == [1, 4]
    E = rng.integers(0, 100, size=g.hist_len).astype(np.int64)
    dens, energy = normalise(E, g, 1000)
    Ef = E.reshape(g.shape, order="F").astype(float)
    d1, d2 = g.obs["dx"], g.obs["dpsi"]
    want = Ef / (d1[:, None] * d2[None, :] * 1000)[:, :, None, None] * d2[None, :, None, None] / (
        g.obs["dy"] * g.obs["dz"])
    assert np.allclose(dens, want)
    assert np.allclose(energy, Ef.sum(axis=(0, 1)) / 1000)


def test_shard_partitions_particle_ids():
    for n, w in ((10, 3), (7, 7), (1000003, 4), (5, 8)):
        parts = [shard(n, r, w) for r in range(w)]
        assert sum(c for _, c in parts) == n
        first = 0
        for f, c in parts:
            assert f == first
            first += c


def test_large_time_steps_scheme_set_up():
    """timeSteps = 1 (propagateParticle.m): continuous-time flights on a 2^20 grid per
    interval, no Q and no boundaries, as the reference's large-dt scheme has none."""
    geo, src, mat, obs, opts = W.c3_halfspace2d(t_end=1.0)
    mat.timeSteps = 1
    prob, grid, N = build_problem(geo, src, mat, obs, opts)
    assert prob.n_sub == 1 << 20 and prob.qrate == (0.0, 0.0) and prob.bnd == []
    assert prob.n_sub * prob.n_obs < 1 << 30
