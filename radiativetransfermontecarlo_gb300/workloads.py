"""Synthetic workloads: the five benchmark configurations of the hot path.

Each returns (geometry, source, material, observation, options) for radiativeTransfer.
Parameters the configurations leave open are fixed here and stated:
  * source lambda = 0.05 (the README example with C1's material uses it);
  * C3: vp = 2, vs = 1.155, rho = 1000, source at depth 1 below the free surface y = 0
    (the reference's 2D plane is x-y, so the free surface is bnd.dir = 2, val = 0);
  * C4: v = 1, acf 'exp', lambda 0.05, C1's grid; one cv applied to both kappa and rho.
"""
from __future__ import annotations

import math

import numpy as np

from .material import MaterialClass
from .observation import colon


def c1_acoustic3d(n: int = 1_000_000, precision: str = "fp64"):
    """3D acoustic isotropic unbounded, spherical frame, 120 radial x 251 time bins."""
    geo = {"dimension": 3, "frame": "spherical"}
    mat = MaterialClass(geo, 10, True, 1, [0.05, 0.05], 0, "exp", 0.1)
    src = {"numberParticles": n, "position": [0, 0, 0], "lambda": 0.05}
    obs = {"x": colon(0, 0.05, 6), "y": [-math.pi, math.pi], "z": [-math.pi / 2, math.pi / 2],
           "directions": [0, math.pi], "time": colon(0, 0.02, 5)}
    return geo, src, mat, obs, {"precision": precision, "seed": 0}


def c2_elastic3d(n: int = 10_000_000, precision: str = "fp32", t_end: float = 5.0):
    """3D elastic isotropic unbounded, cartesian 60^3 x 8 directions x 251 times x 2 modes."""
    geo = {"dimension": 3, "frame": "cartesian"}
    mat = MaterialClass(geo, 5, False, [2, 1.155], [0.1, 0.1, 0.1], [0, 0, 0], "gauss", 0.2)
    src = {"numberParticles": n, "position": [0, 0, 0], "lambda": 0.05, "polarization": "P"}
    e = colon(-5, 1 / 6, 5)
    obs = {"x": e, "y": e, "z": e, "directions": colon(0, math.pi / 8, math.pi), "time": colon(0, 0.02, t_end)}
    return geo, src, mat, obs, {"precision": precision, "seed": 1, "histogram": "extended", "hist_shift": 40}


def c3_halfspace2d(n: int = 100_000_000, precision: str = "fp32", t_end: float = 10.0):
    """2D elastic P-SV half-space with a free surface, Q = 200, cylindrical 200 r x 401 t."""
    geo = {"dimension": 2, "frame": "cylindrical", "bnd": [{"dir": 2, "val": 0.0, "type": "reflective"}]}
    mat = MaterialClass(geo, 8, False, [2, 1.155], [0.2, 0.2, 0.2], [0, 0, 0], "exp", 0.5)
    mat.Q = 200
    mat.rho = 1000.0
    src = {"numberParticles": n, "position": [0, -1], "lambda": 0.05, "polarization": "P"}
    obs = {"x": colon(0, 0.05, 10), "time": colon(0, 0.025, t_end)}
    return geo, src, mat, obs, {"precision": precision, "seed": 2}


def c4_instance(i: int, seed: int = 4):
    """Instance i of the 256-instance acoustic sweep (parameters drawn from a seeded stream)."""
    rng = np.random.default_rng([seed, i])
    lc = math.exp(rng.uniform(math.log(0.02), math.log(1.0)))
    cv = rng.uniform(0.01, 0.2)
    freq = math.exp(rng.uniform(math.log(1.0), math.log(20.0)))
    Q = [math.inf, 100.0, 500.0][int(rng.integers(0, 3))]
    n = int(round(math.exp(rng.uniform(math.log(1e4), math.log(1e7)))))
    geo = {"dimension": 3, "frame": "spherical"}
    mat = MaterialClass(geo, freq, True, 1, [cv, cv], 0, "exp", lc)
    mat.Q = Q
    src = {"numberParticles": n, "position": [0, 0, 0], "lambda": 0.05}
    obs = {"x": colon(0, 0.05, 6), "y": [-math.pi, math.pi], "z": [-math.pi / 2, math.pi / 2],
           "directions": [0, math.pi], "time": colon(0, 0.02, 5)}
    return geo, src, mat, obs, {"precision": "fp32", "seed": seed}
