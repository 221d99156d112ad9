"""Gradient of a histogram misfit with respect to material parameters.

New entry point beside radiativeTransfer (the reference, cottereau/RadiativeTransferMonteCarlo,
has no gradient).  For an acoustic problem, the misfit

    L = sum over bins with E_target > 0 of (E - E_target)^2 / E_target,

E the energyDensity of radiativeTransfer.m:161-188, is differentiated with respect to

    lc        correlation length (MaterialClass CorrelationLength)
    cv_kappa  coefficient of variation of the bulk modulus (coefficients_of_variation(1))
    cv_rho    coefficient of variation of the density (coefficients_of_variation(2))
    Q         quality factor (propagateParticleSmallDt.m:57-82)
    mfp       the scattering mean free path v / Sigma, with the angular distribution held fixed.

The scattering parameters enter the path density of the sub-step scheme
(propagateParticleSmallDt.m:591-632) through sigma(theta) and Sigma; their derivatives are
score-function estimates accumulated by the rt_adjoint kernel, which replays each particle
from its Philox key.  Q only rescales the survival probability exp(-omega t / Q) of every
particle (the kill draw is independent of the path), so it is carried as a weight of each
time slice ("weight mode": the transport runs with qrate = 0) and differentiated exactly.
Bins where the target holds fewer than min_target_count particles (default 1000, so a
relative Monte Carlo error of the target below about 3%; 0 keeps every bin with
E_target > 0) are left out of L: a few-particle bin carries a weight 1 / E_target that
is mostly noise.
"""
from __future__ import annotations

import copy
import math

import numpy as np

from . import _lib
from .material import MaterialClass
from .radiative_transfer import DEFAULT_OPTIONS, build_problem, get_context, normalise

PARAMS = ("lc", "cv_kappa", "cv_rho", "Q", "mfp")
N_THETA = 4097  # grid of the d log sigma tables on [0, pi]


def target_mask(E_target: np.ndarray, grid, n_target: int, min_count: float) -> np.ndarray:
    """Bins kept in L: E_target > 0 and at least min_count target particles, counted as
    E_target x n_target x bin volume (the normalisation of radiativeTransfer.m:161-188)."""
    keep = E_target > 0
    if min_count > 0:
        one = normalise(np.ones(grid.hist_len), grid, 1)[0]  # density of one particle per bin
        keep &= E_target * n_target / one >= min_count - 1e-9
    return keep


def misfit(E: np.ndarray, E_target: np.ndarray) -> tuple[float, np.ndarray]:
    """L and dL/dE over the bins where E_target > 0."""
    m = E_target > 0
    r = np.zeros_like(E)
    r[m] = (E[m] - E_target[m]) / E_target[m]
    return float(np.sum(r[m] * (E[m] - E_target[m]))), 2.0 * r


def _set_param(md: _lib.RtmcMaterial, name: str, value: float) -> None:
    if name == "lc":
        md.lc = value
    elif name == "cv_kappa":
        md.cv[0] = value
    elif name == "cv_rho":
        md.cv[1] = value
    else:
        raise ValueError(name)


def _get_param(md: _lib.RtmcMaterial, name: str) -> float:
    return {"lc": md.lc, "cv_kappa": md.cv[0], "cv_rho": md.cv[1]}[name]


def score_tables(material: MaterialClass, d: int, params, n_theta: int = N_THETA, rel: float = 1e-4):
    """d log sigma(theta) / dp on a uniform grid of [0, pi] and d log Sigma / dp for each
    scattering parameter (central differences of the FP64 cross-sections in p; 'Q' has no
    scattering part and gets zeros).  Returns (dlogsigma [n, n_theta], dlogSigma [n])."""
    lib = _lib.load()
    md = material._descriptor(d)
    theta = np.linspace(0.0, math.pi, n_theta)
    tp = theta.ctypes.data_as(_lib.C.POINTER(_lib.C.c_double))
    base = np.empty(n_theta)
    _lib.check(lib.rtmc_sigma_eval(_lib.C.byref(md), 0, n_theta, tp, _lib.dptr(base)))
    S0 = (_lib.C.c_double * 4)()
    Sp = (_lib.C.c_double * 4)()
    _lib.check(lib.rtmc_sigma_total(_lib.C.byref(md), S0, Sp))
    dls = np.zeros((len(params), n_theta))
    dlS = np.zeros(len(params))
    for q, name in enumerate(params):
        if name == "Q":
            continue
        if name == "mfp":  # sigma scales as 1 / mfp
            mfp = material.v / S0[0]
            dls[q, :] = -1.0 / mfp
            dlS[q] = -1.0 / mfp
            continue
        p0 = _get_param(md, name)
        h = rel * max(abs(p0), 1e-3)
        vals, tots = [], []
        for sgn in (1.0, -1.0):
            m2 = copy.copy(md)
            _set_param(m2, name, p0 + sgn * h)
            out = np.empty(n_theta)
            _lib.check(lib.rtmc_sigma_eval(_lib.C.byref(m2), 0, n_theta, tp, _lib.dptr(out)))
            S = (_lib.C.c_double * 4)()
            _lib.check(lib.rtmc_sigma_total(_lib.C.byref(m2), S, (_lib.C.c_double * 4)()))
            vals.append(out)
            tots.append(S[0])
        ok = base > 0  # angles with sigma = 0 are never drawn
        dls[q, ok] = (vals[0][ok] - vals[1][ok]) / (2 * h * base[ok])
        dlS[q] = (tots[0] - tots[1]) / (2 * h * S0[0])
    return dls, dlS


def with_param(material: MaterialClass, name: str, value: float) -> MaterialClass:
    """A copy of material with one parameter changed and its tables rebuilt on demand."""
    m = copy.copy(material)
    m.invcdf = None
    if name == "lc":
        m.CorrelationLength = value
    elif name in ("cv_kappa", "cv_rho"):
        cv = np.array(m.coefficients_of_variation, dtype=float)
        cv[0 if name == "cv_kappa" else 1] = value
        m.coefficients_of_variation = cv
    elif name == "Q":
        m.Q = value
        m.invcdf = material.invcdf
    else:
        raise ValueError(f"no material field for '{name}'")
    return m


def _slice(v: np.ndarray, like: np.ndarray) -> np.ndarray:
    """A per-time-slice vector shaped to broadcast over [axes..., Nt, modes]."""
    return v.reshape((1,) * (like.ndim - 2) + (-1, 1))


def _weights(material: MaterialClass, grid) -> tuple[np.ndarray, float, float]:
    """exp(-omega t / Q) per time slice, omega, Q."""
    Q = float(np.atleast_1d(material.Q if material.Q is not None else math.inf)[0])
    if not math.isfinite(Q):
        return np.ones(grid.Nt), 0.0, Q
    if material.Frequency is None:
        raise ValueError("A finite quality factor Q needs mat.Frequency")
    omega = 2 * math.pi * float(np.atleast_1d(material.Frequency)[0])
    return np.exp(-omega * grid.t / Q), omega, Q


def forward_weighted(geometry, source, material, observation, options=None, mfp_scale: float = 1.0):
    """energyDensity in weight mode: transport with qrate = 0, time slice t scaled by
    exp(-omega t / Q).  Returns (E, prob, grid, N, counts, stats)."""
    opt = dict(DEFAULT_OPTIONS)
    opt.update(options or {})
    if not material.acoustics:
        raise NotImplementedError("gradients are implemented for acoustic problems")
    prob, grid, N = build_problem(geometry, source, material, observation, opt)
    prob.qrate = (0.0, 0.0)
    if mfp_scale != 1.0:
        prob.mft = tuple(m * mfp_scale for m in prob.mft)
    P, keep = prob.to_ctypes()
    counts, stats = get_context(int(opt["device"])).forward(P, prob.tables)
    dens, _ = normalise(counts, grid, N, prob.hist_shift)
    w, _, _ = _weights(material, grid)
    return dens * _slice(w, dens), prob, grid, N, counts, stats


def radiativeTransferGradient(geometry: dict, source: dict, material: MaterialClass, observation: dict,
                              E_target: np.ndarray, params=("lc", "cv_kappa", "cv_rho", "Q"),
                              options: dict | None = None) -> dict:
    """[g, L] = gradient of L(E(params), E_target) at the material's parameters.

    One weight-mode forward (rtmc_forward) gives E and L; one replay (rtmc_gradient) gives
    the score-function derivatives of the scattering parameters; the Q derivative is
    exact: dE/dQ = E omega t / Q^2.  Returns a dict with L, grad {name: value},
    energyDensity, and the timings of both passes."""
    opt = dict(DEFAULT_OPTIONS)
    opt.update(options or {})
    for p in params:
        if p not in PARAMS:
            raise ValueError(f"unknown parameter '{p}' (one of {PARAMS})")
    E, prob, grid, N, counts, st_f = forward_weighted(geometry, source, material, observation, opt)
    E_target = np.asarray(E_target, dtype=float).reshape(E.shape)
    kept = target_mask(E_target, grid, int(opt.get("target_particles", N)), float(opt.get("min_target_count", 1000)))
    E_target = np.where(kept, E_target, 0.0)
    L, dLdE = misfit(E, E_target)
    w, omega, Q = _weights(material, grid)
    # d E_b / d count_b: the (linear) normalisation times the slice weight
    unit = normalise(np.ones(prob.hist_len), grid, N, prob.hist_shift)[0] * _slice(w, E)
    # E and the score estimate of dE/dp come from the same particles, so sum_b dL/dE_b dE_b/dp
    # over-counts d Var(E_b)/dp / E_target_b: subtracting unit_b / E_target_b from dL/dE_b
    # makes the estimate unbiased for d E[L] / dp, which central differences with common
    # random numbers also estimate
    corr = np.zeros_like(E)
    m = E_target > 0
    corr[m] = unit[m] / E_target[m]
    adj = (dLdE - corr) * unit
    centred = False
    if opt.get("centre_weights", True):
        # Control variate: the score of a path up to an instant has zero mean, so when every
        # particle is observed at every instant (the grid holds all of them, as at Q = Inf
        # in weight mode), subtracting from the weights of instant j their mean over the
        # particles' bins, sum_b w_b count_b / N, leaves the estimate unbiased and removes
        # the part of its variance that the common weight of the instant carries.
        c = counts.reshape(E.shape, order="F").astype(np.float64) / float(1 << prob.hist_shift)
        per_slice = c.sum(axis=tuple(k for k in range(c.ndim) if k != c.ndim - 2))
        if np.all(per_slice[1:] == N):
            wbar = (adj * c).sum(axis=tuple(k for k in range(c.ndim) if k != c.ndim - 2)) / N
            adj = adj - _slice(wbar, adj)
            centred = True
    adjoint = adj.ravel(order="F")
    grad = {}
    scat = [p for p in params if p != "Q"]
    st_a = None
    if scat:
        dls, dlS = score_tables(material, prob.d, scat)
        P, _keep = prob.to_ctypes()
        g, st_a = get_context(int(opt["device"])).gradient(P, prob.tables, dls, dlS, adjoint)
        del _keep
        grad.update({p: float(v) for p, v in zip(scat, g)})
    if "Q" in params:
        tq = (omega * grid.t / Q ** 2) if math.isfinite(Q) else np.zeros(grid.Nt)
        grad["Q"] = float(np.sum(dLdE * E * _slice(tq, E)))
    return {"L": L, "grad": grad, "energyDensity": E, "N": N, "bins": int(kept.sum()), "forward_stats": st_f,
            "adjoint_stats": st_a, "centred": centred}


def finite_difference(geometry, source, material, observation, E_target, name: str, rel: float = 1e-3,
                      options: dict | None = None) -> float:
    """Central difference of L in parameter `name` with common random numbers (the same
    seed, so the same Philox keys, on both sides), step rel * |p|, over the bins that
    radiativeTransferGradient keeps."""
    opt = dict(DEFAULT_OPTIONS)
    opt.update(options or {})
    _, grid, N = build_problem(geometry, source, material, observation, opt)
    E_target = np.asarray(E_target, dtype=float).reshape(grid.shape)
    keep = target_mask(E_target, grid, int(opt.get("target_particles", N)), float(opt.get("min_target_count", 1000)))
    E_target = np.where(keep, E_target, 0.0)
    if name == "mfp":
        mfp = material.meanFreePath if material.meanFreePath is not None else None
        if mfp is None:
            MaterialClass.prepareSigma(material, int(geometry["dimension"]))
            mfp = material.meanFreePath
        Ls = []
        for sgn in (1.0, -1.0):
            E = forward_weighted(geometry, source, material, observation, options, mfp_scale=1 + sgn * rel)[0]
            Ls.append(misfit(E, np.asarray(E_target).reshape(E.shape))[0])
        return (Ls[0] - Ls[1]) / (2 * rel * mfp)
    p0 = {"lc": lambda m: float(m.CorrelationLength),
          "cv_kappa": lambda m: float(np.atleast_1d(m.coefficients_of_variation)[0]),
          "cv_rho": lambda m: float(np.atleast_1d(m.coefficients_of_variation)[1]),
          "Q": lambda m: float(np.atleast_1d(m.Q)[0])}[name](material)
    h = rel * abs(p0)
    Ls = []
    for sgn in (1.0, -1.0):
        m = with_param(material, name, p0 + sgn * h)
        E = forward_weighted(geometry, source, m, observation, options)[0]
        Ls.append(misfit(E, np.asarray(E_target).reshape(E.shape))[0])
    return (Ls[0] - Ls[1]) / (2 * h)
