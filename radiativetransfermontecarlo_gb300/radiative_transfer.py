"""radiativeTransfer(geometry, source, material, observation): the drop-in entry point.

Mirrors radiativeTransfer.m of cottereau/RadiativeTransferMonteCarlo.  The host side
(defaults :7-17, packet rounding :23-24, initializeObservation :27-28, prepareSigma :31,
normalisation :160-191) stays on the host in FP64; the packet x time loop (:40-158,
initializeParticle + propagateParticleSmallDt + observeTime) runs on the GPU through
librtmc's rtmc_forward.
"""
from __future__ import annotations

import math
import warnings
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .material import MaterialClass
from .observation import ObservationGrid, initialize_observation, natural_range_covered

PACKET = 100_000  # Npk of radiativeTransfer.m:23

DEFAULT_OPTIONS = dict(precision="fp32", seed=0, device=0, exact_count=False, histogram="reference",
                       hist_shift=0, pid0=0, return_counts=False)


@dataclass
class TransportProblem:
    """Everything one transport launch needs: the rtmc_problem fields, the edges it points
    to and the tables handle.  Built on the host, consumed by librtmc."""
    d: int
    frame: int
    acoustics: bool
    precision: int
    src_dir: int
    polarization: int
    n_sub: int
    n_obs: int
    n_particles: int
    seed: int
    src_pos: tuple
    src_lambda: float
    v: tuple
    mft: tuple
    p2p: float
    s2s: float
    qrate: tuple
    h: float
    axis_mode: list
    axis_edges: list
    axis_stride: list
    time_stride: int
    mode_stride: int
    hist_len: int
    shape: tuple
    tables: object = None
    pid0: int = 0
    hist_shift: int = 0
    bnd: list = field(default_factory=list)     # [(dir, val, absorbing)]
    zoe_rpp: np.ndarray | None = None
    zoe_rsvsv: np.ndarray | None = None
    src_type: int = 0                            # _lib.SOURCE_POINT / SOURCE_PLANE
    src_aperture: int = 0                        # _lib.APERTURE_RECTANGLE / APERTURE_CIRCLE
    src_normal: tuple = (0.0, 0.0, 1.0)
    src_u: tuple = (1.0, 0.0, 0.0)
    src_v: tuple = (0.0, 1.0, 0.0)
    src_extent: tuple = (0.0, 0.0)
    src_radial: tuple | None = None              # (cdf knots, radii) of a radial point source
    max_events: int = 0                          # per-particle event cap (0: automatic)

    def to_ctypes(self):
        """Return (RtmcProblem, keep-alive list of the arrays it points into)."""
        P = _lib.RtmcProblem()
        P.d, P.frame, P.acoustics, P.precision = self.d, self.frame, int(self.acoustics), self.precision
        P.src_dir, P.polarization, P.n_sub, P.n_obs = self.src_dir, self.polarization, self.n_sub, self.n_obs
        P.n_bnd, P.hist_shift, P.max_events = len(self.bnd), self.hist_shift, self.max_events
        P.n_particles, P.pid0, P.seed = self.n_particles, self.pid0, self.seed
        for i in range(3):
            P.src_pos[i] = self.src_pos[i]
        P.src_lambda = self.src_lambda
        for m in range(2):
            P.v[m], P.mft[m], P.qrate[m] = self.v[m], self.mft[m], self.qrate[m]
        P.p2p, P.s2s, P.h = self.p2p, self.s2s, self.h
        keep = []
        for a in range(4):
            P.axis_mode[a] = self.axis_mode[a]
            if self.axis_mode[a] != _lib.AXIS_IGNORED:
                e = np.ascontiguousarray(self.axis_edges[a], dtype=np.float64)
                keep.append(e)
                P.axis_nedges[a] = e.size
                P.axis_edges[a] = _lib.dptr(e)
            P.axis_stride[a] = self.axis_stride[a]
        P.time_stride, P.mode_stride, P.hist_len = self.time_stride, self.mode_stride, self.hist_len
        for b, (bd, bv, ab) in enumerate(self.bnd):
            P.bnd_dir[b], P.bnd_val[b], P.bnd_absorb[b] = bd, bv, int(ab)
        if self.zoe_rpp is not None:
            for k in range(_lib.ZOE_N):
                P.zoe_rpp[k] = self.zoe_rpp[k]
                P.zoe_rsvsv[k] = self.zoe_rsvsv[k]
        P.src_type, P.src_aperture = self.src_type, self.src_aperture
        for i in range(3):
            P.src_normal[i], P.src_u[i], P.src_v[i] = self.src_normal[i], self.src_u[i], self.src_v[i]
        P.src_extent[0], P.src_extent[1] = self.src_extent
        if self.src_radial is not None:
            c = np.ascontiguousarray(self.src_radial[0], dtype=np.float64)
            r = np.ascontiguousarray(self.src_radial[1], dtype=np.float64)
            keep += [c, r]
            P.src_radial_n = c.size
            P.src_radial_cdf, P.src_radial_r = _lib.dptr(c), _lib.dptr(r)
        return P, keep


def _q_values(material: MaterialClass):
    # propagateParticleSmallDt.m:31-53
    Q = material.Q
    Qv = np.atleast_1d(np.asarray(Q if Q is not None else math.inf, dtype=float)).ravel()
    if Qv.size == 0:
        Qv = np.array([math.inf])
    if material.acoustics:
        return Qv[0], Qv[0]
    return (Qv[0], Qv[0]) if Qv.size == 1 else (Qv[0], Qv[1])


def radial_source_table(f, d: int, rmax: float, n: int = 10000) -> tuple[np.ndarray, np.ndarray]:
    """Inverse CDF of a radial source profile f(r) in dimension d (initializeParticle.m:175-203):
    pdf ~ r^(d-1) f(r) on linspace(0, rmax, n), cumulative sum, end values pinned to 0 and 1,
    flat stretches dropped.  Returns the (cdf, r) knots of the linear interpolant."""
    x = np.linspace(0.0, rmax, n)
    w = x ** (d - 1) * np.asarray(f(x), dtype=float)
    pdf = w / (0.5 * np.sum((w[1:] + w[:-1]) * np.diff(x)))  # trapz
    cdf = np.cumsum(pdf) * np.mean(np.diff(x))
    cdf[0], cdf[-1] = 0.0, 1.0
    i = np.flatnonzero(np.diff(cdf) > 0)
    ind = np.unique(np.concatenate([i, i + 1]))
    c, first = np.unique(np.sort(cdf[ind]), return_index=True)
    r = np.sort(x[ind])[first]
    return c, r


def _radial_profile(source: dict, d: int):
    """source['radial']: a (grid, values) pair read as griddedInterpolant(grid, values) (linear,
    linear extrapolation; Rmax = grid[-1]), or a callable f with source['radialMax']."""
    rad = source["radial"]
    if callable(rad):
        if source.get("radialMax") is None:
            raise ValueError("a callable radial profile needs source['radialMax']")
        return radial_source_table(rad, d, float(source["radialMax"]))
    g, v = (np.asarray(a, dtype=float).ravel() for a in rad)
    if g.size < 2 or g.size != v.size or np.any(np.diff(g) <= 0):
        raise ValueError("radial profile grid must be increasing and match its values")

    def f(x):
        y = np.interp(x, g, v)
        lo, hi = x < g[0], x > g[-1]
        y[lo] = v[0] + (x[lo] - g[0]) * (v[1] - v[0]) / (g[1] - g[0])
        y[hi] = v[-1] + (x[hi] - g[-1]) * (v[-1] - v[-2]) / (g[-1] - g[-2])
        return y
    return radial_source_table(f, d, float(g[-1]))


def _plane_source(source: dict):
    """Plane-wave source geometry (initializeParticle.m:61-148): unit normal n, an orthonormal
    basis (u, v) of the plane normal to n from the SVD of n (as MATLAB's null), the aperture
    and its extent."""
    sd = source.get("direction")
    if sd is None:
        raise ValueError("a plane source needs source['direction'] (+-1, +-2, +-3 or a 3-vector)")
    sd = np.atleast_1d(np.asarray(sd, dtype=float)).ravel()
    if sd.size == 1:
        k = int(sd[0])
        if k != sd[0] or abs(k) not in (1, 2, 3):
            raise ValueError("For a scalar plane-source direction, use +-1, +-2, or +-3.")
        n = np.zeros(3)
        n[abs(k) - 1] = math.copysign(1.0, k)
    elif sd.size == 3:
        n = sd
    else:
        raise ValueError("For a plane source, source.direction must be a 3-component vector or a scalar axis "
                         "+-1, +-2, or +-3.")
    n = n / np.linalg.norm(n)
    vh = np.linalg.svd(n.reshape(1, 3))[2]
    u, v = vh[1], vh[2]
    aperture = str(source.get("aperture") or "rectangle").lower()
    ext = np.atleast_1d(np.asarray(source.get("extent", 0.0), dtype=float)).ravel()
    if aperture == "rectangle":
        ap = _lib.APERTURE_RECTANGLE
        extent = (float(ext[0]), float(ext[0])) if ext.size == 1 else (float(ext[0]), float(ext[1]))
    elif aperture == "circle":
        if ext.size != 1:
            raise ValueError("For source.aperture = 'circle', source.extent must be a scalar radius.")
        ap = _lib.APERTURE_CIRCLE
        extent = (float(ext[0]), 0.0)
    else:
        raise ValueError("Unknown plane-wave aperture: use 'rectangle' or 'circle'.")
    return ap, tuple(n), tuple(u), tuple(v), extent


def build_problem(geometry: dict, source: dict, material: MaterialClass, observation: dict,
                  options: dict | None = None) -> tuple[TransportProblem, ObservationGrid, int]:
    """Host set-up of radiativeTransfer.m:4-38 and propagateParticleSmallDt.m:3-82."""
    opt = dict(DEFAULT_OPTIONS)
    opt.update(options or {})
    geometry = dict(geometry)
    geometry.setdefault("frame", "spherical")
    d = int(geometry["dimension"])
    acoustics = bool(material.acoustics)
    if not acoustics and np.size(material.Q) == 1 and math.isfinite(float(np.atleast_1d(material.Q)[0])):
        warnings.warn(f"Only one quality factor was provided for an elastic simulation. The same value "
                      f"Q = {float(np.atleast_1d(material.Q)[0]):g} will be used for both P and S waves.")
    n_req = int(source["numberParticles"])
    N = n_req if opt["exact_count"] else int(math.ceil(n_req / PACKET)) * PACKET
    grid = initialize_observation(geometry, acoustics, observation, N, extended=opt["histogram"] == "extended")
    if material.invcdf is None:
        MaterialClass.prepareSigma(material, d)
    large_dt = material.timeSteps == 1
    if material.timeSteps not in (0, 1, None):
        raise ValueError("timeSteps must be 0 (small time steps) or 1 (large time steps)")
    t = grid.t
    T = float(np.mean(np.diff(t)))
    mft = np.atleast_1d(np.asarray(material.meanFreeTime, dtype=float)).ravel()
    if mft.size == 1:
        mft = np.array([mft[0], mft[0]])
    if large_dt:
        # propagateParticle.m: exponential flights in continuous time (Poisson jumps per
        # interval, next jump at the minimum of uniform times), no Q and no boundaries.
        # Served by the event kernel on a grid of 2^20 sub-steps per interval (fewer when
        # the run has more than 1023 intervals), where geometric draws are exponential.
        n_sub = 1 << 20
        while n_sub > 1 and n_sub * (grid.Nt - 1) >= (1 << 30):
            n_sub >>= 1
    else:
        # sub-step of propagateParticleSmallDt.m:4-7 (uniform observation times)
        dt = min(0.01 * float(np.min(mft)), T)
        n_sub = int(math.ceil(T / dt))
    h = T / n_sub
    QP, QS = _q_values(material)
    qrate = [0.0, 0.0]
    if not large_dt and (math.isfinite(QP) or math.isfinite(QS)):
        if material.Frequency is None or np.size(material.Frequency) == 0:
            raise ValueError("A finite quality factor Q was provided, but mat.Frequency is empty. Please define "
                             "mat.Frequency before using Q-based attenuation.")
        omega = 2 * math.pi * float(np.atleast_1d(material.Frequency)[0])
        qrate = [omega * h / QP if math.isfinite(QP) else 0.0, omega * h / QS if math.isfinite(QS) else 0.0]
    # source (initializeParticle.m:3-148, 157-160)
    stype = source.get("type", "point")
    pos = list(np.atleast_1d(np.asarray(source.get("position", [0.0, 0.0, 0.0]), dtype=float)))
    if len(pos) == 2:
        pos.append(0.0)
    src_dir = 0
    plane = dict(src_type=_lib.SOURCE_POINT)
    radial = None
    if stype == "point":
        sdir = source.get("direction", "uniform")
        src_dir = {"uniform": 0, "outgoing": 1, "upper": 2}.get(sdir if isinstance(sdir, str) else "uniform", 0)
        if source.get("radial") is not None and np.size(source["radial"]) > 0:
            radial = _radial_profile(source, d)
    elif stype == "plane":
        if d != 3:
            raise ValueError("plane sources are 3D only")
        ap, n, u, v, extent = _plane_source(source)
        plane = dict(src_type=_lib.SOURCE_PLANE, src_aperture=ap, src_normal=n, src_u=u, src_v=v, src_extent=extent)
    else:
        raise ValueError(f"unknown source type '{stype}' (point or plane)")
    pol = 1 if (not acoustics and source.get("polarization", "P") == "S") else 0
    # boundaries (propagateParticleSmallDt.m:146-166)
    bnd = []
    for b in ([] if large_dt else geometry.get("bnd", []) or []):
        btype = (b.get("type") or "reflective").lower()
        if btype not in ("reflective", "absorbing"):
            raise ValueError(f'Unknown boundary type "{btype}". Use "reflective" or "absorbing".')
        if int(b["dir"]) not in (1, 2, 3, 4):
            raise ValueError("boundary dir must be 1, 2, 3 (planes) or 4 (cylinder)")
        bnd.append((int(b["dir"]), float(b["val"]), btype == "absorbing"))
    if len(bnd) > _lib.MAX_BND:
        raise ValueError("at most 4 boundaries")
    zr = zs = None
    if not acoustics and any(not ab for _, _, ab in bnd):
        z = MaterialClass.Zoeppritz(material)
        zr, zs = z["E_Rpp"], z["E_Rsvsv"]
    vel = (material.v, material.v) if acoustics else (material.vp, material.vs)
    # observation axes for the kernel, with always-true range checks dropped
    frame = geometry["frame"]
    modes = list(grid.axis_mode)
    for a in range(4):
        e = grid.edges[a]
        one_bin = modes[a] == _lib.AXIS_BINNED and e.size == 2  # a single bin: index 0 always
        if (modes[a] == _lib.AXIS_RANGE or one_bin) and natural_range_covered(frame, d, a, float(e[0]), float(e[-1])):
            modes[a] = _lib.AXIS_IGNORED
    prob = TransportProblem(
        d=d, frame=_lib.FRAME[frame], acoustics=acoustics,
        precision=_lib.FP64 if opt["precision"] == "fp64" else _lib.FP32,
        src_dir=src_dir, polarization=pol, n_sub=n_sub, n_obs=grid.Nt - 1, n_particles=N, seed=int(opt["seed"]),
        src_pos=tuple(pos[:3]), src_lambda=float(source.get("lambda", 0.0)), v=tuple(float(x) for x in vel),
        mft=(float(mft[0]), float(mft[1])), p2p=float(material.P2P or 1.0), s2s=float(material.S2S or 1.0),
        qrate=tuple(qrate), h=h, axis_mode=modes, axis_edges=list(grid.edges), axis_stride=list(grid.axis_stride),
        time_stride=grid.time_stride, mode_stride=grid.mode_stride, hist_len=grid.hist_len, shape=grid.shape,
        tables=material.invcdf, pid0=int(opt["pid0"]), hist_shift=int(opt["hist_shift"]), bnd=bnd,
        zoe_rpp=zr, zoe_rsvsv=zs, src_radial=radial, **plane)
    return prob, grid, N


def normalise(E: np.ndarray, grid: ObservationGrid, N: int, hist_shift: int = 0) -> tuple[np.ndarray, np.ndarray]:
    """energyDensity and energy from integer counts (radiativeTransfer.m:160-191), FP64."""
    obs = grid.obs
    Ed = E.reshape(grid.shape, order="F").astype(np.float64)
    if hist_shift:
        Ed /= float(2 ** hist_shift)
    nb = len(grid.ibins)
    if nb == 2:
        d1, d2 = np.asarray(grid.weights[0], float), np.asarray(grid.weights[1], float)
        dens = Ed / (d1[:, None] * (d2[None, :] * N))[:, :, None, None]
        ib = grid.ibins
        if obs["d"] == 3:
            if ib == [1, 2]:
                dens = dens / obs["dz"]
            elif ib == [1, 3]:
                dens = dens / obs["dy"]
            elif ib == [1, 4]:
                dens = dens * obs["dpsi"][None, :, None, None] / (obs["dy"] * obs["dz"])
            elif ib == [2, 4]:
                dens = dens * obs["dpsi"][None, :, None, None] / (obs["dx"] * obs["dz"])
            elif ib == [3, 4]:
                dens = dens * obs["dpsi"][None, :, None, None] / (obs["dx"] * obs["dy"])
            elif ib == [2, 3]:
                dens = dens / obs["dx"]
            else:
                raise ValueError("Unsupported bin combination in 3D")
        else:
            if ib == [1, 4]:
                dens = dens * obs["dpsi"][None, :, None, None] / obs["dy"]
            elif ib == [2, 4]:
                dens = dens * obs["dpsi"][None, :, None, None] / obs["dx"]
            elif ib != [1, 2]:
                raise ValueError("Unsupported bin combination in 2D")
    else:
        # extended histogram: density per unit of every binned axis
        w = np.ones(grid.shape[:nb])
        for k, wk in enumerate(grid.weights):
            sh = [1] * nb
            sh[k] = -1
            w = w * np.asarray(wk, float).reshape(sh)
        dens = Ed / (w[..., None, None] * N)
    energy = Ed.sum(axis=tuple(range(nb))) / N
    return dens, energy


_contexts: dict = {}


def get_context(device: int = 0) -> _lib.Context:
    ctx = _contexts.get(device)
    if ctx is None:
        ctx = _contexts[device] = _lib.Context(device)
    return ctx


def run_transport(prob: TransportProblem, device: int = 0, out: np.ndarray | None = None, counts_u32: bool = False):
    """One rtmc_forward call: int64 histogram (host) and the kernel statistics; with
    counts_u32, rtmc_forward_u32's uint32 counts (the reference's E, half the bytes)."""
    P, keep = prob.to_ctypes()
    ctx = get_context(device)
    hist, stats = (ctx.forward_u32 if counts_u32 else ctx.forward)(P, prob.tables, out)
    del keep
    return hist, stats


def radiativeTransfer(geometry: dict, source: dict, material: MaterialClass, observation: dict,
                      options: dict | None = None) -> dict:
    """obs = radiativeTransfer(geometry, source, material, observation) (radiativeTransfer.m:1).

    options (not in the reference): precision 'fp32' | 'fp64', seed, device, exact_count
    (skip the rounding of numberParticles up to a multiple of 1e5), histogram 'reference'
    (two binned axes) | 'extended' (up to four), hist_shift (int64 fixed-point shift),
    return_counts (add the raw int64 histogram as obs['E']; otherwise the histogram comes
    back as uint32 counts, the reference's type).
    """
    opt = dict(DEFAULT_OPTIONS)
    opt.update(options or {})
    prob, grid, N = build_problem(geometry, source, material, observation, opt)
    # uint32 counts as in the reference's E, unless the int64 fixed-point histogram is asked for
    u32 = not opt["return_counts"]
    hist, stats = run_transport(prob, int(opt["device"]), counts_u32=u32)
    obs = dict(grid.obs)
    obs["energyDensity"], obs["energy"] = normalise(hist, grid, N, 0 if u32 else prob.hist_shift)
    obs["stats"] = stats
    if opt["return_counts"]:
        obs["E"] = hist.reshape(grid.shape, order="F")
    return obs
