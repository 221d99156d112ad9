"""Observation grid: initializeObservation.m of cottereau/RadiativeTransferMonteCarlo.

Builds the time vector, bin edges, volume weights and the histogram layout
(initializeObservation.m:4-156), and maps them onto the four observation axes the
transport kernel bins (X, Y, Z, PSI in the frame conventions of observeTime.m:14-127).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib


def colon(a: float, step: float, b: float) -> np.ndarray:
    """a:step:b with both ends computed exactly and the middle symmetric, as MATLAB's colon."""
    n = int(math.floor((b - a) / step + 1e-10))
    k = np.arange(n + 1, dtype=float)
    last = a + n * step
    out = np.where(k < n / 2, a + k * step, last - (n - k) * step)
    return out


def _volume_spherical(d, r, d0r):
    # initializeObservation.m:173-186
    if d == 2:
        dr = r * d0r
        if r.size and r[0] == 0:
            dr[0] = d0r[0] ** 2 / 8
    else:
        dr = r ** 2 * d0r + d0r ** 3 / 12
        if r.size and r[0] == 0:
            dr[0] = d0r[0] ** 3 / 24
    return dr


def _volume_cylindrical(r, d0r):
    # initializeObservation.m:187-193
    dr = r * d0r
    if r.size and r[0] == 0:
        dr[0] = d0r[0] ** 2 / 8
    return dr


@dataclass
class ObservationGrid:
    obs: dict
    t: np.ndarray
    Nt: int
    ibins: list                   # 1-based binned axes, as in the reference
    edges: list                   # edges of axes X, Y, Z, PSI
    weights: list                 # d-weights of the binned axes (d1, d2, ...)
    axis_mode: list = field(default_factory=list)
    axis_stride: list = field(default_factory=list)
    shape: tuple = ()             # histogram shape (column-major)
    time_stride: int = 0
    mode_stride: int = 0
    hist_len: int = 0


def initialize_observation(geometry: dict, acoustics: bool, observation: dict, N: int,
                           extended: bool = False) -> ObservationGrid:
    """initializeObservation.m:1-156.  extended=True allows up to four binned axes."""
    d = int(geometry["dimension"])
    frame = geometry.get("frame", "spherical")
    if frame not in _lib.FRAME:
        raise ValueError("unknown frame type")
    time = np.atleast_1d(np.asarray(observation["time"], dtype=float))
    t = np.concatenate([[0.0], np.setdiff1d(time, [0.0])])
    Nt = t.size
    binX = np.atleast_1d(np.asarray(observation["x"], dtype=float))
    with np.errstate(invalid="ignore"):  # centres of [-Inf Inf] are NaN, as in MATLAB
        x = (binX[:-1] + binX[1:]) / 2
    Nx = x.size
    dx = np.diff(binX)
    if frame == "cartesian":
        binY = np.array([-np.inf, np.inf])
        binZ = np.array([-np.inf, np.inf])
    elif frame == "cylindrical":
        binY = np.array([-np.pi, np.pi])
        binZ = np.array([-np.inf, np.inf])
    else:
        binY = np.array([-np.pi, np.pi])
        binZ = np.array([-np.pi / 2, np.pi / 2])
    if observation.get("y") is not None and np.size(observation["y"]) > 0:
        binY = np.atleast_1d(np.asarray(observation["y"], dtype=float))
    with np.errstate(invalid="ignore"):
        y = (binY[:-1] + binY[1:]) / 2
    Ny = y.size
    dy = np.diff(binY)
    if d == 3 and observation.get("z") is not None and np.size(observation["z"]) > 0:
        binZ = np.atleast_1d(np.asarray(observation["z"], dtype=float))
    if d == 3 and frame == "spherical":
        binZ = np.sin(binZ)
    with np.errstate(invalid="ignore"):
        z = (binZ[:-1] + binZ[1:]) / 2
    Nz = z.size
    dz = np.diff(binZ)
    if observation.get("directions") is not None and np.size(observation["directions"]) > 0:
        binPsi = np.atleast_1d(np.asarray(observation["directions"], dtype=float))
    else:
        binPsi = np.array([0.0, np.pi])
    if d == 3:
        binPsi = np.cos(binPsi[::-1])
    psi = (binPsi[:-1] + binPsi[1:]) / 2
    Npsi = psi.size
    dpsi = np.diff(binPsi)
    if frame == "spherical":
        dx = _volume_spherical(d, x, dx)
    elif frame == "cylindrical":
        dx = _volume_cylindrical(x, dx)
    counts = [Nx, Ny, Nz, Npsi]
    ibins = [i + 1 for i, n in enumerate(counts) if n > 1]
    if not ibins:
        ibins = [1, 2]
    elif len(ibins) == 1:
        ibins = [1, ibins[0]] if ibins[0] != 1 else [1, 2]
    if len(ibins) > 2 and not extended:
        raise ValueError("histograms can only be constructed along two directions")
    if not extended and ibins not in ([1, 2], [1, 3], [1, 4], [2, 4], [3, 4], [2, 3]):
        raise ValueError(f"Bin combination {ibins} not implemented yet")
    edges = [binX, binY, binZ, binPsi]
    widths = [dx, dy, dz, dpsi]
    nmodes = 1 if acoustics else 2
    obs = dict(d=d, acoustics=acoustics, N=N, t=t, Nt=Nt, x=x, Nx=Nx, dx=dx, binX=binX, y=y, Ny=Ny, dy=dy,
               binY=binY, z=z, Nz=Nz, dz=dz, binZ=binZ, psi=psi, Npsi=Npsi, dpsi=dpsi, binPsi=binPsi)
    g = ObservationGrid(obs=obs, t=t, Nt=Nt, ibins=ibins, edges=edges, weights=[widths[a - 1] for a in ibins])
    # axis modes for the kernel (observeTime.m:129-135): binned axes, then range checks on
    # the integrated ones; in 2D the Z axis is never checked
    stride = 1
    shape = []
    g.axis_mode = [0, 0, 0, 0]
    g.axis_stride = [0, 0, 0, 0]
    for a in range(4):
        if (a + 1) in ibins:
            g.axis_mode[a] = _lib.AXIS_BINNED
            g.axis_stride[a] = stride
            n = edges[a].size - 1
            shape.append(n)
            stride *= n
        elif d == 2 and a == 2:
            g.axis_mode[a] = _lib.AXIS_IGNORED
        else:
            g.axis_mode[a] = _lib.AXIS_RANGE
    g.time_stride = stride
    g.mode_stride = stride * Nt
    g.hist_len = g.mode_stride * nmodes
    g.shape = tuple(shape) + (Nt, nmodes)
    return g


def natural_range_covered(frame: str, d: int, axis: int, lo: float, hi: float) -> bool:
    """True when an integrated axis' [lo, hi] contains every value the coordinate can take,
    so the range check can be skipped without changing the result for finite positions."""
    if lo == -math.inf and hi == math.inf:
        return True
    if axis == 1 and frame != "cartesian":          # atan2 in [-pi, pi]
        return lo <= -math.pi and hi >= math.pi
    if axis == 2 and frame == "spherical" and d == 3:  # sin(elevation) in [-1, 1]
        return lo <= -1.0 and hi >= 1.0
    if axis == 3:
        return (lo <= -1.0 and hi >= 1.0) if d == 3 else (lo <= 0.0 and hi >= math.pi)
    return False
