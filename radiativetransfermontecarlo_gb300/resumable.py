"""Checkpoint and resume for radiativeTransfer.

The reference has no checkpoint: its packet loop (radiativeTransfer.m:58-92) runs to the
end or is lost.  Here a run is cut into chunks of particle ids and a snapshot is written
after each chunk: the problem's fingerprint, the next particle id, the partial fixed-point
histogram (unsigned 64-bit, as the device accumulates it) and the event counters.  A particle's trajectory depends only on
(seed, particle id) (Philox keyed by the particle id and its event index) and integer
histograms add exactly, so a run that stops (killed, or after `max_chunks`) and resumes
from its snapshot returns the histogram of an uninterrupted run bit for bit.

A snapshot is two files written side by side and moved into place (`os.replace`), the
histogram first: `<path>.hist` (raw uint64) and `<path>` (JSON: fingerprint, next id,
counters, the histogram's length and checksum).  A snapshot whose fingerprint, length or
checksum does not match is refused with an error rather than silently restarted.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os

import numpy as np

from . import _lib
from .radiative_transfer import DEFAULT_OPTIONS, build_problem, get_context, normalise

SNAPSHOT_VERSION = 1
COUNTERS = ("scatter_events", "boundary_hits", "kills", "absorbed", "observations", "conversions")
_POINTERS = {"axis_edges", "src_radial_cdf", "src_radial_r"}


def problem_fingerprint(prob) -> str:
    """SHA-256 over everything that decides the run's histogram: the rtmc_problem fields
    (the whole particle range included) other than pointers, the arrays those pointers
    reach, and the knots of the tables."""
    P, keep = prob.to_ctypes()
    h = hashlib.sha256()
    base = C.addressof(P)
    for name, _ in _lib.RtmcProblem._fields_:
        if name in _POINTERS:
            continue
        fd = getattr(_lib.RtmcProblem, name)
        h.update(name.encode())
        h.update(C.string_at(base + fd.offset, fd.size))
    for a in keep:
        h.update(np.ascontiguousarray(a).tobytes())
    inf = prob.tables.info()
    for t in range(inf.n_tables):
        c, th = prob.tables.knots(t)
        h.update(c.tobytes())
        h.update(th.tobytes())
    return h.hexdigest()


def narrow_u32(hist: np.ndarray, hist_shift: int) -> np.ndarray:
    """The reference's uint32 counts from the 64-bit fixed-point histogram: (hist >>
    hist_shift) saturated at 2^32 - 1, as rt_narrow_u32 narrows on the device."""
    c = hist.view(np.uint64) >> np.uint64(hist_shift)
    return np.minimum(c, np.uint64(0xFFFFFFFF)).astype(np.uint32)


def _checksum(hist: np.ndarray) -> str:
    return hashlib.sha256(hist.view(np.uint8)).hexdigest()


def load_snapshot(path: str, fingerprint: str, hist_len: int):
    """(next particle offset, uint64 histogram, counters) from the snapshot at path, or
    None when there is none.  Raises ValueError when it belongs to another problem or is
    damaged."""
    if not os.path.exists(path):
        return None
    with open(path) as f:
        meta = json.load(f)
    if meta.get("version") != SNAPSHOT_VERSION:
        raise ValueError(f"checkpoint {path}: unknown snapshot version {meta.get('version')}")
    if meta.get("fingerprint") != fingerprint:
        raise ValueError(f"checkpoint {path} belongs to another problem (fingerprint differs)")
    if meta.get("hist_len") != hist_len:
        raise ValueError(f"checkpoint {path}: histogram length {meta.get('hist_len')} != {hist_len}")
    hist = np.fromfile(path + ".hist", dtype=np.uint64)
    if hist.size != hist_len or _checksum(hist) != meta.get("checksum"):
        raise ValueError(f"checkpoint {path}: histogram file is damaged")
    return int(meta["next"]), hist, {k: int(meta["counters"][k]) for k in COUNTERS}


def save_snapshot(path: str, fingerprint: str, next_offset: int, hist: np.ndarray, counters: dict):
    """Writes the snapshot: the histogram file, then the metadata that names its checksum,
    each moved into place whole."""
    tmp = path + ".hist.tmp"
    hist.tofile(tmp)
    os.replace(tmp, path + ".hist")
    meta = {"version": SNAPSHOT_VERSION, "fingerprint": fingerprint, "next": int(next_offset),
            "hist_len": int(hist.size), "checksum": _checksum(hist), "counters": {k: int(counters[k]) for k in COUNTERS}}
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(meta, f)
    os.replace(tmp, path)


def radiative_transfer_resumable(geometry: dict, source: dict, material, observation: dict,
                                 options: dict | None = None, *, checkpoint: str, chunk: int = 10_000_000,
                                 max_chunks: int | None = None):
    """radiativeTransfer(geometry, source, material, observation, options) run in chunks of
    `chunk` particles with a snapshot at `checkpoint` after each.  An existing snapshot of
    the same problem is resumed.  With max_chunks, at most that many chunks run in this call
    and None is returned while particles remain; the finished call returns obs as
    radiativeTransfer does (plus obs['stats'] summed over the chunks) and leaves the final
    snapshot in place."""
    if chunk < 1:
        raise ValueError("chunk must be at least 1 particle")
    opt = dict(DEFAULT_OPTIONS)
    opt.update(options or {})
    prob, grid, N = build_problem(geometry, source, material, observation, opt)
    fp = problem_fingerprint(prob)
    state = load_snapshot(checkpoint, fp, prob.hist_len)
    if state is None:
        offset, hist, counters = 0, np.zeros(prob.hist_len, dtype=np.uint64), dict.fromkeys(COUNTERS, 0)
    else:
        offset, hist, counters = state
    ctx = get_context(int(opt["device"]))
    done = 0
    while offset < prob.n_particles:
        if max_chunks is not None and done >= max_chunks:
            return None
        P, keep = prob.to_ctypes()
        n = min(chunk, prob.n_particles - offset)
        P.pid0 = prob.pid0 + offset
        P.n_particles = n
        part, st = ctx.forward(P, prob.tables)
        del keep
        hist += part.view(np.uint64)  # below 2^64: the host checks n_particles << hist_shift
        for k in COUNTERS:
            counters[k] += int(st[k])
        offset += n
        save_snapshot(checkpoint, fp, offset, hist, counters)
        done += 1
    obs = dict(grid.obs)
    if opt["return_counts"]:
        if hist.size and int(hist.max()) >= 1 << 63:  # as rtmc_forward refuses it
            raise _lib.RtmcError("a histogram bin reached 2^63 and does not fit int64 at this hist_shift")
        E = hist.view(np.int64)
        obs["energyDensity"], obs["energy"] = normalise(E, grid, N, prob.hist_shift)
        obs["E"] = E.reshape(grid.shape, order="F")
    else:
        # the reference's uint32 E, as rtmc_forward_u32 returns it
        obs["energyDensity"], obs["energy"] = normalise(narrow_u32(hist, prob.hist_shift), grid, N, 0)
    obs["stats"] = dict(counters, particles=int(offset), chunks_this_call=done)
    return obs
