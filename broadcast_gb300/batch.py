"""Residual (+ one tangent direction) of many independent grids of uneven size
in one set of persistent launches, optionally replayed from a CUDA graph
(C ABI: bcg_batch_*), and the autotuner that picks its tile shapes.

    gb = GridBatch([grid dicts], [phys dicts], ndir=1)
    gb.set_states(ws, wds)              # torch tensors, operator layout (5, nj, ni)
    gb.run(use_graph=True)              # queued on torch's current stream
    gb.res[g], gb.resd[g]               # residual / tangent of grid g
    gb.run_host(ws_h, wds_h, res_h, resd_h, geo_h)  # host arrays, copies overlapped
    gb.autotune()                       # times the tile candidates, keeps the best
    gb.autotune_host(ws_h, wds_h, res_h, resd_h, geo_h)   # the same for the host-run chunks

The autotuner measures every candidate on the plan's own grids with CUDA
events and caches the winner per batch signature in a JSON file
(BCG_AUTOTUNE_CACHE, default broadcast_gb300/_lib/autotune.json).
"""
import hashlib
import json
import os

import numpy as np

from . import _lib
from .operator import to_device

PHYS_KEYS = ("cp", "cv", "prandtl", "gam", "rgaz", "cs", "muref", "tref", "s_suth", "k2", "k4")
CANDIDATES = [(tf, tc, ctas) for tf in (64, 128, 256) for tc in (128, 256) for ctas in (1, 2, 3, 4)
              if tf * ctas <= 1024]
DEFAULT_CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "autotune.json")


def _u64(ptrs):
    return np.asarray(ptrs, dtype=np.uint64)


class GridBatch:
    def __init__(self, grids, phys, ndir=1, device="cuda"):
        import torch
        _lib.load()
        if len(grids) != len(phys) or not grids:
            raise ValueError("one phys dictionary per grid")
        self.ndir = int(ndir)
        self.device = device
        self.n = len(grids)
        self.im = np.array([int(g["im"]) for g in grids], dtype=np.int32)
        self.jm = np.array([int(g["jm"]) for g in grids], dtype=np.int32)
        ph = np.ascontiguousarray([[float(p[k]) for k in PHYS_KEYS] for p in phys], dtype=np.float64)
        h = np.zeros(1, np.int64)
        _lib.call("bcg_set_stream", torch.cuda.current_stream().cuda_stream)
        _lib.call("bcg_batch_create", self.n, self.im, self.jm, ph, self.ndir, h)
        self.plan = int(h[0])
        self.geo = [{k: to_device(g[k], device) for k in ("nx", "ny", "vol", "volf")} for g in grids]
        shp = [(5, int(j) + 6, int(i) + 6) for i, j in zip(self.im, self.jm)]
        self.res = [torch.zeros(s, dtype=torch.float64, device=device) for s in shp]
        self.resd = [torch.zeros(s, dtype=torch.float64, device=device) for s in shp] if self.ndir else None
        self.ws = self.wds = None
        self.config = None
        self.host_config = None

    def __del__(self):
        try:
            if getattr(self, "plan", None):
                _lib.call("bcg_batch_destroy", self.plan)
                self.plan = None
        except Exception:
            pass

    @property
    def cells(self):
        return int((self.im.astype(np.int64) * self.jm).sum())

    def device_bytes(self):
        b = np.zeros(1, np.int64)
        _lib.call("bcg_batch_device_bytes", self.plan, b)
        return int(b[0])

    def set_states(self, ws, wds=None):
        """ws (and wds): lists of device tensors in the operator layout."""
        self.ws, self.wds = list(ws), (list(wds) if wds is not None else None)
        ptr = lambda ts: _u64([t.data_ptr() for t in ts])
        wd = ptr(self.wds) if self.ndir else ptr(self.ws)
        rd = ptr(self.resd) if self.ndir else ptr(self.res)
        _lib.call("bcg_batch_set_arrays", self.plan, ptr(self.ws), wd, ptr([g["nx"] for g in self.geo]),
                  ptr([g["ny"] for g in self.geo]), ptr([g["vol"] for g in self.geo]),
                  ptr([g["volf"] for g in self.geo]), ptr(self.res), rd)

    def configure(self, tile_faces, tile_cells, ctas_per_sm):
        _lib.call("bcg_batch_configure", self.plan, int(tile_faces), int(tile_cells), int(ctas_per_sm))
        self.config = (int(tile_faces), int(tile_cells), int(ctas_per_sm))

    def configure_host(self, tile_faces, tile_cells, ctas_per_sm):
        """Tile shapes of the host-run chunks alone (bcg_batch_configure_host)."""
        _lib.call("bcg_batch_configure_host", self.plan, int(tile_faces), int(tile_cells), int(ctas_per_sm))
        self.host_config = (int(tile_faces), int(tile_cells), int(ctas_per_sm))

    def autotune_host(self, ws, wds, res, resd, geo, nchunk=16, candidates=CANDIDATES, repeats=3):
        """Time run_host (wall clock, copies included) with each candidate tile
        shape for the chunks and keep the fastest; the whole batch's own shapes
        (configure / autotune) stay as they are."""
        import time
        timings = []
        for cand in candidates:
            self.configure_host(*cand)
            self.run_host(ws, wds, res, resd, geo, nchunk=nchunk)
            t0 = time.perf_counter()
            for _ in range(repeats):
                self.run_host(ws, wds, res, resd, geo, nchunk=nchunk)
            timings.append(((time.perf_counter() - t0) / repeats * 1e3, cand))
        best_ms, best = min(timings)
        self.configure_host(*best)
        return {"config": list(best), "ms": best_ms, "nchunk": int(nchunk),
                "timings": [[list(c), t] for t, c in timings]}

    def run(self, use_graph=True):
        _lib.call("bcg_batch_run", self.plan, 1 if use_graph else 0)

    def run_pass(self, k):
        """Queue pass k (0 primitives .. 4 faces, 5 balance) alone, for timing."""
        _lib.call("bcg_batch_run_pass", self.plan, int(k))

    def run_host(self, ws, wds, res, resd, geo, nchunk=8):
        """One evaluation with host arrays (bcg_batch_run_host): lists of
        Fortran-ordered float64 numpy arrays per grid (pinned memory copies
        fastest); geo is a list of dicts with nx, ny, vol, volf.  The grids'
        uploads, graph replays and interior downloads overlap in nchunk
        chunks; returns when res / resd hold the results."""
        addr = lambda arrs: _u64([a.ctypes.data for a in arrs])
        for a in list(ws) + list(res) + ([] if not self.ndir else list(wds) + list(resd)):
            if not (a.flags.f_contiguous and a.dtype == np.float64):
                raise ValueError("run_host: Fortran-ordered float64 arrays expected")
        wd = addr(wds) if self.ndir else addr(ws)
        rd = addr(resd) if self.ndir else addr(res)
        _lib.call("bcg_batch_run_host", self.plan, int(nchunk), addr(ws), wd, addr([g["nx"] for g in geo]),
                  addr([g["ny"] for g in geo]), addr([g["vol"] for g in geo]), addr([g["volf"] for g in geo]),
                  addr(res), rd)

    def signature(self):
        key = "%d|%s" % (self.ndir, ",".join("%dx%d" % (i, j) for i, j in zip(self.im, self.jm)))
        return hashlib.sha1(key.encode()).hexdigest()[:16]

    def autotune(self, candidates=CANDIDATES, repeats=5, cache=None, use_cache=True):
        """Time each (tile_faces, tile_cells, ctas_per_sm) candidate, keep the fastest."""
        import torch
        cache = cache or os.environ.get("BCG_AUTOTUNE_CACHE", DEFAULT_CACHE)
        sig = self.signature()
        table = {}
        if use_cache and os.path.exists(cache):
            try:
                table = json.load(open(cache))
            except ValueError:
                table = {}
        if use_cache and sig in table:
            self.configure(*table[sig]["config"])
            return table[sig]
        stream = torch.cuda.current_stream()
        timings = []
        for cand in candidates:
            self.configure(*cand)
            self.run(use_graph=False)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(repeats):
                self.run(use_graph=False)
            b.record(stream)
            b.synchronize()
            timings.append((a.elapsed_time(b) / repeats, cand))
        best_ms, best = min(timings)
        self.configure(*best)
        entry = {"config": list(best), "ms": best_ms, "cells": self.cells, "ndir": self.ndir,
                 "timings": [[list(c), t] for t, c in timings]}
        table[sig] = entry
        try:
            os.makedirs(os.path.dirname(cache), exist_ok=True)
            tmp = cache + ".tmp%d" % os.getpid()
            json.dump(table, open(tmp, "w"), indent=1)
            os.replace(tmp, cache)
        except OSError:
            pass
        return entry
