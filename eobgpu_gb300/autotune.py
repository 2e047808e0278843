"""Launch-parameter autotuner for the fused path.

The integrator's best lanes per binary depends on the batch: one lane per
binary is the most efficient use of the FP64 pipe when the batch fills the
device, many lanes per binary shorten the longest binary's chain when it does
not (configuration 2 is bound by its longest binary, configuration 3 by its
total work).  The block size of the integrator and the spline kernel's
series per block are secondary.  `tune()` times candidate settings on the
caller's batch (or a sample of the same shape) with CUDA events and returns
the fastest as eob_options; results are cached per batch signature, in
memory and optionally in a JSON file.
"""
from __future__ import annotations

import json
import os
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .pipeline import WaveformLikelihood, chirp_duration_M, longest_first

_CACHE: dict = {}


def signature(params: torch.Tensor, n_modes: int, n_samples: int, max_steps: int) -> str:
    """Batch size, modes, samples, capacity and the spread of chirp times
    (log2 buckets of the median and maximum), which set the best launch."""
    tc = chirp_duration_M(params).double().cpu().numpy()
    med = int(np.round(np.log2(max(np.median(tc), 1.0))))
    mx = int(np.round(np.log2(max(np.max(tc), 1.0))))
    B = int(params.shape[0])
    return f"B{1 << int(np.ceil(np.log2(max(B, 1))))}_K{n_modes}_N{n_samples}_L{max_steps}_t{med}_{mx}"


@dataclass
class TuneResult:
    lanes_per_binary: int
    block: int
    spline_series_per_block: int
    ms: float
    table: list
    head_quads: int = -1

    def options(self, base: _lib.EobOptions | None = None) -> _lib.EobOptions:
        o = _lib.default_options() if base is None else base
        o.lanes_per_binary = self.lanes_per_binary
        o.block = self.block
        o.spline_tile = self.spline_series_per_block
        o.head_quads = self.head_quads
        return o


def _time(wl, P, D, dt, amp, order, reps):
    wl.run(P, D, dt, amp, order=order)  # warm-up (and first-touch of the workspace)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ev[0].record()
    for _ in range(reps):
        wl.run(P, D, dt, amp, order=order)
    ev[1].record()
    torch.cuda.synchronize()
    return ev[0].elapsed_time(ev[1]) / reps


def tune(params: torch.Tensor, data: torch.Tensor, dt: float, amp: float, modes=((2, 2),), max_steps: int = 6000,
         lanes=(1, 2, 4, 8, 16, 32, 64, 128), blocks=(64, 128, 256), spline_tiles=(1, 4), heads=(16, 32, 64),
         reps: int = 1, cache_file: str | None = None, base: _lib.EobOptions | None = None) -> TuneResult:
    """Time every candidate on this batch and return the fastest.  The lanes
    per binary are searched first (block 128, the library's head choice),
    then a head of the longest binaries on four warps beside groups of 8..64
    lanes near the best count; the block size only for the best lane count
    (without a head); the spline tile last."""
    key = signature(params, len(modes), int(data.shape[0]), max_steps)
    if key in _CACHE:
        return _CACHE[key]
    if cache_file and os.path.exists(cache_file):
        with open(cache_file) as f:
            disk = json.load(f)
        if key in disk:
            r = TuneResult(**disk[key])
            _CACHE[key] = r
            return r
    B = int(params.shape[0])
    order = longest_first(params)
    table = []

    def run(g, bs, tile, head=-1):
        o = _lib.default_options() if base is None else base
        o.lanes_per_binary, o.block, o.spline_tile, o.head_quads = g, bs, tile, head
        wl = WaveformLikelihood(B, max_steps, list(modes), int(data.shape[0]), device=params.device, options=o)
        ms = _time(wl, params, data, dt, amp, order, reps)
        table.append({"lanes_per_binary": g, "block": bs, "spline_series_per_block": tile, "head_quads": head,
                      "ms": ms})
        del wl
        return ms

    best_g = min(lanes, key=lambda g: run(g, 128, spline_tiles[0]))
    best_head = -1
    best_ms = min(e["ms"] for e in table if e["lanes_per_binary"] == best_g)
    for g in sorted({g for g in (best_g // 2, best_g, best_g * 2, 64) if g in (8, 16, 32, 64)}):
        for h in heads:
            if h >= B:
                continue
            ms = run(g, 128, spline_tiles[0], h)
            if ms < best_ms:
                best_ms, best_g, best_head = ms, g, h
    if best_head == -1:
        best_bs = min(blocks, key=lambda bs: run(best_g, bs, spline_tiles[0]) if bs != 128 else
                      min(t["ms"] for t in table if t["lanes_per_binary"] == best_g and t["block"] == 128
                          and t["head_quads"] == -1))
    else:
        best_bs = 128  # the launch with a head has its own block shape
    best_tile = min(spline_tiles, key=lambda t: run(best_g, best_bs, t, best_head) if t != spline_tiles[0] else
                    min(e["ms"] for e in table if e["lanes_per_binary"] == best_g and e["block"] == best_bs
                        and e["head_quads"] == best_head))
    ms = min(e["ms"] for e in table if e["lanes_per_binary"] == best_g and e["block"] == best_bs
             and e["spline_series_per_block"] == best_tile and e["head_quads"] == best_head)
    r = TuneResult(best_g, best_bs, best_tile, ms, table, best_head)
    _CACHE[key] = r
    if cache_file:
        disk = {}
        if os.path.exists(cache_file):
            with open(cache_file) as f:
                disk = json.load(f)
        disk[key] = r.__dict__
        os.makedirs(os.path.dirname(os.path.abspath(cache_file)), exist_ok=True)
        with open(cache_file, "w") as f:
            json.dump(disk, f, indent=1)
    return r
