"""Request serving over the batched waveform + likelihood path.

A sampler (the reference's BBHWaveformTD.get_ll, eob/seobnrv4phm.py:772-823,
called by eryn walkers) sends requests of 1..512 parameter sets and waits for
their lnL.  The server packs arriving requests into batches (whole requests
in arrival order, a request larger than a batch split over several) and runs
each batch through eob_waveform_lnl on one of a few slots.  A slot is a
workspace, a CUDA stream and pinned host buffers; slots run concurrently, so
a new batch starts while the ragged tail of the previous one (a few long
binaries on a few SMs) still runs.  The number of slots is admitted against
an HBM budget from the workspace size.

Every binary's result depends only on its own parameters (the integrator
gives each binary its own lane group, the synthesis reduces each binary's
samples in a fixed order), provided the lanes per binary are fixed: the
server pins them, so a request's lnL is bitwise the same alone or packed
with others.
"""
from __future__ import annotations

import collections
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from .pipeline import WaveformLikelihood, longest_first


@dataclass
class _Piece:
    req: int      # request index
    lo: int       # first row of the request in this batch's piece
    hi: int
    at: int       # offset of the piece in the batch


@dataclass
class _Slot:
    wl: WaveformLikelihood
    stream: torch.cuda.Stream
    params_h: torch.Tensor
    lnl_h: torch.Tensor
    status_h: torch.Tensor
    done: torch.cuda.Event = None
    start: torch.cuda.Event = None
    pieces: list = field(default_factory=list)
    n: int = 0
    launched_at: float = 0.0


def pack_batch(pending, sizes, max_batch: int):
    """Take up to max_batch rows from the pending queue of [request, next
    row] entries, in arrival order; a request that does not fit is split and
    its remainder stays at the head of the queue.  Returns the pieces."""
    pieces, n = [], 0
    while pending and n < max_batch:
        r, lo = pending[0]
        take = min(sizes[r] - lo, max_batch - n)
        pieces.append(_Piece(r, lo, lo + take, 0))
        n += take
        if lo + take == sizes[r]:
            pending.popleft()
        else:
            pending[0][1] = lo + take
    return pieces


class LikelihoodServer:
    """Continuous batching of lnL requests over `slots` concurrent workspaces.

    data: float64 [N] (shared by every request); dt [s]; amp: template
    amplitude; modes: (l, m) list; max_batch: binaries per launch."""

    def __init__(self, data, dt: float, amp: float, modes=((2, 2),), max_batch: int = 512, max_steps: int = 4000,
                 slots: int = 2, lanes_per_binary: int = 8, hbm_budget_bytes: int | None = None, device="cuda"):
        if not torch.cuda.is_available():
            raise _lib.EOBError("no CUDA device: the EOB path runs only on the GPU")
        self.device = torch.device(device)
        self.dt, self.amp = float(dt), float(amp)
        self.data = torch.as_tensor(np.ascontiguousarray(data), dtype=torch.float64).to(self.device)
        self.modes = [tuple(m) for m in modes]
        self.max_batch = int(max_batch)
        lib = _lib.load()
        ws = int(lib.eob_workspace_bytes(self.max_batch, int(max_steps), len(self.modes), int(self.data.numel())))
        if ws == 0:
            raise _lib.EOBError("invalid workspace capacities")
        if hbm_budget_bytes is not None:
            slots = min(slots, int(hbm_budget_bytes) // ws)
            if slots < 1:
                raise _lib.EOBError(f"HBM budget {hbm_budget_bytes} B is below one workspace ({ws} B)")
        self.workspace_bytes = ws
        opts = _lib.default_options()
        opts.lanes_per_binary = int(lanes_per_binary)
        self.slots = []
        for _ in range(int(slots)):
            wl = WaveformLikelihood(self.max_batch, int(max_steps), self.modes, int(self.data.numel()),
                                    device=self.device, options=opts)
            self.slots.append(_Slot(wl, torch.cuda.Stream(self.device),
                                    torch.empty((self.max_batch, 5), dtype=torch.float64).pin_memory(),
                                    torch.empty(self.max_batch, dtype=torch.float64).pin_memory(),
                                    torch.empty(self.max_batch, dtype=torch.int32).pin_memory()))

    # ------------------------------------------------------------ one batch
    def _launch(self, slot: _Slot, pieces, reqs):
        n = 0
        for p in pieces:
            k = p.hi - p.lo
            slot.params_h[n:n + k] = torch.from_numpy(reqs[p.req][p.lo:p.hi])
            p.at = n
            n += k
        slot.pieces, slot.n = pieces, n
        with torch.cuda.stream(slot.stream):
            slot.start = torch.cuda.Event(enable_timing=True)
            slot.done = torch.cuda.Event(enable_timing=True)
            slot.start.record(slot.stream)
            P = slot.params_h[:n].to(self.device, non_blocking=True)
            lnl, st = slot.wl.run(P, self.data, self.dt, self.amp, order=longest_first(P), stream=slot.stream)
            slot.lnl_h[:n].copy_(lnl, non_blocking=True)
            slot.status_h[:n].copy_(st, non_blocking=True)
            slot.done.record(slot.stream)
            # keep the device tensors alive until the copies finish
            slot._keep = (P, lnl, st)

    def evaluate(self, params: np.ndarray):
        """Synchronous lnL of one parameter array (rows of m1, m2, chi1, chi2, f0)."""
        params = np.ascontiguousarray(params, dtype=np.float64)
        out = np.empty(len(params))
        status = np.empty(len(params), dtype=np.int32)
        slot = self.slots[0]
        for lo in range(0, len(params), self.max_batch):
            hi = min(len(params), lo + self.max_batch)
            self._launch(slot, [_Piece(0, lo, hi, 0)], [params])
            slot.done.synchronize()
            out[lo:hi] = slot.lnl_h[:hi - lo].numpy()
            status[lo:hi] = slot.status_h[:hi - lo].numpy()
        return out, status

    # ------------------------------------------------------------ a trace
    def run_trace(self, arrivals, requests, time_scale: float = 1.0, idle_sleep_s: float = 50e-6):
        """Replay requests arriving at `arrivals` [s] (times time_scale) in
        wall-clock time.  Returns per-request latency [s] (completion minus
        arrival), lnL and status, and summary statistics."""
        arrivals = np.asarray(arrivals, dtype=np.float64) * time_scale
        reqs = [np.ascontiguousarray(r, dtype=np.float64) for r in requests]
        nreq = len(reqs)
        lnl = [np.full(len(r), np.nan) for r in reqs]
        status = [np.full(len(r), -1, dtype=np.int32) for r in reqs]
        remaining = np.array([len(r) for r in reqs])
        done_at = np.full(nreq, np.nan)
        pending = collections.deque()   # (request, next row)
        free = list(range(len(self.slots)))
        busy = []
        nxt = 0
        ndone = 0
        gpu_ms = 0.0
        batches = 0
        t0 = time.perf_counter()
        while ndone < nreq:
            now = time.perf_counter() - t0
            progressed = False
            while nxt < nreq and arrivals[nxt] <= now:
                if len(reqs[nxt]) == 0:
                    done_at[nxt] = now
                    ndone += 1
                else:
                    pending.append([nxt, 0])
                nxt += 1
                progressed = True
            # completions
            for si in list(busy):
                s = self.slots[si]
                if not s.done.query():
                    continue
                tnow = time.perf_counter() - t0
                gpu_ms += s.start.elapsed_time(s.done)
                for p in s.pieces:
                    k = p.hi - p.lo
                    lnl[p.req][p.lo:p.hi] = s.lnl_h[p.at:p.at + k].numpy()
                    status[p.req][p.lo:p.hi] = s.status_h[p.at:p.at + k].numpy()
                    remaining[p.req] -= k
                    if remaining[p.req] == 0:
                        done_at[p.req] = tnow
                        ndone += 1
                busy.remove(si)
                free.append(si)
                progressed = True
            # launches: fill free slots from the pending requests in arrival order
            while free and pending:
                si = free.pop(0)
                pieces = pack_batch(pending, [len(r) for r in reqs], self.max_batch)
                self._launch(self.slots[si], pieces, reqs)
                busy.append(si)
                batches += 1
                progressed = True
            if not progressed:
                time.sleep(idle_sleep_s)
        wall = time.perf_counter() - t0
        lat = done_at - arrivals
        nbin = int(sum(len(r) for r in reqs))
        return {"latency_s": lat, "lnl": lnl, "status": status,
                "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
                "wall_s": wall, "binaries": nbin, "evals_per_s": nbin / wall, "batches": batches,
                "slot_busy_fraction": gpu_ms / 1e3 / wall / len(self.slots)}


def calibrate_rate(server: LikelihoodServer, requests, busy: float = 0.7, n: int = 16) -> float:
    """Poisson rate [requests/s] at which the server is `busy` loaded: the
    mean service time of `n` requests run one at a time, then rate = busy /
    mean time."""
    server.evaluate(requests[0])  # warm-up
    t = []
    for r in requests[:n]:
        t0 = time.perf_counter()
        server.evaluate(r)
        t.append(time.perf_counter() - t0)
    return busy / float(np.mean(t))
