"""Request serving over the batched waveform + likelihood path.

A sampler (the reference's BBHWaveformTD.get_ll, eob/seobnrv4phm.py:772-823,
called by eryn walkers) sends requests of 1..512 parameter sets and waits for
their lnL.  The server runs continuous batching over a few *slots*; a slot is
a workspace, a CUDA stream and pinned host buffers, and slots run
concurrently, so a new batch starts while the ragged tail of another (a few
long binaries on a few SMs) still runs.

Admission follows the HBM footprint of the estimated trajectories.  Slots
come in classes by trajectory capacity (rows per binary): every binary is
routed to the smallest class whose capacity covers its estimated row count
(`estimate_rows`, a fit to the Newtonian chirp time with a safety factor),
so short binaries hold short workspaces.  A binary that still outgrows its
class (status EOB_ST_MAXSTEP) is re-queued to the next class.  The number of
slots of each class is admitted against an HBM budget from the workspace
sizes.  Within a class, batches take binaries in arrival order.

Every binary's result depends only on its own parameters (the integrator
gives each binary its own lane group, the synthesis reduces each binary's
samples in a fixed order), provided the lanes per binary are fixed and its
trajectory fits: the server pins the lanes, so a request's lnL is bitwise the
same alone, packed with others, or in another class.
"""
from __future__ import annotations

import collections
import math
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from .pipeline import WaveformLikelihood, longest_first

MTSUN_SI = 4.925491025543576e-06
EOB_ST_MAXSTEP = 2


def estimate_rows(params: np.ndarray, safety: float = 3.0) -> np.ndarray:
    """Estimated trajectory rows per binary (both passes): a fit of the rows
    of 1024 configuration-2 binaries to the Newtonian chirp time t_c [M] and
    the effective spin, rows ~ 200 + 2.0 t_c^0.536 e^{0.40 chi}, times
    `safety` (the fit's largest under-estimate is 3x)."""
    p = np.atleast_2d(np.asarray(params, dtype=np.float64))
    m1, m2, c1, c2, f0 = p[:, 0], p[:, 1], p[:, 2], p[:, 3], p[:, 4]
    M = m1 + m2
    eta = m1 * m2 / (M * M)
    x = math.pi * M * MTSUN_SI * f0
    tc = (5.0 / 256.0) / eta * x ** (-8.0 / 3.0)
    chi = (c1 * m1 + c2 * m2) / M
    return np.ceil(safety * (200.0 + 2.0 * tc ** 0.536 * np.exp(0.40 * chi))).astype(np.int64)


@dataclass
class _Piece:
    req: int            # request index
    idx: np.ndarray     # rows of the request in this piece
    at: int = 0         # offset of the piece in the batch


@dataclass
class _Slot:
    cls: int
    wl: WaveformLikelihood
    stream: torch.cuda.Stream
    params_h: torch.Tensor
    lnl_h: torch.Tensor
    status_h: torch.Tensor
    done: torch.cuda.Event = None
    start: torch.cuda.Event = None
    pieces: list = field(default_factory=list)
    n: int = 0


def pack_batch(pending, max_batch: int):
    """Take up to max_batch rows from a pending queue of [request, row
    indices, next position] entries, in arrival order; a request that does
    not fit is split and its remainder stays at the head.  Returns pieces."""
    pieces, n = [], 0
    while pending and n < max_batch:
        r, rows, pos = pending[0]
        take = min(len(rows) - pos, max_batch - n)
        pieces.append(_Piece(r, rows[pos:pos + take]))
        n += take
        if pos + take == len(rows):
            pending.popleft()
        else:
            pending[0][2] = pos + take
    return pieces


def route(est_rows: np.ndarray, capacities) -> np.ndarray:
    """Class of each binary: the smallest capacity that covers its estimate
    (the largest class for anything longer)."""
    caps = np.asarray(capacities)
    c = np.searchsorted(caps, est_rows, side="left")
    return np.minimum(c, len(caps) - 1)


def admit_slots(ws_bytes, counts, budget):
    """Slots per class within an HBM budget: drop slots from the largest
    classes first, keeping at least one per class."""
    counts = list(counts)
    if sum(ws_bytes) > budget:
        raise _lib.EOBError(f"HBM budget {budget} B is below one slot per class ({sum(ws_bytes)} B)")
    k = len(counts) - 1
    while sum(w * c for w, c in zip(ws_bytes, counts)) > budget:
        while counts[k] <= 1:
            k = (k - 1) % len(counts)
        counts[k] -= 1
        k = (k - 1) % len(counts)
    return counts


class LikelihoodServer:
    """Continuous batching of lnL requests.

    data: float64 [N] (shared by every request); dt [s]; amp: template
    amplitude; modes: (l, m) list.  classes: list of (max_steps, max_batch,
    slots), by trajectory capacity; default one class (max_steps, max_batch,
    slots).  hbm_budget_bytes caps the workspaces held (slots are dropped
    from the largest classes first, at least one per class remains);
    row_safety multiplies the trajectory-length estimate used for routing;
    precision 1 selects the mixed-precision synthesis."""

    def __init__(self, data, dt: float, amp: float, modes=((2, 2),), max_batch: int = 512, max_steps: int = 4000,
                 slots: int = 2, lanes_per_binary: int = 8, hbm_budget_bytes: int | None = None, classes=None,
                 row_safety: float = 3.0, precision: int = 0, head_quads: int = -1, device="cuda"):
        if not torch.cuda.is_available():
            raise _lib.EOBError("no CUDA device: the EOB path runs only on the GPU")
        self.device = torch.device(device)
        self.dt, self.amp = float(dt), float(amp)
        self.data = torch.as_tensor(np.ascontiguousarray(data), dtype=torch.float64).to(self.device)
        self.modes = [tuple(m) for m in modes]
        N = int(self.data.numel())
        lib = _lib.load()
        if classes is None:
            classes = [(max_steps, max_batch, slots)]
        classes = sorted([(int(a), int(b), int(c)) for a, b, c in classes])
        ws = [int(lib.eob_workspace_bytes(b, L, len(self.modes), N)) for L, b, _ in classes]
        if any(w == 0 for w in ws):
            raise _lib.EOBError("invalid workspace capacities")
        counts = [c for _, _, c in classes]
        if hbm_budget_bytes is not None:
            counts = admit_slots(ws, counts, int(hbm_budget_bytes))
        self.row_safety = float(row_safety)
        self.capacities = [L for L, _, _ in classes]
        self.class_batch = [b for _, b, _ in classes]
        self.class_slots = counts
        self.workspace_bytes = sum(w * c for w, c in zip(ws, counts))
        opts = _lib.default_options()
        opts.lanes_per_binary = int(lanes_per_binary)
        opts.precision = int(precision)
        opts.head_quads = int(head_quads)
        self.slots = []
        for ci, ((L, b, _), cnt) in enumerate(zip(classes, counts)):
            for _ in range(cnt):
                wl = WaveformLikelihood(b, L, self.modes, N, device=self.device, options=opts)
                self.slots.append(_Slot(ci, wl, torch.cuda.Stream(self.device),
                                        torch.empty((b, 5), dtype=torch.float64).pin_memory(),
                                        torch.empty(b, dtype=torch.float64).pin_memory(),
                                        torch.empty(b, dtype=torch.int32).pin_memory()))

    # ------------------------------------------------------------ one batch
    def _launch(self, slot: _Slot, pieces, reqs):
        n = 0
        for p in pieces:
            k = len(p.idx)
            slot.params_h[n:n + k] = torch.from_numpy(reqs[p.req][p.idx])
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
            slot._keep = (P, lnl, st)  # device tensors live until the copies finish

    def evaluate(self, params: np.ndarray):
        """Synchronous lnL of one parameter array (rows of m1, m2, chi1, chi2, f0)."""
        res = self.run_trace(np.zeros(1), [np.ascontiguousarray(params, dtype=np.float64)])
        return res["lnl"][0], res["status"][0]

    # ------------------------------------------------------------ a trace
    def run_trace(self, arrivals, requests, time_scale: float = 1.0, idle_sleep_s: float = 50e-6):
        """Replay requests arriving at `arrivals` [s] (times time_scale) in
        wall-clock time.  Returns per-request latency [s] (completion minus
        arrival), lnL and status, and summary statistics."""
        arrivals = np.asarray(arrivals, dtype=np.float64) * time_scale
        reqs = [np.ascontiguousarray(np.atleast_2d(r), dtype=np.float64).reshape(-1, 5) for r in requests]
        nreq = len(reqs)
        ncls = len(self.capacities)
        lnl = [np.full(len(r), np.nan) for r in reqs]
        status = [np.full(len(r), -1, dtype=np.int32) for r in reqs]
        remaining = np.array([len(r) for r in reqs])
        done_at = np.full(nreq, np.nan)
        pending = [collections.deque() for _ in range(ncls)]  # per class: [request, rows, next]
        free = list(range(len(self.slots)))
        busy = []
        nxt = ndone = batches = requeued = 0
        gpu_ms = 0.0
        t0 = time.perf_counter()
        while ndone < nreq:
            now = time.perf_counter() - t0
            progressed = False
            while nxt < nreq and arrivals[nxt] <= now:
                if len(reqs[nxt]) == 0:
                    done_at[nxt] = now
                    ndone += 1
                else:
                    cls = route(estimate_rows(reqs[nxt], self.row_safety), self.capacities)
                    for c in range(ncls):
                        rows = np.nonzero(cls == c)[0]
                        if len(rows):
                            pending[c].append([nxt, rows, 0])
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
                    k = len(p.idx)
                    got_l = s.lnl_h[p.at:p.at + k].numpy()
                    got_s = s.status_h[p.at:p.at + k].numpy()
                    over = (got_s & EOB_ST_MAXSTEP) != 0
                    if s.cls + 1 < ncls and np.any(over):
                        # outgrew its class: run it again with the next capacity
                        pending[s.cls + 1].append([p.req, p.idx[over], 0])
                        requeued += int(over.sum())
                        keep = ~over
                    else:
                        keep = np.ones(k, dtype=bool)
                    lnl[p.req][p.idx[keep]] = got_l[keep]
                    status[p.req][p.idx[keep]] = got_s[keep]
                    remaining[p.req] -= int(keep.sum())
                    if remaining[p.req] == 0:
                        done_at[p.req] = tnow
                        ndone += 1
                busy.remove(si)
                free.append(si)
                progressed = True
            # launches: each free slot takes the oldest pending binaries of its class
            for si in list(free):
                c = self.slots[si].cls
                if not pending[c]:
                    continue
                pieces = pack_batch(pending[c], self.class_batch[c])
                free.remove(si)
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
                "requeued": requeued, "slot_busy_fraction": gpu_ms / 1e3 / wall / len(self.slots)}


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
