"""Host side of the fused EOB waveform + likelihood path.

`WaveformLikelihood` owns one device workspace (a torch uint8 tensor sized by
eob_workspace_bytes) and runs, on one CUDA stream and with no host
synchronisation, the five stages of the native path:

  setup (tables + initial conditions) -> persistent DOPR853 integrator ->
  multipoles on the trajectory -> not-a-knot splines -> synthesis + lnL.

Inputs and outputs are torch CUDA tensors; the C ABI sees raw pointers.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _lib

MTSUN_SI = 4.925491025543576e-06


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream_handle(stream):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def chirp_duration_M(params: torch.Tensor) -> torch.Tensor:
    """Newtonian time to coalescence from f0, in units of the total mass
    (5/256 eta^-1 (pi M f0)^(-8/3)); a cost estimate for ordering the queue."""
    m1, m2, f0 = params[:, 0], params[:, 1], params[:, 4]
    M = m1 + m2
    eta = m1 * m2 / (M * M)
    x = math.pi * M * MTSUN_SI * f0
    return (5.0 / 256.0) / eta * x.pow(-8.0 / 3.0)


def longest_first(params: torch.Tensor) -> torch.Tensor:
    """Queue order for the persistent integrator: longest estimated trajectory first."""
    return torch.argsort(chirp_duration_M(params), descending=True).to(torch.int32)


class WaveformLikelihood:
    """Batched SEOBNR aligned-spin waveform + white-noise likelihood on one GPU.

    max_batch   binaries per call
    max_steps   trajectory rows per binary (the reference's max_step, raised)
    modes       list of (l, m), subset of [(2,2), (2,1), (3,3), (4,4), (5,5)]
    max_samples samples of the data / uniform time grid
    """

    def __init__(self, max_batch: int, max_steps: int = 20000, modes=((2, 2),), max_samples: int = 8192,
                 device="cuda", options: _lib.EobOptions | None = None):
        if not torch.cuda.is_available():
            raise _lib.EOBError("no CUDA device: the EOB path runs only on the GPU")
        self.lib = _lib.load()
        self.device = torch.device(device)
        self.max_batch, self.max_steps, self.max_samples = int(max_batch), int(max_steps), int(max_samples)
        self.modes = [tuple(m) for m in modes]
        self.max_modes = max(1, len(self.modes))
        self.options = options if options is not None else _lib.default_options()
        # options.imr: the workspace carries the merger-ringdown section
        size = self.lib.eob_workspace_bytes_imr if self.options.imr else self.lib.eob_workspace_bytes
        nbytes = size(self.max_batch, self.max_steps, self.max_modes, self.max_samples)
        if nbytes == 0:
            raise _lib.EOBError("invalid workspace capacities")
        self.ws_bytes = int(nbytes)
        self.ws = torch.empty(self.ws_bytes, dtype=torch.uint8, device=self.device)
        self.ells = (ctypes.c_int * 5)(*[l for l, _ in self.modes])
        self.mms = (ctypes.c_int * 5)(*[m for _, m in self.modes])
        self.last_B = 0

    def capture(self, params: torch.Tensor, data: torch.Tensor, dt: float, amp: float) -> "CapturedLikelihood":
        """The fused lnL path on these (static) tensors as a replayable CUDA graph."""
        return CapturedLikelihood(self, params, data, dt, amp)

    def set_modes(self, modes):
        """Modes of the following calls (at most max_modes of them)."""
        modes = [tuple(int(v) for v in m) for m in modes]
        if not 1 <= len(modes) <= self.max_modes:
            raise _lib.EOBError(f"{len(modes)} modes for a workspace of {self.max_modes}")
        self.modes = modes
        self.ells = (ctypes.c_int * 5)(*[l for l, _ in modes])
        self.mms = (ctypes.c_int * 5)(*[m for _, m in modes])

    def run(self, params: torch.Tensor, data: torch.Tensor, dt: float, amp: float, order: torch.Tensor | None = None,
            lnl: torch.Tensor | None = None, status: torch.Tensor | None = None, stream=None):
        """lnL for every binary of params[B, 5] (m1, m2 [Msun], chi1, chi2, f0 [Hz])."""
        B = int(params.shape[0])
        assert params.is_cuda and params.dtype == torch.float64 and params.is_contiguous()
        assert data.is_cuda and data.dtype == torch.float64 and data.is_contiguous()
        N = int(data.shape[0])
        if lnl is None:
            lnl = torch.empty(B, dtype=torch.float64, device=self.device)
        if status is None:
            status = torch.empty(B, dtype=torch.int32, device=self.device)
        if order is None:
            order = longest_first(params)
        rc = self.lib.eob_waveform_lnl(_ptr(self.ws), self.ws_bytes, self.max_batch, self.max_steps, self.max_modes,
                                       self.max_samples, _ptr(params), _ptr(order), B, self.ells, self.mms,
                                       len(self.modes), float(dt), _ptr(data), N, float(amp),
                                       ctypes.byref(self.options), _ptr(lnl), _ptr(status), _stream_handle(stream))
        _lib.check(rc, "eob_waveform_lnl")
        self.last_B = B
        return lnl, status

    def strain(self, params: torch.Tensor, dt: float, n_samples: int, order: torch.Tensor | None = None,
               status: torch.Tensor | None = None, stream=None):
        """Complex strain sum_lm h_lm(t_k), k < n_samples, per binary: complex128 [B, n_samples]."""
        B = int(params.shape[0])
        assert params.is_cuda and params.dtype == torch.float64 and params.is_contiguous()
        out = torch.empty((B, n_samples, 2), dtype=torch.float64, device=self.device)
        if status is None:
            status = torch.empty(B, dtype=torch.int32, device=self.device)
        if order is None:
            order = longest_first(params)
        rc = self.lib.eob_waveform_strain(_ptr(self.ws), self.ws_bytes, self.max_batch, self.max_steps,
                                          self.max_modes, self.max_samples, _ptr(params), _ptr(order), B, self.ells,
                                          self.mms, len(self.modes), float(dt), int(n_samples),
                                          ctypes.byref(self.options), _ptr(out), _ptr(status),
                                          _stream_handle(stream))
        _lib.check(rc, "eob_waveform_strain")
        self.last_B = B
        return torch.view_as_complex(out), status

    def prepare(self, params: torch.Tensor, dt: float, order: torch.Tensor | None = None, stages: int = 7,
                stream=None):
        """Setup + integrator + multipoles + splines (stages bit mask 1|2|4)."""
        B = int(params.shape[0])
        if order is None:
            order = longest_first(params)
        rc = self.lib.eob_prepare_stages(_ptr(self.ws), self.ws_bytes, self.max_batch, self.max_steps,
                                         self.max_modes, self.max_samples, _ptr(params), _ptr(order), B, self.ells,
                                         self.mms, len(self.modes), float(dt), ctypes.byref(self.options), stages,
                                         _stream_handle(stream))
        _lib.check(rc, "eob_prepare_stages")
        self.last_B = B

    def synth_lnl(self, B: int, data: torch.Tensor, dt: float, amp: float, lnl=None, status=None, stream=None):
        N = int(data.shape[0])
        if lnl is None:
            lnl = torch.empty(B, dtype=torch.float64, device=self.device)
        if status is None:
            status = torch.empty(B, dtype=torch.int32, device=self.device)
        rc = self.lib.eob_synth_lnl(_ptr(self.ws), self.ws_bytes, self.max_batch, self.max_steps, self.max_modes,
                                    self.max_samples, B, self.mms, len(self.modes), float(dt), _ptr(data), N,
                                    float(amp), ctypes.byref(self.options), _ptr(lnl), _ptr(status),
                                    _stream_handle(stream))
        _lib.check(rc, "eob_synth_lnl")
        return lnl, status

    def synth_strain(self, B: int, dt: float, n_samples: int, per_mode: bool = False, status=None, stream=None):
        K = len(self.modes)
        shape = (B, K, n_samples, 2) if per_mode else (B, n_samples, 2)
        out = torch.empty(shape, dtype=torch.float64, device=self.device)
        if status is None:
            status = torch.empty(B, dtype=torch.int32, device=self.device)
        rc = self.lib.eob_synth_strain(_ptr(self.ws), self.ws_bytes, self.max_batch, self.max_steps, self.max_modes,
                                       self.max_samples, B, self.mms, K, float(dt), int(n_samples), int(per_mode),
                                       _ptr(out), _ptr(status), _stream_handle(stream))
        _lib.check(rc, "eob_synth_strain")
        return torch.view_as_complex(out), status

    def counters(self):
        """[rows, chunks, rhs_binaries, rhs_all_lanes] of the last run (synchronises)."""
        buf = (ctypes.c_ulonglong * 8)()
        _lib.check(self.lib.eob_workspace_counters(_ptr(self.ws), self.max_batch, self.max_steps, self.max_modes,
                                                   self.max_samples, buf, _stream_handle(None)),
                   "eob_workspace_counters")
        return {"rows": int(buf[1]), "chunks": int(buf[2]), "rhs_binaries": int(buf[4]), "rhs_all_lanes": int(buf[5])}

    def rhs_counts(self):
        """Right-hand sides evaluated per binary in the last run (host numpy)."""
        torch.cuda.synchronize()
        v = self.views()
        return self._dev_array(v.rhs, self.last_B, torch.int32).cpu().numpy()

    def npts(self):
        torch.cuda.synchronize()
        v = self.views()
        return self._dev_array(v.npts, self.last_B, torch.int32).cpu().numpy()

    # ---- inspection of the last run (tests, API mirror) -----------------
    def views(self) -> _lib.EobViews:
        v = _lib.EobViews()
        _lib.check(self.lib.eob_workspace_views(_ptr(self.ws), self.max_batch, self.max_steps, self.max_modes,
                                                self.max_samples, ctypes.byref(v)), "eob_workspace_views")
        return v

    def _dev_array(self, addr, count, dtype):
        """A torch view of `count` elements at a device address inside the workspace."""
        base = self.ws.data_ptr()
        off = int(addr) - base
        esize = torch.empty(0, dtype=dtype).element_size()
        assert 0 <= off and off + count * esize <= self.ws_bytes
        return self.ws[off:off + count * esize].view(dtype)

    def trajectories(self):
        """(nsteps[B], npts[B], status[B], list of (t [M], y[L, 4])) of the last run (host numpy)."""
        torch.cuda.synchronize()
        v = self.views()
        B = self.last_B
        nsteps = self._dev_array(v.nsteps, B, torch.int32).cpu().numpy()
        npts = self._dev_array(v.npts, B, torch.int32).cpu().numpy()
        status = self._dev_array(v.status, B, torch.int32).cpu().numpy()
        traj = self._dev_array(v.traj, B * self.max_steps * 5, torch.float64).view(B if B else 1, self.max_steps, 5)
        out = []
        for b in range(B):
            L = int(nsteps[b])
            t = traj[b, :L].cpu().numpy()
            out.append((t[:, 0].copy(), t[:, 1:].copy()))
        return nsteps, npts, status, out

    def initial_conditions(self):
        """(r0, pphi0, pr0) per binary of the last run."""
        torch.cuda.synchronize()
        v = self.views()
        traj = self._dev_array(v.traj, self.last_B * self.max_steps * 5, torch.float64).view(-1, self.max_steps, 5)
        first = traj[:, 0].cpu().numpy()
        return np.stack([first[:, 1], first[:, 4], first[:, 3]], axis=1)


class CapturedLikelihood:
    """One WaveformLikelihood.run captured as a CUDA graph.

    The graph holds the whole path (setup, persistent integrator, packing,
    multipoles, splines, synthesis + lnL: about ten launches and one memset)
    for fixed input tensors; a new batch is copied into `params` (and, if it
    changes, `data`) in place and `replay()` re-runs every launch at the cost
    of one graph launch.  The batch size, modes and options are those of the
    capture; `order` (queue order) is recomputed from `params` inside the
    graph."""

    def __init__(self, wl: "WaveformLikelihood", params: torch.Tensor, data: torch.Tensor, dt: float, amp: float):
        self.wl = wl
        self.params = params
        self.data = data
        self.B = int(params.shape[0])
        self.lnl = torch.empty(self.B, dtype=torch.float64, device=wl.device)
        self.status = torch.empty(self.B, dtype=torch.int32, device=wl.device)
        self.order = torch.empty(self.B, dtype=torch.int32, device=wl.device)
        self.graph = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream(wl.device)
        side.wait_stream(torch.cuda.current_stream(wl.device))
        with torch.cuda.stream(side):  # warm-up outside the capture
            self._body(dt, amp, side)
        torch.cuda.current_stream(wl.device).wait_stream(side)
        with torch.cuda.graph(self.graph):
            self._body(dt, amp, torch.cuda.current_stream(wl.device))

    def _body(self, dt, amp, stream):
        self.order.copy_(longest_first(self.params))
        self.wl.run(self.params, self.data, dt, amp, order=self.order, lnl=self.lnl, status=self.status,
                    stream=stream)

    def replay(self):
        """Re-run the captured path on the current contents of params/data;
        returns the (static) lnl and status tensors."""
        self.graph.replay()
        return self.lnl, self.status


def chunk_size_for_budget(budget_bytes: int, max_steps: int, n_modes: int, n_samples: int, upper: int) -> int:
    """Largest batch whose workspace fits in budget_bytes (0 if none does)."""
    lib = _lib.load()
    lo, hi = 0, int(upper)
    while lo < hi:
        mid = (lo + hi + 1) // 2
        need = int(lib.eob_workspace_bytes(mid, int(max_steps), int(n_modes), int(n_samples)))
        if need != 0 and need <= budget_bytes:
            lo = mid
        else:
            hi = mid - 1
    return lo


class ChunkedLikelihood:
    """lnL of batches larger than one workspace, in memory-admitted chunks.

    Chunks are sized so that `slots` workspaces fit in hbm_budget_bytes
    (default: 60 % of the free device memory) for batches of up to
    max_batch binaries; a call orders its batch longest first, cuts it into
    chunks and alternates them over the slots' streams, so that a chunk
    starts while the ragged tail of the previous one still runs.

    head > 0 runs the `head` longest binaries of a call on their own
    workspace and stream with head_lanes lanes per binary, concurrently with
    the rest: the bulk of a large batch is throughput bound (one lane per
    binary), but its few longest binaries would set the time of the first
    chunk; with several lanes each, their sequential chains are shorter."""

    def __init__(self, max_batch: int, n_samples: int, modes=((2, 2),), max_steps: int = 16000,
                 hbm_budget_bytes: int | None = None, slots: int = 2, options: _lib.EobOptions | None = None,
                 head: int = 0, head_lanes: int = 8, device="cuda"):
        self.device = torch.device(device)
        if hbm_budget_bytes is None:
            free, _ = torch.cuda.mem_get_info(self.device)
            hbm_budget_bytes = int(0.6 * free)
        self.budget = int(hbm_budget_bytes)
        lib = _lib.load()
        self.head = max(0, min(int(head), int(max_batch) - 1))
        head_ws = int(lib.eob_workspace_bytes(self.head, max_steps, len(modes), n_samples)) if self.head else 0
        per_slot = (self.budget - head_ws) // max(1, slots)
        rest = int(max_batch) - self.head
        self.chunk = chunk_size_for_budget(per_slot, max_steps, len(modes), n_samples, max(1, -(-rest // slots)))
        if self.chunk < 1:
            raise _lib.EOBError(f"HBM budget {self.budget} B admits no binary at max_steps={max_steps}, "
                                f"N={n_samples}")
        nslots = min(slots, -(-rest // self.chunk))
        self.engines = [WaveformLikelihood(self.chunk, max_steps, modes, n_samples, device=self.device,
                                           options=options) for _ in range(nslots)]
        self.streams = [torch.cuda.Stream(self.device) for _ in range(nslots)]
        self.identity = torch.arange(max(self.chunk, self.head), dtype=torch.int32, device=self.device)
        self.head_engine = None
        if self.head:
            ho = _lib.EobOptions.from_buffer_copy(options) if options is not None else _lib.default_options()
            ho.lanes_per_binary = int(head_lanes)
            self.head_lanes = int(head_lanes)
            self.head_engine = WaveformLikelihood(self.head, max_steps, modes, n_samples, device=self.device,
                                                  options=ho)
            self.head_stream = torch.cuda.Stream(self.device)

    def info(self, B: int):
        d = {"chunk": self.chunk, "chunks": -(-(B - self.head) // self.chunk), "slots": len(self.engines),
             "workspace_bytes_per_slot": self.engines[0].ws_bytes, "budget_bytes": self.budget}
        if self.head:
            d.update({"head": self.head, "head_lanes_per_binary": self.head_lanes})
        return d

    def _one(self, e, s, idx, params, data, dt, amp, lnl, status):
        with torch.cuda.stream(s):
            P = params[idx].contiguous()
            l, st = e.run(P, data, dt, amp, order=self.identity[:len(idx)], stream=s)
            lnl[idx] = l
            status[idx] = st
            for t in (P, l, st, idx):
                t.record_stream(s)

    def run(self, params: torch.Tensor, data: torch.Tensor, dt: float, amp: float):
        B = int(params.shape[0])
        order = longest_first(params).long()
        lnl = torch.empty(B, dtype=torch.float64, device=self.device)
        status = torch.empty(B, dtype=torch.int32, device=self.device)
        main = torch.cuda.current_stream(self.device)
        head = min(self.head, B)
        used = []
        if head:
            self.head_stream.wait_stream(main)
            self._one(self.head_engine, self.head_stream, order[:head], params, data, dt, amp, lnl, status)
            used.append(self.head_stream)
        n = len(self.engines)
        for j, lo in enumerate(range(head, B, self.chunk)):
            e, s = self.engines[j % n], self.streams[j % n]
            s.wait_stream(main)
            self._one(e, s, order[lo:lo + self.chunk], params, data, dt, amp, lnl, status)
            used.append(s)
        for s in used:
            main.wait_stream(s)
        return lnl, status


def lnl_chunked(params: torch.Tensor, data: torch.Tensor, dt: float, amp: float, modes=((2, 2),),
                max_steps: int = 16000, hbm_budget_bytes: int | None = None, slots: int = 2,
                options: _lib.EobOptions | None = None, head: int = 0, head_lanes: int = 8, device="cuda"):
    """One-shot ChunkedLikelihood: (lnl, status, info) in the input order."""
    c = ChunkedLikelihood(int(params.shape[0]), int(data.shape[0]), modes, max_steps, hbm_budget_bytes, slots,
                          options, head, head_lanes, device)
    lnl, status = c.run(params, data, dt, amp)
    return lnl, status, c.info(int(params.shape[0]))
