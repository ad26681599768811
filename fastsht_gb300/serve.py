"""Serving form: a continuous-batching request loop for mixed-size transforms.

Requests (map2alm / alm2map, T or Q/U, any supported nside / lmax / nmaps, FP64 or
split precision) are admitted while earlier ones are still on the GPU, as soon as
a stream slot and enough of the HBM budget are free; admitted work runs
concurrently on the slots' streams.  Waiting requests with the same configuration
(kind, nside, lmax, precision) are fused into one job along the map axis, so they
share the per-(l, m, ring) recursion and fill the kernels' 64-map tiles.  A request
whose footprint exceeds the whole budget is split along maps.  Inputs and results
stay resident on the device (CUDA tensors); host arrays are copied in on the job's
stream.  Each request records arrival, admission and completion times, from which
the server reports p50 / p99 latency beside throughput, overall and per precision.

Head-of-line blocking: a large request (an FP64 transform at nside 2048 takes tens of
seconds) must not hold back small ones.  Three rules keep it from doing so:
  * a job's estimated GPU time (a cost model of its FFT and Legendre work at the
    precision's rate) is capped at max_job_s, in whole 64-map tiles: larger requests run
    as several jobs along maps, so they give their slot and memory back regularly (a job
    of fewer than 64 maps costs a whole tile, so requests are never split below one);
  * jobs estimated below small_s are "small": they run on high-priority streams, so
    their thread blocks are scheduled ahead of the waiting blocks of large kernels;
  * `reserved` of the slots (the high-priority ones) only take small jobs, so a burst
    of large requests cannot occupy every slot.
Kernels are not preempted: a small job can still wait for the large jobs' kernels that are
running when it arrives, so its latency is bounded by a few max_job_s, not by the size of the
large requests.

No counterpart in the reference (one SHT instance, one blocking call at a time,
SHT.py:16-227); every transform runs through the C ABI's fsht_run_job on a shared
table-only plan per (nside, lmax, precision).
"""
from __future__ import annotations

import collections
import ctypes as C
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib

_TILE_MAPS = 64       # maps per contraction tile (FP64 and split kernels alike)

_KINDS = {"t2alm": _lib.FSHT_JOB_T2ALM, "alm2t": _lib.FSHT_JOB_ALM2T,
          "qu2eb": _lib.FSHT_JOB_QU2EB, "eb2qu": _lib.FSHT_JOB_EB2QU}


@dataclass(eq=False)      # identity: requests are found in queues with `in` / remove()
class Request:
    kind: str
    nside: int
    lmax: int
    nmaps: int
    precision: str
    inputs: list                      # device tensors in the library layout (or host arrays)
    t_arrival: float
    future: Future = field(default_factory=Future)
    t_admit: float = 0.0
    t_done: float = 0.0
    parts: int = 0                    # jobs this request ran in (split along maps)
    fused: int = 1                    # largest number of requests sharing one of its jobs
    ready: torch.cuda.Event = None    # inputs written (submitting thread's stream)
    next_map: int = 0                 # first map not yet admitted
    done_parts: list = field(default_factory=list)   # (m0, outputs) per finished piece
    held: list = field(default_factory=list)         # jobs whose outputs hold its pieces

    @property
    def key(self):
        return (self.kind, self.nside, self.lmax, self.precision)

    @property
    def nfields(self):
        return 2 if self.kind in ("qu2eb", "eb2qu") else 1

    @property
    def analysis(self):
        return self.kind in ("t2alm", "qu2eb")


@dataclass(eq=False)
class _Part:
    members: list                     # (request, m0, m1, offset of m0 in this job)
    nmaps: int
    outputs: list
    keep: list                        # tensors the job reads (kept alive until it ends)
    event: torch.cuda.Event = None
    slot: int = -1
    nbytes: int = 0                   # budget charged: inputs + outputs + workspace
    out_bytes: int = 0                # the outputs' share, held until every member completes
    holders: int = 0                  # members not yet completed


def _maps_shape(nside, nmaps):
    return (nmaps, 12 * nside * nside)


def _alm_shape(lmax, nmaps):
    return (lmax + 1, lmax + 1, nmaps)


class Server:
    """Continuous-batching SHT server on one GPU.

    hbm_budget: device bytes the server may hold for in-flight jobs (inputs, outputs and
    workspaces); a job's output stays charged until every request with a piece in it has
    completed (the pieces are views of it), and a request split into several jobs is joined
    into one output at completion, outside the budget for that moment; nslots: concurrent CUDA
    streams; fuse_maps: most maps one fused job may gather from waiting requests of the same
    configuration (0 disables fusing); discard_outputs: complete futures with None and drop
    the results (a client that only measures the service).
    """

    def __init__(self, hbm_budget=150e9, nslots=8, device=None, poll_s=5e-5, fuse_maps=128,
                 max_job_s=1.0, small_s=0.05, reserved=2, discard_outputs=False):
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.budget = int(hbm_budget)
        self.nslots = nslots
        self.poll_s = poll_s
        self.fuse_maps = int(fuse_maps)
        self.max_job_s = float(max_job_s)
        self.small_s = float(small_s)
        self.reserved = max(0, min(int(reserved), nslots - 1))
        self.discard_outputs = bool(discard_outputs)
        with torch.cuda.device(self.device):
            # slots [0, reserved): high-priority streams for small jobs only
            self.streams = [torch.cuda.Stream(self.device, priority=-1 if i < self.reserved else 0)
                            for i in range(nslots)]
        self._plans = {}
        self._ws_cache = {}
        self._pending = collections.deque()
        self._inflight: list[_Part] = []
        self._free_slots = list(range(nslots))
        self._used = 0
        self.high_water = 0
        self.max_inflight = 0
        self.max_fused = 1
        self.completed: list[Request] = []
        self._lock = threading.Condition()
        self._stop = False
        self._error = None
        self._thread = threading.Thread(target=self._loop, name="fsht-server", daemon=True)
        self._thread.start()

    # ------------------------------------------------------------ client side
    def submit(self, kind, nside, lmax, inputs, precision="fp64", t_arrival=None) -> Future:
        """inputs: list of CUDA float64 tensors (maps (nmaps, npix) or alm
        (lmax+1, lmax+1, nmaps), contiguous) or NumPy arrays in the reference's
        Fortran layout (copied to the device on admission)."""
        if kind not in _KINDS:
            raise ValueError(f"kind must be one of {sorted(_KINDS)}")
        if precision not in ("fp64", "split"):
            raise ValueError("precision must be 'fp64' or 'split'")
        nf = 2 if kind in ("qu2eb", "eb2qu") else 1
        if len(inputs) != nf:
            raise ValueError(f"{kind} takes {nf} input field(s)")
        ins = []
        for x in inputs:
            if isinstance(x, torch.Tensor):
                if not (x.is_cuda and x.dtype == torch.float64 and x.is_contiguous()):
                    raise ValueError("device inputs must be contiguous float64 CUDA tensors")
                ins.append(x)
            else:
                ins.append(np.ascontiguousarray(np.asarray(x, dtype=np.float64).T))
        nmaps = ins[0].shape[0] if kind in ("t2alm", "qu2eb") else ins[0].shape[-1]
        req = Request(kind, int(nside), int(lmax), int(nmaps), precision, ins,
                      time.perf_counter() if t_arrival is None else t_arrival)
        if any(isinstance(x, torch.Tensor) for x in ins):
            # device inputs may still be in flight on the caller's stream
            req.ready = torch.cuda.Event()
            req.ready.record(torch.cuda.current_stream(self.device))
        with self._lock:
            if self._error:
                raise RuntimeError(f"server failed: {self._error}")
            self._pending.append(req)
            self._lock.notify()
        return req.future

    def drain(self, timeout=None):
        """Block until every submitted request has completed."""
        t0 = time.perf_counter()
        with self._lock:
            while self._pending or self._inflight:
                if self._error:
                    raise RuntimeError(f"server failed: {self._error}")
                self._lock.wait(0.01)
                if timeout is not None and time.perf_counter() - t0 > timeout:
                    raise TimeoutError("drain timed out")

    def close(self):
        with self._lock:
            self._stop = True
            self._lock.notify()
        self._thread.join()
        for p in self._plans.values():
            _lib.load().fsht_plan_destroy(p)
        self._plans.clear()

    def stats(self):
        lat = np.array([r.t_done - r.t_arrival for r in self.completed])
        if lat.size == 0:
            return {}
        t0 = min(r.t_arrival for r in self.completed)
        t1 = max(r.t_done for r in self.completed)
        mapsht = sum(r.nmaps * r.nfields for r in self.completed)

        def pct(rs):
            x = np.array([r.t_done - r.t_arrival for r in rs])
            return {"requests": int(x.size), "p50_ms": float(np.percentile(x, 50) * 1e3),
                    "p99_ms": float(np.percentile(x, 99) * 1e3)} if x.size else None

        by_prec = {pr: pct([r for r in self.completed if r.precision == pr])
                   for pr in ("fp64", "split")}
        by_nside = {ns: pct([r for r in self.completed if r.nside == ns])
                    for ns in sorted({r.nside for r in self.completed})}
        return {"requests": int(lat.size), "p50_ms": float(np.percentile(lat, 50) * 1e3),
                "p99_ms": float(np.percentile(lat, 99) * 1e3),
                "mean_ms": float(lat.mean() * 1e3), "wall_s": t1 - t0,
                "requests_per_s": lat.size / (t1 - t0),
                "maps_sht_per_s": mapsht / (t1 - t0),
                "by_precision": {k: v for k, v in by_prec.items() if v},
                "by_nside": by_nside,
                "high_water_bytes": self.high_water, "budget_bytes": self.budget,
                "max_inflight": self.max_inflight, "max_fused": self.max_fused,
                "max_parts": max(r.parts for r in self.completed)}

    # ------------------------------------------------------------ internals
    def _plan(self, nside, lmax, precision):
        key = (nside, lmax, precision)
        p = self._plans.get(key)
        if p is None:
            p = C.c_void_p()
            with torch.cuda.device(self.device):
                split = precision == "split"
                flags = _lib.FSHT_FLAG_TABLES_ONLY | (_lib.FSHT_FLAG_POL if split else 0)
                _lib.call("fsht_plan_create", nside, lmax, 1, flags,
                          _lib.FSHT_PREC_SPLIT if split else _lib.FSHT_PREC_FP64,
                          0, None, C.byref(p))
            self._plans[key] = p
        return p

    def _fsht_job(self, req, n, ins=None, outs=None):
        j = _lib.FshtJob()
        j.nside, j.lmax, j.nmaps = req.nside, req.lmax, n
        j.kind = _KINDS[req.kind]
        j.precision = _lib.FSHT_PREC_SPLIT if req.precision == "split" else _lib.FSHT_PREC_FP64
        if ins is not None:
            j.in0 = ins[0].data_ptr()
            j.in1 = ins[1].data_ptr() if len(ins) > 1 else None
            j.out0 = outs[0].data_ptr()
            j.out1 = outs[1].data_ptr() if len(outs) > 1 else None
        return j

    @staticmethod
    def cost_s(kind, nside, lmax, precision, n):
        """Rough GPU seconds of one job of n maps (scheduling only).  The contractions work on
        tiles of 64 maps, so a job of fewer maps costs a whole tile: the Legendre term counts
        ceil(n / 64) tiles of 64 maps at 4 nside (lmax+1)(lmax+2) flop per map (four times that
        per Q/U pair), about 1 TFLOP/s in FP64 and 80 TFLOP/s in the split form, whose
        recursion also runs once per job (about 30 ms at nside 1024 / lmax 2047, scaled by
        nside (lmax+1)^2); the ring FFTs cost about 0.4 ms (df64) / 1.3 ms (FP64) per map per
        field at nside 1024, scaled by the pixel count."""
        nf = 2 if kind in ("qu2eb", "eb2qu") else 1
        split = precision == "split"
        fft = n * (0.4e-3 if split else 1.3e-3) * (nside / 1024.0) ** 2 * nf
        tiles = -(-n // _TILE_MAPS)
        leg = (_TILE_MAPS * tiles * 4.0 * nside * (lmax + 1) * (lmax + 2) *
               (4 if nf == 2 else 1))
        rec = 0.03 * (nside / 1024.0) * ((lmax + 1) / 2048.0) ** 2 if split else 0.0
        return fft + leg / (80e12 if split else 1.0e12) + rec

    def _req_cost(self, req, n):
        return self.cost_s(req.kind, req.nside, req.lmax, req.precision, n)

    def _io_bytes(self, req, n):
        npix = 12 * req.nside ** 2
        L = req.lmax + 1
        return 8 * n * (npix + L * L) * req.nfields

    def _workspace_bytes(self, req, n, kc):
        key = req.key + (n, kc)
        b = self._ws_cache.get(key)
        if b is None:
            plan = self._plan(req.nside, req.lmax, req.precision)
            j = self._fsht_job(req, n)
            out = C.c_size_t()
            _lib.call("fsht_job_workspace", plan, C.byref(j), kc, C.byref(out))
            b = self._ws_cache[key] = int(out.value)
        return b

    def _fit(self, req, n_max, avail):
        """Largest (maps <= n_max, maps-per-chunk) of req's configuration whose footprint fits."""
        n = n_max
        while n >= 1:
            kc = min(n, 128)
            while kc >= 1:
                need = self._io_bytes(req, n) + self._workspace_bytes(req, n, kc)
                if need <= avail:
                    return n, kc, need
                kc //= 2
            n //= 2
        return None

    def _gather(self, head):
        """head plus waiting, not yet started requests of its configuration (arrival
        order), up to fuse_maps maps in total."""
        group = [head]
        if self.fuse_maps and head.next_map == 0:
            total = head.nmaps
            for r in self._pending:
                if r is head or r.next_map or r.key != head.key:
                    continue
                if total + r.nmaps > self.fuse_maps:
                    break
                group.append(r)
                total += r.nmaps
        return group

    def _slot_for(self, small):
        """A free slot for a job: small jobs prefer the reserved high-priority slots, large
        jobs only take the others."""
        free = sorted(self._free_slots)
        if small:
            return free[0] if free else None
        big = [s for s in free if s >= self.reserved]
        return big[0] if big else None

    def _admit(self, head) -> bool:
        """Admit one job led by `head`: the rest of head's maps (as many as fit the budget and
        the max_job_s cap), or head fused with waiting requests of the same configuration."""
        if not self._free_slots:
            return False
        avail = self.budget - self._used
        # maps per job under the duration cap (at least one)
        # maps per job under the duration cap, in whole 64-map tiles: a job of fewer maps
        # costs a whole tile, so splitting below one only multiplies the work
        per_tile = self._req_cost(head, _TILE_MAPS)
        n_cap = _TILE_MAPS * max(1, int(self.max_job_s / per_tile)) if per_tile > 0 else 1 << 30
        group = self._gather(head)
        while True:
            total = min(sum(r.nmaps - r.next_map for r in group), n_cap)
            fit = self._fit(head, total, avail)
            if fit is None or fit[0] == total or len(group) == 1:
                break
            group.pop()                 # the fused job does not fit whole: fuse fewer
        if fit is None:
            if not self._inflight:
                # nothing running will free memory: one map of this request (beside the outputs
                # of its finished pieces) can never fit
                err = ValueError(f"request (nside {head.nside}, lmax {head.lmax}) does not fit "
                                 f"the {self.budget}-byte budget even for one map")
                if not head.future.done():
                    head.future.set_exception(err)
                if head in self._pending:
                    self._pending.remove(head)
                self._release(head)
            return False
        n, kc, need = fit
        slot = self._slot_for(self._req_cost(head, n) <= self.small_s)
        if slot is None:
            return False
        members, off = [], 0
        for r in group:
            k = min(r.nmaps - r.next_map, n - off)
            if k <= 0:
                break
            members.append((r, r.next_map, r.next_map + k, off))
            off += k
        self._free_slots.remove(slot)
        stream = self.streams[slot]
        with torch.cuda.device(self.device), torch.cuda.stream(stream):
            for r, *_ in members:
                if r.ready is not None:
                    stream.wait_event(r.ready)
            ins = []
            for f in range(head.nfields):
                pieces = []
                for r, m0, m1, _ in members:
                    x = r.inputs[f]
                    if isinstance(x, torch.Tensor):
                        pieces.append(x[m0:m1] if r.analysis else x[..., m0:m1])
                    else:
                        part = x[m0:m1] if r.analysis else x[..., m0:m1]
                        pieces.append(torch.from_numpy(np.ascontiguousarray(part)).to(
                            self.device, non_blocking=True))
                if len(pieces) == 1:
                    ins.append(pieces[0].contiguous())
                else:
                    ins.append(torch.cat(pieces, dim=0 if head.analysis else -1))
            shape = _alm_shape(head.lmax, n) if head.analysis else _maps_shape(head.nside, n)
            outs = [torch.empty(shape, dtype=torch.float64, device=self.device)
                    for _ in range(head.nfields)]
            ws = torch.empty(max(self._workspace_bytes(head, n, kc), 256), dtype=torch.uint8,
                             device=self.device)
            plan = self._plan(head.nside, head.lmax, head.precision)
            job = self._fsht_job(head, n, ins, outs)
            _lib.call("fsht_run_job", plan, C.byref(job), C.c_void_p(ws.data_ptr()),
                      ws.numel(), C.c_void_p(stream.cuda_stream))
            ev = torch.cuda.Event()
            ev.record(stream)
        now = time.perf_counter()
        for r, m0, m1, _ in members:
            if r.next_map == 0:
                r.t_admit = now
            r.next_map = m1
            r.parts += 1
            r.fused = max(r.fused, len(members))
            if r.next_map >= r.nmaps:
                self._pending.remove(r)
        self.max_fused = max(self.max_fused, len(members))
        self._used += need
        self.high_water = max(self.high_water, self._used)
        self._inflight.append(_Part(members, n, outs, ins + [ws], ev, slot, need,
                                    out_bytes=sum(o.numel() * o.element_size() for o in outs),
                                    holders=len(members)))
        self.max_inflight = max(self.max_inflight, len(self._inflight))
        return True

    def _release(self, r):
        """r has completed or failed: the jobs holding its pieces lose a holder, and a job's
        outputs leave the budget when no request holds a piece of them."""
        for p in r.held:
            p.holders -= 1
            if p.holders == 0:
                self._used -= p.out_bytes
                p.outputs = []
        r.held = []
        r.done_parts = []

    def _finish(self, part: _Part):
        self._used -= part.nbytes - part.out_bytes     # inputs and workspace
        part.keep = []
        self._free_slots.append(part.slot)
        head = part.members[0][0]
        rc = _lib.load().fsht_plan_check(self._plan(head.nside, head.lmax, head.precision))
        if rc:          # a bounded device-side wait expired: these results are invalid
            err = _lib.FshtError(rc, "fsht_plan_check", _lib.last_error())
            for r, *_ in part.members:
                if not r.future.done():
                    r.future.set_exception(err)
                if r in self._pending:
                    self._pending.remove(r)
                r.held.append(part)
                self._release(r)
            return
        for r, m0, m1, off in part.members:
            if len(part.members) == 1 and m0 == 0 and m1 == r.nmaps:
                piece = part.outputs
            elif r.analysis:
                piece = [o[..., off:off + (m1 - m0)] for o in part.outputs]
            else:
                piece = [o[off:off + (m1 - m0)] for o in part.outputs]
            r.done_parts.append((m0, piece))
            r.held.append(part)
            if r.future.done():           # failed in another job: nothing to assemble
                self._release(r)
                continue
            if sum(p[0].shape[-1 if r.analysis else 0] for _, p in r.done_parts) < r.nmaps:
                continue
            result = None
            if not self.discard_outputs:
                r.done_parts.sort(key=lambda t: t[0])
                with torch.cuda.device(self.device):
                    if len(r.done_parts) == 1:
                        result = [t.contiguous() for t in r.done_parts[0][1]]
                    else:
                        dim = -1 if r.analysis else 0
                        result = [torch.cat([p[f] for _, p in r.done_parts], dim=dim)
                                  for f in range(r.nfields)]
                    torch.cuda.current_stream(self.device).synchronize()
            self._release(r)
            r.t_done = time.perf_counter()
            r.inputs = []                 # the client's tensors: not kept by the statistics
            self.completed.append(r)
            r.future.set_result(result)

    def _loop(self):
        try:
            while True:
                with self._lock:
                    if self._stop and not self._pending and not self._inflight:
                        return
                    still = []
                    for part in self._inflight:
                        if part.event.query():
                            self._finish(part)
                        else:
                            still.append(part)
                    self._inflight = still
                    # admissions in arrival order; a request that does not fit yet does not
                    # block smaller ones behind it
                    for req in list(self._pending):
                        if not self._free_slots:
                            break
                        if req not in self._pending:      # fused into an earlier job
                            continue
                        while self._free_slots and req.next_map < req.nmaps:
                            if not self._admit(req):
                                break
                    self._lock.notify_all()
                    idle = not self._pending and not self._inflight
                    if idle:
                        self._lock.wait(0.01)
                if not idle:
                    time.sleep(self.poll_s)
        except Exception as e:   # surface to clients instead of dying silently
            with self._lock:
                self._error = repr(e)
                for req in list(self._pending):
                    if not req.future.done():
                        req.future.set_exception(e)
                for part in self._inflight:
                    for r, *_ in part.members:
                        if not r.future.done():
                            r.future.set_exception(e)
                self._pending.clear()
                self._inflight.clear()
                self._lock.notify_all()
