"""Batched form: many HEALPix map sets of different nside / lmax / nmaps / spin /
precision executed as one CUDA-graph launch (C ABI: fsht_batch_*).

    from fastsht_gb300.batch import Batch
    b = Batch()
    j = b.add("t2alm", nside=64, lmax=191, nmaps=10)        # allocates device buffers
    j.inputs[0].copy_(maps)                                # (nmaps, npix) float64, CUDA
    b.build()                                              # plans, autotune, workspace
    b.run(); b.sync()                                      # one graph launch
    alm = j.outputs[0]                                     # (lmax+1, lmax+1, nmaps)

Device layouts are the library's: maps (nmaps, npix) contiguous (= the reference's
Fortran (npix, nsim)), alm (lmax+1, lmax+1, nmaps) contiguous (= Fortran
(nsim, lmax+1, lmax+1)).  An I/Q/U set is two jobs: "t2alm" on I and "qu2eb" on Q/U.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import torch

from . import _lib

_KINDS = {"t2alm": _lib.FSHT_JOB_T2ALM, "alm2t": _lib.FSHT_JOB_ALM2T,
          "qu2eb": _lib.FSHT_JOB_QU2EB, "eb2qu": _lib.FSHT_JOB_EB2QU}


@dataclass
class Job:
    kind: str
    nside: int
    lmax: int
    nmaps: int
    precision: str = "fp64"
    inputs: list = field(default_factory=list)
    outputs: list = field(default_factory=list)


class Batch:
    def __init__(self, device=None, nslots=4, workspace_budget=0, autotune=True):
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.nslots = nslots
        self.workspace_budget = workspace_budget
        self.autotune = autotune
        self.jobs: list[Job] = []
        self._b = C.c_void_p()
        self._stream = None

    def add(self, kind, nside, lmax, nmaps, precision="fp64", inputs=None, outputs=None) -> Job:
        if kind not in _KINDS:
            raise ValueError(f"kind must be one of {sorted(_KINDS)}")
        if precision not in ("fp64", "split"):
            raise ValueError("precision must be 'fp64' or 'split'")
        if self._b.value:
            raise RuntimeError("batch already built")
        npix = 12 * nside * nside
        L = lmax + 1
        nf = 2 if kind in ("qu2eb", "eb2qu") else 1
        mk_maps = lambda: torch.zeros((nmaps, npix), dtype=torch.float64, device=self.device)
        mk_alm = lambda: torch.zeros((L, L, nmaps), dtype=torch.float64, device=self.device)
        analysis = kind in ("t2alm", "qu2eb")
        if inputs is None:
            inputs = [mk_maps() if analysis else mk_alm() for _ in range(nf)]
        if outputs is None:
            outputs = [mk_alm() if analysis else mk_maps() for _ in range(nf)]
        for t in list(inputs) + list(outputs):
            if not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
                raise ValueError("job buffers must be contiguous float64 CUDA tensors")
        j = Job(kind, nside, lmax, nmaps, precision, list(inputs), list(outputs))
        self.jobs.append(j)
        return j

    def build(self):
        arr = (_lib.FshtJob * len(self.jobs))()
        for a, j in zip(arr, self.jobs):
            a.nside, a.lmax, a.nmaps = j.nside, j.lmax, j.nmaps
            a.kind = _KINDS[j.kind]
            a.precision = _lib.FSHT_PREC_SPLIT if j.precision == "split" else _lib.FSHT_PREC_FP64
            a.in0 = j.inputs[0].data_ptr()
            a.in1 = j.inputs[1].data_ptr() if len(j.inputs) > 1 else None
            a.out0 = j.outputs[0].data_ptr()
            a.out1 = j.outputs[1].data_ptr() if len(j.outputs) > 1 else None
        with torch.cuda.device(self.device):
            self._stream = torch.cuda.Stream(self.device)
            torch.cuda.synchronize(self.device)     # inputs written on other streams
            _lib.call("fsht_batch_create", C.cast(arr, C.c_void_p), len(self.jobs), self.nslots,
                      int(self.workspace_budget), 1 if self.autotune else 0,
                      C.c_void_p(self._stream.cuda_stream), C.byref(self._b))
        return self

    def run(self):
        if not self._b.value:
            self.build()
        # the batch stream must see inputs written on the current stream
        self._stream.wait_stream(torch.cuda.current_stream(self.device))
        _lib.call("fsht_batch_run", self._b)
        torch.cuda.current_stream(self.device).wait_stream(self._stream)

    def sync(self):
        _lib.call("fsht_batch_sync", self._b)

    def info(self):
        n_plans, n_nodes = C.c_int(), C.c_int()
        _lib.call("fsht_batch_info", self._b, C.byref(n_plans), C.byref(n_nodes))
        return {"plans": n_plans.value, "graph_nodes": n_nodes.value, "jobs": len(self.jobs)}

    def tunings(self):
        """Per plan of the built batch: (nside, lmax, precision) and the launch shapes it runs
        with (FFT maps per CTA and threads, FP64 analysis maps per CTA and rings per chunk,
        split ring-part k-steps; 0 = the kernel's default)."""
        n_plans = C.c_int()
        _lib.call("fsht_batch_info", self._b, C.byref(n_plans), None)
        out = []
        for i in range(n_plans.value):
            ns, lm, pr = C.c_int(), C.c_int(), C.c_int()
            sh = (C.c_int * 5)()
            _lib.call("fsht_batch_plan_tuning", self._b, i, C.byref(ns), C.byref(lm),
                      C.byref(pr), sh)
            out.append({"nside": ns.value, "lmax": lm.value,
                        "precision": "split" if pr.value == _lib.FSHT_PREC_SPLIT else "fp64",
                        "fft_maps_per_cta": sh[0], "fft_threads": sh[1],
                        "fp64_maps_per_cta": sh[2], "fp64_rings_per_chunk": sh[3],
                        "split_part_steps": sh[4]})
        return out

    def close(self):
        if self._b.value:
            _lib.load().fsht_batch_destroy(self._b)
            self._b = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
