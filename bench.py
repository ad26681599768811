#!/usr/bin/env python3
"""Benchmark of the batched HEALPix spherical-harmonic transform on GB300.

Workload (one GPU): map2alm (t2alm) of a batch of 500 temperature maps at
nside 1024 / lmax 2047, maps resident in HBM (50 GB, far above the 129 MB L2, so
no flush is needed between steps).  One step = one t2alm of the whole batch =
500 map.SHT.  Inputs: Gaussian alm with C_l ~ l^-2 (seed 2, a00 = 0) synthesised
to maps on the device by alm2t.  The headline is the split-precision form
(--precision split, the default); the plain FP64 path runs on the same maps and
its throughput, the split form's alm error against it and the round-trip map
residuals go in "fp64_plain".

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference algorithm's CPU restatement (the oracle:
NumPy/OpenBLAS DGEMMs, scipy.fft, the C recursion) on this host's cores on a
sample of the batch, scaled to the batch the way the reference computes it
(recursion once per m for the batch, FFT and DGEMM per map).  The reference's own
Fortran/MKL build cannot be compiled here (no Fortran compiler, no MKL).

Under torchrun (N > 1) every rank runs its own 500-map batch on its own GPU
(replicas; no collective on the data path), value = all maps / max time.
"""
from __future__ import annotations

import os

os.environ.setdefault("OMP_WAIT_POLICY", "PASSIVE")
# the CPU baseline alternates OpenMP loops (recursion, gather) with OpenBLAS DGEMMs: BLAS
# threads that keep spinning after a call would slow the OpenMP loops several times over
os.environ.setdefault("OPENBLAS_THREAD_TIMEOUT", "4")

import argparse
import json
import math
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import numpy as np

from fastsht_gb300.replicas import max_over_ranks

METRIC = "maps·SHT/s at nside 1024 (FP64 vs split-prec @ stated error); p50/p99 latency"
UNIT = "maps·SHT/s"


def flop_per_map(nside, lmax):
    """Algorithmic FLOP of one spin-0 transform direction: one real x complex
    FMA (4 flop) per (north ring, l, m) after north/south folding."""
    return 4.0 * nside * (lmax + 1) * (lmax + 2)


def fft_alg_flop_per_map(nside):
    """Conventional FFT flop count of one map's ring DFTs: 5 n log2 n per complex length-n
    transform, one per north/south ring pair (the equator ring alone)."""
    tot = 0.0
    for i in range(2 * nside):
        n = 4 * (i + 1) if i < nside else 4 * nside
        tot += 5.0 * n * math.log2(n)
    return tot


def fft_dp_ops_per_map(nside):
    """FP64 instructions one forward ring FFT pass executes per map (the kernels' radix-4 /
    radix-2 / radix-3 passes, Bluestein chirps and filter; the fold and phase are left out):
    the FFT is FP64-pipe bound, so this over the DFMA rate is its roofline."""
    def size(n):
        if n & (n - 1) == 0:
            return n, 0
        need = 2 * n - 1
        p2 = 1 << (need - 1).bit_length()
        p3 = 3
        while p3 < need:
            p3 *= 2
        return (p3, 1) if p3 < p2 else (p2, 0)

    def dif(P, r3):
        T = P // 3 if r3 else P
        nblk = 3 if r3 else 1
        ops = 22 * T if r3 else 0
        L = T.bit_length() - 1
        first = True
        while L >= 2:
            ops += nblk * (T // 4) * (16 if L == 2 else 28)
            L -= 2
        if L == 1:
            ops += nblk * (T // 2) * 4
        return ops

    total = 0
    for i in range(2 * nside):                 # ring pairs (N + iS), equator alone
        n = 4 * (i + 1) if i < nside else 4 * nside
        P, r3 = size(n)
        if P == n:
            total += dif(P, 0)
        else:
            total += 2 * dif(P, r3) + 4 * P + 8 * n
    return total


def fft_df_instr_per_map(nside):
    """FP32-pipe instructions (FADD / FMUL / FFMA) of the df64 arithmetic one forward ring FFT
    pass executes per map in the split form (k_ring_fft_fwd_df), counted from the kernel's
    operations: a lazy df64 complex addition 16, a lazy complex product 32, the
    renormalisation of a stored value 6.  Radix-4 butterfly 248 (152 without twiddles, 184 in
    Bluestein's zero-padded first pass, 204 in its last inverse pass that keeps two outputs);
    radix-2 44; radix-3 196 (164 / 174 in the pruned first / last passes); Bluestein chirps
    and filter 38 per point.  Load/store, index and FP64<->df64 conversion instructions are
    left out, as are the fold and phase (the same scope as fft_dp_ops_per_map)."""
    def size(n):
        if n & (n - 1) == 0:
            return n, 0
        need = 2 * n - 1
        p2 = 1 << (need - 1).bit_length()
        p3 = 3
        while p3 < need:
            p3 *= 2
        return (p3, 1) if p3 < p2 else (p2, 0)

    def dif(P, r3, pruned):
        T = P // 3 if r3 else P
        nblk = 3 if r3 else 1
        ops = (164 if pruned else 196) * T if r3 else 0
        L = T.bit_length() - 1
        first = True
        while L >= 2:
            bf = 152 if L == 2 else (184 if (pruned and first and not r3) else 248)
            ops += nblk * (T // 4) * bf
            L -= 2
            first = False
        if L == 1:
            ops += nblk * (T // 2) * 44
        return ops

    def dit(P, r3):
        T = P // 3 if r3 else P
        nblk = 3 if r3 else 1
        L = T.bit_length() - 1
        ops = nblk * (T // 2) * 44 if L & 1 else 0
        span = 3 if L & 1 else 2
        while span <= L:
            last = span == L and not r3
            bf = 152 if span == 2 else (204 if last else 248)
            ops += nblk * (T // 4) * bf
            span += 2
        if r3:
            ops += 174 * T
        return ops

    total = 0
    for i in range(2 * nside):
        n = 4 * (i + 1) if i < nside else 4 * nside
        P, r3 = size(n)
        if P == n:
            total += dif(P, 0, False)
        else:
            total += dif(P, r3, True) + dit(P, r3) + 38 * P + 2 * 38 * n
    return total


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--nside", type=int, default=1024)
    ap.add_argument("--lmax", type=int, default=None)
    ap.add_argument("--nmaps", type=int, default=500)
    ap.add_argument("--cpu-maps", type=int, default=32,
                    help="maps in the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-maps", type=int, default=None)
    ap.add_argument("--precision", choices=["split", "fp64"], default="split",
                    help="split: tcgen05 BF16-digit contraction (the precision form); "
                         "fp64: the plain method")
    ap.add_argument("--no-fp64", action="store_true",
                    help="skip the plain-FP64 comparison run of the split form")
    ap.add_argument("--workload", choices=["c3", "batched", "serving", "qu2eb"], default="c3",
                    help="c3: the headline 500-map nside-1024 analysis; batched: a mix of map "
                         "sets in CUDA-graph launches; serving: a Poisson request stream; "
                         "qu2eb: the spin-2 pair (Q/U -> E/B) in the split form")
    ap.add_argument("--pol-maps", type=int, default=200,
                    help="qu2eb: Q/U map pairs per step")
    ap.add_argument("--sets", type=int, default=64, help="batched: map sets in the mix")
    ap.add_argument("--batch-io-gb", type=float, default=120.0,
                    help="batched: inputs and outputs per graph group")
    ap.add_argument("--batch-ws-gb", type=float, default=48.0,
                    help="batched: workspace budget of each group's batch")
    ap.add_argument("--max-maps", type=int, default=None,
                    help="batched/serving: upper end of the uniform nmaps draw")
    ap.add_argument("--max-nside", type=int, default=1024,
                    help="batched/serving: upper end of the log-uniform nside draw")
    ap.add_argument("--requests", type=int, default=2000, help="serving: requests")
    ap.add_argument("--rate", type=float, default=200.0, help="serving: mean arrivals per s")
    ap.add_argument("--budget-gb", type=float, default=150.0, help="serving: HBM budget")
    ap.add_argument("--nside2048-maps", type=int, default=16,
                    help="serving: cap on nmaps at nside 2048 (a 256-map Q/U request there is "
                         "206 GB of input maps, more than the device or host holds)")
    a = ap.parse_args()
    if a.lmax is None:
        a.lmax = 2 * a.nside - 1
    if a.warmup < 3 and a.impl == "ours":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    return a


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(prefix="clocks_", suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, power = [], [], []
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                    power.append(float(parts[3]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "power_w_max": max(power), "samples": len(sm), "reasons": sorted(reasons)}


# ---------------------------------------------------------------- inputs
def device_alm(nside, lmax, nmaps, seed, device):
    """Gaussian square-real alm (L, L, nmaps) on the device, C_l = l^-2 (l >= 1),
    a00 = 0: N(0, C_l) at m = 0 and N(0, C_l/2) per component at m > 0."""
    import torch
    L = lmax + 1
    l = torch.arange(L, dtype=torch.float64, device=device)
    cl = torch.where(l > 0, 1.0 / torch.clamp(l, min=1.0) ** 2, torch.zeros_like(l))
    c = torch.arange(L, device=device).view(L, 1)          # column
    r = torch.arange(L, device=device).view(1, L)          # row
    # Re of m = c at row l = r (r >= c); Im of m = L - c at l = r + m (r < c)
    m_im = L - c
    l_of = torch.where(r >= c, r, r + m_im)
    half = torch.where((r >= c) & (c == 0), torch.ones_like(r, dtype=torch.float64),
                       torch.full_like(r, 0.5, dtype=torch.float64))
    sd = torch.sqrt(cl[l_of.clamp(max=lmax)] * half)
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    alm = torch.randn((L, L, nmaps), dtype=torch.float64, device=device, generator=g)
    alm *= sd.unsqueeze(-1)
    return alm


# ---------------------------------------------------------------- CPU baseline
class CpuBatchTimer:
    """Times the reference algorithm on the host cores in the reference's own batch shape.

    The reference puts every map of the batch into the M dimension of one DGEMM per order m
    and per Re/Im part (sht_core.f90:51-57, 80-86), computes the recursion once per m for
    the whole batch (get_plm_recursive.f90:17-136) and the ring FFTs per map
    (compute_fft.f90:71-110, MKL DFTI batched per ring length).  One sample (one `run()`):
      * the ring FFTs of `fft_maps` maps (scipy.fft on views of the maps, all cores: the
        belt's equal-length rings in one batched call, each cap ring in one call);
      * every `m_stride`-th order m: the recursion (oracle/plm.c, all cores), the gather of
        the FFT bins into the FFT matrix for `gather_maps` maps (oracle/plm.c, OpenMP, bins in
        the reference's map-fastest order, so each ring's bins are rows of maps) and the two
        DGEMMs with M = all `nmaps` maps (NumPy/OpenBLAS, all cores) on an (nmaps x rlen)
        FFT matrix.
    The batch time is the FFT scaled by nmaps / fft_maps, the gather by nmaps / gather_maps
    and m_stride, and the recursion and DGEMM times (both already at the batch's shape) by
    m_stride; `seconds` is the wall time the sample really took."""

    def __init__(self, nside, lmax, nmaps, ring_tab, fft_maps=8, gather_maps=64, m_stride=16,
                 maps=None):
        from oracle import OracleSHT
        self.threads = os.cpu_count() or 1
        self.o = OracleSHT(nside, lmax, ring_tab=ring_tab, fft_workers=self.threads)
        self.nside, self.lmax, self.nmaps = nside, lmax, nmaps
        self.m_stride = m_stride
        rng = np.random.default_rng(2)
        npix = 12 * nside * nside
        if maps is None:
            maps = rng.standard_normal((npix, fft_maps))
        self.maps = np.asfortranarray(maps[:, :fft_maps])
        self.fft_maps = self.maps.shape[1]
        # FFT bins in the reference's order (map index fastest) for the gather, and the FFT
        # matrix of the whole batch for one m (values do not change the timings)
        self.gather_maps = min(gather_maps, nmaps)
        self.buffT = np.full((npix, self.gather_maps), 1.0)
        self.A = rng.standard_normal((2, nmaps, self.o.nring))
        i1, nfft = self.o.i1, self.o.nfft
        belt = np.nonzero(nfft == 4 * nside)[0]
        self.belt = (int(i1[belt[0]]), len(belt))
        assert int(i1[belt[-1]]) + 4 * nside == self.belt[0] + 4 * nside * len(belt)
        self.cap = [(int(i1[i]), int(nfft[i])) for i in range(len(nfft)) if nfft[i] != 4 * nside]
        # the gather's bin and phase tables, which the reference computes once at set-up
        self.tables = {m: self.o.fft2mat_tables(m) for m in range(0, lmax + 1, m_stride)}

    def ring_ffts(self):
        import scipy.fft
        x = self.maps.T                          # (k, npix), each map contiguous
        k, n4 = x.shape[0], 4 * self.nside
        b0, nb = self.belt
        out = scipy.fft.rfft(x[:, b0:b0 + nb * n4].reshape(k, nb, n4), axis=-1,
                             workers=self.threads)
        for a, n in self.cap:
            out = scipy.fft.rfft(x[:, a:a + n], axis=-1, workers=self.threads)
        return out

    def run(self):
        o, k = self.o, self.fft_maps
        t0 = time.perf_counter()
        self.ring_ffts()
        t1 = time.perf_counter()
        t_plm = t_gather = t_gemm = 0.0
        for m in range(0, self.lmax + 1, self.m_stride):
            n, i0, rlen, i1, p1, p2 = o.locations(m)
            ta = time.perf_counter()
            plm = o.plm(m)
            tb = time.perf_counter()
            o.fft2mat_c(self.buffT, m, self.tables[m])
            tc = time.perf_counter()
            self.A[0, :, :rlen] @ plm
            if m > 0:
                self.A[1, :, :rlen] @ plm
            td = time.perf_counter()
            t_plm += tb - ta
            t_gather += tc - tb
            t_gemm += td - tc
        seconds = time.perf_counter() - t0
        kg = self.gather_maps
        phases = {"fft": (t1 - t0) * self.nmaps / k,
                  "gather": t_gather * self.nmaps / kg * self.m_stride,
                  "plm": t_plm * self.m_stride, "gemm": t_gemm * self.m_stride}
        batch_s = sum(phases.values())
        return {"value": self.nmaps / batch_s, "unit": UNIT, "cores": self.threads,
                "kind": "port", "seconds": seconds, "batch_s_extrapolated": batch_s,
                "sample": (f"one sample = the recursion and two DGEMMs with M = {self.nmaps} "
                           f"maps (the reference's batch shape) and the FFT-matrix gather of "
                           f"{kg} maps at every {self.m_stride}th m, the ring FFTs of {k} maps; "
                           f"batch time = FFT x {self.nmaps}/{k} + gather x {self.nmaps}/{kg} "
                           f"x {self.m_stride} + recursion and DGEMMs x {self.m_stride}"),
                "phase_s": {kk: round(v, 3) for kk, v in phases.items()}}


def reference_arm(args, rank, world):
    if rank != 0:
        return
    golden = np.load(ROOT / "tests" / "golden" / "ring_skip.npz")
    ring_tab = golden[f"ns_{args.nside}"][:args.lmax + 1]
    timer = CpuBatchTimer(args.nside, args.lmax, args.nmaps, ring_tab)
    vals = []
    t_all = time.perf_counter()
    for it in range(args.warmup + args.steps):
        r = timer.run()
        if it >= args.warmup:
            vals.append(r)
    wall = time.perf_counter() - t_all
    v = statistics.median([r["value"] for r in vals])
    sec = statistics.mean([r["seconds"] for r in vals])
    last = vals[-1]
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * sec, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": last["cores"], "kind": "port",
                         "sample": last["sample"]},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "step_timing": {"ms_per_step": "wall time of one sample (measured)",
                        "batch_s_extrapolated": statistics.median(
                            [r["batch_s_extrapolated"] for r in vals]),
                        "value": f"{args.nmaps} maps / batch_s_extrapolated",
                        "wall_s_all_steps": round(wall, 2),
                        "phase_s": last["phase_s"]},
        "note": ("reference CPU build (Fortran/OpenMP + MKL) cannot be compiled here; this is "
                 "the oracle restatement of its algorithm, timed in the reference's batch "
                 "shape (DGEMM M = all maps)"),
    }
    print(json.dumps(line), flush=True)


def workload_config(args):
    method = ("split-precision form (BF16 digit UMMAs on tcgen05, FP64 recursion, "
              "ring FFT in df64 = FP32-pair arithmetic)"
              if getattr(args, "precision", "fp64") == "split" else "plain FP64 method")
    return {"workload": (f"t2alm (map2alm) of {args.nmaps} T maps per GPU, nside {args.nside}, "
                         f"lmax {args.lmax}, {method}"),
            "nside": args.nside, "lmax": args.lmax, "nmaps_per_gpu": args.nmaps,
            "method": getattr(args, "precision", "fp64"), "niter": 0,
            "inputs": "Gaussian alm, C_l ~ l^-2 (seed 2), synthesised to maps on the device",
            "l2": "inputs larger than L2 (maps resident in HBM), no flush",
            "parallelism": f"replicas x{args.gpus}"}


# ---------------------------------------------------------------- our arm
def timed_steps(lib, sht, maps, steps, warmup, world, dist, dev, local, sample_clocks=True):
    """W untimed + K timed t2alm steps on the plan's stream; per-kernel CUDA-event
    times from the library's profiler over the timed region."""
    import ctypes as C
    import torch
    from fastsht_gb300 import _lib
    out = None
    for _ in range(warmup):
        out = sht.t2alm(maps)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    lib.fsht_profile_enable(sht._plan, 1)
    _lib.call("fsht_profile_read", sht._plan, 0, None, None)     # clear
    clocks = ClockSampler(local) if sample_clocks else None
    if clocks:
        clocks.start()
    torch.cuda.synchronize()
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(steps):
        out = sht.t2alm(maps)
    e1.record(s)
    torch.cuda.synchronize()
    clk = clocks.stop() if clocks else None
    ms = e0.elapsed_time(e1)
    counts = (C.c_int * _lib.KCAT_COUNT)()
    kms = (C.c_double * _lib.KCAT_COUNT)()
    _lib.call("fsht_profile_read", sht._plan, _lib.KCAT_COUNT, counts, kms)
    lib.fsht_profile_enable(sht._plan, 0)
    if world > 1:
        ms = max_over_ranks(ms, dist, dev)
        dist.barrier()
    per_kernel = {}
    for i, name in enumerate(_lib.KCAT_NAMES):
        if counts[i]:
            per_kernel[name] = {"launches": counts[i], "ms_total": round(kms[i], 3),
                                "share": round(kms[i] / ms, 4) if ms else None}
    launches = int(sum(counts[i] for i in range(_lib.KCAT_COUNT)))
    return ms, out, per_kernel, [kms[i] for i in range(_lib.KCAT_COUNT)], launches, clk


def rel_err_per_map(a, ref):
    """max over maps of max_{l,m}|a - ref| / max|ref| (device tensors (nmaps, L, L))."""
    import torch
    n = ref.shape[0]
    d = (a - ref).abs().reshape(n, -1).amax(dim=1)
    s = ref.abs().reshape(n, -1).amax(dim=1)
    return float((d / s).max().item())


def ours(args, rank, world, local):
    import ctypes as C
    import torch
    import torch.distributed as dist
    from fastsht_gb300 import SHT, _lib

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = _lib.load(build_if_missing=True)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)

    nside, lmax, nmaps = args.nside, args.lmax, args.nmaps
    npix = 12 * nside * nside
    peak64 = C.c_double()
    _lib.call("fsht_measure_fp64_peak", C.byref(peak64))
    peak32 = C.c_double()
    _lib.call("fsht_measure_fp32_peak", C.byref(peak32))
    peak_dmma = C.c_double()
    _lib.call("fsht_measure_dmma_peak", C.byref(peak_dmma))
    umma = {}
    if args.precision == "split":
        for ncol in (128, 256):
            r = C.c_double()
            _lib.call("fsht_measure_umma_rate", ncol, C.byref(r))
            umma[ncol] = r.value
    peaks = {}
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = json.loads(pk.read_text())

    sht64 = SHT(nside, lmax, nmaps, device=local)
    alm_true = device_alm(nside, lmax, nmaps, 2 + rank, dev)
    maps = sht64.alm2t(alm_true.permute(2, 1, 0))        # (npix, nmaps) Fortran view
    del alm_true
    torch.cuda.synchronize()
    sht = sht64 if args.precision == "fp64" else SHT(nside, lmax, nmaps, device=local,
                                                      precision="split")

    ms, out, per_kernel, kms, launches, clk = timed_steps(lib, sht, maps, args.steps,
                                                          args.warmup, world, dist, dev, local)
    ms_per_step = ms / args.steps
    value = world * nmaps * args.steps / (ms / 1000.0)
    kchunk = sht.plan_info()["maps_per_chunk"]
    fl_step = flop_per_map(nside, lmax) * nmaps
    # dominant kernel of the step and its roofline
    names = _lib.KCAT_NAMES
    top = max(range(len(names)), key=lambda i: kms[i])
    fft_ms, ana_ms = kms[0], kms[2]
    fft_bytes = 16.0 * npix * nmaps * args.steps
    # The FP64 ring FFT is bound by the FP64 pipe (GB300: ~1.25 TFLOP/s FP64 against
    # 6.8 TB/s of HBM, 0.09 flop/B; the FFT does ~3 flop/B), so its roofline is FP64:
    # algorithmic flops = 5 n log2 n per complex length-n ring DFT (N + iS packed).
    fft_alg = fft_alg_flop_per_map(nside) * nmaps * args.steps
    fft_traffic = None
    tf_fft = ROOT / "profiles" / "traffic.json"
    if tf_fft.exists():
        tr = json.loads(tf_fft.read_text()).get(
            "ring_fft_fwd_df" if args.precision == "split" else "ring_fft_fwd")
        if tr and tr.get("bytes_per_map"):
            fft_traffic = tr["bytes_per_map"] * kchunk
    roof_fft = {"bound": "fp64", "kernel": "k_ring_fft_fwd",
                "achieved": fft_alg / (fft_ms / 1000.0) / 1e12 if fft_ms > 0 else None,
                "peak": peak64.value, "unit": "TFLOP/s",
                "peak_source": ("DFMA loop measured by bench.py on this GPU "
                                "(fsht_measure_fp64_peak); MEASURED_PEAKS.json holds HBM and "
                                "BF16 figures only"),
                "algorithmic_flop_per_map": fft_alg_flop_per_map(nside),
                "traffic": fft_traffic,
                "hbm": {"achieved_gbs": fft_bytes / (fft_ms / 1000.0) / 1e9 if fft_ms > 0 else None,
                        "peak_gbs": peaks.get("hbm_gbs", 6800.0),
                        "algorithmic_bytes_per_map": 16.0 * npix}}
    if roof_fft["achieved"] and args.precision == "split":
        # The split form's FFT runs in df64 arithmetic on the FP32 pipe: its roofline is the
        # FP32 instruction rate (FFMA loop measured in this run), its work the modelled df64
        # FP32 instructions; the FP64-equivalent rate is kept beside it.
        fp64_equiv = roof_fft["achieved"]
        ins = fft_df_instr_per_map(nside) * nmaps * args.steps / (fft_ms / 1000.0)
        roof_fft.update({
            "bound": "fp32", "kernel": "k_ring_fft_fwd_df (df64 arithmetic)",
            "achieved": ins / 1e12, "peak": peak32.value / 2, "unit": "Tinstr/s (FP32 pipe)",
            "frac": ins / 1e12 / (peak32.value / 2),
            "peak_source": ("FFMA loop measured by bench.py on this GPU "
                            "(fsht_measure_fp32_peak, TFLOP/s / 2 = FP32 instructions/s); "
                            "MEASURED_PEAKS.json holds HBM and BF16 figures only"),
            "fp32_instr_per_map": fft_df_instr_per_map(nside),
            "fp64_equivalent_tflops": fp64_equiv,
            "note": ("achieved = df64 FP32 instructions of the radix passes, Bluestein chirps "
                     "and filter (model: 16 per lazy complex df64 add, 32 per lazy complex "
                     "product, 6 per renormalised store) / CUDA-event time; loads, stores, "
                     "index math, conversions and the fold are extra issue slots not counted")})
        roof_fft["hbm"]["frac"] = roof_fft["hbm"]["achieved_gbs"] / roof_fft["hbm"]["peak_gbs"]
    elif roof_fft["achieved"]:
        roof_fft["frac"] = roof_fft["achieved"] / roof_fft["peak"]
        roof_fft["hbm"]["frac"] = roof_fft["hbm"]["achieved_gbs"] / roof_fft["hbm"]["peak_gbs"]
        dp = fft_dp_ops_per_map(nside) * nmaps * args.steps / (fft_ms / 1000.0)
        roof_fft["fp64_pipe"] = {"dp_instr_per_map": fft_dp_ops_per_map(nside),
                                 "achieved_g_per_s": dp / 1e9,
                                 "peak_g_per_s": peak64.value * 1e12 / 2 / 1e9,
                                 "frac": dp / (peak64.value * 1e12 / 2),
                                 "note": "FP64 instructions executed (radix passes, Bluestein "
                                         "chirps and filter; an FMA counts once) over the DFMA "
                                         "instruction rate measured in this run"}
    ana_tf = fl_step * args.steps / (ana_ms / 1000.0) / 1e12 if ana_ms > 0 else None
    traffic = None          # bytes per chunk of maps (all of its launches)
    tf = ROOT / "profiles" / "traffic.json"
    if tf.exists():
        tr = json.loads(tf.read_text()).get(
            "legendre_analysis_split" if args.precision == "split" else "legendre_analysis_fp64")
        if tr and tr.get("bytes_per_map"):
            traffic = tr["bytes_per_map"] * kchunk
        elif tr and tr.get("bytes_per_call") and tr.get("maps") == kchunk:
            traffic = tr["bytes_per_call"]          # not per map: measured at this chunk size
    if args.precision == "split":
        bf = peaks.get("bf16_tflops", 1900.0)
        ex_tf = 10 * ana_tf if ana_tf else None
        roof_ana = {"bound": "tensor", "kernel": "k_split_gemm (tcgen05 BF16 digit UMMAs)",
                    "achieved": ana_tf, "peak": bf, "unit": "TFLOP/s",
                    "frac": ana_tf / bf if ana_tf else None,
                    "peak_source": ("MEASURED_PEAKS.json bf16_tflops (measured)"
                                    if "bf16_tflops" in peaks else "fallback 1900 TFLOP/s"),
                    "algorithmic_flop_per_chunk": flop_per_map(nside, lmax) * kchunk,
                    "executed_tensor_tflops": ex_tf,
                    "executed_frac": ex_tf / bf if ex_tf else None,
                    "umma_tile_ceiling": {
                        "n128_tflops": umma.get(128), "n256_tflops": umma.get(256),
                        "executed_frac_of_n128": (ex_tf / umma[128]
                                                  if ex_tf and umma.get(128) else None),
                        "note": ("the contraction's k-step (ten 128 x N x 16 BF16 UMMAs) issued "
                                 "back to back from shared memory, one CTA per SM "
                                 "(fsht_measure_umma_rate), measured in this run: the ceiling "
                                 "of the 128-column tile the kernel uses, and of a 256-column "
                                 "one")},
                    "traffic": traffic,
                    "note": ("achieved counts algorithmic FLOP (4 nside (lmax+1)(lmax+2) per map); "
                             "the kernel executes 10 BF16 digit products per algorithmic FMA "
                             "(executed_*); one chunk of maps is several wave launches, traffic "
                             "is per chunk")}
    else:
        roof_ana = {"bound": "fp64", "kernel": "k_analysis_fp64<0>", "achieved": ana_tf,
                    "peak": peak64.value, "unit": "TFLOP/s",
                    "frac": ana_tf / peak64.value if ana_tf else None,
                    "peak_source": ("DFMA loop measured by bench.py on this GPU "
                                    "(fsht_measure_fp64_peak); MEASURED_PEAKS.json holds HBM "
                                    "and BF16 figures only"),
                    "algorithmic_flop_per_launch": flop_per_map(nside, lmax) * kchunk,
                    "traffic": traffic}
    if names[top] == "ring_fft_fwd" and fft_ms > 0:
        # The dominant kernel against the measured HBM copy rate (MEASURED_PEAKS.json): its
        # algorithmic bytes are the maps read and the phase matrix written, 16 npix per map.
        # The transform is bound by instruction issue on the FP32 pipe (compute_bound below),
        # not by HBM, so this fraction is low by construction; traffic = ncu DRAM bytes per
        # map (profiles/traffic.json) times the maps of the chunk.
        hbm_peak = peaks.get("hbm_gbs")
        ach = fft_bytes / (fft_ms / 1000.0) / 1e9
        roof = {"bound": "hbm", "kernel": roof_fft["kernel"], "achieved": ach,
                "peak": hbm_peak or 6800.0, "unit": "GB/s",
                "frac": ach / (hbm_peak or 6800.0),
                "peak_source": ("MEASURED_PEAKS.json hbm_gbs (measured)" if hbm_peak
                                else "fallback 6.8 TB/s"),
                "traffic": fft_traffic,
                "algorithmic_bytes_per_map": 16.0 * npix,
                "compute_bound": {k: roof_fft.get(k) for k in ("bound", "achieved", "peak",
                                                                "unit", "frac")},
                "note": ("achieved = 16 npix bytes per map (maps read + phase matrix written) "
                         "over the summed CUDA-event time of the forward FFT launches; the "
                         "kernel is bound by FP32 issue (compute_bound, df64 arithmetic)")}
    else:
        roof = roof_ana
    roof = dict(roof, dominant_kernel_share=per_kernel.get(names[top], {}).get("share"))

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else "bf16x4-split of f64 (FP32 accum)",
            "data": "synthetic", "config": workload_config(args), "clocks": clk,
            "gpu_launches": launches, "per_kernel": per_kernel, "roofline": roof,
            "roofline_fft": roof_fft, "roofline_contraction": roof_ana,
            "fp64_peak_tflops": peak64.value, "fp32_peak_tflops": peak32.value,
            "fp64_units": {"dfma_tflops": peak64.value, "dmma_tflops": peak_dmma.value,
                           "dmma_below_dfma": peak_dmma.value < peak64.value,
                           "note": ("FP64 FMA loop (fsht_measure_fp64_peak) against an "
                                    "mma.sync.m8n8k4 f64 loop (fsht_measure_dmma_peak), both "
                                    "measured in this run: the plain contraction uses the "
                                    "faster of the two units, DFMA")}}

    # -------- e2e through the public API with host (pinned) buffers (first, while the
    # device holds only this form's buffers)
    if not args.no_e2e:
        ke = args.e2e_maps or nmaps
        sh = sht if ke == nmaps else SHT(nside, lmax, ke, device=local, precision=args.precision)
        line["e2e"] = e2e(sh, maps, ke, args, world)
        sh.release_staging()
        torch.cuda.empty_cache()
    # -------- the plain FP64 path on the same maps (precision reference + speed ratio)
    if args.precision == "split" and not args.no_fp64:
        ms64, out64, pk64, kms64, _, _ = timed_steps(lib, sht64, maps, 1, 1, world, dist, dev,
                                                     local, sample_clocks=False)
        v64 = world * nmaps / (ms64 / 1000.0)
        sd = float(maps.std().item())

        def maxabs_minus(rt, ref=None, chunk=50):
            # max |rt - ref| over (npix, nmaps) Fortran views, a few maps at a time
            best = 0.0
            for c0 in range(0, nmaps, chunk):
                d = rt[:, c0:c0 + chunk] if ref is None else rt[:, c0:c0 + chunk] - ref[:, c0:c0 + chunk]
                best = max(best, float(d.abs().max().item()))
            return best

        rt = sht64.alm2t(out)
        res_split = maxabs_minus(rt, maps) / sd
        del rt
        rt = sht64.alm2t(out64)
        res_64 = maxabs_minus(rt, maps) / sd
        del rt
        rt = sht64.alm2t(out - out64)          # linearity: the precision-induced part
        res_diff = maxabs_minus(rt) / sd
        del rt
        out64_sample = out64[:min(args.cpu_maps, nmaps)].cpu().numpy()
        line["fp64_plain"] = {
            "value": v64, "unit": UNIT, "ms_per_step": ms64, "per_kernel": pk64,
            "split_speedup": value / v64,
            "max_rel_alm_err_split_vs_fp64": rel_err_per_map(out, out64),
            "roundtrip_map_residual_split": res_split,
            "roundtrip_map_residual_fp64": res_64,
            "roundtrip_split_vs_fp64": res_diff,
            "metric_note": ("alm error = max over maps of max_lm|a - a_fp64| / max_lm|a_fp64|; "
                            "map residuals = max|T' - T| / std(T) (the reference's map metric); "
                            "the round-trip residual of both forms is the niter = 0 quadrature "
                            "error, the split-vs-fp64 term is the precision-induced part")}
        del out64
        torch.cuda.empty_cache()
    # -------- one refinement step (niter = 1) in the split form, against the plain path
    # with the same niter on the first maps of the batch
    ring_tab = sht.ring_skip()
    if args.precision == "split" and not args.no_fp64:
        # the refinement plan holds two phase matrices per map: the niter-0 split plan is
        # released first so that it gets the library's default split workspace (two chunks
        # of the 500-map batch, the recursion once per chunk and pass)
        sht.close()
        torch.cuda.empty_cache()
        sr = SHT(nside, lmax, nmaps, niter=1, device=local, precision="split")
        ms_r, out_r, pk_r, _, _, _ = timed_steps(lib, sr, maps, 1, 1, world, dist, dev, local,
                                                 sample_clocks=False)
        sr.close()
        ks = min(64, nmaps)
        s64r = SHT(nside, lmax, ks, niter=1, device=local)
        out64r = s64r.t2alm(maps[:, :ks])
        vr = world * nmaps / (ms_r / 1000.0)
        sd = float(maps[:, :ks].std().item())
        first = out_r.permute(2, 1, 0)[..., :ks].contiguous().permute(2, 1, 0)   # (ks, L, L) F-order
        res_r = float((s64r.alm2t(first) - maps[:, :ks]).abs().max().item()) / sd
        del first
        line["refined"] = {
            "niter": 1, "value": vr, "unit": UNIT, "ms_per_step": ms_r, "per_kernel": pk_r,
            "speedup_vs_plain_niter0": vr / line["fp64_plain"]["value"] if "fp64_plain" in line else None,
            "max_rel_alm_err_vs_fp64_niter1": rel_err_per_map(out_r[:ks], out64r),
            "roundtrip_map_residual": res_r, "maps_checked": ks,
            "note": ("one Jacobi refinement step: split synthesis, FP64 Fourier-space residual, "
                     "split analysis added; the error is against the plain path with niter = 1")}
        s64r.close()
        del out_r, out64r
        torch.cuda.empty_cache()
    # -------- CPU baseline and parity sample (rank 0, N = 1)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import OracleSHT
        k = min(args.cpu_maps, nmaps)
        maps_np = np.asfortranarray(maps[:, :k].cpu().numpy())
        timer = CpuBatchTimer(nside, lmax, nmaps, ring_tab, maps=maps_np)
        timer.run()                               # warm-up (BLAS threads, first touch)
        line["cpu_baseline"] = timer.run()
        del timer
        alm_ref = OracleSHT(nside, lmax, ring_tab=ring_tab).t2alm(maps_np)
        sc = np.abs(alm_ref).reshape(k, -1).max(axis=1)

        def err_vs_oracle(got):
            return float((np.abs(got - alm_ref).reshape(k, -1).max(axis=1) / sc).max())

        par = {"maps_checked": k,
               "metric": "max over maps of max_lm |a - a_oracle| / max_lm |a_oracle|"}
        if args.precision == "split":
            par["max_rel_alm_err_split_vs_oracle"] = err_vs_oracle(out[:k].cpu().numpy())
            par["tolerance_split"] = 1e-7
            if "fp64_plain" in line:
                par["max_rel_alm_err_fp64_vs_oracle"] = err_vs_oracle(out64_sample)
                par["tolerance_fp64"] = 1e-11
        else:
            par["max_rel_alm_err_fp64_vs_oracle"] = err_vs_oracle(out[:k].cpu().numpy())
            par["tolerance_fp64"] = 1e-11
        line["parity"] = par
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def gpu_local_cpus(dev):
    """Host cores of the GPU's own NUMA node (sysfs local_cpulist of its PCI device, found
    through the device UUID in nvidia-smi), or None."""
    import torch
    try:
        uuid = str(torch.cuda.get_device_properties(dev).uuid)
        out = subprocess.run(["nvidia-smi", "--query-gpu=uuid,pci.bus_id", "--format=csv,noheader"],
                             capture_output=True, text=True, timeout=30).stdout
        for line in out.splitlines():
            u, bus = [x.strip() for x in line.split(",")]
            if u.lower().endswith(uuid.lower()) or uuid.lower() in u.lower():
                dom, rest = bus.split(":", 1)
                path = f"/sys/bus/pci/devices/{int(dom, 16):04x}:{rest.lower()}/local_cpulist"
                cpus = set()
                for part in Path(path).read_text().strip().split(","):
                    lo, _, hi = part.partition("-")
                    cpus.update(range(int(lo), int(hi or lo) + 1))
                return cpus or None
    except Exception:
        return None
    return None


def e2e(sht, maps_dev, ke, args, world):
    """Same metric through SHT.t2alm with host buffers: every step moves the maps
    host->device (read in place by the FFT over the host link, the API's default for pinned
    buffers; the staged copy is timed beside it) and the alm device->host (pinned buffers,
    reused).  The process runs on the
    GPU's own NUMA node's cores while it allocates them (first touch places the pinned pages
    there), as a NUMA-aware user would."""
    import torch
    local = gpu_local_cpus(maps_dev.device)
    saved = os.sched_getaffinity(0)
    if local:
        try:
            os.sched_setaffinity(0, local)
        except OSError:
            local = None
    try:
        return _e2e_run(sht, maps_dev, ke, args, world, local)
    finally:
        os.sched_setaffinity(0, saved)


def _e2e_run(sht, maps_dev, ke, args, world, local):
    import torch
    from fastsht_gb300 import pinned_empty
    npix = sht.npix
    L = sht.lmax + 1
    # page-locked host buffers from the library (cudaHostAlloc), as a user of the host API
    maps_np = pinned_empty((npix, ke))           # Fortran order
    host = torch.from_numpy(maps_np.T)           # (ke, npix) view of the same memory
    host.copy_(maps_dev.T[:ke])
    out_np = pinned_empty((ke, L, L))            # Fortran order
    out_t = torch.from_numpy(out_np.T)           # (L, L, ke) view

    def timed(mode, detail):
        # host_read: "direct" = the FFT reads the pinned maps in place over the host link,
        # "staged" = the maps are copied to device memory in sub-batches first
        import ctypes as C
        from fastsht_gb300 import _lib
        _lib.call("fsht_plan_set_host_read", sht._plan,
                  {"staged": 0, "direct": 1, "direct_chunked": 2}[mode])
        sht.host_read = mode
        sht.t2alm(maps_np, alms_in=out_np)       # warm-up
        torch.cuda.synchronize()
        detail["device_free_gb"] = round(torch.cuda.mem_get_info()[0] / 1e9, 1)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            sht.t2alm(maps_np, alms_in=out_np)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        # one more step with the per-kernel CUDA-event profiler: where the step's time goes
        _lib.load().fsht_profile_enable(sht._plan, 1)
        _lib.call("fsht_profile_read", sht._plan, 0, None, None)
        sht.t2alm(maps_np, alms_in=out_np)
        cnt = (C.c_int * _lib.KCAT_COUNT)()
        kms = (C.c_double * _lib.KCAT_COUNT)()
        _lib.call("fsht_profile_read", sht._plan, _lib.KCAT_COUNT, cnt, kms)
        _lib.load().fsht_profile_enable(sht._plan, 0)
        detail["per_kernel_ms"] = {n: round(kms[i], 1) for i, n in enumerate(_lib.KCAT_NAMES)
                                   if cnt[i]}
        return dt

    mode0 = sht.host_read
    det_staged, det_direct, det_chunked = {}, {}, {}
    try:
        dt_staged = timed("staged", det_staged)
        dt_chunked = timed("direct_chunked", det_chunked)
        dt = timed("direct", det_direct)
    finally:
        from fastsht_gb300 import _lib
        _lib.call("fsht_plan_set_host_read", sht._plan,
                  {"staged": 0, "direct": 1, "direct_chunked": 2}[mode0])
        sht.host_read = mode0
    # the same pinned buffers copied by torch (first 64 maps): a reference for the host link's
    # rate beside the library's own transfers (in-place reads by the FFT, or cudaMemcpyAsync
    # calls on its copy stream)
    kc = min(ke, 64)
    dmaps = torch.empty((kc, npix), dtype=torch.float64, device=maps_dev.device)
    dalm = torch.empty((kc, L * L), dtype=torch.float64, device=maps_dev.device)
    halm = out_t.reshape(-1)[: kc * L * L].view(kc, L * L)
    for _ in range(2):                           # the second pass is the measurement
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        dmaps.copy_(host[:kc], non_blocking=True)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        halm.copy_(dalm, non_blocking=True)
        torch.cuda.synchronize()
        t3 = time.perf_counter()
    del dmaps, dalm
    return {"value": world * ke * args.steps / dt, "unit": UNIT,
            "h2d_bytes_per_step": ke * npix * 8, "d2h_bytes_per_step": ke * L * L * 8,
            "maps_per_step": ke, "ms_per_step": 1000.0 * dt / args.steps,
            "host_read": ("direct: the forward FFT reads the pinned maps in place over the "
                          "host link (the API's default for pinned_empty buffers)"),
            "detail": det_direct,
            "chunked": {"value": world * ke * args.steps / dt_chunked, "unit": UNIT,
                        "ms_per_step": 1000.0 * dt_chunked / args.steps, "detail": det_chunked,
                        "note": "host_read='direct_chunked': 128-map chunks read in place, each "
                                "chunk's contraction beside the next chunk's reads"},
            "staged": {"value": world * ke * args.steps / dt_staged, "unit": UNIT,
                       "ms_per_step": 1000.0 * dt_staged / args.steps,
                       "detail": det_staged,
                       "note": "host_read='staged': maps copied to device memory in "
                               "sub-batches, each transformed as it lands"},
            "host_cpus": ("the GPU's NUMA-local cores (%d)" % len(local)) if local else "default",
            "torch_copy_h2d_gbs": kc * npix * 8 / (t2 - t1) / 1e9,
            "torch_copy_d2h_gbs": kc * L * L * 8 / (t3 - t2) / 1e9}


# ---------------------------------------------------------------- batched form
def batched_mix(nsets, max_nside, max_maps, seed=3):
    """The batched mix: nside = 2^U{5..log2 max_nside}, lmax ~ U[2 nside, 3 nside - 1],
    nmaps ~ U[1, max_maps], even sets T-only and odd sets I/Q/U."""
    rng = np.random.default_rng(seed)
    hi = int(round(math.log2(max_nside)))
    sets = []
    for s in range(nsets):
        ns = int(2 ** rng.integers(5, hi + 1))
        lmax = int(rng.integers(2 * ns, 3 * ns))
        nm = int(rng.integers(1, max_maps + 1))
        sets.append((ns, lmax, nm, bool(s % 2)))
    return sets


def batched_groups(sets, piece_gb, group_gb):
    """The mix as graph-sized groups: each set's jobs (t2alm of I; qu2eb of Q/U for I/Q/U sets)
    are split along maps into pieces of at most piece_gb of inputs and outputs, and the pieces
    are packed, largest first, into groups of at most group_gb (one batch, one graph each).  The
    full mix (nmaps up to 512) is about a terabyte of maps and alm: no single graph holds it."""
    pieces = []
    for ns, lmax, nm, pol in sets:
        npix, L = 12 * ns * ns, lmax + 1
        for kind, nf in (("t2alm", 1),) + ((("qu2eb", 2),) if pol else ()):
            per_map = 8.0 * nf * (npix + L * L)
            step = max(1, int(piece_gb * 1e9 // per_map))
            for m0 in range(0, nm, step):
                k = min(step, nm - m0)
                pieces.append((kind, ns, lmax, k, per_map * k))
    pieces.sort(key=lambda t: -t[4])
    groups = []
    for pc in pieces:
        for g in groups:
            if g["bytes"] + pc[4] <= group_gb * 1e9:
                g["pieces"].append(pc)
                g["bytes"] += pc[4]
                break
        else:
            groups.append({"pieces": [pc], "bytes": pc[4]})
    return groups


def bench_batched(args, rank, world, local):
    """Every set's analysis (t2alm of I; qu2eb of Q/U for I/Q/U sets), split along maps into
    pieces and packed into groups that fit the HBM budget: each group is one batch, run as one
    CUDA-graph launch per step.  value = map.SHT/s over the whole mix (the timed graph launches
    of all groups) in the split-precision form; the same mix all-FP64 is reported beside it
    unless --no-fp64."""
    import torch
    import torch.distributed as dist
    from fastsht_gb300 import _lib
    from fastsht_gb300.batch import Batch

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    _lib.load(build_if_missing=True)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)
    max_maps = args.max_maps or 16
    sets = batched_mix(args.sets, args.max_nside, max_maps, seed=3 + rank)
    mapsht = sum(nm * (3 if pol else 1) for ns, lmax, nm, pol in sets)
    flops = sum(flop_per_map(ns, lmax) * nm * (5 if pol else 1) for ns, lmax, nm, pol in sets)
    groups = batched_groups(sets, piece_gb=24.0, group_gb=args.batch_io_gb)
    ws_budget = int(args.batch_ws_gb * 1e9)

    def build(group, precision):
        b = Batch(device=local, nslots=4, autotune=True, workspace_budget=ws_budget)
        for kind, ns, lmax, k, _ in group["pieces"]:
            j = b.add(kind, ns, lmax, k, precision=precision)
            for t in j.inputs:
                t.normal_()
        b.build()
        torch.cuda.synchronize()
        return b

    def run(b, steps, warmup):
        for _ in range(warmup):
            b.run()
        torch.cuda.synchronize()
        s = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(steps):
            b.run()
        e1.record(s)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    def all_groups(precision, steps, warmup, clocks=None):
        ms, infos, t_build = 0.0, [], 0.0
        tunings = {}
        if world > 1:
            dist.barrier()
        if clocks:
            clocks.start()
        for g in groups:
            t0 = time.perf_counter()
            b = build(g, precision)
            t_build += time.perf_counter() - t0
            ms += run(b, steps, warmup)
            infos.append(b.info())
            for t in b.tunings():
                key = f"{t['precision']} nside {t['nside']} lmax {t['lmax']}"
                tunings[key] = {k: v for k, v in t.items()
                                if k not in ("nside", "lmax", "precision")}
            b.close()
            del b
            torch.cuda.empty_cache()
        clk = clocks.stop() if clocks else None
        if world > 1:
            ms = max_over_ranks(ms, dist, dev)
        return ms, clk, infos, t_build, tunings

    ms, clk, infos, t_build, tunings = all_groups("split", args.steps, args.warmup,
                                                  ClockSampler(local))
    value = world * mapsht * args.steps / (ms / 1000.0)
    fp64 = None
    if not args.no_fp64:
        s64 = max(1, args.steps // 2)
        ms64, _, _, _, tun64 = all_groups("fp64", s64, 1)
        tunings.update(tun64)
        v64 = world * mapsht * s64 / (ms64 / 1000.0)
        fp64 = {"value": v64, "unit": UNIT, "ms_per_step": ms64 / s64, "split_speedup": value / v64}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16x4-split of f64 (FP32 accum)", "data": "synthetic",
        "config": {"workload": (f"batched form: {len(sets)} map sets, nside 2^U{{5..."
                                f"{int(round(math.log2(args.max_nside)))}}}, lmax ~ U[2 nside, "
                                f"3 nside - 1], nmaps ~ U[1, {max_maps}], even sets T, odd "
                                f"sets I/Q/U; analysis (t2alm + qu2eb); seed 3"),
                   "sets": len(sets), "maps_sht_per_step": mapsht,
                   "groups": len(groups), "pieces": sum(len(g["pieces"]) for g in groups),
                   "group_io_gb": [round(g["bytes"] / 1e9, 1) for g in groups],
                   "graphs": infos, "build_s": round(t_build, 1),
                   "grouping": (f"jobs split along maps into pieces of <= 24 GB of inputs and "
                                f"outputs, packed into groups of <= {args.batch_io_gb} GB, one "
                                f"CUDA graph per group (workspace budget {args.batch_ws_gb} GB); "
                                f"ms_per_step sums the groups' timed graph launches"),
                   "l2": "N(0,1) pixel inputs resident in HBM, no flush (sets up to "
                         f"{max(ns for ns, *_ in sets)} nside exceed L2 in total)",
                   "parallelism": f"replicas x{world}"},
        "clocks": clk,
        "flop_rate_tflops": world * flops * args.steps / (ms / 1000.0) / 1e12,
        "fp64_all": fp64,
        # launch shapes the autotuner chose per plan (FFT maps per CTA and threads; FP64 maps
        # per CTA and rings per chunk; split ring-part k-steps; 0 = the kernel's default)
        "autotuned_shapes": tunings,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


# ---------------------------------------------------------------- spin-2 pair
def bench_qu2eb(args, rank, world, local):
    """qu2eb (Q/U maps -> E/B alm, niter 0) of --pol-maps map pairs resident in HBM in the
    split form; value counts Q and U as two maps.  Inputs: Q/U synthesised from Gaussian E/B
    alm (C_l ~ l^-2, seeds 5 and 6).  The plain FP64 path runs the first 16 pairs for the error
    and the speed ratio."""
    import ctypes as C
    import torch
    import torch.distributed as dist
    from fastsht_gb300 import SHT, _lib

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = _lib.load(build_if_missing=True)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)
    nside, lmax, nmaps = args.nside, args.lmax, args.pol_maps
    sp = SHT(nside, lmax, nmaps, pol=True, device=local, precision="split")
    E0 = device_alm(nside, lmax, nmaps, 5 + rank, dev)
    B0 = device_alm(nside, lmax, nmaps, 6 + rank, dev)
    Q, U = sp.eb2qu(E0.permute(2, 1, 0), B0.permute(2, 1, 0))   # (npix, nmaps) Fortran views
    del E0, B0
    torch.cuda.synchronize()
    for _ in range(args.warmup):
        E, B = sp.qu2eb(Q, U)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    lib.fsht_profile_enable(sp._plan, 1)
    _lib.call("fsht_profile_read", sp._plan, 0, None, None)
    clocks = ClockSampler(local)
    clocks.start()
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(args.steps):
        E, B = sp.qu2eb(Q, U)
    e1.record(s)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    counts = (C.c_int * _lib.KCAT_COUNT)()
    kms = (C.c_double * _lib.KCAT_COUNT)()
    _lib.call("fsht_profile_read", sp._plan, _lib.KCAT_COUNT, counts, kms)
    lib.fsht_profile_enable(sp._plan, 0)
    if world > 1:
        ms = max_over_ranks(ms, dist, dev)
    per_kernel = {name: {"launches": counts[i], "ms_per_step": round(kms[i] / args.steps, 2)}
                  for i, name in enumerate(_lib.KCAT_NAMES) if counts[i]}
    ks = min(16, nmaps)
    p64 = SHT(nside, lmax, ks, pol=True, device=local)
    p64.qu2eb(Q[:, :ks], U[:, :ks])                      # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    E64, B64 = p64.qu2eb(Q[:, :ks], U[:, :ks])
    torch.cuda.synchronize()
    t64 = time.perf_counter() - t0
    err = max(rel_err_per_map(E[:ks], E64), rel_err_per_map(B[:ks], B64))
    value = world * 2 * nmaps * args.steps / (ms / 1000.0)
    v64 = 2 * ks / t64
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16x4-split of f64 (FP32 accum)", "data": "synthetic",
        "config": {"workload": (f"qu2eb (spin-2 Q/U -> E/B, niter 0) of {nmaps} map pairs at "
                                f"nside {nside} / lmax {lmax}, split form; Q and U count as two "
                                f"maps"),
                   "l2": "inputs resident in HBM, larger than L2, no flush",
                   "parallelism": f"replicas x{world}"},
        "clocks": clk, "per_kernel": per_kernel,
        "fp64_plain": {"value": v64, "unit": UNIT, "maps_timed": 2 * ks,
                       "split_speedup": value / v64 / world,
                       "max_rel_alm_err_split_vs_fp64": err, "tolerance": 1e-7},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


# ---------------------------------------------------------------- serving form
def bench_serving(args, rank, world, local):
    """Open-loop Poisson stream into fastsht_gb300.serve.Server: map2alm or alm2map, T or
    Q/U with equal odds, nside = 2^U{6..log2 max_nside}, lmax = 2 nside, nmaps ~
    U[1, max_maps], FP64 or split per request, seed 4.  Inputs are device-resident views of
    one pre-generated N(0,1) pool per nside (no per-request copies); the client discards the
    results.  value = map.SHT/s over the run; p50/p99 latency from arrival to result."""
    import torch
    from fastsht_gb300 import _lib
    from fastsht_gb300.serve import Server

    if rank != 0:
        return
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    _lib.load(build_if_missing=True)
    max_maps = args.max_maps or 8
    rng = np.random.default_rng(4)
    hi = int(round(math.log2(args.max_nside)))
    kinds = ["t2alm", "alm2t", "qu2eb", "eb2qu"]
    cap = {2048: args.nside2048_maps}
    reqs = []
    t = 0.0
    for _ in range(args.requests):
        t += rng.exponential(1.0 / args.rate)
        ns = int(2 ** rng.integers(6, hi + 1))
        nm = int(rng.integers(1, max_maps + 1))
        reqs.append((t, kinds[int(rng.integers(0, 4))], ns, 2 * ns, min(nm, cap.get(ns, nm)),
                     "split" if rng.integers(0, 2) else "fp64"))
    # one flat N(0,1) pool per nside and field, large enough for the biggest request of either
    # direction: a request of nm maps views its first nm maps' (or nm alm sets') worth of
    # values in the layout it needs, so requests share the pool without copies
    pools = {}
    for ns in sorted({r[2] for r in reqs}):
        L = 2 * ns + 1
        pm = max(r[4] for r in reqs if r[2] == ns)
        gm = torch.Generator(device=dev)
        gm.manual_seed(ns)
        pools[ns] = torch.randn((2, pm * max(12 * ns * ns, L * L)), dtype=torch.float64,
                                device=dev, generator=gm)

    def inputs(kind, ns, nm):
        pool = pools[ns]
        nf = 2 if kind in ("qu2eb", "eb2qu") else 1
        if kind in ("t2alm", "qu2eb"):
            npix = 12 * ns * ns
            return [pool[f, :nm * npix].view(nm, npix) for f in range(nf)]
        L = 2 * ns + 1
        return [pool[f, :L * L * nm].view(L, L, nm) for f in range(nf)]

    budget = args.budget_gb * 1e9
    # the client discards results (it measures the service): outputs leave the budget as
    # soon as their request completes
    srv = Server(hbm_budget=budget, nslots=8, device=local, discard_outputs=True)
    # warm-up: every (kind, nside, precision) once, so plans and autotuning are in place
    for kind in kinds:
        for ns in pools:
            for prec in ("fp64", "split"):
                srv.submit(kind, ns, 2 * ns, inputs(kind, ns, 1), precision=prec)
    srv.drain()
    srv.completed.clear()
    clocks = ClockSampler(local)
    clocks.start()
    t0 = time.perf_counter()
    futs = []
    for (ta, kind, ns, lmax, nm, prec) in reqs:
        now = time.perf_counter() - t0
        if ta > now:
            time.sleep(ta - now)
        futs.append(srv.submit(kind, ns, lmax, inputs(kind, ns, nm), precision=prec,
                               t_arrival=t0 + ta))
    # requests still queued or running when the last one arrives: a server that keeps up with
    # the offered rate has only the most recent few
    with srv._lock:
        backlog = len(srv._pending) + sum(len(p.members) for p in srv._inflight)
    srv.drain()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    st = srv.stats()
    srv.close()
    failed = {}
    for f, r in zip(futs, reqs):
        e = f.exception(timeout=0)
        if e is not None:
            key = f"{r[1]} nside {r[2]} {r[5]}: {e!r}"[:300]
            failed[key] = failed.get(key, 0) + 1
    ok = [r for f, r in zip(futs, reqs) if f.exception(timeout=0) is None]
    mapsht = sum(nm * (2 if kind in ("qu2eb", "eb2qu") else 1) for _, kind, _, _, nm, _ in ok)
    line = {
        "metric": METRIC, "value": mapsht / wall, "unit": UNIT, "n_gpus": 1,
        "steps": 1, "warmup": 1, "ms_per_step": wall * 1000.0, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 and bf16x4-split of f64 (per request)",
        "data": "synthetic",
        "config": {"workload": (f"serving form: Poisson stream of {args.requests} requests "
                                f"(mean {args.rate}/s), map2alm or alm2map x T or Q/U, nside "
                                f"2^U{{6..{hi}}}, lmax = 2 nside, nmaps ~ U[1, {max_maps}] "
                                f"(at most {args.nside2048_maps} at nside 2048), FP64 or split "
                                f"per request, seed 4; HBM budget {args.budget_gb} GB"),
                   "offered_s": reqs[-1][0], "nslots": 8},
        "clocks": clk,
        "latency_ms": {"p50": st.get("p50_ms"), "p99": st.get("p99_ms"),
                       "mean": st.get("mean_ms")},
        "latency_by_precision_ms": st.get("by_precision"),
        "latency_by_nside_ms": st.get("by_nside"),
        "backlog_at_last_arrival": backlog,
        "offered_requests_per_s": args.requests / reqs[-1][0],
        "max_parts_per_request": st.get("max_parts"),
        "requests_per_s": len(ok) / wall,
        "failed_requests": sum(failed.values()),
        "failures": failed,
        "max_inflight": st.get("max_inflight"),
        "high_water_bytes": st.get("high_water_bytes"),
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        reference_arm(args, rank, world)
        return
    if args.workload == "batched":
        bench_batched(args, rank, world, local)
        return
    if args.workload == "serving":
        bench_serving(args, rank, world, local)
        return
    if args.workload == "qu2eb":
        bench_qu2eb(args, rank, world, local)
        return
    ours(args, rank, world, local)


if __name__ == "__main__":
    main()
