"""alm utilities on the device: spectra, filtering, normalisation and Gaussian realisations.

The reference ships these as IDL-callable Fortran (src/alm2cl_TEB.f90, src/filt_alm.f90,
src/norm_alm.f90, src/cl2alm_TEB.f90); here they are C-ABI kernels (fsht_alm2cl,
fsht_alm_filter, fsht_alm_norm, fsht_cl2alm) with the same square-real alm layout and the
same argument meaning.  alm arrays: NumPy (nsim, lmax+1, lmax+1) in Fortran order, or CUDA
float64 tensors of that shape with Fortran strides (or (lmax+1, lmax+1, nsim) contiguous);
NumPy in gives NumPy out, tensors stay on the device.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib


def _dev_alm(a):
    """-> (device tensor (L, L, nsim) contiguous, is_torch, nsim, lmax)."""
    if isinstance(a, torch.Tensor):
        if not (a.is_cuda and a.dtype == torch.float64):
            raise ValueError("alm tensors must be float64 CUDA tensors")
        if a.dim() != 3:
            raise ValueError("alm must be 3-d")
        if a.is_contiguous() and a.shape[0] == a.shape[1]:          # library layout
            return a, True, a.shape[2], a.shape[0] - 1
        t = a.permute(2, 1, 0)
        if t.is_contiguous() and t.shape[0] == t.shape[1]:          # Fortran (nsim, L, L)
            return t, True, a.shape[0], a.shape[1] - 1
        raise ValueError("alm tensor: expected (nsim, L, L) Fortran or (L, L, nsim) contiguous")
    arr = np.asfortranarray(np.asarray(a, dtype=np.float64))
    if arr.ndim != 3 or arr.shape[1] != arr.shape[2]:
        raise ValueError(f"alm: expected (nsim, L, L), got {arr.shape}")
    return torch.from_numpy(arr.T).cuda(), False, arr.shape[0], arr.shape[1] - 1


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _host_fortran(t):
    """device (L, L, nsim) -> NumPy (nsim, L, L) Fortran."""
    return np.asfortranarray(t.cpu().numpy().T)


def alm2cl(almT, almE=None, almB=None, lmin=0):
    """Spectra of square-real alm (alm2cl_TEB1 / alm2cl_T1, src/alm2cl_TEB.f90:22-110).
    T only: (nsim, lmax+1); with E and B: (nsim, lmax+1, 6) in the order TT EE BB TE TB EB."""
    tT, is_t, nsim, lmax = _dev_alm(almT)
    fields = [tT]
    if almE is not None or almB is not None:
        if almE is None or almB is None:
            raise ValueError("give both almE and almB, or neither")
        fields += [_dev_alm(almE)[0], _dev_alm(almB)[0]]
        pairs = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]
    else:
        pairs = [(0, 0)]
    out = torch.empty((len(pairs), lmax + 1, nsim), dtype=torch.float64, device=tT.device)
    for i, (a, b) in enumerate(pairs):
        _lib.call("fsht_alm2cl", C.c_void_p(fields[a].data_ptr()),
                  C.c_void_p(fields[b].data_ptr()), C.c_void_p(out[i].data_ptr()), lmax, nsim,
                  int(lmin), _stream())
    res = out.permute(2, 1, 0)                       # (nsim, lmax+1, ncl)
    if len(pairs) == 1:
        res = res[..., 0]
    if is_t:
        return res
    return np.asfortranarray(res.cpu().numpy())


def filt_alm(alm, win):
    """alm(l, m) *= win[l] in place (filt_alm1, src/filt_alm.f90:16-37); returns alm."""
    t, is_t, nsim, lmax = _dev_alm(alm)
    w = torch.as_tensor(np.asarray(win, dtype=np.float64), device=t.device)
    if w.numel() < lmax + 1:
        raise ValueError("win needs lmax+1 entries")
    _lib.call("fsht_alm_filter", C.c_void_p(t.data_ptr()), C.c_void_p(w.data_ptr()), lmax, nsim,
              _stream())
    if is_t:
        return alm
    np.asarray(alm)[...] = _host_fortran(t)
    return alm


def norm_alm(alm_in, fac, shift, m0=1.0):
    """alm_in * fac[l] + shift[l], the m = 0 entries also times m0 (norm_alm1,
    src/norm_alm.f90:14-35); returns a new array of alm_in's kind."""
    t, is_t, nsim, lmax = _dev_alm(alm_in)
    f = torch.as_tensor(np.asarray(fac, dtype=np.float64), device=t.device)
    s = torch.as_tensor(np.asarray(shift, dtype=np.float64), device=t.device)
    out = torch.empty_like(t)
    _lib.call("fsht_alm_norm", C.c_void_p(t.data_ptr()), C.c_void_p(out.data_ptr()),
              C.c_void_p(f.data_ptr()), C.c_void_p(s.data_ptr()), float(m0), lmax, nsim,
              _stream())
    return out.permute(2, 1, 0) if is_t else _host_fortran(out)


def cl2alm(cl, lmax, nsim, lmin=0, seed=0, device=None):
    """Gaussian square-real alm on the device (cl2alm_TEB1 / cl2alm_T1,
    src/cl2alm_TEB.f90:25-171).  cl: (lmax+1,) for T, or (lmax+1, 6) with TT EE BB TE TB EB;
    returns almT, or (almT, almE, almB), as CUDA tensors (nsim, L, L) in Fortran strides.
    Draws come from a counter-based generator keyed by seed (not MKL's stream)."""
    cl = np.ascontiguousarray(np.asarray(cl, dtype=np.float64))
    ncl = 1 if cl.ndim == 1 else cl.shape[1]
    if cl.shape[0] < lmax + 1 or ncl not in (1, 6):
        raise ValueError("cl must be (lmax+1,) or (lmax+1, 6)")
    dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
    dcl = torch.from_numpy(cl[:lmax + 1]).to(dev)
    L = lmax + 1
    nout = 1 if ncl == 1 else 3
    outs = [torch.empty((L, L, nsim), dtype=torch.float64, device=dev) for _ in range(nout)]
    ptr = [C.c_void_p(o.data_ptr()) for o in outs] + [None] * (3 - len(outs))
    with torch.cuda.device(dev):
        _lib.call("fsht_cl2alm", C.c_void_p(dcl.data_ptr()), ncl, int(lmin), lmax, nsim,
                  C.c_ulonglong(seed & (2 ** 64 - 1)), *ptr, _stream())
    res = [o.permute(2, 1, 0) for o in outs]
    return res[0] if ncl == 1 else tuple(res)
