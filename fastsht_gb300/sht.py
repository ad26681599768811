"""Drop-in ``SHT`` class for the batched HEALPix transform path on GB300.

Mirrors the reference's Python surface (SHT.py:16-227): same constructor, same
method names, argument meanings, array layouts and return conventions, with the
transforms running in the fastsht_gb300 CUDA library through its C ABI.

Arrays (exactly the reference's):
  maps : float64 (npix, nsim), Fortran order (each map contiguous), RING ordering
  alms : float64 (nsim, lmax+1, lmax+1), Fortran order, square-real packing
Inputs may be NumPy arrays (host; results come back as NumPy arrays in pinned
host memory, like the reference's numba pinned outputs) or CUDA torch tensors of
the same logical shape and Fortran strides (results stay on the device).
"""
from __future__ import annotations

import ctypes as C
import weakref

import numpy as np
import torch

from . import _lib

__all__ = ["SHT"]


def _is_torch(x):
    return isinstance(x, torch.Tensor)


def _fortran_view_ok(t: torch.Tensor) -> bool:
    """True when t's memory is Fortran-contiguous (first index fastest)."""
    return t.permute(*reversed(range(t.dim()))).is_contiguous()


def pinned_empty(shape, order="F"):
    """float64 NumPy array in page-locked host memory (fsht_host_alloc), freed with the array;
    host buffers of this kind let SHT.t2alm overlap its copies with the transform."""
    n = int(np.prod(shape)) if len(shape) else 1
    ptr = C.c_void_p()
    try:
        _lib.call("fsht_host_alloc", C.c_size_t(8 * max(n, 1)), C.byref(ptr))
    except Exception:
        return np.empty(shape, dtype=np.float64, order=order)
    buf = (C.c_double * max(n, 1)).from_address(ptr.value)
    arr = np.frombuffer(buf, dtype=np.float64, count=n).reshape(shape, order=order)
    weakref.finalize(buf, _lib.load().fsht_host_free, C.c_void_p(ptr.value))
    return arr


# host_read modes of fsht_plan_set_host_read: maps in a pinned_empty buffer read in place by
# the forward FFT ("direct"), in place as overlapped chunks (split form, 128 or more maps: each
# chunk's contraction beside the next chunk's reads), or copied to device memory first
_HOST_READ = {"staged": 0, "direct": 1, "direct_chunked": 2}


class SHT:
    """Batched spherical-harmonic transforms of ``nsim`` HEALPix maps.

    SHT(nside, lmax, nsim, niter=0, pol=False, all_buff=False) as in the
    reference (SHT.py:17).  Extra keywords: ``device`` (CUDA device index),
    ``workspace_limit`` (bytes of workspace, 0 = library default) and ``precision``:
    "fp64" (the plain method, all FP64) or "split" (the Legendre contractions of t2alm,
    alm2t, qu2eb / qu2e / qu2b and eb2qu as BF16 digit products on the tensor cores, ~3e-8
    max relative alm error; niter > 0 refines with the FP64 Fourier-space residual).
    ``host_read``: how t2alm takes NumPy maps that sit in a ``pinned_empty`` buffer -
    "direct" (read in place by the FFT over the host link), "direct_chunked" (in place, in the
    split form with 128 or more maps as chunks, each chunk's contraction running beside the next
    chunk's reads) or "staged" (copied to device memory first); the results are the same.
    """

    def __init__(self, nside, lmax, nsim, niter=0, pol=False, all_buff=False, *,
                 device=None, workspace_limit=0, precision="fp64", host_read="direct"):
        if not torch.cuda.is_available():
            raise RuntimeError("fastsht_gb300 needs a CUDA device (no CPU fallback)")
        self.nside = int(nside)
        self.lmax = int(lmax)
        self.nsim = int(nsim)
        self.niter = int(niter)
        self.pol = 1 if pol else 0
        self.nring = 4 * self.nside - 1
        self.npix = 12 * self.nside ** 2
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        if precision not in ("fp64", "split"):
            raise ValueError("precision must be 'fp64' or 'split'")
        if host_read not in _HOST_READ:
            raise ValueError(f"host_read must be one of {sorted(_HOST_READ)}")
        self.precision = precision
        self.host_read = host_read
        # workspace buffers, like the reference's nbuff (SHT.py:52-59)
        flags = 0
        if pol or all_buff:
            flags |= _lib.FSHT_FLAG_POL
        if niter > 0 or all_buff:
            flags |= _lib.FSHT_FLAG_ITER
        self._flags = flags
        self.maps = None
        self.alms = None
        self._dev_alm = None
        plan = C.c_void_p()
        with torch.cuda.device(self.device):
            stream = torch.cuda.current_stream(self.device).cuda_stream
            _lib.call("fsht_plan_create", self.nside, self.lmax, self.nsim, flags,
                      _lib.FSHT_PREC_SPLIT if precision == "split" else _lib.FSHT_PREC_FP64,
                      int(workspace_limit), C.c_void_p(stream), C.byref(plan))
        self._plan = plan
        _lib.call("fsht_plan_set_host_read", plan, _HOST_READ[host_read])

    # ------------------------------------------------------------ lifetime
    def close(self):
        if getattr(self, "_plan", None) and self._plan.value:
            _lib.load().fsht_plan_destroy(self._plan)
            self._plan = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------ plan info
    def ring_skip(self) -> np.ndarray:
        """First kept ring per m (the reference's SHT_ring_skip_table row)."""
        out = (C.c_int * (self.lmax + 1))()
        _lib.call("fsht_plan_ring_skip", self._plan, out)
        return np.frombuffer(out, dtype=np.int32).copy()

    def plan_info(self):
        b = C.c_size_t()
        k = C.c_int()
        _lib.call("fsht_plan_info", self._plan, C.byref(b), C.byref(k))
        return {"device_bytes": b.value, "maps_per_chunk": k.value}

    # ------------------------------------------------------------ helpers
    def _stream(self):
        s = torch.cuda.current_stream(self.device).cuda_stream
        _lib.call("fsht_plan_set_stream", self._plan, C.c_void_p(s))

    def _dev_maps(self, x, name):
        """-> (device tensor (nsim, npix) contiguous, is_torch)."""
        if x is None:
            raise ValueError(f"No input {name}!")
        if _is_torch(x):
            if x.device.type != "cuda" or x.dtype != torch.float64:
                raise ValueError(f"{name}: expected a float64 CUDA tensor")
            if x.shape == (self.npix, self.nsim) and _fortran_view_ok(x):
                return x.T, True
            if x.shape == (self.nsim, self.npix) and x.is_contiguous():
                return x, True
            raise ValueError(f"{name}: expected shape ({self.npix}, {self.nsim}) in Fortran order")
        a = np.asarray(x)
        if a.shape != (self.npix, self.nsim):
            raise ValueError(f"{name}: expected shape ({self.npix}, {self.nsim}), got {a.shape}")
        a = np.asfortranarray(a, dtype=np.float64)
        return torch.from_numpy(a.T).to(self.device, non_blocking=True), False

    def _dev_alm_in(self, x, name):
        L = self.lmax + 1
        if x is None:
            raise ValueError(f"No input {name}!")
        if _is_torch(x):
            if x.device.type != "cuda" or x.dtype != torch.float64:
                raise ValueError(f"{name}: expected a float64 CUDA tensor")
            if x.shape == (self.nsim, L, L) and _fortran_view_ok(x):
                return x.permute(2, 1, 0), True
            if x.shape == (L, L, self.nsim) and x.is_contiguous():
                return x, True
            raise ValueError(f"{name}: expected shape ({self.nsim}, {L}, {L}) in Fortran order")
        a = np.asarray(x)
        if a.shape != (self.nsim, L, L):
            raise ValueError(f"{name}: expected shape ({self.nsim}, {L}, {L}), got {a.shape}")
        a = np.asfortranarray(a, dtype=np.float64)
        return torch.from_numpy(a.T).to(self.device, non_blocking=True), False

    def _new_dev_alm(self):
        L = self.lmax + 1
        return torch.empty((L, L, self.nsim), dtype=torch.float64, device=self.device)

    def _new_dev_maps(self):
        return torch.empty((self.nsim, self.npix), dtype=torch.float64, device=self.device)

    def _alm_out(self, dev, alms_in, as_torch):
        """Deliver a device alm (L, L, nsim) into alms_in (if given) or a new array."""
        if alms_in is not None:
            if _is_torch(alms_in):
                tgt = alms_in.permute(2, 1, 0) if alms_in.shape[0] == self.nsim else alms_in
                if tgt.data_ptr() != dev.data_ptr():
                    tgt.copy_(dev)
            else:
                torch.from_numpy(np.asarray(alms_in).T).copy_(dev, non_blocking=False)
            return 0
        if as_torch:
            return dev.permute(2, 1, 0)
        out = pinned_empty((self.nsim, self.lmax + 1, self.lmax + 1))
        torch.from_numpy(out.T).copy_(dev, non_blocking=False)
        return out

    def _maps_out(self, dev, maps_in, as_torch):
        if maps_in is not None:
            if _is_torch(maps_in):
                tgt = maps_in.T if maps_in.shape[0] == self.npix else maps_in
                if tgt.data_ptr() != dev.data_ptr():
                    tgt.copy_(dev)
            else:
                torch.from_numpy(np.asarray(maps_in).T).copy_(dev, non_blocking=False)
            return 0
        if as_torch:
            return dev.T
        out = pinned_empty((self.npix, self.nsim))
        torch.from_numpy(out.T).copy_(dev, non_blocking=False)
        return out

    # ------------------------------------------------------------ reference API
    def set_maps(self, maps_in):
        self.maps = maps_in

    def set_alms(self, alms_in):
        # the reference's set_alms lacks `self` (SHT.py:69); this is the fixed form
        self.alms = alms_in

    def t2alm(self, maps_in=None, alms_in=None, method='old', get_alm=True):
        """Temperature map -> alm (reference SHT.t2alm, SHT.py:72-107).

        niter == 0: t2alm; niter > 0: t2alm_iter_old (method='old') or
        t2alm_iter (any other method).  Returns alm, or 0 when alms_in is given.
        get_alm=False leaves the result on the device (fetch it with get_alms()).
        """
        maps = self.maps if maps_in is None else maps_in
        if maps is None:
            raise ValueError('No input maps AND no internal maps! Check the parameters or call '
                             'set_maps(maps_in)!')
        with torch.cuda.device(self.device):
            self._stream()
            if get_alm and not _is_torch(maps) and self._host_alm_ok(alms_in):
                return self._t2alm_host(maps, alms_in, method)
            dmaps, as_torch = self._dev_maps(maps, "maps")
            dalm = self._new_dev_alm()
            _lib.call("fsht_t2alm", self._plan, C.c_void_p(dmaps.data_ptr()),
                      C.c_void_p(dalm.data_ptr()), self.nsim, self.niter,
                      0 if method == 'old' else 1)
            if self.precision == "split":
                _lib.call("fsht_plan_sync", self._plan)   # surfaces expired device waits
            self._dev_alm = dalm
            if not get_alm:
                return None
            return self._alm_out(dalm, alms_in, as_torch)

    def release_staging(self):
        """Frees the device buffers that t2alm keeps between calls for NumPy (host) inputs
        (maps and alm of nsim maps); the next host-buffer call allocates them again."""
        hd = getattr(self, "_host_dev", None)
        if hd is not None and self._dev_alm is hd[1]:
            self._dev_alm = None          # get_alms() has nothing to read any more
        self._host_dev = None

    def _host_alm_ok(self, alms_in):
        if alms_in is None:
            return True
        if _is_torch(alms_in):
            return False
        a = np.asarray(alms_in)
        L = self.lmax + 1
        return a.dtype == np.float64 and a.flags.f_contiguous and a.shape == (self.nsim, L, L)

    def _t2alm_host(self, maps, alms_in, method):
        """Host maps -> host alm through fsht_t2alm_host.  Maps in a pinned_empty buffer are
        read in place by the FFT over the host link (host_read="direct"); other maps go to the
        device in sub-batches that the FFT consumes as they land.  Finished alm columns come
        back while later waves run (copies overlap the transform)."""
        a = np.asarray(maps)
        if a.shape != (self.npix, self.nsim):
            raise ValueError(f"maps: expected shape ({self.npix}, {self.nsim}), got {a.shape}")
        a = np.asfortranarray(a, dtype=np.float64)
        L = self.lmax + 1
        out = np.asarray(alms_in) if alms_in is not None else pinned_empty((self.nsim, L, L))
        # device staging buffers of the host path, kept between calls (like the reference's
        # persistent device arrays); the alm buffer is also what get_alms() reads, the maps
        # buffer is only made for maps that are not read in place
        hd = getattr(self, "_host_dev", None)
        if hd is None:
            hd = self._host_dev = [None, self._new_dev_alm()]
        mapped = C.c_int(0)
        if self.host_read != "staged":
            _lib.call("fsht_host_mapped", C.c_void_p(a.ctypes.data), C.c_size_t(a.nbytes),
                      C.byref(mapped))
        if not mapped.value and hd[0] is None:
            hd[0] = self._new_dev_maps()
        dmaps, dalm = hd
        _lib.call("fsht_t2alm_host", self._plan, C.c_void_p(a.ctypes.data),
                  C.c_void_p(out.ctypes.data),
                  C.c_void_p(dmaps.data_ptr() if dmaps is not None else None),
                  C.c_void_p(dalm.data_ptr()), self.nsim, self.niter,
                  0 if method == 'old' else 1)
        _lib.call("fsht_plan_sync", self._plan)
        self._dev_alm = dalm
        return 0 if alms_in is not None else out

    def alm2t(self, alms, maps_in=None):
        """alm -> temperature maps (reference SHT.alm2t, SHT.py:109-122)."""
        with torch.cuda.device(self.device):
            self._stream()
            dalm, as_torch = self._dev_alm_in(alms, "alms")
            dmaps = self._new_dev_maps()
            _lib.call("fsht_alm2t", self._plan, C.c_void_p(dalm.data_ptr()),
                      C.c_void_p(dmaps.data_ptr()), self.nsim)
            if self.precision == "split":
                _lib.call("fsht_plan_sync", self._plan)   # surfaces expired device waits
            return self._maps_out(dmaps, maps_in, as_torch)

    def qu2eb(self, Q, U, almEs_in=None, almBs_in=None, method='old'):
        """Q/U maps -> E/B alm (reference SHT.qu2eb, SHT.py:124-144)."""
        if method != 'old' and self.niter > 0:
            raise ValueError("qu2eb with niter > 0 supports method='old' only "
                             "(the reference defines no other spin-2 iteration)")
        with torch.cuda.device(self.device):
            self._stream()
            dQ, as_torch = self._dev_maps(Q, "Q")
            dU, _ = self._dev_maps(U, "U")
            dE, dB = self._new_dev_alm(), self._new_dev_alm()
            _lib.call("fsht_qu2eb", self._plan, C.c_void_p(dQ.data_ptr()), C.c_void_p(dU.data_ptr()),
                      C.c_void_p(dE.data_ptr()), C.c_void_p(dB.data_ptr()), self.nsim, self.niter)
            if almEs_in is None or almBs_in is None:
                return (self._alm_out(dE, None, as_torch), self._alm_out(dB, None, as_torch))
            self._alm_out(dE, almEs_in, as_torch)
            self._alm_out(dB, almBs_in, as_torch)
            return 0

    def qu2e(self, Q, U, almEs_in=None):
        """Q/U -> E only, no iterations (reference SHT.qu2e, SHT.py:146-160)."""
        with torch.cuda.device(self.device):
            self._stream()
            dQ, as_torch = self._dev_maps(Q, "Q")
            dU, _ = self._dev_maps(U, "U")
            dE = self._new_dev_alm()
            _lib.call("fsht_qu2e", self._plan, C.c_void_p(dQ.data_ptr()), C.c_void_p(dU.data_ptr()),
                      C.c_void_p(dE.data_ptr()), self.nsim)
            return self._alm_out(dE, almEs_in, as_torch)

    def qu2b(self, Q, U, almBs_in=None):
        """Q/U -> B only, no iterations (reference SHT.qu2b, SHT.py:162-176)."""
        with torch.cuda.device(self.device):
            self._stream()
            dQ, as_torch = self._dev_maps(Q, "Q")
            dU, _ = self._dev_maps(U, "U")
            dB = self._new_dev_alm()
            _lib.call("fsht_qu2b", self._plan, C.c_void_p(dQ.data_ptr()), C.c_void_p(dU.data_ptr()),
                      C.c_void_p(dB.data_ptr()), self.nsim)
            return self._alm_out(dB, almBs_in, as_torch)

    def eb2qu(self, almEs, almBs):
        """E/B alm -> Q/U maps (reference SHT.eb2qu, SHT.py:179-190)."""
        with torch.cuda.device(self.device):
            self._stream()
            dE, as_torch = self._dev_alm_in(almEs, "almEs")
            dB, _ = self._dev_alm_in(almBs, "almBs")
            dQ, dU = self._new_dev_maps(), self._new_dev_maps()
            _lib.call("fsht_eb2qu", self._plan, C.c_void_p(dE.data_ptr()), C.c_void_p(dB.data_ptr()),
                      C.c_void_p(dQ.data_ptr()), C.c_void_p(dU.data_ptr()), self.nsim)
            return (self._maps_out(dQ, None, as_torch), self._maps_out(dU, None, as_torch))

    def convert_alm_healpy(self, alms):
        """Square-real alm -> healpy complex (nalm, nsim) (SHT.py:204-210)."""
        with torch.cuda.device(self.device):
            self._stream()
            dalm, as_torch = self._dev_alm_in(alms, "alms")
            nalm = (self.lmax + 1) * (self.lmax + 2) // 2
            out = torch.empty((self.nsim, nalm), dtype=torch.complex128, device=self.device)
            _lib.call("fsht_convert_alm_healpy", self._plan, C.c_void_p(dalm.data_ptr()),
                      C.c_void_p(out.data_ptr()), self.nsim)
            if as_torch:
                return out.T
            return out.cpu().numpy().T

    def convert_alm_healpy_inv(self, alms_hp):
        """healpy complex (nalm, nsim) -> square-real alm (convert_alm_healpy_inv1)."""
        with torch.cuda.device(self.device):
            self._stream()
            if _is_torch(alms_hp):
                src = alms_hp.T.contiguous()
                as_torch = True
            else:
                src = torch.from_numpy(np.ascontiguousarray(np.asarray(alms_hp).T,
                                                            dtype=np.complex128)).to(self.device)
                as_torch = False
            dalm = self._new_dev_alm()
            _lib.call("fsht_convert_alm_healpy_inv", self._plan, C.c_void_p(src.data_ptr()),
                      C.c_void_p(dalm.data_ptr()), self.nsim)
            return self._alm_out(dalm, None, as_torch)

    def get_alms(self, alms_in=None):
        """Fetch the alm left on the device by t2alm(get_alm=False) (SHT.py:214-227)."""
        if self._dev_alm is None:
            raise ValueError("no device alm: call t2alm first")
        with torch.cuda.device(self.device):
            return self._alm_out(self._dev_alm, alms_in, False)

    def fix_eb(self, Q, U, mask):
        """EB-leakage cleaning on a masked sky (reference SHT.fix_eb, SHT.py:192-202, over
        fix_eb in src/sht_main.f90:801-941): mask Q/U, iterate (niter) to E/B, synthesise
        Q/U from E alone, mask again, iterate to the leakage template's B, take the B alm and
        the template to pixels with the spin-0 synthesis, and on the pixels where mask == 1
        return the residual of the per-map linear fit (lin_resi_mini, src/sht_core.f90:232-
        253) of the B map on the template; zero elsewhere.  As in the reference, Q and U
        are masked in place.  Returns Bmap (npix, nsim), on the device for tensor inputs."""
        if not self.pol:
            raise ValueError("fix_eb needs SHT(..., pol=True)")
        with torch.cuda.device(self.device):
            self._stream()
            dQ, as_torch = self._dev_maps(Q, "Q")
            dU, _ = self._dev_maps(U, "U")
            m = torch.as_tensor(np.asarray(mask, dtype=np.float64) if not _is_torch(mask) else mask,
                                dtype=torch.float64, device=self.device).reshape(-1)
            if m.numel() != self.npix:
                raise ValueError(f"mask: expected {self.npix} pixels")
            dQ.mul_(m)                                  # (nsim, npix): masked in place
            dU.mul_(m)
            if not as_torch:                            # the reference masks the caller's arrays
                np.asarray(Q)[...] = dQ.cpu().numpy().T
                np.asarray(U)[...] = dU.cpu().numpy().T
            E, B = self.qu2eb(dQ.T, dU.T)
            q2, u2 = self.eb2qu(E, torch.zeros_like(E))
            q2.mul_(m[:, None])
            u2.mul_(m[:, None])
            _, btpl_alm = self.qu2eb(q2, u2)
            y_all = self.alm2t(B)                       # (npix, nsim) views
            x_all = self.alm2t(btpl_alm)
            vid = torch.nonzero(m == 1).reshape(-1)
            x, y = x_all[vid], y_all[vid]
            mx, my = x.mean(dim=0), y.mean(dim=0)
            a1 = ((y - my) * (x - mx)).sum(dim=0) / ((x - mx) ** 2).sum(dim=0)
            a0 = my - mx * a1
            out = torch.zeros((self.nsim, self.npix), dtype=torch.float64, device=self.device).T
            out[vid] = y - a0 - a1 * x
            if as_torch:
                return out
            res = pinned_empty((self.npix, self.nsim))
            torch.from_numpy(res.T).copy_(out.T)
            return res
