"""FP64 CPU restatement of liuhao-cn/fastSHT's batched HEALPix SHT (the oracle).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).  Each function names the
reference routine it restates.  Array conventions are the reference's:

  maps  : float64 (npix, nsim), Fortran order (each map contiguous), RING ordering
  alm   : float64 (nsim, lmax+1, lmax+1), Fortran order, "square-real" packing:
          Re a_lm at [k, l, m] (m <= l), Im a_lm at [k, l-m, lmax+1-m] (m >= 1)
  buff  : float64 (nsim, npix): per-ring real FFT in MKL PERM packing, transposed
  mat1/2: float64 (nsim, nring): Re/Im of the per-m "FFT matrix"

The ring FFTs use scipy.fft (unnormalised, like MKL DFTI's defaults) and the per-m
DGEMMs use NumPy BLAS; both compute the same exact-arithmetic quantities as the
reference's MKL/cuBLAS calls.
"""
from __future__ import annotations

import math
import os

import numpy as np
import scipy.fft

__all__ = [
    "ring_info", "ring_angles", "ring_skip_table", "recursion_constants",
    "plm_T", "plm_pol", "OracleSHT", "alm_square_to_healpy", "alm_healpy_to_square",
    "gaussian_alm", "lm_count", "plm_c", "c_recursion", "alm2cl", "filt_alm", "norm_alm",
]

PI = math.pi

_CLIB = None


def c_recursion():
    """The compiled C restatement of the recursion (oracle/plm.c), or None."""
    global _CLIB
    if _CLIB is None:
        import ctypes
        from pathlib import Path
        path = Path(__file__).resolve().parent / "_build" / "liboracle_plm.so"
        if not path.exists():
            try:
                from . import build_oracle
                build_oracle.build()
            except Exception:
                _CLIB = False
                return None
        lib = ctypes.CDLL(str(path))
        dp = ctypes.POINTER(ctypes.c_double)
        lib.oracle_plm.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp,
                                   ctypes.c_double, ctypes.c_int, ctypes.c_int, dp, dp, dp]
        lib.oracle_plm.restype = None
        lib.oracle_plm_sphere.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          dp, dp, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                          dp, dp, dp]
        lib.oracle_plm_sphere.restype = None
        lib.oracle_fft2mat.argtypes = [ctypes.c_int, ctypes.c_int, dp,
                                       ctypes.POINTER(ctypes.c_longlong), dp, dp, dp, dp, dp, dp]
        lib.oracle_fft2mat.restype = None
        _CLIB = lib
    return _CLIB or None


def plm_c(m: int, lmax: int, nside: int, k: dict, i0: int, pol: bool, scaled: bool | None = None):
    """Same values as plm_T / plm_pol, computed by oracle/plm.c."""
    import ctypes
    lib = c_recursion()
    if scaled is None:
        scaled = nside > 512
    cc = np.ascontiguousarray(k["cc"][i0:2 * nside])
    ss = np.ascontiguousarray(k["ss"][i0:2 * nside])
    nr = cc.shape[0]
    dp = ctypes.POINTER(ctypes.c_double)
    p0 = np.zeros((nr, lmax + 1))
    p1 = np.zeros((nr, lmax + 1)) if pol else p0
    p2 = np.zeros((nr, lmax + 1)) if pol else p0
    if nr:
        pref = math.sqrt(k["diag_fac"][m] / 4 / PI)
        lib.oracle_plm(m, lmax, nr, cc.ctypes.data_as(dp), ss.ctypes.data_as(dp), pref,
                       int(scaled), int(pol), p0.ctypes.data_as(dp), p1.ctypes.data_as(dp),
                       p2.ctypes.data_as(dp))
    return (p0, p1, p2) if pol else p0


# ---------------------------------------------------------------------------
# geometry
# ---------------------------------------------------------------------------
def ring_info(nside: int):
    """Ring start pixel i1 and length nfft for rings 0..4*nside-2.

    Restates ``get_ring_info`` (src/sht_data_init.f90:644-686).
    """
    ns = nside
    nring = 4 * ns - 1
    i = np.arange(nring, dtype=np.int64)
    i1 = np.where(i < ns, 2 * i * (i + 1),
                  np.where(i < 3 * ns - 1, 2 * ns + 4 * ns * i - 2 * ns * ns,
                           12 * ns * ns - 2 * (4 * ns - i - 1) * (4 * ns - i)))
    nfft = np.where(i < ns, 4 * (i + 1),
                    np.where(i < 3 * ns - 1, 4 * ns, 4 * (4 * ns - 1 - i)))
    return i1.astype(np.int64), nfft.astype(np.int64)


def ring_angles(nside: int):
    """Colatitude theta and first-pixel longitude phi0 of the 2*nside north rings.

    The reference takes these from ``healpy.pix2ang(nside, TJI)`` at the ring start
    pixels (SHT.py:47-50) and passes the first 2*nside entries
    (sht_data_init.f90:285).  healpy is absent, so this restates HEALPix's
    ``pix2loc`` for the first pixel of each ring: polar cap z = 1 - r^2*4/npix with
    theta = atan2(sqrt(t(2-t)), z) when z > 0.99, else acos(z); belt
    z = (2 nside - r)*2/(3 nside), phi0 = (1 - fodd)*pi/(2 nside).
    """
    ns = nside
    npix = 12 * ns * ns
    fact2 = 4.0 / npix
    fact1 = (ns << 1) * fact2
    theta = np.empty(2 * ns)
    phi0 = np.empty(2 * ns)
    for i in range(2 * ns):
        ir = i + 1
        if ir < ns:
            tmp = (ir * ir) * fact2
            z = 1.0 - tmp
            if z > 0.99:
                theta[i] = math.atan2(math.sqrt(tmp * (2.0 - tmp)), z)
            else:
                theta[i] = math.acos(z)
            phi0[i] = (1 - 0.5) * (0.5 * PI) / ir
        else:
            z = (2 * ns - ir) * fact1
            theta[i] = math.acos(z)
            fodd = 1.0 if ((ir + ns) & 1) else 0.5
            phi0[i] = (1 - fodd) * PI * 0.75 * fact1
    return theta, phi0


def lm_count(lmax: int) -> int:
    return (lmax + 1) * (lmax + 2) // 2


# ---------------------------------------------------------------------------
# recursion
# ---------------------------------------------------------------------------
def recursion_constants(nside: int, lmax: int, theta: np.ndarray):
    """Restates ``set_out_of_loop_constants`` (src/sht_data_init.f90:383-419)."""
    cc = np.cos(theta)
    ss = np.sin(theta)
    two_on_s2 = 2 / ss ** 2
    b_w = cc / ss ** 2
    l = np.arange(lmax + 1, dtype=np.float64)
    normal_l = np.zeros(lmax + 1)
    if lmax >= 2:
        ll = l[2:]
        normal_l[2:] = 1 / np.sqrt((ll + 2) * (ll + 1) * ll * (ll - 1))
    normal_m = 2 * l * (1 - l)
    c1 = (l - 1) ** 2
    c2 = (2 * l - 3) * (2 * l - 1)
    c3 = (2 * l - 1) * (2 * l + 1)
    c4 = l ** 2
    c1[0] = c2[0] = c3[0] = c4[0] = 0
    diag_fac = np.empty(lmax + 1)
    diag_fac[0] = 1
    for m in range(1, lmax + 1):
        diag_fac[m] = diag_fac[m - 1] * (2 * m + 1) / 2 / m
    return dict(cc=cc, ss=ss, two_on_s2=two_on_s2, b_w=b_w, normal_l=normal_l,
                normal_m=normal_m, c1=c1, c2=c2, c3=c3, c4=c4, diag_fac=diag_fac)


def _ab(m: int, lmax: int, k: dict):
    """a_l, b_l for l=m..lmax (get_plm_recursive.f90:31-37)."""
    a = np.zeros(lmax + 1)
    b = np.zeros(lmax + 1)
    a[m] = 0.0
    b[m] = -1.0
    if m < lmax:
        l = slice(m + 1, lmax + 1)
        a[l] = np.sqrt(k["c3"][l] / (k["c4"][l] - m * m))
        b[l] = np.sqrt((k["c1"][l] - m * m) / k["c2"][l]) * a[l]
    return a, b


_SCALE_BITS = 600          # one exponent step of the scaled recursion: 2**600
_SCALE_HI = 2.0 ** 300     # rescale when |value| exceeds this


def plm_T(m: int, lmax: int, nside: int, k: dict, i0: int, scaled: bool | None = None):
    """lambda_lm(theta_i) for north rings i0..2ns-1 and l = m..lmax.

    Restates ``get_plm_recursive`` with pol=0 (src/get_plm_recursive.f90:17-98):
    seed lambda_mm = sqrt(diag_fac(m)/(4 pi)) (-sin theta)^m, then the three-term
    recursion lambda_l = a_l cos(theta) lambda_{l-1} - b_l lambda_{l-2}.

    For nside <= 512 the reference seeds directly (no scaling); this is what
    ``scaled=False`` does (the default for nside <= 512).  For nside > 512 it seeds
    from precomputed "safe start" tables that are missing from the reference
    snapshot; ``scaled=True`` replaces them with an exponent-rescaled recursion
    (values carried as v * 2**(600 e), e <= 0) that yields the same exact values.
    Values whose exponent index is still negative at a given l are below 2**-300 and
    are returned as 0.

    Returns an array (2*nside - i0, lmax+1); columns < m are zero.
    """
    if scaled is None:
        scaled = nside > 512
    a, b = _ab(m, lmax, k)
    cc = k["cc"][i0:2 * nside]
    ss = k["ss"][i0:2 * nside]
    nr = cc.shape[0]
    out = np.zeros((nr, lmax + 1))
    if nr == 0:
        return out
    if not scaled:
        p2 = math.sqrt(k["diag_fac"][m] / 4 / PI) * (-ss) ** m   # plm0(m-2)
        p1 = np.zeros(nr)                                          # plm0(m-1)
        for l in range(m, lmax + 1):
            p = a[l] * cc * p1 - b[l] * p2
            out[:, l] = p
            p2, p1 = p1, p
        return out
    # exponent-rescaled recursion; seed sin(theta)^m by binary powering on
    # (mantissa, exponent) pairs so nothing underflows and the error stays ~log2(m) ulp
    rm = np.ones(nr)
    re = np.zeros(nr, dtype=np.int64)
    bm, be = np.frexp(ss)
    be = be.astype(np.int64)
    kk = m
    while kk:
        if kk & 1:
            rm = rm * bm
            re = re + be
            rm, t = np.frexp(rm)
            re = re + t
        kk >>= 1
        if kk:
            bm = bm * bm
            be = be * 2
            bm, t = np.frexp(bm)
            be = be + t
    rm = rm * math.sqrt(k["diag_fac"][m] / 4 / PI)
    rm, t = np.frexp(rm)
    re = re + t
    e = np.where(re >= -300, 0, np.floor((re + 300) / _SCALE_BITS)).astype(np.int64)
    mant = np.ldexp(rm, (re - _SCALE_BITS * e).astype(np.int32))
    sign = -1.0 if (m & 1) else 1.0
    p2 = sign * mant
    p1 = np.zeros(nr)
    for l in range(m, lmax + 1):
        p = a[l] * cc * p1 - b[l] * p2
        p2, p1 = p1, p
        big = (np.abs(p1) > _SCALE_HI) & (e < 0)
        if big.any():
            p1 = np.where(big, p1 * 2.0 ** -_SCALE_BITS, p1)
            p2 = np.where(big, p2 * 2.0 ** -_SCALE_BITS, p2)
            e = np.where(big, e + 1, e)
        out[:, l] = np.where(e == 0, p1, 0.0)
    return out


def plm_pol(m: int, lmax: int, nside: int, k: dict, i0: int, plm0: np.ndarray):
    """Spin-2 lambda1/lambda2 for north rings i0..2ns-1 from plm0.

    Restates the pol=1 branch of ``get_plm_recursive``
    (src/get_plm_recursive.f90:101-125).
    """
    ss = k["ss"][i0:2 * nside]
    cc = k["cc"][i0:2 * nside]
    b_w = k["b_w"][i0:2 * nside]
    two_on_s2 = k["two_on_s2"][i0:2 * nside]
    normal_l = k["normal_l"]
    nr = ss.shape[0]
    plm1 = np.zeros((nr, lmax + 1))
    plm2 = np.zeros((nr, lmax + 1))
    if nr == 0:
        return plm1, plm2
    m1 = max(1, m)
    lam_fact = np.zeros(lmax + 1)
    if m1 < lmax:
        l = np.arange(m1 + 1, lmax + 1, dtype=np.float64)
        lam_fact[m1 + 1:] = 2 * np.sqrt((2 * l + 1) / (2 * l - 1) * (l ** 2 - m ** 2))
    c_w = m / ss ** 2
    nm = k["normal_m"][m] * normal_l[m]
    plm1[:, m] = nm * plm0[:, m] * (0.5 - 1.0 / ss ** 2)
    plm2[:, m] = nm * plm0[:, m] * cc / ss ** 2
    if m < lmax:
        for l in range(m + 1, lmax + 1):
            plm1[:, l] = (plm0[:, l - 1] * lam_fact[l] * b_w
                          - plm0[:, l] * (two_on_s2 * (l - m ** 2) + l * (l - 1.0))) * normal_l[l]
            plm2[:, l] = (plm0[:, l - 1] * lam_fact[l]
                          - plm0[:, l] * (2.0 * cc * (l - 1.0))) * c_w * normal_l[l]
    return plm1, plm2


def _mirror(north: np.ndarray, m: int, nside: int, i0: int, parity_shift: int = 0):
    """Full-sphere (rlen, lmax+1) table from the north rows: south ring i mirrors
    ring nring-1-i with sign (-1)^(l+m+shift) (get_plm_recursive.f90:93-98, 128-134)."""
    lmax = north.shape[1] - 1
    nn = north.shape[0]                 # rings i0..2ns-1
    sgn = np.where((np.arange(lmax + 1) + m + parity_shift) % 2 == 0, 1.0, -1.0)
    south = north[:nn - 1][::-1] * sgn  # rings 2ns..nring-1-i0
    return np.concatenate([north, south], axis=0)


def ring_skip_table(nside: int, mmax: int, thresh: float = 1e-20, lcap: int | None = None):
    """First kept ring i0(m) for m = 0..mmax.

    The reference reads ``SHT_ring_skip_table/<nside>.bin`` (SHT.py:31-32); its
    generator is not in the reference tree.  The tables match the rule "drop ring i
    for order m when max_{m<=l<=4 nside} |lambda_lm(theta_i)| < 1e-20" (made
    monotone in m), which is what this computes (scaled recursion).  Skipped
    contributions are below 1e-20 relative, far under every tolerance.
    """
    if lcap is None:
        lcap = 4 * nside
    theta, _ = ring_angles(nside)
    k = recursion_constants(nside, max(lcap, mmax), theta)
    out = np.zeros(mmax + 1, dtype=np.int32)
    prev = 0
    for m in range(mmax + 1):
        lam = plm_T(m, lcap, nside, k, 0, scaled=True)
        mx = np.abs(lam).max(axis=1)
        kept = np.nonzero(mx >= thresh)[0]
        first = int(kept[0]) if kept.size else 2 * nside - 1
        prev = max(prev, first)
        out[m] = prev
    return out


# ---------------------------------------------------------------------------
# alm layout helpers
# ---------------------------------------------------------------------------
def alm_square_to_healpy(alm: np.ndarray) -> np.ndarray:
    """Square-real (nsim, L, L) F-order -> healpy complex (nalm, nsim).

    Restates ``convert_alm_healpy1`` (src/convert_alm.f90:34-56) as used by
    SHT.convert_alm_healpy (SHT.py:204-210); index = m(2 lmax + 1 - m)/2 + l.
    """
    nsim, L, _ = alm.shape
    lmax = L - 1
    out = np.zeros((lm_count(lmax), nsim), dtype=np.complex128)
    pos = 0
    for m in range(lmax + 1):
        n = lmax + 1 - m
        re = alm[:, m:, m].T
        im = alm[:, 0:n, lmax + 1 - m].T if m > 0 else 0.0
        out[pos:pos + n] = re + 1j * im
        pos += n
    return out


def alm_healpy_to_square(alm_hp: np.ndarray, lmax: int) -> np.ndarray:
    """Inverse of ``alm_square_to_healpy`` (convert_alm_healpy_inv1, convert_alm.f90:87-107).
    Unused slots are zero."""
    nsim = alm_hp.shape[1]
    L = lmax + 1
    out = np.zeros((nsim, L, L), order="F")
    pos = 0
    for m in range(lmax + 1):
        n = lmax + 1 - m
        out[:, m:, m] = alm_hp[pos:pos + n].real.T
        if m > 0:
            out[:, 0:n, lmax + 1 - m] = alm_hp[pos:pos + n].imag.T
        pos += n
    return out


def gaussian_alm(cl: np.ndarray, lmax: int, nsim: int, rng: np.random.Generator,
                 lmin: int = 0) -> np.ndarray:
    """Gaussian square-real alm with power C_l: N(0, C_l) at m=0, N(0, C_l/2) per
    component at m>0 (the maths of cl2alm_T1, src/cl2alm_TEB.f90:127-171; the
    reference's MKL MCG31 stream is not reproducible, so this uses NumPy's PCG64)."""
    L = lmax + 1
    alm = np.zeros((nsim, L, L), order="F")
    sd = np.sqrt(np.maximum(cl[:L], 0.0))
    l = np.arange(L)
    alm[:, :, 0] = rng.standard_normal((nsim, L)) * sd[None, :]
    for m in range(1, L):
        n = L - m
        alm[:, m:, m] = rng.standard_normal((nsim, n)) * (sd[m:] / math.sqrt(2))[None, :]
        alm[:, 0:n, L - m] = rng.standard_normal((nsim, n)) * (sd[m:] / math.sqrt(2))[None, :]
    if lmin > 0:
        for m in range(0, min(lmin, L)):
            for ll in range(m, lmin):
                alm[:, ll, m] = 0
                if m > 0:
                    alm[:, ll - m, L - m] = 0
    del l
    return alm


def alm2cl(alm1: np.ndarray, alm2: np.ndarray | None = None, lmin: int = 0) -> np.ndarray:
    """Cross spectrum of square-real alm (nsim, L, L) -> (nsim, L): restates the loops of
    alm2cl_TEB1 / alm2cl_T1 (src/alm2cl_TEB.f90:22-110): sum over m of fac (Re Re + Im Im)
    / (2l+1), fac = 1 at m = 0 and 2 above; zero below lmin."""
    if alm2 is None:
        alm2 = alm1
    nsim, L, _ = alm1.shape
    cl = np.zeros((nsim, L))
    for m in range(L):
        fac = 1.0 if m == 0 else 2.0
        for l in range(max(m, lmin), L):
            t = alm1[:, l, m] * alm2[:, l, m]
            if m > 0:
                t = t + alm1[:, l - m, L - m] * alm2[:, l - m, L - m]
            cl[:, l] += t * fac / (2 * l + 1)
    return cl


def filt_alm(alm: np.ndarray, win: np.ndarray) -> np.ndarray:
    """alm(l, m) *= win(l) (filt_alm1, src/filt_alm.f90:16-37), returned as a new array."""
    out = np.array(alm, order="F", copy=True)
    nsim, L, _ = out.shape
    out[:, :, 0] *= win[None, :L]
    for m in range(1, L):
        out[:, m:, m] *= win[None, m:L]
        out[:, 0:L - m, L - m] *= win[None, m:L]
    return out


def norm_alm(alm: np.ndarray, fac: np.ndarray, shift: np.ndarray, m0: float) -> np.ndarray:
    """alm * fac(l) + shift(l), the m = 0 column also times m0 (norm_alm1,
    src/norm_alm.f90:14-35)."""
    out = np.empty_like(alm, order="F")
    nsim, L, _ = alm.shape
    out[:, :, 0] = alm[:, :, 0] * (fac[:L] * m0)[None, :] + shift[None, :L]
    for m in range(1, L):
        out[:, m:, m] = alm[:, m:, m] * fac[None, m:L] + shift[None, m:L]
        out[:, 0:L - m, L - m] = alm[:, 0:L - m, L - m] * fac[None, m:L] + shift[None, m:L]
    return out


# ---------------------------------------------------------------------------
# the transform object (one "plan"; the reference keeps this as module state)
# ---------------------------------------------------------------------------
class OracleSHT:
    """FP64 restatement of the reference's SHT state + drivers.

    ``ring_tab`` is the per-m first kept ring (the reference reads it from
    SHT_ring_skip_table; pass the reference's table to follow it exactly, or leave
    None to compute it with ``ring_skip_table``).
    """

    def __init__(self, nside: int, lmax: int, ring_tab=None, fft_workers: int | None = None,
                 use_c: bool = True):
        self.nside = nside
        self.lmax = lmax
        self.nring = 4 * nside - 1
        self.npix = 12 * nside * nside
        self.pa = 4 * PI / self.npix                      # sht_data_init.f90:18
        self.i1, self.nfft = ring_info(nside)
        self.theta, self.phi0 = ring_angles(nside)
        self.k = recursion_constants(nside, lmax, self.theta)
        if ring_tab is None:
            ring_tab = ring_skip_table(nside, lmax)
        self.ring_tab = np.asarray(ring_tab[:lmax + 1], dtype=np.int64)
        self.workers = fft_workers if fft_workers is not None else (os.cpu_count() or 1)
        self.use_c = bool(use_c) and c_recursion() is not None
        self._cc = np.ascontiguousarray(self.k["cc"])
        self._ss = np.ascontiguousarray(self.k["ss"])

    # --- set_locations (src/sht_core.f90:183-205)
    def locations(self, m):
        lmax, nring = self.lmax, self.nring
        n = lmax + 1 - m
        i0 = int(self.ring_tab[m])
        rlen = nring - 2 * i0
        i1 = i0 + rlen - 1
        p1 = (lmax + 2) * m
        p2 = (lmax + 1) * n
        return n, i0, rlen, i1, p1, p2

    # --- get_plm_recursive: full-sphere rows i0..nring-1-i0, columns l = m..lmax
    def plm(self, m, pol=False):
        i0 = int(self.ring_tab[m])
        n = self.lmax + 1 - m
        if self.use_c:
            import ctypes
            lib = c_recursion()
            rlen = self.nring - 2 * i0
            dp = ctypes.POINTER(ctypes.c_double)
            o0 = np.empty((rlen, n)) if not pol else np.empty((1, 1))
            o1 = np.empty((rlen, n)) if pol else o0
            o2 = np.empty((rlen, n)) if pol else o0
            pref = math.sqrt(self.k["diag_fac"][m] / 4 / PI)
            lib.oracle_plm_sphere(m, self.lmax, self.nside, i0, self._cc.ctypes.data_as(dp),
                                  self._ss.ctypes.data_as(dp), pref, int(self.nside > 512),
                                  int(pol), o0.ctypes.data_as(dp), o1.ctypes.data_as(dp),
                                  o2.ctypes.data_as(dp))
            return (o1, o2) if pol else o0
        p0n = plm_T(m, self.lmax, self.nside, self.k, i0)
        if not pol:
            return _mirror(p0n, m, self.nside, i0)[:, m:]
        p1n, p2n = plm_pol(m, self.lmax, self.nside, self.k, i0, p0n)
        return (_mirror(p1n, m, self.nside, i0)[:, m:], _mirror(p2n, m, self.nside, i0, 1)[:, m:])

    # --- map2fft (src/compute_fft.f90:71-110): unnormalised real FFT, PERM packing
    def map2fft(self, maps: np.ndarray) -> np.ndarray:
        nsim = maps.shape[1]
        buff = np.empty((nsim, self.npix))
        mT = np.ascontiguousarray(maps.T)                  # (nsim, npix)
        for n in np.unique(self.nfft):
            rings = np.nonzero(self.nfft == n)[0]
            idx = self.i1[rings][:, None] + np.arange(n)[None, :]
            x = mT[:, idx]                                 # (nsim, nr, n)
            X = scipy.fft.rfft(x, axis=-1, workers=self.workers)
            perm = np.empty_like(x)
            perm[..., 0] = X[..., 0].real
            perm[..., 1] = X[..., n // 2].real
            perm[..., 2::2] = X[..., 1:n // 2].real
            perm[..., 3::2] = X[..., 1:n // 2].imag
            buff[:, idx] = perm
        return buff

    # --- fft2map (src/compute_fft.f90:226-280): unnormalised inverse real FFT
    def fft2map(self, buff: np.ndarray) -> np.ndarray:
        nsim = buff.shape[0]
        out = np.empty((nsim, self.npix))
        for n in np.unique(self.nfft):
            rings = np.nonzero(self.nfft == n)[0]
            idx = self.i1[rings][:, None] + np.arange(n)[None, :]
            perm = buff[:, idx]
            X = np.empty(perm.shape[:-1] + (n // 2 + 1,), dtype=np.complex128)
            X[..., 0] = perm[..., 0]
            X[..., n // 2] = perm[..., 1]
            X[..., 1:n // 2] = perm[..., 2::2] + 1j * perm[..., 3::2]
            x = scipy.fft.irfft(X, n=n, axis=-1, workers=self.workers) * n
            out[:, idx] = x
        return np.asfortranarray(out.T)

    # --- fft2mat tables (src/sht_data_init.f90:438-492) for one m
    def _fwd_table(self, m):
        nfft, i1 = self.nfft, self.i1
        pos = m % nfft
        tab = np.where(pos == 0, i1, np.where(pos < nfft // 2, i1 + pos * 2,
                       np.where(pos == nfft // 2, i1 + 1, i1 + (nfft - pos) * 2)))
        ph = self.phi0
        c = np.cos(-m * ph)
        s = np.sin(-m * ph)
        posn = pos[:2 * self.nside]
        nn = nfft[:2 * self.nside]
        z = np.zeros_like(c)
        dc = (posn == 0) | (posn == nn // 2)
        posf = (posn > 0) & (posn < nn // 2)
        fac1 = c
        fac2 = np.where(dc, z, np.where(posf, -s, s))
        fac3 = s
        fac4 = np.where(dc, z, np.where(posf, c, -c))
        return tab, fac1, fac2, fac3, fac4

    # --- mat2fft tables (src/sht_data_init.f90:508-575) for one m
    def _inv_table(self, m):
        nfft, i1 = self.nfft, self.i1
        pos = m % nfft
        tab = np.where(pos == 0, i1, np.where(pos < nfft // 2, i1 + pos * 2,
                       np.where(pos == nfft // 2, i1 + 1, i1 + (nfft - pos) * 2)))
        fm0 = 1.0 if m == 0 else 2.0
        ph = self.phi0
        c = np.cos(m * ph)
        s = np.sin(m * ph)
        posn = pos[:2 * self.nside]
        nn = nfft[:2 * self.nside]
        dc = (posn == 0) | (posn == nn // 2)
        posf = (posn > 0) & (posn < nn // 2)
        z = np.zeros_like(c)
        fac1 = np.where(dc, c * fm0, c)
        fac2 = np.where(dc, -s * fm0, -s)
        fac3 = np.where(dc, z, np.where(posf, s, -s))
        fac4 = np.where(dc, z, np.where(posf, c, -c))
        return tab, fac1, fac2, fac3, fac4

    def _mirror_index(self, rings):
        return np.minimum(rings, self.nring - 1 - rings)

    # --- fft2mat_fast (src/fft_mapping.f90:19-68)
    def fft2mat(self, buff, m):
        n, i0, rlen, i1, p1, p2 = self.locations(m)
        tab, f1, f2, f3, f4 = self._fwd_table(m)
        rings = np.arange(i0, self.nring - i0)
        jf = self._mirror_index(rings)
        j = tab[rings]
        x0 = buff[:, j]
        x1 = buff[:, j + 1]
        mat1 = x0 * f1[jf] + x1 * f2[jf]
        mat2 = x0 * f3[jf] + x1 * f4[jf]
        return mat1, mat2                                   # (nsim, rlen), rings i0..i1

    def fft2mat_tables(self, m):
        """Per kept ring of order m: the first PERM bin and the four phase factors of
        fft2mat_fast (the reference computes these once, fft2mat_compute_table,
        sht_data_init.f90:438-492)."""
        n, i0, rlen, i1, p1, p2 = self.locations(m)
        tab, f1, f2, f3, f4 = self._fwd_table(m)
        rings = np.arange(i0, self.nring - i0)
        jf = self._mirror_index(rings)
        j = np.ascontiguousarray(tab[rings], dtype=np.int64)
        return j, [np.ascontiguousarray(f[jf], dtype=np.float64) for f in (f1, f2, f3, f4)]

    def fft2mat_c(self, buffT, m, tables=None):
        """fft2mat with the bins in the reference's memory order, buffT (npix, nsim) with the
        map index fastest, by oracle/plm.c (OpenMP over rings, like fft_mapping.f90:41).
        Returns (mat1, mat2) as (rlen, nsim) arrays: the transposes of fft2mat's.  `tables`:
        fft2mat_tables(m), when computed beforehand."""
        import ctypes
        lib = c_recursion()
        j, fs = tables if tables is not None else self.fft2mat_tables(m)
        rlen = len(j)
        nsim = buffT.shape[1]
        b = np.ascontiguousarray(buffT)
        mat1 = np.empty((rlen, nsim))
        mat2 = np.empty((rlen, nsim))
        dp = ctypes.POINTER(ctypes.c_double)
        lib.oracle_fft2mat(nsim, rlen, b.ctypes.data_as(dp),
                           j.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)),
                           *[f.ctypes.data_as(dp) for f in fs],
                           mat1.ctypes.data_as(dp), mat2.ctypes.data_as(dp))
        return mat1, mat2

    # --- mat2fft_fast (src/fft_mapping.f90:84-128)
    def mat2fft(self, buff, mat1, mat2, m):
        n, i0, rlen, i1, p1, p2 = self.locations(m)
        tab, f1, f2, f3, f4 = self._inv_table(m)
        rings = np.arange(i0, self.nring - i0)
        jf = self._mirror_index(rings)
        j = tab[rings]
        fac = np.where(2 * (m + 1) > self.nfft[rings], 1.0, 0.0)
        buff[:, j] = buff[:, j] * fac + mat1 * f1[jf] + mat2 * f2[jf]
        buff[:, j + 1] = buff[:, j + 1] * fac + mat1 * f3[jf] + mat2 * f4[jf]

    # --- mat2fft_fast_iter (src/fft_mapping.f90:142-190)
    def mat2fft_iter(self, buff1, buff2, mat1, mat2, m):
        n, i0, rlen, i1, p1, p2 = self.locations(m)
        tab, f1, f2, f3, f4 = self._inv_table(m)
        rings = np.arange(i0, self.nring - i0)
        jf = self._mirror_index(rings)
        j = tab[rings]
        nf = self.nfft[rings].astype(np.float64)
        acc = 2 * (m + 1) > self.nfft[rings]
        base0 = np.where(acc, buff2[:, j], buff1[:, j])
        base1 = np.where(acc, buff2[:, j + 1], buff1[:, j + 1])
        buff2[:, j] = base0 - mat1 * f1[jf] * nf - mat2 * f2[jf] * nf
        buff2[:, j + 1] = base1 - mat1 * f3[jf] * nf - mat2 * f4[jf] * nf

    # --- set_gemm_params_for_fft2alm (src/sht_data_init.f90:595-639)
    def gemm_params(self, inv, typ):
        s = self.pa if inv == 0 else 1.0
        if typ == 0:
            return s, s, 0
        if typ == 1:
            return -s, -s, 0
        if typ == 2:
            return s, -s, 1
        return -s, s, 1

    # --- mat2alm (src/sht_core.f90:62-89); alm2 is alm viewed (nsim, (lmax+1)^2) F-order
    def mat2alm(self, alm2, mat1, mat2, plm, m, typ, beta):
        n, i0, rlen, i1, p1, p2 = self.locations(m)
        a1, a2, swap = self.gemm_params(0, typ)
        B = plm                                             # (rlen, n): l = m..lmax
        A1, A2 = (mat1, mat2) if swap == 0 else (mat2, mat1)
        alm2[:, p1:p1 + n] = a1 * (A1 @ B) + beta * alm2[:, p1:p1 + n]
        if m > 0:
            alm2[:, p2:p2 + n] = a2 * (A2 @ B) + beta * alm2[:, p2:p2 + n]

    # --- alm2mat (src/sht_core.f90:141-168)
    def alm2mat(self, alm2, plm, m, typ, beta, mat1, mat2):
        n, i0, rlen, i1, p1, p2 = self.locations(m)
        a1, a2, swap = self.gemm_params(1, typ)
        B = plm                                             # (rlen, n): l = m..lmax
        if swap == 0:
            mat1[:] = a1 * (alm2[:, p1:p1 + n] @ B.T) + beta * mat1
            if m > 0:
                mat2[:] = a2 * (alm2[:, p2:p2 + n] @ B.T) + beta * mat2
        else:
            if m == 0:
                mat1[:] = a1 * (alm2[:, p1:p1 + n] @ B.T) + beta * mat1
            else:
                mat2[:] = a1 * (alm2[:, p1:p1 + n] @ B.T) + beta * mat2
                mat1[:] = a2 * (alm2[:, p2:p2 + n] @ B.T) + beta * mat1

    # ------------------------------------------------------------------
    # drivers (src/sht_main.f90)
    # ------------------------------------------------------------------
    def _new_alm(self, nsim):
        L = self.lmax + 1
        alm = np.zeros((nsim, L, L), order="F")
        return alm, alm.reshape(nsim, L * L, order="F")

    def _zero_unused_bins(self, buff):
        """sht_main.f90:138-146: zero PERM slots above 2(lmax+1) on long rings."""
        for i in range(self.nring):
            if 2 * (self.lmax + 1) < self.nfft[i]:
                buff[:, 2 * (self.lmax + 1) + self.i1[i]:self.i1[i] + self.nfft[i]] = 0

    def _analysis_T(self, buff, alm2, beta):
        for m in range(self.lmax + 1):
            mat1, mat2 = self.fft2mat(buff, m)
            self.mat2alm(alm2, mat1, mat2, self.plm(m), m, 0, beta)

    def t2alm_timed(self, maps, m_stride=1):
        """t2alm with wall-clock phase times (seconds): ring FFT, recursion (which
        the reference computes once per m for the whole batch) and the per-m
        gather + DGEMMs.  Used by the CPU baseline to scale a map sample to a batch.
        m_stride > 1 times every m_stride-th order only and scales the recursion and
        GEMM times by m_stride (the alm of the other orders stay zero)."""
        import time
        t0 = time.perf_counter()
        nsim = maps.shape[1]
        buff = self.map2fft(maps)
        t1 = time.perf_counter()
        alm, alm2 = self._new_alm(nsim)
        t_plm = 0.0
        t_gemm = 0.0
        for m in range(0, self.lmax + 1, m_stride):
            ta = time.perf_counter()
            plm = self.plm(m)
            tb = time.perf_counter()
            mat1, mat2 = self.fft2mat(buff, m)
            self.mat2alm(alm2, mat1, mat2, plm, m, 0, 0.0)
            tc = time.perf_counter()
            t_plm += tb - ta
            t_gemm += tc - tb
        return alm, {"fft": t1 - t0, "plm": t_plm * m_stride, "gemm": t_gemm * m_stride}

    def t2alm(self, maps):
        """t2alm (sht_main.f90:38-89)."""
        nsim = maps.shape[1]
        buff = self.map2fft(maps)
        alm, alm2 = self._new_alm(nsim)
        self._analysis_T(buff, alm2, 0.0)
        return alm

    def _synth_T_bins(self, alm2, nsim):
        buff = np.zeros((nsim, self.npix))
        for m in range(self.lmax + 1):
            n, i0, rlen, i1, p1, p2 = self.locations(m)
            mat1 = np.zeros((nsim, rlen))
            mat2 = np.zeros((nsim, rlen))
            self.alm2mat(alm2, self.plm(m), m, 0, 0.0, mat1, mat2)
            self.mat2fft(buff, mat1, mat2, m)
        return buff

    def alm2t(self, alm):
        """alm2t (sht_main.f90:96-155)."""
        nsim = alm.shape[0]
        alm2 = np.asfortranarray(alm).reshape(nsim, -1, order="F")
        buff = self._synth_T_bins(alm2, nsim)
        self._zero_unused_bins(buff)
        return self.fft2map(buff)

    def t2alm_iter_old(self, maps, niter):
        """t2alm_iter_old (sht_main.f90:276-367): Jacobi iterations in Fourier space."""
        nsim = maps.shape[1]
        buff1 = self.map2fft(maps)
        alm, alm2 = self._new_alm(nsim)
        self._analysis_T(buff1, alm2, 0.0)
        buff2 = np.zeros_like(buff1)
        for _ in range(niter):
            for m in range(self.lmax + 1):
                n, i0, rlen, i1, p1, p2 = self.locations(m)
                mat1 = np.zeros((nsim, rlen))
                mat2 = np.zeros((nsim, rlen))
                self.alm2mat(alm2, self.plm(m), m, 0, 0.0, mat1, mat2)
                self.mat2fft_iter(buff1, buff2, mat1, mat2, m)
            self._analysis_T(buff2, alm2, 1.0)
        return alm

    def t2alm_iter(self, maps, niter):
        """t2alm_iter (sht_main.f90:171-264): per-m interleaved update ("new" method)."""
        nsim = maps.shape[1]
        buff1 = self.map2fft(maps)
        alm, alm2 = self._new_alm(nsim)
        self._analysis_T(buff1, alm2, 0.0)
        buff2 = np.zeros_like(buff1)
        for _ in range(niter):
            for m in range(self.lmax + 1):
                n, i0, rlen, i1, p1, p2 = self.locations(m)
                mat1 = np.zeros((nsim, rlen))
                mat2 = np.zeros((nsim, rlen))
                plm = self.plm(m)
                self.alm2mat(alm2, plm, m, 0, 0.0, mat1, mat2)
                self.mat2fft_iter(buff1, buff2, mat1, mat2, m)
                m1, m2 = self.fft2mat(buff2, m)
                self.mat2alm(alm2, m1, m2, plm, m, 0, 1.0)
        return alm

    # --- spin 2
    def _analysis_pol(self, bq, bu, e2, b2, beta, which="EB"):
        for m in range(self.lmax + 1):
            plm1, plm2 = self.plm(m, pol=True)
            q1, q2 = self.fft2mat(bq, m)
            u1, u2 = self.fft2mat(bu, m)
            if "E" in which:
                self.mat2alm(e2, q1, q2, plm1, m, 1, beta)
                self.mat2alm(e2, u1, u2, plm2, m, 2, 1.0)
            if "B" in which:
                self.mat2alm(b2, q1, q2, plm2, m, 3, beta)
                self.mat2alm(b2, u1, u2, plm1, m, 1, 1.0)

    def qu2eb(self, Q, U):
        """QU2EB (sht_main.f90:383-436)."""
        nsim = Q.shape[1]
        bq, bu = self.map2fft(Q), self.map2fft(U)
        almE, e2 = self._new_alm(nsim)
        almB, b2 = self._new_alm(nsim)
        self._analysis_pol(bq, bu, e2, b2, 0.0)
        return almE, almB

    def qu2e(self, Q, U):
        """QU2E (sht_main.f90:955-1005)."""
        nsim = Q.shape[1]
        bq, bu = self.map2fft(Q), self.map2fft(U)
        almE, e2 = self._new_alm(nsim)
        self._analysis_pol(bq, bu, e2, None, 0.0, which="E")
        return almE

    def qu2b(self, Q, U):
        """QU2B (sht_main.f90:1016-1064): B from U with plm1 (type 1) then Q with plm2 (type 3)."""
        nsim = Q.shape[1]
        bq, bu = self.map2fft(Q), self.map2fft(U)
        almB, b2 = self._new_alm(nsim)
        self._analysis_pol(bq, bu, None, b2, 0.0, which="B")
        return almB

    def _synth_pol_bins(self, e2, b2, nsim, base=None):
        bq = np.zeros((nsim, self.npix))
        bu = np.zeros((nsim, self.npix))
        for m in range(self.lmax + 1):
            n, i0, rlen, i1, p1, p2 = self.locations(m)
            plm1, plm2 = self.plm(m, pol=True)
            mq1 = np.zeros((nsim, rlen)); mq2 = np.zeros((nsim, rlen))
            mu1 = np.zeros((nsim, rlen)); mu2 = np.zeros((nsim, rlen))
            self.alm2mat(e2, plm1, m, 1, 0.0, mq1, mq2)
            self.alm2mat(b2, plm2, m, 3, 1.0, mq1, mq2)
            self.alm2mat(e2, plm2, m, 2, 0.0, mu1, mu2)
            self.alm2mat(b2, plm1, m, 1, 1.0, mu1, mu2)
            if base is None:
                self.mat2fft(bq, mq1, mq2, m)
                self.mat2fft(bu, mu1, mu2, m)
            else:
                self.mat2fft_iter(base[0], bq, mq1, mq2, m)
                self.mat2fft_iter(base[1], bu, mu1, mu2, m)
        return bq, bu

    def eb2qu(self, almE, almB):
        """EB2QU (sht_main.f90:1079-1147)."""
        nsim = almE.shape[0]
        e2 = np.asfortranarray(almE).reshape(nsim, -1, order="F")
        b2 = np.asfortranarray(almB).reshape(nsim, -1, order="F")
        bq, bu = self._synth_pol_bins(e2, b2, nsim)
        self._zero_unused_bins(bq)
        self._zero_unused_bins(bu)
        return self.fft2map(bq), self.fft2map(bu)

    def fix_eb(self, Q, U, mask, niter):
        """EB-leakage cleaning (fix_eb, sht_main.f90:801-941; lin_resi_mini,
        sht_core.f90:232-253): mask Q/U, iterate to E/B, synthesise Q/U from E alone, mask
        again, iterate to the leakage template's B, take both B alm to pixels with the
        spin-0 synthesis, and on the pixels where mask == 1 return the residual of the
        per-map linear fit of the B map on the template (zero elsewhere)."""
        m = np.asarray(mask, dtype=np.float64)[:, None]
        almE, almB = self.qu2eb_iter_old(Q * m, U * m, niter)
        q2, u2 = self.eb2qu(almE, np.zeros_like(almE))
        _, btpl_alm = self.qu2eb_iter_old(q2 * m, u2 * m, niter)
        bmap = self.alm2t(almB)
        btpl = self.alm2t(btpl_alm)
        vid = np.flatnonzero(np.asarray(mask) == 1)
        out = np.zeros_like(bmap)
        x, y = btpl[vid], bmap[vid]
        mx, my = x.mean(axis=0), y.mean(axis=0)
        a1 = ((y - my) * (x - mx)).sum(axis=0) / ((x - mx) ** 2).sum(axis=0)
        a0 = my - mx * a1
        out[vid] = y - a0 - a1 * x
        return out

    def qu2eb_iter_old(self, Q, U, niter):
        """qu2eb_iter_old (sht_main.f90:563-673)."""
        nsim = Q.shape[1]
        bq, bu = self.map2fft(Q), self.map2fft(U)
        almE, e2 = self._new_alm(nsim)
        almB, b2 = self._new_alm(nsim)
        self._analysis_pol(bq, bu, e2, b2, 0.0)
        for _ in range(niter):
            rq, ru = self._synth_pol_bins(e2, b2, nsim, base=(bq, bu))
            self._analysis_pol(rq, ru, e2, b2, 1.0)
        return almE, almB
