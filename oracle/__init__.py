"""CPU oracle for the batched HEALPix SHT path.

TEST INFRASTRUCTURE ONLY. This package is the checker: a plain FP64 NumPy/SciPy
restatement of liuhao-cn/fastSHT's transform path (ring FFT -> FFT-matrix -> per-m
Legendre DGEMM and back). Only ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline leg may import it. The product path
(``fastsht_gb300``) never imports, calls or links anything here.

Parity pins (checked by ``tests/test_oracle_golden.py``):
  * ``plm_table/plm_val{1,2}_*.bin``: lambda_{pos,m}(theta_i), lambda_{pos+1,m}(theta_i)
    at the HEALPix ring colatitudes (golden vectors for theta_i and the recursion);
  * ``SHT_ring_skip_table/*.bin``: which rings the reference drops per m;
  * analytic known answers: a constant map gives a00 = sqrt(4 pi) c; alm2map of a
    single a_lm equals Y_lm at the pixel centres.
The FFT/DGEMM library boundary (MKL DFTI, MKL/cuBLAS DGEMM) is not vendored in the
reference, so those steps use scipy.fft and NumPy BLAS, which compute the same
exact-arithmetic quantities.
"""
import os as _os

# The C recursion (OpenMP) alternates with multithreaded BLAS calls; spinning
# OpenMP workers would starve the BLAS threads.  Must be set before libgomp loads.
_os.environ.setdefault("OMP_WAIT_POLICY", "PASSIVE")

from .sht_oracle import *  # noqa: F401,F403,E402
