"""fastsht_gb300: batched HEALPix spherical-harmonic transforms on NVIDIA GB300.

A from-scratch sm_103a implementation of the batched SHT path of
liuhao-cn/fastSHT behind the same ``SHT`` class surface (see ``sht.SHT``), with
the transforms in a C-ABI CUDA library (``include/fastsht.h``).
"""
from .sht import SHT, pinned_empty  # noqa: F401

__all__ = ["SHT", "pinned_empty"]
