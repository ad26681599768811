"""Regenerates the golden fixtures from the reference tree (run in a container
where the reference is mounted; the GPU machine does not need it).

    python tests/golden/make_golden.py /root/reference

Writes:
  plm_golden.npz   : for nside in 1..128 (every m up to 32, then every 2nd / 8th m): the reference's
                     plm_table/plm_{pos,val1,val2}_<nside>.bin, i.e.
                     lambda_{pos,m}(theta_i), lambda_{pos+1,m}(theta_i) for north
                     rings i < 2 nside (Fortran order (2 nside, 4 nside + 1)).
  ring_skip.npz    : the reference's SHT_ring_skip_table/<nside>.bin for every
                     nside it ships (first kept ring per m).
"""
import sys
from pathlib import Path

import numpy as np

if len(sys.argv) != 2:
    sys.exit("usage: make_golden.py <path of the reference tree>")
ref = Path(sys.argv[1])
out = Path(__file__).resolve().parent

plm = {}
for ns in (1, 2, 4, 8, 16, 32, 64, 128):
    pos = np.fromfile(ref / f"plm_table/plm_pos_{ns:04d}.bin", dtype=np.int32)
    v1 = np.fromfile(ref / f"plm_table/plm_val1_{ns:04d}.bin", dtype=np.float64)
    v2 = np.fromfile(ref / f"plm_table/plm_val2_{ns:04d}.bin", dtype=np.float64)
    ncol = len(pos) // (2 * ns)
    pos = pos.reshape(2 * ns, ncol, order="F")
    v1 = v1.reshape(2 * ns, ncol, order="F")
    v2 = v2.reshape(2 * ns, ncol, order="F")
    step = 1 if ns <= 32 else (2 if ns == 64 else 8)
    cols = np.arange(0, ncol, step)
    plm[f"cols_{ns}"] = cols.astype(np.int32)
    plm[f"pos_{ns}"] = pos[:, cols]
    plm[f"val1_{ns}"] = v1[:, cols]
    plm[f"val2_{ns}"] = v2[:, cols]
np.savez_compressed(out / "plm_golden.npz", **plm)

skip = {}
for f in sorted((ref / "SHT_ring_skip_table").glob("*.bin")):
    skip[f"ns_{int(f.stem)}"] = np.fromfile(f, dtype=np.int32)
np.savez_compressed(out / "ring_skip.npz", **skip)
print("wrote", out / "plm_golden.npz", out / "ring_skip.npz")
