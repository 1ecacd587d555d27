"""Block/cell agreement rules of the particle parity checks (GPU against the
FP64 oracle).

The GPU keeps positions as FP32 block-local offsets u in [0, 8) cell units;
the oracle keeps FP64 positions.  Both locate a particle with the same rules
(findTreeNode / FindCellIndex, src/meshAMR/meshAMRgeneric.h:2256-2320,
2852-2883), so their block and cell agree unless a cell face lies between the
two positions.  A disagreement is accepted only when

  * a face of the oracle's cell lies between the oracle's and the GPU's
    position along some axis (the face is within |dx_gpu - dx_oracle| of the
    oracle position on that axis), and
  * that position difference is at most ULP_BOUND units in the last place of
    an offset in [4, 8) (2^-21 cell), the FP32 rounding of the offset.

Everything here is plain numpy on exported arrays.
"""
import numpy as np

ULP8 = 2.0 ** -21          # one FP32 ulp of a block-local offset in [4, 8), in cells
ULP_BOUND = 4.0            # accepted position difference of a face particle, in ULP8


def _wrap(d, L):
    return d - L * np.rint(d / L)


def mismatch_report(x_gpu, blk_gpu, cell_gpu, x_orc, blk_orc, cell_orc, origins, dxb, L):
    """x_* (n,3) FP64 positions, blk_*/cell_* ids, origins (nblocks,3) block
    origins, dxb (nblocks,) cell size per block, L (3,) periodic domain length.
    Returns a dict: mismatches, the largest position difference of a
    mismatched particle in ULP8 of its GPU block, whether every mismatch
    straddles a face of the oracle's cell, and the ids of those that do not."""
    same = (blk_gpu == blk_orc) & (cell_gpu == cell_orc)
    bad = np.flatnonzero(~same)
    out = {"particles": int(len(same)), "mismatches": int(bad.size), "max_offset_ulps": 0.0,
           "face_rule_holds": True, "violations": []}
    if bad.size == 0:
        return out
    dlt = np.abs(_wrap(x_gpu[bad] - x_orc[bad], np.asarray(L, float)))      # (m,3)
    bo = blk_orc[bad]
    u = (x_orc[bad] - origins[bo]) / dxb[bo][:, None]                       # oracle cell units
    u = np.where(u < 0, u + (np.asarray(L, float) / dxb[bo][:, None]), u)    # periodic image
    face = np.abs(u - np.rint(u)) * dxb[bo][:, None]                        # distance to a face
    straddle = np.any(face <= dlt * (1 + 1e-9) + 1e-15, axis=1)
    ulps = np.max(dlt, axis=1) / (dxb[blk_gpu[bad]] * ULP8)
    ok = straddle & (ulps <= ULP_BOUND)
    out["max_offset_ulps"] = float(ulps.max())
    out["face_rule_holds"] = bool(ok.all())
    out["violations"] = [int(i) for i in bad[~ok][:10]]
    return out
