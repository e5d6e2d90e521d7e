"""Decoder of the wide / quantised node records (layout in csrc/wide.h), for
inspection, serialisation and tests."""
from __future__ import annotations

import numpy as np


def header_bytes(bits: int) -> int:
    return 0 if bits == 32 else 16


def layout(W: int, bits: int):
    cnt = header_bytes(bits) + 4 * W
    bounds = (cnt + W + 3) // 4 * 4
    size = (bounds + 6 * W * (bits // 8) + 15) // 16 * 16
    return {"refs": header_bytes(bits), "cnt": cnt, "bounds": bounds, "size": size}


def decode(raw: np.ndarray, W: int, bits: int) -> dict:
    """raw: (n, node_bytes) uint8. Returns refs (n, W) uint32, cnt (n, W) uint8,
    and for quantised layouts origin (n, 3) float32, exponent (n, 3) int, q (n, 6, W)
    (lo x/y/z then hi x/y/z); for 32-bit layouts bounds (n, 6, W) float32."""
    L = layout(W, bits)
    n = raw.shape[0]
    out = {"refs": raw[:, L["refs"]:L["refs"] + 4 * W].copy().view("<u4").reshape(n, W),
           "cnt": raw[:, L["cnt"]:L["cnt"] + W].copy()}
    b = raw[:, L["bounds"]:L["bounds"] + 6 * W * (bits // 8)].copy()
    if bits == 32:
        out["bounds"] = b.view("<f4").reshape(n, 6, W)
    else:
        out["origin"] = raw[:, 0:12].copy().view("<f4").reshape(n, 3)
        out["exponent"] = raw[:, 12:15].astype(np.int32) - 127
        out["q"] = (b.view("<u2") if bits == 16 else b).reshape(n, 6, W).astype(np.uint32)
    return out
