"""Generate tests/golden/zfp_large.json: SHA-256 digests of the streams the REFERENCE's own
zfp2d_lossyCompression (ZFP 0.5.5 built from the reference's sources by oracle/build_ref.sh)
writes for a large seismogram-like field, and of their decodes.

The field (portable_field) is built from integer arithmetic only, so that every machine
regenerates it bit for bit; the digests then pin the engine's encoder and decoder on a field
large enough for the threaded encoder, on machines without the reference tree.

    python tests/golden/make_zfp_large.py
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import Reference  # noqa: E402

OUT = os.path.join(HERE, "zfp_large.json")
SHAPE = (3400, 750)            # receivers x time samples (zfp nx = receivers, fastest)
TOLERANCES = (1e-4, 1e-6, 0.0)


def portable_field() -> np.ndarray:
    """A (3400, 750) float32 field of integer multiples of 2^-20: hyperbola-like events
    (integer distance arithmetic), a seeded integer noise floor, and 48 all-zero leading
    samples (empty blocks)."""
    nrec, nt = SHAPE
    x = np.arange(nrec, dtype=np.int64)[:, None]
    t = np.arange(nt, dtype=np.int64)[None, :]
    f = np.zeros(SHAPE, np.int64)
    for k, (t0, v) in enumerate(((120, 7), (260, 5), (410, 9), (600, 4))):
        # arrival sample of event k at receiver x: t0 + |x - 1700| * |x - 1700| / (v * 4096)
        dx = np.abs(x - 1700)
        tk = t0 + (dx * dx) // (v * 4096)
        d = t - tk
        amp = (1 << 20) >> k
        f += np.where(np.abs(d) < 12, amp * (12 - np.abs(d)) * np.where(d % 2 == 0, 1, -1) // 12, 0)
    rng = np.random.default_rng(2024)
    f += rng.integers(-1024, 1025, size=SHAPE, dtype=np.int64)
    f[:, :48] = 0
    return (f.astype(np.float64) / float(1 << 20)).astype(np.float32)


def sha(b: bytes) -> str:
    return hashlib.sha256(b).hexdigest()


def main():
    ref = Reference()
    f = np.ascontiguousarray(portable_field())
    out = {"shape": list(SHAPE), "field_sha256": sha(f.tobytes()), "streams": {}}
    for tol in TOLERANCES:
        blob = ref.zfp_compress(f, SHAPE[0], SHAPE[1], tol)
        with tempfile.NamedTemporaryFile(suffix=".zfp", delete=False) as fh:
            fh.write(blob)
            path = fh.name
        try:
            dec = ref.zfp_decompress(path, SHAPE[0], SHAPE[1], tol)
        finally:
            os.unlink(path)
        out["streams"][repr(tol)] = {"bytes": len(blob), "stream_sha256": sha(blob),
                                     "decoded_sha256": sha(np.ascontiguousarray(dec, np.float32).tobytes())}
    with open(OUT, "w") as fh:
        json.dump(out, fh, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
