"""Persisted autotuner decisions.

``BandDetect.autotune`` times the record-identical variants of the fused kernel -- Radon tile
shapes: the whole padded Radon image as one tile with one, two, four or eight patterns per block
pass, and theta slabs of several widths -- on a sample.  With ``cache=`` the decision is stored in
a JSON file keyed by everything that can change it -- the GPU (name and SM count), the
library version, the pattern shape and input type, the Radon geometry (nTheta, nRho, nBands,
LoG size, padding, a digest of the lookup table, background) and the method -- and a later
call with the same key applies the stored choice without timing anything.  The reference has
no autotuner; its nearest counterpart sizes GPU chunks from the device's memory
(``__optimizegpuchunk__``, _ebsd_index_parallel.py:768-828) each run.

File layout: ``{"format": 1, "entries": {key: {"patterns_per_pass": p, "tile": t, "slabs": s,
"timed_patterns": n}}}`` (tile 1: one tile, 2: theta slabs, s slabs; entries written before the
tile shape was tuned hold the patterns per pass alone and keep the plan's rule for the shape).
Writes merge with what the file holds and replace it atomically, so processes that tune
different plans can share one file.
"""
from __future__ import annotations

import hashlib
import json
import os
import tempfile

__all__ = ["TuningCache", "default_path", "plan_key"]

ENV_PATH = "PYEBSDINDEX_GB300_TUNING"
FORMAT = 1


def default_path() -> str:
    """``$PYEBSDINDEX_GB300_TUNING``, else ``$XDG_CACHE_HOME`` (or ``~/.cache``) /
    ``pyebsdindex_gb300/tuning.json``."""
    p = os.environ.get(ENV_PATH)
    if p:
        return p
    base = os.environ.get("XDG_CACHE_HOME") or os.path.join(os.path.expanduser("~"), ".cache")
    return os.path.join(base, "pyebsdindex_gb300", "tuning.json")


def lut_digest(lut) -> str:
    """Short digest of a Radon lookup table (its shape and entries)."""
    import numpy as np
    a = np.ascontiguousarray(lut)
    h = hashlib.sha1(repr((a.shape, str(a.dtype))).encode())
    h.update(a.tobytes())
    return h.hexdigest()[:16]


def plan_key(*, gpu: str, sms: int, library: str, shape, dtype: int, method: str, nTheta: int, nRho: int,
             nBands: int, kernel_shape, padding, peakPad, lut: str, background: bool) -> str:
    """The key under which a tuning decision is stored."""
    parts = [f"gpu={gpu}", f"sms={int(sms)}", f"lib={library}", "shape=%dx%d" % tuple(int(v) for v in shape),
             f"dtype={int(dtype)}", f"method={method}", f"nTheta={int(nTheta)}", f"nRho={int(nRho)}",
             f"nBands={int(nBands)}", "kernel=%s" % "x".join(str(int(v)) for v in kernel_shape),
             "padding=%s" % ",".join(str(int(v)) for v in padding),
             "peakPad=%s" % ",".join(str(int(v)) for v in peakPad), f"lut={lut}", f"bg={int(bool(background))}"]
    return "|".join(parts)


class TuningCache:
    """A JSON file of tuning decisions (``path``: a file name, or True for ``default_path()``)."""

    def __init__(self, path=True):
        self.path = default_path() if path is True else os.fspath(path)

    def _load(self) -> dict:
        try:
            with open(self.path, "r", encoding="utf-8") as f:
                doc = json.load(f)
        except FileNotFoundError:
            return {}
        except (OSError, ValueError):
            return {}  # unreadable or corrupt: treated as empty, rewritten on the next put
        if not isinstance(doc, dict) or doc.get("format") != FORMAT or not isinstance(doc.get("entries"), dict):
            return {}
        return doc["entries"]

    def get(self, key: str):
        """The stored decision for ``key`` (a dict), or None."""
        v = self._load().get(key)
        return v if isinstance(v, dict) else None

    def put(self, key: str, value: dict) -> None:
        """Store ``value`` under ``key``: merged with the file's entries, written atomically."""
        entries = self._load()
        entries[key] = dict(value)
        d = os.path.dirname(os.path.abspath(self.path))
        os.makedirs(d, exist_ok=True)
        fd, tmp = tempfile.mkstemp(prefix=".tuning.", suffix=".json", dir=d)
        try:
            with os.fdopen(fd, "w", encoding="utf-8") as f:
                json.dump({"format": FORMAT, "entries": entries}, f, indent=1, sort_keys=True)
            os.replace(tmp, self.path)
        except BaseException:
            try:
                os.unlink(tmp)
            except OSError:
                pass
            raise
