"""Golden pattern files: small .ebsp, .pat and .up2 files written by the reference's own writers,
with what the reference's own readers return for them.

Run from the repository root on a machine that has the reference source tree:

    python tests/golden/make_pattern_file_golden.py   # writes tests/golden/patfiles/*

For each case the reference's writer (``EBSPFile`` / ``TFPatFile`` / ``UPFile`` ``write_data`` on a
new file, ebsd_pattern.py:335-400 with each format's ``write_header`` / ``pat_writer``) writes
the file, then the reference's ``get_pattern_file_obj`` reads it back (``read_header``, then
``read_data`` of every pattern and of a slab).  Stored beside each file, in ``<name>.npz``: the
header attributes, the patterns and positions of both reads.  The reference is imported through
``oracle/refshim.py``.
"""
from __future__ import annotations

import os
import sys
import warnings

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "patfiles")

from oracle import refshim  # noqa: E402

ATTRS = ("version", "patternW", "patternH", "filePos", "nPatterns", "nCols", "nRows", "xStep", "yStep",
         "filedatatype", "hasxypos", "bitdepth", "hasbackground", "extraPatterns", "hexflag")
SLAB = [[1, 1], [2, 2]]


def patterns(seed, n, h, w, hi, dtype):
    return np.random.default_rng(seed).integers(0, hi, size=(n, h, w)).astype(dtype)


def write_ebsp(rp, path, version, xy):
    pats = patterns(10 + version, 12, 9, 11, 256, np.uint8)
    f = rp.EBSPFile(path)
    f.version = np.int64(version)  # numpy 2 refuses np.uint64 of a negative Python int
    f.nCols, f.nRows, f.nPatterns, f.patternW, f.patternH = 4, 3, 12, 11, 9
    f.xStep, f.yStep, f.hasxypos = 0.5, 0.75, xy
    f.write_data(newpatterns=pats, patStartCount=[0, -1])


def write_tfpat(rp, path):
    pats = patterns(20, 12, 9, 11, 4096, np.uint16)
    f = rp.TFPatFile(path)
    f.version, f.nCols, f.nRows, f.nPatterns = 1, np.uint32(4), np.uint32(3), 12
    f.patternW, f.patternH, f.bitdepth, f.hasbackground = np.uint32(11), np.uint32(9), 12, True
    f.filedatatype = np.uint16
    f.filePos = 25 + 11 * 9 * 2
    f.write_data(newpatterns=pats, patStartCount=[0, -1])


def write_up2(rp, path):
    pats = patterns(30, 12, 9, 11, 4096, np.uint16)
    f = rp.UPFile(path)
    f.version, f.patternW, f.patternH = 3, 11, 9
    f.nCols, f.nRows, f.nPatterns, f.xStep, f.yStep = 4, 3, 12, 1.5, 2.25
    f.extraPatterns, f.hexflag, f.filedatatype = 0, 0, np.uint16
    f.write_data(newpatterns=pats, patStartCount=[0, -1], writeHead=True)


def main():
    rp = refshim.pattern_module()
    os.makedirs(OUT, exist_ok=True)
    cases = {"ebsp_v2_xy.ebsp": lambda p: write_ebsp(rp, p, 2, True),
             "ebsp_v4_noxy.ebsp": lambda p: write_ebsp(rp, p, 4, False),
             "tfpat_bg12.pat": lambda p: write_tfpat(rp, p),
             "up2_v3.up2": lambda p: write_up2(rp, p)}
    for name, write in cases.items():
        path = os.path.join(OUT, name)
        if os.path.exists(path):
            os.remove(path)
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            write(path)
            f = rp.get_pattern_file_obj(path)
            allp, allxy = f.read_data(patStartCount=[0, -1], returnArrayOnly=True)
            slab, slabxy = f.read_data(patStartCount=SLAB, returnArrayOnly=True)
        rec = {"patterns": allp, "xy": allxy, "slab": slab, "slab_xy": slabxy}
        for a in ATTRS:
            if hasattr(f, a):
                v = getattr(f, a)
                rec["attr_" + a] = np.asarray(np.dtype(v).name if a == "filedatatype" else v)
        np.savez(os.path.join(OUT, os.path.splitext(name)[0] + ".npz"), **rec)
        print(name, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
