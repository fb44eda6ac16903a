"""Drop-in for an installed PyEBSDIndex.

``gpu_band_detect_class(base)`` returns a subclass of ``base`` (normally the reference's
``pyebsdindex.band_detect.BandDetect``) whose ``find_bands`` runs on the GPU.  The reference's
own ``band_detect_setup``/``collect_background`` then build the plan, and its ``radonPlan`` stays
a reference ``radon_fast.Radon`` -- which ``EBSDIndexer`` requires (it hands the object to
``gnomonic_correction.GnomonicCorrection``, which type-checks it).  Install with::

    from pyebsdindex import band_detect, ebsd_index
    from pyebsdindex_gb300.plugin import gpu_band_detect_class
    BD = gpu_band_detect_class(band_detect.BandDetect)
    indexer = ebsd_index.EBSDIndexer(bandDetectPlan=BD(nRho=90, nTheta=180, ...), patDim=(H, W))
    indexer.index_pats(patterns)          # band detection on the GPU, voting unchanged

(the seam is ``EBSDIndexer(bandDetectPlan=...)``, _ebsd_index_single.py:386-398).
"""
from __future__ import annotations

from .band_detect import GPUFindBands

_cache = {}


def gpu_band_detect_class(base):
    """Subclass ``base`` so that ``find_bands`` dispatches to the GPU."""
    if base in _cache:
        return _cache[base]

    def __init__(self, *args, method=None, gpu_id=0, **kwargs):
        base.__init__(self, *args, **kwargs)
        self.useCPU = False
        self.gpu_id = int(gpu_id or 0)
        if method is not None:
            self.default_method = method

    cls = type("BandDetectGPU", (GPUFindBands, base), {"__init__": __init__, "__doc__": GPUFindBands.__doc__})
    _cache[base] = cls
    return cls
