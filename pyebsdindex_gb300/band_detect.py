"""GPU band detection behind the reference ``BandDetect`` interface.

``BandDetect`` here has the constructor, attributes and methods of the reference's
``band_detect.BandDetect`` (band_detect.py:67-933) that ``EBSDIndexer``, ``pcopt`` and user code
touch -- ``band_detect_setup``, ``collect_background``, ``backsub_fit``, ``find_bands``,
``radonPlan``, ``rdnmask``, ``kernel``, ``peakPad``, ``padding``, ``dataType`` ... -- but
``find_bands`` runs on the GPU through libebsdgpu.so.  There is no CPU fallback: without the
library or a CUDA device, ``find_bands`` raises.

``GPUFindBands`` is the find_bands implementation on its own, usable as a mixin over any class
that carries the reference's plan attributes; ``pyebsdindex_gb300.plugin`` uses it to subclass
the reference's own ``BandDetect`` when PyEBSDIndex is installed.
"""
from __future__ import annotations

import hashlib
from timeit import default_timer as timer

import numpy as np
import scipy.ndimage as ndi
import scipy.optimize as opt

from . import _lib
from .radon_fast import Radon

RADEG = 180.0 / np.pi

__all__ = ["BandDetect", "GPUFindBands", "getopenclparam", "record_dtype"]


def record_dtype(nPhases=10):
    """The band record (band_detect.py:110-115)."""
    return np.dtype([('id', np.int32), ('max', np.float32), ('normmax', np.float32),
                     ('maxloc', np.float32, (2)), ('avemax', np.float32), ('aveloc', np.float32, (2)),
                     ('pqmax', np.float32), ('width', np.float32), ('theta', np.float32),
                     ('rho', np.float32), ('valid', np.int8),
                     ('band_match_index', np.int64, (nPhases,)),
                     ('bandfit', np.float64, (nPhases,))])


def getopenclparam(**kwargs):
    """Compatibility stub for callers of band_detect.getopenclparam (band_detect.py:932-933)."""
    return None


def _digest(*arrays):
    """Key of the plan inputs for the device-plan cache.  Arrays up to 1 MiB are hashed in
    full; larger ones (the Radon LUT, 13.8 MB at 80x80) by 4,096 evenly spaced elements, so
    that the per-call cost stays far below a chunk's GPU time (EBSDIndexer calls find_bands per
    chunk of ~528 patterns).  Large arrays are also matched by object identity: the cache
    holds a reference to them (``_large_inputs``), so a new array can never take a cached
    array's address.  Editing a large array in place is detected only where the sample
    changes."""
    h = hashlib.sha1()
    for a in arrays:
        if a is None:
            h.update(b"none")
            continue
        a = np.asarray(a)
        h.update(str(a.dtype).encode() + str(a.shape).encode())
        if a.nbytes <= (1 << 20):
            h.update(np.ascontiguousarray(a).tobytes())
        else:
            flat = a.reshape(-1)
            step = max(1, flat.size // 4096)
            h.update(np.ascontiguousarray(flat[::step]).tobytes())
            h.update(np.ascontiguousarray(flat[-1:]).tobytes())
    return h.hexdigest()


def _input_code(pats):
    """The EBSD_* input type find_bands hands the library for ``pats`` (numpy or torch)."""
    name = str(getattr(pats, "dtype", "")).replace("torch.", "")
    return {"uint8": _lib.EBSD_U8, "uint16": _lib.EBSD_U16}.get(name, _lib.EBSD_F32)


def _large_inputs(*arrays):
    """The plan inputs above 1 MiB, as objects (compared by identity)."""
    return tuple(a for a in arrays if a is not None and np.asarray(a).nbytes > (1 << 20))


class GPUFindBands:
    """``find_bands`` on the GPU, reading the plan attributes the reference defines."""

    default_method = "fused"
    gpu_id = 0

    def _device_plan(self, gpu_id=None):
        dev = self.gpu_id if gpu_id is None else int(gpu_id)
        rp = self.radonPlan
        bg = self.backgroundsub
        inputs = (rp.indexPlan, self.kernel, self.rdnmask, rp.theta, rp.rho, bg)
        key = (dev, tuple(np.asarray(self.patDim).tolist()), int(rp.nTheta), int(rp.nRho), int(self.nBands),
               tuple(np.asarray(self.padding).tolist()), tuple(np.asarray(self.peakPad).tolist()),
               _digest(*inputs))
        large = _large_inputs(*inputs)
        cache = getattr(self, "_gpu_plan_cache", None)
        if (cache is not None and cache[0] == key and len(cache[2]) == len(large)
                and all(x is y for x, y in zip(cache[2], large))):
            return cache[1]
        bgarr = None
        if bg is not None:
            bgarr = np.asarray(bg)
            if bgarr.dtype != np.float32:
                bgarr = bgarr.astype(np.float64)
        plan = _lib.DevicePlan(
            H=int(rp.imDim[0]), W=int(rp.imDim[1]), nTheta=int(rp.nTheta), nRho=int(rp.nRho),
            nBands=int(self.nBands), padding=np.asarray(self.padding), peakPad=np.asarray(self.peakPad),
            kernel=np.asarray(self.kernel, dtype=np.float32).reshape(np.asarray(self.kernel).shape[-2:]),
            lut=rp.indexPlan, rdnmask=np.asarray(self.rdnmask).astype(np.uint8), theta=rp.theta,
            rho=rp.rho, background=bgarr, device=dev)
        self._gpu_plan_cache = (key, plan, large)
        return plan

    def _pick_method(self, plan, method, dtype=None):
        """The method a call runs: the requested (or default) one, the per-stage FP32 method
        where a fused kernel cannot take the plan (or the input type, ``dtype`` an EBSD_* code).

        FP16 storage on a plan that runs in theta slabs needs room for its theta-max rows beside
        the 16-bit tile, which the widest slabs may not leave (240x240: 10 slabs instead of 9):
        the slab tables are then re-laid to the widest slabs that take it, and FP32 calls run
        those slabs too until ``set_tile`` changes them (CUDA graphs captured before a re-layout
        are captured again: the old tables are freed)."""
        m = self.default_method if method is None else method
        if m == "fused16" and dtype in (None, _lib.EBSD_U8, _lib.EBSD_U16) and not plan.supported(m, dtype):
            info = plan.get_tile()
            if info["slabs"] and not info["single_fits"] and not info["slabs_fp16"]:
                for ns in range(info["slabs"] + 1, info["slabs_max"] + 1):
                    plan.set_tile(0, ns)
                    if plan.supported(m, dtype):
                        break
                else:
                    plan.set_tile(0, info["slabs"])
        if m in ("fused", "fused32", "fused16") and not plan.supported(m, dtype):
            m = "plain"
        return m

    def find_bands(self, patternsIn, verbose=0, chunksize=528, clparams=None, gpu_id=None, useCPU=None,
                   method=None, **kwargs):
        """BandDetect.find_bands (band_detect.py:411-526) on the GPU.

        patternsIn: [n, H, W] or [H, W] array (numpy, or a torch tensor on the plan's device) of
        uint8, uint16 or float32 (other numeric types are converted to float32 first).
        ``chunksize`` is the number of patterns per device chunk for the per-stage method (the
        fused method streams at its own chunk size); ``clparams``/``useCPU`` are accepted for
        interface compatibility and ignored.  ``method``: "fused" (default), "fused16",
        "plain" or "plain64".  Returns the (nPats, nBands) record array of ``self.dataType``.
        """
        tic0 = timer()
        is_torch = type(patternsIn).__module__.startswith("torch")
        pats = patternsIn
        if pats.ndim == 2:
            pats = pats[None]
        nP = int(pats.shape[0])
        if self.patDim is None or tuple(np.asarray(self.patDim)[-2:]) != tuple(pats.shape[-2:]):
            self.band_detect_setup(patDim=pats.shape[-2:])
        plan = self._device_plan(gpu_id)
        m = self._pick_method(plan, method, _input_code(pats))
        chunk = int(chunksize) if (chunksize is not None and chunksize > 0) else 0
        if m.startswith("fused"):
            chunk = 0
        soa = None
        if is_torch:
            dev_out = self._find_bands_dev(plan, pats, m, chunk)
            soa = {k: v.cpu().numpy() for k, v in dev_out.items()}
        else:
            arr = np.asarray(pats)
            if arr.dtype not in (np.uint8, np.uint16, np.float32):
                arr = arr.astype(np.float32)
            bandData = plan.find_bands_host_records(arr, m, self.dataType, chunk=chunk)
        if soa is not None:
            bandData = self._records(soa, nP)
        if verbose > 0:
            print('Band Find Time (GPU, %s):' % m, timer() - tic0)
        return bandData

    def _find_bands_dev(self, plan, t, m, chunk):
        """Device band fields (SoA torch tensors) for CUDA patterns ``t`` [n, H, W]."""
        import torch
        u16 = getattr(torch, "uint16", None)
        if t.dtype == torch.uint8:
            dt = _lib.EBSD_U8
        elif u16 is not None and t.dtype == u16:
            dt = _lib.EBSD_U16
        else:
            t = t.to(torch.float32)
            dt = _lib.EBSD_F32
        t = t.contiguous()
        nP, nB = int(t.shape[0]), int(self.nBands)
        dev_out = {f: torch.empty((nP, nB, 2) if f in ("maxloc", "aveloc") else (nP, nB),
                                  dtype=torch.int8 if f == "valid" else torch.float32, device=t.device)
                   for f in _lib.BAND_FIELDS}
        stream = torch.cuda.current_stream(t.device).cuda_stream
        plan.find_bands_device(t.data_ptr(), dt, nP, {k: v.data_ptr() for k, v in dev_out.items()}, m,
                               chunk=chunk, stream=stream)
        return dev_out

    def find_bands_file(self, path, patStart=0, nPat=-1, method=None, chunk=0, gpu_id=None):
        """find_bands on patterns [patStart, patStart + nPat) of an EDAX UP1 / UP2, Oxford .ebsp
        or ThermoFisher .pat file (nPat -1: to the end; clamped to the file as read_data does,
        ebsd_pattern.py:253-262), streamed by ebsd_find_bands_file: a reader thread fills pinned
        chunk buffers while two CUDA streams copy and detect, so the file read overlaps the GPU
        work.  The plan is set
        up for the file's pattern size if it is not already.  Returns the record array."""
        from .ebsd_pattern import get_pattern_file_obj
        f = get_pattern_file_obj(path)
        dim = (int(f.patternH), int(f.patternW))
        if self.patDim is None or tuple(np.asarray(self.patDim)[-2:]) != dim:
            self.band_detect_setup(patDim=dim)
        start = int(patStart)
        n = int(f.nPatterns) - start if int(nPat) == -1 else max(int(nPat), 1)
        n = min(n, int(f.nPatterns) - start)
        if start < 0 or n < 0:
            raise ValueError("patStart outside the file")
        plan = self._device_plan(gpu_id)
        m = self._pick_method(plan, method)
        return plan.find_bands_file_records(str(f.filepath), start, n, m, self.dataType, chunk=chunk)

    def find_bands_normals(self, patterns, PC=None, vendor='EDAX', method=None, gpu_id=None):
        """find_bands followed by Radon.radon2pole (radon_fast.py:314-397) with the band
        normals computed on the device from the device theta/rho fields -- no host round trip
        between detection and normals.  ``patterns``: [n, H, W] or [H, W], numpy or CUDA torch.
        Returns (records, normals [n, nBands, 3] float32 numpy)."""
        import torch
        from .radon_fast import radon2pole_gpu
        pats = patterns if type(patterns).__module__.startswith("torch") else torch.from_numpy(np.ascontiguousarray(patterns))
        if pats.ndim == 2:
            pats = pats[None]
        if self.patDim is None or tuple(np.asarray(self.patDim)[-2:]) != tuple(pats.shape[-2:]):
            self.band_detect_setup(patDim=pats.shape[-2:])
        plan = self._device_plan(gpu_id)
        m = self._pick_method(plan, method, _input_code(pats))
        pats = pats.to(torch.device("cuda", plan.device))
        dev_out = self._find_bands_dev(plan, pats, m, 0)
        normals = radon2pole_gpu(dev_out["theta"], dev_out["rho"], self.radonPlan.imDim, PC=PC, vendor=vendor)
        soa = {k: v.cpu().numpy() for k, v in dev_out.items()}
        return self._records(soa, int(pats.shape[0])), normals.cpu().numpy()

    def autotune(self, sample, method=None, gpu_id=None, cache=None):
        """Time the record-identical variants of the fused kernel on ``sample`` ([n, H, W]
        numpy or torch, uint8/uint16/float32) and keep the fastest in the device plan for later
        ``find_bands`` calls.  The variants are Radon tile shapes: the whole padded Radon image
        as one tile with one, two, four or eight patterns per block pass, and theta slabs of
        several widths (``DevicePlan.get_tile`` reads the choice back; it is also kept in
        ``self.tuned``).  No counterpart in the reference.  Returns the chosen patterns per
        pass (1 for slabs).

        ``cache``: None (default) times every call; a JSON file name, or True for
        ``tuning.default_path()``, keeps the decision per GPU, library version, plan geometry,
        input type and method (``tuning.TuningCache``): a call whose key is stored applies the
        stored choice without timing, a new key is timed and stored."""
        import torch
        plan = self._device_plan(gpu_id)
        dev = torch.device("cuda", plan.device)
        t = sample if type(sample).__module__.startswith("torch") else torch.from_numpy(np.ascontiguousarray(sample))
        if t.ndim == 2:
            t = t[None]
        u16 = getattr(torch, "uint16", None)
        if t.dtype == torch.uint8:
            dt = _lib.EBSD_U8
        elif u16 is not None and t.dtype == u16:
            dt = _lib.EBSD_U16
        else:
            t = t.to(torch.float32)
            dt = _lib.EBSD_F32
        m = self._pick_method(plan, method, dt)
        store = key = None
        if cache is not None and cache is not False:
            from . import tuning
            store = tuning.TuningCache(cache)
            key = self._tuning_key(plan, m, dt)
            hit = store.get(key)
            if hit is not None and int(hit.get("patterns_per_pass", 0)) in (1, 2, 4, 8):
                ppp = int(hit["patterns_per_pass"])
                tile, slabs = int(hit.get("tile", 0)), int(hit.get("slabs", 0))
                try:
                    if tile in (1, 2):
                        plan.set_tile(tile, slabs if tile == 2 else 0)
                    plan.set_patterns_per_pass(ppp)
                except RuntimeError:
                    hit = None  # a shape this plan cannot take: tune afresh
                if hit is not None:
                    self.tuned = dict(plan.get_tile(), patterns_per_pass=ppp, cached=True)
                    return ppp
        t = t.to(dev).contiguous()
        stream = torch.cuda.current_stream(dev).cuda_stream
        ppp = plan.autotune(t.data_ptr(), dt, int(t.shape[0]), m, stream=stream)
        info = plan.get_tile()
        self.tuned = dict(info, patterns_per_pass=int(ppp), cached=False)
        if store is not None:
            store.put(key, {"patterns_per_pass": int(ppp), "tile": info["tile"],
                            "slabs": info["slabs"] if info["tile"] == 2 else 0,
                            "timed_patterns": int(t.shape[0])})
        return ppp

    def _tuning_key(self, plan, method, dtype):
        """The tuning-cache key of this plan on its GPU (tuning.plan_key)."""
        import torch
        from . import tuning
        props = torch.cuda.get_device_properties(plan.device)
        lut = self.radonPlan.indexPlan
        if getattr(self, "_tuning_lut", (None, None))[0] is not lut:
            self._tuning_lut = (lut, tuning.lut_digest(lut))
        return tuning.plan_key(gpu=props.name, sms=props.multi_processor_count, library=_lib.version(),
                               shape=np.asarray(self.patDim)[-2:], dtype=dtype, method=method,
                               nTheta=self.nTheta, nRho=self.nRho, nBands=self.nBands,
                               kernel_shape=np.shape(self.kernel)[-2:], padding=np.asarray(self.padding),
                               peakPad=np.asarray(self.peakPad), lut=self._tuning_lut[1],
                               background=self.backgroundsub is not None)

    def _records(self, soa, nP):
        out = np.zeros((nP, int(self.nBands)), dtype=self.dataType)
        for f in _lib.BAND_FIELDS:
            out[f] = soa[f]
        return out


class BandDetect(GPUFindBands):
    """Band-detection plan with the reference BandDetect's interface (band_detect.py:67-136)."""

    def __init__(self, patterns=None, patDim=None, nTheta=180, nRho=90, tSigma=None, rSigma=None,
                 rhoMaskFrac=0.1, nBands=9, nPhases=10, **kwargs):
        self.patDim = None
        self.nTheta = nTheta
        self.nRho = nRho
        self.dTheta = None
        self.dRho = None
        self.rhoMax = None
        self.radonPlan = Radon()
        self.rdnNorm = None
        self.tSigma = tSigma
        self.rSigma = rSigma
        self.kernel = None
        self.peakPad = np.array([11, 11])
        self.padding = np.array([11, 11])
        self.rhoMaskFrac = rhoMaskFrac
        self.rhomask1thresh = None
        self.rhomask1 = None
        self.nBands = nBands
        self.nPhases = 10 if nPhases is None else nPhases
        self.EDAXIQ = False
        self.backgroundsub = None
        self.useCPU = False
        self.gpu_id = int(kwargs.get("gpu_id", 0) or 0)
        if "method" in kwargs and kwargs["method"] is not None:
            self.default_method = kwargs["method"]
        self.dataType = record_dtype(self.nPhases)
        if patterns is not None or patDim is not None:
            self.patDim = np.asarray(patterns.shape[-2:] if patterns is not None else patDim)
            if 'patternmask' in kwargs:
                self.radonPlan.mask = kwargs.get('patternmask')
            if 'patternmaskindex' in kwargs:
                self.radonPlan.maskindex = kwargs.get('patternmaskindex')
            self.band_detect_setup(patterns, self.patDim, self.nTheta, self.nRho, self.tSigma, self.rSigma,
                                   self.rhoMaskFrac, self.nBands, patternmask=self.radonPlan.mask,
                                   patternmaskindex=self.radonPlan.maskindex)

    def band_detect_setup(self, patterns=None, patDim=None, nTheta=None, nRho=None, tSigma=None, rSigma=None,
                          rhoMaskFrac=None, nBands=None, patternmask=None, patternmaskindex=None, **kwargs):
        """Plan setup (band_detect.py:138-294): rhoMax/dRho, Radon LUT, Radon-space mask,
        LoG kernel and peak/padding windows."""
        newdim = None
        redo_radon = False
        redo_masks = False
        if patterns is None and patDim is not None:
            newdim = np.asarray(patDim, dtype=np.int64)
        if patterns is not None:
            newdim = np.asarray(np.shape(patterns)[-2:])
        if newdim is not None:
            if self.patDim is None or np.sum(np.abs(np.asarray(self.patDim)[-2:] - newdim[-2:])) != 0:
                redo_radon = True
                self.patDim = newdim
        if nTheta is not None:
            self.nTheta = nTheta
            redo_radon = redo_masks = True
        if self.nTheta is not None:
            self.dTheta = 180.0 / self.nTheta
        if nRho is not None:
            self.nRho = nRho
            redo_radon = redo_masks = True
        if self.dRho is None:
            redo_radon = True
        if patternmask is not None:
            self.radonPlan.mask = patternmask
            redo_radon = True
        if patternmaskindex is not None:
            self.radonPlan.maskindex = patternmaskindex
            redo_radon = True

        if redo_radon:
            dim = np.asarray(self.patDim)
            if 0 < self.rhoMaskFrac < 1:
                self.rhoMax = 0.5 * np.float32(dim.min())
            else:
                self.rhoMax = 0.5 * np.float32(np.sqrt(np.float32(dim[-2]) ** 2 + np.float32(dim[-1]) ** 2))
            self.rhomask1thresh = np.float32(dim.min()) * 0.1
            self.dRho = self.rhoMax / np.float32(self.nRho)
            self.radonPlan.radon_plan_setup(imageDim=dim, nTheta=self.nTheta, nRho=self.nRho, rhoMax=self.rhoMax,
                                            mask=patternmask, maskindex=patternmaskindex)
            # Radon of the mask image without normalisation = in-mask pixel count per ray
            # (band_detect.py:203-215); its positive cells are the searchable Radon cells.
            cnt = self.radonPlan.ray_counts()
            self.rhomask1 = (cnt >= self.rhomask1thresh).astype(np.ubyte)
            rmask = cnt > 0
            if self.rhoMaskFrac >= (1 - 1.0e-12):
                rmask = ndi.binary_erosion(rmask, structure=np.ones((3, 1)), iterations=int(self.rhoMaskFrac))
            else:
                limit = rmask.copy()
                if self.rhoMaskFrac > 0:
                    edge = max(int(self.nRho * self.rhoMaskFrac), 1)
                    limit[0:edge, :] = 0
                    limit[-edge:, :] = 0
                elif self.rhoMaskFrac < 0:
                    # rays that touch the circle of radius rhoMax*(1+rhoMaskFrac) (band_detect.py:232-238)
                    ny, nx = int(dim[-2]), int(dim[-1])
                    rad = np.sqrt(((np.arange(nx) - nx * 0.5) ** 2).reshape(1, nx)
                                  + ((np.arange(ny) - ny * 0.5) ** 2).reshape(ny, 1))
                    inside = np.concatenate(((rad < self.rhoMax * (1.0 + self.rhoMaskFrac)).ravel(), [False, False]))
                    lut = np.minimum(self.radonPlan.indexPlan, nx * ny)
                    limit = np.any(inside[lut], axis=-1) & (cnt > 0)
                rmask = rmask & (limit > 0)
            self.rdnmask = rmask > 0

        if tSigma is not None:
            self.tSigma = tSigma
            redo_masks = True
        if rSigma is not None:
            self.rSigma = rSigma
            redo_masks = True
        if rhoMaskFrac is not None:
            self.rhoMaskFrac = rhoMaskFrac
        if self.rhoMaskFrac is not None:
            redo_masks = True
        if self.tSigma is None and self.dTheta is not None:
            self.tSigma = 1.0 / self.dTheta
            redo_masks = True
        if self.rSigma is None and self.dRho is not None:
            self.rSigma = 0.5 / np.float32(self.dRho)
            redo_masks = True
        if redo_masks:
            # LoG: -d2/drho2 of a Gaussian, smoothed along theta, normalised to max 1
            ksz = np.array([max(np.int64(4 * self.rSigma), 5), max(np.int64(4 * self.tSigma), 5)])
            ksz = ksz + ((ksz % 2) == 0)
            delta = np.zeros(ksz, dtype=np.float32)
            delta[int(ksz[0] / 2), int(ksz[1] / 2)] = 1
            k = -1.0 * ndi.gaussian_filter(delta, [self.rSigma, self.tSigma], order=[2, 0])
            k *= 1.0 / np.max(k)
            self.kernel = k.reshape((1, ksz[0], ksz[1]))
            self.peakPad = np.array(np.around([2 * ksz[0], 2 * ksz[1]]), dtype=np.int64)
            self.peakPad += 1 - np.mod(self.peakPad, 2)
        self.padding = np.array([max(self.peakPad[0], self.padding[0]), max(self.peakPad[1], self.padding[1])])
        if nBands is not None:
            self.nBands = nBands

    def collect_background(self, fileobj=None, patsIn=None, nsample=None, method='randomStride', sigma=None):
        """The static background subtracted before the Radon (band_detect.py:297-348): the mean
        of a sample of the patterns, smoothed by ``backsub_fit`` into a 2-D Gaussian on a tilted
        plane.  The sample is every pattern when ``nsample`` covers them, else ``nsample`` drawn
        at random without replacement ('randomStride') or every int(n / nsample)-th
        ('evenStride').  Patterns come from ``patsIn`` ([n, H, W] or one [H, W]) or, failing
        that, from a pattern file read in runs of consecutive patterns."""
        mean = None
        if patsIn is not None:
            stack = patsIn if patsIn.ndim == 3 else patsIn[np.newaxis]
            n = stack.shape[0]
            want = n if nsample is None else nsample
            pick = None if n <= want else _sample_picks(n, want, method)
            if n <= want:
                mean = np.mean(stack, axis=0)
            elif pick is not None:
                mean = np.mean(stack[pick], axis=0)
        if mean is None and fileobj is not None:
            mean = _file_sample_mean(fileobj, nsample, method)
        self.backgroundsub = None if mean is None else self.backsub_fit(np.squeeze(mean))

    def backsub_fit(self, back, mask=None):
        """Smooth background model of a mean pattern (band_detect.py:350-408): a 2-D Gaussian on a
        tilted plane fitted by least squares (scipy's curve_fit, started from a tenth of the
        median-filtered range at the brightest pixel with widths of a sixth of the pattern) to
        the 3x3 median-filtered pattern inside ``mask`` (default: the disc of radius 0.49 * H
        about the centre), evaluated on the whole pattern, its mean removed.  If the fit does
        not converge, the mean pattern itself, mean removed."""
        ny, nx = back.shape[-2], back.shape[-1]
        yy, xx = np.indices((ny, nx), dtype=float)
        if mask is None:
            mask = np.sqrt((xx - nx * 0.5) ** 2 + (yy - ny * 0.5) ** 2) < (ny * 0.49)
        inside = np.asarray(mask).ravel() != 0
        smooth = ndi.median_filter(np.squeeze(back), 3).ravel()[inside]
        brightest = np.unravel_index(back.argmax(), back.shape)
        start = [(smooth.max() - smooth.min()) * 0.1, brightest[1], brightest[0], nx / 2.355, ny / 2.355,
                 smooth.min(), 0, 0]
        fitted = _fit_gaussian_plane(xx.ravel(), yy.ravel(), inside, smooth, start)
        model = back if fitted is None else fitted.reshape(ny, nx)
        if fitted is None:
            print('Warning: no convergence on background gaussian fit ... using mean of the patterns.')
        return model - np.mean(model)

    def _circmask(self, im):
        nx, ny = im.shape[-1], im.shape[-2]
        cx = (np.arange(nx) - nx * 0.5) ** 2
        cy = (np.arange(ny) - ny * 0.5) ** 2
        return np.sqrt(np.broadcast_to(cx.reshape(1, nx), (ny, nx)) + np.broadcast_to(cy, (nx, ny)).T)


def _device_input(t, dev):
    """(contiguous CUDA tensor on ``dev``, EBSD_* input code) for a pattern batch: uint8 and
    uint16 as they are, anything else as float32."""
    import torch
    u16 = getattr(torch, "uint16", None)
    if t.dtype == torch.uint8:
        dt = _lib.EBSD_U8
    elif u16 is not None and t.dtype == u16:
        dt = _lib.EBSD_U16
    else:
        t = t.to(torch.float32)
        dt = _lib.EBSD_F32
    return t.to(dev).contiguous(), dt


def _sample_picks(n, want, method):
    """Indices of the background sample: ``want`` of ``n`` at random without replacement,
    sorted ('randomStride'), or every int(n / want)-th ('evenStride'); None for another
    method."""
    kind = method.upper()
    if kind == 'RANDOMSTRIDE':
        return np.sort(np.random.choice(n, size=want, replace=False))
    if kind == 'EVENSTRIDE':
        return np.arange(0, n, int(n / want))
    return None


def _file_sample_mean(fileobj, nsample, method):
    """Mean of the background sample of a pattern file: the sampled patterns read as float32
    in runs of consecutive indices and summed one by one in index order."""
    if fileobj.version is None:
        fileobj.read_header()
    n = int(fileobj.nPatterns)
    want = n if (nsample is None or n <= nsample) else nsample
    pick = _sample_picks(n, want, method)
    if pick is None:
        return None
    pick = np.asarray(pick, dtype=np.int64)
    breaks = np.nonzero(np.diff(pick) != 1)[0] + 1
    total = None
    for run in np.split(pick, breaks):
        block = fileobj.read_data(convertToFloat=True, patStartCount=[int(run[0]), len(run)],
                                  returnArrayOnly=True)[0]
        for pat in block:
            total = pat.copy() if total is None else total + pat
    return total / float(len(pick))


def _gaussian_plane(x, y, amp, x0, y0, sx, sy, c, d, e):
    """amp * exp(-(x - x0)^2 / (2 sx^2) - (y - y0)^2 / (2 sy^2)) + c + d x + e y."""
    return amp * np.exp(- ((x - x0) ** 2) / (2.0 * sx ** 2) - ((y - y0) ** 2) / (2.0 * sy ** 2)) + c + d * x + e * y


def _fit_gaussian_plane(x, y, inside, z, start):
    """Least-squares fit of ``_gaussian_plane`` to z at the pixels ``inside``; the fitted
    surface on every pixel, or None when curve_fit does not converge."""
    try:
        params, _ = opt.curve_fit(lambda xy, *p: _gaussian_plane(xy[0], xy[1], *p),
                                  np.vstack((x[inside], y[inside])), z, start)
    except RuntimeError:
        return None
    return _gaussian_plane(x, y, *params)


class MixedBandDetect:
    """Band detection over a batch of patterns of different sizes.

    The reference handles one pattern size per ``BandDetect`` plan (band_detect.py:138-155
    rebuilds the plan when the size changes).  Here one plan is kept per size, and a batch
    holding several sizes runs as ONE persistent fused launch over all of them
    (``ebsd_find_bands_mixed``: every CTA strides over the patterns of every size, each
    detected in theta slabs with its size's tables), up to eight sizes of one input type.
    Other methods, or more sizes, run size by size, each on its own CUDA stream.  ``nRho`` for
    a size comes from ``nRho_for(H, W)`` (default 1.5 * min(H, W)).  uint16 patterns need a
    torch build with ``torch.uint16``; otherwise pass float32.
    """

    MAX_MIXED = 8

    def __init__(self, nTheta=180, nRho_for=None, tSigma=1.0, rSigma=1.0, rhoMaskFrac=0.1, nBands=10,
                 mask_for=None, method="fused", gpu_id=0, **kwargs):
        self.nTheta, self.tSigma, self.rSigma = nTheta, tSigma, rSigma
        self.rhoMaskFrac, self.nBands, self.method, self.gpu_id = rhoMaskFrac, nBands, method, gpu_id
        self.nRho_for = nRho_for or (lambda h, w: int(round(1.5 * min(h, w))))
        self.mask_for = mask_for
        self.kwargs = kwargs
        self.plans = {}
        self.last_mixed = False  # whether the last call ran as one mixed-size launch

    def plan(self, h, w):
        key = (int(h), int(w))
        if key not in self.plans:
            bd = BandDetect(nTheta=self.nTheta, nRho=self.nRho_for(h, w), tSigma=self.tSigma, rSigma=self.rSigma,
                            rhoMaskFrac=self.rhoMaskFrac, nBands=self.nBands, gpu_id=self.gpu_id, **self.kwargs)
            bd.band_detect_setup(patDim=key, patternmask=None if self.mask_for is None else self.mask_for(h, w))
            self.plans[key] = bd
        return self.plans[key]

    def method_for(self, h, w, dtype=None):
        """The method a size runs (for input of ``dtype``, an EBSD_* code, if given)."""
        bd = self.plan(h, w)
        m = self.method
        return m if not m.startswith("fused") or bd._device_plan().supported(m, dtype) else "plain"

    def find_bands(self, patterns, method=None):
        """patterns: sequence of [H, W] arrays (numpy, or CUDA tensors), sizes mixed.  Returns an
        (n, nBands) record array in input order."""
        import torch
        groups = {}
        for k, p in enumerate(patterns):
            groups.setdefault(tuple(p.shape[-2:]), []).append(k)
        batches = {}
        for key, idx in groups.items():
            first = patterns[idx[0]]
            if type(first).__module__.startswith("torch"):
                batches[key] = torch.stack([patterns[k] for k in idx])
            else:
                batches[key] = np.stack([np.asarray(patterns[k]) for k in idx])
        recs = self.find_bands_grouped(batches, method=method)
        out = np.zeros((len(patterns), self.nBands), dtype=record_dtype(10))
        for key, idx in groups.items():
            out[np.asarray(idx)] = recs[key]
        return out

    def find_bands_device(self, batches, method=None, stream=None, out=None):
        """batches: {(H, W): CUDA tensor [n, H, W]} (one input type) -> {(H, W): dict of device
        band arrays}, asynchronous on ``stream`` (default: the current stream).  With the fused
        method and at most eight sizes that the slab kernel takes, one launch serves them all.
        ``out``: the dict a previous call returned, written again instead of new arrays (the
        same sizes and counts) -- with it the call allocates nothing and can be captured in a
        CUDA graph (after a first call has set the kernels up)."""
        import torch
        dev = torch.device("cuda", self.gpu_id)
        st = stream if stream is not None else torch.cuda.current_stream(dev)
        m = method or self.method
        ins, dts = {}, set()
        for key, t in batches.items():
            ins[key] = _device_input(t, dev)
            dts.add(ins[key][1])
        if out is not None:
            if set(out) != set(ins) or any(out[k]["valid"].shape[0] != ins[k][0].shape[0] for k in ins):
                raise ValueError("out must be a previous result for the same sizes and counts")
            outs = out
        else:
            outs = {key: self._device_outputs(t.shape[0], dev) for key, (t, _) in ins.items()}
        plans = {key: self.plan(*key)._device_plan() for key in ins}
        dt0 = next(iter(dts)) if len(dts) == 1 else None
        mixed = (m in ("fused", "fused32") and dt0 is not None and 1 <= len(ins) <= self.MAX_MIXED
                 and all(p.supported("fused", dt0) for p in plans.values()))
        self.last_mixed = False
        if mixed:
            keys = list(ins)
            try:
                _lib.DevicePlan.find_bands_mixed([plans[k] for k in keys], dt0, [ins[k][0].data_ptr() for k in keys],
                                                 [ins[k][0].shape[0] for k in keys],
                                                 [{f: v.data_ptr() for f, v in outs[k].items()} for k in keys],
                                                 stream=st.cuda_stream)
                self.last_mixed = True
                return outs
            except RuntimeError as e:
                if "not supported" not in str(e):
                    raise
        for key, (t, dt) in ins.items():
            mk = m if not m.startswith("fused") or plans[key].supported(m, dt) else "plain"
            plans[key].find_bands_device(t.data_ptr(), dt, t.shape[0], {f: v.data_ptr() for f, v in outs[key].items()},
                                         mk, stream=st.cuda_stream)
        return outs

    def _device_outputs(self, n, dev):
        import torch
        return {f: torch.empty((n, self.nBands, 2) if f in ("maxloc", "aveloc") else (n, self.nBands),
                               dtype=torch.int8 if f == "valid" else torch.float32, device=dev)
                for f in _lib.BAND_FIELDS}

    def autotune(self, batches, stream=None, max_extra=3):
        """Choose each size's theta-slab width for the one-launch mixed path.  For every size in
        ``batches`` ({(H, W): CUDA tensor [n, H, W]}, a sample of each), the slab counts from
        the widest slabs that fit to ``max_extra`` narrower ones are timed on that size alone
        (the slab kernel, CUDA events on ``stream``, best of two runs after a warm-up), and the
        fastest count's tables are kept in the size's plan (``ebsd_plan_set_tile``); calls of
        one size keep the rule (one tile when it fits).  Records do not depend on the choice.
        No counterpart in the reference.  Returns {(H, W): {"slabs": count, "ms": {count: ms}}}."""
        import torch
        dev = torch.device("cuda", self.gpu_id)
        st = stream if stream is not None else torch.cuda.current_stream(dev)
        chosen = {}
        for key, t in batches.items():
            t, dt = _device_input(t, dev)
            plan = self.plan(*key)._device_plan()
            info = plan.get_tile()
            if info["slabs"] == 0 or not plan.supported("fused", dt):
                continue
            outs = {f: v.data_ptr() for f, v in self._device_outputs(t.shape[0], dev).items()}
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            times = {}
            try:
                for ns in range(info["slabs_min"], min(info["slabs_max"], info["slabs_min"] + max_extra) + 1):
                    plan.set_tile(2, ns)
                    best = None
                    for rep in range(3):
                        e0.record(st)
                        plan.find_bands_device(t.data_ptr(), dt, t.shape[0], outs, "fused", stream=st.cuda_stream)
                        e1.record(st)
                        e1.synchronize()
                        if rep > 0:
                            ms = e0.elapsed_time(e1)
                            best = ms if best is None else min(best, ms)
                    times[ns] = best
            finally:
                pick = min(times, key=times.get) if times else 0
                plan.set_tile(0, pick)
            chosen[key] = {"slabs": pick, "ms": times}
        return chosen

    def find_bands_grouped(self, batches, method=None):
        """batches: {(H, W): [n, H, W] array (numpy or CUDA tensor)} -> {(H, W): record array}."""
        import torch
        tb = {k: (v if type(v).__module__.startswith("torch") else torch.from_numpy(np.ascontiguousarray(v)))
              for k, v in batches.items()}
        outs = self.find_bands_device(tb, method=method)
        torch.cuda.synchronize(torch.device("cuda", self.gpu_id))
        res = {}
        for key, o in outs.items():
            rec = np.zeros((o["valid"].shape[0], self.nBands), dtype=record_dtype(10))
            for f in _lib.BAND_FIELDS:
                rec[f] = o[f].cpu().numpy()
            res[key] = rec
        return res
