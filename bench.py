"""Band-detection throughput benchmark (one JSON line on stdout).

Workload (the batched configuration): 1,000,000 synthetic 80x80 uint8 EBSD patterns, Radon
nTheta=180 x nRho=120, LoG sigma 1.0 px, rhoMaskFrac 0.1, nBands=9, circular detector mask;
10% of the patterns carry no bands (background + Poisson noise only).  A step is one
find_bands pass over the whole batch.  The patterns are a pool of 65,536 seeded distinct
patterns (pattern i uses seed BASE+i; generated by a process pool before the GPU is touched)
tiled to the batch size; the 6.4 GB input is larger than L2, so no L2 flush is needed
between steps.

The line carries the accuracy of the timed method's records: against the FP64 per-stage
method (plain64, the FP64 GPU oracle) on 32,768 patterns of the timed batch, and -- in the
CPU-baseline leg -- against the oracle's FFT restatement of the reference's find_bands on
2,048 of them.

  python bench.py [--gpus N --steps K --warmup W] [--method fused16|fused|plain|plain64]
  python bench.py --impl reference     # the CPU restatement of the reference on the host cores

Under torchrun (N > 1) every rank runs its own replica of the batch (weak scaling, no
collective in the data path); value = patterns processed by all ranks / max rank time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "band-detect patterns/sec on 1 GB300: batched FP16 vs plain FP32, at <=1e-3 px error"
H = W = 80
NRHO, NTHETA, NBANDS = 120, 180, 9
BYTES_PER_PATTERN = H * W * 1 + 41 * NBANDS   # algorithmic bytes: pattern in, band fields out
# DRAM bytes (read + write) per pattern of the fused kernel at eight patterns per pass, from an
# ncu capture of the same launch configuration on 40,000 patterns (dram__bytes_read.sum +
# dram__bytes_write.sum = 0.648 GB + 2.273 GB); the traffic grows with the patterns, so a
# launch's traffic is this times its patterns.  Most of it is the write-back of the parked
# ray means (seven rows per CTA per eight patterns), not input re-reads.
DRAM_BYTES_PER_PATTERN = (648_438_528 + 2_272_787_200) / 40_000
# warp instructions per pattern of the same kernel (ncu smsp__inst_executed.sum, same capture):
# the issue roofline of an issue-bound kernel is 4 warp-instructions per SM per clock
WARP_INST_PER_PATTERN = 6.546e9 / 40_000
ACCURACY_PATTERNS = 32_768      # timed-batch patterns graded against plain64 (FP64 GPU oracle)
ORACLE_PATTERNS = 2_048         # of those, graded against the oracle's FFT path (CPU leg)
SEED = 1_000_000
WORKLOAD = ("find_bands on 1,000,000 80x80 uint8 patterns, nTheta 180, nRho 120, nBands 9, LoG sigma 1, "
            "rhoMaskFrac 0.1, circular mask, 10% noise-only")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--method", default=None)
    ap.add_argument("--patterns", type=int, default=1_000_000)
    ap.add_argument("--pool", type=int, default=65_536)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-sample", type=int, default=0, help="patterns in the timed CPU sample")
    ap.add_argument("--no-variants", action="store_true", help="skip timing the other methods")
    ap.add_argument("--no-graph", action="store_true", help="launch directly instead of replaying a CUDA graph")
    ap.add_argument("--no-autotune", action="store_true", help="keep the plan's rule-based kernel variant")
    ap.add_argument("--no-index", action="store_true", help="skip timing the device indexing after detection")
    ap.add_argument("--no-file", action="store_true", help="skip timing detection streamed from a UP1 file")
    ap.add_argument("--file-patterns", type=int, default=262_144, help="patterns in the file timed")
    ap.add_argument("--file-format", default="up1", choices=["up1", "ebsp", "pat"],
                    help="format of the file timed (EDAX UP1, Oxford .ebsp, ThermoFisher .pat)")
    ap.add_argument("--nlpar-file", action="store_true",
                    help="also time NLPAR's file interface (opt_lambda, calcnlpar) on a 400x500 UP1 scan")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-size (60/120/240 uint16) figure")
    ap.add_argument("--mixed-patterns", type=int, default=300_000, help="patterns of the mixed-size step")
    ap.add_argument("--no-nlpar", action="store_true", help="skip the NLPAR -> detection figure")
    ap.add_argument("--no-diff", action="store_true", help="skip the differentiable-path figure")
    ap.add_argument("--lambda-scan", action="store_true",
                    help="also time NLPAR's lambda optimisation on a 400x500 scan of 80x80 patterns")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_plan():
    import pyebsdindex_gb300 as pg
    from pyebsdindex_gb300 import synthetic as syn
    bd = pg.BandDetect(nTheta=NTHETA, nRho=NRHO, tSigma=1.0, rSigma=1.0, rhoMaskFrac=0.1, nBands=NBANDS)
    bd.band_detect_setup(patDim=(H, W), patternmask=syn.circular_mask(H, W))
    return bd


def _pool_part(args):
    start, count = args
    from pyebsdindex_gb300 import synthetic as syn
    return syn.make_patterns(count, H, W, seed=SEED, start=start, noise_frac=0.1)[0]


def host_executor():
    """A spawn process pool over the host cores (pattern generation, the oracle leg)."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor
    return ProcessPoolExecutor(max_workers=max(1, min(16, os.cpu_count() or 1)), mp_context=mp.get_context("spawn"))


def make_pool(n, ex=None):
    """Patterns 0..n-1 of the seeded pool (pattern i from seed SEED + i), in parallel parts."""
    parts = [(s, min(1024, n - s)) for s in range(0, n, 1024)]
    if ex is None or len(parts) == 1:
        return np.concatenate([_pool_part(a) for a in parts])
    return np.concatenate(list(ex.map(_pool_part, parts)))


def _oracle_part(pats):
    from oracle import band_oracle as bo
    from pyebsdindex_gb300 import synthetic as syn
    plan = bo.Plan((H, W), NTHETA, NRHO, 1.0, 1.0, 0.1, NBANDS, mask=syn.circular_mask(H, W))
    return bo.find_bands(plan, pats, conv="fft")


def oracle_accuracy(ex, pats, dev_fields):
    """CPU-baseline leg: the oracle's FFT restatement of the reference find_bands on ``pats``
    (the first patterns of the timed batch) -> agreement of the device records with it."""
    from pyebsdindex_gb300.accuracy import compare_records
    chunks = [pats[s:s + 256] for s in range(0, len(pats), 256)]
    ref = np.concatenate(list(ex.map(_oracle_part, chunks)))
    got = {k: v[:len(pats)].cpu().numpy() for k, v in dev_fields.items()}
    return compare_records(got, ref)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def start(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()

    def _run(self):
        while not self._stop.is_set():
            try:
                r = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                    "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if r.returncode == 0 and r.stdout.strip():
                    self.samples.append([x.strip() for x in r.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def stop(self):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 5 + i and s[5 + i].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def cpu_baseline(pool, sample, impl_kind):
    """Time the CPU restatement of the reference find_bands on a bounded sample."""
    from oracle import cport
    try:
        cport.build()
        fn = cport.find_bands
        kind, cores = "port", os.cpu_count()
    except Exception:
        fn, kind, cores = None, None, 1
    plan = None
    from oracle import band_oracle as bo
    from pyebsdindex_gb300 import synthetic as syn
    plan = bo.Plan((H, W), NTHETA, NRHO, 1.0, 1.0, 0.1, NBANDS, mask=syn.circular_mask(H, W))
    pats = pool[:sample]
    if fn is not None:
        fn(plan, pats[: min(8, len(pats))], threads=cores)  # warm-up
        t0 = time.perf_counter()
        fn(plan, pats, threads=cores)
        dt = time.perf_counter() - t0
        desc = f"C/OpenMP restatement of find_bands, {len(pats)} patterns of the bench pool, {cores} threads"
    else:
        bo.find_bands(plan, pats[:4])
        t0 = time.perf_counter()
        bo.find_bands(plan, pats)
        dt = time.perf_counter() - t0
        desc = f"numpy restatement of find_bands, {len(pats)} patterns, 1 process"
    return {"value": len(pats) / dt, "unit": "patterns/s", "cores": cores, "kind": "port", "sample": desc}


VOTE_LIBRARY = os.path.join(ROOT, "tests", "golden", "vote_fcc_orient.npz")


def time_lambda(dev):
    """NLPAR.opt_lambda_array (the reference's opt_lambda_cpu, nlpar_cpu.py:94-155) on a 400x500
    scan of 80x80 patterns held on the device as float32: per-tile sigma and neighbour
    distances, then three bounded Nelder-Mead searches on the device objective.  The scan is
    a seeded 50x50 Voronoi scan tiled 8x10."""
    import torch
    import pyebsdindex_gb300 as pg
    from pyebsdindex_gb300 import synthetic as syn
    small, _ = syn.voronoi_scan(50, 50, ngrains=40, h=H, w=W, seed=11)
    grid = np.tile(small.reshape(50, 50, H, W), (8, 10, 1, 1)).reshape(400 * 500, H, W)
    d = torch.from_numpy(grid).to(dev).to(torch.float32)
    nl = pg.NLPAR(lam=0.7, searchradius=3)
    nl.opt_lambda_array(d[:2500], 50, 50)  # warm-up (kernels, pools)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lam = nl.opt_lambda_array(d, 400, 500)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    return {"seconds": dt, "patterns_per_s": 400 * 500 / dt, "lambda": [float(x) for x in lam],
            "workload": "opt_lambda on a 400x500 scan of 80x80 patterns (device float32), target weights "
                        "0.5 / 0.34 / 0.25"}


def time_nlpar_file():
    """NLPAR's file interface on a 400x500 scan of 80x80 uint8 patterns in a UP1 file (a seeded
    50x50 Voronoi scan tiled 8x10, written just before): opt_lambda (sigma and distances per
    tile, three Nelder-Mead searches), then calcnlpar (per tile: read, sigma, the average on
    the device, the interior clipped and written to the output file), wall-clock each."""
    import shutil
    import tempfile
    import pyebsdindex_gb300 as pg
    from pyebsdindex_gb300 import synthetic as syn
    from pyebsdindex_gb300.ebsd_pattern import write_up
    d = tempfile.mkdtemp(prefix="ebsdbench_")
    try:
        if shutil.disk_usage(d).free < 3 * 400 * 500 * H * W:
            return {"skipped": "the scan does not fit the temporary directory"}
        small, _ = syn.voronoi_scan(50, 50, ngrains=40, h=H, w=W, seed=11)
        grid = np.tile(small.reshape(50, 50, H, W), (8, 10, 1, 1)).reshape(400 * 500, H, W)
        src = os.path.join(d, "scan.up1")
        write_up(src, grid, nCols=500, nRows=400)
        del grid
        warm = os.path.join(d, "warm.up1")
        write_up(warm, small, nCols=50, nRows=50)
        pg.NLPAR(warm, searchradius=3).auto_nlpar(fileout=os.path.join(d, "warm_out.up1"), verbose=0)
        nl = pg.NLPAR(src, searchradius=3)
        t0 = time.perf_counter()
        lam = nl.opt_lambda(verbose=0)
        t1 = time.perf_counter()
        nl.calcnlpar(fileout=os.path.join(d, "out.up1"), verbose=0)
        t2 = time.perf_counter()
        return {"opt_lambda_s": t1 - t0, "calcnlpar_s": t2 - t1, "calcnlpar_patterns_per_s": 400 * 500 / (t2 - t1),
                "lambda": [float(x) for x in lam],
                "workload": "NLPAR file interface, 400x500 scan of 80x80 uint8 patterns, UP1 in the page cache, "
                            "search radius 3"}
    finally:
        shutil.rmtree(d, ignore_errors=True)


def time_file(bd, plan, method, pool, n, fmt="up1"):
    """find_bands streamed from a pattern file -- EDAX UP1 (default), Oxford .ebsp (uint8
    records with x, y footers) or ThermoFisher .pat (uint16 records) -- by
    ebsd_find_bands_file: parallel reads into pinned buffers overlapping the copies and the
    detection, records to host memory.  The file is written just before, so it is read from
    the page cache."""
    import shutil
    import tempfile
    from pyebsdindex_gb300.ebsd_pattern import write_ebsp, write_tfpat, write_up
    n = max(512, (n // 512) * 512)  # a 512-column scan
    d = tempfile.mkdtemp(prefix="ebsdbench_")
    try:
        need = n * H * W * (2 if fmt == "pat" else 1) + n * 64 + 4096
        if shutil.disk_usage(d).free < 3 * need:
            return {"skipped": f"{need / 1e9:.1f} GB file does not fit the temporary directory"}
        reps = (n + len(pool) - 1) // len(pool)
        pats = np.tile(pool, (reps, 1, 1))[:n]
        path = os.path.join(d, "bench." + fmt)
        if fmt == "ebsp":
            write_ebsp(path, pats, nCols=512, nRows=n // 512)
        elif fmt == "pat":
            write_tfpat(path, pats.astype(np.uint16), nCols=512, nRows=n // 512, bitdepth=8)
        else:
            write_up(path, pats, nCols=512, nRows=n // 512)
        del pats
        import torch
        from pyebsdindex_gb300 import _lib
        from pyebsdindex_gb300.ebsd_pattern import _bind as bind_up
        lib = bind_up()
        hout = {k: torch.empty(((n, NBANDS, 2) if k in ("maxloc", "aveloc") else (n, NBANDS)),
                               dtype=torch.int8 if k == "valid" else torch.float32, pin_memory=True)
                for k in _lib.BAND_FIELDS}
        hb = _lib.Bands(**{k: _lib.C.c_void_p(v.data_ptr()) for k, v in hout.items()})

        def run(count):
            _lib.check(lib.ebsd_find_bands_file(plan.handle, _lib.method_id(method), path.encode(), 0, 0, count,
                                                _lib.C.byref(hb), 0), "ebsd_find_bands_file")
        run(min(n, 65536))  # pinned chunk buffers, page cache
        t0 = time.perf_counter()
        run(n)
        dt = time.perf_counter() - t0
        kind = {"up1": "UP1", "ebsp": "EBSP", "pat": "TFPAT"}[fmt]
        return {"value": n / dt, "unit": "patterns/s", "patterns": n, "file_bytes": os.path.getsize(path),
                "source": f"ebsd_find_bands_file: {kind} file in the page cache, 65,536-pattern chunks, band "
                          "fields to pinned host arrays"}
    finally:
        shutil.rmtree(d, ignore_errors=True)


def time_indexing(outs, bd, N, stream, with_cpu, detect_ms):
    """The records -> orientations chain on the device after detection (EBSDIndexer's
    _indexbandsphase, _ebsd_index_single.py:720-800, for the FCC phase): band normals
    (ebsd_radon2pole), band weights (ebsd_band_intensity) and triplet voting (ebsd_band_index),
    each timed with CUDA events on the records of the whole batch, inputs resident."""
    import torch
    from pyebsdindex_gb300 import radon_fast, tripletvote as tv
    d = np.load(VOTE_LIBRARY)
    params = json.loads(str(d["params"]))
    lib = {k[4:]: d[k] for k in d.files if k.startswith("lib_")}
    bi = tv.BandIndexer(lib=lib, angTol=params["angTol"], nband_earlyexit=params["nband_earlyexit"],
                        simpleqweights=params["simpleqweights"])
    pc = [0.46, 0.70, 0.64]
    st = stream.cuda_stream
    vout = None

    def stage(fn, reps=2):
        fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            r = fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps, r

    ms_n, normals = stage(lambda: radon_fast.radon2pole_gpu(outs["theta"], outs["rho"], (H, W), PC=pc, vendor="EDAX",
                                                            stream=st))
    ms_i, (adj, pq, iq) = stage(lambda: tv.band_intensity_gpu(outs["max"], outs["normmax"], outs["theta"],
                                                              outs["rho"], outs["valid"], bd.rhoMax, stream=st))
    vout = bi.bandindex_device(normals, adj, stream=st)
    ms_v, _ = stage(lambda: bi.bandindex_device(normals, adj, out=vout, stream=st))
    indexed = float((vout["nmatch"] >= 3).float().mean().item())
    res = {
        "workload": f"records of the {N:,} detected patterns -> FCC orientations (angTol 2, QUEST), PC (0.46, 0.70, 0.64) EDAX",
        "normals_patterns_per_s": N / (ms_n / 1000.0),
        "intensity_patterns_per_s": N / (ms_i / 1000.0),
        "vote_patterns_per_s": N / (ms_v / 1000.0),
        "patterns_to_orientations_per_s": N / ((detect_ms + ms_n + ms_i + ms_v) / 1000.0),
        "fraction_indexed": indexed,
        "kernels": ["k_radon2pole", "k_band_intensity", "k_band_index"],
    }
    if with_cpu:
        from oracle import votecport  # the CPU leg: the C/OpenMP restatement of bandindex
        m = min(N, 65536)
        nrm = normals[:m].cpu().numpy()
        w = adj[:m].cpu().numpy()
        votecport.bandindex(lib, params, nrm[:1024], w[:1024])  # threads up
        t0 = time.perf_counter()
        votecport.bandindex(lib, params, nrm, w)
        dt = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": m / dt, "unit": "patterns/s", "cores": votecport.threads(), "kind": "port",
                               "sample": f"bandindex of the first {m} patterns' records, C/OpenMP restatement, "
                                         f"all host threads"}
    return res


def time_diff(dev):
    """The differentiable configuration: 4096 patterns (a 64 x 64 scan, 120x120 float32, peak
    50 counts), NLPAR radius 2 -> Gaussian background subtraction -> Radon (nTheta 180, nRho
    180) -> LoG -> soft-argmax band sharpness; forward plus backward (dJ/dlambda, dJ/dsigma,
    dJ/dx through every stage, the NLPAR weights' dependence on the patterns included)."""
    import torch
    import pyebsdindex_gb300 as pg
    from pyebsdindex_gb300 import diff, synthetic as syn
    n_r = n_c = 64
    hh = 120
    bd = pg.BandDetect(nTheta=180, nRho=180, tSigma=1.0, rSigma=1.0, rhoMaskFrac=0.1, nBands=9)
    bd.band_detect_setup(patDim=(hh, hh), patternmask=syn.circular_mask(hh, hh))
    t0 = time.perf_counter()
    obj = diff.BandSharpness(bd, n_r, n_c, searchradius=2, tau=2.0)
    setup_s = time.perf_counter() - t0
    scan = syn.voronoi_scan_rows(n_r, n_c, 0, n_r, ngrains=60, h=hh, w=hh, seed=9, peak_range=(50.0, 50.0))
    x0 = torch.from_numpy(scan.reshape(n_r * n_c, hh * hh).astype(np.float32)).to(dev)

    def step():
        x = x0.clone().requires_grad_(True)
        lam = torch.tensor(0.9, device=dev, requires_grad=True)
        bgs = torch.tensor(6.0, device=dev, requires_grad=True)
        J = obj(x, lam, bgs)
        J.backward()
        return J, lam.grad, bgs.grad
    step()
    torch.cuda.synchronize()
    reps = 3
    t0 = time.perf_counter()
    for _ in range(reps):
        J, gl, gs = step()
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) / reps * 1e3
    return {"workload": "4096 x 120x120 float32 (64x64 scan, peak 50), NLPAR radius 2, background sigma, Radon "
                        "nTheta 180 x nRho 180, LoG, soft-argmax; forward + backward",
            "ms_forward_backward": ms, "patterns_per_s": n_r * n_c / ms * 1e3, "operator_setup_s": setup_s,
            "J": float(J.detach()), "dJ_dlambda": float(gl), "dJ_dsigma": float(gs)}


MIXED_SIZES = (60, 120, 240)


def _mixed_part(args):
    h, start, count = args
    from pyebsdindex_gb300 import synthetic as syn
    pats, _, noise_only = syn.make_patterns(count, h, h, seed=3_000_000 + 1_000 * h, start=start, dtype=np.uint16,
                                            peak=4000.0, noise_frac=0.1)
    return pats, noise_only


def mixed_pools(ex, per_size):
    """Seeded uint16 patterns (Poisson peak 4000 counts) per size of the mixed-size configuration,
    with the flags of the noise-only patterns: {h: (patterns, noise_only)}."""
    out = {}
    for h in MIXED_SIZES:
        parts = [(h, s, min(256, per_size - s)) for s in range(0, per_size, 256)]
        got = list(ex.map(_mixed_part, parts))
        out[h] = (np.concatenate([g[0] for g in got]), np.concatenate([g[1] for g in got]))
    return out


def time_mixed(pools, n_total, steps, dev):
    """The mixed-size configuration: n_total uint16 patterns, one third each at 60x60, 120x120
    and 240x240 (nRho 1.5 * size, nTheta 180, nBands 10, circular mask), one persistent fused
    launch over all three sizes per step (MixedBandDetect / ebsd_find_bands_mixed), inputs
    resident, each size's slab width autotuned first; then each size alone and the per-stage
    FP32 path for comparison; and, on each size's pool of distinct patterns, the accuracy of the
    mixed launch and of FP16 Radon storage (where a kernel has it) against the FP64 method
    (plain64), with the FCC orientations indexed from each set of records compared with those
    from the FP64 records."""
    import torch
    from pyebsdindex_gb300 import synthetic as syn
    from pyebsdindex_gb300.band_detect import MixedBandDetect
    from pyebsdindex_gb300 import _lib
    from pyebsdindex_gb300.accuracy import compare_records, orientation_agreement
    mb = MixedBandDetect(nBands=10, mask_for=syn.circular_mask)
    each = n_total // len(MIXED_SIZES)
    batches = {}
    for h in MIXED_SIZES:
        # tiled as int16 (torch's uint16 has few device operations), then viewed as uint16
        pd = torch.from_numpy(pools[h][0].view(np.int16)).to(dev)
        reps = (each + pd.shape[0] - 1) // pd.shape[0]
        batches[(h, h)] = pd.repeat(reps, 1, 1)[:each].contiguous().view(torch.uint16)
    st = torch.cuda.current_stream(dev)
    # the slab width of every size, autotuned on a sample of that size before the timed steps
    tuned = mb.autotune({k: v[:4096 if k[0] < 240 else 1024] for k, v in batches.items()}, stream=st)

    def run(b):
        return mb.find_bands_device(b, stream=st)
    outs = run(batches)
    torch.cuda.synchronize()
    mixed = mb.last_mixed
    # one persistent launch over all sizes (and the per-size float64 epilogues), captured once in
    # a CUDA graph writing the same outputs, then replayed per step
    side = torch.cuda.Stream(dev)
    side.wait_stream(st)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=side):
        mb.find_bands_device(batches, stream=side, out=outs)
    torch.cuda.synchronize()
    graph.replay()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ev[0].record(st)
    for _ in range(steps):
        graph.replay()
    ev[1].record(st)
    torch.cuda.synchronize()
    ms = ev[0].elapsed_time(ev[1]) / steps
    res = {"workload": f"{3 * each:,} uint16 patterns (Poisson peak 4000), one third each at 60x60 / 120x120 / "
                       "240x240, nRho 1.5*size, nTheta 180, nBands 10; pools of distinct seeded patterns per size "
                       f"({pools[60][0].shape[0]}) tiled",
           "one_launch": mixed, "cuda_graph": True, "ms_per_step": ms, "patterns_per_s": 3 * each / ms * 1e3,
           "autotuned_slabs": {f"{k[0]}x{k[1]}": {"slabs": v["slabs"], "ms_per_sample": v["ms"]} for k, v in tuned.items()},
           "per_size": {}}
    for h in MIXED_SIZES:
        key = (h, h)
        t = batches[key]
        plan = mb.plan(h, h)._device_plan()
        sub = {key: t}
        run(sub)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        run(sub)
        e1.record(st)
        torch.cuda.synchronize()
        entry = {"fused_patterns_per_s": t.shape[0] / e0.elapsed_time(e1) * 1e3}
        npl = min(t.shape[0], 16384 if h < 240 else 4096)
        po = {f: torch.empty((npl,) + tuple(v.shape[1:]), dtype=v.dtype, device=dev) for f, v in outs[key].items()}
        plan.find_bands_device(t.data_ptr(), 1, npl, {f: v.data_ptr() for f, v in po.items()}, "plain", stream=st.cuda_stream)
        torch.cuda.synchronize()
        e0.record(st)
        plan.find_bands_device(t.data_ptr(), 1, npl, {f: v.data_ptr() for f, v in po.items()}, "plain", stream=st.cuda_stream)
        e1.record(st)
        torch.cuda.synchronize()
        entry["plain_patterns_per_s"] = npl / e0.elapsed_time(e1) * 1e3
        na = min(t.shape[0], pools[h][0].shape[0])
        plan.find_bands_device(t.data_ptr(), 1, na, {f: v.data_ptr() for f, v in po.items()}, "plain64", stream=st.cuda_stream)
        torch.cuda.synchronize()
        entry["accuracy_vs_plain64"] = dict(compare_records({f: v[:na] for f, v in outs[key].items()},
                                                            {f: v[:na] for f, v in po.items()}), patterns=na)
        ref64 = {f: v[:na].clone() for f, v in po.items()}
        # FP16 Radon storage: the single-tile kernel where its FP16 tile fits, else theta slabs
        # (re-laid to the widest slabs whose FP16 tile fits, then put back for the FP32 path)
        tile_fp32 = plan.get_tile()
        if mb.plan(h, h)._pick_method(plan, "fused16", _lib.EBSD_U16) == "fused16":
            plan.find_bands_device(t.data_ptr(), _lib.EBSD_U16, na, {f: v.data_ptr() for f, v in po.items()}, "fused16",
                                   stream=st.cuda_stream)
            torch.cuda.synchronize()
            f16 = {f: v[:na].clone() for f, v in po.items()}
            t16 = plan.get_tile()
            entry["fused16_accuracy_vs_plain64"] = dict(compare_records(f16, ref64), patterns=na,
                                                        kernel="one tile" if t16["single_fits"] else
                                                        f"{t16['slabs']} theta slabs")
        else:
            f16 = None
            entry["fused16_accuracy_vs_plain64"] = "no FP16-storage kernel for this plan"
        plan.set_tile(0, tile_fp32["slabs"])
        # indexing agreement: FCC orientations (triplet voting on the device) from these records
        # against those from the FP64 method's records, over the patterns that carry bands (the
        # noise-only tenth has no orientation to agree on)
        rho_max = mb.plan(h, h).rhoMax
        bands = ~pools[h][1][:na]
        q64, n64 = index_records(ref64, h, rho_max, st)
        q32, n32 = index_records({f: v[:na] for f, v in outs[key].items()}, h, rho_max, st)
        entry["indexing_vs_plain64"] = {"fused": orientation_agreement(q32[bands], n32[bands], q64[bands], n64[bands])}
        if f16 is not None:
            q16, n16 = index_records(f16, h, rho_max, st)
            entry["indexing_vs_plain64"]["fused16"] = orientation_agreement(q16[bands], n16[bands], q64[bands],
                                                                            n64[bands])
        res["per_size"][str(h)] = entry
    return res


_INDEXER = None


def index_records(recs, h, rho_max, stream):
    """FCC orientations (quaternions, nMatch; numpy) of device band records of h x h patterns:
    band normals (PC 0.46, 0.70, 0.64, EDAX), band weights (the plan's rhoMax) and triplet
    voting on the device."""
    global _INDEXER
    from pyebsdindex_gb300 import radon_fast, tripletvote as tv
    if _INDEXER is None:
        d = np.load(VOTE_LIBRARY)
        params = json.loads(str(d["params"]))
        lib = {k[4:]: d[k] for k in d.files if k.startswith("lib_")}
        _INDEXER = tv.BandIndexer(lib=lib, angTol=params["angTol"], nband_earlyexit=params["nband_earlyexit"],
                                  simpleqweights=params["simpleqweights"])
    normals = radon_fast.radon2pole_gpu(recs["theta"], recs["rho"], (h, h), PC=[0.46, 0.70, 0.64], vendor="EDAX",
                                        stream=stream.cuda_stream)
    adj, _, _ = tv.band_intensity_gpu(recs["max"], recs["normmax"], recs["theta"], recs["rho"], recs["valid"],
                                      rho_max, stream=stream.cuda_stream)
    out = _INDEXER.bandindex_device(normals, adj, stream=stream.cuda_stream)
    return out["quat"].cpu().numpy().astype(np.float64), out["nmatch"].cpu().numpy()


SCAN_ROWS, SCAN_COLS = 400, 500


def _scan_part(args):
    r0, r1 = args
    from pyebsdindex_gb300 import synthetic as syn
    return syn.voronoi_scan_rows(SCAN_ROWS, SCAN_COLS, r0, r1, ngrains=300, h=H, w=W, seed=5, peak_range=(30.0, 200.0))


def nlpar_scan(ex):
    """The NLPAR configuration's scan: 400 x 500 80x80 uint8 patterns from 300 seeded Voronoi
    grains, per-pixel Poisson peak counts drawn from 30-200 (row blocks generated in parallel)."""
    parts = [(r, min(r + 16, SCAN_ROWS)) for r in range(0, SCAN_ROWS, 16)]
    return np.concatenate(list(ex.map(_scan_part, parts)))


def time_nlpar_detect(scan, plan_bd, dev):
    """NLPAR (radius 3, lambda 0.7, nlpar_cpu.py:821-936) on the 400 x 500 scan held on the
    device, its average stored as uint8 straight from the averaging kernel (as the reference
    writes its NLPAR output file, pat_flt2int 'clip'), then band detection (fused kernel) on it:
    the pair's rate, each stage's time, and the same chain with a float32 intermediate."""
    import torch
    import pyebsdindex_gb300 as pg
    from pyebsdindex_gb300 import _lib
    from pyebsdindex_gb300.accuracy import compare_records
    n = SCAN_ROWS * SCAN_COLS
    x = torch.from_numpy(scan).to(dev).to(torch.float32).reshape(n, H, W)
    nl = pg.NLPAR(lam=0.7, searchradius=3)
    plan = plan_bd._device_plan(dev.index or 0)
    st = torch.cuda.current_stream(dev)
    outs = {f: torch.empty((n, NBANDS, 2) if f in ("maxloc", "aveloc") else (n, NBANDS),
                           dtype=torch.int8 if f == "valid" else torch.float32, device=dev) for f in _lib.BAND_FIELDS}
    outs32 = {f: torch.empty_like(v) for f, v in outs.items()}

    def chain(out_dtype, o):
        a = nl.calcnlpar_array(x, SCAN_ROWS, SCAN_COLS, reset_sigma=True, out_dtype=out_dtype)
        b = torch.cuda.Event(enable_timing=True)
        b.record(st)
        dt = _lib.EBSD_U8 if out_dtype is np.uint8 else _lib.EBSD_F32
        plan.find_bands_device(a.data_ptr(), dt, n, {f: v.data_ptr() for f, v in o.items()},
                               "fused", stream=st.cuda_stream)
        return a, b
    chain(np.uint8, outs)  # warm-up
    torch.cuda.synchronize()
    e0, e2 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    avg, e1 = chain(np.uint8, outs)
    e2.record(st)
    torch.cuda.synchronize()
    total, t_nlpar = e0.elapsed_time(e2), e0.elapsed_time(e1)
    f0, f2 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    chain(np.float32, outs32)
    torch.cuda.synchronize()
    f0.record(st)
    _, f1 = chain(np.float32, outs32)
    f2.record(st)
    torch.cuda.synchronize()
    c = compare_records(outs, outs32)
    return {"workload": "NLPAR radius 3, lambda 0.7 on a 400x500 scan of 80x80 uint8 patterns (300 Voronoi grains, "
                        "peaks 30-200 counts), average stored uint8, then find_bands (nTheta 180, nRho 120, nBands 9)",
            "patterns_per_s": n / total * 1e3, "ms": total, "nlpar_ms": t_nlpar, "detect_ms": total - t_nlpar,
            "float32_intermediate": {"patterns_per_s": n / f0.elapsed_time(f2) * 1e3, "nlpar_ms": f0.elapsed_time(f1),
                                     "detect_ms": f0.elapsed_time(f2) - f0.elapsed_time(f1)},
            "uint8_vs_float32_intermediate": c}, avg


def _nlpar_oracle_chain(sub):
    """The oracle's NLPAR (restating nlpar_nb) of a sub-scan, stored uint8 as the reference's
    writer does (clip, truncate), then the oracle's FFT restatement of find_bands."""
    from oracle import band_oracle as bo, nlpar_oracle as no
    from pyebsdindex_gb300 import synthetic as syn
    r, c = sub.shape[0], sub.shape[1]
    data = sub.reshape(r * c, H * W).astype(np.float32)
    ind = np.nonzero(no.automask(H, W).ravel())[0]
    sig = no.sigma(data, r, c, ind)
    avg = no.nlpar(data, 0.7, 3, 0.0, sig, r, c, ind)
    pats = np.clip(avg, 0, 255).astype(np.uint8).reshape(r * c, H, W)
    plan = bo.Plan((H, W), NTHETA, NRHO, 1.0, 1.0, 0.1, NBANDS, mask=syn.circular_mask(H, W))
    return bo.find_bands(plan, pats, conv="fft"), pats


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    sample = args.cpu_sample or 4096
    with host_executor() as ex:
        pool = make_pool(min(args.pool, sample), ex)
    pool = np.concatenate([pool] * ((sample + len(pool) - 1) // len(pool)))[:sample]
    vals = []
    base = None
    for i in range(args.warmup + args.steps):
        b = cpu_baseline(pool, sample, "port")
        if i >= args.warmup:
            vals.append(b["value"])
        base = b
    v = float(np.median(vals)) if vals else base["value"]
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "patterns/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * sample / v,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "method": "cpu restatement (C/OpenMP)",
                   "patterns_per_step": sample,
                   "sample": f"each step times {sample} patterns of the 1,000,000-pattern workload's pool"},
        "cpu_baseline": dict(base, value=v),
        "e2e": {"value": v, "unit": "patterns/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    # the pattern pool is generated by spawned host processes before the GPU is touched
    ex = host_executor()
    pool = make_pool(args.pool, ex)
    mpools = None if args.no_mixed else mixed_pools(ex, 2048)
    scan = None if args.no_nlpar else nlpar_scan(ex)
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    bd = make_plan()
    bd.gpu_id = local
    plan = bd._device_plan(local)
    method = args.method
    if method is None:
        method = "fused" if plan.supported("fused") else "plain"
    if method.startswith("fused") and not plan.supported(method):
        method = "plain"
    from pyebsdindex_gb300 import _lib

    N = args.patterns
    pool_d = torch.from_numpy(pool).to(dev)
    reps = (N + len(pool) - 1) // len(pool)
    pats_d = pool_d.repeat(reps, 1, 1)[:N].contiguous()
    del pool_d
    nB = NBANDS
    outs = {
        "max": torch.empty((N, nB), dtype=torch.float32, device=dev),
        "normmax": torch.empty((N, nB), dtype=torch.float32, device=dev),
        "maxloc": torch.empty((N, nB, 2), dtype=torch.float32, device=dev),
        "avemax": torch.empty((N, nB), dtype=torch.float32, device=dev),
        "aveloc": torch.empty((N, nB, 2), dtype=torch.float32, device=dev),
        "width": torch.empty((N, nB), dtype=torch.float32, device=dev),
        "theta": torch.empty((N, nB), dtype=torch.float32, device=dev),
        "rho": torch.empty((N, nB), dtype=torch.float32, device=dev),
        "valid": torch.empty((N, nB), dtype=torch.int8, device=dev),
    }
    ptrs = {k: v.data_ptr() for k, v in outs.items()}
    stream = torch.cuda.current_stream(dev)

    # autotune the patterns per block pass on a sample of the batch, then capture one step
    # (the whole batch is one persistent launch per 1M-pattern chunk) in a CUDA graph
    ppp = "rule: 8 for uint8 without background"
    if not args.no_autotune:
        ppp = plan.autotune(pats_d.data_ptr(), _lib.EBSD_U8, min(N, 16384), method, stream=stream.cuda_stream)
    radon_tile = plan.get_tile()
    plan.reserve(method, N)

    def launch(st):
        plan.find_bands_device(pats_d.data_ptr(), _lib.EBSD_U8, N, ptrs, method, stream=st.cuda_stream)

    launch(stream)
    torch.cuda.synchronize()
    launches_per_step = plan.last_launches()
    graph = None
    if not args.no_graph:
        side = torch.cuda.Stream(dev)
        side.wait_stream(stream)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=side):
            launch(side)
        torch.cuda.synchronize()

    def step():
        if graph is not None:
            graph.replay()
        else:
            launch(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clk = ClockSampler(local)
    clk.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    step_ms = []
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(args.steps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        step()
        b.record(stream)
        step_ms.append((a, b))
    ev1.record(stream)
    torch.cuda.synchronize()
    clocks = clk.stop()
    total_ms = ev0.elapsed_time(ev1)
    per_step = [a.elapsed_time(b) for a, b in step_ms]
    if world > 1:
        t = torch.tensor([total_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * N * args.steps / (total_ms / 1000.0)

    # roofline: the dominant kernel (one fused launch per chunk, or the per-stage sequence)
    hbm = None
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
        hbm, peak_src = float(peaks["hbm_gbs"]), "measured"
    except Exception:
        hbm, peak_src = 6800.0, "fallback"
    # fused methods launch the fused kernel plus a small float64 epilogue pass per chunk; the
    # per-launch time is the step time per fused launch (the epilogue is ~0.01% of it)
    fused_launches = max(launches_per_step // 2, 1)
    launch_ms = float(np.mean(per_step)) / fused_launches if method.startswith("fused") else float(np.mean(per_step))
    units_per_launch = N / fused_launches if method.startswith("fused") else N
    achieved = BYTES_PER_PATTERN * units_per_launch / (launch_ms / 1000.0) / 1e9
    traffic = DRAM_BYTES_PER_PATTERN * units_per_launch if method == "fused" and ppp in (8, "rule: 8 for uint8 without background") else None
    roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
            "traffic": traffic, "traffic_source": "ncu capture, 40,000 patterns, scaled per pattern" if traffic else None,
            "peak_source": peak_src,
            "kernel": "k_fused (+ k_band_epilogue)" if method.startswith("fused") else "per-stage sequence (7 kernels/chunk)"}
    if method == "fused" and clocks.get("sm_mhz"):
        # the roofline that binds this kernel: instruction issue, 4 warp-instructions per SM
        # per clock at the sampled SM clock; warp-instructions per pattern from ncu
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        issue_peak = 4.0 * sms * clocks["sm_mhz"] * 1e6
        issue_achieved = WARP_INST_PER_PATTERN * units_per_launch / (launch_ms / 1000.0)
        roof.update({"issue_achieved": issue_achieved, "issue_peak": issue_peak, "issue_unit": "warp-inst/s",
                     "issue_frac": issue_achieved / issue_peak,
                     "issue_source": "smsp__inst_executed.sum per pattern from ncu (40,000 patterns); peak = 4 x SMs x "
                                     "median sampled SM clock"})

    # accuracy of the timed records: against the FP64 per-stage method (plain64, the FP64 GPU
    # oracle) on the first patterns of the timed batch, whose records the last step wrote
    acc = None
    if method != "plain64":
        from pyebsdindex_gb300.accuracy import compare_records
        na = min(N, ACCURACY_PATTERNS)
        ref64 = {k: torch.empty((na,) + tuple(v.shape[1:]), dtype=v.dtype, device=dev) for k, v in outs.items()}
        plan.find_bands_device(pats_d.data_ptr(), _lib.EBSD_U8, na, {k: v.data_ptr() for k, v in ref64.items()},
                               "plain64", stream=stream.cuda_stream)
        torch.cuda.synchronize()
        acc = {"vs_plain64": dict(compare_records({k: v[:na] for k, v in outs.items()}, ref64), patterns=na),
               "bar": "integer peaks identical on >= 99.9% of bands, aveloc within 1e-3 Radon px"}
    else:
        ref64 = None

    # end to end through the drop-in call: BandDetect.find_bands(numpy uint8 [N, 80, 80]) ->
    # the reference's (N, nBands) record array (band_detect.py:411, dtype :110-115); every
    # step moves the patterns from host memory to the GPU and the records back
    e2e = None
    if not args.no_e2e:
        host_np = np.ascontiguousarray(np.tile(pool, (reps, 1, 1))[:N])
        e2e_steps = max(1, min(args.steps, 3))
        # one full-size warm-up call (pinned staging slots, device buffers), then the timed calls;
        # each returns a fresh record array, as the reference's find_bands does
        del_rec = bd.find_bands(host_np, method=method)
        del del_rec
        step_s = []
        for _ in range(e2e_steps):
            t0 = time.perf_counter()
            rec = bd.find_bands(host_np, method=method)
            step_s.append(time.perf_counter() - t0)
            assert rec.shape == (N, nB) and rec.dtype == bd.dataType
            del rec
        dt = float(np.median(step_s)) * e2e_steps
        # the C ABI with pinned host buffers, band fields as arrays (no record packing)
        host = torch.empty((N, H, W), dtype=torch.uint8, pin_memory=True)
        host.copy_(torch.from_numpy(host_np))
        hout = {k: torch.empty(v.shape, dtype=v.dtype, pin_memory=True) for k, v in outs.items()}
        hb = _lib.Bands(**{k: _lib.C.c_void_p(v.data_ptr()) for k, v in hout.items()})
        lib = _lib.load()

        def soa_step():
            _lib.check(lib.ebsd_find_bands_host(plan.handle, _lib.method_id(method), _lib.EBSD_U8,
                                                _lib.C.c_void_p(host.data_ptr()), N, _lib.C.byref(hb), 0))
        soa_step()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            soa_step()
        dt_soa = time.perf_counter() - t0
        in_place = plan.host_input_in_place()
        # the same with the input staged by copy engines instead of read in place
        plan.set_host_input(0)
        soa_step()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            soa_step()
        dt_copy = time.perf_counter() - t0
        plan.set_host_input(-1)
        e2e = {"value": N * e2e_steps / dt * world, "unit": "patterns/s", "h2d_bytes_per_step": N * H * W,
               "d2h_bytes_per_step": N * nB * 41,
               "call": "BandDetect.find_bands(numpy uint8 [N, 80, 80]) -> reference record array (209 B per band)",
               "timing": f"median of {e2e_steps} calls after one full-size warm-up call",
               "call_s": [round(v, 4) for v in step_s],
               "c_abi_value": N * e2e_steps / dt_soa * world,
               "c_abi_call": "ebsd_find_bands_host, pinned patterns and pinned band-field arrays",
               "c_abi_input_path": ("pinned patterns read in place by the kernels over NVLink-C2C (every byte crosses "
                                    "the link each step)") if in_place else "pinned patterns staged by copy engines",
               "c_abi_copy_engine_value": N * e2e_steps / dt_copy * world}
        del host, hout, host_np

    # the other methods on the same device-resident input, for the batched-vs-plain comparison
    variants, variants_acc = {}, {}
    if not args.no_variants:
        # separate outputs: `outs` keeps the timed method's records for the indexing below
        vouts = {k: torch.empty_like(v) for k, v in outs.items()}
        vptrs = {k: v.data_ptr() for k, v in vouts.items()}
        for vm, vn in (("plain", min(N, 131072)), ("fused", N), ("fused16", N)):
            if vm == method or (vm.startswith("fused") and not plan.supported(vm)):
                continue
            def vstep():
                plan.find_bands_device(pats_d.data_ptr(), _lib.EBSD_U8, vn, vptrs, vm, stream=stream.cuda_stream)
            vstep()
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(2):
                vstep()
            b.record(stream)
            torch.cuda.synchronize()
            variants[vm] = vn * 2 / (a.elapsed_time(b) / 1000.0)
            if ref64 is not None and vm != "plain":
                from pyebsdindex_gb300.accuracy import compare_records
                na = ref64["valid"].shape[0]
                variants_acc[vm] = dict(compare_records({k: v[:na] for k, v in vouts.items()}, ref64), patterns=na)
        variants[method] = value / world
        if "plain" in variants:
            variants["batched_over_plain_fp32"] = {m: variants[m] / variants["plain"] for m in ("fused", "fused16")
                                                   if m in variants}
        del vouts
    ref64 = None

    file_e2e = None
    if rank == 0 and not args.no_file:
        file_e2e = time_file(bd, plan, method, pool, args.file_patterns, args.file_format)

    nlpar_lambda = None
    if rank == 0 and args.lambda_scan:
        nlpar_lambda = time_lambda(dev)
    nlpar_file = None
    if rank == 0 and args.nlpar_file:
        nlpar_file = time_nlpar_file()

    mixed = None
    if mpools is not None and rank == 0:
        mixed = time_mixed(mpools, args.mixed_patterns, max(2, min(args.steps, 5)), dev)

    nlpar_detect = None
    if scan is not None and rank == 0:
        nlpar_detect, _ = time_nlpar_detect(scan, bd, dev)

    diffp = None
    if not args.no_diff and rank == 0:
        diffp = time_diff(dev)

    indexing = None
    if not args.no_index:
        indexing = time_indexing(outs, bd, N, stream, rank == 0 and world == 1 and not args.no_cpu,
                                 float(np.mean(per_step)))

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        try:
            cpu = cpu_baseline(pool, args.cpu_sample or min(len(pool), 2048), "port")
        except Exception as e:  # reported, never silently replaced
            cpu = {"value": None, "error": str(e)}
        if acc is not None:
            # the oracle's FFT restatement of the reference find_bands on the first patterns of
            # the timed batch, run by the host process pool; the records graded are the timed
            # step's (plain64 above overwrote nothing of `outs`)
            try:
                no = min(N, ORACLE_PATTERNS)
                acc["vs_oracle_fft"] = dict(oracle_accuracy(ex, pool[:no] if no <= len(pool) else
                                                            pats_d[:no].cpu().numpy(), outs), patterns=no)
            except Exception as e:
                acc["vs_oracle_fft"] = {"error": str(e)}
        if nlpar_detect is not None:
            # the oracle chain on the scan's top-left 32 x 32 block, against the device chain on
            # the same block (NLPAR windows shift inward at a scan's edges)
            try:
                import pyebsdindex_gb300 as pg
                from pyebsdindex_gb300.accuracy import compare_records
                sub = scan.reshape(SCAN_ROWS, SCAN_COLS, H, W)[:32, :32]
                ref, ref_pats = ex.submit(_nlpar_oracle_chain, sub).result()
                nl = pg.NLPAR(lam=0.7, searchradius=3)
                got_pats = nl.calcnlpar_array(sub.reshape(32 * 32, H, W), 32, 32, out_dtype=np.uint8)
                got = bd.find_bands(got_pats, method="fused")
                nlpar_detect["vs_oracle_chain"] = dict(
                    compare_records(got, ref), patterns=32 * 32,
                    pattern_pixels_differing=float(np.mean(got_pats != ref_pats)),
                    oracle="nlpar_nb restatement -> clip/truncate uint8 -> find_bands restatement with FFT, 32x32 "
                           "sub-scan")
            except Exception as e:
                nlpar_detect["vs_oracle_chain"] = {"error": str(e)}
    ex.shutdown()

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "patterns/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "u8 in, f16 Radon storage, f32 accumulate" if method == "fused16" else
                     ("u8 in, f32" if method in ("plain", "fused") else "u8 in, f64"),
            "data": "synthetic",
            "config": {"workload": WORKLOAD,
                       "method": method, "patterns_per_step": N, "distinct_patterns": len(pool),
                       "patterns_per_block_pass": ppp, "radon_tile": radon_tile, "cuda_graph": graph is not None,
                       "l2": "input 6.4 GB > L2, no flush", "parallelism": f"replicas x{world}"},
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks, "accuracy": acc,
            "variants_patterns_per_s": variants, "variants_accuracy_vs_plain64": variants_acc,
            "indexing": indexing, "file_e2e": file_e2e,
            "nlpar_lambda": nlpar_lambda, "nlpar_file": nlpar_file, "mixed_sizes": mixed,
            "nlpar_detect": nlpar_detect, "differentiable": diffp,
            "gpu_launches": launches_per_step * args.steps,
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
