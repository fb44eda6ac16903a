/*
 * ebsdgpu.h -- C ABI of the GB300 band-detection library (libebsdgpu.so).
 *
 * The library replaces the hot path behind PyEBSDIndex's BandDetect.find_bands:
 *   background subtraction + lookup-table Radon  (radon_fast.py:242-310)
 *   theta/rho padding + LoG convolution + stats  (band_detect.py:562-637)
 *   11x11 max-filter peak search + Radon mask    (band_detect.py:639-664, :811-843)
 *   top-N band labelling + 3x3 sub-pixel fit     (band_detect.py:667-809)
 *   normmax / theta / rho epilogue               (band_detect.py:457-460, :519-524)
 * and its OpenCL dispatch (opencl/band_detect_cl.py:51-199).
 *
 * Conventions
 *   - Every entry point returns 0 on success or a negative EBSD_E* code; ebsd_strerror()
 *     turns a code into text.  Nothing falls back to the CPU.
 *   - Device pointers are plain CUDA device addresses; streams are cudaStream_t passed as
 *     void*.  Plans own their device tables; callers own pattern and output buffers.
 *   - A plan may be used from one host thread at a time.  Calls on one plan with different
 *     streams are serialised by the plan's internal workspace lock.
 */
#ifndef EBSDGPU_H
#define EBSDGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------- */
#define EBSD_OK 0
#define EBSD_E_ARG (-1)        /* bad argument (null pointer, size, shape)              */
#define EBSD_E_DTYPE (-2)      /* unsupported pattern data type                          */
#define EBSD_E_NOMEM (-3)      /* device or pinned-host allocation failed                 */
#define EBSD_E_LAUNCH (-4)     /* a kernel launch or CUDA runtime call failed            */
#define EBSD_E_UNSUPPORTED (-5)/* plan shape outside what a method supports              */
#define EBSD_E_DEVICE (-6)     /* no usable CUDA device / wrong device                    */
#define EBSD_E_TIMEOUT (-7)    /* a bounded device-side wait gave up                      */
#define EBSD_E_SCRATCH (-8)    /* request needs more scratch than the static array holds   */
#define EBSD_E_IO (-9)         /* a pattern file could not be opened, read or parsed       */
#define EBSD_E_FORMAT (-10)    /* a pattern file in a form not read (compressed, version 0) */

/* ---- pattern element types (BandDetect.find_bands accepts uint8, uint16, float32) ---- */
#define EBSD_U8 0
#define EBSD_U16 1
#define EBSD_F32 2

/* ---- methods --------------------------------------------------------------------------
 * EBSD_PLAIN_F32  per-stage kernels, FP32 intermediates in HBM (the structure of the
 *                 reference's OpenCL path, opencl/band_detect_cl.py:51-199).
 * EBSD_PLAIN_F64  the same pipeline in FP64 end to end: the FP64 GPU oracle.
 * EBSD_FUSED_F32  one persistent fused kernel per chunk, Radon image stored FP32 on chip.
 * EBSD_FUSED_F16  the fused kernel with the Radon image stored FP16 (FP32 accumulation). */
#define EBSD_PLAIN_F32 0
#define EBSD_PLAIN_F64 1
#define EBSD_FUSED_F32 2
#define EBSD_FUSED_F16 3

typedef struct ebsd_plan_s* ebsd_plan_t;
typedef struct ebsd_linop_s* ebsd_linop_t;

/* Everything BandDetect.band_detect_setup (band_detect.py:138-294) derives for one pattern
 * size.  All pointers are HOST pointers, copied during ebsd_plan_create. */
typedef struct {
    int32_t H, W;                 /* pattern rows, columns                                  */
    int32_t nTheta, nRho;         /* Radon samples (radonPlan.nTheta / .nRho)              */
    int32_t nBands;               /* bands per pattern, 1..32                              */
    int32_t pad_rho, pad_theta;   /* BandDetect.padding                                    */
    int32_t peak_rho, peak_theta; /* BandDetect.peakPad (odd max-filter window sizes)      */
    int32_t ksz_rho, ksz_theta;   /* LoG kernel shape (BandDetect.kernel[0].shape)         */
    const float* kernel;          /* [ksz_rho*ksz_theta] LoG taps, row-major                */
    int32_t lut_len;              /* third extent of radonPlan.indexPlan (max(H, W))       */
    const int64_t* lut;           /* radonPlan.indexPlan [nRho][nTheta][lut_len], each ray
                                     sorted ascending; entries >= H*W end the ray           */
    const uint8_t* rdnmask;       /* BandDetect.rdnmask [nRho][nTheta] (0/1)               */
    const float* theta;           /* radonPlan.theta [nTheta], degrees                     */
    const float* rho;             /* radonPlan.rho [nRho]                                  */
    const double* background;     /* BandDetect.backgroundsub [H][W] or NULL               */
    int32_t background_f32;       /* 1: background was float32 (subtract in float32)      */
} ebsd_plan_desc;

/* Structure-of-arrays band output; n patterns x nBands, row-major.  All nine arrays are
 * required.  Device pointers for ebsd_find_bands, host pointers for ebsd_find_bands_host.
 * maxloc/aveloc are (rho, theta) pairs in the un-padded Radon frame, as in the record. */
typedef struct {
    float* max;      /* 'max'      */
    float* normmax;  /* 'normmax'  */
    float* maxloc;   /* 'maxloc'   [..][2] */
    float* avemax;   /* 'avemax'   */
    float* aveloc;   /* 'aveloc'   [..][2] */
    float* width;    /* 'width'    */
    float* theta;    /* 'theta'    radians */
    float* rho;      /* 'rho'      */
    int8_t* valid;   /* 'valid'    */
} ebsd_bands;

/* Replaces BandDetect.band_detect_setup's products (band_detect.py:138-294) and the
 * radon_fast.Radon lookup table (radon_fast.py:64-165) on the device.  The LUT is
 * re-encoded for the GPU (ray-interleaved for the per-stage kernels, ray-major packed for
 * the fused kernel).  `device` is the CUDA ordinal the plan lives on. */
int ebsd_plan_create(const ebsd_plan_desc* desc, int device, ebsd_plan_t* out);

/* Frees the plan's device tables and workspaces. */
int ebsd_plan_destroy(ebsd_plan_t plan);

/* Whether `method` can run this plan (the fused kernels need the plan's on-chip tile to fit
 * in shared memory).  Returns 1 / 0, or a negative code. */
int ebsd_method_supported(ebsd_plan_t plan, int method);

/* The same for input of `dtype`: the theta-slab form of the fused FP32 method (plans too
 * large for one on-chip tile) takes float32 input only where a float32 pattern tile fits. */
int ebsd_method_supported_for(ebsd_plan_t plan, int method, int dtype);

/* Reserves the per-plan workspace for chunks of up to max_chunk patterns so that later
 * calls allocate nothing.  Optional: find_bands reserves on first use. */
int ebsd_plan_reserve(ebsd_plan_t plan, int method, int64_t max_chunk);

/* BandDetect.find_bands (band_detect.py:411-526) on device-resident patterns:
 * d_pats [n][H][W] of `dtype`, outputs into device arrays.  Asynchronous on `stream`.
 * `chunk` <= 0 picks the plan's default chunk size. */
int ebsd_find_bands(ebsd_plan_t plan, int method, int dtype, const void* d_pats, int64_t n,
                    const ebsd_bands* d_out, int64_t chunk, void* stream);

/* Mixed pattern sizes in one persistent launch: the FP32 fused method for up to 8 plans at
 * once (e.g. one plan per detector size), plan k's d_pats[k] [n[k]][H_k][W_k] of `dtype`
 * into d_out[k].  The reference runs one size per BandDetect plan and rebuilds the plan when
 * the size changes (band_detect.py:138-155); here every persistent CTA strides over the
 * patterns of all plans, each pattern detected in theta slabs with its plan's tables.  All
 * plans live on one device and share the LoG size; each must report
 * ebsd_method_supported(plan, EBSD_FUSED_F32) and qualify for the slab kernel (uint8 /
 * uint16 input; float32 where its pattern tile fits), else EBSD_E_UNSUPPORTED.  Records equal
 * those of ebsd_find_bands with EBSD_FUSED_F32 on each plan alone, up to the last bit of
 * normmax.  Asynchronous on `stream`; allocates nothing. */
int ebsd_find_bands_mixed(const ebsd_plan_t* plans, int nplans, int dtype, const void* const* d_pats,
                          const int64_t* n, const ebsd_bands* d_out, void* stream);

/* The same on HOST buffers: copies each chunk in, runs it and copies the bands out, with
 * two streams so copies overlap compute.  Pinned host memory gives overlapped copies;
 * pageable memory works but serialises.  Synchronous: returns when the outputs are
 * written. */
int ebsd_find_bands_host(ebsd_plan_t plan, int method, int dtype, const void* h_pats,
                         int64_t n, const ebsd_bands* h_out, int64_t chunk);

/* How ebsd_find_bands_host[_records] moves PINNED host input to the GPU.  -1 (default):
 * the kernels read it in place over the CPU-GPU link when the device uses the host's page
 * tables (GB300's NVLink-C2C), else copy engines stage it chunk by chunk; 0: always stage
 * with copies; 1: always read in place.  Either way every input byte crosses the link once
 * per call.  Pageable input is always staged through pinned buffers. */
int ebsd_plan_set_host_input(ebsd_plan_t plan, int mode);

/* 1 when pinned host input is read in place under the plan's current mode, 0 when copied. */
int ebsd_plan_host_input_in_place(ebsd_plan_t plan);

/* Number of kernel launches the last ebsd_find_bands / ebsd_find_bands_host call on this
 * plan issued (for launch accounting by benchmarks). */
int64_t ebsd_last_launch_count(ebsd_plan_t plan);

/* Autotuner -- no counterpart in the reference, whose OpenCL path sizes its work by fixed
 * rules (band_detect_cl.py:252-286).  Times the fused-kernel variants that give identical
 * records for (method, dtype) on the caller's device-resident sample d_pats [n][H][W] and keeps
 * the fastest in the plan for later calls.  The variants are the Radon tile shapes the plan
 * can take: the whole padded Radon image as one tile with one, two, four or eight patterns per
 * block pass (uint8 input), and, for EBSD_FUSED_F32, theta slabs -- the widest slabs that fit
 * and up to three narrower slab counts.  Writes the patterns per pass of the choice to
 * *patterns_per_pass (may be NULL; 1 for slabs and where only one pass width applies:
 * per-stage methods, uint16/float32 input, a fitted background, FP16 storage); the tile
 * shape is read back with ebsd_plan_get_tile.  Synchronous on `stream`; allocates temporary
 * outputs. */
int ebsd_plan_autotune(ebsd_plan_t plan, int method, int dtype, const void* d_pats, int64_t n,
                       void* stream, int* patterns_per_pass);

/* Pins the fused kernel's patterns per block pass for later calls: 1, 2, 4 or 8 (capped at what
 * a call allows), or 0 for the rule (the most a call allows).  For callers that tuned
 * offline; no counterpart in the reference.  Records do not depend on the choice. */
int ebsd_plan_set_patterns_per_pass(ebsd_plan_t plan, int patterns_per_pass);

/* The plan's Radon tile shape for EBSD_FUSED_F32 calls (no counterpart in the reference). */
typedef struct {
    int tile;               /* 1: the whole padded Radon image as one tile (when it fits);
                               2: theta slabs; 0: neither fits (per-stage methods only) */
    int patterns_per_pass;  /* one tile, uint8 input: 1, 2, 4 or 8 as pinned, 0 the rule */
    int slabs;              /* slab count of the plan's slab tables (0: the plan has none) */
    int slab_columns;       /* output theta columns of the widest slab */
    int slabs_min;          /* widest slabs that fit */
    int slabs_max;          /* narrowest slabs that still hold the filters' theta reach */
    int single_fits;        /* 1 when the one-tile kernel can take the plan */
    int slabs_fp16;         /* 1 when the current slab tables also take EBSD_FUSED_F16 (integer
                               patterns, 5x5 LoG): its theta-max rows need room beside the 16-bit
                               tile, so the widest slabs may leave none (240x240: from 10 slabs) */
} ebsd_tile_info;

int ebsd_plan_get_tile(ebsd_plan_t plan, ebsd_tile_info* info);

/* Pins the Radon tile shape for later EBSD_FUSED_F32 calls: tile 1 one tile, 2 theta slabs,
 * 0 the rule (one tile when it fits); slabs = the slab count for the slab tables, in
 * [slabs_min, slabs_max], or 0 for the widest.  The slab tables also serve
 * ebsd_find_bands_mixed.  EBSD_E_UNSUPPORTED for a shape the plan cannot take.  Waits for
 * the device when it rebuilds the slab tables, and frees the old ones: a CUDA graph captured
 * with the old slab count must be captured again (ebsd_plan_autotune and EBSD_FUSED_F16 on a
 * slab plan re-lay the tables too).  For callers that tuned offline; records do not depend on
 * the choice. */
int ebsd_plan_set_tile(ebsd_plan_t plan, int tile, int slabs);

/* Band detection that allocates nothing -- no counterpart in the reference, which always
 * allocates per chunk (band_detect.py:425, band_detect_cl.py:252-286).  For callers that may
 * not allocate device memory: applications whose device memory belongs to their framework's
 * pool allocator, and streaming loops that must keep a fixed footprint because
 * cudaMalloc/cudaFree can synchronise the device.  Runs the EBSD_PLAIN_F32 kernels on device
 * buffers (same results as ebsd_find_bands with EBSD_PLAIN_F32), with their scratch in a
 * 64 MiB file-scope device array that every GPU loading the library holds until exit.
 * At most floor((64 MiB - 1 KiB - 4*ksz_rho*ksz_theta) / (12*(nRho+2*pad_rho)*(nTheta+
 * 2*pad_theta) + nRho*nTheta + 8)) patterns per call (183 at 80x80, nRho 120, nTheta 180);
 * larger n returns EBSD_E_SCRATCH.  The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress, device current) and caches it: make that first call before
 * any stream capture.  All calls share the array; calls that overlap on the GPU race.  The
 * caller's current device is the same after the call as before it. */
int ebsd_find_bands_static(ebsd_plan_t plan, int dtype, const void* d_pats, int64_t n,
                           const ebsd_bands* d_out, void* stream);

/* NLPAR noise estimate (NLPAR.sigma_numba, nlpar_cpu.py:753-796, nn = 1): for each of the
 * nrows x ncols scan pixels, sqrt of the minimum over its clipped 3x3 neighbourhood of
 * SSD / (2 n) over the masked pixels d_indices[nind] whose values are both below the
 * saturation level (0.9961 * datamax, or datamax + 1 without saturation protection).
 * d_data [nrows*ncols][npx] float32 (device); d_sigma [nrows*ncols] float32 (device). */
int ebsd_nlpar_sigma(const float* d_data, int32_t nrows, int32_t ncols, int32_t npx,
                     const int32_t* d_indices, int32_t nind, float datamax, int saturation_protect,
                     float* d_sigma, void* stream);

/* One scan tile of NLPAR's sigma estimate for the lambda optimisation (NLPAR.calcsigma_cpu,
 * nlpar_cpu.py:157-264, which runs sigma_numba per tile with nn = 1 as uint64: the tile's first
 * row and column get empty windows).  Tile = rows [r0, r1) x columns [c0, c1) of the scan;
 * datamax is the tile's own maximum (computed here).  Merges into the scan arrays: d_sigma
 * [nrows*ncols] = min(d_sigma, tile sigma); d_d2 / d_n2 [nrows*ncols][9] (normalised distance
 * and pixel count per window slot, nlpar_cpu.py:805-817) replaced where the tile's count is
 * positive.  Initialise d_sigma to 1e18 and d_d2, d_n2 to 0, then call once per tile in
 * NLPAR._calcchunks order (nlpar_cpu.py:973-1065).  d_work: (r1-r0)*(c1-c0)*19 + 1 floats. */
int ebsd_nlpar_sigma_tile(const float* d_data, int32_t nrows, int32_t ncols, int32_t npx, int32_t r0,
                          int32_t r1, int32_t c0, int32_t c1, const int32_t* d_indices, int32_t nind,
                          int saturation_protect, float* d_sigma, float* d_d2, float* d_n2,
                          float* d_work, void* stream);

/* The lambda objective of NLPAR.opt_lambda_cpu (nlpar_cpu.py:107-113): mean over scan pixels
 * (rows and columns stepped by `stride`) of |tw - 1 / (sum_q exp(-max(d2_q, dthresh) / lam^2)
 * + 1e-12)|, in float64, into *d_out (device).  d_work: 256 doubles.  Deterministic. */
int ebsd_nlpar_lambda_metric(const float* d_d2, int32_t nrows, int32_t ncols, int32_t stride,
                             float dthresh, double lam, double tw, double* d_work, double* d_out,
                             void* stream);

/* NLPAR weighted neighbour average (NLPAR.nlpar_nb, nlpar_cpu.py:821-936) over a
 * (2 sr + 1)^2 search window (0 <= sr <= 10, shifted inward at the scan edges): d_out
 * [nrows*ncols][npx] float32.  d_work: caller-provided device scratch of
 * nrows*ncols*(2 sr + 1)^2 floats (the normalised window weights). */
int ebsd_nlpar(const float* d_data, int32_t nrows, int32_t ncols, int32_t npx,
               const int32_t* d_indices, int32_t nind, float datamax, float lam, int32_t sr,
               float dthresh, const float* d_sigma, int saturation_protect, float* d_work,
               float* d_out, void* stream);

/* ebsd_nlpar with the averaged patterns stored as `out_dtype`: EBSD_F32, or EBSD_U8 /
 * EBSD_U16 as the reference writes NLPAR's output file (calcnlpar_cpu -> write_data with
 * pat_flt2int 'clip', ebsd_pattern.py:118-182: clipped to the type's range, truncated), so that
 * band detection reads its usual integer input straight from the averaging kernel.
 * d_centre_offset (NULL: none) [nrows*ncols] is added to each pixel's own window weight before
 * the normalisation -- nlpar_nb's diff_offset addition (nlpar_cpu.py:880-925), which the
 * caller computes per pixel. */
int ebsd_nlpar_out(const float* d_data, int32_t nrows, int32_t ncols, int32_t npx,
                   const int32_t* d_indices, int32_t nind, float datamax, float lam, int32_t sr,
                   float dthresh, const float* d_sigma, int saturation_protect, float* d_work,
                   int out_dtype, void* d_out, const float* d_centre_offset, void* stream);

/* Noise sigma (optional), weights and average of ebsd_nlpar_out in one call for search radii
 * 1 <= sr <= 3, with each unordered pair's distance summed once: the squared difference of a
 * pair is symmetric bit for bit, so a pixel's window slot at offset -o reads the sum its
 * neighbour made for +o (slots beyond +-sr, which only windows shifted inward at the scan edges
 * have, are summed directly).  The results equal ebsd_nlpar_sigma + ebsd_nlpar_out bit for bit.
 * compute_sigma = 1: d_sigma [nrows*ncols] is written (NLPAR.sigma_numba, nn = 1, from the same
 * pass over the patterns); 0: d_sigma is read.  d_work (8-byte aligned): nrows*ncols*(W + 2 F + 8)
 * + 2 E W + 1 floats, W = (2 sr + 1)^2, F = sr (2 sr + 1) + sr, E = 2 sr (nrows + ncols - 2 sr)
 * (the edge pixels, whose windows are shifted inward).  EBSD_E_UNSUPPORTED where the staged
 * tiles pass 48 KB. */
int ebsd_nlpar_pairs_out(const float* d_data, int32_t nrows, int32_t ncols, int32_t npx,
                         const int32_t* d_indices, int32_t nind, float datamax, float lam, int32_t sr,
                         float dthresh, float* d_sigma, int compute_sigma, int saturation_protect,
                         float* d_work, int out_dtype, void* d_out, const float* d_centre_offset,
                         void* stream);

/* ---- band normals (Radon.radon2pole, radon_fast.py:314-397) ---------------------------- */
#define EBSD_VENDOR_EDAX 0
#define EBSD_VENDOR_OXFORD 1
#define EBSD_VENDOR_EMSOFT 2
#define EBSD_VENDOR_KIKUCHIPY 3
#define EBSD_VENDOR_BRUKER 4

/* Band (theta, rho) -> unit plane normals on the device, for [npat][nBands] bands (device
 * arrays, e.g. the theta/rho fields ebsd_find_bands wrote): d_normals [npat][nBands][3].
 * d_pc: DEVICE array of pattern centres in the vendor's convention, [npat][pc_stride] floats
 * (pc_stride 3, or 4 for EMSOFT with the pixel size), or one shared row when pc_stride is 0.
 * H, W: pattern rows, columns.  float32 arithmetic in the reference's order (sin/cos within
 * an ulp or two of numpy's).  Asynchronous on `stream`. */
int ebsd_radon2pole(const float* d_theta, const float* d_rho, int64_t npat, int32_t nBands,
                    int32_t H, int32_t W, int32_t vendor, const float* d_pc, int32_t pc_stride,
                    float* d_normals, void* stream);

/* ---- EDAX UP1 / UP2 pattern files (ebsd_pattern.UPFile, ebsd_pattern.py:435-570) ------- */
/* Header fields as UPFile.read_header (ebsd_pattern.py:449-513) sets them. */
typedef struct {
    int32_t version;         /* format version: 1, or >= 3                                  */
    int32_t W, H;            /* patternW, patternH                                           */
    int32_t bytes_per_px;    /* 1 (.up1, uint8) or 2 (.up2, uint16)                          */
    int64_t file_pos;        /* byte offset of the first pattern (filePos)                   */
    int64_t n_patterns;      /* nPatterns (version 1: from the file size)                    */
    int64_t n_cols, n_rows;  /* nCols, nRows (version 1: nPatterns x 1)                      */
    int32_t extra_patterns;  /* extraPatterns (version >= 3)                                 */
    int32_t hexflag;         /* hexflag (version >= 3)                                       */
    double x_step, y_step;   /* xStep, yStep (version >= 3, else 0)                          */
    int64_t file_bytes;      /* file size                                                    */
} ebsd_up_info;

/* Parses the header of `path` (.up1 / .up2, else bitdepth 8 or 16 decides the pixel type). */
int ebsd_up_read_header(const char* path, int bitdepth, ebsd_up_info* info);

/* Reads patterns [pat_start, pat_start + n) into h_dst (n * H * W pixels of the file's type)
 * with `threads` parallel positional reads (0: a default); pinned destinations make the later
 * host-to-device copies asynchronous.  UPFile.pat_reader (ebsd_pattern.py:515-537). */
int ebsd_up_read(const char* path, const ebsd_up_info* info, int64_t pat_start, int64_t n,
                 void* h_dst, int threads);

/* ---- Oxford .ebsp and ThermoFisher .pat pattern files (ebsd_pattern.EBSPFile, :709-1088;
 * ebsd_pattern.TFPatFile, :1090-1395) ---------------------------------------------------- */
#define EBSD_PF_EBSP 2
#define EBSD_PF_TFPAT 3

/* Header fields as EBSPFile.read_header (ebsd_pattern.py:724-918) / TFPatFile.read_header
 * (:1113-1167) find them.  Both formats keep one record per pattern: `record_head` bytes, the
 * pixels, then (EBSP) an optional x, y footer.  EBSP records sit where a table of uint64
 * positions (filePos; 0: pattern not stored, read as zeros) says; TFPAT records follow one
 * another from `first_record`, each an (x, y) pixel location pair of uint32 and the pixels. */
typedef struct {
    int32_t format;          /* EBSD_PF_EBSP or EBSD_PF_TFPAT                                */
    int32_t version;         /* EBSP: minus the leading int64 (1-5); TFPAT: the leading uint32 */
    int32_t W, H;            /* patternW, patternH                                           */
    int32_t bytes_per_px;    /* EBSP 1, 2 or 4 (from the first record); TFPAT 2 (uint16)     */
    int32_t record_head;     /* bytes in front of the pixels: EBSP 16 (24 from version 5), TFPAT 8 */
    int64_t n_patterns;      /* nPatterns                                                    */
    int64_t first_record;    /* EBSP: byte of the position table; TFPAT: byte of the first record (filePos) */
    int64_t record_bytes;    /* TFPAT: bytes per record; EBSP: 0 (positions from the table)  */
    int64_t file_bytes;      /* file size                                                    */
    int32_t has_xy;          /* EBSP: records carry x, y (float64) after the pixels           */
    int32_t xy_flag_bytes;   /* EBSP: 1 (a flag byte in front of x and of y) or 0 (version 1) */
    int32_t is_scan;         /* TFPAT: the header's scan flag (< 0: n_cols x n_rows patterns) */
    int32_t bitdepth;        /* TFPAT: the header's bit depth                                 */
    int32_t has_background;  /* TFPAT: a background pattern (uint16) at byte 25               */
    int32_t reserved;
    int64_t n_cols, n_rows;  /* TFPAT: the header's scan columns and rows                    */
} ebsd_pf_info;

/* Parses the header of an .ebsp or .pat file (by extension).  EBSD_E_IO for a file that cannot
 * be read or parsed, EBSD_E_FORMAT for compressed EBSP files and version 0 of either format,
 * which the reference does not read either. */
int ebsd_pf_read_header(const char* path, ebsd_pf_info* info);

/* EBSP: the n_patterns record positions (filePos) into h_pos. */
int ebsd_pf_read_positions(const char* path, const ebsd_pf_info* info, uint64_t* h_pos);

/* Reads patterns [pat_start, pat_start + n) into h_dst (n * H * W pixels of the file's type;
 * may be NULL to read h_aux only) and, when h_aux is not NULL, per pattern: EBSP x, y as two
 * float64 (zeros without a footer), TFPAT the record's two uint32 pixel locations.  h_pos:
 * the positions ebsd_pf_read_positions returned (EBSP; ignored for TFPAT).  Runs of records at
 * a constant spacing are read in large positional reads, by `threads` threads (0: a default).
 * EBSPFile.pat_reader (ebsd_pattern.py:920-958), TFPatFile.pat_reader (:1190-1225). */
int ebsd_pf_read(const char* path, const ebsd_pf_info* info, const uint64_t* h_pos,
                 int64_t pat_start, int64_t n, void* h_dst, void* h_aux, int threads);

/* find_bands on patterns [pat_start, pat_start + n) of a UP1 / UP2, EBSP or TFPAT file (by
 * extension; any other extension is read as UP with `bitdepth` 8 or 16), records to host
 * arrays: a reader thread fills three pinned chunk buffers from the file while two CUDA
 * streams copy, detect and copy back, so file reads, copies and compute overlap.  The file's
 * pattern size must be the plan's; the pixel type is the file's (uint8 / uint16).  `chunk`
 * <= 0 picks the plan's default.  Synchronous. */
int ebsd_find_bands_file(ebsd_plan_t plan, int method, const char* path, int bitdepth,
                         int64_t pat_start, int64_t n, const ebsd_bands* h_out, int64_t chunk);

/* ebsd_find_bands_host / ebsd_find_bands_file with the bands written as records: h_records
 * [n][nBands] records of `itemsize` bytes (the reference's BandDetect.dataType,
 * band_detect.py:110-115), the nine band fields (max, normmax, maxloc[2], avemax, aveloc[2],
 * width, theta, rho as float32, valid as int8, in ebsd_bands order) at field_offsets[9] bytes;
 * every other byte is zero.  Records are packed on the host, in parallel, while the next
 * chunk runs on the GPU. */
int ebsd_find_bands_host_records(ebsd_plan_t plan, int method, int dtype, const void* h_pats,
                                 int64_t n, void* h_records, int32_t itemsize,
                                 const int32_t* field_offsets, int64_t chunk);
int ebsd_find_bands_file_records(ebsd_plan_t plan, int method, const char* path, int bitdepth,
                                 int64_t pat_start, int64_t n, void* h_records, int32_t itemsize,
                                 const int32_t* field_offsets, int64_t chunk);

/* ---- band weights and pattern quality (_ebsd_index_single.py:751-763) ------------------
 * For [n][nBands] band fields (device arrays, e.g. what ebsd_find_bands wrote):
 *   adj[p][b] = (1 - |rho| * 0.5 / rhomax) * max * (theta > 2 deg ? 0.75 : 0.25)
 *               * (theta < 178 deg ? 0.75 : 0.25) * valid        (the vote's band intensity)
 *   pq[p] = mean_b(max * valid),  iq[p] = mean_b(normmax * valid)
 * in float32 with the reference's operation order (means summed in numpy's pairwise order).
 * d_pq / d_iq may be NULL.  nBands 1..128. */
int ebsd_band_intensity(const float* d_max, const float* d_normmax, const float* d_theta,
                        const float* d_rho, const int8_t* d_valid, int64_t n, int32_t nBands,
                        float rhomax, float* d_adj, float* d_pq, float* d_iq, void* stream);

/* ---- band indexing by triplet voting (tripletvote.BandIndexer.bandindex,
 * tripletvote.py:492-633, with high_fidelity on) --------------------------------------- */
typedef struct ebsd_vote_plan_s* ebsd_vote_plan_t;

/* One phase library as BandIndexer.build_trip_lib (tripletvote.py:320-490) leaves it.  All
 * pointers are HOST pointers, copied during ebsd_vote_plan_create. */
typedef struct {
    int32_t nfam;                /* pole families, 2..16 (BandIndexer.polefamilies rows)       */
    int32_t ntrip;               /* triplets (angtriplets['angles'] rows), 1..8192              */
    const double* trip_angles;   /* angtriplets['angles'] [ntrip][3], degrees, rows ascending  */
    const int64_t* trip_family;  /* angtriplets['familyid'] [ntrip][3], each < nfam            */
    const int64_t* lut;          /* BandIndexer.lut [3][3][3][3], entries 0..2                */
    int32_t npoles;              /* completelib['polesCart'] rows, 1..512                     */
    const double* poles_cart;    /* completelib['polesCart'] [npoles][3]                      */
    const int32_t* pole_family;  /* completelib['familyid'] [npoles], each < nfam             */
    const double* ang_table;     /* completelib['angTable'] [npoles][npoles], degrees         */
    const int32_t* fam_count;    /* completelib['nFamily'] [nfam]                             */
    const int64_t* fam_index;    /* completelib['famIndex'] [nfam]                            */
    double ang_tol;              /* BandIndexer.angTol, degrees                               */
    int32_t nband_earlyexit;     /* BandIndexer.nband_earlyexit                               */
    int32_t simple_qweights;     /* BandIndexer.simpleqweights (0/1)                          */
} ebsd_triplib_desc;

/* bandindex outputs for n patterns (DEVICE arrays, row-major).  The last five are the
 * vote's intermediates, written when non-NULL. */
typedef struct {
    double* quat;          /* [n][4] QUEST orientation (avequat)                           */
    double* fit;           /* [n] mean band misfit, degrees                                */
    float* cm;             /* [n] vote confidence of the matched bands (-1: < 3 matched)   */
    int64_t* polematch;    /* [n][nBands] library pole per band (-1000: pattern unindexed) */
    int64_t* nmatch;       /* [n] bands matched                                            */
    int64_t* ij;           /* [n][4] (ii, jj, band1, band2) of the winning band pair       */
    int32_t* acc_correct;  /* [n] matched bands whose voted family agrees                  */
    double* bandfit;       /* [n][nBands] per-band misfit, degrees                         */
    float* accw;           /* [n][nfam][nBands] weighted votes, or NULL                    */
    float* accn;           /* [n][nfam][nBands] vote counts, or NULL                       */
    int32_t* bandfam;      /* [n][nBands] voted family, or NULL                            */
    float* bandrank;       /* [n][nBands] band rank, or NULL                               */
    uint8_t* polevalid;    /* [n][nBands] band matched within angTol, or NULL              */
} ebsd_index_out;

int ebsd_vote_plan_create(const ebsd_triplib_desc* desc, int device, ebsd_vote_plan_t* out);
int ebsd_vote_plan_destroy(ebsd_vote_plan_t plan);

/* d_norms [n][nBands][3] float32 unit band normals (ebsd_radon2pole); d_intensity [n][nBands]
 * float32 band weights (ebsd_band_intensity) or NULL for all ones.  nBands 1..32.  One warp
 * per pattern for the vote and the band assignment, then one thread per pattern for the QUEST
 * solve and the fits, through a plan-owned hand-over buffer of up to 2^20 patterns: the first
 * call allocates it (make that call outside a CUDA-graph capture); later calls allocate
 * nothing and do not synchronise with the host.  One plan per stream: calls on one plan from
 * different streams at the same time share that buffer. */
int ebsd_band_index(ebsd_vote_plan_t plan, const float* d_norms, const float* d_intensity, int64_t n,
                    int32_t nBands, const ebsd_index_out* out, void* stream);

/* ---- differentiable path (no counterpart in the reference beyond the empty DIFF_NLPAR
 * placeholder, nlpar.py:75-77) --------------------------------------------------------- */

/* A sparse linear operator y = A x held on the device in CSR form (host arrays copied):
 * rowptr[nrows+1] (int64), col[nnz] (int32, < ncols), val[nnz] (float).  Used for the
 * Radon transform (val = 1/count over a ray's pixels, radon_fast.py:281-310), its transpose
 * (back-projection), and the LoG-with-padding operator of band_detect.py:573-606 and its
 * transpose.  The transpose is built on the host as its own operator, so both directions are
 * gathers. */
int ebsd_linop_create(int64_t nrows, int64_t ncols, const int64_t* rowptr, const int32_t* col,
                      const float* val, int device, ebsd_linop_t* out);

/* y[b] = A x[b] for b < n (n <= 65535); fp64 = 1 uses double values and double x / y. */
int ebsd_linop_apply(ebsd_linop_t op, int fp64, const void* d_x, int64_t n, void* d_y, void* stream);

/* The same with the patterns along the fast axis: x^T [ncols][ldx] and y^T [nrows][ldy] hold
 * pattern b in column b (b < n <= ldx, ldy).  Results equal ebsd_linop_apply's bit for bit;
 * the operator's rows are read once per 32 patterns and the reads of x^T are coalesced, which
 * is the layout a batch of thousands of patterns wants. */
int ebsd_linop_apply_cols(ebsd_linop_t op, int fp64, const void* d_xT, int64_t ldx, int64_t n, void* d_yT,
                          int64_t ldy, void* stream);

int ebsd_linop_destroy(ebsd_linop_t op);

/* NLPAR window weights of nlpar_nb (nlpar_cpu.py:866-927) exposed for differentiation:
 * d_w[p][c] normalised weights, d_m[p][c] = max(d_pc - dthresh, 0) (0 for the centre), so
 * that w_pc = exp(-m_pc / lam^2) / sum_c'.  Arrays nrows*ncols*(2 sr + 1)^2 floats. */
int ebsd_nlpar_weights(const float* d_data, int32_t nrows, int32_t ncols, int32_t npx,
                       const int32_t* d_indices, int32_t nind, float datamax, float lam, int32_t sr,
                       float dthresh, const float* d_sigma, int saturation_protect, float* d_w,
                       float* d_m, void* stream);

/* y = W x with given window weights (the averaging step of nlpar_nb, nlpar_cpu.py:929-934). */
int ebsd_nlpar_apply(const float* d_x, int32_t nrows, int32_t ncols, int32_t npx, const float* d_w,
                     int32_t sr, float* d_out, void* stream);

/* W^T g: the adjoint of ebsd_nlpar_apply. */
int ebsd_nlpar_apply_t(const float* d_g, int32_t nrows, int32_t ncols, int32_t npx, const float* d_w,
                       int32_t sr, float* d_out, void* stream);

/* float64 forms of ebsd_nlpar_apply / ebsd_nlpar_apply_t (weights given as float64), for
 * gradient checks of the differentiable path in double precision. */
int ebsd_nlpar_apply64(const double* d_x, int32_t nrows, int32_t ncols, int32_t npx,
                       const double* d_w, int32_t sr, double* d_out, void* stream);
int ebsd_nlpar_apply_t64(const double* d_g, int32_t nrows, int32_t ncols, int32_t npx,
                         const double* d_w, int32_t sr, double* d_out, void* stream);

/* One axis of a separable filter with reflect padding (torch's "reflect": index -q reads q,
 * L-1+q reads L-1-q; radius r < L): out[o] = sum_{t=-r..r} taps[t+r] in[refl(o+t)] along
 * axis 0 (rows) or 1 (columns) of [n][H][W], or with adjoint = 1 the transpose of that map
 * (a gather, no atomics).  fp64 selects double data and taps.  The background blur of the
 * differentiable path: forward along x then y, its adjoint, and d/dsigma with the taps'
 * derivative. */
int ebsd_blur1d(int fp64, int adjoint, int axis, const void* d_in, int64_t n, int32_t H, int32_t W,
                const void* d_taps, int32_t r, void* d_out, void* stream);

/* Soft-argmax band sharpness of n LoG-filtered Radon images [n][ncell]: per image
 * J_p = sum_i s_i c_i with s = softmax(c / tau) over the cells d_cells[ncm] (the Radon mask),
 * into d_J[n] (float64), and the gradient dJ_p / dc_i = s_i (1 + (c_i - J_p) / tau) into
 * d_grad (same layout as c; only the listed cells are written).  Sums in float64. */
int ebsd_softargmax(int fp64, const void* d_c, int64_t n, int64_t ncell, const int32_t* d_cells,
                    int32_t ncm, double tau, double* d_J, void* d_grad, void* stream);

/* NLPAR noise sigma (NLPAR.sigma_numba, nlpar_cpu.py:753-796, nn = 1) with what its
 * derivative needs: d_sig2 = sigma^2 (sigma rounded as the weights read it), d_arg = the 3x3
 * neighbour whose SSD / (2 n) is the minimum (-1: none), d_nsig = that pair's count. */
int ebsd_nlpar_sigma_arg(const float* d_data, int32_t nrows, int32_t ncols, int32_t npx,
                         const int32_t* d_indices, int32_t nind, float datamax, int saturation_protect,
                         float* d_sig2, int32_t* d_arg, float* d_nsig, void* stream);

/* The window weights of ebsd_nlpar_weights from sigma^2 (d_sig2), plus the partial
 * derivatives of each pair's normalised distance d = (S - n s) / (s sqrt(2 n))
 * (nlpar_cpu.py:897-917): d_dS = dd/dS, d_dsig = dd/ds with s = sigma_p^2 + sigma_c^2; both 0
 * at the centre, where d is replaced by 1e6 n, and where max(d - dthresh, 0) clamps. */
int ebsd_nlpar_weights_d(const float* d_data, int32_t nrows, int32_t ncols, int32_t npx,
                         const int32_t* d_indices, int32_t nind, float datamax, float lam, int32_t sr,
                         float dthresh, const float* d_sig2, int saturation_protect, float* d_w, float* d_m,
                         float* d_dS, float* d_dsig, void* stream);

/* Backward of the weights for y = W(lambda, x) x given g = dL/dy: into d_gx the part of dL/dx
 * that flows through the weights -- each pair's SSD over the masked pixels d_pmask[npx] where
 * both values pass the 0.999 saturation test, and each pattern's noise sigma through its
 * minimising pair (0.9961 test) -- and into d_glam[nrows*ncols] the per-pixel terms of
 * dL/dlambda.  (W^T g, the direct part, is ebsd_nlpar_apply_t.)  d_scratch holds
 * 3 * nrows*ncols*(2 sr + 1)^2 + nrows*ncols doubles.  fp64 selects double g, x and gx. */
int ebsd_nlpar_weights_grad(int fp64, const void* d_g, const void* d_x, int32_t nrows, int32_t ncols,
                            int32_t npx, int32_t sr, const float* d_w, const float* d_m, const float* d_dS,
                            const float* d_dsig, double lam, const uint8_t* d_pmask, float datamax,
                            int saturation_protect, const int32_t* d_arg, const float* d_nsig,
                            double* d_scratch, double* d_glam, void* d_gx, void* stream);

/* Per scan pixel p: sum_c dw_pc/dlambda (g_p . x_c) in float64 (d_out[nrows*ncols]); the sum
 * over p is dL/dlambda for L with dL/dy = g. */
int ebsd_nlpar_lambda_grad(const float* d_g, const float* d_x, int32_t nrows, int32_t ncols,
                           int32_t npx, const float* d_w, const float* d_m, int32_t sr, float lam,
                           double* d_out, void* stream);
/* The same with float64 g and x. */
int ebsd_nlpar_lambda_grad64(const double* d_g, const double* d_x, int32_t nrows, int32_t ncols,
                             int32_t npx, const float* d_w, const float* d_m, int32_t sr, float lam,
                             double* d_out, void* stream);

/* Text for a status code. */
const char* ebsd_strerror(int code);

/* Library version string. */
const char* ebsd_version(void);

#ifdef __cplusplus
}
#endif
#endif /* EBSDGPU_H */
