// Internal declarations shared by the libebsdgpu translation units.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include <algorithm>
#include <mutex>
#include <vector>

#include "../../include/ebsdgpu.h"

namespace ebsd {

constexpr int kMaxBands = 32;

// Fused-kernel geometry chosen at plan creation (see fused.cu).
struct FusedGeom {
    int ok = 0;                 // the tile fits on chip (FP16 Radon storage)
    int ok_f32 = 0;             // ... and with FP32 Radon storage
    int threads = 0;            // threads per block
    int smem_f32 = 0;           // dynamic shared memory bytes, FP32 Radon storage
    int smem_f16 = 0;           // dynamic shared memory bytes, FP16 Radon storage
    // Radon tile = padded rows [row0, row1) x padded columns [col0, col1)
    int row0 = 0, row1 = 0, col0 = 0, col1 = 0;
    // conv region (rows/cols of the padded frame whose LoG value is needed)
    int crow0 = 0, crow1 = 0, ccol0 = 0, ccol1 = 0;
    int tile_pitch = 0;         // pattern tile row pitch (elements)
    float ksum = 0.0f;          // sum of the LoG taps
    int nGroups = 0;            // 32-ray groups of the fused LUT
    int nRaysPad = 0;           // nGroups * 32
    int gpt = 0;                // groups per theta column (ceil(nRho / 32))
    int npad = 0;               // padding cells of the Radon tile
    int quad = 0;               // the 4/8-patterns-per-pass tile (8-byte elements) fits
};

// Theta-slab fused geometry (slab.cu): plans whose padded Radon image does not fit on chip
// next to its LoG image run the fused path in theta slabs of up to Ts output columns.
struct SlabGeom {
    int ok = 0;                 // the slab kernel takes this plan (uint8 / uint16 input)
    int ok_f32 = 0;             // ... and float32 input (a float32 pattern tile fits)
    int nslab = 0, Ts = 0;      // slabs; widest slab's output columns
    int maxg = 0;               // most 32-ray groups of one slab
    int TR = 0, TBP = 0, CCP = 0, MP = 0, rho0 = 0, rpad_end = 0, CR = 0, statR = 0;
    int pitch = 0;              // pattern tile row pitch (elements)
    int smem[3] = {0, 0, 0};    // dynamic shared memory bytes per dtype (uint8, uint16, float32)
    int regb = 0;               // bytes of the FP32 Radon-tile region
    int nslab_min = 0, nslab_max = 0;  // slab counts whose tiles fit (nslab_min: the widest slabs)
    // FP16 Radon storage (integer patterns, 5x5 LoG): theta-max rows of pitch MP16 (tmb16
    // bytes) before the 16-bit tile; region regb16 bytes; shared memory per dtype (uint8, uint16)
    int ok16 = 0, MP16 = 0, tmb16 = 0, regb16 = 0;
    int smem16[2] = {0, 0};
};

// Host copy of the slab kernel's per-source-group LUT slots (one group = 32 neighbouring rho at
// one theta), kept with the plan so that the slab count can be changed after plan creation
// (ebsd_plan_set_tile, ebsd_plan_autotune) without the reference's lookup table.
struct SlabSource {
    int gpt = 0, nsrc = 0;
    int TR = 0, CR = 0, rho0 = 0, rpad_end = 0, statR = 0, pitch = 0;
    size_t pat_elems = 0;
    uint16_t zero = 0;                 // element offset of the tile's zero element
    std::vector<int> gch;              // [nsrc] 8-slot chunks per group
    std::vector<size_t> goff;          // [nsrc] first slot of the group in `slots`
    std::vector<uint16_t> slots;       // per group: [chunk][lane][8] element offsets
    std::vector<int32_t> count;        // [nsrc * 32] entries per ray
};

struct Workspace {
    void* ptr = nullptr;
    size_t bytes = 0;
};

}  // namespace ebsd

struct ebsd_plan_s {
    int device = 0;
    int H = 0, W = 0, nPx = 0, nTheta = 0, nRho = 0, nRays = 0, nB = 0;
    int p0 = 0, p1 = 0;     // padding (rho, theta)
    int pk0 = 0, pk1 = 0;   // peak windows (rho, theta)
    int k0 = 0, k1 = 0;     // kernel shape (rho, theta)
    int R = 0, Tp = 0;      // padded Radon extent
    int maxCount = 0;       // longest ray
    int bg_mode = 0;        // 0 none, 1 float64 subtraction, 2 float32 subtraction

    // ---- device tables ----
    uint16_t* d_lut16 = nullptr;   // [maxCount][nRays] entry-major, pixel index
    int32_t* d_lut32 = nullptr;    // same when H*W >= 65535
    int32_t* d_count = nullptr;    // [nRays]
    uint8_t* d_rdnmask = nullptr;  // [nRays]
    uint32_t* d_rdnbits = nullptr; // [nTheta][rdn_words]: bit (i & 31) of word i >> 5 = rdnmask[i][j]
    int rdn_words = 0;             // (nRho + 31) / 32 + 1: a word past the last, for two-word reads
    float* d_kernel = nullptr;     // [k0*k1]
    std::vector<float> h_kernel;   // host copy of the taps (fused-kernel parameters)
    // separable LoG: taps[a][b] = ku[a] * kw[b] to within two float32 ulps of the largest tap
    // (the reference's kernel, a Gaussian second derivative along rho times a Gaussian along
    // theta, always is); the FP32 paths then convolve by rows, then by columns
    int sep = 0;
    std::vector<float> h_ku, h_kw;  // [k0], [k1]
    float* d_ksep = nullptr;        // [k0 + k1]: ku then kw
    double* d_kernel64 = nullptr;  // [k0*k1]
    double* d_theta = nullptr;     // [nTheta] degrees (float32 values widened)
    double* d_rho = nullptr;       // [nRho]
    double* d_bg = nullptr;        // [nPx]
    float* d_bgf = nullptr;        // [nPx]

    // fused-kernel tables
    ebsd::FusedGeom fg;
    uint16_t* d_flut = nullptr;    // fused LUT (see fused.cu)
    uint16_t* d_flut8 = nullptr;   // the same with offsets for 8-byte tile elements (fg.quad)
    int32_t* d_fgroup = nullptr;   // [nRaysPad] entry counts, then [nGroups] chunks per group
    unsigned* d_fpad = nullptr;    // [npad] padding cell list of the fused Radon tile
    float* d_fray = nullptr;       // [nPx] weights: sum_px w*pixel = mean of the non-empty rays
    int64_t flut_entries = 0;
    // patterns per block pass of the fused FP32 uint8 kernel: -1 = rule (the most the plan
    // allows: 8, else 2), else 1, 2, 4 or 8 as chosen by ebsd_plan_autotune
    int fused_ppp = -1;

    // theta-slab fused tables (see slab.cu)
    ebsd::SlabGeom sg;
    uint16_t* d_slut = nullptr;    // per-slab, per-warp LUT streams (pattern element offsets)
    int32_t* d_stab = nullptr;     // [gst][gtb][slab_g][slab_j][wofs][count]
    int32_t s_gst = 0, s_gtb = 0, s_slabg = 0, s_slabj = 0, s_wofs = 0, s_count = 0;  // offsets into d_stab
    ebsd::SlabSource* ssrc = nullptr;  // host slots for re-layout (slab.cu)
    float* d_swimg = nullptr;      // [nPx] slab plans' pixel weights: sum_px w*pixel = Radon mean (FP16 centring)
    // FP32 fused calls that both kernels can serve: 0 rule (the single tile when it fits),
    // 1 the single tile, 2 theta slabs (ebsd_plan_set_tile, ebsd_plan_autotune)
    int tile_mode = 0;

    // ---- workspaces ----
    std::mutex mtx;
    ebsd::Workspace ws;            // per-stage intermediates
    ebsd::Workspace stats;         // per-pattern min/mean
    int64_t ws_chunk = 0;
    int ws_method = -1;

    // host-pipeline buffers (ebsd_find_bands_host)
    cudaStream_t hstream[2] = {nullptr, nullptr};
    cudaEvent_t hevent[2] = {nullptr, nullptr};
    void* h_in_dev[2] = {nullptr, nullptr};
    void* h_out_dev[2] = {nullptr, nullptr};
    size_t h_in_bytes = 0, h_out_bytes = 0;

    // host pipelines (ebsd_find_bands_host for pageable input, ebsd_find_bands_file): pinned
    // chunk buffers the filler thread fills
    void* h_pin[3] = {nullptr, nullptr, nullptr};
    size_t h_pin_bytes = 0;
    // pinned host input: -1 read in place when the GPU reaches host memory through the host
    // page tables (NVLink-C2C), else copy; 0 always copy; 1 always read in place
    int host_input_mode = -1;
    // pinned staging of records for pageable output arrays (two chunk slots)
    void* h_outpin[2] = {nullptr, nullptr};
    size_t h_outpin_bytes = 0;

    int64_t last_launches = 0;
};

namespace ebsd {

// Error helpers -------------------------------------------------------------------------
#define EBSD_CUDA_TRY(expr)                                                        \
    do {                                                                           \
        cudaError_t _e = (expr);                                                   \
        if (_e != cudaSuccess) {                                                   \
            return (_e == cudaErrorMemoryAllocation) ? EBSD_E_NOMEM : EBSD_E_LAUNCH; \
        }                                                                          \
    } while (0)

inline int launch_status() {
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) return EBSD_OK;
    return (e == cudaErrorMemoryAllocation) ? EBSD_E_NOMEM : EBSD_E_LAUNCH;
}

inline size_t elem_size(int dtype) {
    return dtype == EBSD_U8 ? 1 : (dtype == EBSD_U16 ? 2 : 4);
}

// UP pattern files: patfile.cu ----------------------------------------------------------
int up_parse_header(const char* path, int bitdepth, ebsd_up_info* info);
int up_read_range(int fd, const ebsd_up_info* info, int64_t start, int64_t n, void* dst, int threads);
int default_read_threads();
// Oxford EBSP / ThermoFisher TFPAT files: patfile.cu
bool pf_path(const char* path);  // .ebsp or .pat
int pf_parse_header(const char* path, ebsd_pf_info* info);
int pf_read_positions(int fd, const ebsd_pf_info* info, uint64_t* pos);
int pf_read_range(int fd, const ebsd_pf_info* info, const uint64_t* pos, int64_t start, int64_t n, void* dst,
                  void* aux, int threads);

// Per-stage (plain) path: plain.cu ------------------------------------------------------
size_t plain_workspace_bytes(const ebsd_plan_s* p, int method, int64_t chunk);
int plain_run_chunk(ebsd_plan_s* p, int method, int dtype, const void* d_pats, int64_t n,
                    const ebsd_bands* out, int64_t out_offset, cudaStream_t st, int64_t* launches);
// The same with an explicit workspace of plain_workspace_bytes(p, method, n) bytes.
int plain_run_chunk_ws(ebsd_plan_s* p, int method, int dtype, const void* d_pats, int64_t n,
                       const ebsd_bands* out, int64_t out_offset, cudaStream_t st,
                       int64_t* launches, void* workspace);

// Fused path: fused.cu -------------------------------------------------------------------
int fused_prepare(ebsd_plan_s* p, const ebsd_plan_desc* d);
void fused_release(ebsd_plan_s* p);
int fused_supported(const ebsd_plan_s* p, int method);
size_t fused_workspace_bytes(const ebsd_plan_s* p, int method, int64_t chunk);
// 1, 2, 4 or 8: patterns one block pass of the fused kernel would process for this call
int fused_patterns_per_pass(const ebsd_plan_s* p, int method, int dtype, int64_t n);
int fused_run_chunk(ebsd_plan_s* p, int method, int dtype, const void* d_pats, int64_t n,
                    const ebsd_bands* out, int64_t out_offset, cudaStream_t st, int64_t* launches);

// Theta-slab fused path: slab.cu -----------------------------------------------------------
int slab_prepare(ebsd_plan_s* p, const ebsd_plan_desc* d);
// Rebuild the slab tables for nslab slabs (0: the widest slabs that fit); EBSD_E_UNSUPPORTED
// when the plan has no slab tables or nslab is out of [nslab_min, nslab_max].  Waits for the
// device before it frees the old tables.
int slab_relayout(ebsd_plan_s* p, int nslab);
void slab_release(ebsd_plan_s* p);
// the slab kernel serves this (method, dtype): the FP32 method when the plan is too large for
// the single tile or set to theta slabs (tile_mode 2); FP16 storage (uint8 / uint16, 5x5 LoG)
// when the single FP16 tile does not fit
bool slab_serves(const ebsd_plan_s* p, int method, int dtype);
int slab_run_chunk(ebsd_plan_s* p, int method, int dtype, const void* d_pats, int64_t n, const ebsd_bands* out,
                   int64_t out_offset, cudaStream_t st, int64_t* launches);
// mixed pattern sizes in one launch: up to 8 plans of one input type and LoG size
constexpr int kMaxMixedPlans = 8;
bool slab_mixable(const ebsd_plan_s* p, int dtype);
int slab_run_mixed(ebsd_plan_s* const* plans, int nplans, int dtype, const void* const* d_pats, const int64_t* n,
                   const ebsd_bands* out, cudaStream_t st, int64_t* launches);

}  // namespace ebsd
