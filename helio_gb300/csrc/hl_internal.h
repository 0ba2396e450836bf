// hl_internal.h — launchers shared between the kernel translation units and the
// C-ABI layer (hl_api.cu). Not part of the public interface.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "../../include/helio_gb300.h"

namespace hl {

struct BinLight;
struct SliceTable;
struct BinViewDesc;

// Device view of a G-buffer (validated by the API layer).
struct GBufView {
    const unsigned char* plane[HL_GBUF_MAX_PLANES];
    uint64_t pitch[HL_GBUF_MAX_PLANES];
    uint32_t width, height;
};

struct TargetView {
    unsigned char* data;
    uint64_t pitch;
};

struct GridView {
    const uint32_t* lists;
    const uint32_t* counts;
    uint32_t lists_capacity;  // entries in lists
    uint32_t tiles;           // number of tiles (tile grid)
    hl_froxel_params fp;      // froxel grid
};

cudaError_t launch_prep_bin_lights(const void* camera, const void* lights, uint32_t n, bool froxel_margin,
                                   BinLight* out, cudaStream_t stream);
cudaError_t launch_bin_tiles_ref(const void* camera, const BinLight* bl, uint32_t n, uint32_t W, uint32_t H,
                                 uint32_t* lists, uint32_t* counts, cudaStream_t stream);
cudaError_t launch_bin_froxels(const void* camera, const BinLight* bl, uint32_t n, const hl_froxel_params& p,
                               const SliceTable& tab, uint32_t* counts_scratch, uint32_t* offsets,
                               uint32_t* indices, uint32_t capacity, int* status, cudaStream_t stream);

// One view of a batch, as the batched shading kernel reads it (froxel grid).
struct ShadeViewDesc {
    const void* camera;
    GBufView gb;
    GridView grid;
    TargetView out;
    const float* tabz;     // the view's slice boundaries (device memory)
    float4* cand;          // cand_table_len(n_lights) entries: the view's candidate-test light table
    uint32_t tiles_x;      // 32x16 tiles per row
    uint32_t tile_start;   // first CTA of this view in the batched launch
};

// Single-launch froxel binning (count, chained scan, fill) over work items of a
// froxel column's slice group (groups per column from bin_item_groups). chain: one word
// per item and state: both zeroed when allocated; launches sharing them must not
// overlap. stall_item (~0u: none) never publishes its chain word and the look-back
// gives up after stall_spins polls: a failure-injection test of the bounded wait.
struct BinChainState;
uint32_t bin_item_groups(int device, const hl_froxel_params& p);
cudaError_t launch_bin_froxels_items(const void* camera, const void* lights, uint32_t n, const hl_froxel_params& p,
                                     const SliceTable& tab, uint32_t groups, uint32_t* offsets, uint32_t* indices,
                                     uint32_t capacity, int* status, unsigned long long* chain, BinChainState* state,
                                     uint32_t stall_item, uint32_t stall_spins, cudaStream_t stream);

// Froxel binning of every view of a batch (descs: device array of n_views).
cudaError_t launch_bin_froxels_batched(const BinViewDesc* descs, uint32_t n_views, uint32_t total_columns,
                                       const void* lights, uint32_t n, int* status, cudaStream_t stream);

// Shading. layout: HL_GBUF_*, grid_kind: HL_GRID_*, target_format: HL_TARGET_*.
// stats != nullptr selects the pair-statistics variant (no radiance written).
// cand: n_lights float4 of scratch for the candidate-test light table.
// The pass's optional bindings as the extended shading kernel reads them (validated by
// the API layer): shadow maps (dyn == nullptr: none) and radiance-cascade probes
// (rc == nullptr: none).
struct ExtView {
    const float* dyn;            // dynamic atlas, layers x size x size
    const float* sta;            // static atlas
    const float* mats;           // GpuShadowMatrix[layers], 16 floats each, column major
    const unsigned char* cfg;    // ShadowConfig, 80 bytes
    int* status;
    const float* csm;            // DeferredGlobals.csm_splits (device)
    uint32_t size, layers, max_lights;
    float fsize;                 // float(size): the shader's ATLAS_SIZE
    const unsigned char* rc;     // rc_cascade0, RGBA16F
    uint64_t rc_pitch;
};

// Record of the (pixel, light) pairs a shading launch lit: pairs[k] = (y * W + x, light
// index) for k < min(*count, capacity); *count counts every lit pair. pairs == nullptr:
// nothing is recorded (the normal case).
struct PairLog {
    uint2* pairs;
    uint32_t* count;
    uint32_t capacity;
};

// ext != nullptr selects the extended variant (hl_shade_ex, hl_shade_shadowed).
cudaError_t launch_shade(uint32_t layout, uint32_t grid_kind, uint32_t target_format, const void* camera,
                         const void* globals, const GBufView& gb, const void* lights, uint32_t n_lights,
                         const GridView& grid, const SliceTable& tab, const TargetView& out, uint32_t* stats,
                         int* status, float4* cand, const PairLog& log, cudaStream_t stream,
                         const ExtView* ext = nullptr);

// Length in float4 of a candidate-test light table of n lights: n candidate records
// followed by n floats, each light's largest colour channel times its intensity.
constexpr size_t cand_table_len(uint32_t n) { return size_t(n) + (size_t(n) + 3) / 4; }

// The candidate-test light table of the shading kernels: per light its position
// (camera-relative when `relative`) and range^2 (1 + 2^-9), or -1 for a directional
// light. Launched as a dependent launch of its predecessor.
cudaError_t launch_prep_cand(const void* camera, const void* lights, uint32_t n, bool relative, float4* cand,
                             cudaStream_t stream);

// Shading of an FP16 G-buffer over froxel lists (hl_shade's headline form).
cudaError_t launch_shade_f16(uint32_t target_format, const void* camera, const void* globals, const GBufView& gb,
                             const void* lights, uint32_t n_lights, const GridView& grid, const SliceTable& tab,
                             const TargetView& out, int* status, float4* cand, const PairLog& log,
                             cudaStream_t stream);

// The batched form of launch_shade_f16: one launch over every (view, tile) of a batch
// (the views' candidate tables already written).
cudaError_t launch_shade_f16_batched(uint32_t target_format, const ShadeViewDesc* descs, uint32_t n_views,
                                     uint32_t total_tiles, const void* globals, const void* lights, uint32_t n,
                                     int* status, cudaStream_t stream);

// Batched views of an FP16 G-buffer in one persistent launch: froxel binning items of
// every view, then the (view, tile) shading items `tiles` (x: view, y: tile), taken by
// ticket from `state`; `chain` holds one word per binning item, `view_done` one counter
// per view (all zeroed when allocated). grid: batch_persistent_grid (resident CTAs).
size_t batch_persistent_smem();
uint32_t batch_persistent_grid(int device);
cudaError_t launch_batch_persistent(uint32_t target_format, const BinViewDesc* bd, const ShadeViewDesc* sd,
                                    uint32_t n_views, const uint2* tiles, uint32_t total_bin, uint32_t total_tiles,
                                    uint32_t grid, const void* globals, const void* lights, uint32_t n,
                                    unsigned long long* chain, BinChainState* state, uint32_t* view_done,
                                    int* status, cudaStream_t stream);
// The views' candidate-test light tables of a batch (one launch).
cudaError_t launch_prep_cand_batched(const ShadeViewDesc* descs, uint32_t n_views, const void* lights, uint32_t n,
                                     bool relative, cudaStream_t stream);

// Adjoint of shading. partials: grid_size * n_lights * 8 floats of scratch.
uint32_t adjoint_grid_size(int device, uint32_t width, uint32_t height);
cudaError_t launch_shade_adjoint(uint32_t layout, uint32_t grid_kind, const void* camera, const void* globals,
                                 const GBufView& gb, const void* lights, uint32_t n_lights, const GridView& grid,
                                 const SliceTable& tab, const void* d_radiance, uint64_t d_radiance_pitch,
                                 float* partials, uint32_t grid_size, double* d_lights, float* d_pixels, int* status,
                                 cudaStream_t stream);

// Shading of every view of a batch in one launch (total_tiles CTAs).
cudaError_t launch_shade_batched(uint32_t layout, uint32_t target_format, const ShadeViewDesc* descs,
                                 uint32_t n_views, uint32_t total_tiles, const void* globals, const void* lights,
                                 uint32_t n_lights, int* status, cudaStream_t stream);

// Fragment lighting (Forward+ / transparent light loops). light_scratch: n_lights x
// frag_light_bytes().
size_t frag_light_bytes();
cudaError_t launch_shade_fragments(const void* camera, const hl_fragment_params& prm, const void* frags, uint32_t n,
                                   const void* lights, uint32_t n_lights, const uint32_t* entity,
                                   const void* transforms, uint32_t n_xf, uint32_t grid_kind, const GridView& grid,
                                   const SliceTable& tab, void* light_scratch, float* out, int* status,
                                   cudaStream_t stream);

cudaError_t run_fp32_probe(int device, double* tflops);

}  // namespace hl
