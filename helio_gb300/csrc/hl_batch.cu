// hl_batch.cu — batched views (no reference counterpart): one plan lights many views
// (cube-map probe faces, several viewports) against one shared light buffer.
//
// A plan owns, in one set of device buffers, every view's froxel lists and the
// per-view descriptors the batched kernels read. Executing it replays a CUDA graph of
// six launches whatever the number of views: light preparation for binning in every
// view, froxel counts, per-view scans, froxel fills, the shading light tables of every
// view, and one shading launch whose CTAs walk the (view, 32x16 tile) work list.
// Per-view launches of hl_bin_froxels + hl_shade cost six launches per view instead,
// most of them too small to fill the GPU.
//
// Froxel grids are chosen per view size: given in the config, or by the autotuner,
// which builds a one-class plan for each candidate grid of a view size, times its graph
// and keeps the fastest; results can be kept in a text cache file keyed by the view
// size, G-buffer layout, light count and GPU name.
#include <algorithm>
#include <array>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "hl_common.cuh"
#include "hl_host.h"
#include "hl_internal.h"
#include "hl_bin_item.cuh"

using namespace hl_host;

struct hl_batch_plan {
    int device = 0;
    int* d_status = nullptr;  // the creating context's status word
    uint32_t n_views = 0, n_lights = 0, layout = 0, target_format = 0;
    uint32_t total_cols = 0, total_tiles = 0;
    std::vector<uint32_t> grid;  // 3 per view
    hl::BinViewDesc* d_bin = nullptr;
    hl::ShadeViewDesc* d_shade = nullptr;
    hl::BinLight* bl = nullptr;
    float4* cand = nullptr;
    uint32_t* counts = nullptr;
    uint32_t* offsets = nullptr;
    uint32_t* indices = nullptr;
    cudaStream_t capture_stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    // the persistent form (FP16 G-buffers): binning and shading items in one launch
    bool persistent = false;
    uint32_t total_bin = 0, grid_ctas = 0;
    uint2* tiles = nullptr;                 // work list: (view, binning item), then (view, tile)
    unsigned long long* chain = nullptr;    // one word per binning item
    hl::BinChainState* state = nullptr;     // ticket counter and epoch
    uint32_t* view_done = nullptr;          // binning items finished per view, over all launches
};

namespace {

constexpr float kFroxelNear = 0.5f;  // prelude.wgsl:195

struct HostView {
    const void* camera;
    hl::GBufView gb;
    hl::TargetView out;
    float far_plane;
};

void free_plan(hl_batch_plan* p) {
    if (!p) return;
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    if (p->capture_stream) cudaStreamDestroy(p->capture_stream);
    cudaFree(p->d_bin);
    cudaFree(p->d_shade);
    cudaFree(p->bl);
    cudaFree(p->cand);
    cudaFree(p->counts);
    cudaFree(p->offsets);
    cudaFree(p->indices);
    cudaFree(p->tiles);
    cudaFree(p->chain);
    cudaFree(p->state);
    cudaFree(p->view_done);
    delete p;
}

hl_froxel_params params_for(const HostView& v, const uint32_t* g) {
    hl_froxel_params p{};
    p.grid_x = g[0];
    p.grid_y = g[1];
    p.grid_z = g[2];
    p.width = v.gb.width;
    p.height = v.gb.height;
    p.slice_near = kFroxelNear;
    p.slice_far = v.far_plane;
    p.reserved = 0;
    return p;
}

// One execution of a plan's work: the persistent form (candidate tables, then one launch
// of binning and shading items) or six launches (light preparation, froxel counts,
// scans, fills, candidate tables, shading).
cudaError_t record_plan(hl_batch_plan* p, const void* lights, const void* globals, cudaStream_t st) {
    if (p->persistent) {
        cudaError_t e = hl::launch_prep_cand_batched(p->d_shade, p->n_views, lights, p->n_lights, true, st);
        if (e != cudaSuccess) return e;
        return hl::launch_batch_persistent(p->target_format, p->d_bin, p->d_shade, p->n_views, p->tiles, p->total_bin,
                                           p->total_tiles, p->grid_ctas, globals, lights, p->n_lights, p->chain,
                                           p->state, p->view_done, p->d_status, st);
    }
    cudaError_t e = hl::launch_bin_froxels_batched(p->d_bin, p->n_views, p->total_cols, lights, p->n_lights, p->d_status, st);
    if (e != cudaSuccess) return e;
    return hl::launch_shade_batched(p->layout, p->target_format, p->d_shade, p->n_views, p->total_tiles, globals,
                                    lights, p->n_lights, p->d_status, st);
}

// Builds a plan over `views` with grids `grid` (3 per view): buffers, descriptors,
// one uncaptured binning pass to size the froxel index buffers, then the graph.
hl_status build_plan(hl_ctx* ctx, const std::vector<HostView>& views, const std::vector<uint32_t>& grid,
                     const void* lights, uint32_t n_lights, const void* globals, uint32_t layout, uint32_t target,
                     hl_batch_plan** out) {
    const uint32_t V = uint32_t(views.size());
    hl_batch_plan* p = new hl_batch_plan();
    p->device = ctx->device;
    p->d_status = ctx->d_status;
    p->n_views = V;
    p->n_lights = n_lights;
    p->layout = layout;
    p->target_format = target;
    p->grid = grid;
    std::vector<hl::BinViewDesc> bd(V);
    std::vector<hl::ShadeViewDesc> sd(V);
    std::vector<uint64_t> f_base(V + 1, 0), o_base(V + 1, 0);
    uint64_t cols = 0, tiles = 0;
    for (uint32_t v = 0; v < V; ++v) {
        const hl_froxel_params fp = params_for(views[v], &grid[3 * v]);
        hl_status s = check_froxel_params(ctx, &fp);
        if (s != HL_OK) {
            free_plan(p);
            return s;
        }
        const uint64_t F = uint64_t(fp.grid_x) * fp.grid_y * fp.grid_z;
        f_base[v + 1] = f_base[v] + F;
        // every view's offsets and indices start on a 128-byte line of their own: no line
        // holds two views' lists (the persistent launch reads a view's lists through L1
        // once that view's binning has finished, while other views are still binned)
        o_base[v + 1] = o_base[v] + ((F + 1 + 31) & ~31ull);
        std::memset(&bd[v], 0, sizeof bd[v]);
        bd[v].camera = views[v].camera;
        bd[v].p = fp;
        bd[v].col_start = uint32_t(cols);
        slice_table(fp, bd[v].tab.z);
        cols += uint64_t(fp.grid_x) * fp.grid_y;
        sd[v].camera = views[v].camera;
        sd[v].gb = views[v].gb;
        sd[v].out = views[v].out;
        sd[v].tiles_x = (views[v].gb.width + 31) / 32;
        sd[v].tile_start = uint32_t(tiles);
        tiles += uint64_t(sd[v].tiles_x) * ((views[v].gb.height + 15) / 16);
    }
    if (cols > 0x7FFFFFFFull || tiles > 0x7FFFFFFFull || o_base[V] > 0xFFFFFFFFull) {
        free_plan(p);
        return fail(ctx, HL_ERR_SIZE, "batch of %u views is too large (%llu columns, %llu tiles)", V,
                    (unsigned long long)cols, (unsigned long long)tiles);
    }
    p->total_cols = uint32_t(cols);
    p->total_tiles = uint32_t(tiles);
    cudaError_t e = cudaMalloc(&p->d_bin, sizeof(hl::BinViewDesc) * V);
    if (e == cudaSuccess) e = cudaMalloc(&p->d_shade, sizeof(hl::ShadeViewDesc) * V);
    if (e == cudaSuccess) e = cudaMalloc(&p->bl, sizeof(hl::BinLight) * size_t(V) * std::max(n_lights, 1u));
    if (e == cudaSuccess) e = cudaMalloc(&p->cand, sizeof(float4) * size_t(V) * hl::cand_table_len(std::max(n_lights, 1u)));
    if (e == cudaSuccess) e = cudaMalloc(&p->counts, sizeof(uint32_t) * std::max<uint64_t>(f_base[V], 1));
    if (e == cudaSuccess) e = cudaMalloc(&p->offsets, sizeof(uint32_t) * o_base[V]);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->capture_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        free_plan(p);
        return cuda_fail(ctx, e, "batch plan buffers");
    }
    for (uint32_t v = 0; v < V; ++v) {
        bd[v].bl = p->bl + size_t(v) * n_lights;
        bd[v].counts = p->counts + f_base[v];
        bd[v].offsets = p->offsets + o_base[v];
        bd[v].indices = nullptr;
        bd[v].capacity = 0;
    }
    // sizing pass: counts and offsets only (capacity 0 writes no index)
    cudaStream_t st = p->capture_stream;
    e = cudaMemcpyAsync(p->d_bin, bd.data(), sizeof(hl::BinViewDesc) * V, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = hl::launch_bin_froxels_batched(p->d_bin, V, p->total_cols, lights, n_lights, nullptr, st);
    std::vector<uint32_t> totals(V, 0);
    for (uint32_t v = 0; v < V && e == cudaSuccess; ++v) {
        const hl_froxel_params& fp = bd[v].p;
        const uint64_t F = uint64_t(fp.grid_x) * fp.grid_y * fp.grid_z;
        e = cudaMemcpyAsync(&totals[v], bd[v].offsets + F, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        free_plan(p);
        return cuda_fail(ctx, e, "batch plan sizing pass");
    }
    // index capacity: twice the lists at creation, so lights may move between executions
    std::vector<uint64_t> i_base(V + 1, 0);
    for (uint32_t v = 0; v < V; ++v) {
        const uint64_t cap = std::max<uint64_t>(1024, 2ull * totals[v]);
        i_base[v + 1] = i_base[v] + ((cap + 31) & ~31ull);
    }
    if (i_base[V] > 0xFFFFFFFFull) {
        free_plan(p);
        return fail(ctx, HL_ERR_SIZE, "batch froxel lists need %llu entries", (unsigned long long)i_base[V]);
    }
    e = cudaMalloc(&p->indices, sizeof(uint32_t) * i_base[V]);
    if (e != cudaSuccess) {
        free_plan(p);
        return cuda_fail(ctx, e, "batch froxel index buffer");
    }
    // the persistent form: binning items per view (slice groups only when the batch has
    // too few columns to fill the GPU) and the shading work list, heaviest views first
    std::vector<uint2> work;
    if (layout == HL_GBUF_F16) {
        int sms = 1;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device) != cudaSuccess || sms <= 0) sms = 1;
        std::vector<uint32_t> order(V);
        for (uint32_t v = 0; v < V; ++v) order[v] = v;
        // list entries per froxel column: the mean length of a view's pixel lists, up to the slice count
        std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
            const double ca = double(totals[a]) / (double(bd[a].p.grid_x) * bd[a].p.grid_y);
            const double cb = double(totals[b]) / (double(bd[b].p.grid_x) * bd[b].p.grid_y);
            return ca > cb;
        });
        // the views' binning items in the same order as their shading items, so that the
        // first shading items find their view's lists finished earliest
        uint64_t items = 0;
        for (uint32_t v : order) {
            bd[v].groups = p->total_cols >= 2u * uint32_t(sms) ? 1u : hl::bin::item_groups(bd[v].p, 2u * uint32_t(sms));
            bd[v].item_start = uint32_t(items);
            const uint32_t n_items = bd[v].p.grid_x * bd[v].p.grid_y * bd[v].groups;
            for (uint32_t k = 0; k < n_items; ++k) work.push_back(make_uint2(v, k));
            items += n_items;
        }
        for (uint32_t v : order) {
            const uint32_t nt = sd[v].tiles_x * ((views[v].gb.height + 15) / 16);
            for (uint32_t t = 0; t < nt; ++t) work.push_back(make_uint2(v, t));
        }
        if (work.size() > 0x7FFFFFFFull) {
            free_plan(p);
            return fail(ctx, HL_ERR_SIZE, "batch has %llu work items", (unsigned long long)work.size());
        }
        p->persistent = true;
        p->total_bin = uint32_t(items);
        p->grid_ctas = std::min<uint32_t>(hl::batch_persistent_grid(p->device), uint32_t(work.size()));
        e = cudaMalloc(&p->tiles, sizeof(uint2) * std::max<size_t>(work.size(), 1));
        if (e == cudaSuccess) e = cudaMalloc(&p->chain, sizeof(unsigned long long) * std::max<uint64_t>(items, 1));
        if (e == cudaSuccess) e = cudaMalloc(&p->state, sizeof(hl::BinChainState));
        if (e == cudaSuccess) e = cudaMalloc(&p->view_done, sizeof(uint32_t) * V);
        if (e == cudaSuccess) e = cudaMemsetAsync(p->chain, 0, sizeof(unsigned long long) * std::max<uint64_t>(items, 1), st);
        if (e == cudaSuccess) e = cudaMemsetAsync(p->state, 0, sizeof(hl::BinChainState), st);
        if (e == cudaSuccess) e = cudaMemsetAsync(p->view_done, 0, sizeof(uint32_t) * V, st);
        if (e == cudaSuccess && !work.empty())
            e = cudaMemcpyAsync(p->tiles, work.data(), sizeof(uint2) * work.size(), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // `work` is a host temporary
        if (e != cudaSuccess) {
            free_plan(p);
            return cuda_fail(ctx, e, "batch plan work list");
        }
    }
    for (uint32_t v = 0; v < V; ++v) {
        bd[v].indices = p->indices + i_base[v];
        bd[v].capacity = uint32_t(i_base[v + 1] - i_base[v]);
        hl::GridView g{};
        g.lists = bd[v].indices;
        g.counts = bd[v].offsets;
        g.lists_capacity = bd[v].capacity;
        g.tiles = 0;
        g.fp = bd[v].p;
        sd[v].grid = g;
        sd[v].cand = p->cand + size_t(v) * hl::cand_table_len(n_lights);
        sd[v].tabz = reinterpret_cast<const float*>(reinterpret_cast<const unsigned char*>(p->d_bin + v) +
                                                    offsetof(hl::BinViewDesc, tab));
    }
    e = cudaMemcpyAsync(p->d_bin, bd.data(), sizeof(hl::BinViewDesc) * V, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(p->d_shade, sd.data(), sizeof(hl::ShadeViewDesc) * V, cudaMemcpyHostToDevice, st);
    // one uncaptured run (sets kernel attributes and checks the launches), then the graph
    if (e == cudaSuccess) e = record_plan(p, lights, globals, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaError_t e1 = record_plan(p, lights, globals, st);
        e = cudaStreamEndCapture(st, &p->graph);
        if (e == cudaSuccess) e = e1;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&p->exec, p->graph, 0);
    if (e != cudaSuccess) {
        cudaGetLastError();
        free_plan(p);
        return cuda_fail(ctx, e, "batch plan graph");
    }
    *out = p;
    return HL_OK;
}

// Median device time of `reps` replays of a plan's graph (after two warm-up replays).
float time_plan(hl_batch_plan* p, int reps) {
    cudaStream_t st = p->capture_stream;
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess) return 1e30f;
    if (cudaEventCreate(&b) != cudaSuccess) {
        cudaEventDestroy(a);
        return 1e30f;
    }
    std::vector<float> ms;
    bool ok = true;
    for (int i = 0; i < reps + 2 && ok; ++i) {
        ok = cudaEventRecord(a, st) == cudaSuccess && cudaGraphLaunch(p->exec, st) == cudaSuccess &&
             cudaEventRecord(b, st) == cudaSuccess && cudaEventSynchronize(b) == cudaSuccess;
        float t = 0.0f;
        if (ok && cudaEventElapsedTime(&t, a, b) == cudaSuccess && i >= 2) ms.push_back(t);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (!ok || ms.empty()) return 1e30f;
    std::sort(ms.begin(), ms.end());
    return ms[ms.size() / 2];
}

// Candidate froxel grids of a W x H view: columns of 32, 64 or 128 pixels, 16/24/32 slices.
std::vector<std::array<uint32_t, 3>> candidates(uint32_t W, uint32_t H) {
    std::vector<std::array<uint32_t, 3>> c;
    for (uint32_t px : {32u, 64u, 128u})
        for (uint32_t gz : {16u, 24u, 32u}) {
            const uint32_t gx = std::max(1u, std::min(W, (W + px - 1) / px));
            const uint32_t gy = std::max(1u, std::min(H, (H + px - 1) / px));
            c.push_back({gx, gy, gz});
        }
    return c;
}

using ClassKey = std::tuple<uint32_t, uint32_t>;  // view width, height

std::string cache_key(uint32_t W, uint32_t H, uint32_t layout, uint32_t n_lights, const char* gpu) {
    std::string g(gpu);
    for (char& ch : g)
        if (ch == ' ') ch = '_';
    char buf[256];
    std::snprintf(buf, sizeof buf, "%u %u %u %u %s", W, H, layout, n_lights, g.c_str());
    return buf;
}

std::map<std::string, std::array<uint32_t, 3>> read_cache(const char* path) {
    std::map<std::string, std::array<uint32_t, 3>> m;
    if (!path) return m;
    FILE* f = std::fopen(path, "r");
    if (!f) return m;
    char line[512];
    while (std::fgets(line, sizeof line, f)) {
        unsigned w, h, l, n, gx, gy, gz;
        char gpu[256];
        if (std::sscanf(line, "%u %u %u %u %255s %u %u %u", &w, &h, &l, &n, gpu, &gx, &gy, &gz) == 8)
            m[cache_key(w, h, l, n, gpu)] = {gx, gy, gz};
    }
    std::fclose(f);
    return m;
}

void write_cache(const char* path, const std::map<std::string, std::array<uint32_t, 3>>& m) {
    if (!path) return;
    FILE* f = std::fopen(path, "w");
    if (!f) return;
    std::fprintf(f, "# helio-gb300 batch autotuner: width height layout n_lights gpu -> grid_x grid_y grid_z\n");
    for (const auto& kv : m) std::fprintf(f, "%s %u %u %u\n", kv.first.c_str(), kv.second[0], kv.second[1], kv.second[2]);
    std::fclose(f);
}

}  // namespace

extern "C" {

hl_status hl_batch_plan_create(hl_ctx* ctx, const hl_view* views, uint32_t n_views, const void* lights,
                               uint32_t n_lights, const void* globals, const hl_batch_config* config,
                               hl_batch_plan** out_plan, void* stream) {
    if (out_plan) *out_plan = nullptr;
    if (!ctx) return HL_ERR_INVALID_ARGUMENT;
    if (!out_plan || !views || !config) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "batch: NULL views/config/out_plan");
    if (n_views == 0 || n_views > 65536) return fail(ctx, HL_ERR_SIZE, "batch: %u views (1..65536)", n_views);
    hl_status s = check_common(ctx, views[0].camera, lights, n_lights);
    if (s != HL_OK) return s;
    if (!globals || !aligned(globals, 16)) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "globals is NULL or misaligned");
    if (config->autotune == 0 && (config->grid_x == 0 || config->grid_y == 0 || config->grid_z == 0))
        return fail(ctx, HL_ERR_INVALID_ARGUMENT, "batch: grid %ux%ux%u without autotune", config->grid_x,
                    config->grid_y, config->grid_z);
    std::vector<HostView> hv(n_views);
    const uint32_t layout = views[0].gbuffer.layout, target = views[0].radiance.format;
    for (uint32_t v = 0; v < n_views; ++v) {
        if (!views[v].camera || !aligned(views[v].camera, 16))
            return fail(ctx, HL_ERR_INVALID_ARGUMENT, "batch view %u: camera NULL or misaligned", v);
        if ((s = check_gbuffer(ctx, &views[v].gbuffer, hv[v].gb)) != HL_OK) return s;
        if ((s = check_target(ctx, &views[v].radiance, views[v].gbuffer.width, hv[v].out)) != HL_OK) return s;
        if (views[v].gbuffer.layout != layout || views[v].radiance.format != target)
            return fail(ctx, HL_ERR_NOT_SUPPORTED, "batch view %u: every view needs the same layout and target format",
                        v);
        hv[v].camera = views[v].camera;
    }
    DeviceGuard dg(ctx->device);
    if (!dg.ok) return fail(ctx, HL_ERR_CUDA, "cudaSetDevice(%d) failed", ctx->device);
    // far planes of the views (the froxel slices end there)
    cudaStream_t st = as_stream(stream);
    std::vector<hl::GpuCamera> cams(n_views);
    cudaError_t e = cudaSuccess;
    for (uint32_t v = 0; v < n_views && e == cudaSuccess; ++v)
        e = cudaMemcpyAsync(&cams[v], views[v].camera, sizeof(hl::GpuCamera), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "batch: camera readback");
    for (uint32_t v = 0; v < n_views; ++v) hv[v].far_plane = cams[v].forward_far[3];

    std::vector<uint32_t> grid(3 * size_t(n_views));
    if (!config->autotune) {
        for (uint32_t v = 0; v < n_views; ++v) {
            grid[3 * v + 0] = std::min(config->grid_x, hv[v].gb.width);
            grid[3 * v + 1] = std::min(config->grid_y, hv[v].gb.height);
            grid[3 * v + 2] = config->grid_z;
        }
    } else {
        cudaDeviceProp prop{};
        if ((e = cudaGetDeviceProperties(&prop, ctx->device)) != cudaSuccess) return cuda_fail(ctx, e, "device name");
        auto cache = read_cache(config->cache_path);
        bool dirty = false;
        std::map<ClassKey, std::vector<uint32_t>> classes;
        for (uint32_t v = 0; v < n_views; ++v) classes[ClassKey(hv[v].gb.width, hv[v].gb.height)].push_back(v);
        for (const auto& kv : classes) {
            const uint32_t W = std::get<0>(kv.first), H = std::get<1>(kv.first);
            const std::string key = cache_key(W, H, layout, n_lights, prop.name);
            std::array<uint32_t, 3> best{};
            auto it = cache.find(key);
            if (it != cache.end()) {
                best = it->second;
            } else {
                std::vector<HostView> sub;
                for (uint32_t v : kv.second) sub.push_back(hv[v]);
                float best_ms = 1e30f;
                for (const auto& c : candidates(W, H)) {
                    std::vector<uint32_t> g;
                    for (size_t i = 0; i < sub.size(); ++i) g.insert(g.end(), c.begin(), c.end());
                    hl_batch_plan* trial = nullptr;
                    if (build_plan(ctx, sub, g, lights, n_lights, globals, layout, target, &trial) != HL_OK) continue;
                    const float ms = time_plan(trial, 5);
                    free_plan(trial);
                    if (ms < best_ms) {
                        best_ms = ms;
                        best = c;
                    }
                }
                if (best_ms >= 1e30f) return fail(ctx, HL_ERR_CUDA, "batch autotune: no candidate ran for %ux%u", W, H);
                cache[key] = best;
                dirty = true;
            }
            for (uint32_t v : kv.second) std::copy(best.begin(), best.end(), grid.begin() + 3 * v);
        }
        if (dirty) write_cache(config->cache_path, cache);
    }
    return build_plan(ctx, hv, grid, lights, n_lights, globals, layout, target, out_plan);
}

hl_status hl_batch_execute(hl_ctx* ctx, hl_batch_plan* plan, void* stream) {
    if (!ctx || !plan) return HL_ERR_INVALID_ARGUMENT;
    if (plan->device != ctx->device) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "plan belongs to another device");
    DeviceGuard dg(ctx->device);
    if (!dg.ok) return fail(ctx, HL_ERR_CUDA, "cudaSetDevice(%d) failed", ctx->device);
    const cudaError_t e = cudaGraphLaunch(plan->exec, as_stream(stream));
    return e == cudaSuccess ? HL_OK : cuda_fail(ctx, e, "batch graph launch");
}

hl_status hl_batch_plan_view_grid(const hl_batch_plan* plan, uint32_t view, uint32_t* grid_xyz) {
    if (!plan || !grid_xyz || view >= plan->n_views) return HL_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < 3; ++i) grid_xyz[i] = plan->grid[3 * size_t(view) + i];
    return HL_OK;
}

hl_status hl_batch_plan_destroy(hl_batch_plan* plan) {
    if (!plan) return HL_OK;
    DeviceGuard dg(plan->device);
    cudaStreamSynchronize(plan->capture_stream);
    free_plan(plan);
    return HL_OK;
}

}  // extern "C"
