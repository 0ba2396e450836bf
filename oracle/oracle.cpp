// oracle.cpp — CPU restatement of Helio's deferred-lighting hot path.
//
// TEST INFRASTRUCTURE ONLY. This file is the checker for the CUDA library in
// helio_gb300/: only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline /
// reference legs load it. The product never links or calls it.
//
// Parity status: UNPINNED against the reference's own execution. The reference is
// WGSL run by wgpu 30 / naga 30 on a graphics driver; there is no graphics stack and
// no Rust toolchain on these machines, and the reference's tests pin no lighting
// value (helio-pass-deferred-light/tests/*.rs assert only struct sizes and
// constants; helio-pass-light-cull has no tests). This restatement is pinned instead
// by (a) the reference's layout constants, (b) closed-form known-answer cases and
// (c) golden vectors from an independent multi-precision Python restatement
// (tests/golden/make_golden.py).
//
// Everything is templated on the arithmetic type T:
//   T = double : the accuracy oracle for radiance and gradients.
//   T = float  : compiled with -ffp-contract=off, the bit-exact oracle for the light
//                lists (the CUDA binning kernels use the same f32 operation order with
//                correctly rounded __f*_rn operations) and the timed CPU baseline.
//
// Declared f32 operation order (shared with the CUDA kernels):
//   dot(a,b)        = (a.x*b.x + a.y*b.y) + a.z*b.z
//   normalize(v)    = v / sqrt(dot(v,v)), one division per component
//   cross(a,b)      = (a.y*b.z - a.z*b.y, a.z*b.x - a.x*b.z, a.x*b.y - a.y*b.x)
//   M*(x,y,z,1)[r]  = ((M[0][r]*x + M[1][r]*y) + M[2][r]*z) + M[3][r]   (column major)

#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>
#include <vector>
#include <limits>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "rc_gi.h"
#include "shadow_factor.h"

namespace {

// ----------------------------------------------------------------------------------
// Byte layouts (libhelio/src/light.rs:60-115, libhelio/src/camera.rs:12-29,
// helio-pass-deferred-light/src/lib.rs:17-52)
// ----------------------------------------------------------------------------------
constexpr int kLightFloats = 32;   // 128 B
constexpr int kCameraFloats = 92;  // 368 B
constexpr uint32_t kTile = 16;     // light_cull.wgsl:17
constexpr uint32_t kMaxPerTile = 64;  // light_cull.wgsl:18

struct RawLight {
    float pos[3], range;
    float dir[3], cos_outer;
    float color[3], intensity;
    uint32_t shadow_index, type;
    float cos_inner;
    uint32_t pad;
    float god_rays[5];
    float flare[7];
    int32_t ies_profile, light_function;
    float ies_scale, ies_offset;
};
static_assert(sizeof(RawLight) == 128, "GpuLight is 128 bytes (light.rs:111)");

struct RawCamera {
    float view[16], proj[16], view_proj[16], inv_view_proj[16];
    float position_near[4], forward_far[4], jitter_frame[4], prev_view_proj[16];
};
static_assert(sizeof(RawCamera) == 368, "GpuCameraUniforms is 368 bytes");

struct RawGlobals {
    uint32_t frame;
    float delta_time;
    uint32_t light_count;
    float ambient_intensity;
    float ambient_color[4];
    float rc_world_min[4], rc_world_max[4], csm_splits[4];
    uint32_t debug_mode, has_rc_gi, num_tiles_x, reflection_capture_count;
    uint32_t enable_reflections, enable_env_reflections, pad[2];
};
static_assert(sizeof(RawGlobals) == 112, "DeferredGlobals is 112 bytes");

template <class T> struct V3 {
    T x, y, z;
};
template <class T> inline V3<T> v3(T x, T y, T z) { return V3<T>{x, y, z}; }
template <class T> inline V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline V3<T> operator*(V3<T> a, V3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> inline V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> inline V3<T> operator/(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> inline T dot(V3<T> a, V3<T> b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
template <class T> inline V3<T> cross(V3<T> a, V3<T> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T> inline T tsqrt(T x) { return std::sqrt(x); }
template <class T> inline V3<T> normalize(V3<T> v) { return v / tsqrt(dot(v, v)); }
template <class T> inline T tmin(T a, T b) { return b < a ? b : a; }
template <class T> inline T tmax(T a, T b) { return a < b ? b : a; }
template <class T> inline T clampt(T x, T lo, T hi) { return tmin(tmax(x, lo), hi); }
// WGSL mix(e1,e2,e3) = e1*(1-e3) + e2*e3
template <class T> inline T mixt(T a, T b, T t) { return a * (T(1) - t) + b * t; }
// WGSL smoothstep(low, high, x): t = clamp((x-low)/(high-low), 0, 1); t*t*(3-2t)
template <class T> inline T smoothstept(T lo, T hi, T x) {
    T t = clampt((x - lo) / (hi - lo), T(0), T(1));
    return t * t * (T(3) - T(2) * t);
}

// Column-major 4x4 times (x,y,z,w) in the declared order; returns the 4 rows.
template <class T> inline void mat4_mul(const T* m, T x, T y, T z, T w, T out[4]) {
    for (int r = 0; r < 4; ++r) out[r] = ((m[0 + r] * x + m[4 + r] * y) + m[8 + r] * z) + m[12 + r] * w;
}

template <class T> struct Cam {
    T view[16], proj[16], inv_view_proj[16];
    V3<T> pos;
    T near_, far_;
};
template <class T> Cam<T> load_camera(const void* bytes) {
    RawCamera rc;
    std::memcpy(&rc, bytes, sizeof rc);
    Cam<T> c;
    for (int i = 0; i < 16; ++i) {
        c.view[i] = T(rc.view[i]);
        c.proj[i] = T(rc.proj[i]);
        c.inv_view_proj[i] = T(rc.inv_view_proj[i]);
    }
    c.pos = v3<T>(rc.position_near[0], rc.position_near[1], rc.position_near[2]);
    c.near_ = rc.position_near[3];
    c.far_ = rc.forward_far[3];
    return c;
}

inline RawLight load_light(const void* lights, uint32_t i) {
    RawLight l;
    std::memcpy(&l, static_cast<const unsigned char*>(lights) + size_t(i) * 128, 128);
    return l;
}

// ----------------------------------------------------------------------------------
// Reference tile culling — light_cull.wgsl:85-180
// ----------------------------------------------------------------------------------

// make_plane_from_ndc_edge (light_cull.wgsl:85-100); d = 0 is implicit.
template <class T> V3<T> plane_from_ndc_edge(const Cam<T>& c, T p0x, T p0y, T p1x, T p1y) {
    // proj[0][0] is float 0 of the proj block, proj[1][1] is float 5.
    V3<T> r0 = normalize(v3<T>(p0x / c.proj[0], p0y / c.proj[5], T(-1)));
    V3<T> r1 = normalize(v3<T>(p1x / c.proj[0], p1y / c.proj[5], T(-1)));
    return normalize(cross(r0, r1));
}

template <class T> struct TilePlanes {
    V3<T> n[4];
};

// Tile NDC rectangle and planes (light_cull.wgsl:131-151).
template <class T>
TilePlanes<T> tile_planes(const Cam<T>& c, uint32_t tx, uint32_t ty, uint32_t W, uint32_t H) {
    const T fw = T(W), fh = T(H), ts = T(kTile);
    T left = (T(tx) * ts / fw) * T(2) - T(1);
    T right = tmin((T(tx + 1) * ts / fw) * T(2) - T(1), T(1));
    T top = T(1) - (T(ty) * ts / fh) * T(2);
    T bottom = tmax(T(1) - (T(ty + 1) * ts / fh) * T(2), T(-1));
    TilePlanes<T> p;
    p.n[0] = plane_from_ndc_edge(c, left, bottom, left, top);     // left
    p.n[1] = plane_from_ndc_edge(c, right, top, right, bottom);   // right
    p.n[2] = plane_from_ndc_edge(c, left, top, right, top);       // top
    p.n[3] = plane_from_ndc_edge(c, right, bottom, left, bottom); // bottom
    return p;
}

template <class T> V3<T> light_view_pos(const Cam<T>& c, const RawLight& l) {
    T o[4];
    mat4_mul(c.view, T(l.pos[0]), T(l.pos[1]), T(l.pos[2]), T(1), o);
    return v3<T>(o[0], o[1], o[2]);
}

// sphere_inside_tile_frustum (light_cull.wgsl:105-117): plane w is 0.
template <class T> bool sphere_in_planes(const V3<T>* n, V3<T> c, T r) {
    for (int i = 0; i < 4; ++i) {
        T dist = dot(n[i], c) + T(0);
        if (dist < -r) return false;
    }
    return true;
}

template <class T>
void bin_tiles_ref_impl(const void* camera, const void* lights, uint32_t n, uint32_t W, uint32_t H,
                        uint32_t* lists, uint32_t* counts) {
    const uint32_t tiles_x = (W + kTile - 1) / kTile, tiles_y = (H + kTile - 1) / kTile;
    const uint32_t tiles = tiles_x * tiles_y;
    if (n == 0) {  // LightCullPass::execute clears both buffers (light-cull/src/lib.rs:285-292)
        std::memset(lists, 0, size_t(tiles) * kMaxPerTile * 4);
        std::memset(counts, 0, size_t(tiles) * 4);
        return;
    }
    Cam<T> c = load_camera<T>(camera);
    std::vector<RawLight> L(n);
    std::vector<V3<T>> pv(n);
    for (uint32_t i = 0; i < n; ++i) {
        L[i] = load_light(lights, i);
        pv[i] = light_view_pos(c, L[i]);
    }
#pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < int64_t(tiles); ++t) {
        uint32_t tx = uint32_t(t) % tiles_x, ty = uint32_t(t) / tiles_x;
        TilePlanes<T> p = tile_planes(c, tx, ty, W, H);
        uint32_t count = 0;
        for (uint32_t i = 0; i < n; ++i) {
            if (L[i].type == 0u) {
                if (count < kMaxPerTile) lists[size_t(t) * kMaxPerTile + count++] = i;
                continue;
            }
            if (sphere_in_planes(p.n, pv[i], T(L[i].range))) {
                if (count < kMaxPerTile) lists[size_t(t) * kMaxPerTile + count++] = i;
            }
        }
        counts[t] = count;
    }
}

// ----------------------------------------------------------------------------------
// Froxel clustering (new capability; slice convention of prelude.wgsl:185-211)
//
// A light is listed in froxel (fx,fy,s) when it is directional, or when all of:
//   (1) its margin sphere is not outside any of the 4 lateral planes of the froxel
//       column (planes built exactly like the reference tile planes, from the NDC
//       edges of the column's pixel range);
//   (2) its margin sphere meets the column's view-space box for slice s, widened by
//       2^-10 of the slice's far depth (+2^-12);
//   (3) for a spot with 0 < cos_outer < cos_inner: its outer cone (margin range)
//       meets the bounding sphere of that box.
// Margin radius rm = r + (r + 1)*2^-10. All in the declared f32 order.
// ----------------------------------------------------------------------------------
struct FroxelParams {
    uint32_t gx, gy, gz, W, H;
    float slice_near, slice_far;
    uint32_t reserved;
};
static_assert(sizeof(FroxelParams) == 32, "hl_froxel_params is 32 bytes");

void slice_table(const FroxelParams& p, float* out) {
    const double nr = double(p.slice_near);
    const double F = std::max(double(p.slice_far), 2.0 * nr);
    out[0] = 0.0f;
    for (uint32_t k = 1; k < p.gz; ++k) out[k] = float(nr * std::pow(F / nr, double(k) / double(p.gz)));
    out[p.gz] = float(F);
}

inline uint32_t ceil_div_u64(uint64_t a, uint64_t b) { return uint32_t((a + b - 1) / b); }

template <class T> struct LightPrep {
    V3<T> c;     // view-space position
    T rm;        // margin radius
    uint32_t type;
    V3<T> axis;  // view-space unit direction (spots)
    T cos_o, sin_o;
    bool cone;   // cone test applies
};

template <class T> LightPrep<T> prep_light(const Cam<T>& c, const RawLight& l) {
    LightPrep<T> p;
    p.c = light_view_pos(c, l);
    const T r = T(l.range);
    p.rm = r + (r + T(1)) * T(1.0 / 1024.0);
    p.type = l.type;
    T d[4];
    mat4_mul(c.view, T(l.dir[0]), T(l.dir[1]), T(l.dir[2]), T(0), d);
    p.axis = normalize(v3<T>(d[0], d[1], d[2]));
    p.cos_o = T(l.cos_outer);
    p.sin_o = tsqrt(tmax(T(1) - p.cos_o * p.cos_o, T(0)));
    p.cone = (l.type == 2u) && (T(0) < p.cos_o) && (p.cos_o < T(l.cos_inner));
    return p;
}

template <class T> struct FroxelBox {
    V3<T> lo, hi, center;
    T radius;
};

// Column (fx,fy): pixel ranges [px0,px1) x [py0,py1).
template <class T> struct Column {
    V3<T> n[4];
    T kx0, kx1, ky_bot, ky_top;  // ndc/proj scale factors: view x = k*depth
};

template <class T>
Column<T> froxel_column(const Cam<T>& c, const FroxelParams& p, uint32_t fx, uint32_t fy) {
    const uint32_t px0 = ceil_div_u64(uint64_t(fx) * p.W, p.gx);
    const uint32_t px1 = ceil_div_u64(uint64_t(fx + 1) * p.W, p.gx);
    const uint32_t py0 = ceil_div_u64(uint64_t(fy) * p.H, p.gy);
    const uint32_t py1 = ceil_div_u64(uint64_t(fy + 1) * p.H, p.gy);
    const T fw = T(p.W), fh = T(p.H);
    T left = (T(px0) / fw) * T(2) - T(1);
    T right = (T(px1) / fw) * T(2) - T(1);
    T top = T(1) - (T(py0) / fh) * T(2);
    T bottom = T(1) - (T(py1) / fh) * T(2);
    Column<T> col;
    col.n[0] = plane_from_ndc_edge(c, left, bottom, left, top);
    col.n[1] = plane_from_ndc_edge(c, right, top, right, bottom);
    col.n[2] = plane_from_ndc_edge(c, left, top, right, top);
    col.n[3] = plane_from_ndc_edge(c, right, bottom, left, bottom);
    col.kx0 = left / c.proj[0];
    col.kx1 = right / c.proj[0];
    col.ky_bot = bottom / c.proj[5];
    col.ky_top = top / c.proj[5];
    return col;
}

template <class T>
FroxelBox<T> froxel_box(const Column<T>& col, T z0, T z1) {
    FroxelBox<T> b;
    const T m = z1 * T(1.0 / 1024.0) + T(1.0 / 4096.0);
    b.lo.x = tmin(col.kx0 * z0, col.kx0 * z1) - m;
    b.hi.x = tmax(col.kx1 * z0, col.kx1 * z1) + m;
    b.lo.y = tmin(col.ky_bot * z0, col.ky_bot * z1) - m;
    b.hi.y = tmax(col.ky_top * z0, col.ky_top * z1) + m;
    b.lo.z = -z1 - m;
    b.hi.z = -z0 + m;
    b.center = (b.lo + b.hi) * T(0.5);
    V3<T> e = b.hi - b.lo;
    b.radius = tsqrt(dot(e, e)) * T(0.5);
    return b;
}

template <class T> inline T axis_gap(T c, T lo, T hi) {
    return c < lo ? lo - c : (hi < c ? c - hi : T(0));
}

template <class T> bool sphere_meets_box(const LightPrep<T>& l, const FroxelBox<T>& b) {
    T dx = axis_gap(l.c.x, b.lo.x, b.hi.x);
    T dy = axis_gap(l.c.y, b.lo.y, b.hi.y);
    T dz = axis_gap(l.c.z, b.lo.z, b.hi.z);
    T d2 = (dx * dx + dy * dy) + dz * dz;
    return d2 <= l.rm * l.rm;
}

// Cone vs bounding sphere: culled when the sphere lies wholly outside the cone's
// angle, beyond its range along the axis, or behind the apex.
template <class T> bool cone_meets_sphere(const LightPrep<T>& l, const FroxelBox<T>& b) {
    V3<T> v = b.center - l.c;
    T vlen2 = dot(v, v);
    T v1 = dot(v, l.axis);
    T closest = l.cos_o * tsqrt(tmax(vlen2 - v1 * v1, T(0))) - v1 * l.sin_o;
    if (closest > b.radius) return false;
    if (v1 > b.radius + l.rm) return false;
    if (v1 < -b.radius) return false;
    return true;
}

template <class T>
void bin_froxels_impl(const void* camera, const void* lights, uint32_t n, const FroxelParams& p,
                      uint32_t* offsets, uint32_t* indices, uint32_t capacity) {
    Cam<T> c = load_camera<T>(camera);
    const uint32_t F = p.gx * p.gy * p.gz;
    std::vector<float> tab(p.gz + 1);
    slice_table(p, tab.data());
    const T zlast = tmax(T(tab[p.gz]), c.far_);
    std::vector<LightPrep<T>> L(n);
    for (uint32_t i = 0; i < n; ++i) L[i] = prep_light(c, load_light(lights, i));
    std::vector<std::vector<uint32_t>> lists(F);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t col_id = 0; col_id < int64_t(p.gx) * p.gy; ++col_id) {
        uint32_t fx = uint32_t(col_id) % p.gx, fy = uint32_t(col_id) / p.gx;
        Column<T> col = froxel_column(c, p, fx, fy);
        std::vector<uint32_t> col_list;
        for (uint32_t i = 0; i < n; ++i) {
            if (L[i].type == 0u || sphere_in_planes(col.n, L[i].c, L[i].rm)) col_list.push_back(i);
        }
        for (uint32_t s = 0; s < p.gz; ++s) {
            T z0 = T(tab[s]);
            T z1 = (s + 1 == p.gz) ? zlast : T(tab[s + 1]);
            FroxelBox<T> b = froxel_box(col, z0, z1);
            std::vector<uint32_t>& out = lists[size_t(col_id) * p.gz + s];
            for (uint32_t i : col_list) {
                const LightPrep<T>& l = L[i];
                if (l.type == 0u) { out.push_back(i); continue; }
                if (!sphere_meets_box(l, b)) continue;
                if (l.cone && !cone_meets_sphere(l, b)) continue;
                out.push_back(i);
            }
        }
    }
    uint64_t total = 0;
    for (uint32_t f = 0; f < F; ++f) {
        offsets[f] = uint32_t(total);
        for (size_t j = 0; j < lists[f].size(); ++j)
            if (total + j < capacity) indices[total + j] = lists[f][j];
        total += lists[f].size();
    }
    offsets[F] = uint32_t(total);
}

// ----------------------------------------------------------------------------------
// Shading — fs_main (deferred_lighting.wgsl:991-1259) under fallback bindings, and
// pbr_direct_light (:699-820) with pbr_eval.wgsl:6-66.
// ----------------------------------------------------------------------------------
constexpr double kPi = 3.14159265359;  // pbr_eval.wgsl:6

inline double half_to_double(uint16_t h) {
    const uint32_t s = h >> 15, e = (h >> 10) & 31u, m = h & 1023u;
    double v;
    if (e == 0) v = std::ldexp(double(m), -24);
    else if (e == 31) v = m ? std::numeric_limits<double>::quiet_NaN() : std::numeric_limits<double>::infinity();
    else v = std::ldexp(double(m | 1024u), int(e) - 25);
    return s ? -v : v;
}

template <class T> struct Surface {
    T depth;
    V3<T> albedo;
    T alpha;
    V3<T> n_raw;   // normal before normalize (reference reads normal.xyz)
    T ao, rough, metal;
    V3<T> f0;
    V3<T> emissive;
    bool has_f0;   // reference layout carries F0 in the alphas
};

struct GBufferDesc {
    uint32_t layout, W, H, reserved;
    const void* planes[6];
    uint64_t pitch[6];
};

template <class T> inline const unsigned char* texel(const GBufferDesc& g, int plane, uint32_t x, uint32_t y, uint32_t bpp) {
    return static_cast<const unsigned char*>(g.planes[plane]) + g.pitch[plane] * y + size_t(x) * bpp;
}

template <class T> V3<T> oct_decode(T u, T v) {
    // Octahedral unit-vector decode (Cigolle et al. 2014), z-up, signNotZero.
    V3<T> n = v3<T>(u, v, T(1) - std::fabs(u) - std::fabs(v));
    if (n.z < T(0)) {
        T ox = (T(1) - std::fabs(n.y)) * (n.x >= T(0) ? T(1) : T(-1));
        T oy = (T(1) - std::fabs(n.x)) * (n.y >= T(0) ? T(1) : T(-1));
        n.x = ox;
        n.y = oy;
    }
    return n;
}

template <class T> Surface<T> load_surface(const GBufferDesc& g, uint32_t x, uint32_t y) {
    Surface<T> s{};
    auto h = [](const unsigned char* p, int i) {
        uint16_t v;
        std::memcpy(&v, p + 2 * i, 2);
        return T(half_to_double(v));
    };
    auto f = [](const unsigned char* p, int i) {
        float v;
        std::memcpy(&v, p + 4 * i, 4);
        return T(v);
    };
    if (g.layout == 0) {  // reference: albedo RGBA8, normal RGBA16F, orm RGBA8, emissive RGBA16F, depth R32F
        const unsigned char* a = texel<T>(g, 0, x, y, 4);
        const unsigned char* nr = texel<T>(g, 1, x, y, 8);
        const unsigned char* o = texel<T>(g, 2, x, y, 4);
        const unsigned char* e = texel<T>(g, 3, x, y, 8);
        s.depth = f(texel<T>(g, 4, x, y, 4), 0);
        s.albedo = v3<T>(T(a[0]) / T(255), T(a[1]) / T(255), T(a[2]) / T(255));
        s.alpha = T(a[3]) / T(255);
        s.n_raw = v3<T>(h(nr, 0), h(nr, 1), h(nr, 2));
        s.ao = T(o[0]) / T(255);
        s.rough = T(o[1]) / T(255);
        s.metal = T(o[2]) / T(255);
        s.f0 = v3<T>(h(nr, 3), T(o[3]) / T(255), h(e, 3));
        s.emissive = v3<T>(h(e, 0), h(e, 1), h(e, 2));
        s.has_f0 = true;
    } else if (g.layout == 1) {  // F32: albedo+rough RGBA32F, N+metal RGBA32F, depth R32F
        const unsigned char* a = texel<T>(g, 0, x, y, 16);
        const unsigned char* nr = texel<T>(g, 1, x, y, 16);
        s.depth = f(texel<T>(g, 2, x, y, 4), 0);
        s.albedo = v3<T>(f(a, 0), f(a, 1), f(a, 2));
        s.rough = f(a, 3);
        s.n_raw = v3<T>(f(nr, 0), f(nr, 1), f(nr, 2));
        s.metal = f(nr, 3);
    } else {  // F16: albedo+rough RGBA16F, oct normal RG16F, metal R16F, depth R32F
        const unsigned char* a = texel<T>(g, 0, x, y, 8);
        const unsigned char* on = texel<T>(g, 1, x, y, 4);
        const unsigned char* m = texel<T>(g, 2, x, y, 2);
        s.depth = f(texel<T>(g, 3, x, y, 4), 0);
        s.albedo = v3<T>(h(a, 0), h(a, 1), h(a, 2));
        s.rough = h(a, 3);
        s.n_raw = oct_decode<T>(h(on, 0), h(on, 1));
        s.metal = h(m, 0);
    }
    if (g.layout != 0) {
        s.alpha = T(1);
        s.ao = T(1);
        s.emissive = v3<T>(0, 0, 0);
        s.has_f0 = false;
        // gbuffer.wgsl:323-328: F0 = clamp(mix(0.04, albedo, metallic), 0, 0.999)
        s.f0 = v3<T>(clampt(mixt(T(0.04), s.albedo.x, s.metal), T(0), T(0.999)),
                     clampt(mixt(T(0.04), s.albedo.y, s.metal), T(0), T(0.999)),
                     clampt(mixt(T(0.04), s.albedo.z, s.metal), T(0), T(0.999)));
    }
    return s;
}

template <class T> struct PairStats {
    uint64_t listed = 0, in_range = 0, full = 0;
};

// pbr_direct_light, non-anisotropic, no SSS, sf = 1. Returns true when the full
// BRDF was evaluated (passed the NdL and radiance cuts). force: the pair is evaluated
// as lit whatever the cuts decide (range, NdL == 0, radiance < 0.002: :725, :779,
// :781), i.e. with another evaluation's branch decisions; beyond the range the falloff
// max(0, 1 - (d/r)^4) and below the horizon max(N.L, 0) make the value 0, so only the
// radiance cut changes the result.
template <class T>
bool pbr_direct_light(const RawLight& l, V3<T> P, V3<T> N, V3<T> V, V3<T> F0, V3<T> albedo, T rough,
                      T metal, V3<T>& out, bool radiance_cut = true, bool force = false) {
    V3<T> L, radiance;
    const V3<T> color = v3<T>(l.color[0], l.color[1], l.color[2]);
    const T intensity = T(l.intensity);
    if (l.type == 0u) {
        L = normalize(v3<T>(-T(l.dir[0]), -T(l.dir[1]), -T(l.dir[2])));
        radiance = color * intensity;
    } else {
        V3<T> to_light = v3<T>(l.pos[0], l.pos[1], l.pos[2]) - P;
        T dist = tsqrt(dot(to_light, to_light));
        if (dist > T(l.range) && !force) { out = v3<T>(0, 0, 0); return false; }
        L = to_light / dist;
        T atten = T(1) / (dist * dist + T(0.0001));
        T nd = dist / T(l.range);
        atten *= tmax(T(0), T(1) - nd * nd * nd * nd);
        if (l.type == 2u) {
            T cos_a = dot(v3<T>(-L.x, -L.y, -L.z), v3<T>(l.dir[0], l.dir[1], l.dir[2]));
            atten *= smoothstept(T(l.cos_outer), T(l.cos_inner), cos_a);
        }
        radiance = (color * intensity) * atten;
    }
    T NdL = tmax(dot(N, L), T(0));
    if (NdL == T(0) && !force) { out = v3<T>(0, 0, 0); return false; }
    const T cut = T(0.002);
    if (radiance_cut && !force && radiance.x < cut && radiance.y < cut && radiance.z < cut) {
        out = v3<T>(0, 0, 0);
        return false;
    }

    V3<T> H = normalize(V + L);
    // fresnel_schlick (pbr_eval.wgsl:59-61)
    T ct = tmax(dot(H, V), T(0));
    T x = clampt(T(1) - ct, T(0), T(1));
    T x2 = x * x;
    T p5 = x2 * x2 * x;
    V3<T> F = v3<T>(F0.x + (T(1) - F0.x) * p5, F0.y + (T(1) - F0.y) * p5, F0.z + (T(1) - F0.z) * p5);
    V3<T> kD = v3<T>((T(1) - F.x) * (T(1) - metal), (T(1) - F.y) * (T(1) - metal), (T(1) - F.z) * (T(1) - metal));
    T NdV = tmax(dot(N, V), T(0));
    // distribution_ggx (pbr_eval.wgsl:12-18)
    T a = rough * rough;
    T a2 = a * a;
    T NdH = tmax(dot(N, H), T(0));
    T denom = NdH * NdH * (a2 - T(1)) + T(1);
    T D = a2 / (T(kPi) * denom * denom + T(0.0001));
    // geometry_smith (pbr_eval.wgsl:33-43)
    T r1 = rough + T(1);
    T k = (r1 * r1) / T(8);
    T gv = NdV / (NdV * (T(1) - k) + k + T(0.0001));
    T gl = NdL / (NdL * (T(1) - k) + k + T(0.0001));
    T G = gv * gl;
    T sden = T(4) * NdV * NdL + T(0.0001);
    V3<T> spec = v3<T>(D * G * F.x / sden, D * G * F.y / sden, D * G * F.z / sden);
    V3<T> diffuse = v3<T>(kD.x * albedo.x / T(kPi), kD.y * albedo.y / T(kPi), kD.z * albedo.z / T(kPi));
    // (diffuse + specular) * radiance * NdotL * sf, sf = 1
    out = v3<T>((diffuse.x + spec.x) * radiance.x * NdL * T(1), (diffuse.y + spec.y) * radiance.y * NdL * T(1),
                (diffuse.z + spec.z) * radiance.z * NdL * T(1));
    return true;
}

struct GridDesc {
    uint32_t kind, reserved;
    const uint32_t* lists;
    const uint32_t* counts;
    FroxelParams froxel;
};

// Linear view depth from NDC depth (prelude.wgsl:69-71).
template <class T> T view_depth(T depth, T n, T f) { return n * f / (f - depth * (f - n)); }

template <class T>
uint32_t froxel_of_pixel(const FroxelParams& p, const float* tab, uint32_t x, uint32_t y, T d) {
    const uint32_t fx = uint32_t((uint64_t(x) * p.gx) / p.W);
    const uint32_t fy = uint32_t((uint64_t(y) * p.gy) / p.H);
    uint32_t s = 0;
    for (uint32_t k = 1; k < p.gz; ++k)
        if (T(tab[k]) <= d) s = k;
    return (fy * p.gx + fx) * p.gz + s;
}

template <class T>
void shade_impl(const void* camera, const void* globals, const GBufferDesc& g, const void* lights,
                uint32_t n_lights, const GridDesc& grid, double* out_rgba /* W*H*4 */,
                uint32_t* pair_counts /* W*H*3 or null */, uint32_t row0, uint32_t row1,
                const shadow_oracle::ShadowDesc* shadows = nullptr, int* shadow_bounds = nullptr,
                const rc_oracle::RcDesc* rc = nullptr, const uint32_t* forced_off = nullptr,
                const uint32_t* forced_lights = nullptr, uint32_t* flips = nullptr) {
    Cam<T> c = load_camera<T>(camera);
    RawGlobals gl;
    std::memcpy(&gl, globals, sizeof gl);
    std::vector<RawLight> L(n_lights);
    for (uint32_t i = 0; i < n_lights; ++i) L[i] = load_light(lights, i);
    std::vector<float> tab;
    if (grid.kind == 1) {
        tab.resize(grid.froxel.gz + 1);
        slice_table(grid.froxel, tab.data());
    }
    const V3<T> sky = v3<T>(T(gl.ambient_color[0]) * T(gl.ambient_intensity), T(gl.ambient_color[1]) * T(gl.ambient_intensity),
                            T(gl.ambient_color[2]) * T(gl.ambient_intensity));
    const V3<T> ground = sky * T(0.15);
    const uint32_t W = g.W, H = g.H;
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t yy = row0; yy < int64_t(row1); ++yy) {
        const uint32_t y = uint32_t(yy);
        for (uint32_t x = 0; x < W; ++x) {
            Surface<T> s = load_surface<T>(g, x, y);
            const size_t pix = size_t(y) * W + x;
            if (!(s.depth < T(1))) {  // depth >= 1: discarded, target untouched
                if (pair_counts) pair_counts[pix * 3] = pair_counts[pix * 3 + 1] = pair_counts[pix * 3 + 2] = 0;
                continue;
            }
            V3<T> N = normalize(s.n_raw);
            // world position (deferred_lighting.wgsl:1043-1047); frag coord is the pixel centre
            T u = (T(x) + T(0.5)) / T(W);
            T v = (T(y) + T(0.5)) / T(H);
            T ndc_x = u * T(2) - T(1);
            T ndc_y = T(1) - v * T(2);
            T h[4];
            mat4_mul(c.inv_view_proj, ndc_x, ndc_y, s.depth, T(1), h);
            V3<T> P = v3<T>(h[0] / h[3], h[1] / h[3], h[2] / h[3]);
            V3<T> F0 = v3<T>(clampt(s.f0.x, T(0), T(0.999)), clampt(s.f0.y, T(0), T(0.999)), clampt(s.f0.z, T(0), T(0.999)));
            V3<T> V = normalize(c.pos - P);
            // Light list of this pixel
            const uint32_t* list;
            uint32_t count;
            if (grid.kind == 0) {
                const uint32_t tile = (y / kTile) * gl.num_tiles_x + x / kTile;
                count = grid.counts[tile];
                list = grid.lists + size_t(tile) * kMaxPerTile;
            } else {
                T d = view_depth(s.depth, c.near_, c.far_);
                uint32_t f = froxel_of_pixel<T>(grid.froxel, tab.data(), x, y, d);
                count = grid.counts[f + 1] - grid.counts[f];
                list = grid.lists + grid.counts[f];
            }
            V3<T> Lo = v3<T>(0, 0, 0);
            uint32_t n_range = 0, n_full = 0, n_flip = 0;
            // forced branches: the ascending lights another evaluation lit at this pixel
            const bool forced = forced_off != nullptr;
            const uint32_t* fb = forced ? forced_lights + forced_off[pix] : nullptr;
            const uint32_t* fe = forced ? forced_lights + forced_off[pix + 1] : nullptr;
            for (uint32_t j = 0; j < count; ++j) {
                const uint32_t idx = list[j];
                if (idx >= n_lights) continue;
                const RawLight& l = L[idx];
                bool forced_lit = false;
                if (forced) {
                    while (fb < fe && *fb < idx) ++fb;  // lit lights missing from the list: counted below
                    forced_lit = fb < fe && *fb == idx;
                    if (forced_lit) ++fb;
                }
                bool in_range = true;
                if (l.type != 0u) {
                    V3<T> dl = v3<T>(l.pos[0], l.pos[1], l.pos[2]) - P;
                    T dist = tsqrt(dot(dl, dl));
                    in_range = !(dist > T(l.range));
                }
                if (!in_range && !forced_lit) continue;
                if (in_range) ++n_range;
                V3<T> contrib = v3<T>(0, 0, 0);
                const bool own = in_range && pbr_direct_light(l, P, N, V, F0, s.albedo, s.rough, s.metal, contrib);
                if (forced) {
                    if (own != forced_lit) ++n_flip;
                    if (!forced_lit) contrib = v3<T>(0, 0, 0);
                    else if (!own) pbr_direct_light(l, P, N, V, F0, s.albedo, s.rough, s.metal, contrib, true, true);
                }
                if (forced ? forced_lit : own) {
                    if (own) ++n_full;
                    // the pair's shadow factor sf (deferred_lighting.wgsl:1136-1141, 819)
                    if (shadows && idx < shadows->max_lights && l.shadow_index != shadow_oracle::kNoShadow) {
                        const double sf = shadow_oracle::shadow_factor<T>(
                            *shadows, idx, l.pos, l.dir, l.shadow_index, l.type, P.x, P.y, P.z, N.x, N.y, N.z,
                            float(x) + 0.5f, float(y) + 0.5f, c.pos.x, c.pos.y, c.pos.z, gl.csm_splits, shadow_bounds);
                        contrib = contrib * T(sf);
                    }
                }
                Lo = Lo + contrib;
            }
            // Hemisphere ambient (deferred_lighting.wgsl:1196-1199) with ao * ssao(=1)
            T hemi_t = N.y * T(0.5) + T(0.5);
            V3<T> hemi = v3<T>(mixt(ground.x, sky.x, hemi_t), mixt(ground.y, sky.y, hemi_t), mixt(ground.z, sky.z, hemi_t)) * s.albedo;
            if (rc && gl.has_rc_gi != 0u) {
                // RC indirect diffuse over the hemisphere (deferred_lighting.wgsl:1159-1163, 1197-1209)
                T irr[3];
                rc_oracle::irradiance<T>(*rc, gl.rc_world_min, gl.rc_world_max, P.x, P.y, P.z, N.x, N.y, N.z, irr);
                const T NdV = tmax(dot(N, V), T(0));
                const T x = clampt(T(1) - NdV, T(0), T(1));
                const T p5 = x * x * x * x * x;
                const T f0[3] = {F0.x, F0.y, F0.z}, alb[3] = {s.albedo.x, s.albedo.y, s.albedo.z};
                const T w = clampt(tsqrt(irr[0] * irr[0] + irr[1] * irr[1] + irr[2] * irr[2]) * T(4), T(0), T(1));
                T amb[3] = {hemi.x, hemi.y, hemi.z};
                for (int ch = 0; ch < 3; ++ch) {
                    const T F = f0[ch] + (tmax(T(1) - s.rough, f0[ch]) - f0[ch]) * p5;
                    const T diff = (T(1) - F) * (T(1) - s.metal) * irr[ch] * alb[ch];
                    amb[ch] = mixt(amb[ch], diff, w);
                }
                hemi = v3<T>(amb[0], amb[1], amb[2]);
            }
            T ao = s.ao * T(1);
            V3<T> color = Lo + hemi * ao;
            color = color + s.emissive;
            double* o = out_rgba + pix * 4;
            uint32_t dm = gl.debug_mode;
            if (dm == 1 || dm == 2 || dm == 4 || dm == 20 || dm == 21) {
                o[0] = double(s.albedo.x); o[1] = double(s.albedo.y); o[2] = double(s.albedo.z); o[3] = double(s.alpha);
            } else if (dm == 5) {
                o[0] = double(N.x * T(0.5) + T(0.5)); o[1] = double(N.y * T(0.5) + T(0.5)); o[2] = double(N.z * T(0.5) + T(0.5)); o[3] = 1.0;
            } else if (dm == 10) {
                // shadow factor heatmap (deferred_lighting.wgsl:1049-1064): the mean of
                // shadow_factor over the first light_count lights (1 without shadow maps)
                const uint32_t nl = gl.light_count < n_lights ? gl.light_count : n_lights;
                float sum = 0.0f;
                for (uint32_t i = 0; i < nl; ++i) {
                    float sf = 1.0f;
                    if (shadows) {
                        const RawLight& l = L[i];
                        sf = float(shadow_oracle::shadow_factor<T>(*shadows, i, l.pos, l.dir, l.shadow_index, l.type,
                                                                   P.x, P.y, P.z, N.x, N.y, N.z, float(x) + 0.5f,
                                                                   float(y) + 0.5f, c.pos.x, c.pos.y, c.pos.z,
                                                                   gl.csm_splits, shadow_bounds));
                    }
                    sum = sum + sf;
                }
                sum = sum + float(gl.light_count - nl);  // lights beyond the buffer: lit
                const float cnt = float(gl.light_count);
                const float sf = sum / (cnt < 1.0f ? 1.0f : cnt);
                o[0] = o[1] = o[2] = double(sf);
                o[3] = 1.0;
            } else if (dm == 11 && gl.light_count > 0u && shadows) {
                // light-space projection by the first shadow matrix (:1066-1080), in f32
                // with the shader's operations in order (uv = frag / size, ndc, M v / w)
                const float fw = float(W), fh = float(H);
                const float ux = (float(x) + 0.5f) / fw, uy = (float(y) + 0.5f) / fh;
                const float nx = ux * 2.0f - 1.0f, ny = 1.0f - uy * 2.0f;
                float ivp[16], h[4], lc[4];
                const RawCamera* rc = static_cast<const RawCamera*>(camera);
                for (int k = 0; k < 16; ++k) ivp[k] = rc->inv_view_proj[k];
                mat4_mul<float>(ivp, nx, ny, float(s.depth), 1.0f, h);
                const float wx = h[0] / h[3], wy = h[1] / h[3], wz = h[2] / h[3];
                mat4_mul<float>(shadows->mats, wx, wy, wz, 1.0f, lc);
                float r[4] = {0.0f, 0.0f, 0.2f, 1.0f};
                if (lc[3] > 0.001f) {
                    const float n0 = lc[0] / lc[3], n1 = lc[1] / lc[3], n2 = lc[2] / lc[3];
                    const float u = n0 * 0.5f + 0.5f, v = -n1 * 0.5f + 0.5f;
                    if (u >= 0.0f && v >= 0.0f && u <= 1.0f && v <= 1.0f && n2 >= 0.0f && n2 <= 1.0f) {
                        r[0] = n2;
                        r[1] = n2 * 0.3f;
                        r[2] = 0.0f;
                    }
                }
                for (int k = 0; k < 4; ++k) o[k] = double(r[k]);
            } else {
                o[0] = double(color.x); o[1] = double(color.y); o[2] = double(color.z); o[3] = double(s.alpha);
            }
            if (pair_counts) {
                pair_counts[pix * 3] = count;
                pair_counts[pix * 3 + 1] = n_range;
                pair_counts[pix * 3 + 2] = n_full;
            }
            if (flips) {
                // the forced pairs the list walk never reached: lit lights absent from the list
                uint32_t unlisted = 0;
                if (forced) {
                    const uint32_t* a = forced_lights + forced_off[pix];
                    const uint32_t* b = forced_lights + forced_off[pix + 1];
                    for (; a < b; ++a) {
                        bool found = false;
                        for (uint32_t j = 0; j < count && !found; ++j) found = list[j] == *a;
                        unlisted += found ? 0u : 1u;
                    }
                }
                flips[pix] = n_flip | (unlisted << 16);
            }
        }
    }
}

// ---- the reflection draw (fs_reflection, deferred_lighting.wgsl:1265-1341) ----

inline void half4(const unsigned char* p, double* o) {
    for (int i = 0; i < 4; ++i) {
        uint16_t v;
        std::memcpy(&v, p + 2 * i, 2);
        o[i] = half_to_double(v);
    }
}

struct EnvDesc {  // hl_reflection_env with host pointers
    const void* captures;
    uint32_t count, face_size, mip_levels, layers;
    const void* texels;
};
static_assert(sizeof(EnvDesc) == 32, "hl_reflection_env is 32 bytes");

struct ReflectImages {  // hl_reflection_inputs with host pointers; rc, env: null = unbound
    const unsigned char* ssr;
    uint64_t ssr_pitch;
    const unsigned char* planar;
    uint64_t planar_pitch;
    const unsigned char* lmuv;
    uint64_t lmuv_pitch;
    const rc_oracle::RcDesc* rc;
    const EnvDesc* env;
};

// One level of one cube layer as the pass's env sampler reads it (linear within the
// level, clamp to edge): the face of the direction's major axis (ties to z, then y),
// the Vulkan / WebGPU face coordinates, bilinear within the face.
template <class T>
void cube_sample(const EnvDesc& e, T dx, T dy, T dz, uint32_t layer, uint32_t level, T out[3]) {
    const T ax = std::fabs(dx), ay = std::fabs(dy), az = std::fabs(dz);
    uint32_t face;
    T sc, tc, ma;
    if (az >= ax && az >= ay) {
        face = dz >= T(0) ? 4u : 5u;
        sc = dz >= T(0) ? dx : -dx;
        tc = -dy;
        ma = az;
    } else if (ay >= ax) {
        face = dy >= T(0) ? 2u : 3u;
        sc = dx;
        tc = dy >= T(0) ? dz : -dz;
        ma = ay;
    } else {
        face = dx >= T(0) ? 0u : 1u;
        sc = dx >= T(0) ? -dz : dz;
        tc = -dy;
        ma = ax;
    }
    const T s = ma > T(0) ? T(0.5) * (sc / ma + T(1)) : T(0.5), t = ma > T(0) ? T(0.5) * (tc / ma + T(1)) : T(0.5);
    uint64_t chain = 0, off = 0;
    for (uint32_t m = 0; m < e.mip_levels; ++m) {
        const uint64_t nm = std::max<uint64_t>(1, e.face_size >> m);
        if (m < level) off += nm * nm;
        chain += nm * nm;
    }
    const uint32_t n = std::max<uint32_t>(1u, e.face_size >> level);
    const unsigned char* base =
        static_cast<const unsigned char*>(e.texels) + 8ull * ((uint64_t(layer) * 6u + face) * chain + off);
    const T u = s * T(n) - T(0.5), v = t * T(n) - T(0.5);
    const T fu = std::floor(u), fv = std::floor(v);
    const T wu = u - fu, wv = v - fv;
    const int64_t iu = int64_t(fu), iv = int64_t(fv), top = int64_t(n) - 1;
    auto cl = [&](int64_t k) { return k < 0 ? 0 : (k > top ? top : k); };
    double t00[4], t01[4], t10[4], t11[4];
    half4(base + 8ull * (uint64_t(cl(iv)) * n + cl(iu)), t00);
    half4(base + 8ull * (uint64_t(cl(iv)) * n + cl(iu + 1)), t01);
    half4(base + 8ull * (uint64_t(cl(iv + 1)) * n + cl(iu)), t10);
    half4(base + 8ull * (uint64_t(cl(iv + 1)) * n + cl(iu + 1)), t11);
    for (int k = 0; k < 3; ++k)
        out[k] = (T(t00[k]) * (T(1) - wu) + T(t01[k]) * wu) * (T(1) - wv) + (T(t10[k]) * (T(1) - wu) + T(t11[k]) * wu) * wv;
}

// sample_reflection_environment (deferred_lighting.wgsl:646-694) with capture_weight
// (:618-638), parallax_box (:596-616) and parallax_sphere (:575-588).
template <class T>
void reflection_environment(const EnvDesc& e, uint32_t count, V3<T> P, V3<T> R, T lod, T out[3], int* bounds) {
    const int64_t lvl = int64_t(std::ceil(lod + T(0.5))) - 1;
    const uint32_t level = uint32_t(std::min<int64_t>(std::max<int64_t>(lvl, 0), int64_t(e.mip_levels) - 1));
    T acc_c[3] = {0, 0, 0}, acc = 0;
    const uint32_t n = std::min(std::min(count, 64u), e.count);
    for (uint32_t i = 0; i < n; ++i) {
        if (acc >= T(0.999)) break;
        const unsigned char* cp = static_cast<const unsigned char*>(e.captures) + 112ull * i;
        float pr[4], et[4], m[16], brightness;
        int32_t layer;
        uint32_t shape;
        std::memcpy(pr, cp, 16);
        std::memcpy(et, cp + 16, 16);
        std::memcpy(m, cp + 32, 64);
        std::memcpy(&layer, cp + 96, 4);
        std::memcpy(&shape, cp + 100, 4);
        std::memcpy(&brightness, cp + 108, 4);
        if (layer < 0) continue;
        if (uint32_t(layer) >= e.layers) {
            *bounds = 1;
            continue;
        }
        auto row = [&](int r, T x, T y, T z, T w) { return T(m[r]) * x + T(m[4 + r]) * y + T(m[8 + r]) * z + T(m[12 + r]) * w; };
        T w;
        if (shape == 1u) {
            const T gx = T(et[0]) - std::fabs(row(0, P.x, P.y, P.z, T(1)));
            const T gy = T(et[1]) - std::fabs(row(1, P.x, P.y, P.z, T(1)));
            const T gz = T(et[2]) - std::fabs(row(2, P.x, P.y, P.z, T(1)));
            w = (gx < T(0) || gy < T(0) || gz < T(0))
                    ? T(0) : clampt(tmin(tmin(gx, gy), gz) / tmax(T(et[3]), T(1e-4)), T(0), T(1));
        } else {
            const V3<T> o = P - v3<T>(pr[0], pr[1], pr[2]);
            const T dist = tsqrt(dot(o, o));
            w = dist > T(pr[3]) ? T(0) : clampt((T(pr[3]) - dist) / tmax(T(pr[3]) * T(0.1), T(1e-4)), T(0), T(1));
        }
        if (w <= T(0)) continue;
        V3<T> dir = R;
        if (shape == 1u) {
            const T pl[3] = {row(0, P.x, P.y, P.z, T(1)), row(1, P.x, P.y, P.z, T(1)), row(2, P.x, P.y, P.z, T(1))};
            const T rl[3] = {row(0, R.x, R.y, R.z, T(0)), row(1, R.x, R.y, R.z, T(0)), row(2, R.x, R.y, R.z, T(0))};
            T t = std::numeric_limits<T>::infinity();
            for (int k = 0; k < 3; ++k) {
                const T inv = T(1) / rl[k];
                t = tmin(t, tmax((-T(et[k]) - pl[k]) * inv, (T(et[k]) - pl[k]) * inv));
            }
            if (t > T(0) && t < T(3.402823e38)) dir = (P + R * t) - v3<T>(pr[0], pr[1], pr[2]);
        } else {
            const V3<T> o = P - v3<T>(pr[0], pr[1], pr[2]);
            const T b = dot(o, R);
            const T c = dot(o, o) - T(pr[3]) * T(pr[3]);
            const T disc = b * b - c;
            if (disc >= T(0)) {
                const T t = -b + tsqrt(disc);
                if (t > T(0)) dir = (P + R * t) - v3<T>(pr[0], pr[1], pr[2]);
            }
        }
        T smp[3];
        cube_sample<T>(e, dir.x, dir.y, dir.z, uint32_t(layer), level, smp);
        const T contrib = w * (T(1) - acc);
        for (int k = 0; k < 3; ++k) acc_c[k] += smp[k] * T(brightness) * contrib;
        acc += contrib;
    }
    if (acc < T(0.999)) {
        T sky[3];
        cube_sample<T>(e, R.x, R.y, R.z, 0u, level, sky);
        for (int k = 0; k < 3; ++k) acc_c[k] += sky[k] * (T(1) - acc);
    }
    for (int k = 0; k < 3; ++k) out[k] = acc_c[k];
}

// out_rgba holds the lit target (fs_main's output) and receives the blended result:
// rgb += contribution (One + One), alpha kept (deferred-light/src/lib.rs:464-475); debug
// modes 30/31 replace the pixel (the replacement pipeline, lib.rs:1188-1193).
// *unsupported is set when a pixel needs the RC fallback and no probes are bound.
template <class T>
void reflect_impl(const void* camera, const void* globals, const GBufferDesc& g, const ReflectImages& im,
                  double* out_rgba, int* unsupported) {
    Cam<T> c = load_camera<T>(camera);
    RawGlobals gl;
    std::memcpy(&gl, globals, sizeof gl);
    const uint32_t W = g.W, H = g.H;
    for (uint32_t y = 0; y < H; ++y) {
        for (uint32_t x = 0; x < W; ++x) {
            Surface<T> s = load_surface<T>(g, x, y);
            if (!(s.depth < T(1))) continue;  // discard (:1268)
            double* o = out_rgba + (size_t(y) * W + x) * 4;
            double ssr[4] = {0, 0, 0, 0};  // black fallback
            if (im.ssr) half4(im.ssr + im.ssr_pitch * y + 8ull * x, ssr);
            const uint32_t dm = gl.debug_mode;
            if (dm == 30 || dm == 31) {  // :1271-1276
                for (int k = 0; k < 3; ++k) o[k] = dm == 30 ? ssr[3] : ssr[k];
                o[3] = 1.0;
                continue;
            }
            if (dm == 1 || dm == 2 || dm == 4 || dm == 5 || dm == 10 || dm == 11 || dm == 20 || dm == 21) continue;
            const V3<T> N = normalize(s.n_raw);
            const T rough = s.rough;
            const T F0[3] = {clampt(s.f0.x, T(0), T(0.999)), clampt(s.f0.y, T(0), T(0.999)),
                             clampt(s.f0.z, T(0), T(0.999))};
            // lightmap sentinel (:1300-1303); without the image every pixel holds (-1, -1)
            T lm_x = T(-1);
            if (im.lmuv) {
                uint16_t v;
                std::memcpy(&v, im.lmuv + im.lmuv_pitch * y + 4ull * x, 2);
                lm_x = T(half_to_double(v));
            }
            const bool has_lightmap = !(lm_x < T(-1.5)) && lm_x >= T(0);
            // world position, V, F_ibl, R (:1305-1311)
            const T u = (T(x) + T(0.5)) / T(W), v = (T(y) + T(0.5)) / T(H);
            T h[4];
            mat4_mul(c.inv_view_proj, u * T(2) - T(1), T(1) - v * T(2), s.depth, T(1), h);
            const V3<T> P = v3<T>(h[0] / h[3], h[1] / h[3], h[2] / h[3]);
            const V3<T> V = normalize(c.pos - P);
            const T NdV = tmax(dot(N, V), T(0));
            const T q = clampt(T(1) - NdV, T(0), T(1));
            const T p5 = q * q * q * q * q;
            T F[3];
            for (int k = 0; k < 3; ++k) F[k] = F0[k] + (tmax(T(1) - rough, F0[k]) - F0[k]) * p5;
            const T nv = dot(N, V);
            const V3<T> R = v3<T>(T(2) * nv * N.x - V.x, T(2) * nv * N.y - V.y, T(2) * nv * N.z - V.z);
            T spec[3] = {0, 0, 0};  // environment term: the black fallback cube (lib.rs:542) ...
            if (im.env && gl.enable_env_reflections != 0u && gl.enable_reflections != 0u) {
                // ... or the captures' (:1313-1318)
                T env[3];
                int env_bounds = 0;  // layer indices beyond the array: skipped (the kernel reports them)
                reflection_environment<T>(*im.env, gl.reflection_capture_count, P, R, rough * T(8), env, &env_bounds);
                const T r0 = rough * T(-1) + T(1), r1 = rough * T(-0.0275) + T(0.0425);
                const T r2 = rough * T(-0.572) + T(1.04), r3 = rough * T(0.022) + T(-0.04);
                const T a004 = tmin(r0 * r0, T(std::exp2(T(-9.28) * NdV))) * r0 + r1;
                const T bx = T(-1.04) * a004 + r2, by = T(1.04) * a004 + r3;
                for (int k = 0; k < 3; ++k) spec[k] = env[k] * (F0[k] * bx + by);
            }
            if (gl.enable_reflections != 0u && T(ssr[3]) > T(0))
                for (int k = 0; k < 3; ++k) spec[k] = mixt(spec[k], T(ssr[k]) * F[k], T(ssr[3]));
            if (gl.enable_reflections != 0u && im.planar) {
                double pl[4];
                half4(im.planar + im.planar_pitch * y + 8ull * x, pl);
                if (T(pl[3]) > T(0))
                    for (int k = 0; k < 3; ++k) spec[k] = mixt(spec[k], T(pl[k]) * F[k], T(pl[3]));
            }
            if (gl.has_rc_gi > 0u && rough > T(0.6)) {
                if (!im.rc) {
                    *unsupported = 1;
                    continue;
                }
                // sample_rc_specular (:928-980): the RC irradiance along mix(R, N, 0.5 r)
                const T hr = rough * T(0.5);
                const V3<T> look = normalize(v3<T>(mixt(R.x, N.x, hr), mixt(R.y, N.y, hr), mixt(R.z, N.z, hr)));
                T irr[3];
                rc_oracle::irradiance<T>(*im.rc, gl.rc_world_min, gl.rc_world_max, P.x, P.y, P.z, look.x, look.y,
                                         look.z, irr);
                const T w = smoothstept(T(0.6), T(0.9), rough) * T(0.4);
                for (int k = 0; k < 3; ++k) spec[k] = mixt(spec[k], irr[k], w);
            }
            const T ao = has_lightmap ? T(1) : s.ao * T(1);  // screen AO: the white fallback
            for (int k = 0; k < 3; ++k) o[k] += double(spec[k] * ao);
        }
    }
}

// ---- fragment lighting (forward_lit.wgsl:443-494, transparent_base.wgsl:181-220) ----

struct RawFragment {
    float pos[3];
    uint32_t pixel;
    float normal[3], alpha;
    float albedo[3], rough;
    float f0[3], metal;
    float emissive[3], ao;
};
static_assert(sizeof(RawFragment) == 80, "hl_fragment is 80 bytes");

struct RawTransform {
    float pos[3], rot[3], scale[3];
};
static_assert(sizeof(RawTransform) == 36, "Transform is 36 bytes (forward_lit.wgsl:118-122)");

struct FragmentParams {
    uint32_t mode, num_tiles_x;
    float ambient_intensity, ambient_color[3];
};

// Light direction of a Transform rotation (forward_lit.wgsl:374-383): the rotation
// q = qy(yaw) qx(pitch) qz(roll) of Euler order Y, X, Z applied to (0, 0, -1).
template <class T> V3<T> light_dir_from_rotation(const float rot_deg[3]) {
    const T deg = T(3.14159265358979323846) / T(180);
    const T hp = T(rot_deg[0]) * deg * T(0.5), hy = T(rot_deg[1]) * deg * T(0.5), hr = T(rot_deg[2]) * deg * T(0.5);
    struct Q { T x, y, z, w; };
    auto mul = [](Q a, Q b) {
        return Q{a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y, a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x,
                 a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w, a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z};
    };
    const Q qy{T(0), std::sin(hy), T(0), std::cos(hy)};
    const Q qx{std::sin(hp), T(0), T(0), std::cos(hp)};
    const Q qz{T(0), T(0), std::sin(hr), std::cos(hr)};
    const Q q = mul(mul(qy, qx), qz);
    // v + w t + q.xyz x t with t = 2 q.xyz x v, v = (0, 0, -1)
    const V3<T> qv = v3<T>(q.x, q.y, q.z), v = v3<T>(T(0), T(0), T(-1));
    const V3<T> t = cross(qv, v) * T(2);
    return normalize(v + t * q.w + cross(qv, t));
}

template <class T>
void shade_fragments_impl(const void* camera, const FragmentParams& fp, const RawFragment* frags, uint32_t n,
                          const void* lights, uint32_t n_lights, const uint32_t* entity, const RawTransform* xf,
                          uint32_t n_xf, const GridDesc& grid, double* out_rgba /* n*4, untouched if discarded */) {
    Cam<T> c = load_camera<T>(camera);
    RawCamera rc;
    std::memcpy(&rc, camera, sizeof rc);
    std::vector<RawLight> L(n_lights);
    std::vector<uint8_t> usable(n_lights, 1);
    for (uint32_t i = 0; i < n_lights; ++i) {
        L[i] = load_light(lights, i);
        if (fp.mode == 0 && entity) {
            if (entity[i] >= n_xf) {
                usable[i] = 0;
                continue;
            }
            const RawTransform& t = xf[entity[i]];
            const V3<T> d = light_dir_from_rotation<T>(t.rot);
            for (int k = 0; k < 3; ++k) L[i].pos[k] = t.pos[k];
            L[i].dir[0] = float(d.x);
            L[i].dir[1] = float(d.y);
            L[i].dir[2] = float(d.z);
        }
    }
    std::vector<float> tab;
    if (grid.kind == 1) {
        tab.resize(grid.froxel.gz + 1);
        slice_table(grid.froxel, tab.data());
    }
    const V3<T> amb = v3<T>(T(fp.ambient_color[0]) * T(fp.ambient_intensity), T(fp.ambient_color[1]) * T(fp.ambient_intensity),
                            T(fp.ambient_color[2]) * T(fp.ambient_intensity));
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t ii = 0; ii < int64_t(n); ++ii) {
        const RawFragment& f = frags[ii];
        if (fp.mode == 0 && !(f.alpha > 0.001f)) continue;  // discard
        const uint32_t x = f.pixel & 0xFFFFu, y = f.pixel >> 16;
        const V3<T> P = v3<T>(f.pos[0], f.pos[1], f.pos[2]);
        const V3<T> N = normalize(v3<T>(f.normal[0], f.normal[1], f.normal[2]));
        const V3<T> V = normalize(c.pos - P);
        const V3<T> F0 = v3<T>(f.f0[0], f.f0[1], f.f0[2]);
        const V3<T> albedo = v3<T>(f.albedo[0], f.albedo[1], f.albedo[2]);
        const uint32_t* list = nullptr;
        uint32_t count = 0;
        if (grid.kind == 0) {
            const uint32_t tile = (y / kTile) * fp.num_tiles_x + x / kTile;
            count = grid.counts[tile];
            list = grid.lists + size_t(tile) * kMaxPerTile;
        } else {
            // view depth -(view * P).z, column-major view matrix
            const T zv = T(rc.view[2]) * P.x + T(rc.view[6]) * P.y + T(rc.view[10]) * P.z + T(rc.view[14]);
            const uint32_t fr = froxel_of_pixel<T>(grid.froxel, tab.data(), x, y, -zv);
            count = grid.counts[fr + 1] - grid.counts[fr];
            list = grid.lists + grid.counts[fr];
        }
        V3<T> Lo = v3<T>(0, 0, 0);
        for (uint32_t j = 0; j < count; ++j) {
            const uint32_t idx = list[j];
            if (idx >= n_lights || !usable[idx]) continue;
            const RawLight& l = L[idx];
            if (l.type != 0u) {
                V3<T> dl = v3<T>(l.pos[0], l.pos[1], l.pos[2]) - P;
                if (tsqrt(dot(dl, dl)) > T(l.range)) continue;
            }
            V3<T> contrib;
            pbr_direct_light(l, P, N, V, F0, albedo, T(f.rough), T(f.metal), contrib, fp.mode != 0);
            Lo = Lo + contrib;
        }
        V3<T> color;
        if (fp.mode == 0)
            color = Lo + (amb * albedo) * T(f.ao) + v3<T>(f.emissive[0], f.emissive[1], f.emissive[2]);
        else
            color = v3<T>(f.emissive[0], f.emissive[1], f.emissive[2]) + Lo;
        double* o = out_rgba + size_t(ii) * 4;
        o[0] = double(color.x);
        o[1] = double(color.y);
        o[2] = double(color.z);
        o[3] = double(f.alpha);
    }
}

}  // namespace

// ----------------------------------------------------------------------------------
// Adjoint (FP64): gradient of sum_px sum_c w[px][c] * radiance_c(px) with respect
// to light position, intensity, colour and per-pixel albedo, roughness, metallic,
// the branch decisions held fixed. Written from the forward formulas above by hand.
// ----------------------------------------------------------------------------------
namespace {

struct D3 {
    double x, y, z;
};
inline D3 d3(double x, double y, double z) { return D3{x, y, z}; }
inline D3 operator+(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline D3 operator-(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline D3 operator*(D3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double ddot(D3 a, D3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }

// Vector-Jacobian product of normalize(v) = v/|v| : given g = dOut, returns dv.
inline D3 normalize_vjp(D3 v, D3 g) {
    double len = std::sqrt(ddot(v, v));
    D3 n = v * (1.0 / len);
    return (g - n * ddot(g, n)) * (1.0 / len);
}

// One (pixel, light) pair. Adds d/d light params to gl[7] and d/d pixel params to gp[5].
void pair_adjoint(const RawLight& l, D3 P, D3 N, D3 V, D3 albedo, double rough, double metal, bool f0_from_albedo,
                  D3 F0_in, const double w[3], double gl[7], double gp[5]) {
    if (l.type == 0u) {
        // Directional light: depends on colour and intensity only.
    }
    D3 color = d3(l.color[0], l.color[1], l.color[2]);
    double I = l.intensity;
    D3 L;
    double atten = 1.0;
    D3 to_light{0, 0, 0};
    double dist = 0;
    if (l.type == 0u) {
        L = d3(-double(l.dir[0]), -double(l.dir[1]), -double(l.dir[2]));
        double ln = std::sqrt(ddot(L, L));
        L = L * (1.0 / ln);
    } else {
        to_light = d3(l.pos[0], l.pos[1], l.pos[2]) - P;
        dist = std::sqrt(ddot(to_light, to_light));
        if (dist > double(l.range)) return;
        L = to_light * (1.0 / dist);
        double r = l.range;
        double a0 = 1.0 / (dist * dist + 0.0001);
        double nd = dist / r;
        double fall = std::max(0.0, 1.0 - nd * nd * nd * nd);
        atten = a0 * fall;
        if (l.type == 2u) {
            double cos_a = -ddot(L, d3(l.dir[0], l.dir[1], l.dir[2]));
            atten *= smoothstept<double>(l.cos_outer, l.cos_inner, cos_a);
        }
    }
    D3 rad = d3(color.x * I * atten, color.y * I * atten, color.z * I * atten);
    double NdL = std::max(ddot(N, L), 0.0);
    if (NdL == 0.0) return;
    if (rad.x < 0.002 && rad.y < 0.002 && rad.z < 0.002) return;

    // ---- forward recompute with intermediates ----
    D3 hv = V + L;
    double hl = std::sqrt(ddot(hv, hv));
    D3 H = hv * (1.0 / hl);
    double hdv = ddot(H, V);
    double ct = std::max(hdv, 0.0);
    double xx = 1.0 - ct;
    bool x_clamped = !(xx > 0.0 && xx < 1.0);
    xx = std::min(std::max(xx, 0.0), 1.0);
    double p5 = xx * xx * xx * xx * xx;
    D3 F0 = F0_in;
    double F[3] = {F0.x + (1 - F0.x) * p5, F0.y + (1 - F0.y) * p5, F0.z + (1 - F0.z) * p5};
    double NdV = std::max(ddot(N, V), 0.0);
    double a = rough * rough, a2 = a * a;
    double ndh_raw = ddot(N, H);
    double NdH = std::max(ndh_raw, 0.0);
    double den = NdH * NdH * (a2 - 1) + 1;
    double Dden = kPi * den * den + 0.0001;
    double D = a2 / Dden;
    double r1 = rough + 1, k = r1 * r1 / 8;
    double gvd = NdV * (1 - k) + k + 0.0001, gld = NdL * (1 - k) + k + 0.0001;
    double gv = NdV / gvd, glv = NdL / gld;
    double G = gv * glv;
    double sden = 4 * NdV * NdL + 0.0001;
    double alb[3] = {albedo.x, albedo.y, albedo.z};
    double radv[3] = {rad.x, rad.y, rad.z};
    double cols[3] = {color.x, color.y, color.z};

    // out_c = (kD_c*alb_c/pi + D*G*F_c/sden) * rad_c * NdL
    double dD = 0, dG = 0, dsden = 0, dNdL = 0, dp5 = 0, dmetal = 0, datten = 0;
    for (int ch = 0; ch < 3; ++ch) {
        double kD = (1 - F[ch]) * (1 - metal);
        double diff = kD * alb[ch] / kPi;
        double spec = D * G * F[ch] / sden;
        double brdf = diff + spec;
        double go = w[ch];
        // d/d rad_c, d/d NdL
        double g_rad = go * brdf * NdL;
        dNdL += go * brdf * radv[ch];
        double g_brdf = go * radv[ch] * NdL;
        // diff branch
        double g_kD = g_brdf * alb[ch] / kPi;
        gp[ch] += g_brdf * kD / kPi;  // d/d albedo via diffuse
        double g_F = -g_kD * (1 - metal);
        dmetal += -g_kD * (1 - F[ch]);
        // spec branch
        dD += g_brdf * G * F[ch] / sden;
        dG += g_brdf * D * F[ch] / sden;
        g_F += g_brdf * D * G / sden;
        dsden += -g_brdf * D * G * F[ch] / (sden * sden);
        // F_c = F0_c + (1 - F0_c) p5
        dp5 += g_F * (1 - (ch == 0 ? F0.x : ch == 1 ? F0.y : F0.z));
        double g_F0 = g_F * (1 - p5);
        if (f0_from_albedo) {
            // F0 = clamp(0.04*(1-m) + alb*m, 0, 0.999)
            double f0raw = 0.04 * (1 - metal) + alb[ch] * metal;
            if (f0raw > 0.0 && f0raw < 0.999) {
                gp[ch] += g_F0 * metal;
                dmetal += g_F0 * (alb[ch] - 0.04);
            }
        }
        // rad_c = col_c * I * atten
        gl[4 + ch] += g_rad * I * atten;
        gl[3] += g_rad * cols[ch] * atten;
        datten += g_rad * cols[ch] * I;
    }
    gp[4] += dmetal;
    // sden = 4 NdV NdL + 1e-4
    dNdL += dsden * 4 * NdV;
    // G = gv * gl(NdL), gl = NdL/(NdL(1-k)+k+1e-4)
    double dglv = dG * gv;
    double dgv = dG * glv;
    dNdL += dglv * (gld - NdL * (1 - k)) / (gld * gld);
    // d/dk of gv and glv
    double dk = dgv * (-NdV * (-NdV + 1)) / (gvd * gvd) + dglv * (-NdL * (-NdL + 1)) / (gld * gld);
    // k = (r+1)^2/8 -> dk/drough = (r+1)/4
    double drough = dk * r1 / 4.0;
    // D = a2 / (pi den^2 + 1e-4), den = NdH^2 (a2-1) + 1
    double dDden = -dD * a2 / (Dden * Dden);
    double dden = dDden * 2 * kPi * den;
    double da2 = dD / Dden + dden * NdH * NdH;
    double dNdH = dden * 2 * NdH * (a2 - 1);
    drough += da2 * 2 * a * 2 * rough;  // a2 = r^4
    gp[3] += drough;
    // p5 = x^5, x = clamp(1 - max(H.V,0))
    double dct = x_clamped ? 0.0 : -dp5 * 5 * xx * xx * xx * xx;
    double dhdv = (hdv > 0) ? dct : 0.0;
    double dndh = (ndh_raw > 0) ? dNdH : 0.0;
    // H = normalize(V + L); hdv = H.V, ndh = N.H
    D3 dH = V * dhdv + N * dndh;
    D3 dL = normalize_vjp(hv, dH);
    // NdL = max(N.L, 0) (positive here)
    dL = dL + N * dNdL;
    if (l.type == 0u) return;  // L does not depend on the light position
    // atten chain: atten = a0 * fall * spot
    double r = l.range;
    double a0 = 1.0 / (dist * dist + 0.0001);
    double nd = dist / r;
    double fall_raw = 1.0 - nd * nd * nd * nd;
    double fall = std::max(0.0, fall_raw);
    double spot = 1.0;
    double dspot_dcos = 0.0;
    if (l.type == 2u) {
        double cos_a = -ddot(L, d3(l.dir[0], l.dir[1], l.dir[2]));
        double lo = l.cos_outer, hi = l.cos_inner;
        double t = (cos_a - lo) / (hi - lo);
        if (t <= 0) { spot = 0; }
        else if (t >= 1) { spot = 1; }
        else { spot = t * t * (3 - 2 * t); dspot_dcos = 6 * t * (1 - t) / (hi - lo); }
    }
    double ddist = datten * spot * (fall * (-2 * dist) * a0 * a0 + (fall_raw > 0 ? a0 * (-4 * nd * nd * nd / r) : 0.0));
    // spot depends on L: cos_a = -L.dir
    if (l.type == 2u) {
        double dcos = datten * a0 * fall * dspot_dcos;
        dL = dL + d3(-l.dir[0], -l.dir[1], -l.dir[2]) * dcos;
    }
    // L = to_light / dist ; dist = |to_light|
    D3 dto = normalize_vjp(to_light, dL) + L * ddist;
    // to_light = light_pos - P
    gl[0] += dto.x;
    gl[1] += dto.y;
    gl[2] += dto.z;
}

}  // namespace

// ----------------------------------------------------------------------------------
// extern "C" entry points for the ctypes wrapper (oracle/__init__.py)
// ----------------------------------------------------------------------------------
extern "C" {

int oracle_abi_version() { return 3; }

int oracle_num_threads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

void oracle_bin_tiles_ref_f32(const void* cam, const void* lights, uint32_t n, uint32_t W, uint32_t H, uint32_t* lists,
                              uint32_t* counts) {
    bin_tiles_ref_impl<float>(cam, lights, n, W, H, lists, counts);
}
void oracle_bin_tiles_ref_f64(const void* cam, const void* lights, uint32_t n, uint32_t W, uint32_t H, uint32_t* lists,
                              uint32_t* counts) {
    bin_tiles_ref_impl<double>(cam, lights, n, W, H, lists, counts);
}

void oracle_froxel_slice_table(const void* params, float* out) {
    FroxelParams p;
    std::memcpy(&p, params, sizeof p);
    slice_table(p, out);
}

void oracle_bin_froxels_f32(const void* cam, const void* lights, uint32_t n, const void* params, uint32_t* offsets,
                            uint32_t* indices, uint32_t capacity) {
    FroxelParams p;
    std::memcpy(&p, params, sizeof p);
    bin_froxels_impl<float>(cam, lights, n, p, offsets, indices, capacity);
}

// grid: kind (0 tiles, 1 froxels), lists, counts/offsets, froxel params (32 B)
static GridDesc make_grid(uint32_t kind, const uint32_t* lists, const uint32_t* counts, const void* froxel) {
    GridDesc g{};
    g.kind = kind;
    g.lists = lists;
    g.counts = counts;
    if (froxel) std::memcpy(&g.froxel, froxel, sizeof g.froxel);
    return g;
}

static GBufferDesc make_gbuf(uint32_t layout, uint32_t W, uint32_t H, const void* const* planes, const uint64_t* pitch) {
    GBufferDesc g{};
    g.layout = layout;
    g.W = W;
    g.H = H;
    for (int i = 0; i < 6; ++i) {
        g.planes[i] = planes[i];
        g.pitch[i] = pitch[i];
    }
    return g;
}

void oracle_shade_f64(const void* cam, const void* globals, uint32_t layout, uint32_t W, uint32_t H, const void* const* planes,
                      const uint64_t* pitch, const void* lights, uint32_t n, uint32_t grid_kind, const uint32_t* lists,
                      const uint32_t* counts, const void* froxel, double* out_rgba, uint32_t* pair_counts, uint32_t row0,
                      uint32_t row1) {
    GBufferDesc g = make_gbuf(layout, W, H, planes, pitch);
    GridDesc gr = make_grid(grid_kind, lists, counts, froxel);
    shade_impl<double>(cam, globals, g, lights, n, gr, out_rgba, pair_counts, row0, row1);
}

// oracle_shade_f64 with forced branch decisions: forced_off[W*H+1] / forced_lights (CSR,
// each pixel's lights ascending) name the (pixel, light) pairs another evaluation lit;
// those are evaluated as lit whatever the f64 cuts decide and every other pair
// contributes nothing. flips[W*H] = pairs whose f64 decision differs, plus 65536 x
// lit pairs whose light is not in the pixel's list.
void oracle_shade_forced_f64(const void* cam, const void* globals, uint32_t layout, uint32_t W, uint32_t H,
                             const void* const* planes, const uint64_t* pitch, const void* lights, uint32_t n,
                             uint32_t grid_kind, const uint32_t* lists, const uint32_t* counts, const void* froxel,
                             const void* shadows, const uint32_t* forced_off, const uint32_t* forced_lights,
                             double* out_rgba, uint32_t* flips, uint32_t row0, uint32_t row1, int* bounds) {
    GBufferDesc g = make_gbuf(layout, W, H, planes, pitch);
    GridDesc gr = make_grid(grid_kind, lists, counts, froxel);
    *bounds = 0;
    shade_impl<double>(cam, globals, g, lights, n, gr, out_rgba, nullptr, row0, row1,
                       static_cast<const shadow_oracle::ShadowDesc*>(shadows), bounds, nullptr, forced_off,
                       forced_lights, flips);
}

// oracle_shade_f64 with the pass's optional bindings: shadows (an hl_shadow_maps whose
// pointers are host memory, or NULL) and radiance-cascade probes (an hl_rc_cascade with
// host texels, or NULL). *bounds is set when a shadow layer index is beyond the atlas.
void oracle_shade_ex_f64(const void* cam, const void* globals, uint32_t layout, uint32_t W, uint32_t H,
                         const void* const* planes, const uint64_t* pitch, const void* lights, uint32_t n,
                         uint32_t grid_kind, const uint32_t* lists, const uint32_t* counts, const void* froxel,
                         const void* shadows, const void* rc, double* out_rgba, uint32_t* pair_counts, uint32_t row0,
                         uint32_t row1, int* bounds) {
    GBufferDesc g = make_gbuf(layout, W, H, planes, pitch);
    GridDesc gr = make_grid(grid_kind, lists, counts, froxel);
    *bounds = 0;
    shade_impl<double>(cam, globals, g, lights, n, gr, out_rgba, pair_counts, row0, row1,
                       static_cast<const shadow_oracle::ShadowDesc*>(shadows), bounds,
                       static_cast<const rc_oracle::RcDesc*>(rc));
}

// The reflection draw over a lit target (out_rgba: W*H*4 doubles, updated in place).
void oracle_reflections_f64(const void* cam, const void* globals, uint32_t layout, uint32_t W, uint32_t H,
                            const void* const* planes, const uint64_t* pitch, const void* ssr, uint64_t ssr_pitch,
                            const void* planar, uint64_t planar_pitch, const void* lmuv, uint64_t lmuv_pitch,
                            const void* rc, const void* env, double* out_rgba, int* unsupported) {
    GBufferDesc g = make_gbuf(layout, W, H, planes, pitch);
    ReflectImages im{static_cast<const unsigned char*>(ssr), ssr_pitch, static_cast<const unsigned char*>(planar),
                     planar_pitch, static_cast<const unsigned char*>(lmuv), lmuv_pitch,
                     static_cast<const rc_oracle::RcDesc*>(rc), static_cast<const EnvDesc*>(env)};
    *unsupported = 0;
    reflect_impl<double>(cam, globals, g, im, out_rgba, unsupported);
}

void oracle_shade_f32(const void* cam, const void* globals, uint32_t layout, uint32_t W, uint32_t H, const void* const* planes,
                      const uint64_t* pitch, const void* lights, uint32_t n, uint32_t grid_kind, const uint32_t* lists,
                      const uint32_t* counts, const void* froxel, double* out_rgba, uint32_t* pair_counts, uint32_t row0,
                      uint32_t row1) {
    GBufferDesc g = make_gbuf(layout, W, H, planes, pitch);
    GridDesc gr = make_grid(grid_kind, lists, counts, froxel);
    shade_impl<float>(cam, globals, g, lights, n, gr, out_rgba, pair_counts, row0, row1);
}

// Adjoint on an F32 G-buffer with a froxel (or tile) grid. w: W*H*4 (alpha ignored).
// d_lights: n*7 doubles (pos xyz, intensity, color rgb); d_pix: W*H*5 doubles.
void oracle_shade_fragments_f64(const void* cam, const void* params, const void* frags, uint32_t n, const void* lights,
                                uint32_t n_lights, const uint32_t* entity, const void* transforms, uint32_t n_xf,
                                uint32_t grid_kind, const uint32_t* lists, const uint32_t* counts, const void* froxel,
                                double* out_rgba) {
    FragmentParams fp;
    std::memcpy(&fp, params, sizeof fp);
    GridDesc gr = make_grid(grid_kind, lists, counts, froxel);
    shade_fragments_impl<double>(cam, fp, static_cast<const RawFragment*>(frags), n, lights, n_lights, entity,
                                 static_cast<const RawTransform*>(transforms), n_xf, gr, out_rgba);
}

void oracle_shade_fragments_f32(const void* cam, const void* params, const void* frags, uint32_t n, const void* lights,
                                uint32_t n_lights, const uint32_t* entity, const void* transforms, uint32_t n_xf,
                                uint32_t grid_kind, const uint32_t* lists, const uint32_t* counts, const void* froxel,
                                double* out_rgba) {
    FragmentParams fp;
    std::memcpy(&fp, params, sizeof fp);
    GridDesc gr = make_grid(grid_kind, lists, counts, froxel);
    shade_fragments_impl<float>(cam, fp, static_cast<const RawFragment*>(frags), n, lights, n_lights, entity,
                                static_cast<const RawTransform*>(transforms), n_xf, gr, out_rgba);
}

void oracle_light_dir_from_rotation(const float* rot_deg, double* out) {
    const V3<double> d = light_dir_from_rotation<double>(rot_deg);
    out[0] = d.x;
    out[1] = d.y;
    out[2] = d.z;
}

void oracle_shade_adjoint_f64(const void* cam, const void* globals, uint32_t layout, uint32_t W, uint32_t H,
                              const void* const* planes, const uint64_t* pitch, const void* lights, uint32_t n,
                              uint32_t grid_kind, const uint32_t* lists, const uint32_t* counts, const void* froxel,
                              const double* w, double* d_lights, double* d_pix) {
    GBufferDesc g = make_gbuf(layout, W, H, planes, pitch);
    GridDesc grid = make_grid(grid_kind, lists, counts, froxel);
    Cam<double> c = load_camera<double>(cam);
    RawGlobals gl;
    std::memcpy(&gl, globals, sizeof gl);
    std::vector<RawLight> L(n);
    for (uint32_t i = 0; i < n; ++i) L[i] = load_light(lights, i);
    std::vector<float> tab;
    if (grid.kind == 1) {
        tab.resize(grid.froxel.gz + 1);
        slice_table(grid.froxel, tab.data());
    }
    const double sky[3] = {double(gl.ambient_color[0]) * gl.ambient_intensity, double(gl.ambient_color[1]) * gl.ambient_intensity,
                           double(gl.ambient_color[2]) * gl.ambient_intensity};
    std::memset(d_lights, 0, sizeof(double) * 7 * n);
    int nt = 1;
#ifdef _OPENMP
    nt = omp_get_max_threads();
#endif
    std::vector<std::vector<double>> part(nt, std::vector<double>(size_t(7) * n, 0.0));
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t yy = 0; yy < int64_t(H); ++yy) {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double* gacc = part[tid].data();
        const uint32_t y = uint32_t(yy);
        for (uint32_t x = 0; x < W; ++x) {
            const size_t pix = size_t(y) * W + x;
            double* gp = d_pix + pix * 5;
            for (int q = 0; q < 5; ++q) gp[q] = 0;
            Surface<double> s = load_surface<double>(g, x, y);
            if (!(s.depth < 1.0)) continue;
            V3<double> Nn = normalize(s.n_raw);
            double u = (double(x) + 0.5) / double(W), v = (double(y) + 0.5) / double(H);
            double h[4];
            mat4_mul(c.inv_view_proj, u * 2 - 1, 1 - v * 2, s.depth, 1.0, h);
            D3 P = d3(h[0] / h[3], h[1] / h[3], h[2] / h[3]);
            D3 Vv = d3(c.pos.x - P.x, c.pos.y - P.y, c.pos.z - P.z);
            double vl = std::sqrt(ddot(Vv, Vv));
            Vv = Vv * (1.0 / vl);
            D3 N = d3(Nn.x, Nn.y, Nn.z);
            D3 alb = d3(s.albedo.x, s.albedo.y, s.albedo.z);
            D3 F0 = d3(clampt(s.f0.x, 0.0, 0.999), clampt(s.f0.y, 0.0, 0.999), clampt(s.f0.z, 0.0, 0.999));
            const double* wp = w + pix * 4;
            const uint32_t* list;
            uint32_t count;
            if (grid.kind == 0) {
                const uint32_t tile = (y / kTile) * gl.num_tiles_x + x / kTile;
                count = grid.counts[tile];
                list = grid.lists + size_t(tile) * kMaxPerTile;
            } else {
                double d = view_depth(s.depth, c.near_, c.far_);
                uint32_t f = froxel_of_pixel<double>(grid.froxel, tab.data(), x, y, d);
                count = grid.counts[f + 1] - grid.counts[f];
                list = grid.lists + grid.counts[f];
            }
            for (uint32_t j = 0; j < count; ++j) {
                const uint32_t idx = list[j];
                if (idx >= n) continue;
                double gll[7] = {0, 0, 0, 0, 0, 0, 0};
                pair_adjoint(L[idx], P, N, Vv, alb, s.rough, s.metal, !s.has_f0, F0, wp, gll, gp);
                for (int q = 0; q < 7; ++q) gacc[size_t(idx) * 7 + q] += gll[q];
            }
            // ambient: hemi * ao, hemi = mix(ground, sky, t) * albedo
            double t = N.y * 0.5 + 0.5;
            for (int ch = 0; ch < 3; ++ch) {
                double hemi = (sky[ch] * 0.15) * (1 - t) + sky[ch] * t;
                gp[ch] += wp[ch] * hemi * s.ao;
            }
        }
    }
    for (int t = 0; t < nt; ++t)
        for (size_t q = 0; q < size_t(7) * n; ++q) d_lights[q] += part[t][q];
}

}  // extern "C"
