// gbuffer_write.cpp — CPU restatement of the fragment stage of Helio's GBufferPass
// (crates/passes/3d/helio-pass-gbuffer/shaders/gbuffer.wgsl:287-497, default PBR
// template) in double precision.
//
// TEST INFRASTRUCTURE ONLY: the checker for hl_write_gbuffer. Only tests/ and
// bench.py's error report load it; the product never links or calls it.
//
// Parity status: UNPINNED against the reference's own execution (WGSL through wgpu on
// a graphics driver, unavailable on these machines). The restatement follows the
// shader line by line; the texture sampling follows the Vulkan / WebGPU definition of
// level-0 sampling (texel coordinate u*W - 0.5, floor, fraction; per-coordinate
// repeat / clamp-to-edge / mirrored-repeat; bilinear blend; sRGB decoded per texel
// before filtering). The texel coordinate is taken as the single f32 rounding of
// u*W - 0.5, and select_uv (gbuffer.wgsl:287-297) runs in f32 without contraction
// (this file is compiled with -ffp-contract=off), because the shader computes UVs in
// f32; everything after the texel coordinate is f64, except the velocity, a difference
// of two pixel coordinates that the shader forms in f32 and that is restated in f32 in
// the same operation order. Outputs are the f64 values before the targets'
// quantisation.

#include <cmath>
#include <cstdint>
#include <cstring>

namespace {

struct TexDesc {  // hl_texture (include/helio_gb300.h), texels in host memory here
    const void* texels;
    uint64_t pitch;
    uint32_t width, height, format, address_u, address_v, filter;
};
static_assert(sizeof(TexDesc) == 40, "hl_texture is 40 bytes");

struct D4 {
    double x, y, z, w;
};

constexpr uint32_t kNoTexture = 0xFFFFFFFFu;
constexpr uint32_t kNoFragment = 0xFFFFFFFFu;

double half_bits_to_double(uint16_t h) {
    const uint32_t s = h >> 15, e = (h >> 10) & 31u, m = h & 1023u;
    double v;
    if (e == 0) v = std::ldexp(double(m), -24);
    else if (e == 31) v = m ? NAN : INFINITY;
    else v = std::ldexp(double(m | 1024u), int(e) - 25);
    return s ? -v : v;
}

double srgb_to_linear(double c) { return c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4); }

// Address modes on an integer texel coordinate (Vulkan spec, "Texel Coordinate Systems").
long long wrap(long long i, long long n, uint32_t mode) {
    if (mode == 1) return i < 0 ? 0 : (i >= n ? n - 1 : i);  // clamp to edge
    const long long period = mode == 2 ? 2 * n : n;
    long long m = i % period;
    if (m < 0) m += period;
    if (mode == 2 && m >= n) m = period - 1 - m;  // mirrored repeat
    return m;
}

D4 fetch(const TexDesc& t, long long ix, long long iy) {
    const unsigned char* p = static_cast<const unsigned char*>(t.texels) + t.pitch * uint64_t(iy);
    switch (t.format) {
        case 3: {
            float v[4];
            std::memcpy(v, p + 16 * ix, 16);
            return D4{v[0], v[1], v[2], v[3]};
        }
        case 2: {
            uint16_t v[4];
            std::memcpy(v, p + 8 * ix, 8);
            return D4{half_bits_to_double(v[0]), half_bits_to_double(v[1]), half_bits_to_double(v[2]),
                      half_bits_to_double(v[3])};
        }
        default: {
            const unsigned char* c = p + 4 * ix;
            if (t.format == 1)
                return D4{srgb_to_linear(c[0] / 255.0), srgb_to_linear(c[1] / 255.0), srgb_to_linear(c[2] / 255.0),
                          c[3] / 255.0};
            return D4{c[0] / 255.0, c[1] / 255.0, c[2] / 255.0, c[3] / 255.0};
        }
    }
}

D4 sample(const TexDesc& t, float u, float v) {
    const long long W = t.width, H = t.height;
    if (t.filter == 0) {
        const double fx = std::floor(double(u * float(W))), fy = std::floor(double(v * float(H)));
        return fetch(t, wrap((long long)fx, W, t.address_u), wrap((long long)fy, H, t.address_v));
    }
    const double fx = double(std::fmaf(u, float(W), -0.5f)), fy = double(std::fmaf(v, float(H), -0.5f));
    const double x0 = std::floor(fx), y0 = std::floor(fy);
    const double ax = fx - x0, ay = fy - y0;
    const long long i0 = (long long)x0, j0 = (long long)y0;
    const D4 a = fetch(t, wrap(i0, W, t.address_u), wrap(j0, H, t.address_v));
    const D4 b = fetch(t, wrap(i0 + 1, W, t.address_u), wrap(j0, H, t.address_v));
    const D4 c = fetch(t, wrap(i0, W, t.address_u), wrap(j0 + 1, H, t.address_v));
    const D4 d = fetch(t, wrap(i0 + 1, W, t.address_u), wrap(j0 + 1, H, t.address_v));
    auto mix = [](double p, double q, double s) { return p * (1.0 - s) + q * s; };
    D4 r;
    r.x = mix(mix(a.x, b.x, ax), mix(c.x, d.x, ax), ay);
    r.y = mix(mix(a.y, b.y, ax), mix(c.y, d.y, ax), ay);
    r.z = mix(mix(a.z, b.z, ax), mix(c.z, d.z, ax), ay);
    r.w = mix(mix(a.w, b.w, ax), mix(c.w, d.w, ax), ay);
    return r;
}

struct Ctx {
    const unsigned char* mtex;  // GpuMaterialTextures of the pixel's material
    const TexDesc* tex;
    uint32_t n_tex;
    int* bounds;
};

float f32_at(const unsigned char* p, int off) {
    float v;
    std::memcpy(&v, p + off, 4);
    return v;
}
uint32_t u32_at(const unsigned char* p, int off) {
    uint32_t v;
    std::memcpy(&v, p + off, 4);
    return v;
}

// sample_texture (gbuffer.wgsl:300-306) with select_uv (:287-297) in f32.
D4 sample_slot(const Ctx& c, int slot, float u, float v, D4 fallback) {
    const unsigned char* s = c.mtex + 48 * slot;
    const uint32_t idx = u32_at(s, 0);
    if (idx == kNoTexture) return fallback;
    if (idx >= c.n_tex) {
        *c.bounds = 1;
        return fallback;
    }
    const float ox = f32_at(s, 16), oy = f32_at(s, 20), sz = f32_at(s, 24), sw = f32_at(s, 28);
    const float rs = f32_at(s, 32), rc = f32_at(s, 36);
    const float sx = u * sz, sy = v * sw;
    const float rx = sx * rc - sy * rs;
    const float ry = sx * rs + sy * rc;
    return sample(c.tex[idx], rx + ox, ry + oy);
}

void normalize3(double& x, double& y, double& z) {
    const double l = std::sqrt(x * x + y * y + z * z);
    x /= l;
    y /= l;
    z /= l;
}

double clampd(double x, double lo, double hi) { return x < lo ? lo : (x > hi ? hi : x); }

}  // namespace

extern "C" {

// Per pixel (x, y), out[(y*W + x)*20 + k] holds the f64 values of the targets before
// quantisation: albedo 0-3, normal 4-7, orm 8-11, emissive 12-15, lightmap_uv 16-17,
// velocity 18-19 (sss and extra are zero in the default template). written[y*W + x] is 1
// when fs_main writes the pixel and 0 when it is discarded or uncovered. *bounds is set
// to 1 when a material id or texture index is out of range.
void oracle_write_gbuffer(const void* globals, const void* surfaces, uint64_t surfaces_pitch, const void* materials,
                          const void* material_textures, uint32_t n_materials, const void* textures,
                          uint32_t n_textures, uint32_t W, uint32_t H, double* out, uint8_t* written, int* bounds) {
    const uint32_t debug = u32_at(static_cast<const unsigned char*>(globals), 80);
    const TexDesc* tex = static_cast<const TexDesc*>(textures);
    *bounds = 0;
    for (uint32_t y = 0; y < H; ++y) {
        for (uint32_t x = 0; x < W; ++x) {
            double* o = out + (size_t(y) * W + x) * 20;
            for (int k = 0; k < 20; ++k) o[k] = 0.0;
            uint8_t& wr = written[size_t(y) * W + x];
            wr = 0;
            const unsigned char* r = static_cast<const unsigned char*>(surfaces) + surfaces_pitch * y + 64ull * x;
            const uint32_t mid = u32_at(r, 28);
            if (mid == kNoFragment) continue;
            if (mid >= n_materials) {
                *bounds = 1;
                continue;
            }
            const float u = f32_at(r, 32), v = f32_at(r, 36);
            // compute_velocity (gbuffer.wgsl:417-423), in f32 as the shader computes it (a
            // difference of two pixel coordinates); clip_position.xy is the pixel centre
            const float pw = f32_at(r, 60);
            const float pnx = f32_at(r, 48) / pw, pny = f32_at(r, 52) / pw;
            o[18] = double((float(x) + 0.5f) - (pnx * 0.5f + 0.5f) * float(W));
            o[19] = double((float(y) + 0.5f) - (0.5f - pny * 0.5f) * float(H));
            const unsigned char* mat = static_cast<const unsigned char*>(materials) + 96ull * mid;
            const Ctx c{static_cast<const unsigned char*>(material_textures) + 352ull * mid, tex, n_textures, bounds};
            const D4 one{1, 1, 1, 1};
            wr = 1;
            if (debug == 1 || debug == 2) {  // gbuffer.wgsl:431-459
                D4 a{u, v, 0.0, 1.0};
                if (debug == 2) {
                    const D4 b = sample_slot(c, 0, u, v, one);
                    a = D4{b.x, b.y, b.z, 1.0};
                }
                o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
                o[6] = 1.0;
                continue;
            }
            const D4 base = sample_slot(c, 0, u, v, one);
            const double alb[4] = {f32_at(mat, 0) * base.x, f32_at(mat, 4) * base.y, f32_at(mat, 8) * base.z,
                                   f32_at(mat, 12) * base.w};
            double gx = f32_at(r, 0), gy = f32_at(r, 4), gz = f32_at(r, 8);
            normalize3(gx, gy, gz);
            const D4 orm = sample_slot(c, 2, u, v, one);
            const double rough = clampd(f32_at(mat, 32) * orm.y, 0.045, 1.0);
            const double metal = clampd(f32_at(mat, 36) * orm.z, 0.0, 1.0);
            if (debug == 3) {  // gbuffer.wgsl:461-478
                for (int k = 0; k < 4; ++k) o[k] = alb[k];
                o[4] = gx; o[5] = gy; o[6] = gz;
                o[8] = 1.0; o[9] = rough; o[10] = metal;
                continue;
            }
            // default_pbr_surface (gbuffer.wgsl:333-364)
            const double alpha = alb[3];
            const double normal_scale = f32_at(c.mtex, 336), occ_strength = f32_at(c.mtex, 340);
            const double cutoff = f32_at(c.mtex, 344);
            if (alpha <= 0.001 || alpha < cutoff) {  // :484-485
                wr = 0;
                continue;
            }
            double nx = gx, ny = gy, nz = gz;
            if ((u32_at(mat, 72) & (1u << 3)) != 0 && u32_at(c.mtex, 48) != kNoTexture) {
                const double tw[3] = {f32_at(r, 16), f32_at(r, 20), f32_at(r, 24)};
                const double td = tw[0] * gx + tw[1] * gy + tw[2] * gz;
                double tx = tw[0] - td * gx, ty = tw[1] - td * gy, tz = tw[2] - td * gz;
                normalize3(tx, ty, tz);
                const double bsg = f32_at(r, 12);
                const double bx = (gy * tz - gz * ty) * bsg, by = (gz * tx - gx * tz) * bsg,
                             bz = (gx * ty - gy * tx) * bsg;
                const D4 ns = sample_slot(c, 1, u, v, D4{0.5, 0.5, 1.0, 1.0});
                const double sx = (ns.x * 2.0 - 1.0) * normal_scale, sy = (ns.y * 2.0 - 1.0) * normal_scale,
                             sz = ns.z * 2.0 - 1.0;
                nx = tx * sx + bx * sy + gx * sz;
                ny = ty * sx + by * sy + gy * sz;
                nz = tz * sx + bz * sy + gz * sz;
                normalize3(nx, ny, nz);
            }
            const D4 occ = sample_slot(c, 4, u, v, one);
            const D4 em = sample_slot(c, 3, u, v, one);
            const double ao = 1.0 + (occ.x - 1.0) * occ_strength;
            double f0[3];
            if (u32_at(mat, 68) == 1) {  // resolve_specular_f0, specular workflow (:315-321)
                const D4 sc = sample_slot(c, 5, u, v, one);
                const D4 sw = sample_slot(c, 6, u, v, one);
                const double ior = f32_at(mat, 40) < 1.0f ? 1.0 : double(f32_at(mat, 40));
                const double q = (ior - 1.0) / (ior + 1.0);
                const double k = f32_at(mat, 44) * sw.w;
                f0[0] = k * sc.x * (q * q);
                f0[1] = k * sc.y * (q * q);
                f0[2] = k * sc.z * (q * q);
            } else {  // metallic workflow (:324-328)
                for (int i = 0; i < 3; ++i) f0[i] = clampd(0.04 * (1.0 - metal) + alb[i] * metal, 0.0, 0.999);
            }
            const double ew = f32_at(mat, 28);
            o[0] = alb[0]; o[1] = alb[1]; o[2] = alb[2]; o[3] = alpha;
            o[4] = nx; o[5] = ny; o[6] = nz; o[7] = f0[0];
            o[8] = ao; o[9] = rough; o[10] = metal; o[11] = f0[1];
            o[12] = f32_at(mat, 16) * ew * em.x; o[13] = f32_at(mat, 20) * ew * em.y;
            o[14] = f32_at(mat, 24) * ew * em.z; o[15] = f0[2];
            o[16] = f32_at(r, 40); o[17] = f32_at(r, 44);
        }
    }
}

}  // extern "C"
