// hl_shade_math.cuh — f32 per-pixel and per-(pixel, light) shading math of
// fs_main / pbr_direct_light (deferred_lighting.wgsl:699-820, 991-1259) and
// pbr_eval.wgsl:6-66, written for accuracy against a float64 evaluation of the same
// formulas. Compiles as CUDA device code and as plain C++ (host emulation).
//
// Accuracy measures (each keeps the result within ~1e-6 relative of the float64
// evaluation where the reference's own f32 formulation loses digits):
//  * world position: inv_view_proj * (ndc, depth, 1) as a compensated dot product
//    (Ogita-Rump-Oishi Dot2) with the pixel-centre NDC carried as a double-float,
//    renormalised, then P = h.xyz / h.w kept as hi + lo. At depth ~100 the plain f32
//    product loses ~1e-4 relative to cancellation in h.w.
//  * to_light = (light.pos - P.hi) - P.lo, and the range falloff
//    1 - (d/r)^4 = (r^2 - d^2)(r^2 + d^2)/r^4 with r^2 - d^2 from double-float
//    squares, so lights near the edge of their range keep their relative accuracy.
//  * GGX denominator NdH^2 (a^2 - 1) + 1 = |N x H|^2 + a^2 NdH^2 for unit N, H (no
//    cancellation at the highlight of smooth surfaces).
// The PRECISE=false variant (FP16 G-buffers, 2e-3 tolerance) skips the first two.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define HL_HD __host__ __device__ __forceinline__
#else
#define HL_HD inline
#include <cmath>
#endif

namespace hl {
namespace sm {

constexpr float kPi = 3.14159265359f;      // pbr_eval.wgsl:6
constexpr float kInvPi = 1.0f / 3.14159265359f;
constexpr float kRadianceCut = 0.002f;     // deferred_lighting.wgsl:781

HL_HD float fma_(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return std::fmaf(a, b, c);
#endif
}
HL_HD float mul_(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
HL_HD float add_(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
HL_HD float div_(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}
// Reciprocal and reciprocal square root: correctly rounded reciprocal, hardware rsqrt.
HL_HD float rcp_(float x) {
#if defined(__CUDA_ARCH__)
    return __frcp_rn(x);
#else
    return 1.0f / x;
#endif
}
HL_HD float rsqrt_(float x) {
#if defined(__CUDA_ARCH__)
    return rsqrtf(x);
#else
    return 1.0f / std::sqrt(x);
#endif
}
// Reciprocal from the hardware approximation refined by one Newton-Raphson step
// (r' = r + r(1 - x r)), within ~1 ulp; the division a/b as a * rcpn_(b) is within
// ~2 ulp. Used on the shading path where the f64 comparison tolerates it.
HL_HD float rcpn_(float x) {
#if defined(__CUDA_ARCH__)
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return __fmaf_rn(__fmaf_rn(-x, r, 1.0f), r, r);
#else
    return 1.0f / x;
#endif
}
HL_HD float divn_(float a, float b) { return a * rcpn_(b); }
HL_HD float fmax_(float a, float b) { return a < b ? b : a; }
HL_HD float fmin_(float a, float b) { return b < a ? b : a; }
HL_HD float clamp01(float x) { return fmin_(fmax_(x, 0.0f), 1.0f); }

// ---- error-free transformations -------------------------------------------------
struct DF {
    float hi, lo;
};
HL_HD DF two_sum(float a, float b) {
    float s = add_(a, b);
    float bb = add_(s, -a);
    float e = add_(add_(a, -add_(s, -bb)), add_(b, -bb));
    return DF{s, e};
}
HL_HD DF two_prod(float a, float b) {
    float p = mul_(a, b);
    return DF{p, fma_(a, b, -p)};
}

// Unit vector of the double-float vector (x + xl, y + yl, z + zl), as double-floats
// accurate to ~2^-44: |v|^2 as a double-float, an f32 rsqrt refined by one Newton step
// whose residual 1 - |v|^2 r^2 is formed in double-float arithmetic.
HL_HD void df_unit(float x, float xl, float y, float yl, float z, float zl, float& ux, float& uxl, float& uy,
                   float& uyl, float& uz, float& uzl) {
    const DF qx = two_prod(x, x), qy = two_prod(y, y), qz = two_prod(z, z);
    const DF a = two_sum(qx.hi, qy.hi), b = two_sum(a.hi, qz.hi);
    const float lo = (a.lo + b.lo) + (qx.lo + qy.lo + qz.lo) + 2.0f * fma_(x, xl, fma_(y, yl, z * zl));
    const DF s = two_sum(b.hi, lo);
    const float r = rsqrt_(s.hi);
    const DF r2 = two_prod(r, r);
    const DF p1 = two_prod(s.hi, r2.hi);
    const float e = ((1.0f - p1.hi) - p1.lo) - fma_(s.hi, r2.lo, s.lo * r2.hi);  // 1 - |v|^2 r^2
    const float rl = r * e * 0.5f;                                                // r (1 + e/2) = r + rl
    const DF px = two_prod(x, r), py = two_prod(y, r), pz = two_prod(z, r);
    ux = px.hi;
    uy = py.hi;
    uz = pz.hi;
    uxl = px.lo + fma_(x, rl, xl * r);
    uyl = py.lo + fma_(y, rl, yl * r);
    uzl = pz.lo + fma_(z, rl, zl * r);
}

// ---- per-pixel surface ------------------------------------------------------------
struct Pixel {
    float Px, Py, Pz;      // world position (hi)
    float Plx, Ply, Plz;   // world position (lo)
    float Nx, Ny, Nz;      // unit normal
    float Vx, Vy, Vz;      // unit view vector
    float f0r, f0g, f0b;   // clamped F0
    float dr, dg, db;      // albedo / pi
    float rough, metal;
    float NdV;             // max(dot(N,V), 0)
    float nrx, nry, nrz;   // normal as stored (before normalisation)
    float inv_n;           // 1 / |stored normal|
};

// Derived per-pixel BRDF constants hoisted out of the light loop.
struct PixelBrdf {
    float a2;          // roughness^4
    float k, omk;      // (r+1)^2/8, 1-k
    float gv;          // Schlick-GGX for the view
    float one_m_metal;
    float nv4;         // 4*NdV
    float vlx, vly, vlz;  // low words of V as a double-float unit vector (df_view), else 0
};

HL_HD PixelBrdf pixel_brdf(const Pixel& p) {
    PixelBrdf b;
    const float a = p.rough * p.rough;
    b.a2 = a * a;
    const float r1 = p.rough + 1.0f;
    b.k = (r1 * r1) * 0.125f;
    b.omk = 1.0f - b.k;
    b.gv = divn_(p.NdV, fma_(p.NdV, b.omk, b.k + 0.0001f));
    b.one_m_metal = 1.0f - p.metal;
    b.nv4 = 4.0f * p.NdV;
    b.vlx = b.vly = b.vlz = 0.0f;
    return b;
}

// V = normalize(camera - P) as a double-float unit vector from the pixel's double-float
// position: p.V* its high words, b.vl* its low words (read by eval<true> for lights
// nearly opposite the view).
HL_HD void df_view(Pixel& p, PixelBrdf& b, float cx, float cy, float cz) {
    const DF ux = two_sum(cx, -p.Px), uy = two_sum(cy, -p.Py), uz = two_sum(cz, -p.Pz);
    const DF vx = two_sum(ux.hi, ux.lo - p.Plx), vy = two_sum(uy.hi, uy.lo - p.Ply), vz = two_sum(uz.hi, uz.lo - p.Plz);
    df_unit(vx.hi, vx.lo, vy.hi, vy.lo, vz.hi, vz.lo, p.Vx, b.vlx, p.Vy, b.vly, p.Vz, b.vlz);
}

// Camera-relative reconstruction rows: with M = inv_view_proj and c the camera
// position, P - c = (M_r - c_r M_3) v / (M_3 v) for v = (ndc, depth, 1). The rows
// M_r - c_r M_3 are each one fma (exact product, one rounding), so they carry no
// cancellation for points far from the origin. rel[r*4 + k] = row r, w[k] = M_3.
HL_HD void camera_relative_rows(const float* m, float cx, float cy, float cz, float* rel, float* w) {
    const float c[3] = {cx, cy, cz};
    for (int k = 0; k < 4; ++k) w[k] = m[4 * k + 3];
    for (int r = 0; r < 3; ++r)
        for (int k = 0; k < 4; ++k) rel[r * 4 + k] = fma_(-c[r], m[4 * k + 3], m[4 * k + r]);
}

// P - camera for a pixel centre, from the camera-relative rows (FMA rows; the
// DirectX-style perspective makes the w row a single-rounding fma of depth).
HL_HD void reconstruct_relative(const float* rel, const float* w, float ndc_x, float ndc_y, float depth, float& Px,
                                float& Py, float& Pz) {
    const float hw = fma_(w[2], depth, fma_(w[1], ndc_y, fma_(w[0], ndc_x, w[3])));
    const float iw = rcpn_(hw);
    float h[3];
    for (int r = 0; r < 3; ++r)
        h[r] = fma_(rel[r * 4 + 2], depth, fma_(rel[r * 4 + 1], ndc_y, fma_(rel[r * 4 + 0], ndc_x, rel[r * 4 + 3])));
    Px = h[0] * iw;
    Py = h[1] * iw;
    Pz = h[2] * iw;
}

// World position of a pixel centre: inv_view_proj (column major, 16 floats) times
// (ndc_x, ndc_y, depth, 1), ndc of pixel centre (x+0.5, y+0.5) of a W x H target.
// RENORM (precise): renormalise the rows before the division, which keeps P to ~2^-44
// relative (without it ~4e-10 at far depth, ample for the FP16 G-buffer's paths).
template <bool PRECISE, bool RENORM = true>
HL_HD void reconstruct(const float* m, uint32_t x, uint32_t y, float W, float H, float depth, float& Px, float& Py,
                       float& Pz, float& Plx, float& Ply, float& Plz) {
    if (!PRECISE) {
        // uv*2-1 and 1-uv*2 (deferred_lighting.wgsl:1043-1047) with FMA rows.
        const float ux = div_(float(x) + 0.5f, W), uy = div_(float(y) + 0.5f, H);
        const float nx = fma_(ux, 2.0f, -1.0f), ny = fma_(uy, -2.0f, 1.0f);
        float h[4];
        for (int r = 0; r < 4; ++r) h[r] = fma_(m[8 + r], depth, fma_(m[4 + r], ny, fma_(m[r], nx, m[12 + r])));
        const float iw = rcp_(h[3]);
        Px = h[0] * iw;
        Py = h[1] * iw;
        Pz = h[2] * iw;
        Plx = Ply = Plz = 0.0f;
        return;
    }
    // ndc_x = (2x+1)/W - 1 and ndc_y = 1 - (2y+1)/H as double-floats.
    const float numx = float(2u * x + 1u), numy = float(2u * y + 1u);
    const float qx = div_(numx, W), qy = div_(numy, H);
    const float qxl = fma_(-qx, W, numx) * rcp_(W);
    const float qyl = fma_(-qy, H, numy) * rcp_(H);
    DF ndx = two_sum(qx, -1.0f);
    ndx.lo += qxl;
    DF ndy = two_sum(1.0f, -qy);
    ndy.lo -= qyl;
    float hh[4], hl[4];
    for (int r = 0; r < 4; ++r) {
        // Dot2 over (m0*ndx.hi, m1*ndy.hi, m2*depth) starting from m3; lo terms added.
        float p = m[12 + r], s = 0.0f;
        DF t = two_prod(m[r], ndx.hi);
        DF u = two_sum(p, t.hi);
        p = u.hi;
        s = s + (u.lo + t.lo);
        t = two_prod(m[4 + r], ndy.hi);
        u = two_sum(p, t.hi);
        p = u.hi;
        s = s + (u.lo + t.lo);
        t = two_prod(m[8 + r], depth);
        u = two_sum(p, t.hi);
        p = u.hi;
        s = s + (u.lo + t.lo);
        s = fma_(m[r], ndx.lo, s);
        s = fma_(m[4 + r], ndy.lo, s);
        // renormalise: after cancellation (the w row at far depth) s can be ~1e-5 of p,
        // and the quotient's correction below assumes |lo| <= ulp(hi)
        if (RENORM) {
            const DF n = two_sum(p, s);
            hh[r] = n.hi;
            hl[r] = n.lo;
        } else {
            hh[r] = p;
            hl[r] = s;
        }
    }
    const float w = hh[3], wl = hl[3];
    float* outs[3] = {&Px, &Py, &Pz};
    float* outl[3] = {&Plx, &Ply, &Plz};
    const float iw = rcp_(w);
    for (int r = 0; r < 3; ++r) {
        const float q = div_(hh[r], w);
        // residual of (hh + hl) / (w + wl) around q
        const float res = fma_(-q, w, hh[r]) + fma_(-q, wl, hl[r]);
        // renormalise so that |lo| <= ulp(hi)/2
        const DF n = two_sum(q, res * iw);
        *outs[r] = n.hi;
        *outl[r] = n.lo;
    }
}

// Finishes a Pixel from decoded G-buffer values (albedo, roughness, metallic, raw
// normal, F0) and the camera position.
template <bool PRECISE>
HL_HD void finish_pixel(Pixel& p, float nx, float ny, float nz, float ar, float ag, float ab, float rough, float metal,
                        float f0r, float f0g, float f0b, float cx, float cy, float cz) {
    const float in = rsqrt_(fma_(nz, nz, fma_(ny, ny, nx * nx)));
    p.nrx = nx;
    p.nry = ny;
    p.nrz = nz;
    p.inv_n = in;
    p.Nx = nx * in;
    p.Ny = ny * in;
    p.Nz = nz * in;
    if (PRECISE) {
        // V = cam - P as normalised double-floats
        const DF ux = two_sum(cx, -p.Px), uy = two_sum(cy, -p.Py), uz = two_sum(cz, -p.Pz);
        const DF vx = two_sum(ux.hi, ux.lo - p.Plx), vy = two_sum(uy.hi, uy.lo - p.Ply),
                 vz = two_sum(uz.hi, uz.lo - p.Plz);
        const float iv = rsqrt_(fma_(vz.hi, vz.hi, fma_(vy.hi, vy.hi, vx.hi * vx.hi)));
        p.Vx = vx.hi * iv;
        p.Vy = vy.hi * iv;
        p.Vz = vz.hi * iv;
        // NdV = (n_raw . v) / (|n_raw| |v|) with a compensated dot product: at grazing
        // view angles the specular term is proportional to NdV.
        DF d = two_prod(nx, vx.hi);
        const DF t1 = two_prod(ny, vy.hi), t2 = two_prod(nz, vz.hi);
        const DF s1 = two_sum(d.hi, t1.hi);
        const DF s2 = two_sum(s1.hi, t2.hi);
        float lo = d.lo + t1.lo + t2.lo + s1.lo + s2.lo;
        lo = fma_(nx, vx.lo, fma_(ny, vy.lo, fma_(nz, vz.lo, lo)));
        p.NdV = fmax_((s2.hi + lo) * in * iv, 0.0f);
    } else {
        const float vx = cx - p.Px, vy = cy - p.Py, vz = cz - p.Pz;
        const float iv = rsqrt_(fma_(vz, vz, fma_(vy, vy, vx * vx)));
        p.Vx = vx * iv;
        p.Vy = vy * iv;
        p.Vz = vz * iv;
        p.NdV = fmax_(fma_(nz, vz, fma_(ny, vy, nx * vx)) * in * iv, 0.0f);
    }
    p.f0r = fmin_(fmax_(f0r, 0.0f), 0.999f);
    p.f0g = fmin_(fmax_(f0g, 0.0f), 0.999f);
    p.f0b = fmin_(fmax_(f0b, 0.0f), 0.999f);
    p.dr = ar * kInvPi;
    p.dg = ag * kInvPi;
    p.db = ab * kInvPi;
    p.rough = rough;
    p.metal = metal;
}

// F0 of the metallic workflow (gbuffer.wgsl:323-328): clamp(mix(0.04, albedo, m), 0, 0.999)
HL_HD float metallic_f0(float albedo, float metal) { return fma_(albedo, metal, 0.04f * (1.0f - metal)); }

// Octahedral unit-vector decode (Cigolle et al. 2014), z up; not normalised.
HL_HD void oct_decode(float u, float v, float& x, float& y, float& z) {
    z = 1.0f - fabsf(u) - fabsf(v);
    if (z < 0.0f) {
        const float ox = (1.0f - fabsf(v)) * (u >= 0.0f ? 1.0f : -1.0f);
        const float oy = (1.0f - fabsf(u)) * (v >= 0.0f ? 1.0f : -1.0f);
        u = ox;
        v = oy;
    }
    x = u;
    y = v;
}

// Light fields used by shading (from a GpuLight, deferred_lighting.wgsl:70-98).
struct ShadeLight {
    float px, py, pz, range;
    float dx, dy, dz, cos_outer;
    float cr, cg, cb, intensity;
    uint32_t type;
    float cos_inner;
};

// Cheap candidate test of phase 1: inside the range and in front of the surface.
// Returns true when the pair may contribute; the exact cuts are re-applied by eval.
// r2m is the light's squared range widened by a relative margin; pairs whose N.to_light
// is within sqrt(slack2) of zero are kept so the exact NdL cut decides them.
HL_HD bool candidate(float px, float py, float pz, float plx, float ply, float plz, float nx, float ny, float nz,
                     float lx, float ly, float lz, float r2m, float slack2, bool check_ndl) {
    const float tx = (lx - px) - plx, ty = (ly - py) - ply, tz = (lz - pz) - plz;
    const float d2 = fma_(tz, tz, fma_(ty, ty, tx * tx));
    const float ndl = fma_(nz, tz, fma_(ny, ty, nx * tx));
    return (d2 <= r2m) && (!check_ndl || ndl > 0.0f || ndl * ndl <= slack2);
}

// Range test of the reference's light loop (deferred_lighting.wgsl:1128-1131).
HL_HD bool in_range(const Pixel& p, const ShadeLight& l) {
    if (l.type == 0u) return true;
    const float tx = (l.px - p.Px) - p.Plx, ty = (l.py - p.Py) - p.Ply, tz = (l.pz - p.Pz) - p.Plz;
    const float d2 = fma_(tz, tz, fma_(ty, ty, tx * tx));
    return d2 <= l.range * l.range;
}

// Results of eval().
constexpr int kCut = 0;           // a cut applies: no contribution
constexpr int kLit = 1;           // contribution written to out*
constexpr int kNeedsPrecise = 2;  // fast path only: ill-conditioned pair, redo with PRECISE

// Guard of the fast path, for a pixel whose camera-relative position P is a plain f32
// value: its rounding (|P| 2^-24) turns the light direction by |P| 2^-24 / dist. The
// guard G = |P|^2 2^-26 flags the pairs where that moves the result by more than
// ~2^-11 relative: NdL dist < |P| 2^-13, dist < |P| 2^-12, or, near the end of the
// range, falloff * dist < |P| 2^-11. Such pairs are re-evaluated on the precise path.
HL_HD float fast_guard(const Pixel& p) {
    return fma_(p.Pz, p.Pz, fma_(p.Py, p.Py, p.Px * p.Px)) * (1.0f / 67108864.0f);
}
// Pixels with NdV below this are set up on the precise path from the start.
constexpr float kFastMinNdV = 1.0f / 8192.0f;

// pbr_direct_light (deferred_lighting.wgsl:699-820) for a non-anisotropic, non-SSS
// surface, sf = 1. Returns kCut (out* untouched) when a cut applies, kLit with the
// contribution in out*, or — on the fast path with guard > 0 — kNeedsPrecise. `cut` is
// the radiance cut (0.002, :781); 0 disables it, as the Forward+ shader has none.
// DF_HALF (precise evaluations): H from double-float unit vectors when V and L are
// nearly opposite, with V's low words from df_view (b.vl*, 0 without it); the FP16
// path's precise re-evaluation (tolerance 2e-3) passes false.
template <bool PRECISE, bool DF_HALF = PRECISE>
HL_HD int eval(const Pixel& p, const PixelBrdf& b, const ShadeLight& l, float& outr, float& outg, float& outb,
               float guard = 0.0f, float cut = kRadianceCut) {
    float Lx, Ly, Lz, rr, rg, rb;
    float NdL, d2_near = 0.0f, fall_near = 1.0f;
    float tx = -l.dx, ty = -l.dy, tz = -l.dz, ex = 0.0f, ey = 0.0f, ez = 0.0f;  // to_light as hi + lo
    if (l.type == 0u) {
        const float il = rsqrt_(fma_(l.dz, l.dz, fma_(l.dy, l.dy, l.dx * l.dx)));
        Lx = -l.dx * il;
        Ly = -l.dy * il;
        Lz = -l.dz * il;
        rr = l.cr * l.intensity;
        rg = l.cg * l.intensity;
        rb = l.cb * l.intensity;
        NdL = fma_(p.Nz, Lz, fma_(p.Ny, Ly, p.Nx * Lx));
    } else {
        float d2, fall, ntl = 0.0f;
        const float r2 = l.range * l.range;
        if (PRECISE) {
            // to_light = (light - P.hi) - P.lo as normalised double-floats
            const DF ux = two_sum(l.px, -p.Px), uy = two_sum(l.py, -p.Py), uz = two_sum(l.pz, -p.Pz);
            const DF sx = two_sum(ux.hi, ux.lo - p.Plx), sy = two_sum(uy.hi, uy.lo - p.Ply),
                     sz = two_sum(uz.hi, uz.lo - p.Plz);
            ex = sx.lo;
            ey = sy.lo;
            ez = sz.lo;
            tx = sx.hi;
            ty = sy.hi;
            tz = sz.hi;
            // d^2 = sum (s + e)^2 as a double-float
            const DF qx = two_prod(sx.hi, sx.hi), qy = two_prod(sy.hi, sy.hi), qz = two_prod(sz.hi, sz.hi);
            DF acc = two_sum(qx.hi, qy.hi);
            DF acc2 = two_sum(acc.hi, qz.hi);
            float lo = acc.lo + acc2.lo + qx.lo + qy.lo + qz.lo;
            lo = fma_(2.0f * sx.hi, ex, lo);
            lo = fma_(2.0f * sy.hi, ey, lo);
            lo = fma_(2.0f * sz.hi, ez, lo);
            d2 = acc2.hi + lo;
            // r^2 - d^2 as a double-float difference
            const DF rr2 = two_prod(l.range, l.range);
            const DF diff = two_sum(rr2.hi, -acc2.hi);
            const float gap = diff.hi + (diff.lo + (rr2.lo - lo));
            if (gap < 0.0f) return kCut;  // dist > range
            fall = divn_(gap * (r2 + d2), r2 * r2);
            // n_raw . to_light, compensated: at grazing light angles the diffuse and
            // specular terms are proportional to NdL.
            const DF q1 = two_prod(p.nrx, tx), q2 = two_prod(p.nry, ty), q3 = two_prod(p.nrz, tz);
            const DF c1 = two_sum(q1.hi, q2.hi);
            const DF c2 = two_sum(c1.hi, q3.hi);
            float cl = q1.lo + q2.lo + q3.lo + c1.lo + c2.lo;
            cl = fma_(p.nrx, ex, fma_(p.nry, ey, fma_(p.nrz, ez, cl)));
            ntl = c2.hi + cl;
        } else {
            tx = (l.px - p.Px) - p.Plx;
            ty = (l.py - p.Py) - p.Ply;
            tz = (l.pz - p.Pz) - p.Plz;
            d2 = fma_(tz, tz, fma_(ty, ty, tx * tx));
            if (d2 > r2) return kCut;
            const float nd2 = d2 * rcpn_(r2);
            fall = fmax_(0.0f, fma_(-nd2, nd2, 1.0f));
        }
        d2_near = d2;
        fall_near = fall;
        const float inv_d = rsqrt_(d2);
        Lx = tx * inv_d;
        Ly = ty * inv_d;
        Lz = tz * inv_d;
        NdL = PRECISE ? ntl * p.inv_n * inv_d : fma_(p.Nz, Lz, fma_(p.Ny, Ly, p.Nx * Lx));
        float atten = rcpn_(d2 + 0.0001f) * fall;
        if (l.type == 2u) {
            const float cos_a = -fma_(Lz, l.dz, fma_(Ly, l.dy, Lx * l.dx));
            const float t = clamp01(div_(cos_a - l.cos_outer, l.cos_inner - l.cos_outer));
            atten *= t * t * fma_(-2.0f, t, 3.0f);
        }
        const float ia = l.intensity * atten;
        rr = l.cr * ia;
        rg = l.cg * ia;
        rb = l.cb * ia;
    }
    if (!PRECISE && guard > 0.0f && l.type != 0u) {
        const float ndl2d2 = NdL * NdL * d2_near;
        if (ndl2d2 < guard || d2_near < 4.0f * guard || fall_near * fall_near * d2_near < 16.0f * guard)
            return kNeedsPrecise;
    }
    if (!(NdL > 0.0f)) return kCut;
    if (rr < cut && rg < cut && rb < cut) return kCut;
    // H = normalize(V + L)
    float hx = p.Vx + Lx, hy = p.Vy + Ly, hz = p.Vz + Lz;
    if (PRECISE && DF_HALF && fma_(hz, hz, fma_(hy, hy, hx * hx)) < 0.25f) {
        // V and L nearly opposite (H.V < 1/4): the sum cancels and would turn the f32
        // rounding of V and L into an error of H's direction; form it from
        // double-float unit vectors instead
        float lx, lxl, ly, lyl, lz, lzl;
        df_unit(tx, ex, ty, ey, tz, ez, lx, lxl, ly, lyl, lz, lzl);
        const DF sx = two_sum(p.Vx, lx), sy = two_sum(p.Vy, ly), sz = two_sum(p.Vz, lz);
        hx = sx.hi + (sx.lo + (b.vlx + lxl));
        hy = sy.hi + (sy.lo + (b.vly + lyl));
        hz = sz.hi + (sz.lo + (b.vlz + lzl));
    }
    const float ih = rsqrt_(fma_(hz, hz, fma_(hy, hy, hx * hx)));
    const float Hx = hx * ih, Hy = hy * ih, Hz = hz * ih;
    // Fresnel-Schlick
    const float HdV = fmax_(fma_(Hz, p.Vz, fma_(Hy, p.Vy, Hx * p.Vx)), 0.0f);
    const float x = clamp01(1.0f - HdV);
    const float x2 = x * x;
    const float p5 = x2 * x2 * x;
    const float Fr = fma_(1.0f - p.f0r, p5, p.f0r);
    const float Fg = fma_(1.0f - p.f0g, p5, p.f0g);
    const float Fb = fma_(1.0f - p.f0b, p5, p.f0b);
    // GGX: NdH^2 (a2 - 1) + 1 = |N x H|^2 + a2 NdH^2
    const float ndh_raw = fma_(p.Nz, Hz, fma_(p.Ny, Hy, p.Nx * Hx));
    float den;
    if (ndh_raw > 0.0f) {
        const float cx = fma_(p.Ny, Hz, -p.Nz * Hy), cy = fma_(p.Nz, Hx, -p.Nx * Hz), cz = fma_(p.Nx, Hy, -p.Ny * Hx);
        const float s2 = fma_(cz, cz, fma_(cy, cy, cx * cx));
        den = fma_(b.a2 * ndh_raw, ndh_raw, s2);
    } else {
        den = 1.0f;
    }
    const float D = divn_(b.a2, fma_(kPi * den, den, 0.0001f));
    // Smith-Schlick G
    const float gl = divn_(NdL, fma_(NdL, b.omk, b.k + 0.0001f));
    const float G = b.gv * gl;
    const float spec = divn_(D * G, fma_(b.nv4, NdL, 0.0001f));
    // (kD * albedo / pi + spec * F) * radiance * NdL
    const float wr = rr * NdL, wg = rg * NdL, wb = rb * NdL;
    outr = fma_((1.0f - Fr) * b.one_m_metal, p.dr, spec * Fr) * wr;
    outg = fma_((1.0f - Fg) * b.one_m_metal, p.dg, spec * Fg) * wg;
    outb = fma_((1.0f - Fb) * b.one_m_metal, p.db, spec * Fb) * wb;
    return kLit;
}

// Adjoint of one (pixel, light) pair of pbr_direct_light. Given w = dLoss/d(out.rgb),
// adds dLoss/d(light position xyz, intensity, colour rgb) to gl[0..6] and
// dLoss/d(pixel albedo rgb, roughness, metallic) to gp[0..4], with the pair's branch
// decisions (range, NdL == 0, radiance < 0.002, clamps) held fixed. f0_from_albedo:
// F0 = clamp(mix(0.04, albedo, metallic)) (FP32/FP16 layouts) so albedo and metallic
// reach F0; the reference layout stores F0. BRDF terms are recomputed here, nothing
// per pair is stored by the forward pass. Returns false when a cut applies.
template <bool PRECISE>
HL_HD bool eval_adjoint(const Pixel& p, const PixelBrdf& b, const ShadeLight& l, float wr, float wg, float wb,
                        bool f0_from_albedo, float* gl, float* gp) {
    // ---- forward, keeping the intermediates ----
    float Lx, Ly, Lz, tx = 0, ty = 0, tz = 0, dist = 0, inv_d = 0, a0 = 0, fall = 1, nd = 0, spot = 1, dspot = 0;
    float NdL, atten;
    if (l.type == 0u) {
        const float il = rsqrt_(fma_(l.dz, l.dz, fma_(l.dy, l.dy, l.dx * l.dx)));
        Lx = -l.dx * il;
        Ly = -l.dy * il;
        Lz = -l.dz * il;
        atten = 1.0f;
        NdL = fma_(p.Nz, Lz, fma_(p.Ny, Ly, p.Nx * Lx));
    } else {
        float d2;
        if (PRECISE) {
            const DF ux = two_sum(l.px, -p.Px), uy = two_sum(l.py, -p.Py), uz = two_sum(l.pz, -p.Pz);
            const DF sx = two_sum(ux.hi, ux.lo - p.Plx), sy = two_sum(uy.hi, uy.lo - p.Ply),
                     sz = two_sum(uz.hi, uz.lo - p.Plz);
            tx = sx.hi;
            ty = sy.hi;
            tz = sz.hi;
        } else {
            tx = (l.px - p.Px) - p.Plx;
            ty = (l.py - p.Py) - p.Ply;
            tz = (l.pz - p.Pz) - p.Plz;
        }
        d2 = fma_(tz, tz, fma_(ty, ty, tx * tx));
        const float r2 = l.range * l.range;
        if (d2 > r2) return false;
        inv_d = rsqrt_(d2);
        dist = d2 * inv_d;
        Lx = tx * inv_d;
        Ly = ty * inv_d;
        Lz = tz * inv_d;
        NdL = fma_(p.Nz, Lz, fma_(p.Ny, Ly, p.Nx * Lx));
        a0 = rcpn_(d2 + 0.0001f);
        nd = dist * rcpn_(l.range);
        const float nd2 = nd * nd;
        fall = fmax_(0.0f, fma_(-nd2, nd2, 1.0f));
        if (l.type == 2u) {
            const float cos_a = -fma_(Lz, l.dz, fma_(Ly, l.dy, Lx * l.dx));
            const float span = l.cos_inner - l.cos_outer;
            const float tt = div_(cos_a - l.cos_outer, span);
            if (tt <= 0.0f) {
                spot = 0.0f;
            } else if (tt >= 1.0f) {
                spot = 1.0f;
            } else {
                spot = tt * tt * fma_(-2.0f, tt, 3.0f);
                dspot = div_(6.0f * tt * (1.0f - tt), span);
            }
        }
        atten = a0 * fall * spot;
    }
    const float ia = l.intensity * atten;
    const float rr = l.cr * ia, rg = l.cg * ia, rb = l.cb * ia;
    if (!(NdL > 0.0f)) return false;
    if (rr < kRadianceCut && rg < kRadianceCut && rb < kRadianceCut) return false;
    const float hx = p.Vx + Lx, hy = p.Vy + Ly, hz = p.Vz + Lz;
    const float ih = rsqrt_(fma_(hz, hz, fma_(hy, hy, hx * hx)));
    const float Hx = hx * ih, Hy = hy * ih, Hz = hz * ih;
    const float hdv = fma_(Hz, p.Vz, fma_(Hy, p.Vy, Hx * p.Vx));
    const float x = clamp01(1.0f - fmax_(hdv, 0.0f));
    const bool x_free = (hdv > 0.0f) && (x > 0.0f) && (x < 1.0f);
    const float x2 = x * x;
    const float p5 = x2 * x2 * x;
    const float F[3] = {fma_(1.0f - p.f0r, p5, p.f0r), fma_(1.0f - p.f0g, p5, p.f0g), fma_(1.0f - p.f0b, p5, p.f0b)};
    const float F0[3] = {p.f0r, p.f0g, p.f0b};
    const float ndh = fma_(p.Nz, Hz, fma_(p.Ny, Hy, p.Nx * Hx));
    float den = 1.0f;
    if (ndh > 0.0f) {
        const float cx = fma_(p.Ny, Hz, -p.Nz * Hy), cy = fma_(p.Nz, Hx, -p.Nx * Hz), cz = fma_(p.Nx, Hy, -p.Ny * Hx);
        den = fma_(b.a2 * ndh, ndh, fma_(cz, cz, fma_(cy, cy, cx * cx)));
    }
    const float Q = fma_(kPi * den, den, 0.0001f);
    const float D = divn_(b.a2, Q);
    const float gld = fma_(NdL, b.omk, b.k + 0.0001f);
    const float glv = divn_(NdL, gld);
    const float G = b.gv * glv;
    const float S = fma_(b.nv4, NdL, 0.0001f);
    const float spec = divn_(D * G, S);
    const float alb[3] = {p.dr * kPi, p.dg * kPi, p.db * kPi};
    const float rad[3] = {rr, rg, rb};
    const float w[3] = {wr, wg, wb};
    const float col[3] = {l.cr, l.cg, l.cb};
    // ---- adjoint ----
    float dNdL = 0.0f, dspec = 0.0f, dp5 = 0.0f, dmetal = 0.0f, datten = 0.0f;
    for (int c = 0; c < 3; ++c) {
        const float kd = (1.0f - F[c]) * b.one_m_metal;
        const float brdf = fma_(kd, alb[c] * kInvPi, spec * F[c]);
        const float drad = w[c] * brdf * NdL;
        dNdL = fma_(w[c] * brdf, rad[c], dNdL);
        const float dbrdf = w[c] * rad[c] * NdL;
        gp[c] += dbrdf * kd * kInvPi;
        const float dkd = dbrdf * alb[c] * kInvPi;
        const float dF = fma_(dbrdf, spec, -dkd * b.one_m_metal);
        dmetal -= dkd * (1.0f - F[c]);
        dspec = fma_(dbrdf, F[c], dspec);
        dp5 = fma_(dF, 1.0f - F0[c], dp5);
        if (f0_from_albedo) {
            const float f0raw = fma_(alb[c], p.metal, 0.04f * (1.0f - p.metal));
            if (f0raw > 0.0f && f0raw < 0.999f) {
                const float dF0 = dF * (1.0f - p5);
                gp[c] = fma_(dF0, p.metal, gp[c]);
                dmetal = fma_(dF0, alb[c] - 0.04f, dmetal);
            }
        }
        // rad_c = col_c * I * atten
        gl[4 + c] = fma_(drad, ia, gl[4 + c]);
        gl[3] = fma_(drad, col[c] * atten, gl[3]);
        datten = fma_(drad, col[c] * l.intensity, datten);
    }
    gp[4] += dmetal;
    // spec = D G / S
    const float dD = dspec * G / S, dG = dspec * D / S, dS = -dspec * spec / S;
    dNdL = fma_(dS, b.nv4, dNdL);
    const float dglv = dG * b.gv, dgv = dG * glv;
    dNdL = fma_(dglv, divn_(gld - NdL * b.omk, gld * gld), dNdL);
    float dk = dglv * divn_(-NdL * (1.0f - NdL), gld * gld);
    // gv = NdV / (NdV (1-k) + k + 1e-4), NdV of the pixel
    const float gvd = fma_(p.NdV, b.omk, b.k + 0.0001f);
    dk = fma_(dgv, divn_(-p.NdV * (1.0f - p.NdV), gvd * gvd), dk);
    float drough = dk * (p.rough + 1.0f) * 0.25f;
    // D = a2 / Q, Q = pi den^2 + 1e-4, den = NdH^2 (a2 - 1) + 1
    float da2 = dD / Q;
    const float dden = -dD * D / Q * 2.0f * kPi * den;
    float dndh = 0.0f;
    if (ndh > 0.0f) {
        da2 = fma_(dden, ndh * ndh, da2);
        dndh = dden * 2.0f * ndh * (b.a2 - 1.0f);
    }
    drough = fma_(da2, 4.0f * p.rough * p.rough * p.rough, drough);
    gp[3] += drough;
    // p5 = x^5, x = clamp(1 - max(H.V, 0))
    const float dhdv = x_free ? -dp5 * 5.0f * x2 * x2 : 0.0f;
    // H = normalize(V + L): dhv = (dH - H (dH.H)) / |hv|, dH = V dhdv + N dndh
    const float dHx = fma_(p.Vx, dhdv, p.Nx * dndh), dHy = fma_(p.Vy, dhdv, p.Ny * dndh),
                dHz = fma_(p.Vz, dhdv, p.Nz * dndh);
    const float hdot = fma_(dHz, Hz, fma_(dHy, Hy, dHx * Hx));
    float dLx = (dHx - Hx * hdot) * ih + p.Nx * dNdL;
    float dLy = (dHy - Hy * hdot) * ih + p.Ny * dNdL;
    float dLz = (dHz - Hz * hdot) * ih + p.Nz * dNdL;
    if (l.type == 0u) return true;  // no dependence on the light position
    // atten = a0 * fall * spot
    float ddist = datten * spot * (fall * (-2.0f * dist) * a0 * a0);
    if (fall > 0.0f) ddist = fma_(datten * spot * a0, -4.0f * nd * nd * nd * rcpn_(l.range), ddist);
    if (l.type == 2u) {
        const float dcos = datten * a0 * fall * dspot;  // cos_a = -L.dir
        dLx = fma_(-l.dx, dcos, dLx);
        dLy = fma_(-l.dy, dcos, dLy);
        dLz = fma_(-l.dz, dcos, dLz);
    }
    // L = t / |t|: dt = (dL - L (dL.L)) / |t| + L ddist
    const float ldot = fma_(dLz, Lz, fma_(dLy, Ly, dLx * Lx));
    gl[0] += fma_(dLx - Lx * ldot, inv_d, Lx * ddist);
    gl[1] += fma_(dLy - Ly * ldot, inv_d, Ly * ddist);
    gl[2] += fma_(dLz - Lz * ldot, inv_d, Lz * ddist);
    return true;
}

// Kahan (compensated) accumulation of one channel.
HL_HD void kahan_add(float& sum, float& comp, float v) {
    const float y = add_(v, -comp);
    const float t = add_(sum, y);
    comp = add_(add_(t, -sum), -y);
    sum = t;
}

}  // namespace sm
}  // namespace hl
