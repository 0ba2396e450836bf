// hl_precise.cuh — the precise re-evaluation of one (pixel, light) pair that the
// FP16 G-buffer's fast shading path hands over when its guard flags the pair as
// ill-conditioned (grazing light, very close light, end of the range falloff), or when
// the pixel itself is seen at a grazing angle. Shared by the shading kernels.
#pragma once

#include "hl_common.cuh"
#include "hl_shade_math.cuh"

namespace hl {

using namespace sm;

// Precise re-evaluation of an ill-conditioned pair of the fast path: the pixel's
// position as a camera-relative double-float (the light's rounding residual r folded
// into its lo part), compensated NdV and NdL. Rare; kept out of line.
static __device__ __noinline__ int precise_pair(const GpuCamera* cam, uint32_t x, uint32_t y, float W, float H,
                                                float depth, const Pixel& pin, float ar, float ag, float ab,
                                                const ShadeLight& l, float rx, float ry, float rz, float& cr,
                                                float& cg, float& cb) {
    Pixel p = pin;
    const float camx = cam->position_near[0], camy = cam->position_near[1], camz = cam->position_near[2];
    reconstruct<true, false>(cam->inv_view_proj, x, y, W, H, depth, p.Px, p.Py, p.Pz, p.Plx, p.Ply, p.Plz);
    const DF ax = two_sum(p.Px, -camx), ay = two_sum(p.Py, -camy), az = two_sum(p.Pz, -camz);
    const DF bx = two_sum(ax.hi, ax.lo + p.Plx), by = two_sum(ay.hi, ay.lo + p.Ply), bz = two_sum(az.hi, az.lo + p.Plz);
    p.Px = bx.hi; p.Plx = bx.lo - rx;
    p.Py = by.hi; p.Ply = by.lo - ry;
    p.Pz = bz.hi; p.Plz = bz.lo - rz;
    // V = -(true P): the camera sits at minus the residual
    finish_pixel<true>(p, p.nrx, p.nry, p.nrz, ar, ag, ab, p.rough, p.metal, p.f0r, p.f0g, p.f0b, -rx, -ry, -rz);
    const PixelBrdf pb = pixel_brdf(p);
    return eval<true, false>(p, pb, l, cr, cg, cb);
}

}  // namespace hl
