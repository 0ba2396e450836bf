/*
 * hl_flops.h — algorithmic operation counts of the deferred-lighting path, used as the
 * numerator of the FP32 roofline fraction. Each IEEE operation of the reference's
 * formulas (add, sub, mul, div, sqrt, min, max, compare, select; an fma counts 2) is
 * counted once, as written in deferred_lighting.wgsl / pbr_eval.wgsl for a point light,
 * independent of how the kernels compute it.
 *
 *   FLOPs(frame) = listed_pairs * HL_FLOPS_CULL + full_pairs * HL_FLOPS_FULL
 *                + lit_pixels * HL_FLOPS_PIXEL
 *
 * listed_pairs: (pixel, light) pairs of the pixels' lists; full_pairs: pairs that pass
 * the range, NdL == 0 and radiance < 0.002 cuts; lit_pixels: pixels with depth < 1.
 */
#ifndef HL_FLOPS_H
#define HL_FLOPS_H

/* Light-loop range test (deferred_lighting.wgsl:1128-1131):
 * to_light 3 sub, length 3 mul + 2 add + 1 sqrt, compare 1. */
#define HL_FLOPS_CULL 10

/* pbr_direct_light for a point light (deferred_lighting.wgsl:699-820, pbr_eval.wgsl):
 * radiance/attenuation 29, NdL + cuts 10, H 12, Fresnel 21, kD 7, NdV 6, GGX D 16,
 * Smith G 29, specular 10, diffuse 6, combine 12, accumulate 3. */
#define HL_FLOPS_FULL 161

/* Per-pixel setup and composition of fs_main (deferred_lighting.wgsl:991-1258):
 * normalize N 9, NDC 8, inv_view_proj product 28, divide by w 3, F0 clamp 6,
 * V 12, NdV 6, depth test 1, hemisphere ambient + composition 32. */
#define HL_FLOPS_PIXEL 105

#endif /* HL_FLOPS_H */
