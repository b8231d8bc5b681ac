// exact.cuh -- FP64 arithmetic that reproduces the reference's host results
// bit for bit.  Every operation is an explicitly rounded intrinsic, so the
// compiler cannot contract a multiply and an add into an FMA (the reference
// is built with -std=c99 -O2, which does not contract either).
#pragma once

namespace exact {

// squared distance, summed in axis order from 0.0 (kdtree.c:530-531)
__device__ __forceinline__ double dist2(double ox, double oy, double qx, double qy)
{
    double d0 = __dsub_rn(ox, qx), d1 = __dsub_rn(oy, qy);
    return __dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1));
}

__device__ __forceinline__ double dist3(double ox, double oy, double oz, double qx, double qy, double qz)
{
    double d0 = __dsub_rn(ox, qx), d1 = __dsub_rn(oy, qy), d2 = __dsub_rn(oz, qz);
    return __dadd_rn(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1)), __dmul_rn(d2, d2));
}

// Gaspari-Cohn taper with support at x = 1 (utils.c:1425-1443): the same
// polynomial pieces, evaluated in the same order.
__device__ __forceinline__ double taper_gc(double x)
{
    if (x >= 1.0) return 0.0;
    x = __dmul_rn(x, 2.0);
    double x2 = __dmul_rn(x, x);
    double x3 = __dmul_rn(x2, x);
    double f;
    // x/4 and x/2 are exact scalings: multiplying by 0.25 and 0.5 gives the
    // same double as the division, without the division's instruction sequence
    if (x < 1.0) {
        double a = __dadd_rn(__dmul_rn(-x3, 0.25), __dmul_rn(x2, 0.5));
        f = __dadd_rn(1.0, __dmul_rn(x2, a));
        f = __dadd_rn(f, __dmul_rn(x3, 5.0 / 8.0));
        f = __dsub_rn(f, __dmul_rn(x2, 5.0 / 3.0));
    } else {
        double a = __dsub_rn(__ddiv_rn(x3, 12.0), __dmul_rn(x2, 0.5));
        f = __dmul_rn(x2, a);
        f = __dadd_rn(f, __dmul_rn(x3, 5.0 / 8.0));
        f = __dadd_rn(f, __dmul_rn(x2, 5.0 / 3.0));
        f = __dsub_rn(f, __dmul_rn(x, 5.0));
        f = __dadd_rn(f, 4.0);
        f = __dsub_rn(f, __ddiv_rn(2.0 / 3.0, x));
    }
    return (f >= 0.0) ? f : 0.0;
}

// multi-radius taper coefficient (obstypes.c:800-809)
__device__ __forceinline__ double calclcoeff(int nlocrad, const double* locrad, const double* locweight, double dist)
{
    double sum = 0.0;
    for (int i = 0; i < nlocrad; ++i)
        if (dist <= locrad[i]) sum = __dadd_rn(sum, __dmul_rn(locweight[i], taper_gc(__ddiv_rn(dist, locrad[i]))));
    return sum;
}

// FP32 taper for the mixed-precision path (about 1e-7 relative everywhere);
// the membership test stays exact in FP64.  With z = 2 d / r, the outer piece
// of the Gaspari-Cohn function, multiplied by 12 z, is the polynomial
// z^6 - 6 z^5 + 7.5 z^4 + 20 z^3 - 60 z^2 + 48 z - 8 = (z - 2)^4 (z^2 + 2 z - 0.5),
// so for 1 <= z < 2
//     f = (2 - z)^4 (z^2 + 2 z - 0.5) / (12 z) = (4/3) u^4 (z^2 + 2 z - 0.5) / z,
// u = 1 - d / r.  Taking u = (r^2 - d^2) / (r (r + d)) with r^2 - d^2 formed in
// FP64 avoids the cancellation the expanded form suffers in FP32 near the
// edge of the support.
__device__ __forceinline__ float taper_gc_f(float u, float z)
{
    if (u <= 0.0f) return 0.0f;
    float f;
    if (z < 1.0f) {
        float z2 = z * z, z3 = z2 * z;
        f = 1.0f + z2 * (-z3 * 0.25f + z2 * 0.5f) + z3 * 0.625f - z2 * (5.0f / 3.0f);
    } else {
        float u2 = u * u;
        f = (4.0f / 3.0f) * (u2 * u2) * (z * z + 2.0f * z - 0.5f) / z;
    }
    return f >= 0.0f ? f : 0.0f;
}

__device__ __forceinline__ float calclcoeff_f(int nlocrad, const double* locrad, const double* locweight, double d2)
{
    const float dist = sqrtf((float)d2);
    float sum = 0.0f;
    for (int i = 0; i < nlocrad; ++i) {
        const double r = locrad[i];
        const double e = r * r - d2;
        if (e < 0.0) continue;
        const float rf = (float)r;
        const float u = (float)e / (rf * (rf + dist));
        const float z = 2.0f * (1.0f - u);
        sum += (float)locweight[i] * taper_gc_f(u, z);
    }
    return sum;
}

// Squared distance as a double-float (FP32 instructions only) for the mixed
// path.  ox, oy: observation coordinates (floats, exact); the query is split
// into hi + lo floats.  dx = (ox - qh) - ql is kept as the pair (xh, xl) with
// the exact error of the first difference (TwoSum); the squares use the exact
// FMA residual.  Returns the high part (d2h, also the FP32 squared distance)
// and the low part d2l; together they carry about 2^-44 relative accuracy.
__device__ __forceinline__ void dist2_df(float ox, float oy, float qxh, float qxl, float qyh, float qyl, float& d2h,
                                         float& d2l)
{
    float xh = __fsub_rn(ox, qxh);
    float xe;
    {
        // TwoSum error of xh = ox + (-qxh)
        const float bp = __fsub_rn(xh, ox);
        xe = __fadd_rn(__fsub_rn(ox, __fsub_rn(xh, bp)), __fsub_rn(-qxh, bp));
    }
    const float xl = __fsub_rn(xe, qxl);
    float yh = __fsub_rn(oy, qyh);
    float ye;
    {
        const float bp = __fsub_rn(yh, oy);
        ye = __fadd_rn(__fsub_rn(oy, __fsub_rn(yh, bp)), __fsub_rn(-qyh, bp));
    }
    const float yl = __fsub_rn(ye, qyl);
    const float px = __fmul_rn(xh, xh), pxe = fmaf(xh, xh, -px);
    const float py = __fmul_rn(yh, yh), pye = fmaf(yh, yh, -py);
    const float sh = __fadd_rn(px, py);
    const float bp = __fsub_rn(sh, px);
    const float se = __fadd_rn(__fsub_rn(px, __fsub_rn(sh, bp)), __fsub_rn(py, bp));
    const float low = se + pxe + pye + 2.0f * (xh * xl + yh * yl) + (xl * xl + yl * yl);
    d2h = __fadd_rn(sh, low);
    d2l = __fsub_rn(low, __fsub_rn(d2h, sh));
}

// Taper coefficient from the double-float squared distance (mixed path):
// e = r^2 - d^2 formed from double-float parts (no cancellation near the
// edge), then the factorised outer piece as in calclcoeff_f.
__device__ __forceinline__ float calclcoeff_df(const TypeIndex& t, float d2h, float d2l)
{
    const float dist = sqrtf(d2h);
    float sum = 0.0f;
    for (int i = 0; i < t.nlocrad; ++i) {
        const float e = __fsub_rn(t.r2_f[i], d2h) + __fsub_rn(t.r2_fl[i], d2l);
        if (e < 0.0f) continue;
        const float rf = t.locrad_f[i];
        const float u = e / (rf * (rf + dist));
        const float z = 2.0f * (1.0f - u);
        sum += t.locweight_f[i] * taper_gc_f(u, z);
    }
    return sum;
}

}  // namespace exact
