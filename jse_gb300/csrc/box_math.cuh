// FP64 box arithmetic with explicit round-to-nearest operations (no contraction, so
// every rounding matches the reference's Java doubles) and float-float helpers on the
// FP32 pipe.  Shared by the neighbour kernels of the one-shot and resident paths.
#pragma once

#include "common.cuh"

namespace nnapgb {

// ----------------------------------------------------------------- exact FP64 box math
__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dd(double a, double b) { return __ddiv_rn(a, b); }

__device__ __forceinline__ double snap_int(double v) {
    double r = rint(v);
    return fabs(ds(v, r)) < 1.0e-10 ? r : v;
}

__device__ inline void to_direct(const StructDev& S, double p[3]) {
    const double x = p[0], y = p[1], z = p[2];
    if (S.kind == 0) {
        p[0] = dd(x, S.a[0]); p[1] = dd(y, S.b[1]); p[2] = dd(z, S.c[2]);
    } else if (S.kind == 1) {
        const double X = S.a[0], Y = S.b[1], Z = S.c[2], XY = S.b[0], XZ = S.c[0], YZ = S.c[1];
        // x/X - XY*y/(X*Y) + (XY*YZ - XZ*Y)*z/(X*Y*Z)
        p[0] = da(ds(dd(x, X), dd(dm(XY, y), dm(X, Y))), dd(dm(ds(dm(XY, YZ), dm(XZ, Y)), z), dm(dm(X, Y), Z)));
        p[1] = ds(dd(y, Y), dd(dm(YZ, z), dm(Y, Z)));
        p[2] = dd(z, Z);
    } else {
        p[0] = dd(da(da(dm(S.bc[0], x), dm(S.bc[1], y)), dm(S.bc[2], z)), S.vol);
        p[1] = dd(da(da(dm(S.ca[0], x), dm(S.ca[1], y)), dm(S.ca[2], z)), S.vol);
        p[2] = dd(da(da(dm(S.ab[0], x), dm(S.ab[1], y)), dm(S.ab[2], z)), S.vol);
    }
    p[0] = snap_int(p[0]); p[1] = snap_int(p[1]); p[2] = snap_int(p[2]);
}

__device__ inline void to_cartesian(const StructDev& S, double s[3]) {
    const double u = s[0], v = s[1], w = s[2];
    if (S.kind == 0) {
        s[0] = dm(u, S.a[0]); s[1] = dm(v, S.b[1]); s[2] = dm(w, S.c[2]);
    } else if (S.kind == 1) {
        s[0] = da(da(dm(S.a[0], u), dm(S.b[0], v)), dm(S.c[0], w));
        s[1] = da(dm(S.b[1], v), dm(S.c[1], w));
        s[2] = dm(S.c[2], w);
    } else {
        s[0] = da(da(dm(S.a[0], u), dm(S.b[0], v)), dm(S.c[0], w));
        s[1] = da(da(dm(S.a[1], u), dm(S.b[1], v)), dm(S.c[1], w));
        s[2] = da(da(dm(S.a[2], u), dm(S.b[2], v)), dm(S.c[2], w));
    }
}

// shift = (na*a + nb*b) + nc*c, component-wise, in this order.
__device__ __forceinline__ void image_shift(const StructDev& S, int na, int nb, int nc, double sh[3]) {
#pragma unroll
    for (int d = 0; d < 3; ++d) sh[d] = da(da(dm((double)na, S.a[d]), dm((double)nb, S.b[d])), dm((double)nc, S.c[d]));
}

// ----------------------------------------------------------------- float-float helpers
// Error-free transformations on the FP32 pipe (the FP64 pipe of this GPU is narrow).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}
// The image shift (na*a + nb*b) + nc*c as a float-float pair hi + lo, from the box rows
// in float-float form (a = fa + la to about 48 bits): exact products of the float parts
// (FMA residuals), their sum by two-sums, and the low parts added in FP32.  hi + lo is
// within about 2^-45 of the shift's magnitude, on the FP32 pipe; zero for the zero image.
__device__ __forceinline__ void image_shift_ff(const StructDev& S, int na, int nb, int nc, float hi[3], float lo[3]) {
    const float xa = (float)na, xb = (float)nb, xc = (float)nc;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const float p1 = xa * S.fa[d], e1 = fmaf(xa, S.fa[d], -p1);
        const float p2 = xb * S.fb[d], e2 = fmaf(xb, S.fb[d], -p2);
        const float p3 = xc * S.fc[d], e3 = fmaf(xc, S.fc[d], -p3);
        float s1, t1, s2, t2;
        two_sum(p1, p2, s1, t1);
        two_sum(s1, p3, s2, t2);
        const float l = ((t1 + t2) + ((e1 + e2) + e3)) + ((xa * S.la[d] + xb * S.lb[d]) + xc * S.lc[d]);
        two_sum(s2, l, hi[d], lo[d]);
    }
}

// hi + lo += v
__device__ __forceinline__ void ff_acc(float& hi, float& lo, float v) {
    float s, e;
    two_sum(hi, v, s, e);
    hi = s;
    lo += e;
}
// hi + lo += x * y (exact product)
__device__ __forceinline__ void ff_acc_prod(float& hi, float& lo, float x, float y) {
    const float p = x * y;
    const float pe = fmaf(x, y, -p);
    ff_acc(hi, lo, p);
    lo += pe;
}

}  // namespace nnapgb
