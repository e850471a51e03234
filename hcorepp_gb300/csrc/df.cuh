// Float-float ("double-float") arithmetic: a value is the unevaluated sum h + l of two floats
// (|l| <= ulp(h) / 2), 48 significant bits, computed on the FP32 pipe (about 70x the FP64 rate of
// this GPU).  Error-free transformations (Knuth two-sum, FMA two-product; Dekker's double-length
// arithmetic) with explicitly rounded intrinsics so that nothing is contracted or reassociated.
// Used by the mixed form of the recompression (core pivoted QR and Jacobi, Householder panels).
#pragma once

#include <cuda_runtime.h>

namespace hcgb {

struct df {
    float h, l;
    __device__ __forceinline__ df() {}
    __device__ __forceinline__ df(double v) {
        h = __double2float_rn(v);
        l = __double2float_rn(v - (double) h);
    }
    __device__ __forceinline__ explicit operator double() const { return (double) h + (double) l; }
};
__device__ __forceinline__ df operator-(df a) {
    df r;
    r.h = -a.h;
    r.l = -a.l;
    return r;
}
// c + a * b
__device__ __forceinline__ df df_fma(df a, df b, df c) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    const float s = __fadd_rn(c.h, p);
    const float bb = __fsub_rn(s, c.h);
    float err = __fadd_rn(__fsub_rn(c.h, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    err = __fadd_rn(err, __fadd_rn(c.l, e));
    df r;
    r.h = __fadd_rn(s, err);
    r.l = __fsub_rn(err, __fsub_rn(r.h, s));
    return r;
}
__device__ __forceinline__ df df_add(df a, df b) {
    const float s = __fadd_rn(a.h, b.h);
    const float bb = __fsub_rn(s, a.h);
    float err = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(b.h, bb));
    err = __fadd_rn(err, __fadd_rn(a.l, b.l));
    df r;
    r.h = __fadd_rn(s, err);
    r.l = __fsub_rn(err, __fsub_rn(r.h, s));
    return r;
}
__device__ __forceinline__ df df_mul(df a, df b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    df r;
    r.h = __fadd_rn(p, e);
    r.l = __fsub_rn(e, __fsub_rn(r.h, p));
    return r;
}
__device__ __forceinline__ df df_f(float v) {
    df r;
    r.h = v;
    r.l = 0.f;
    return r;
}
// 1 / sqrt(q) for q >= 1 to float-float accuracy: two Newton steps r <- r + r (1 - q r^2) / 2 from
// the float reciprocal square root (about 22 -> 44 -> 48 correct bits).
__device__ __forceinline__ df df_rsqrt(df q) {
    df r = df_f(rsqrtf(q.h));
#pragma unroll
    for (int it = 0; it < 2; it++) {
        const df res = df_add(df_f(1.f), -df_mul(q, df_mul(r, r)));  // 1 - q r^2, small
        r = df_add(r, df_mul(df_mul(r, res), df_f(0.5f)));
    }
    return r;
}

// Float-float reciprocal and square root (one correction step each from the float result).
__device__ __forceinline__ df df_div(df a, df b) {
    const float q0 = __fdiv_rn(a.h, b.h);
    const df r = df_add(a, -df_mul(df_f(q0), b));  // a - q0 b
    const float q1 = __fdiv_rn(r.h, b.h);
    df q;
    q.h = __fadd_rn(q0, q1);
    q.l = __fsub_rn(q1, __fsub_rn(q.h, q0));
    return q;
}
__device__ __forceinline__ df df_sqrt(df v) {
    if (v.h <= 0.f) return df_f(0.f);
    const float s0 = sqrtf(v.h);
    const df r = df_add(v, -df_mul(df_f(s0), df_f(s0)));  // v - s0^2
    const float s1 = __fdiv_rn(r.h, 2.f * s0);
    df q;
    q.h = __fadd_rn(s0, s1);
    q.l = __fsub_rn(s1, __fsub_rn(q.h, s0));
    return q;
}

// Compensated accumulator for sums of float-float products (Ogita, Rump and Oishi's Dot2, "Accurate
// sum and dot product", SIAM J. Sci. Comput. 26 (2005), extended to float-float operands): s holds
// the running float sum, e the float sum of every rounding error (the exact error of a.h * b.h,
// the cross terms a.h * b.l + a.l * b.h, and the exact error of each addition into s).  The
// result is as accurate as float-float accumulation (a.l * b.l, below 2^-48 relative, is dropped
// by both) but renormalises once at the end: 12 FP32 instructions per term instead of 15.
struct df_acc {
    float s, e;
};
__device__ __forceinline__ df_acc df_acc_init(df c) { return df_acc{c.h, c.l}; }
__device__ __forceinline__ void df_acc_fma(df_acc &acc, df a, df b) {
    const float p = __fmul_rn(a.h, b.h);
    float ep = __fmaf_rn(a.h, b.h, -p);
    ep = __fmaf_rn(a.h, b.l, ep);
    ep = __fmaf_rn(a.l, b.h, ep);
    const float t = __fadd_rn(acc.s, p);
    const float z = __fsub_rn(t, acc.s);
    const float es = __fadd_rn(__fsub_rn(acc.s, __fsub_rn(t, z)), __fsub_rn(p, z));
    acc.s = t;
    acc.e = __fadd_rn(acc.e, __fadd_rn(ep, es));
}
__device__ __forceinline__ df df_acc_value(df_acc acc) {  // two-sum: |e| may exceed |s| after cancellation
    df r;
    r.h = __fadd_rn(acc.s, acc.e);
    const float z = __fsub_rn(r.h, acc.s);
    r.l = __fadd_rn(__fsub_rn(acc.s, __fsub_rn(r.h, z)), __fsub_rn(acc.e, z));
    return r;
}

// Sum over groups of G consecutive lanes (G a power of two <= 32), every lane gets its group's sum.
__device__ __forceinline__ df df_group_sum(df v, int G) {
    for (int o = G >> 1; o > 0; o >>= 1) {
        df w;
        w.h = __shfl_xor_sync(0xffffffffu, v.h, o);
        w.l = __shfl_xor_sync(0xffffffffu, v.l, o);
        v = df_add(v, w);
    }
    return v;
}

}  // namespace hcgb
