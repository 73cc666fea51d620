// Double-FP32 ("df32") arithmetic: a value is hi + lo with |lo| <= ulp(hi)/2
// (after normalisation), built from error-free transformations on the FP32 pipe:
//   two_sum  (Knuth):             a + b = s + e exactly
//   two_prod (fused multiply-add): a * b = p + e exactly
// On GB300 the FP32 pipe issues 64x more instructions per clock than the FP64
// pipe, so a df32 operation (4-20 FP32 instructions, ~48-bit significand) is
// several times cheaper than one FP64 operation while being far more accurate
// than FP32.
#pragma once

struct df32 {
    float hi, lo;
};

__device__ __forceinline__ df32 df_make(const float hi, const float lo) { return df32{hi, lo}; }

__device__ __forceinline__ df32 df_from_double(const double d)
{
    const float hi = (float)d;
    return df32{hi, (float)(d - (double)hi)};
}

__device__ __forceinline__ double df_to_double(const df32 a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ void two_sum(const float a, const float b, float &s, float &e)
{
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ void two_prod(const float a, const float b, float &p, float &e)
{
    p = a * b;
    e = fmaf(a, b, -p);
}

__device__ __forceinline__ df32 df_add(const df32 a, const df32 b)
{
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    e += a.lo + b.lo;
    float h, l;
    two_sum(s, e, h, l);  // renormalise
    return df32{h, l};
}

__device__ __forceinline__ df32 df_sub(const df32 a, const df32 b) { return df_add(a, df32{-b.hi, -b.lo}); }

__device__ __forceinline__ df32 df_mul(const df32 a, const df32 b)
{
    float p, e;
    two_prod(a.hi, b.hi, p, e);
    e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
    float h, l;
    two_sum(p, e, h, l);
    return df32{h, l};
}

__device__ __forceinline__ df32 df_mul_f(const df32 a, const float b)
{
    float p, e;
    two_prod(a.hi, b, p, e);
    e = fmaf(a.lo, b, e);
    float h, l;
    two_sum(p, e, h, l);
    return df32{h, l};
}

// a*b - c*d with one renormalisation (both products error-free)
__device__ __forceinline__ df32 df_fms(const df32 a, const df32 b, const df32 c, const df32 d)
{
    float p1, e1, p2, e2;
    two_prod(a.hi, b.hi, p1, e1);
    two_prod(c.hi, d.hi, p2, e2);
    float s, e;
    two_sum(p1, -p2, s, e);
    e += e1 - e2;
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    e = fmaf(-c.hi, d.lo, e);
    e = fmaf(-c.lo, d.hi, e);
    float h, l;
    two_sum(s, e, h, l);
    return df32{h, l};
}

// a*b + c*d
__device__ __forceinline__ df32 df_fma2(const df32 a, const df32 b, const df32 c, const df32 d)
{
    return df_fms(a, b, df32{-c.hi, -c.lo}, d);
}

// acc += x without renormalising lo every step (accumulator form)
__device__ __forceinline__ void df_acc(df32 &acc, const df32 x)
{
    float s, e;
    two_sum(acc.hi, x.hi, s, e);
    acc.hi = s;
    acc.lo += e + x.lo;
}

__device__ __forceinline__ void df_acc_f(df32 &acc, const float x)
{
    float s, e;
    two_sum(acc.hi, x, s, e);
    acc.hi = s;
    acc.lo += e;
}

// 1/sqrt(r2) for r2 = hi + lo, as df32: FP32 reciprocal square root plus one
// Newton correction whose residual 1 - r2 y^2 is formed exactly with FMA.
__device__ __forceinline__ df32 df_rsqrt(const df32 r2)
{
    const float y = rsqrtf(r2.hi);
    float yy, yye;
    two_prod(y, y, yy, yye);
    const float rho = fmaf(-r2.hi, yy, 1.0f) - fmaf(r2.hi, yye, r2.lo * yy);
    return df32{y, 0.5f * y * rho};
}
