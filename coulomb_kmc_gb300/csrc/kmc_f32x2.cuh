// Packed FP32 pairs: two FP32 lanes in one 64-bit register, operated on by the
// sm_100-family packed instructions add/sub/mul/fma .rn.f32x2 (PTX ISA 8.6+).
// One packed instruction does the work of two FP32 instructions in one issue
// slot; each lane is rounded exactly as the scalar instruction would round it,
// so the error-free transformations of kmc_df32.cuh (two_sum, two_prod with
// FMA) stay exact lane by lane.  Used where a warp is limited by instruction
// issue rather than by the FP32 pipe.
#pragma once

typedef unsigned long long f2x;  // lane 0 in the low word, lane 1 in the high word

__device__ __forceinline__ f2x f2_pack(const float a, const float b)
{
    f2x r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}

__device__ __forceinline__ void f2_unpack(const f2x v, float &a, float &b)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}

__device__ __forceinline__ f2x f2_splat(const float a) { return f2_pack(a, a); }

__device__ __forceinline__ f2x f2_add(const f2x a, const f2x b)
{
    f2x d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

__device__ __forceinline__ f2x f2_sub(const f2x a, const f2x b)
{
    f2x d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

__device__ __forceinline__ f2x f2_mul(const f2x a, const f2x b)
{
    f2x d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

// a * b + c, one rounding per lane
__device__ __forceinline__ f2x f2_fma(const f2x a, const f2x b, const f2x c)
{
    f2x d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

// lane-wise rsqrtf (the special-function unit has no packed form)
__device__ __forceinline__ f2x f2_rsqrt(const f2x v)
{
    float a, b;
    f2_unpack(v, a, b);
    return f2_pack(rsqrtf(a), rsqrtf(b));
}

// lane-wise select: keep lane i of v unless z_i, then 0
__device__ __forceinline__ f2x f2_zero_lanes(const f2x v, const bool z0, const bool z1)
{
    float a, b;
    f2_unpack(v, a, b);
    return f2_pack(z0 ? 0.0f : a, z1 ? 0.0f : b);
}

// both lanes negated: a flip of their sign bits (exact; integer pipe)
__device__ __forceinline__ f2x f2_neg(const f2x v) { return v ^ 0x8000000080000000ull; }

// acc(hi, lo) += t(hi) + pl(lo), lane-wise, in the accumulator form of df_acc:
// two_sum on the high words, the rest gathered in the low word
__device__ __forceinline__ void f2_acc(f2x &ah, f2x &al, const f2x th, const f2x pl)
{
    const f2x s = f2_add(ah, th);
    const f2x bb = f2_sub(s, ah);
    const f2x e = f2_add(f2_sub(ah, f2_sub(s, bb)), f2_sub(th, bb));
    ah = s;
    al = f2_add(al, f2_add(e, pl));
}
