// FP32-pair ("double-single") arithmetic shared by the FP64 advection
// kernels that keep FP64 in HBM (adv_ds.cu: staged column pairs and
// contiguous lines; adv_stream_ds.cu: streamed column pairs): the split of a
// double into two FP32 parts, the stencil sum of a column pair from exact
// products and a TwoSum tree, and the widening back to FP64. Every kernel
// that uses them computes a cell with the same operations, so they give the
// same bits.
#pragma once
#include <cstdint>

namespace bkma {

// |x| in [2^-74, 2^126), or +-0: the split below is exact to 2^-48 |x| and
// every intermediate FP32 value stays normal and finite.
__device__ __forceinline__ bool ds_splittable(double x) {
    const uint32_t xh = (uint32_t)__double2hiint(x), xl = (uint32_t)__double2loint(x);
    const uint32_t e = (xh >> 20) & 0x7FFu;
    return (e - 949u < 200u) || ((xh << 1) | xl) == 0u;  // in range, or +-0
}

// x = h + l + r, |r| <= 2^-48 |x| (x splittable). h keeps x's sign, exponent
// and leading 23 stored mantissa bits; l is the rest, the low 29 bits times
// 2^(E-52), rounded to 24 bits.
__device__ __forceinline__ void ds_split(double x, float &h, float &l) {
    const uint32_t xh = (uint32_t)__double2hiint(x), xl = (uint32_t)__double2loint(x);
    const uint32_t sign = xh & 0x80000000u;
    const uint32_t e = (xh >> 20) & 0x7FFu;
    // exponent rebased from 1023 to 127 in place, then the 8-bit exponent and
    // 23 mantissa bits moved up by 3 (the sign bit is restored after)
    const uint32_t hb = __funnelshift_l(xl, xh - (896u << 20), 3) | sign;
    const float lo = __uint2float_rn(xl & 0x1FFFFFFFu) * __uint_as_float(((e - 948u) << 23) | sign);
    // +-0 gives l = +-0 with no select (a zero mantissa times a finite scale);
    // a subnormal x is not splittable and its pairs are redone in FP64
    h = e ? __uint_as_float(hb) : __uint_as_float(sign);
    l = lo;
}

// FP32 -> FP64 by moving the bits, with no FP64-pipe conversion. A subnormal
// (below 2^-126, which only a pair part of an output far smaller than the
// tile's values can be: every input is >= 2^-74 or zero) becomes a double
// below 2^-1022 (its high word zeroed), an error below 2^-52 of the smallest
// nonzero input; zero stays zero.
__device__ __forceinline__ double ds_widen(float f) {
    const uint32_t u = __float_as_uint(f);
    const uint32_t mag = u & 0x7FFFFFFFu;
    const bool normal = mag >= 0x00800000u;
    const uint32_t hi = (normal ? (mag >> 3) + (896u << 20) : 0u) | (u & 0x80000000u);
    return __hiloint2double((int)hi, (int)(mag << 29));
}

__device__ __forceinline__ float2 neg2(float2 v) { return make_float2(-v.x, -v.y); }

// Split both doubles of a column pair into v = (h0, h1, l0, l1); false when
// either value is outside the split's range.
__device__ __forceinline__ bool ds_split2(double2 x, float4 &v) {
    ds_split(x.x, v.x, v.z);
    ds_split(x.y, v.y, v.w);
    return ds_splittable(x.x) && ds_splittable(x.y);
}

// TwoSum (Knuth) on both lanes of a pair: t = fl(a + b) and t + (ea + eb) =
// a + b exactly; err = fl(ea + eb).
__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2 &t, float2 &err) {
    const float2 m1 = make_float2(-1.0f, -1.0f);
    t = __fadd2_rn(a, b);
    const float2 bv = __ffma2_rn(a, m1, t);   // t - a
    const float2 av = __ffma2_rn(bv, m1, t);  // t - bv
    const float2 eb = __ffma2_rn(bv, m1, b);  // b - bv
    const float2 ea = __ffma2_rn(av, m1, a);  // a - av
    err = __fadd2_rn(ea, eb);
}

// sum_k w_k x_k of a column pair from its NT split taps T[(u + k) % NS]
// (u: ring position of tap 0, NS >= NT ring slots), or T[(u + NT - 1 - k) %
// NS] when REV (a ring filled from the last tap down); two FP64 results. The
// high products a h are
// summed exactly by a pairwise TwoSum tree (taps (0,1), (2,3), (4,5), then
// the partial sums); the low-order terms (a l, b h, the product errors and
// the tree's errors) are added in FP32 in short independent chains.
template <int NT, bool REV = false, int NS>
__device__ __forceinline__ double2 ds_stencil(const float4 (&T)[NS], int u, const float2 (&A)[NT],
                                              const float2 (&B)[NT]) {
    static_assert(NT == 4 || NT == 6, "4 or 6 taps");
    static_assert(NS >= NT, "a ring of at least NT taps");
    float2 p[NT], e[NT], La, Lb;
#pragma unroll
    for (int k = 0; k < NT; ++k) {
        const float4 v = T[(u + (REV ? NT - 1 - k : k)) % NS];
        const float2 h = make_float2(v.x, v.y), l = make_float2(v.z, v.w);
        p[k] = __fmul2_rn(h, A[k]);
        e[k] = __ffma2_rn(h, A[k], neg2(p[k]));  // exact error of the product
        La = k ? __ffma2_rn(l, A[k], La) : __fmul2_rn(l, A[0]);
        Lb = k ? __ffma2_rn(h, B[k], Lb) : __fmul2_rn(h, B[0]);
    }
    float2 s01, r01, s23, r23, S, rS, E, R;
    two_sum2(p[0], p[1], s01, r01);
    two_sum2(p[2], p[3], s23, r23);
    if constexpr (NT == 6) {
        float2 s45, r45, s03, r03;
        two_sum2(p[4], p[5], s45, r45);
        two_sum2(s01, s23, s03, r03);
        two_sum2(s03, s45, S, rS);
        E = __fadd2_rn(__fadd2_rn(__fadd2_rn(e[0], e[1]), __fadd2_rn(e[2], e[3])),
                       __fadd2_rn(__fadd2_rn(e[4], e[5]), __fadd2_rn(r01, r23)));
        R = __fadd2_rn(__fadd2_rn(r45, r03), rS);
    } else {
        two_sum2(s01, s23, S, rS);
        E = __fadd2_rn(__fadd2_rn(e[0], e[1]), __fadd2_rn(e[2], e[3]));
        R = __fadd2_rn(__fadd2_rn(r01, r23), rS);
    }
    const float2 L = __fadd2_rn(__fadd2_rn(La, Lb), __fadd2_rn(E, R));
    // S + L rounded once to FP64: both parts are exact in FP64, so one DADD
    // of the widened parts is the correctly rounded pair sum
    return make_double2(__dadd_rn(ds_widen(S.x), ds_widen(L.x)),
                        __dadd_rn(ds_widen(S.y), ds_widen(L.y)));
}

}  // namespace bkma
