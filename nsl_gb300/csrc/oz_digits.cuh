// Balanced split-BF16 digits of FP64 rows (the operand format of the split-BF16 tensor-core operator,
// fm_apply_oz.cu), shared by the operator's digit pre-pass and the CG kernel that writes the next search direction's
// digits itself (cg.cu). A row v is scaled by 2^e (|v| < 2^e), rounded to a 53-bit integer N and written as S = 6
// balanced base-512 digits, N = sum_k a_k 2^{9(S-1-k)}, each an integer of magnitude <= 256 (exact in BF16).
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace nslg {

constexpr int OZ_W = 9;      // bits per balanced digit: |digit| <= 2^(W-1) = 256, exact in BF16
constexpr int OZ_S = 6;      // digits per operand (9 S - 1 = 53 bits)
constexpr int OZ_CACHE = 12;  // operand values a lane keeps in registers (rows of <= 384 sites)

// round(v 2^{9S-1-e}) as a signed integer from the FP64 bit pattern (|v| < 2^e, so |result| <= 2^53).
__device__ __forceinline__ long long scaled_int(unsigned long long bits, int e) {
    const int ex = (int)((bits >> 52) & 0x7FF);
    if (ex == 0) return 0ll;  // zero (subnormals are far below every row scale)
    const unsigned long long mant = (bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int sh = 1075 + e - ex - (OZ_W * OZ_S - 1);  // |v| = mant 2^{ex - 1075}; sh >= 0 as |v| < 2^e
    unsigned long long u;
    if (sh >= 64) u = 0ull;
    else if (sh == 0) u = mant;
    else u = (mant + (1ull << (sh - 1))) >> sh;  // round half up (|result| stays <= 2^53)
    return (bits >> 63) ? -(long long)u : (long long)u;
}

// Balanced base-2^W digits of N (|N| <= 2^{WS-1}): N = sum_k a_k 2^{W(S-1-k)}, a_k in [-2^{W-1}, 2^{W-1}) for k > 0
// and |a_0| <= 2^{W-1}; every digit is exact in BF16. In 32-bit integer arithmetic: N = hi 2^27 + lo with
// 0 <= lo < 2^27 gives the three low digits and a carry into hi, which gives the rest.
__device__ __forceinline__ void balanced_digits(long long N, float (&a)[OZ_S]) {
    static_assert(OZ_W == 9 && OZ_S == 6, "three digits per 27-bit half");
    constexpr int HALF = 1 << (OZ_W - 1), MASK = (1 << OZ_W) - 1;
    int lo = (int)(N & ((1ll << 27) - 1));
    int hi = (int)(N >> 27);  // |hi| <= 2^26
#pragma unroll
    for (int k = OZ_S - 1; k >= 3; --k) {
        const int d = ((lo + HALF) & MASK) - HALF;
        a[k] = (float)d;
        lo = (lo - d) >> OZ_W;  // exact: lo - d is a multiple of 2^W; ends as the carry 0 or 1
    }
    hi += lo;
#pragma unroll
    for (int k = 2; k > 0; --k) {
        const int d = ((hi + HALF) & MASK) - HALF;
        a[k] = (float)d;
        hi = (hi - d) >> OZ_W;
    }
    a[0] = (float)hi;
}

// |v| as an ordered integer: the FP64 bit pattern without the sign.
__device__ __forceinline__ unsigned long long abs_bits(double v) {
    return (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;
}

// frexp exponent of the largest |v| from its bit pattern: |v| < 2^e (0 for an all-zero row).
__device__ __forceinline__ int scale_exponent(unsigned long long maxbits) {
    return maxbits == 0 ? 0 : (int)(maxbits >> 52) - 1022;
}

// Digits of the complex operand values at sites y, y + 1 (y even) given by their FP64 bit patterns (integer work
// only: scale, round, digits), written as BF16 pairs.
__device__ __forceinline__ void write_digits2(__nv_bfloat16 *__restrict__ planes, int64_t mreal, int64_t grow,
                                              int ld, int y, const unsigned long long (&b)[4], int er, int ei) {
    float a0[OZ_S], a1[OZ_S], i0[OZ_S], i1[OZ_S];
    balanced_digits(scaled_int(b[0], er), a0);
    balanced_digits(scaled_int(b[1], ei), i0);
    balanced_digits(scaled_int(b[2], er), a1);
    balanced_digits(scaled_int(b[3], ei), i1);
#pragma unroll
    for (int l = 0; l < OZ_S; ++l) {
        *reinterpret_cast<__nv_bfloat162 *>(planes + ((int64_t)l * mreal + 2 * grow) * ld + y) =
            __floats2bfloat162_rn(a0[l], a1[l]);
        *reinterpret_cast<__nv_bfloat162 *>(planes + ((int64_t)l * mreal + 2 * grow + 1) * ld + y) =
            __floats2bfloat162_rn(i0[l], i1[l]);
    }
}

}  // namespace nslg
