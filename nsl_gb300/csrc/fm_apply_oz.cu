// FP64-class fermion-matrix applications on the tensor cores: split BF16 digits with exact FP32 accumulation.
//
// The CG on MM^dagger at low temperature is so ill-conditioned (|A| |x| / |b| ~ 1e7 at beta = 8) that an FP32-class
// operator stops reducing the true residual near 1e-6; the last decades need an FP64-class operator. GB300 executes
// FP64 at ~1.2 TFLOP/s (about 2 FP64 operations per clock per SM), so this kernel builds one from BF16 tensor-core
// products whose sums are exact integers:
//
//   every operand row is scaled by a power of two 2^e (|v| 2^-e < 1) and cut into S signed 7-bit digits
//     v = 2^e sum_{k<S} a_k 2^{-7(k+1)},   a_k integer in [-127, 127]  (exactly representable in BF16),
//   a product of two digit matrices over K sites is an integer matrix with entries below K 127^2; grouping the digit
//   products by d = k + l (the same power of two) into TMEM accumulators G_d and keeping d < S gives
//     Y E^T = 2^{e_row + e_x - 14} sum_{d<S} 2^{-7d} G_d  (+ the dropped orders d >= S, below S K 127^2 2^{-7S}).
//   An accumulator that sums p digit products stays exact in FP32 while p K 127^2 < 2^24. G_3 is split over two
//   accumulators (2 + 2 products), so for K <= 346 (up to ~115 honeycomb unit cells) every order d <= 3 is exact;
//   the orders d >= 4 may round, with weight 2^{-28} or less. S = 7 (28 BF16 MMAs per 16-site step) leaves a relative
//   error near 1e-13 of the row and column maxima.
//
// For K > 1024 the G_0 and G_1 sums are split over two halves of K into separate accumulators.
//
// GB300's FP64 pipe, not HBM, bounds the element-wise work around the MMAs, so both kernels keep FP64 arithmetic to
// what the result needs:
//  * k_oz_digits: one warp per (r, t) row computes Y = phase o psi (M) or psi (M^dagger) once (kept in registers
//    for rows of up to 32 * OZ_CACHE sites), the row's power-of-two scales (real and imaginary rows separately) from
//    integer maxima of the FP64 bit patterns, and writes the S digit planes of the operand (BF16, rows padded to a
//    multiple of 32 sites) with integer shifts. FP64 work: the phase product only.
//  * k_fm_apply_oz: a TMA -> tcgen05 pipeline: warp 0 streams the operand and exp(delta K) digit tiles (16-site
//    k-blocks, 32-byte swizzle, 3 stages), one thread of warp 1 issues the S(S+1)/2 digit MMAs per k-block into the
//    TMEM accumulators, all 4 warps run the epilogue: the integer-valued G_d are recombined in 64-bit integers (two
//    partial sums, exact), converted to FP64 once, scaled by a power of two built from the exponent bits, then the
//    time shift, boundary sign, conj(phase) (M^dagger) and psi - are applied; the psi operand of the epilogue is
//    loaded into registers while the MMAs run. Tile: 128 real GEMM rows (64 complex rows) x 32 output sites with
//    256 TMEM columns, so two CTAs share an SM and one CTA's epilogue overlaps the other's main loop.
//
// The same pipeline serves (oz_gemm, MODE_OZ_GEMM) the matrix chains of the log-det gradient: a plain product
// out = (Y o pro) E^T (o epi) of a complex matrix Y with a real matrix E, optionally column-scaled before (in the
// digit pre-pass) or after (in the epilogue).

#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include "fm_internal.cuh"
#include "tc_common.cuh"

namespace nslg {

namespace {

constexpr int OZ_THREADS = 128;  // 4 warps: TMA producer (warp 0), MMA issuer (warp 1), all four run the epilogue
constexpr int OZ_BM = 128;       // real GEMM rows per tile (64 complex rows)
constexpr int OZ_BK = 16;        // sites per k-block: 32 bytes of BF16, one MMA K step
constexpr int OZ_STAGES = 3;     // TMA -> MMA pipeline depth
constexpr int OZ_S = 7;          // digits per operand
constexpr int OZ_ROWB = OZ_BK * 2;           // bytes per smem row
constexpr int OZ_A_SLICE = OZ_BM * OZ_ROWB;  // 4 KB
constexpr int OZ_LD_ALIGN = 32;              // digit-plane rows are padded to a multiple of 32 sites
constexpr int OZ_CACHE = 12;                 // operand values a lane keeps in registers (rows of <= 384 sites)
constexpr int OZ_HI = 4;                     // orders d < OZ_HI recombine into the high 64-bit partial sum
static_assert(OZ_S > OZ_HI && OZ_S <= 8, "the two 64-bit partial sums hold S <= 8 orders exactly");
// One 64-bit integer per output: hi 2^HI_SHIFT + round(lo 2^-LO_SHIFT) (|hi| < 2^48, so it stays below 2^59).
constexpr int OZ_HI_SHIFT = 11;
constexpr int OZ_LO_SHIFT = 7 * (OZ_S - OZ_HI) - OZ_HI_SHIFT;
static_assert(OZ_LO_SHIFT > 0, "lo is rounded into the combined integer");

// Tile configuration. K <= 1024 (KSPLIT 1): 32 output sites, S + 1 accumulators (G_0..G_{S-1} and the second half
// of G_3) = 256 TMEM columns, so two CTAs share an SM and one's epilogue overlaps the other's MMAs. K > 1024
// (KSPLIT 2): also the second K halves of G_0 and G_1 (S + 3 accumulators), 48 sites, 512 columns, one CTA per SM.
template <int KSPLIT> struct OzTile {
    static constexpr int BN = KSPLIT == 2 ? 48 : 32;
    static constexpr int NACC = KSPLIT == 2 ? OZ_S + 3 : OZ_S + 1;
    static constexpr int TMEM_COLS = NACC * BN <= 256 ? 256 : 512;
    static constexpr int CTAS_PER_SM = TMEM_COLS == 256 ? 2 : 1;
    static constexpr int B_SLICE = BN * OZ_ROWB;
    static constexpr int STAGE = OZ_S * (OZ_A_SLICE + B_SLICE);
    static constexpr int SMEM = OZ_STAGES * STAGE + 1024 /*alignment*/ + 1024 /*barriers, row/col exponents*/;
    static_assert(NACC * BN <= TMEM_COLS && TMEM_COLS <= 512, "TMEM columns");
    static_assert(CTAS_PER_SM * SMEM <= 228 * 1024, "shared memory per SM");
    static_assert(BN % 16 == 0 && BN % 8 == 0, "MMA N for M = 128");
};
// accumulator of the digit products (a, 3 - a) with a >= 2
template <int KSPLIT> __host__ __device__ constexpr int oz_acc_g3b() { return KSPLIT == 2 ? OZ_S + 2 : OZ_S; }
// order d that accumulator `acc` belongs to
template <int KSPLIT> __host__ __device__ constexpr int oz_acc_order(int acc) {
    return acc < OZ_S ? acc : (acc == oz_acc_g3b<KSPLIT>() ? 3 : acc - OZ_S);
}

// Shared-memory matrix descriptor: K-major operand rows of 32 B, 32-byte swizzle, 8-row core groups 256 B apart.
__device__ __forceinline__ uint64_t sdesc_kmajor_sw32(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)1 << 16;           // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(256 >> 4) << 32;  // stride byte offset: 8 rows x 32 B
    d |= (uint64_t)1 << 46;           // descriptor version (sm_100)
    d |= (uint64_t)6 << 61;           // layout: SWIZZLE_32B
    return d;
}

__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4)     // D: F32
           | (1u << 7)   // A: BF16
           | (1u << 10)  // B: BF16
           | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// D[tmem] (+)= A[smem] * B[smem]^T, kind::f16 (BF16 operands, FP32 accumulation), issued by one thread.
// COLL selects the A collector buffer: 0 = none, 1 = fill (read A and keep it), 2 = use (A from the buffer),
// 3 = lastuse (A from the buffer, then released). Consecutive MMAs on the same A slice read it from shared memory once.
template <int COLL>
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
#define NSLG_MMA_F16(Q)                                                                         \
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16" Q \
                 " [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),                                   \
                 "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)                           \
                 : "memory")
    if constexpr (COLL == 1) NSLG_MMA_F16(".collector::a::fill");
    else if constexpr (COLL == 2) NSLG_MMA_F16(".collector::a::use");
    else if constexpr (COLL == 3) NSLG_MMA_F16(".collector::a::lastuse");
    else NSLG_MMA_F16("");
#undef NSLG_MMA_F16
}

// floor(|v| 2^{7S - e}) from the FP64 bit pattern (|v| < 2^e, so the result has at most 7S bits).
__device__ __forceinline__ unsigned long long scaled_magnitude(unsigned long long bits, int e) {
    const int ex = (int)((bits >> 52) & 0x7FF);
    if (ex == 0) return 0ull;  // zero (subnormals are far below every row scale)
    const unsigned long long mant = (bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int sh = 1075 + e - ex - 7 * OZ_S;  // |v| = mant 2^{ex - 1075}
    if (sh >= 64) return 0ull;
    return sh >= 0 ? (mant >> sh) : (mant << (-sh));
}
__device__ __forceinline__ unsigned long long scaled_magnitude(double v, int e) {
    return scaled_magnitude((unsigned long long)__double_as_longlong(v), e);
}

__device__ __forceinline__ __nv_bfloat16 digit(unsigned long long U, int k, bool neg) {
    const int dk = (int)((U >> (7 * (OZ_S - 1 - k))) & 127ull);
    return __float2bfloat16_rn((float)(neg ? -dk : dk));
}

// |v| as an ordered integer: the FP64 bit pattern without the sign.
__device__ __forceinline__ unsigned long long abs_bits(double v) {
    return (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;
}

// frexp exponent of the largest |v| from its bit pattern: |v| < 2^e (0 for an all-zero row).
__device__ __forceinline__ int scale_exponent(unsigned long long maxbits) {
    return maxbits == 0 ? 0 : (int)(maxbits >> 52) - 1022;
}

// 2^e as an FP64 value, from the exponent bits in the normal range.
__device__ __forceinline__ double pow2i(int e) {
    return (e >= -1022 && e <= 1023) ? __longlong_as_double((long long)(e + 1023) << 52) : ldexp(1.0, e);
}

// -2^e (negative) or +2^e, from the exponent and sign bits in the normal range.
__device__ __forceinline__ double signed_pow2(int e, bool negative) {
    if (e >= -1022 && e <= 1023)
        return __longlong_as_double(((long long)(e + 1023) << 52) | (negative ? (long long)(1ull << 63) : 0ll));
    return ldexp(negative ? -1.0 : 1.0, e);
}

template <int MODE>
__device__ __forceinline__ double2 oz_operand(const double2 *__restrict__ psi, const double2 *__restrict__ phase,
                                              int64_t grow, int t, int Nx, int y) {
    double2 v = psi[grow * Nx + y];
    if (MODE == MODE_M) v = cmul(phase[(int64_t)t * Nx + y], v);
    return v;
}

// Digits of one complex operand value given by its FP64 bit patterns (integer work only: sign, scale, digits).
__device__ __forceinline__ void write_digits(__nv_bfloat16 *__restrict__ planes, int64_t mreal, int64_t grow, int ld,
                                             int y, unsigned long long bx, unsigned long long by, int er, int ei) {
    const unsigned long long Ur = scaled_magnitude(bx, er), Ui = scaled_magnitude(by, ei);
    const bool nr = (bx >> 63) != 0, ni = (by >> 63) != 0;
#pragma unroll
    for (int l = 0; l < OZ_S; ++l) {
        planes[((int64_t)l * mreal + 2 * grow) * ld + y] = digit(Ur, l, nr);
        planes[((int64_t)l * mreal + 2 * grow + 1) * ld + y] = digit(Ui, l, ni);
    }
}

// One warp per complex row (r, t): scales e (max |Y| < 2^e, real and imaginary GEMM rows separately) and the digit
// planes A[l][2 row + c][y] (ld sites, zero padded).
template <int MODE>
__global__ void __launch_bounds__(256, 2) k_oz_digits(const double2 *__restrict__ psi, const double2 *__restrict__ phase, int Nt, int Nx,
                            int64_t rows, int ld, __nv_bfloat16 *__restrict__ planes, int *__restrict__ ex,
                            const int *__restrict__ go, int64_t sys_rows) {
    const int64_t grow = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x % 32;
    if (grow >= rows) return;
    if (go && !go[grow / sys_rows]) return;  // a finished system's row (one warp per row: the warp leaves whole)
    const int t = (int)(grow % Nt);
    // the row's operand values as FP64 bit patterns; everything after the phase product is integer work
    unsigned long long cx[OZ_CACHE], cy[OZ_CACHE];
    unsigned long long mr = 0, mi = 0;
#pragma unroll
    for (int c = 0; c < OZ_CACHE; ++c) {
        const int y = lane + 32 * c;
        cx[c] = cy[c] = 0ull;
        if (y < Nx) {
            const double2 v = oz_operand<MODE>(psi, phase, grow, t, Nx, y);
            cx[c] = (unsigned long long)__double_as_longlong(v.x);
            cy[c] = (unsigned long long)__double_as_longlong(v.y);
        }
        mr = max(mr, cx[c] & 0x7FFFFFFFFFFFFFFFull);
        mi = max(mi, cy[c] & 0x7FFFFFFFFFFFFFFFull);
    }
    for (int y = lane + 32 * OZ_CACHE; y < Nx; y += 32) {  // rows longer than the register cache
        const double2 v = oz_operand<MODE>(psi, phase, grow, t, Nx, y);
        mr = max(mr, abs_bits(v.x));
        mi = max(mi, abs_bits(v.y));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mr = max(mr, __shfl_xor_sync(0xffffffffu, mr, o));
        mi = max(mi, __shfl_xor_sync(0xffffffffu, mi, o));
    }
    const int er = scale_exponent(mr), ei = scale_exponent(mi);
    if (lane == 0) {
        ex[2 * grow] = er;
        ex[2 * grow + 1] = ei;
    }
    const int64_t mreal = 2 * rows;
#pragma unroll
    for (int c = 0; c < OZ_CACHE; ++c) {
        const int y = lane + 32 * c;
        if (y < ld) write_digits(planes, mreal, grow, ld, y, cx[c], cy[c], er, ei);
    }
    for (int y = lane + 32 * OZ_CACHE; y < ld; y += 32) {
        unsigned long long bx = 0ull, by = 0ull;
        if (y < Nx) {
            const double2 v = oz_operand<MODE>(psi, phase, grow, t, Nx, y);
            bx = (unsigned long long)__double_as_longlong(v.x);
            by = (unsigned long long)__double_as_longlong(v.y);
        }
        write_digits(planes, mreal, grow, ld, y, bx, by, er, ei);
    }
}

template <int MODE, int KSPLIT, int EPI>
__global__ void __launch_bounds__(OZ_THREADS, OzTile<KSPLIT>::CTAS_PER_SM)
    k_fm_apply_oz(const double2 *__restrict__ psi, double2 *__restrict__ out, const double2 *__restrict__ phase,
                  const int *__restrict__ row_exp, const int *__restrict__ col_exp,
                  const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b, int Nt,
                  int Nx, int64_t rows, int nkb, int *err, const OzEpi epi) {
    using TL = OzTile<KSPLIT>;
    constexpr int NACC = TL::NACC, BN = TL::BN, B_SLICE = TL::B_SLICE, STAGE = TL::STAGE;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *bar_full = reinterpret_cast<uint64_t *>(smem + OZ_STAGES * STAGE);
    uint64_t *bar_empty = bar_full + OZ_STAGES;
    uint64_t *bar_done = bar_empty + OZ_STAGES;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bar_done + 1);
    int *abort_flag = reinterpret_cast<int *>(bar_done + 2);
    int *sh_rowexp = reinterpret_cast<int *>(bar_done + 4);  // OZ_BM ints
    int *sh_colexp = sh_rowexp + OZ_BM;                       // BN ints

    const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
    const int64_t grow0 = (int64_t)blockIdx.x * (OZ_BM / 2);
    const int64_t mrow0 = (int64_t)blockIdx.x * OZ_BM;
    const int64_t mreal = 2 * rows;
    const int n0 = blockIdx.y * BN;

    if (epi.go) {  // every row of the tile belongs to a finished system: the whole CTA leaves before any barrier
        const int64_t last = min(rows, grow0 + OZ_BM / 2) - 1;
        bool any = false;
        for (int64_t s = grow0 / epi.sys_rows; s <= last / epi.sys_rows; ++s) any |= epi.go[s] != 0;
        if (!any) return;
    }

    if (tid == 0) {
        for (int i = 0; i < OZ_STAGES; ++i) {
            tc::mbar_init(&bar_full[i], 1);
            tc::mbar_init(&bar_empty[i], 1);
        }
        tc::mbar_init(bar_done, 1);
        *abort_flag = 0;
        tc::fence_mbar_init();
        tc::prefetch_tmap(&map_a);
        tc::prefetch_tmap(&map_b);
    }
    sh_rowexp[tid] = (mrow0 + tid < mreal) ? row_exp[mrow0 + tid] : 0;  // OZ_THREADS == OZ_BM
    if (tid < BN) sh_colexp[tid] = (n0 + tid < Nx) ? col_exp[n0 + tid] : 0;
    if (warp == 0) tc::tmem_alloc(tmem_slot, TL::TMEM_COLS);
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    constexpr uint32_t idesc = idesc_bf16(OZ_BM, BN);
    const int half_kb = (nkb + 1) / 2;

    // Epilogue coordinates of this thread (GEMM row m, all BN output sites) and its psi operand, loaded now so that
    // the loads overlap the main loop.
    const int m = tid;
    const int j = m >> 1, comp = m & 1;
    const int64_t grow = grow0 + j;
    const int64_t r = grow / Nt;
    const int t = (int)(grow - r * Nt);
    int to;
    bool wrap;  // boundary slice: out = psi + z instead of psi - z
    if (MODE == MODE_M) {
        to = (t + 1 == Nt) ? 0 : t + 1;
        wrap = (to == 0);
    } else if (MODE == MODE_MDAG) {
        to = (t == 0) ? Nt - 1 : t - 1;
        wrap = (t == 0);
    } else {  // MODE_OZ_GEMM: out = Y E^T (o column scale), no shift
        to = t;
        wrap = false;
    }
    const int64_t orow = (r * Nt + to) * Nx;
    const bool row_ok = grow < rows;
    const double *psid = reinterpret_cast<const double *>(psi);
    double pre[BN];
#pragma unroll
    for (int c = 0; c < BN; ++c) {
        const int x = n0 + c;
        pre[c] = (MODE != MODE_OZ_GEMM && row_ok && x < Nx) ? psid[(orow + x) * 2 + comp] : 0.0;
    }

    if (warp == 0 && lane == 0) {
        // TMA producer: S operand-digit tiles and S exp(delta K)-digit tiles per k-block
        int kb = 0;
        for (; kb < nkb; ++kb) {
            const int s = kb % OZ_STAGES;
            if (kb >= OZ_STAGES && !tc::mbar_wait(&bar_empty[s], ((kb / OZ_STAGES) - 1) & 1, err, 21)) {
                *abort_flag = 1;
                break;
            }
            uint8_t *a_base = smem + s * STAGE;
            uint8_t *b_base = a_base + OZ_S * OZ_A_SLICE;
            tc::mbar_arrive_expect_tx(&bar_full[s], STAGE);
#pragma unroll
            for (int l = 0; l < OZ_S; ++l) {
                tc::tma_load_2d(a_base + l * OZ_A_SLICE, &map_a, kb * OZ_BK, (int)(l * mreal + mrow0), &bar_full[s]);
                tc::tma_load_2d(b_base + l * B_SLICE, &map_b, kb * OZ_BK, l * Nx + n0, &bar_full[s]);
            }
        }
        // the last copy into each stage has landed (at once in the normal case; bounded after an abort)
        for (int u = kb - 1; u >= 0 && u >= kb - OZ_STAGES; --u)
            if (!tc::mbar_wait(&bar_full[u % OZ_STAGES], (u / OZ_STAGES) & 1, err, 24)) *abort_flag = 1;
    } else if (warp == 1 && lane == 0) {
        // MMA issuer: per k-block one K = 16 step of every digit pair (a, d - a), d < S
        for (int kb = 0; kb < nkb; ++kb) {
            const int s = kb % OZ_STAGES;
            if (*reinterpret_cast<volatile int *>(abort_flag) ||
                !tc::mbar_wait(&bar_full[s], (kb / OZ_STAGES) & 1, err, 22)) {
                *abort_flag = 1;
                break;
            }
            tc::tc_fence_after();
            uint8_t *a_base = smem + s * STAGE;
            uint8_t *b_base = a_base + OZ_S * OZ_A_SLICE;
            const bool second = (KSPLIT == 2) && (kb >= half_kb);
            const bool first_of_half = (kb == 0) || (KSPLIT == 2 && kb == half_kb);
            // ordered by the operand digit a, so that the A collector buffer serves the S - a products of slice a
#pragma unroll
            for (int a = 0; a < OZ_S; ++a) {
                const uint64_t da = sdesc_kmajor_sw32(tc::smem_addr(a_base + a * OZ_A_SLICE));
#pragma unroll
                for (int b = 0; b < OZ_S - a; ++b) {
                    const int d = a + b;
                    const bool fresh = (KSPLIT == 2 && d < 2) ? first_of_half : kb == 0;
                    // G_3 keeps (0,3), (1,2) in accumulator 3 and (2,1), (3,0) in its own accumulator
                    const bool g3b = (d == 3 && a >= 2);
                    const int acc = g3b ? oz_acc_g3b<KSPLIT>() : ((KSPLIT == 2 && d < 2 && second) ? OZ_S + d : d);
                    const uint32_t dt = tmem + (uint32_t)(acc * BN);
                    const bool first = fresh && (a == 0 || (d == 3 && a == 2));
                    const uint64_t db = sdesc_kmajor_sw32(tc::smem_addr(b_base + b * B_SLICE));
                    const uint32_t accum = first ? 0u : 1u;
                    if (OZ_S - a == 1) mma_bf16<0>(dt, da, db, idesc, accum);
                    else if (b == 0) mma_bf16<1>(dt, da, db, idesc, accum);
                    else if (b == OZ_S - a - 1) mma_bf16<3>(dt, da, db, idesc, accum);
                    else mma_bf16<2>(dt, da, db, idesc, accum);
                }
            }
            tc::mma_commit(&bar_empty[s]);
        }
        tc::mma_commit(bar_done);
    }
    __syncthreads();
    if (!(*abort_flag == 0 && tc::mbar_wait(bar_done, 0, err, 23))) *abort_flag = 1;
    __syncthreads();
    const bool ready = (*abort_flag == 0);  // block-uniform: tcgen05.ld below is warp-collective
    tc::tc_fence_after();

    // epilogue: z = 2^{e_row + e_x - 14} sum_d 2^{-7 d} G_d, then shift / sign / phase / psi -
    // sum_d 2^{-7d} G_d = 2^{-7(OZ_HI-1)} (hi + 2^{-7(S-OZ_HI)} lo), hi = sum_{d<OZ_HI} G_d 2^{7(OZ_HI-1-d)},
    // lo = sum_{d>=OZ_HI} G_d 2^{7(S-1-d)}; |G_d| < 2^26, so hi, lo and the combined integer are exact in 64 bits
    // (up to the rounding of lo's last LO_SHIFT bits, weighted 2^-53 of hi's leading bit). One integer -> FP64
    // conversion per output; the power-of-two scale (and the sign of the M update) come from exponent bits.
    const int escale = sh_rowexp[m] - 14 - 7 * (OZ_HI - 1) - OZ_HI_SHIFT;
    double *outd = reinterpret_cast<double *>(out);
    const uint32_t lane_addr = tmem + ((uint32_t)(32 * warp) << 16);
    // CG extensions: the row's partial sum of squares, and (EPI 2) the system's step and activity
    double sq = 0.0;
    double alpha = 0.0;
    bool act = false;
    if (EPI == 2 && row_ok) {
        const int64_t sys = grow / epi.sys_rows;
        act = epi.active[sys] != 0;
        if (act) alpha = epi.alpha[sys];
    }
    double *rd = reinterpret_cast<double *>(epi.r);
#pragma unroll
    for (int q = 0; q < BN / 8; ++q) {
        const int c0 = 8 * q;
        double rq[8];
        if (EPI == 2 && act) {
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const int x = n0 + c0 + i;
                rq[i] = (x < Nx) ? rd[(orow + x) * 2 + comp] : 0.0;
            }
        }
        double2 ph[8];
        if (MODE == MODE_MDAG || (MODE == MODE_OZ_GEMM && phase)) {
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const int x = n0 + c0 + i;
                ph[i] = (row_ok && x < Nx) ? phase[(int64_t)to * Nx + x] : make_double2(0.0, 0.0);
            }
        }
        uint32_t v[NACC][8];
        if (ready) {
#pragma unroll
            for (int acc = 0; acc < NACC; ++acc) tc::tmem_ld8_async(lane_addr + (uint32_t)(acc * BN + c0), v[acc]);
            tc::tmem_wait_ld<NACC>(v);
        } else {
#pragma unroll
            for (int acc = 0; acc < NACC; ++acc)
#pragma unroll
                for (int i = 0; i < 8; ++i) v[acc][i] = 0u;
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            long long hi = 0, lo = 0;
#pragma unroll
            for (int acc = 0; acc < NACC; ++acc) {
                const int d = oz_acc_order<KSPLIT>(acc);
                const long long g = (long long)__float2int_rn(__uint_as_float(v[acc][i]));  // integer-valued
                if (d < OZ_HI) hi += g * (1ll << (7 * (OZ_HI - 1 - d)));
                else lo += g * (1ll << (7 * (OZ_S - 1 - d)));
            }
            const long long zint = hi * (1ll << OZ_HI_SHIFT) + ((lo + (1ll << (OZ_LO_SHIFT - 1))) >> OZ_LO_SHIFT);
            const int c = c0 + i;
            const int x = n0 + c;
            const int e = escale + sh_colexp[c];
            double res;
            if (MODE == MODE_M) {
                res = fma(signed_pow2(e, !wrap), (double)zint, pre[c]);  // psi -/+ z
            } else if (MODE == MODE_OZ_GEMM) {
                res = (double)zint * pow2i(e);
                if (phase) {  // warp-uniform: column scale z * ph[x]
                    const double partner = __shfl_xor_sync(0xffffffffu, res, 1);
                    const double zr = comp ? partner : res, zi = comp ? res : partner;
                    res = comp ? (ph[i].x * zi + ph[i].y * zr) : (ph[i].x * zr - ph[i].y * zi);
                }
            } else {
                const double zz = (double)zint * pow2i(e);
                const double partner = __shfl_xor_sync(0xffffffffu, zz, 1);
                const double zr = comp ? partner : zz, zi = comp ? zz : partner;
                const double w = comp ? (ph[i].x * zi - ph[i].y * zr) : (ph[i].x * zr + ph[i].y * zi);  // conj(ph) z
                res = fma(wrap ? 1.0 : -1.0, w, pre[c]);
            }
            if (ready && row_ok && x < Nx) {
                const int64_t e = (orow + x) * 2 + comp;
                if (EPI == 2) {
                    if (act) {  // res = (A p) at this site
                        const double rn = fma(-alpha, res, rq[i]);
                        rd[e] = rn;
                        sq = fma(rn, rn, sq);
                    }
                } else {
                    outd[e] = res;
                    if (EPI == 1) sq = fma(res, res, sq);
                }
            }
        }
    }
    if (EPI != 0 && ready && row_ok) epi.part[(grow * 2 + comp) * gridDim.y + blockIdx.y] = sq;
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, TL::TMEM_COLS);
}

// Digit planes of the real part of exp(d K): plane l holds digit l of every row x (scale 2^{e_x} per row), rows of
// ld BF16 (zero padded), the planes stacked along the row axis (S * Nx rows) for one 2-D tensor map.
__global__ void k_oz_planes(const double2 *__restrict__ E, __nv_bfloat16 *planes, int *col_exp, int Nx, int ld) {
    const int x = blockIdx.x;
    double m = 0;
    for (int y = threadIdx.x; y < Nx; y += blockDim.x) m = fmax(m, fabs(E[(int64_t)x * Nx + y].x));
    __shared__ double red[256];
    red[threadIdx.x] = m;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
        __syncthreads();
    }
    int e = 0;
    if (red[0] > 0) frexp(red[0], &e);
    if (threadIdx.x == 0) col_exp[x] = e;
    for (int y = threadIdx.x; y < ld; y += blockDim.x) {
        const double v = (y < Nx) ? E[(int64_t)x * Nx + y].x : 0.0;
        const unsigned long long U = scaled_magnitude(v, e);
#pragma unroll
        for (int l = 0; l < OZ_S; ++l) planes[((int64_t)l * Nx + x) * ld + y] = digit(U, l, v < 0.0);
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void *p = nullptr;
        if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

int make_map_bf16(CUtensorMap *map, const void *base, int64_t rows, int ld, int box_rows) {
    auto fn = encode_fn();
    NSLG_REQUIRE(fn != nullptr, NSLG_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    const cuuint64_t dims[2] = {(cuuint64_t)ld, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    const cuuint32_t box[2] = {(cuuint32_t)OZ_BK, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_32B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    NSLG_REQUIRE(r == CUDA_SUCCESS, NSLG_ERR_CUDA,
                 "cuTensorMapEncodeTiled (bf16) failed (" + std::to_string((int)r) + ")");
    return NSLG_OK;
}

template <int MODE, int KSPLIT> int set_smem_attr_gemm() {
    NSLG_CUDA(cudaFuncSetAttribute(k_fm_apply_oz<MODE, KSPLIT, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   OzTile<KSPLIT>::SMEM));
    return NSLG_OK;
}

template <int MODE, int KSPLIT> int set_smem_attr() {
    NSLG_CUDA(cudaFuncSetAttribute(k_fm_apply_oz<MODE, KSPLIT, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   OzTile<KSPLIT>::SMEM));
    NSLG_CUDA(cudaFuncSetAttribute(k_fm_apply_oz<MODE, KSPLIT, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   OzTile<KSPLIT>::SMEM));
    NSLG_CUDA(cudaFuncSetAttribute(k_fm_apply_oz<MODE, KSPLIT, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   OzTile<KSPLIT>::SMEM));
    return NSLG_OK;
}

}  // namespace

int oz_ld(int Nx) { return (int)ceil_div(Nx, OZ_LD_ALIGN) * OZ_LD_ALIGN; }
int oz_digits() { return OZ_S; }

int oz_planes(nslg_fm *fm, const ExpEntry *e, OzPlanes **out) {
    auto *E = const_cast<ExpEntry *>(e);
    if (!E->oz) {
        NSLG_REQUIRE(E->is_real, NSLG_ERR_UNSUPPORTED, "split-BF16 operator needs a real exp(delta K)");
        const int Nx = (int)fm->Nx;
        NSLG_REQUIRE(Nx <= 2048, NSLG_ERR_UNSUPPORTED, "split-BF16 operator supports Nx <= 2048");
        auto *P = new OzPlanes;
        P->ld = oz_ld(Nx);
        const size_t n = (size_t)OZ_S * Nx * P->ld;
        if (cudaMalloc(&P->planes, n * sizeof(__nv_bfloat16)) != cudaSuccess ||
            cudaMalloc(&P->col_exp, Nx * sizeof(int)) != cudaSuccess) {
            cudaGetLastError();
            cudaFree(P->planes);
            delete P;
            set_error("split-BF16 planes: device allocation failed");
            return NSLG_ERR_OOM;
        }
        k_oz_planes<<<Nx, 256, 0, fm->ctx->stream>>>(E->full, static_cast<__nv_bfloat16 *>(P->planes), P->col_exp,
                                                      Nx, P->ld);
        note_launch(fm->ctx->stream);
        NSLG_CUDA(cudaGetLastError());
        NSLG_TRY(make_map_bf16(&P->map, P->planes, (int64_t)OZ_S * Nx, P->ld, P->ld > 1024 ? OzTile<2>::BN : OzTile<1>::BN));
        NSLG_TRY(set_smem_attr<MODE_M, 1>());
        NSLG_TRY(set_smem_attr<MODE_M, 2>());
        NSLG_TRY(set_smem_attr<MODE_MDAG, 1>());
        NSLG_TRY(set_smem_attr<MODE_MDAG, 2>());
        NSLG_TRY(set_smem_attr_gemm<MODE_OZ_GEMM, 1>());
        NSLG_TRY(set_smem_attr_gemm<MODE_OZ_GEMM, 2>());
        E->oz = P;
    }
    *out = E->oz;
    return NSLG_OK;
}

// digits: workspace of S * 2 * rows * ld BF16; rexp: 2 * rows ints.
namespace {

template <int KSPLIT, int EPI>
void launch_oz(int mode, dim3 grid, cudaStream_t st, const double2 *psi, double2 *out, const double2 *phase,
               const int *rexp, const int *col_exp, const CUtensorMap &map_a, const CUtensorMap &map_b, int Nt, int Nx,
               int64_t rows, int nkb, int *err, const OzEpi &epi) {
    constexpr int smem = OzTile<KSPLIT>::SMEM;
    if (mode == MODE_M)
        k_fm_apply_oz<MODE_M, KSPLIT, EPI><<<grid, OZ_THREADS, smem, st>>>(psi, out, phase, rexp, col_exp, map_a, map_b,
                                                                           Nt, Nx, rows, nkb, err, epi);
    else
        k_fm_apply_oz<MODE_MDAG, KSPLIT, EPI><<<grid, OZ_THREADS, smem, st>>>(psi, out, phase, rexp, col_exp, map_a,
                                                                              map_b, Nt, Nx, rows, nkb, err, epi);
}

template <int KSPLIT>
void launch_oz_epi(int mode, dim3 grid, cudaStream_t st, const double2 *psi, double2 *out, const double2 *phase,
                   const int *rexp, const int *col_exp, const CUtensorMap &map_a, const CUtensorMap &map_b, int Nt,
                   int Nx, int64_t rows, int nkb, int *err, const OzEpi &epi) {
    if (epi.mode == 1)
        launch_oz<KSPLIT, 1>(mode, grid, st, psi, out, phase, rexp, col_exp, map_a, map_b, Nt, Nx, rows, nkb, err, epi);
    else if (epi.mode == 2)
        launch_oz<KSPLIT, 2>(mode, grid, st, psi, out, phase, rexp, col_exp, map_a, map_b, Nt, Nx, rows, nkb, err, epi);
    else
        launch_oz<KSPLIT, 0>(mode, grid, st, psi, out, phase, rexp, col_exp, map_a, map_b, Nt, Nx, rows, nkb, err, epi);
}

}  // namespace

int oz_ntiles(int Nx) {
    return (int)ceil_div(Nx, oz_ld(Nx) > 1024 ? OzTile<2>::BN : OzTile<1>::BN);
}

int oz_gemm(const double2 *Y, double2 *out, const double2 *pro_scale, const double2 *epi_scale, const OzPlanes &P,
            void *digits, int *rexp, int Nx, int64_t rows, int *err, cudaStream_t st) {
    if (rows == 0) return NSLG_OK;
    auto *dg = static_cast<__nv_bfloat16 *>(digits);
    const unsigned blocks = (unsigned)ceil_div(rows, 8);
    // the operand's digits: Y o pro_scale (one row of Nx per column) or Y itself (one "time slice": Nt = 1)
    if (pro_scale) k_oz_digits<MODE_M><<<blocks, 256, 0, st>>>(Y, pro_scale, 1, Nx, rows, P.ld, dg, rexp, nullptr, 1);
    else k_oz_digits<MODE_MDAG><<<blocks, 256, 0, st>>>(Y, nullptr, 1, Nx, rows, P.ld, dg, rexp, nullptr, 1);
    note_launch(st);
    NSLG_CUDA(cudaGetLastError());
    CUtensorMap map_a;
    NSLG_TRY(make_map_bf16(&map_a, digits, (int64_t)OZ_S * 2 * rows, P.ld, OZ_BM));
    const int nkb = P.ld / OZ_BK;
    const OzEpi plain;
    if (P.ld > 1024) {
        dim3 grid((unsigned)ceil_div(rows, OZ_BM / 2), (unsigned)ceil_div(Nx, OzTile<2>::BN));
        k_fm_apply_oz<MODE_OZ_GEMM, 2, 0><<<grid, OZ_THREADS, OzTile<2>::SMEM, st>>>(
            nullptr, out, epi_scale, rexp, P.col_exp, map_a, P.map, 1, Nx, rows, nkb, err, plain);
    } else {
        dim3 grid((unsigned)ceil_div(rows, OZ_BM / 2), (unsigned)ceil_div(Nx, OzTile<1>::BN));
        k_fm_apply_oz<MODE_OZ_GEMM, 1, 0><<<grid, OZ_THREADS, OzTile<1>::SMEM, st>>>(
            nullptr, out, epi_scale, rexp, P.col_exp, map_a, P.map, 1, Nx, rows, nkb, err, plain);
    }
    note_launch(st);
    NSLG_CUDA(cudaGetLastError());
    return NSLG_OK;
}

int fm_apply_oz(int mode, const double2 *psi, double2 *out, const double2 *phase, const OzPlanes &P, void *digits,
                int *rexp, int Nt, int Nx, int64_t rows, int *err, cudaStream_t st, const OzEpi *epi) {
    if (rows == 0) return NSLG_OK;
    const OzEpi plain;
    const OzEpi &E = epi ? *epi : plain;
    // the residual epilogue divides rows into systems: a system is at least one row, and rows cover whole systems
    NSLG_REQUIRE(E.mode != 2 || (E.sys_rows >= 1 && rows % E.sys_rows == 0), NSLG_ERR_ARG,
                 "split-BF16 CG epilogue: rows per system must divide the rows");
    auto *dg = static_cast<__nv_bfloat16 *>(digits);
    const unsigned blocks = (unsigned)ceil_div(rows, 8);
    NSLG_REQUIRE(!E.go || (E.sys_rows >= 1 && rows % E.sys_rows == 0), NSLG_ERR_ARG,
                 "split-BF16 system skipping: rows per system must divide the rows");
    if (mode == MODE_M)
        k_oz_digits<MODE_M><<<blocks, 256, 0, st>>>(psi, phase, Nt, Nx, rows, P.ld, dg, rexp, E.go, E.sys_rows);
    else
        k_oz_digits<MODE_MDAG><<<blocks, 256, 0, st>>>(psi, phase, Nt, Nx, rows, P.ld, dg, rexp, E.go, E.sys_rows);
    note_launch(st);
    NSLG_CUDA(cudaGetLastError());
    CUtensorMap map_a;
    NSLG_TRY(make_map_bf16(&map_a, digits, (int64_t)OZ_S * 2 * rows, P.ld, OZ_BM));
    const int nkb = P.ld / OZ_BK;
    if (P.ld > 1024) {
        dim3 grid((unsigned)ceil_div(rows, OZ_BM / 2), (unsigned)ceil_div(Nx, OzTile<2>::BN));
        launch_oz_epi<2>(mode, grid, st, psi, out, phase, rexp, P.col_exp, map_a, P.map, Nt, Nx, rows, nkb, err, E);
    } else {
        dim3 grid((unsigned)ceil_div(rows, OZ_BM / 2), (unsigned)ceil_div(Nx, OzTile<1>::BN));
        launch_oz_epi<1>(mode, grid, st, psi, out, phase, rexp, P.col_exp, map_a, P.map, Nt, Nx, rows, nkb, err, E);
    }
    note_launch(st);
    NSLG_CUDA(cudaGetLastError());
    return NSLG_OK;
}

}  // namespace nslg
