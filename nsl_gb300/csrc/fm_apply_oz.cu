// FP64-class fermion-matrix applications on the tensor cores: split BF16 digits with exact FP32 accumulation.
//
// The CG on MM^dagger at low temperature is so ill-conditioned (|A| |x| / |b| ~ 1e7 at beta = 8) that an FP32-class
// operator stops reducing the true residual near 1e-6; the last decades need an FP64-class operator. GB300 executes
// FP64 at ~1.2 TFLOP/s (about 2 FP64 operations per clock per SM), so this kernel builds one from BF16 tensor-core
// products whose sums are exact integers:
//
//   every operand row is scaled by a power of two 2^e (|v| < 2^e), rounded to a 53-bit integer and cut into S = 6
//   balanced base-512 digits
//     v = 2^{e-8} sum_{k<S} a_k 2^{-9k},   a_0 in [-256, 256], a_k in [-256, 255] (k > 0),
//   every one of them an integer of magnitude <= 2^8, exactly representable in BF16 (8 significant bits). A product
//   of two digit matrices over K sites is an integer matrix; grouping the digit products by d = k + l (the same power
//   of two) into TMEM accumulators G_d and keeping d < S gives
//     Y E^T = 2^{e_row + e_x - 16} sum_{d<S} 2^{-9d} G_d  (+ the dropped orders d >= S).
//   Rounding to nearest and balanced (signed) digits make the representation and the dropped orders unbiased, so
//   the result carries ~53 bits: measured 1e-15..3e-15 relative to the output's maximum, against 1e-15 for an FP64
//   product over the same K.
//
// Exactness. An FP32 accumulator is exact while every partial sum is an integer below 2^24. With |a_k| <= 256,
//   |G_d(x)| <= 256 sum_{l<=d} B_l(x),   B_l(x) = sum_y |b_l(x, y)|
// for EVERY operand, where b_l are the digits of row x of exp(delta K). exp(delta K) is localised (its entries decay
// like delta^dist / dist!), so B_l is far below its K 256 worst case: at honeycomb 12x12, delta = 1/8, the bound of
// G_3 is 0.23 2^24 and that of G_5 0.68 2^24. k_oz_planes evaluates the bound once per exp(delta K); the orders
// d <= 3 must stay below 2^24 (exact), d = 4, 5 (weight 2^-36 or less) below 2^30 (their rounding is below the
// representation's own error). A matrix that fails the bound (exp(delta K) of a very large delta) is flagged: every
// launch with it reports NSLG_ERR_CUDA through the handle's tensor-core error flag, so its results are never used
// silently.
//
// GB300's FP64 pipe (~2 operations per clock per SM) and, for N = 32 MMAs, the tensor core's shared-memory operand
// reads (~44 cycles per M = 128, N = 32, K = 16 instruction measured on this part, 128 at N = 256) bound the work, so:
//  * k_oz_digits: one warp per (r, t) row computes Y = phase o psi (M) or psi (M^dagger) once (kept in registers
//    for rows of up to 32 * OZ_CACHE sites), the row's power-of-two scales (real and imaginary rows separately) from
//    integer maxima of the FP64 bit patterns, and writes the S digit planes of the operand (BF16 pairs, rows padded
//    to a multiple of 32 sites) with integer operations. FP64 work: the phase product only. (In the fused CG
//    iteration on M M^dagger the operands come ready: the M^dagger epilogue forms phase o tmp and the CG update
//    kernel writes the digits of the next search direction.)
//  * k_fm_apply_oz: a persistent, warp-specialised TMA -> tcgen05 pipeline (see the kernel): 21 digit MMAs per
//    16-site k-block into S = 6 TMEM accumulators, two accumulator sets so that the epilogue of one 128 x 32 tile
//    overlaps the MMAs of the next; the epilogue recombines the integer-valued G_d in 64-bit integers (exact),
//    builds the FP64 value from integer operations, then applies the time shift, boundary sign, conj(phase)
//    (M^dagger) and psi -.
//
// The same pipeline serves (oz_gemm, MODE_OZ_GEMM) the matrix chains of the log-det gradient: a plain product
// out = (Y o pro) E^T (o epi) of a complex matrix Y with a real matrix E, optionally column-scaled before (in the
// digit pre-pass) or after (in the epilogue).

#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>

#include "fm_internal.cuh"
#include "oz_digits.cuh"
#include "tc_common.cuh"

namespace nslg {

namespace {

constexpr int OZ_BM = 128;       // real GEMM rows per tile (64 complex rows)
constexpr int OZ_BK = 16;        // sites per k-block: 32 bytes of BF16, one MMA K step
constexpr int OZ_NACC = OZ_S;    // one TMEM accumulator per order d < S
constexpr int OZ_BN = 32;        // output sites per tile
constexpr int OZ_ROWB = OZ_BK * 2;           // bytes per smem row
constexpr int OZ_A_SLICE = OZ_BM * OZ_ROWB;  // 4 KB
constexpr int OZ_B_SLICE = OZ_BN * OZ_ROWB;  // 1 KB
constexpr int OZ_STAGE = OZ_S * (OZ_A_SLICE + OZ_B_SLICE);  // 30 KB per k-block
constexpr int OZ_LD_ALIGN = 32;              // digit-plane rows are padded to a multiple of 32 sites
// persistent kernel: one CTA per SM, warp 0 TMA, warp 1 MMA + TMEM, OZP_EPI_WARPS epilogue warps
constexpr int OZP_EPI_WARPS = 8;
constexpr int OZP_THREADS = 64 + 32 * OZP_EPI_WARPS;
constexpr int OZP_STAGES = 7;                // TMA -> MMA ring depth (7 x 30 KB)
constexpr int OZP_TMEM_COLS = 512;           // two accumulator sets of OZ_NACC * OZ_BN = 192 columns
constexpr int OZP_SMEM = OZP_STAGES * OZ_STAGE + 1024 /*alignment*/ + 1024 /*barriers*/;
static_assert(OZ_W * OZ_S - 1 == 53, "the operand is rounded to a 53-bit integer (sh >= 0 in scaled_int)");
static_assert(2 * OZ_NACC * OZ_BN <= OZP_TMEM_COLS, "TMEM columns");
static_assert(OZP_SMEM <= 227 * 1024, "shared memory per CTA");
static_assert(OZ_BN % 16 == 0 && OZ_BN == 32, "MMA N for M = 128; the epilogue groups take 16 sites each");
static_assert(OZP_EPI_WARPS == 8, "two epilogue groups of four warps (one per TMEM lane quarter)");
// Recombination: sum_d 2^{-9d} G_d = 2^{-9(HI-1)} (hi + 2^{-9(S-HI)} lo), hi = sum_{d<HI} G_d 2^{9(HI-1-d)},
// lo = sum_{d>=HI} G_d 2^{9(S-1-d)}. With |G_d| < 2^24 (d <= 3) and < 2^30 (d > 3), |hi|, |lo| < 2^42.2; one 64-bit
// integer per output is hi 2^HI_SHIFT + round(lo 2^-LO_SHIFT) < 2^61.2.
constexpr int OZ_HI = 3;
constexpr int OZ_HI_SHIFT = 19;
constexpr int OZ_LO_SHIFT = OZ_W * (OZ_S - OZ_HI) - OZ_HI_SHIFT;
static_assert(OZ_LO_SHIFT > 0, "lo is rounded into the combined integer");
// z = 2^{e_row + e_x - 16} sum_d 2^{-9d} G_d = 2^{e_row + e_x - OZ_ZSHIFT} zint
constexpr int OZ_ZSHIFT = 2 * (OZ_W - 1) + OZ_W * (OZ_HI - 1) + OZ_HI_SHIFT;
static_assert(OZ_ZSHIFT == 53, "recombination scale");
// Digit-sum bounds (k_oz_planes): orders d < OZ_EXACT must stay exact (< 2^24), the others below 2^30.
constexpr int OZ_EXACT = 4;
constexpr int OZ_ERR_BOUND = 31;  // tensor-core error code: exp(delta K) fails the digit-sum bound

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
// 3 = lastuse (A from the buffer, then released): consecutive MMAs on the same A slice may reuse it (the instruction
// rate measured on this part is the same with and without the collector, ~44 cycles per N = 32 MMA).
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

// zint 2^e as an FP64 value (rounded to nearest, ties away from zero) from integer operations only: GB300 runs an
// integer -> FP64 conversion and the scaling multiply on its FP64 pipe, ~2 operations per clock per SM.
__device__ __forceinline__ double scaled_to_double(long long zint, int e) {
    if (zint == 0) return 0.0;
    const unsigned long long sign = zint < 0 ? (1ull << 63) : 0ull;
    unsigned long long u = zint < 0 ? 0ull - (unsigned long long)zint : (unsigned long long)zint;
    const int lz = __clzll((long long)u);
    u <<= lz;                                                 // leading one at bit 63: |zint| = u 2^-lz
    unsigned long long m = (u >> 11) + ((u >> 10) & 1ull);    // 53 significant bits, rounded
    int ex = e + 63 - lz;                                     // |zint| 2^e = (m / 2^52) 2^ex
    if (m >> 53) {                                            // the rounding carried into a 54th bit
        m >>= 1;
        ++ex;
    }
    if (ex < -1022) return __longlong_as_double((long long)sign);                         // below the normal range: 0
    if (ex > 1023) return __longlong_as_double((long long)(sign | 0x7FF0000000000000ull));  // above it: infinity
    return __longlong_as_double((long long)(sign | ((unsigned long long)(ex + 1023) << 52) | (m & 0xFFFFFFFFFFFFFull)));
}

template <int MODE>
__device__ __forceinline__ double2 oz_operand(const double2 *__restrict__ psi, const double2 *__restrict__ phase,
                                              int64_t grow, int t, int Nx, int y) {
    double2 v = psi[grow * Nx + y];
    if (MODE == MODE_M) v = cmul(phase[(int64_t)t * Nx + y], v);
    return v;
}

// FP64 bit patterns (re, im at y; re, im at y + 1) of the operand at the site pair y, y + 1 (zero beyond Nx).
template <int MODE>
__device__ __forceinline__ void operand_pair(const double2 *__restrict__ psi, const double2 *__restrict__ phase,
                                             int64_t grow, int t, int Nx, int y, unsigned long long (&b)[4]) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        b[2 * h] = b[2 * h + 1] = 0ull;
        if (y + h < Nx) {
            const double2 v = oz_operand<MODE>(psi, phase, grow, t, Nx, y + h);
            b[2 * h] = (unsigned long long)__double_as_longlong(v.x);
            b[2 * h + 1] = (unsigned long long)__double_as_longlong(v.y);
        }
    }
}

// One warp per complex row (r, t): scales e (max |Y| < 2^e, real and imaginary GEMM rows separately) and the digit
// planes A[l][2 row + c][y] (ld sites, zero padded). Lanes take site pairs (4-byte BF16 stores).
template <int MODE>
__global__ void __launch_bounds__(256, 2)
    k_oz_digits(const double2 *__restrict__ psi, const double2 *__restrict__ phase, int Nt, int Nx, int64_t rows,
                int ld, __nv_bfloat16 *__restrict__ planes, int *__restrict__ ex, const int *__restrict__ go,
                int64_t sys_rows) {
    constexpr int NP = OZ_CACHE / 2;  // site pairs a lane keeps in registers (rows of <= 64 * NP sites)
    const int64_t grow = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x % 32;
    if (grow >= rows) return;
    if (go && !go[grow / sys_rows]) return;  // a finished system's row (one warp per row: the warp leaves whole)
    const int t = (int)(grow % Nt);
    // the row's operand values as FP64 bit patterns; everything after the phase product is integer work
    unsigned long long c[NP][4];
    unsigned long long mr = 0, mi = 0;
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        operand_pair<MODE>(psi, phase, grow, t, Nx, 2 * (lane + 32 * k), c[k]);
        mr = max(mr, max(c[k][0] & 0x7FFFFFFFFFFFFFFFull, c[k][2] & 0x7FFFFFFFFFFFFFFFull));
        mi = max(mi, max(c[k][1] & 0x7FFFFFFFFFFFFFFFull, c[k][3] & 0x7FFFFFFFFFFFFFFFull));
    }
    for (int y = 2 * (lane + 32 * NP); y < Nx; y += 64) {  // rows longer than the register cache
        unsigned long long b[4];
        operand_pair<MODE>(psi, phase, grow, t, Nx, y, b);
        mr = max(mr, max(b[0] & 0x7FFFFFFFFFFFFFFFull, b[2] & 0x7FFFFFFFFFFFFFFFull));
        mi = max(mi, max(b[1] & 0x7FFFFFFFFFFFFFFFull, b[3] & 0x7FFFFFFFFFFFFFFFull));
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
    for (int k = 0; k < NP; ++k) {
        const int y = 2 * (lane + 32 * k);
        if (y < ld) write_digits2(planes, mreal, grow, ld, y, c[k], er, ei);
    }
    for (int y = 2 * (lane + 32 * NP); y < ld; y += 64) {
        unsigned long long b[4];
        operand_pair<MODE>(psi, phase, grow, t, Nx, y, b);
        write_digits2(planes, mreal, grow, ld, y, b, er, ei);
    }
}

// Persistent, warp-specialised split-BF16 kernel: one CTA per SM walks the (row block, site block) tiles
// t = blockIdx.x, blockIdx.x + gridDim.x, ... (site blocks fastest, so the CTAs working at one time share the
// operand rows of a few row blocks in L2). Warp 0 (one thread) streams the digit tiles of every k-block of every tile
// through an OZP_STAGES-deep TMA ring; warp 1 (one thread) issues the 21 MMAs per k-block into one of two TMEM
// accumulator sets (2 x 192 columns) and commits each finished tile to its set's `full` barrier; warps 2..9 (two
// groups of four, one TMEM lane quarter each; group g takes sites [16 g, 16 g + 16) of the tile) recombine, finish
// and store a tile while the MMAs of the next one run, then release its accumulator set. Every wait is bounded: a
// timeout records an error code, sets the CTA's abort flag, and all roles leave their loops; the producer waits
// (bounded) for its own copies and the issuer for its own MMAs before TMEM is freed.
template <int MODE, int EPI>
__global__ void __launch_bounds__(OZP_THREADS, 1)
    k_fm_apply_oz(const double2 *__restrict__ psi, double2 *__restrict__ out, const double2 *__restrict__ phase,
                  const int *__restrict__ row_exp, const int *__restrict__ col_exp,
                  const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b, int Nt,
                  int Nx, int64_t rows, int nkb, int *err, const OzEpi epi) {
    constexpr int BN = OZ_BN, STAGE = OZ_STAGE, NACC = OZ_NACC;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *bar_full = reinterpret_cast<uint64_t *>(smem + OZP_STAGES * STAGE);
    uint64_t *bar_empty = bar_full + OZP_STAGES;
    uint64_t *bar_tfull = bar_empty + OZP_STAGES;  // [2]: an accumulator set holds a finished tile
    uint64_t *bar_tempty = bar_tfull + 2;          // [2]: the epilogue has read an accumulator set
    uint64_t *bar_done = bar_tempty + 2;           // every MMA of this CTA has completed
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bar_done + 1);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(bar_done + 2);

    const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
    const int64_t mreal = 2 * rows;
    const int nmt = (int)((rows + OZ_BM / 2 - 1) / (OZ_BM / 2));
    const int ntn = (Nx + BN - 1) / BN;
    const int ntiles = nmt * ntn;
    // a tile whose rows all belong to finished systems is skipped by every role alike
    auto live = [&](int t) -> bool {
        if (!epi.go) return true;
        const int64_t g0 = (int64_t)(t / ntn) * (OZ_BM / 2);
        const int64_t last = min(rows, g0 + OZ_BM / 2) - 1;
        for (int64_t s = g0 / epi.sys_rows; s <= last / epi.sys_rows; ++s)
            if (epi.go[s] != 0) return true;
        return false;
    };

    if (tid == 0) {
        for (int i = 0; i < OZP_STAGES; ++i) {
            tc::mbar_init(&bar_full[i], 1);
            tc::mbar_init(&bar_empty[i], 1);
        }
        for (int i = 0; i < 2; ++i) {
            tc::mbar_init(&bar_tfull[i], 1);
            tc::mbar_init(&bar_tempty[i], OZP_EPI_WARPS);
        }
        tc::mbar_init(bar_done, 1);
        *abort_flag = 0;
        tc::fence_mbar_init();
        tc::prefetch_tmap(&map_a);
        tc::prefetch_tmap(&map_b);
        if (col_exp[Nx] != 0 && err) atomicExch(err, OZ_ERR_BOUND);  // exp(delta K) failed the digit-sum bound
    }
    if (warp == 1) tc::tmem_alloc(tmem_slot, OZP_TMEM_COLS);
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    constexpr uint32_t idesc = idesc_bf16(OZ_BM, BN);

    if (warp == 0) {
        if (lane == 0) {  // TMA producer: S operand-digit tiles and S exp(delta K)-digit tiles per k-block
            int it = 0;
            for (int t = blockIdx.x; t < ntiles && !*abort_flag; t += gridDim.x) {
                if (!live(t)) continue;
                const int64_t mrow0 = (int64_t)(t / ntn) * OZ_BM;
                const int n0 = (t % ntn) * BN;
                for (int kb = 0; kb < nkb; ++kb, ++it) {
                    const int s = it % OZP_STAGES;
                    if (it >= OZP_STAGES &&
                        (*abort_flag || !tc::mbar_wait(&bar_empty[s], ((it / OZP_STAGES) - 1) & 1, err, 21))) {
                        *abort_flag = 1;
                        break;
                    }
                    uint8_t *a_base = smem + s * STAGE;
                    uint8_t *b_base = a_base + OZ_S * OZ_A_SLICE;
                    tc::mbar_arrive_expect_tx(&bar_full[s], STAGE);
#pragma unroll
                    for (int l = 0; l < OZ_S; ++l) {
                        tc::tma_load_2d(a_base + l * OZ_A_SLICE, &map_a, kb * OZ_BK, (int)(l * mreal + mrow0),
                                        &bar_full[s]);
                        tc::tma_load_2d(b_base + l * OZ_B_SLICE, &map_b, kb * OZ_BK, l * Nx + n0, &bar_full[s]);
                    }
                }
            }
            // the last copy into each stage has landed (at once in the normal case; bounded after an abort)
            for (int u = it - 1; u >= 0 && u >= it - OZP_STAGES; --u)
                if (!tc::mbar_wait(&bar_full[u % OZP_STAGES], (u / OZP_STAGES) & 1, err, 24)) *abort_flag = 1;
        }
    } else if (warp == 1) {
        if (lane == 0) {  // MMA issuer
            int it = 0, tc_n = 0;
            const uint64_t dsm0 = sdesc_kmajor_sw32(tc::smem_addr(smem));  // descriptor of stage 0, slice 0
            for (int t = blockIdx.x; t < ntiles && !*abort_flag; t += gridDim.x) {
                if (!live(t)) continue;
                const int buf = tc_n & 1, use = tc_n >> 1;
                if (use >= 1 && !tc::mbar_wait(&bar_tempty[buf], (use - 1) & 1, err, 25)) {
                    *abort_flag = 1;
                    break;
                }
                tc::tc_fence_after();
                const uint32_t dbase = tmem + (uint32_t)(buf * NACC * BN);
                bool ok = true;
                for (int kb = 0; kb < nkb; ++kb, ++it) {
                    const int s = it % OZP_STAGES;
                    if (*abort_flag || !tc::mbar_wait(&bar_full[s], (it / OZP_STAGES) & 1, err, 22)) {
                        ok = false;
                        break;
                    }
                    // (no tcgen05 fence here: the stage's completed transaction count already makes the TMA writes
                    // visible to the MMAs; a fence per k-block costs ~250 cycles of this thread's issue stream)
                    // ordered by the operand digit a, so that the A collector buffer serves the S - a products of
                    // slice a; accumulator d = a + b starts (accumulate = 0) with its first product (0, d) of the
                    // tile's first k-block. The issue rate of this one thread bounds the kernel (N = 32 MMAs take
                    // ~17 tensor-pipe cycles each), so every descriptor is the stage's base descriptor plus a
                    // compile-time offset (the address field is bits 0-13 of the descriptor, in 16-byte units).
                    const uint64_t dst = dsm0 + (uint64_t)((s * STAGE) >> 4);
                    const uint32_t acc0 = kb == 0 ? 0u : 1u;
#pragma unroll
                    for (int a = 0; a < OZ_S; ++a) {
                        const uint64_t da = dst + (uint64_t)((a * OZ_A_SLICE) >> 4);
#pragma unroll
                        for (int b = 0; b < OZ_S - a; ++b) {
                            const uint32_t dt = dbase + (uint32_t)((a + b) * BN);
                            const uint64_t db = dst + (uint64_t)((OZ_S * OZ_A_SLICE + b * OZ_B_SLICE) >> 4);
                            const uint32_t accum = a == 0 ? acc0 : 1u;
                            if (OZ_S - a == 1) mma_bf16<0>(dt, da, db, idesc, accum);
                            else if (b == 0) mma_bf16<1>(dt, da, db, idesc, accum);
                            else if (b == OZ_S - a - 1) mma_bf16<3>(dt, da, db, idesc, accum);
                            else mma_bf16<2>(dt, da, db, idesc, accum);
                        }
                    }
                    tc::mma_commit(&bar_empty[s]);
                }
                if (!ok) {
                    *abort_flag = 1;
                    break;
                }
                tc::mma_commit(&bar_tfull[buf]);
                ++tc_n;
            }
            // every MMA issued by this thread has completed before TMEM may be freed
            tc::mma_commit(bar_done);
            if (!tc::mbar_wait(bar_done, 0, err, 23)) *abort_flag = 1;
        }
    } else {
        // Epilogue. TMEM lane = GEMM row m of the tile (real or imaginary part of complex row j), sites
        // [16 g, 16 g + 16) of its 32. After recombination the two lanes of a complex row swap halves, so that each
        // lane finishes whole complex values at alternate sites (even sites: the real-part lane, odd: the imaginary
        // one): complex arithmetic without further shuffles, and every global access of the warp covers 16 rows x
        // 32 contiguous bytes. The operands of a tile (psi, and r or the phases) are loaded before its
        // accumulators are ready.
        const int ew = warp - 2;
        const int g = ew / 4;
        const int m = 32 * (warp % 4) + lane;
        const int j = m >> 1, comp = m & 1;
        const uint32_t lane_base = tmem + ((uint32_t)(32 * (warp % 4)) << 16);
        constexpr int EC = BN / 2;  // sites per lane pair
        constexpr int NS = EC / 2;  // complex values per lane
        int tc_n = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
            if (!live(t)) continue;
            if (*abort_flag) break;
            const int buf = tc_n & 1, use = tc_n >> 1;
            const int mt = t / ntn, nt = t % ntn;
            const int64_t grow = (int64_t)mt * (OZ_BM / 2) + j;
            const int64_t r = grow / Nt;
            const int tt = (int)(grow - r * Nt);
            int to;
            bool wrap;  // boundary slice: out = psi + z instead of psi - z
            if (MODE == MODE_M) {
                to = (tt + 1 == Nt) ? 0 : tt + 1;
                wrap = (to == 0);
            } else if (MODE == MODE_MDAG) {
                to = (tt == 0) ? Nt - 1 : tt - 1;
                wrap = (tt == 0);
            } else {  // MODE_OZ_GEMM: out = Y E^T (o column scale), no shift
                to = tt;
                wrap = false;
            }
            const int64_t orow = (r * Nt + to) * Nx;
            const bool row_ok = grow < rows;
            const int x0 = nt * BN + g * EC;
            double alpha = 0.0;
            bool act = false;
            if (EPI == 2 && row_ok) {
                const int64_t sys = grow / epi.sys_rows;
                act = epi.active[sys] != 0;
                if (act) alpha = epi.alpha[sys];
            }
            // this lane's complex values: sites x0 + 2 s + comp
            constexpr bool PH = MODE != MODE_M;  // the epilogue multiplies by phases (M^dagger, scaled products)
            double2 pre[NS], rq[NS], ph[NS];       // psi; r (EPI 2); the phases
#pragma unroll
            for (int s = 0; s < NS; ++s) {
                const int x = x0 + 2 * s + comp;
                const bool ok = row_ok && x < Nx;
                pre[s] = (MODE != MODE_OZ_GEMM && ok) ? psi[orow + x] : make_double2(0.0, 0.0);
                rq[s] = (EPI == 2 && act && x < Nx) ? epi.r[orow + x] : make_double2(0.0, 0.0);
                ph[s] = (PH && ok && (MODE == MODE_MDAG || phase)) ? phase[(int64_t)to * Nx + x]
                                                                    : make_double2(0.0, 0.0);
            }
            const int escale = (row_ok ? row_exp[(int64_t)mt * OZ_BM + m] : 0) - OZ_ZSHIFT;
            if (!tc::mbar_wait(&bar_tfull[buf], use & 1, err, 26)) {
                *abort_flag = 1;
                break;
            }
            tc::tc_fence_after();
            double sq = 0.0;
#pragma unroll
            for (int q = 0; q < EC / 8; ++q) {
                const int c0 = 8 * q;
                uint32_t v[NACC][8];
#pragma unroll
                for (int d = 0; d < NACC; ++d)
                    tc::tmem_ld8_async(lane_base + (uint32_t)(buf * NACC * BN + d * BN + g * EC + c0), v[d]);
                tc::tmem_wait_ld<NACC>(v);
                double z[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    long long hi = 0, lo = 0;
#pragma unroll
                    for (int d = 0; d < NACC; ++d) {
                        const long long gd = (long long)__float2int_rn(__uint_as_float(v[d][i]));  // integer-valued
                        if (d < OZ_HI) hi += gd * (1ll << (OZ_W * (OZ_HI - 1 - d)));
                        else lo += gd * (1ll << (OZ_W * (OZ_S - 1 - d)));
                    }
                    const long long zint =
                        hi * (1ll << OZ_HI_SHIFT) + ((lo + (1ll << (OZ_LO_SHIFT - 1))) >> OZ_LO_SHIFT);
                    const int x = x0 + c0 + i;
                    z[i] = scaled_to_double(zint, escale + ((x < Nx) ? col_exp[x] : 0));
                }
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int s = 4 * q + k;
                    // the partner's half of the complex value at site x0 + 2 s + comp
                    const double recv = __shfl_xor_sync(0xffffffffu, comp ? z[2 * k] : z[2 * k + 1], 1);
                    const double2 zc = comp ? make_double2(recv, z[2 * k + 1]) : make_double2(z[2 * k], recv);
                    const int x = x0 + 2 * s + comp;
                    double2 res;
                    if (MODE == MODE_M) {
                        res = wrap ? make_double2(pre[s].x + zc.x, pre[s].y + zc.y)
                                   : make_double2(pre[s].x - zc.x, pre[s].y - zc.y);  // psi -/+ z
                    } else if (MODE == MODE_OZ_GEMM) {
                        res = zc;
                        if (phase)  // column scale z * ph[x]
                            res = make_double2(fma(ph[s].x, zc.x, -ph[s].y * zc.y), fma(ph[s].x, zc.y, ph[s].y * zc.x));
                    } else {  // psi -/+ conj(ph) z
                        const double2 w = make_double2(fma(ph[s].x, zc.x, ph[s].y * zc.y),
                                                       fma(ph[s].x, zc.y, -ph[s].y * zc.x));
                        res = wrap ? make_double2(pre[s].x + w.x, pre[s].y + w.y)
                                   : make_double2(pre[s].x - w.x, pre[s].y - w.y);
                    }
                    if (row_ok && x < Nx) {
                        if (EPI == 2) {
                            if (act) {  // res = (A p) at this site
                                const double2 rn = make_double2(fma(-alpha, res.x, rq[s].x),
                                                                fma(-alpha, res.y, rq[s].y));
                                epi.r[orow + x] = rn;
                                sq = fma(rn.x, rn.x, fma(rn.y, rn.y, sq));
                            }
                        } else {
                            out[orow + x] = res;
                            if (EPI == 1) sq = fma(res.x, res.x, fma(res.y, res.y, sq));
                            if (MODE == MODE_MDAG && EPI == 1 && epi.u)  // u = ph o out
                                epi.u[orow + x] = make_double2(fma(ph[s].x, res.x, -ph[s].y * res.y),
                                                               fma(ph[s].x, res.y, ph[s].y * res.x));
                        }
                    }
                }
            }
            // the accumulator set is read: release it to the MMA issuer
            tc::tc_fence_before();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&bar_tempty[buf]);
            // partial |.|^2 over this lane's complex values (the two lanes of a row take one slot each)
            if (EPI != 0 && row_ok) epi.part[(grow * 2 + comp) * (2 * ntn) + 2 * nt + g] = sq;
            ++tc_n;
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc::tc_fence_after();
        tc::tmem_dealloc(tmem, OZP_TMEM_COLS);
    }
}

// Digit planes of the real part of exp(d K): plane l holds digit l of every row x (scale 2^{e_x} per row), rows of
// ld BF16 (zero padded), the planes stacked along the row axis (S * Nx rows) for one 2-D tensor map. One block of
// 256 threads per row x; it also evaluates the row's digit-sum bounds (256 sum_{l<=d} B_l(x), B_l(x) = sum_y |b_l|)
// and sets col_exp[Nx] (zeroed before the launch) when an order d < OZ_EXACT reaches 2^24 or any order 2^30.
__global__ void __launch_bounds__(256) k_oz_planes(const double2 *__restrict__ E, __nv_bfloat16 *planes, int *col_exp,
                                                   int Nx, int ld) {
    const int x = blockIdx.x;
    unsigned long long m = 0ull;
    for (int y = threadIdx.x; y < Nx; y += blockDim.x) m = max(m, abs_bits(E[(int64_t)x * Nx + y].x));
    __shared__ unsigned long long red[256];
    __shared__ int sums[OZ_S][8];
    red[threadIdx.x] = m;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] = max(red[threadIdx.x], red[threadIdx.x + w]);
        __syncthreads();
    }
    const int e = scale_exponent(red[0]);
    if (threadIdx.x == 0) col_exp[x] = e;
    int B[OZ_S];
#pragma unroll
    for (int l = 0; l < OZ_S; ++l) B[l] = 0;
    for (int y = threadIdx.x; y < ld; y += blockDim.x) {
        const double v = (y < Nx) ? E[(int64_t)x * Nx + y].x : 0.0;
        float a[OZ_S];
        balanced_digits(scaled_int((unsigned long long)__double_as_longlong(v), e), a);
#pragma unroll
        for (int l = 0; l < OZ_S; ++l) {
            planes[((int64_t)l * Nx + x) * ld + y] = __float2bfloat16_rn(a[l]);
            B[l] += (int)fabsf(a[l]);
        }
    }
    const int lane = threadIdx.x % 32, warp = threadIdx.x / 32;
#pragma unroll
    for (int l = 0; l < OZ_S; ++l) {
        int s = B[l];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) sums[l][warp] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long acc = 0;
        bool bad = false;
        for (int d = 0; d < OZ_S; ++d) {
            for (int w = 0; w < 8; ++w) acc += sums[d][w];
            const long long bound = acc << (OZ_W - 1);  // max |a_k| = 2^{W-1}
            bad |= bound >= (1ll << (d < OZ_EXACT ? 24 : 30));
        }
        if (bad) atomicExch(&col_exp[Nx], 1);
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

int set_smem_attr() {
    NSLG_CUDA(cudaFuncSetAttribute(k_fm_apply_oz<MODE_M, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, OZP_SMEM));
    NSLG_CUDA(cudaFuncSetAttribute(k_fm_apply_oz<MODE_M, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, OZP_SMEM));
    NSLG_CUDA(cudaFuncSetAttribute(k_fm_apply_oz<MODE_M, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, OZP_SMEM));
    NSLG_CUDA(cudaFuncSetAttribute(k_fm_apply_oz<MODE_MDAG, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   OZP_SMEM));
    NSLG_CUDA(cudaFuncSetAttribute(k_fm_apply_oz<MODE_MDAG, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   OZP_SMEM));
    NSLG_CUDA(cudaFuncSetAttribute(k_fm_apply_oz<MODE_MDAG, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   OZP_SMEM));
    NSLG_CUDA(cudaFuncSetAttribute(k_fm_apply_oz<MODE_OZ_GEMM, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   OZP_SMEM));
    return NSLG_OK;
}

// Persistent grid: one CTA per SM of the current device, at most one per tile.
unsigned oz_grid(int64_t rows, int Nx) {
    static std::atomic<int> sms[64] = {};  // SM count per device ordinal (0: not looked up yet)
    int dev = 0;
    cudaGetDevice(&dev);
    int n = (dev >= 0 && dev < 64) ? sms[dev].load() : 0;
    if (n == 0) {
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
            cudaGetLastError();
            n = 1;
        }
        if (dev >= 0 && dev < 64) sms[dev].store(n);
    }
    const int64_t tiles = ceil_div(rows, OZ_BM / 2) * ceil_div(Nx, OZ_BN);
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(tiles, n));
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
        // col_exp[Nx] is the digit-sum bound flag
        if (cudaMalloc(&P->planes, n * sizeof(__nv_bfloat16)) != cudaSuccess ||
            cudaMalloc(&P->col_exp, (Nx + 1) * sizeof(int)) != cudaSuccess) {
            cudaGetLastError();
            cudaFree(P->planes);
            delete P;
            set_error("split-BF16 planes: device allocation failed");
            return NSLG_ERR_OOM;
        }
        NSLG_CUDA(cudaMemsetAsync(P->col_exp + Nx, 0, sizeof(int), fm->ctx->stream));
        k_oz_planes<<<Nx, 256, 0, fm->ctx->stream>>>(E->full, static_cast<__nv_bfloat16 *>(P->planes), P->col_exp,
                                                      Nx, P->ld);
        note_launch(fm->ctx->stream);
        NSLG_CUDA(cudaGetLastError());
        NSLG_TRY(make_map_bf16(&P->map, P->planes, (int64_t)OZ_S * Nx, P->ld, OZ_BN));
        NSLG_TRY(set_smem_attr());
        E->oz = P;
    }
    *out = E->oz;
    return NSLG_OK;
}

// digits: workspace of S * 2 * rows * ld BF16; rexp: 2 * rows ints.
namespace {

template <int EPI>
void launch_oz(int mode, dim3 grid, cudaStream_t st, const double2 *psi, double2 *out, const double2 *phase,
               const int *rexp, const int *col_exp, const CUtensorMap &map_a, const CUtensorMap &map_b, int Nt, int Nx,
               int64_t rows, int nkb, int *err, const OzEpi &epi) {
    if (mode == MODE_M)
        k_fm_apply_oz<MODE_M, EPI><<<grid, OZP_THREADS, OZP_SMEM, st>>>(psi, out, phase, rexp, col_exp, map_a, map_b,
                                                                        Nt, Nx, rows, nkb, err, epi);
    else
        k_fm_apply_oz<MODE_MDAG, EPI><<<grid, OZP_THREADS, OZP_SMEM, st>>>(psi, out, phase, rexp, col_exp, map_a,
                                                                           map_b, Nt, Nx, rows, nkb, err, epi);
}

}  // namespace

// partial sums per GEMM row of the CG epilogues: one per 16-site half of every 32-site tile
int oz_ntiles(int Nx) { return 2 * (int)ceil_div(Nx, OZ_BN); }

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
    k_fm_apply_oz<MODE_OZ_GEMM, 0><<<oz_grid(rows, Nx), OZP_THREADS, OZP_SMEM, st>>>(
        nullptr, out, epi_scale, rexp, P.col_exp, map_a, P.map, 1, Nx, rows, nkb, err, plain);
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
    if (!E.digits_ready) {
        if (mode == MODE_M && !E.operand)
            k_oz_digits<MODE_M><<<blocks, 256, 0, st>>>(psi, phase, Nt, Nx, rows, P.ld, dg, rexp, E.go, E.sys_rows);
        else  // M^dagger's operand is psi itself; a given operand is used as it is
            k_oz_digits<MODE_MDAG><<<blocks, 256, 0, st>>>(E.operand ? E.operand : psi, nullptr, Nt, Nx, rows, P.ld,
                                                           dg, rexp, E.go, E.sys_rows);
        note_launch(st);
        NSLG_CUDA(cudaGetLastError());
    }
    CUtensorMap map_a;
    NSLG_TRY(make_map_bf16(&map_a, digits, (int64_t)OZ_S * 2 * rows, P.ld, OZ_BM));
    const int nkb = P.ld / OZ_BK;
    const dim3 grid(oz_grid(rows, Nx));
    if (E.mode == 1)
        launch_oz<1>(mode, grid, st, psi, out, phase, rexp, P.col_exp, map_a, P.map, Nt, Nx, rows, nkb, err, E);
    else if (E.mode == 2)
        launch_oz<2>(mode, grid, st, psi, out, phase, rexp, P.col_exp, map_a, P.map, Nt, Nx, rows, nkb, err, E);
    else
        launch_oz<0>(mode, grid, st, psi, out, phase, rexp, P.col_exp, map_a, P.map, Nt, Nx, rows, nkb, err, E);
    note_launch(st);
    NSLG_CUDA(cudaGetLastError());
    return NSLG_OK;
}

}  // namespace nslg
