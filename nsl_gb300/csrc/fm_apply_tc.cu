// Fermion-matrix applications M psi / M^dagger psi on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// Same contraction and fusion as the CUDA-core kernel (fm_apply.cu): Z[(r,t), x] = sum_y Y[(r,t), y] E[x, y] with
// the phase in the operand load and the time shift, boundary sign, conj(phase) and "psi -" in the epilogue. Here the
// product runs as three TF32 tensor-core MMAs with FP32 accumulation in TMEM (split precision, "3xTF32"):
//   Y E^T ~= Y_hi E_hi^T + Y_hi E_lo^T + Y_lo E_hi^T,
// where v_hi is v rounded to FP32 with the low 13 mantissa bits cleared (exactly a TF32 value) and v_lo = v - v_hi.
// That keeps ~21 bits of every operand and is as accurate as an FP32 CUDA-core product, at tensor-core rate.
//
// GEMM view: the real and imaginary parts of each complex row (r, t) are two real GEMM rows (M = 2 R Nt), the
// reduction runs over the input site y (K = Nx) and the columns are the output site x (N = Nx). exp(delta K) is real
// for real delta and hopping (the case this kernel serves); its TF32 hi/lo planes are built once per memo entry and
// streamed by TMA (128-byte swizzle, no multicast). The operand rows come from FP64 psi: the CTA's threads load them
// with coalesced reads, multiply by the phase (M), split hi/lo and store them in the same swizzled layout.
//
// CTA tile: 128 real rows (64 complex rows) x BN sites, 256 threads, K in 32-site blocks through a 2-stage ring:
// the threads build stage s+1 while the tensor core works on stage s. One thread issues the MMAs and commits them to
// an mbarrier per stage. The accumulator (128 lanes x BN FP32 columns) is read back with tcgen05.ld by all 8 warps.

#include <cudaTypedefs.h>

#include "fm_internal.cuh"
#include "tc_common.cuh"

namespace nslg {

namespace {

constexpr int TC_THREADS = 256;
constexpr int TC_BM = 128;  // real rows per CTA
constexpr int TC_BK = 32;   // sites per k-block (128 bytes of FP32)
constexpr int TC_A_BYTES = TC_BM * TC_BK * 4;

template <int BN> struct TcSmem {
    static constexpr int B_BYTES = BN * TC_BK * 4;
    static constexpr int STAGE = 2 * TC_A_BYTES + 2 * B_BYTES;  // A_hi, A_lo, B_hi, B_lo
    static constexpr int TOTAL = 2 * STAGE + 1024 /*alignment*/ + 128 /*barriers*/;
};

template <int BN> __host__ __device__ constexpr uint32_t tmem_cols() { return BN <= 32 ? 32 : BN <= 64 ? 64 : BN <= 128 ? 128 : 256; }

template <int MODE, int BN>
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_fm_apply_tc(const double2 *__restrict__ psi, double2 *__restrict__ out, const double2 *__restrict__ phase,
                  const __grid_constant__ CUtensorMap map_hi, const __grid_constant__ CUtensorMap map_lo, int Nt,
                  int Nx, int64_t rows, int nkb, int *err) {
    using S = TcSmem<BN>;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *bar_load = reinterpret_cast<uint64_t *>(smem + 2 * S::STAGE);
    uint64_t *bar_mma = bar_load + 2;
    uint64_t *bar_done = bar_load + 4;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bar_load + 5);
    int *abort_flag = reinterpret_cast<int *>(bar_load + 6);

    const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
    const int64_t grow0 = (int64_t)blockIdx.x * (TC_BM / 2);
    const int n0 = blockIdx.y * BN;

    if (tid == 0) {
        for (int i = 0; i < 2; ++i) {
            tc::mbar_init(&bar_load[i], 1);
            tc::mbar_init(&bar_mma[i], 1);
        }
        tc::mbar_init(bar_done, 1);
        *abort_flag = 0;
        tc::fence_mbar_init();
        tc::prefetch_tmap(&map_hi);
        tc::prefetch_tmap(&map_lo);
    }
    if (warp == 0) tc::tmem_alloc(tmem_slot, tmem_cols<BN>());
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    constexpr uint32_t idesc = tc::idesc_tf32(TC_BM, BN);

    for (int kb = 0; kb < nkb; ++kb) {
        const int s = kb & 1;
        uint8_t *a_hi = smem + s * S::STAGE;
        uint8_t *a_lo = a_hi + TC_A_BYTES;
        uint8_t *b_hi = a_lo + TC_A_BYTES;
        uint8_t *b_lo = b_hi + S::B_BYTES;
        if (kb >= 2) {  // the MMAs of k-block kb-2 have finished reading this stage
            if (!tc::mbar_wait(&bar_mma[s], ((kb - 2) >> 1) & 1, err, 1)) *abort_flag = 1;
        }
        __syncthreads();
        if (*abort_flag) break;
        if (tid == 0) {
            tc::mbar_arrive_expect_tx(&bar_load[s], 2 * S::B_BYTES);
            tc::tma_load_2d(b_hi, &map_hi, kb * TC_BK, n0, &bar_load[s]);
            tc::tma_load_2d(b_lo, &map_lo, kb * TC_BK, n0, &bar_load[s]);
        }
        // operand rows: 64 complex rows x 32 sites; a warp reads one 512-byte row segment per step
        const int k = lane;
        const int y = kb * TC_BK + k;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int j = warp + 8 * i;  // complex row within the tile
            const int64_t grow = grow0 + j;
            double2 v = make_double2(0.0, 0.0);
            if (grow < rows && y < Nx) {
                v = psi[grow * Nx + y];
                if (MODE == MODE_M) v = cmul(phase[(int64_t)(grow % Nt) * Nx + y], v);
            }
            float hr, lr, hi_, li;
            tc::split_tf32(v.x, hr, lr);
            tc::split_tf32(v.y, hi_, li);
            const uint32_t o_re = tc::sw128_offset(2 * j, k), o_im = tc::sw128_offset(2 * j + 1, k);
            *reinterpret_cast<float *>(a_hi + o_re) = hr;
            *reinterpret_cast<float *>(a_lo + o_re) = lr;
            *reinterpret_cast<float *>(a_hi + o_im) = hi_;
            *reinterpret_cast<float *>(a_lo + o_im) = li;
        }
        tc::fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            if (tc::mbar_wait(&bar_load[s], (kb >> 1) & 1, err, 2)) {
                tc::tc_fence_after();
                const uint32_t ah = tc::smem_addr(a_hi), al = tc::smem_addr(a_lo);
                const uint32_t bh = tc::smem_addr(b_hi), bl = tc::smem_addr(b_lo);
#pragma unroll
                for (int kk = 0; kk < TC_BK / 8; ++kk) {  // K = 8 per TF32 MMA: 32 bytes along the swizzled row
                    const uint32_t off = kk * 32;
                    const uint64_t dah = tc::sdesc_kmajor_sw128(ah + off), dal = tc::sdesc_kmajor_sw128(al + off);
                    const uint64_t dbh = tc::sdesc_kmajor_sw128(bh + off), dbl = tc::sdesc_kmajor_sw128(bl + off);
                    tc::mma_tf32(tmem, dah, dbh, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
                    tc::mma_tf32(tmem, dah, dbl, idesc, 1u);
                    tc::mma_tf32(tmem, dal, dbh, idesc, 1u);
                }
                tc::mma_commit(&bar_mma[s]);
            } else {
                *abort_flag = 1;
            }
        }
    }
    __syncthreads();
    const bool ok = (*abort_flag == 0);
    if (ok && tid == 0) tc::mma_commit(bar_done);
    if (!(ok && tc::mbar_wait(bar_done, 0, err, 3))) *abort_flag = 1;
    __syncthreads();
    const bool ready = (*abort_flag == 0);  // block-uniform: tcgen05.ld below is warp-collective
    tc::tc_fence_after();

    // epilogue: warps w and w+4 share TMEM lanes 32(w%4).. and split the BN columns
    const int m = 32 * (warp & 3) + lane;  // real row of the tile = TMEM lane
    const int j = m >> 1, comp = m & 1;
    const int64_t grow = grow0 + j;
    const int64_t r = grow / Nt;
    const int t = (int)(grow - r * Nt);
    int to;
    double sgn;
    if (MODE == MODE_M) {
        to = (t + 1 == Nt) ? 0 : t + 1;
        sgn = (to == 0) ? -1.0 : 1.0;
    } else {
        to = (t == 0) ? Nt - 1 : t - 1;
        sgn = (t == 0) ? -1.0 : 1.0;
    }
    const int64_t orow = (r * Nt + to) * Nx;
    const double *psid = reinterpret_cast<const double *>(psi);
    double *outd = reinterpret_cast<double *>(out);
    const uint32_t lane_addr = tmem + ((uint32_t)(32 * (warp & 3)) << 16);
    constexpr int HALF = BN / 2;
#pragma unroll 1
    for (int q = 0; q < HALF / 16; ++q) {
        const int c0 = (warp >> 2) * HALF + 16 * q;
        float v[16];
        if (ready) tc::tmem_ld16(lane_addr + c0, v);
        else
#pragma unroll
            for (int i = 0; i < 16; ++i) v[i] = 0.f;
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const float partner = __shfl_xor_sync(0xffffffffu, v[i], 1);
            const int x = n0 + c0 + i;
            if (!ready || grow >= rows || x >= Nx) continue;
            double z = (double)v[i];
            if (MODE == MODE_MDAG) {
                const double zr = comp ? (double)partner : z, zi = comp ? z : (double)partner;
                const double2 ph = phase[(int64_t)to * Nx + x];
                // conj(ph) * (zr + i zi)
                z = comp ? (ph.x * zi - ph.y * zr) : (ph.x * zr + ph.y * zi);
            }
            const int64_t e = (orow + x) * 2 + comp;
            outd[e] = psid[e] - sgn * z;
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, tmem_cols<BN>());
}

// TF32 hi/lo planes of the real part of exp(d K), rows padded to ld (zeros), for the B operand.
__global__ void k_tf32_planes(const double2 *__restrict__ E, float *hi, float *lo, int Nx, int ld) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)Nx * ld) return;
    const int row = (int)(i / ld), col = (int)(i % ld);
    float h = 0.f, l = 0.f;
    if (col < Nx) {
        const double v = E[(int64_t)row * Nx + col].x;
        const float f = (float)v;
        h = __uint_as_float(__float_as_uint(f) & 0xFFFFE000u);
        l = (float)(v - (double)h);
    }
    hi[i] = h;
    lo[i] = l;
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

int make_map(CUtensorMap *map, float *base, int Nx, int ld, int BN) {
    auto fn = encode_fn();
    NSLG_REQUIRE(fn != nullptr, NSLG_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    const cuuint64_t dims[2] = {(cuuint64_t)ld, (cuuint64_t)Nx};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * 4};
    const cuuint32_t box[2] = {(cuuint32_t)TC_BK, (cuuint32_t)BN};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    NSLG_REQUIRE(r == CUDA_SUCCESS, NSLG_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return NSLG_OK;
}

template <int MODE, int BN>
int launch_tc(const double2 *psi, double2 *out, const double2 *phase, const TcPlanes &P, int Nt, int Nx,
              int64_t rows, int *err, cudaStream_t st) {
    constexpr int smem = TcSmem<BN>::TOTAL;
    static bool attr_set = false;
    if (!attr_set) {
        NSLG_CUDA(cudaFuncSetAttribute(k_fm_apply_tc<MODE, BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        attr_set = true;
    }
    dim3 grid((unsigned)ceil_div(rows, TC_BM / 2), (unsigned)ceil_div(Nx, BN));
    k_fm_apply_tc<MODE, BN><<<grid, TC_THREADS, smem, st>>>(psi, out, phase, P.map_hi, P.map_lo, Nt, Nx, rows,
                                                            P.ld / TC_BK, err);
    note_launch(st);
    NSLG_CUDA(cudaGetLastError());
    return NSLG_OK;
}

}  // namespace

int tc_choose_bn(int Nx) {
    if (Nx <= 32) return 32;
    if (Nx <= 64) return 64;
    if (Nx <= 96 || Nx == 288) return 96;
    if (Nx <= 128) return 128;
    return 192;
}

int tc_planes(nslg_fm *fm, const ExpEntry *e, TcPlanes **out) {
    auto *E = const_cast<ExpEntry *>(e);
    if (!E->tc) {
        NSLG_REQUIRE(E->is_real, NSLG_ERR_UNSUPPORTED, "tensor-core operator needs a real exp(delta K)");
        auto *P = new TcPlanes;
        const int Nx = (int)fm->Nx;
        P->ld = (int)ceil_div(Nx, TC_BK) * TC_BK;
        P->bn = tc_choose_bn(Nx);
        const int64_t n = (int64_t)Nx * P->ld;
        if (cudaMalloc(&P->hi, n * sizeof(float)) != cudaSuccess || cudaMalloc(&P->lo, n * sizeof(float)) != cudaSuccess) {
            cudaGetLastError();
            cudaFree(P->hi);
            delete P;
            set_error("tensor-core planes: device allocation failed");
            return NSLG_ERR_OOM;
        }
        k_tf32_planes<<<(unsigned)ceil_div(n, 256), 256, 0, fm->ctx->stream>>>(E->full, P->hi, P->lo, Nx, P->ld);
        note_launch(fm->ctx->stream);
        NSLG_CUDA(cudaGetLastError());
        NSLG_TRY(make_map(&P->map_hi, P->hi, Nx, P->ld, P->bn));
        NSLG_TRY(make_map(&P->map_lo, P->lo, Nx, P->ld, P->bn));
        E->tc = P;
    }
    *out = E->tc;
    return NSLG_OK;
}

int fm_apply_tc(int mode, const double2 *psi, double2 *out, const double2 *phase, const TcPlanes &P, int Nt, int Nx,
                int64_t rows, int *err, cudaStream_t st) {
    if (rows == 0) return NSLG_OK;
#define NSLG_TC_CASE(BNV)                                                                                       \
    case BNV:                                                                                                   \
        return mode == MODE_M ? launch_tc<MODE_M, BNV>(psi, out, phase, P, Nt, Nx, rows, err, st)             \
                              : launch_tc<MODE_MDAG, BNV>(psi, out, phase, P, Nt, Nx, rows, err, st);
    switch (P.bn) {
        NSLG_TC_CASE(32)
        NSLG_TC_CASE(64)
        NSLG_TC_CASE(96)
        NSLG_TC_CASE(128)
        NSLG_TC_CASE(192)
        default: break;
    }
#undef NSLG_TC_CASE
    set_error("tensor-core operator: unsupported tile width");
    return NSLG_ERR_UNSUPPORTED;
}

}  // namespace nslg
