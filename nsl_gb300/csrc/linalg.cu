// Dense FP64 complex linear algebra used off the per-iteration path: a batched complex GEMM, the matrix exponential
// exp(d K) of the hopping matrix (SpatialLattice::exp_hopping_matrix, lattice.tpp:52-58) and the phase factors of
// HubbardExp::populate (hubbardExp.hpp:116-128).

#include <cstdlib>
#include <map>
#include <mutex>
#include <tuple>

#include "fm_internal.cuh"

namespace nslg {

namespace {

constexpr int GK = 8;  // reduction depth per stage

// C = alpha * A @ B (+ I) (+ C with accumulate), batched over blockIdx.z. A CTA owns a TB x TB tile of C; (TB/TI)^2 threads each own a
// TI x TI block (rows ty + (TB/TI) i, cols tx + (TB/TI) j). GB300 runs FP64 at ~2 FMAs per clock per SM, so what
// matters is that every SM gets work: large or batched products use 64-wide tiles, a single product of a few hundred
// rows uses 16-wide tiles (324 CTAs for Nx = 288 instead of 25).
// REAL: bit 0 = A holds real numbers (imaginary parts zero), bit 1 = B does; the product then skips the FMAs with
// the zero imaginary parts (2 instead of 4 per term), which is what bounds these FP64 products.
template <int TB, int TI, int REAL = 0>
__global__ void __launch_bounds__((TB / TI) * (TB / TI))
    k_zgemm(int M, int N, int K, double2 alpha, const double2 *__restrict__ A, int64_t lda, int64_t sA,
            const double2 *__restrict__ B, int64_t ldb, int64_t sB, double2 *__restrict__ C, int64_t ldc, int64_t sC,
            bool add_identity, bool accumulate, int batch2, int64_t sA2, int64_t sB2, int64_t sC2) {
    constexpr int TD = TB / TI;  // threads per tile edge
    constexpr int NT = TD * TD;
    static_assert((TB * GK) % NT == 0, "tile loads");
    __shared__ double2 As[GK][TB + 1];
    __shared__ double2 Bs[GK][TB + 1];
    const int tid = threadIdx.x, tx = tid % TD, ty = tid / TD;
    const int m0 = blockIdx.x * TB, n0 = blockIdx.y * TB;
    // two-level batch: z = z1 * batch2 + z2
    const int z1 = blockIdx.z / batch2, z2 = blockIdx.z % batch2;
    A += sA * z1 + sA2 * z2;
    B += sB * z1 + sB2 * z2;
    C += sC * z1 + sC2 * z2;

    double2 acc[TI][TI];
#pragma unroll
    for (int i = 0; i < TI; ++i)
#pragma unroll
        for (int j = 0; j < TI; ++j) acc[i][j] = make_double2(0, 0);

    for (int k0 = 0; k0 < K; k0 += GK) {
#pragma unroll
        for (int l = 0; l < TB * GK / NT; ++l) {
            const int idx = tid + NT * l;
            // A tile TB x GK: thread -> (row = idx / GK, k = idx % GK)
            const int ar = idx / GK, ak = idx % GK;
            const int gr = m0 + ar, gk = k0 + ak;
            As[ak][ar] = (gr < M && gk < K) ? A[(int64_t)gr * lda + gk] : make_double2(0, 0);
            // B tile GK x TB: thread -> (k = idx / TB, col = idx % TB)
            const int bk = idx / TB, bc = idx % TB;
            const int gk2 = k0 + bk, gc = n0 + bc;
            Bs[bk][bc] = (gk2 < K && gc < N) ? B[(int64_t)gk2 * ldb + gc] : make_double2(0, 0);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GK; ++kk) {
            double2 a[TI], b[TI];
#pragma unroll
            for (int i = 0; i < TI; ++i) a[i] = As[kk][ty + TD * i];
#pragma unroll
            for (int j = 0; j < TI; ++j) b[j] = Bs[kk][tx + TD * j];
#pragma unroll
            for (int i = 0; i < TI; ++i)
#pragma unroll
                for (int j = 0; j < TI; ++j) {
                    if constexpr (REAL == 2) {  // B real
                        acc[i][j].x = fma(a[i].x, b[j].x, acc[i][j].x);
                        acc[i][j].y = fma(a[i].y, b[j].x, acc[i][j].y);
                    } else if constexpr (REAL == 1) {  // A real
                        acc[i][j].x = fma(a[i].x, b[j].x, acc[i][j].x);
                        acc[i][j].y = fma(a[i].x, b[j].y, acc[i][j].y);
                    } else {
                        acc[i][j].x = fma(a[i].x, b[j].x, acc[i][j].x);
                        acc[i][j].x = fma(-a[i].y, b[j].y, acc[i][j].x);
                        acc[i][j].y = fma(a[i].x, b[j].y, acc[i][j].y);
                        acc[i][j].y = fma(a[i].y, b[j].x, acc[i][j].y);
                    }
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < TI; ++i) {
        const int r = m0 + ty + TD * i;
        if (r >= M) continue;
#pragma unroll
        for (int j = 0; j < TI; ++j) {
            const int c = n0 + tx + TD * j;
            if (c >= N) continue;
            double2 v = cmul(alpha, acc[i][j]);
            if (add_identity && r == c) v.x += 1.0;
            if (accumulate) {
                const double2 o = C[(int64_t)r * ldc + c];
                v.x += o.x;
                v.y += o.y;
            }
            C[(int64_t)r * ldc + c] = v;
        }
    }
}

// Small products (M, N, K <= 32): one CTA per 16x16 output tile and product, the whole K range loaded once, and the
// K sum split over ZS_KG warp pairs whose partial sums are added in shared memory. FP64 arithmetic is slow per SM
// partition on this part, so for these latency-bound products short dependent chains and more warps per product
// matter more than operand reuse.
constexpr int ZS_TB = 16, ZS_KG = 4, ZS_K = 32;

__global__ void __launch_bounds__(64 * ZS_KG)
    k_zgemm_small(int M, int N, int K, double2 alpha, const double2 *__restrict__ A, int64_t lda, int64_t sA,
                  const double2 *__restrict__ B, int64_t ldb, int64_t sB, double2 *__restrict__ C, int64_t ldc,
                  int64_t sC, bool add_identity, bool accumulate, int batch2, int64_t sA2, int64_t sB2,
                  int64_t sC2) {
    __shared__ double2 As[ZS_K][ZS_TB + 1];
    __shared__ double2 Bs[ZS_K][ZS_TB + 1];
    __shared__ double2 red[ZS_KG][ZS_TB * ZS_TB];
    const int z1 = blockIdx.z / batch2, z2 = blockIdx.z % batch2;
    A += sA * z1 + sA2 * z2;
    B += sB * z1 + sB2 * z2;
    C += sC * z1 + sC2 * z2;
    const int m0 = blockIdx.x * ZS_TB, n0 = blockIdx.y * ZS_TB;
    const int tid = threadIdx.x;
    for (int e = tid; e < ZS_K * ZS_TB; e += 64 * ZS_KG) {
        const int k = e / ZS_TB, i = e % ZS_TB;
        As[k][i] = (m0 + i < M && k < K) ? A[(int64_t)(m0 + i) * lda + k] : make_double2(0, 0);
        Bs[k][i] = (k < K && n0 + i < N) ? B[(int64_t)k * ldb + n0 + i] : make_double2(0, 0);
    }
    __syncthreads();
    const int g = tid / 64, t = tid % 64, tx = t % 8, ty = t / 8;
    double2 acc[2][2];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) acc[i][j] = make_double2(0, 0);
    for (int k = g; k < K; k += ZS_KG) {
        const double2 a0 = As[k][ty], a1 = As[k][ty + 8], b0 = Bs[k][tx], b1 = Bs[k][tx + 8];
        const double2 a[2] = {a0, a1}, b[2] = {b0, b1};
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                acc[i][j].x = fma(a[i].x, b[j].x, acc[i][j].x);
                acc[i][j].x = fma(-a[i].y, b[j].y, acc[i][j].x);
                acc[i][j].y = fma(a[i].x, b[j].y, acc[i][j].y);
                acc[i][j].y = fma(a[i].y, b[j].x, acc[i][j].y);
            }
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) red[g][(ty + 8 * i) * ZS_TB + tx + 8 * j] = acc[i][j];
    __syncthreads();
    for (int e = tid; e < ZS_TB * ZS_TB; e += 64 * ZS_KG) {
        const int r = m0 + e / ZS_TB, c = n0 + e % ZS_TB;
        if (r >= M || c >= N) continue;
        double2 v = red[0][e];
#pragma unroll
        for (int q = 1; q < ZS_KG; ++q) {
            v.x += red[q][e].x;
            v.y += red[q][e].y;
        }
        v = cmul(alpha, v);
        if (add_identity && r == c) v.x += 1.0;
        if (accumulate) {
            const double2 o = C[(int64_t)r * ldc + c];
            v.x += o.x;
            v.y += o.y;
        }
        C[(int64_t)r * ldc + c] = v;
    }
}

__global__ void k_set_identity(double2 *A, int n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)n * n) return;
    const int r = (int)(i / n), c = (int)(i % n);
    A[i] = make_double2(r == c ? 1.0 : 0.0, 0.0);
}

__global__ void k_scale(double2 *out, const double2 *in, double2 s, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = cmul(s, in[i]);
}

// Planes of exp(d K): re/im FP64 and FP32, plus a flag set when any imaginary part is nonzero.
__global__ void k_split_planes(const double2 *E, double *re, double *im, float *re32, float *im32, int64_t n,
                               int *nonreal) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double2 v = E[i];
    re[i] = v.x;
    im[i] = v.y;
    re32[i] = (float)v.x;
    im32[i] = (float)v.y;
    if (v.y != 0.0) atomicOr(nonreal, 1);
}

// 1-norm (max column sum of |K|) of a complex (n, n) matrix, one block.
__global__ void k_norm1(const double2 *A, int n, double *out) {
    __shared__ double red[256];
    double best = 0;
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
        double s = 0;
        for (int r = 0; r < n; ++r) {
            const double2 v = A[(int64_t)r * n + c];
            s += hypot(v.x, v.y);
        }
        best = fmax(best, s);
    }
    red[threadIdx.x] = best;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = red[0];
        double2 tr = make_double2(0, 0);
        for (int i = 0; i < n; ++i) {
            tr.x += A[(int64_t)i * n + i].x;
            tr.y += A[(int64_t)i * n + i].y;
        }
        out[1] = tr.x;
        out[2] = tr.y;
    }
}

// phase = exp(i sgn phi + sgn mu), phase_inv = exp(-i sgn phi - sgn mu)  (hubbardExp.hpp:121-127)
__global__ void k_phases(const double2 *phi, double2 *phase, double2 *phase_inv, float2 *phase32, int sgn,
                         double2 mu, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double2 f = phi[i];
    // i*sgn*phi + sgn*mu = (-sgn*f.y + sgn*mu.x) + i (sgn*f.x + sgn*mu.y)
    const double a = sgn * (mu.x - f.y);
    const double b = sgn * (f.x + mu.y);
    double sb, cb;
    sincos(b, &sb, &cb);
    const double ea = exp(a), eia = exp(-a);
    phase[i] = make_double2(ea * cb, ea * sb);
    phase_inv[i] = make_double2(eia * cb, -eia * sb);
    phase32[i] = make_float2((float)(ea * cb), (float)(ea * sb));
}

}  // namespace

namespace {

void launch_zgemm(int tile, cudaStream_t st, int M, int N, int K, double2 alpha, const double2 *A, int64_t lda,
                  int64_t sA, const double2 *B, int64_t ldb, int64_t sB, double2 *C, int64_t ldc, int64_t sC,
                  int batch, bool add_identity, bool accumulate, int batch2 = 1, int64_t sA2 = 0, int64_t sB2 = 0,
                  int64_t sC2 = 0, int real = 0) {
    const unsigned z = (unsigned)batch * (unsigned)batch2;
    if (real && !(M <= ZS_K && N <= ZS_K && K <= ZS_K)) {  // a real operand: the 2-FMA products
        const bool t64 = tile == 64;
        dim3 grid((unsigned)ceil_div(M, t64 ? 64 : 16), (unsigned)ceil_div(N, t64 ? 64 : 16), z);
        if (t64 && real == 1)
            k_zgemm<64, 4, 1><<<grid, 256, 0, st>>>(M, N, K, alpha, A, lda, sA, B, ldb, sB, C, ldc, sC, add_identity,
                                                     accumulate, batch2, sA2, sB2, sC2);
        else if (t64)
            k_zgemm<64, 4, 2><<<grid, 256, 0, st>>>(M, N, K, alpha, A, lda, sA, B, ldb, sB, C, ldc, sC, add_identity,
                                                     accumulate, batch2, sA2, sB2, sC2);
        else if (real == 1)
            k_zgemm<16, 2, 1><<<grid, 64, 0, st>>>(M, N, K, alpha, A, lda, sA, B, ldb, sB, C, ldc, sC, add_identity,
                                                    accumulate, batch2, sA2, sB2, sC2);
        else
            k_zgemm<16, 2, 2><<<grid, 64, 0, st>>>(M, N, K, alpha, A, lda, sA, B, ldb, sB, C, ldc, sC, add_identity,
                                                    accumulate, batch2, sA2, sB2, sC2);
        note_launch(st);
        return;
    }
    if (M <= ZS_K && N <= ZS_K && K <= ZS_K) {
        dim3 grid((unsigned)ceil_div(M, ZS_TB), (unsigned)ceil_div(N, ZS_TB), z);
        k_zgemm_small<<<grid, 64 * ZS_KG, 0, st>>>(M, N, K, alpha, A, lda, sA, B, ldb, sB, C, ldc, sC, add_identity,
                                                  accumulate, batch2, sA2, sB2, sC2);
    } else if (tile == 64) {
        dim3 grid((unsigned)ceil_div(M, 64), (unsigned)ceil_div(N, 64), z);
        k_zgemm<64, 4><<<grid, 256, 0, st>>>(M, N, K, alpha, A, lda, sA, B, ldb, sB, C, ldc, sC, add_identity,
                                              accumulate, batch2, sA2, sB2, sC2);
    } else {
        dim3 grid((unsigned)ceil_div(M, 16), (unsigned)ceil_div(N, 16), z);
        k_zgemm<16, 2><<<grid, 64, 0, st>>>(M, N, K, alpha, A, lda, sA, B, ldb, sB, C, ldc, sC, add_identity,
                                             accumulate, batch2, sA2, sB2, sC2);
    }
    note_launch(st);
}

// Tile choice per (M, N, K, batch): measured once per process on the first overwriting call that is not being
// captured (both tile variants write the same result: every output element sums over k in the same order), the
// SM-count heuristic otherwise. NSLG_AUTOTUNE=0 keeps the heuristic.
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int, int>, int> g_tile;

}  // namespace

int zgemm(cudaStream_t st, int M, int N, int K, double2 alpha, const double2 *A, int64_t lda, int64_t sA,
          const double2 *B, int64_t ldb, int64_t sB, double2 *C, int64_t ldc, int64_t sC, int batch,
          bool add_identity, bool accumulate) {
    if (M == 0 || N == 0 || batch == 0) return NSLG_OK;
    static int sms = 0;
    static const bool tune = [] {
        const char *e = std::getenv("NSLG_AUTOTUNE");
        return !(e && e[0] == '0');
    }();
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    int tile = (ceil_div(M, 64) * ceil_div(N, 64) * batch >= 2 * sms) ? 64 : 16;
    const auto key = std::make_tuple(M, N, K, batch);
    bool measure = false;
    if (tune) {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        auto it = g_tile.find(key);
        if (it != g_tile.end()) {
            tile = it->second;
        } else if (!accumulate) {
            cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
            if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) cudaGetLastError();
            measure = cs == cudaStreamCaptureStatusNone;
        }
    }
    if (measure) {
        cudaEvent_t ev[3];
        for (auto &e : ev) NSLG_CUDA(cudaEventCreate(&e));
        NSLG_CUDA(cudaEventRecord(ev[0], st));
        launch_zgemm(16, st, M, N, K, alpha, A, lda, sA, B, ldb, sB, C, ldc, sC, batch, add_identity, false);
        NSLG_CUDA(cudaEventRecord(ev[1], st));
        launch_zgemm(64, st, M, N, K, alpha, A, lda, sA, B, ldb, sB, C, ldc, sC, batch, add_identity, false);
        NSLG_CUDA(cudaEventRecord(ev[2], st));
        NSLG_CUDA(cudaEventSynchronize(ev[2]));
        float t16 = 0, t64 = 0;
        cudaEventElapsedTime(&t16, ev[0], ev[1]);
        cudaEventElapsedTime(&t64, ev[1], ev[2]);
        for (auto &e : ev) cudaEventDestroy(e);
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tile[key] = t64 <= t16 ? 64 : 16;
        NSLG_CUDA(cudaGetLastError());
        return NSLG_OK;  // C holds the product (written by both variants)
    }
    launch_zgemm(tile, st, M, N, K, alpha, A, lda, sA, B, ldb, sB, C, ldc, sC, batch, add_identity, accumulate);
    NSLG_CUDA(cudaGetLastError());
    return NSLG_OK;
}

// Two-level batched product: C[z1, z2] = alpha A[z1, z2] B[z1, z2] with element offsets z1 * s + z2 * s2, for
// batch x batch2 products in one launch (16-wide tiles: these are the small products of the scans).
int zgemm2(cudaStream_t st, int M, int N, int K, double2 alpha, const double2 *A, int64_t lda, int64_t sA,
           int64_t sA2, const double2 *B, int64_t ldb, int64_t sB, int64_t sB2, double2 *C, int64_t ldc, int64_t sC,
           int64_t sC2, int batch, int batch2, int real) {
    if (M == 0 || N == 0 || batch == 0 || batch2 == 0) return NSLG_OK;
    NSLG_REQUIRE((int64_t)batch * batch2 <= 65535, NSLG_ERR_SHAPE, "zgemm2: at most 65535 products per launch");
    // 64-wide tiles once they alone fill the GPU twice (the stratified products of large lattices), else 16-wide
    const int tile = ceil_div(M, 64) * ceil_div(N, 64) * (int64_t)batch * batch2 >= 2 * num_sms() ? 64 : 16;
    launch_zgemm(tile, st, M, N, K, alpha, A, lda, sA, B, ldb, sB, C, ldc, sC, batch, false, false, batch2, sA2, sB2,
                 sC2, real);
    NSLG_CUDA(cudaGetLastError());
    return NSLG_OK;
}

int compute_phases(nslg_fm *fm) {
    const int64_t n = fm->Nt * fm->Nx;
    const double2 mu = fm->mu_tilde;
    k_phases<<<(unsigned)ceil_div(n, 256), 256, 0, fm->ctx->stream>>>(fm->phi, fm->phase, fm->phase_inv,
                                                                     fm->phase32, fm->sgn, mu, n);
    note_launch(fm->ctx->stream);
    NSLG_CUDA(cudaGetLastError());
    return NSLG_OK;
}

static int make_entry(nslg_fm *fm, double2 *full, nslg::ExpEntry *e) {
    const int64_t n = fm->Nx * fm->Nx;
    cudaStream_t st = fm->ctx->stream;
    e->full = full;
    NSLG_CUDA(cudaMalloc(&e->re, n * sizeof(double)));
    NSLG_CUDA(cudaMalloc(&e->im, n * sizeof(double)));
    NSLG_CUDA(cudaMalloc(&e->re32, n * sizeof(float)));
    NSLG_CUDA(cudaMalloc(&e->im32, n * sizeof(float)));
    int *flag;
    NSLG_TRY(ws_get(fm, "exp_flag", 1, &flag));
    NSLG_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), st));
    k_split_planes<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(full, e->re, e->im, e->re32, e->im32, n, flag);
    note_launch(st);
    NSLG_CUDA(cudaGetLastError());
    int h = 0;
    NSLG_CUDA(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    NSLG_CUDA(cudaStreamSynchronize(st));
    e->is_real = (h == 0);
    return NSLG_OK;
}

int install_exp(nslg_fm *fm, double2 d, const double2 *E_dev) {
    const auto key = std::make_pair(d.x, d.y);
    const int64_t n = fm->Nx * fm->Nx;
    auto it = fm->memo.find(key);
    if (it != fm->memo.end()) {
        NSLG_CUDA(cudaMemcpyAsync(it->second.full, E_dev, n * sizeof(double2), cudaMemcpyDeviceToDevice,
                                  fm->ctx->stream));
        cudaFree(it->second.re);
        cudaFree(it->second.im);
        cudaFree(it->second.re32);
        cudaFree(it->second.im32);
        return make_entry(fm, it->second.full, &it->second);
    }
    double2 *full;
    NSLG_CUDA(cudaMalloc(&full, n * sizeof(double2)));
    NSLG_CUDA(cudaMemcpyAsync(full, E_dev, n * sizeof(double2), cudaMemcpyDeviceToDevice, fm->ctx->stream));
    ExpEntry e;
    NSLG_TRY(make_entry(fm, full, &e));
    fm->memo[key] = e;
    return NSLG_OK;
}

__global__ void k_lin(const double2 *__restrict__ K, double2 d, int one_minus, double2 *__restrict__ out, int n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)n * n) return;
    double2 v = cmul(d, K[i]);
    if (one_minus) {
        v.x = -v.x;
        v.y = -v.y;
        if (i / n == i % n) v.x += 1.0;
    }
    out[i] = v;
}

int get_lin(nslg_fm *fm, double2 d, int one_minus, const ExpEntry **out) {
    const auto key = std::make_tuple(d.x, d.y, one_minus);
    auto it = fm->lin.find(key);
    if (it == fm->lin.end()) {
        const int n = (int)fm->Nx;
        double2 *full;
        NSLG_CUDA(cudaMalloc(&full, (size_t)n * n * sizeof(double2)));
        k_lin<<<(unsigned)ceil_div((int64_t)n * n, 256), 256, 0, fm->ctx->stream>>>(fm->hops, d, one_minus, full, n);
        note_launch(fm->ctx->stream);
        NSLG_CUDA(cudaGetLastError());
        ExpEntry e;
        NSLG_TRY(make_entry(fm, full, &e));
        it = fm->lin.emplace(key, e).first;
    }
    *out = &it->second;
    return NSLG_OK;
}

int get_factor(nslg_fm *fm, double2 d, const ExpEntry **out) {
    return fm->kind == NSLG_FM_DIAG ? get_lin(fm, d, 0, out) : get_exp(fm, d, out);
}

// exp(d K) by scaling and squaring of the Taylor series: A = d K / 2^s with |A|_1 <= 1/2, T = sum_{k<=14} A^k/k!
// (Horner form, truncation below 3e-17 relative), then T <- T^2 s times.
int get_exp(nslg_fm *fm, double2 d, const ExpEntry **out) {
    const auto key = std::make_pair(d.x, d.y);
    auto it = fm->memo.find(key);
    if (it != fm->memo.end()) {
        *out = &it->second;
        return NSLG_OK;
    }
    const int n = (int)fm->Nx;
    const int64_t nn = (int64_t)n * n;
    cudaStream_t st = fm->ctx->stream;
    const double anorm = hypot(d.x, d.y) * fm->hops_norm1;
    int s = 0;
    while (anorm / std::ldexp(1.0, s) > 0.5) ++s;
    const double scale = std::ldexp(1.0, -s);
    double2 *A, *T0, *T1;
    NSLG_TRY(ws_get(fm, "expm_A", nn, &A));
    NSLG_TRY(ws_get(fm, "expm_T0", nn, &T0));
    NSLG_TRY(ws_get(fm, "expm_T1", nn, &T1));
    k_scale<<<(unsigned)ceil_div(nn, 256), 256, 0, st>>>(A, fm->hops, make_double2(d.x * scale, d.y * scale), nn);
    note_launch(st);
    NSLG_CUDA(cudaGetLastError());
    k_set_identity<<<(unsigned)ceil_div(nn, 256), 256, 0, st>>>(T0, n);
    note_launch(st);
    NSLG_CUDA(cudaGetLastError());
    const int m = 14;
    for (int j = m; j >= 1; --j) {  // T <- I + (A / j) T
        NSLG_TRY(zgemm(st, n, n, n, make_double2(1.0 / j, 0), A, n, 0, T0, n, 0, T1, n, 0, 1, true));
        std::swap(T0, T1);
    }
    for (int k = 0; k < s; ++k) {
        NSLG_TRY(zgemm(st, n, n, n, make_double2(1, 0), T0, n, 0, T0, n, 0, T1, n, 0, 1, false));
        std::swap(T0, T1);
    }
    NSLG_TRY(install_exp(fm, d, T0));
    *out = &fm->memo[key];
    return NSLG_OK;
}

int compute_hops_norm(nslg_fm *fm) {
    double *dn;
    NSLG_TRY(ws_get(fm, "norm1", 3, &dn));
    k_norm1<<<1, 256, 0, fm->ctx->stream>>>(fm->hops, (int)fm->Nx, dn);
    note_launch(fm->ctx->stream);
    NSLG_CUDA(cudaGetLastError());
    double h[3];
    NSLG_CUDA(cudaMemcpyAsync(h, dn, sizeof h, cudaMemcpyDeviceToHost, fm->ctx->stream));
    NSLG_CUDA(cudaStreamSynchronize(fm->ctx->stream));
    fm->hops_norm1 = h[0];
    fm->hops_trace = make_double2(h[1], h[2]);
    return NSLG_OK;
}

}  // namespace nslg
