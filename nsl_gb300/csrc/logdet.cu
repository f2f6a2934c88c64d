// log det M and its gradient d log det M / d phi in FP64 on the device (HubbardExp::logDetM / gradLogDetM,
// hubbardExp.tpp:129-211; HubbardDiag::logDetM / gradLogDetM, hubbardDiag.tpp:169-250, with the time-slice matrix
// 1 - sgn delta K in place of exp(+-sgn delta K), the product taken in increasing t and i sgn sum(phi) added).
//
// logDetM: the time-slice matrices B_t = exp(sgn delta K) diag(phiExp[(t+1) % Nt]) (hubbardExp.tpp:142) are built by
// one kernel, multiplied as a balanced product tree of batched complex GEMMs (log2(Nt) levels instead of Nt
// sequential products; the product is the same B_{Nt-1} ... B_0), then 1 + prod is LU-factorised with partial
// pivoting (right-looking, panels of 32 columns: one panel kernel, the row swaps, a triangular solve for the block
// row of U and one GEMM update of the trailing matrix per panel) and log det = sum log(u_kk) + i pi (#row swaps),
// folded onto the principal branch like log(det(.))
// (src/NSL/LinAlg/det.tpp:15-20). Summing logs instead of forming det() avoids the overflow that makes the
// reference's value NaN at low temperature.
//
// gradLogDetM: Fk(t) = diag(phiExpInv[(t-1) % Nt]) exp(-sgn delta K); suffix products S(t) = Fk(t) ... Fk(Nt-1)
// and prefix products P(t) = (1 + S(0))^{-1} Fk(0) ... Fk(t) (hubbardExp.tpp:165-208) are each evaluated as a
// sequence of Nt-1 batched GEMM steps; the diagonal of S(t+1) P(t) needs only O(Nx^2) per slice (a row-column dot
// per site) instead of the reference's full GEMM per slice.

#include <algorithm>
#include <cmath>
#include <mutex>
#include <set>
#include <string>
#include <vector>

#include "fm_internal.cuh"

namespace nslg {

namespace {

// B[t, i, j] = E[i, j] * ph[(t + shift) mod Nt, j]          (column scaling: E diag(ph))
// or, with rowscale, B[t, i, j] = ph[(t + shift) mod Nt, i] * E[i, j]   (row scaling: diag(ph) E)
// With reverse, slice t is stored at position Nt - 1 - t (the product tree then forms M_0 M_1 ... M_{Nt-1}).
__global__ void k_slices(const double2 *__restrict__ E, const double2 *__restrict__ ph, double2 *__restrict__ B,
                         int Nt, int Nx, int shift, bool rowscale, bool reverse = false) {
    const int64_t nn = (int64_t)Nx * Nx;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nn * Nt) return;
    const int t = (int)(idx / nn);
    const int64_t ij = idx - (int64_t)t * nn;
    const int i = (int)(ij / Nx), j = (int)(ij - (int64_t)i * Nx);
    const int ts = ((t + shift) % Nt + Nt) % Nt;
    const double2 s = ph[(int64_t)ts * Nx + (rowscale ? i : j)];
    B[(reverse ? (int64_t)(Nt - 1 - t) * nn : (int64_t)t * nn) + ij] = cmul(E[ij], s);
}

// Sum of n complex values in a fixed order (one block).
__global__ void k_sum_c128(const double2 *__restrict__ v, int64_t n, double2 *__restrict__ out) {
    __shared__ double2 red[256];
    double2 acc = make_double2(0, 0);
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        acc.x += v[i].x;
        acc.y += v[i].y;
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            red[threadIdx.x].x += red[threadIdx.x + w].x;
            red[threadIdx.x].y += red[threadIdx.x + w].y;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

__global__ void k_add_identity(double2 *A, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) A[(int64_t)i * n + i].x += 1.0;
}

// ---- LU with partial pivoting -------------------------------------------------------------------------------------
// Pivot of column k: p = argmax_{i>=k} |A[i,k]| (first index on ties); the multipliers l_ik = A[i,k] / A[k,k] are
// stored in place, the running log of the pivots and the number of row swaps give log det.
constexpr int LT = 1024;

// ---- blocked LU: panels of NB columns ------------------------------------------------------------------------------
// Right-looking: factor the panel (one block, column by column, pivots as above), apply its row swaps
// to the other columns, solve for the panel's block row of U, update the trailing matrix with one GEMM. Every step
// of the column-at-a-time version becomes one of four launches per panel.
//
// Panel width: FP64 arithmetic is slow per SM on this part (a panel runs on one SM per matrix), so large matrices use
// narrow panels (NB = 8: a quarter of the in-panel work of NB = 32, the rest moves into the trailing GEMM, which
// spreads over the GPU); matrices of at most 64 rows keep NB = 32 (one panel, fewest launches).
inline int panel_width(int n) { return n <= 64 ? 32 : 8; }

__global__ void __launch_bounds__(LT) k_lu_panel(double2 *A, int n, int k0, int nb, int *piv, double2 *pivots,
                                                 int *swaps, int *singular, int64_t mstride, bool pivoting) {
    // matrix blockIdx.x of a batch
    A += blockIdx.x * mstride;
    piv += (int64_t)blockIdx.x * n;
    pivots += (int64_t)blockIdx.x * n;
    swaps += blockIdx.x;
    __shared__ double best[LT];
    __shared__ int bidx[LT];
    for (int k = k0; k < k0 + nb; ++k) {
        double bv = -1.0;
        int bi = n;
        for (int i = k + threadIdx.x; i < (pivoting ? n : k + 1); i += LT) {  // without pivoting: row k only
            const double2 v = A[(int64_t)i * n + k];
            const double m = hypot(v.x, v.y);
            if (m > bv || (m == bv && i < bi)) {
                bv = m;
                bi = i;
            }
        }
        best[threadIdx.x] = bv;
        bidx[threadIdx.x] = bi;
        __syncthreads();
        for (int w = LT / 2; w > 0; w >>= 1) {
            if (threadIdx.x < w) {
                const double o = best[threadIdx.x + w];
                const int oi = bidx[threadIdx.x + w];
                if (o > best[threadIdx.x] || (o == best[threadIdx.x] && oi < bidx[threadIdx.x])) {
                    best[threadIdx.x] = o;
                    bidx[threadIdx.x] = oi;
                }
            }
            __syncthreads();
        }
        const int p = bidx[0];
        if (p != k)  // the panel's columns; the others are swapped by k_lu_laswp
            for (int j = k0 + threadIdx.x; j < k0 + nb; j += LT) {
                const double2 a = A[(int64_t)k * n + j];
                A[(int64_t)k * n + j] = A[(int64_t)p * n + j];
                A[(int64_t)p * n + j] = a;
            }
        __syncthreads();
        const double2 d = A[(int64_t)k * n + k];
        const double dd = d.x * d.x + d.y * d.y;
        const double2 inv = dd == 0.0 ? make_double2(0.0, 0.0) : make_double2(d.x / dd, -d.y / dd);
        for (int i = k + 1 + threadIdx.x; i < n; i += LT) A[(int64_t)i * n + k] = cmul(A[(int64_t)i * n + k], inv);
        if (threadIdx.x == 0) {
            piv[k] = p;
            pivots[k] = d;
            if (p != k) *swaps += 1;
            if (dd == 0.0) *singular = 1;
        }
        __syncthreads();
        // rank-1 update of the rest of the panel: A[i, j] -= l_ik u_kj, i > k, k < j < k0 + nb
        const int w = k0 + nb - k - 1;
        const int64_t cnt = (int64_t)(n - k - 1) * w;
        for (int64_t e = threadIdx.x; e < cnt; e += LT) {
            const int i = k + 1 + (int)(e / w), j = k + 1 + (int)(e % w);
            const double2 l = A[(int64_t)i * n + k], u = A[(int64_t)k * n + j];
            double2 a = A[(int64_t)i * n + j];
            a.x -= l.x * u.x - l.y * u.y;
            a.y -= l.x * u.y + l.y * u.x;
            A[(int64_t)i * n + j] = a;
        }
        __syncthreads();
    }
}

// The same panel factorisation with the panel (rows [k0, n), columns [k0, k0 + nb)) held in shared memory, row
// stride NB + 1 so that a column read spreads over the banks. Used while the panel fits (PANEL_SMEM bytes):
// one load and one store of the panel instead of global traffic and a block-wide reduction tree per column.
constexpr int PANEL_SMEM = 219648;  // dynamic shared memory of the panel kernel: 416 rows at NB = 32, 1525 at NB = 8

__device__ __forceinline__ bool piv_better(double m, int i, double bm, int bi) {
    return m > bm || (m == bm && i < bi);
}

template <int LPT, int NB>
__global__ void __launch_bounds__(LPT) k_lu_panel_smem(double2 *A, int n, int k0, int nb, int *piv, double2 *pivots,
                                                       int *swaps, int *singular, int64_t mstride, bool pivoting) {
    constexpr int PS = NB + 1;
    extern __shared__ double2 Ps[];  // (n - k0) x PS
    // matrix blockIdx.x of a batch (LPT threads: 512 for large panels, 128 for small matrices)
    A += blockIdx.x * mstride;
    piv += (int64_t)blockIdx.x * n;
    pivots += (int64_t)blockIdx.x * n;
    swaps += blockIdx.x;
    __shared__ double wbest[LPT / 32];
    __shared__ int widx[LPT / 32];
    __shared__ int pivot;
    const int rows = n - k0;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int e = threadIdx.x; e < rows * nb; e += LPT) {
        const int i = e / nb, j = e % nb;
        Ps[i * PS + j] = A[(int64_t)(k0 + i) * n + k0 + j];
    }
    __syncthreads();
    int nswap = 0, sing = 0;
    for (int kk = 0; kk < nb; ++kk) {
        // pivot: largest |a_ik|^2 over rows i >= kk, first index on ties
        double bm = -1.0;
        int bi = rows;
        for (int i = kk + threadIdx.x; i < (pivoting ? rows : kk + 1); i += LPT) {  // without pivoting: row kk only
            const double2 v = Ps[i * PS + kk];
            const double m = v.x * v.x + v.y * v.y;
            if (piv_better(m, i, bm, bi)) {
                bm = m;
                bi = i;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double om = __shfl_down_sync(0xffffffffu, bm, o);
            const int oi = __shfl_down_sync(0xffffffffu, bi, o);
            if (piv_better(om, oi, bm, bi)) {
                bm = om;
                bi = oi;
            }
        }
        if (lane == 0) {
            wbest[warp] = bm;
            widx[warp] = bi;
        }
        __syncthreads();
        if (warp == 0) {
            bm = lane < LPT / 32 ? wbest[lane] : -1.0;
            bi = lane < LPT / 32 ? widx[lane] : rows;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const double om = __shfl_down_sync(0xffffffffu, bm, o);
                const int oi = __shfl_down_sync(0xffffffffu, bi, o);
                if (piv_better(om, oi, bm, bi)) {
                    bm = om;
                    bi = oi;
                }
            }
            if (lane == 0) pivot = bi;
        }
        __syncthreads();
        const int p = pivot;
        if (p != kk && threadIdx.x < nb) {
            const double2 a = Ps[kk * PS + threadIdx.x];
            Ps[kk * PS + threadIdx.x] = Ps[p * PS + threadIdx.x];
            Ps[p * PS + threadIdx.x] = a;
        }
        __syncthreads();
        const double2 d = Ps[kk * PS + kk];
        const double dd = d.x * d.x + d.y * d.y;
        const double rdd = dd == 0.0 ? 0.0 : 1.0 / dd;
        const double2 inv = make_double2(d.x * rdd, -d.y * rdd);
        for (int i = kk + 1 + threadIdx.x; i < rows; i += LPT) Ps[i * PS + kk] = cmul(Ps[i * PS + kk], inv);
        if (threadIdx.x == 0) {
            piv[k0 + kk] = k0 + p;
            pivots[k0 + kk] = d;  // log det's terms are summed afterwards, off this column-by-column path
            if (p != kk) ++nswap;
            if (dd == 0.0) sing = 1;
        }
        __syncthreads();
        // rank-1 update of the rest of the panel: A[i, j] -= l_ik u_kj, i > kk, kk < j < nb
        const int w = nb - kk - 1;
        if (w > 0) {
            const int cnt = (rows - kk - 1) * w;
            for (int e = threadIdx.x; e < cnt; e += LPT) {
                const int i = kk + 1 + e / w, j = kk + 1 + e % w;
                const double2 l = Ps[i * PS + kk], u = Ps[kk * PS + j];
                double2 a = Ps[i * PS + j];
                a.x -= l.x * u.x - l.y * u.y;
                a.y -= l.x * u.y + l.y * u.x;
                Ps[i * PS + j] = a;
            }
        }
        __syncthreads();
    }
    for (int e = threadIdx.x; e < rows * nb; e += LPT) {
        const int i = e / nb, j = e % nb;
        A[(int64_t)(k0 + i) * n + k0 + j] = Ps[i * PS + j];
    }
    // panel rows swapped above are whole rows of the panel only; k_lu_laswp swaps the other columns
    if (threadIdx.x == 0) {
        *swaps += nswap;
        if (sing) *singular = 1;
    }
}

// Row swaps of the panel [k0, k0 + nb) applied to every column outside it, in order; one thread per column.
__global__ void k_lu_laswp(double2 *A, int n, int k0, int nb, const int *piv, int64_t mstride) {
    A += blockIdx.y * mstride;  // matrix blockIdx.y of a batch
    piv += (int64_t)blockIdx.y * n;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n || (c >= k0 && c < k0 + nb)) return;
    for (int k = k0; k < k0 + nb; ++k) {
        const int p = piv[k];
        if (p != k) {
            const double2 a = A[(int64_t)k * n + c];
            A[(int64_t)k * n + c] = A[(int64_t)p * n + c];
            A[(int64_t)p * n + c] = a;
        }
    }
}

// Unit-lower triangular solve with the diagonal block L[k0:k0+nb, k0:k0+nb] on columns [c0, n) of rows
// k0..k0+nb of X (X = A for the U block row, X = B for a forward substitution); one thread per column, the
// column's nb unknowns in registers (loops fully unrolled over the LB-row block), four independent partial sums per
// row so that the dependent FP64 chain is a quarter as long, TRSM_T threads per block so that the few columns of a
// small matrix still spread over many SMs. Matrix blockIdx.y of a batch (strides sL, sX).
constexpr int TRSM_T = 32;

__device__ __forceinline__ void csub_mul(double2 &a, double2 l, double2 x) {
    a.x -= l.x * x.x - l.y * x.y;
    a.y -= l.x * x.y + l.y * x.x;
}

template <int LB>
__global__ void __launch_bounds__(TRSM_T) k_trsm_lower_block(const double2 *__restrict__ L, double2 *X, int n, int k0,
                                                             int nb, int c0, int64_t sL, int64_t sX) {
    L += blockIdx.y * sL;
    X += blockIdx.y * sX;
    __shared__ double2 Ls[LB][LB];
    for (int e = threadIdx.x; e < nb * nb; e += blockDim.x)
        Ls[e / nb][e % nb] = L[(int64_t)(k0 + e / nb) * n + k0 + e % nb];
    __syncthreads();
    const int c = c0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    double2 x[LB];
#pragma unroll
    for (int r = 0; r < LB; ++r)  // all loads first: one memory latency instead of one per row
        if (r < nb) x[r] = X[(int64_t)(k0 + r) * n + c];
#pragma unroll
    for (int r = 0; r < LB; ++r) {
        if (r < nb) {
            double2 a[4] = {x[r], make_double2(0, 0), make_double2(0, 0), make_double2(0, 0)};
#pragma unroll
            for (int q = 0; q < r; ++q) csub_mul(a[q & 3], Ls[r][q], x[q]);
            x[r] = make_double2((a[0].x + a[1].x) + (a[2].x + a[3].x), (a[0].y + a[1].y) + (a[2].y + a[3].y));
        }
    }
#pragma unroll
    for (int r = 0; r < LB; ++r)
        if (r < nb) X[(int64_t)(k0 + r) * n + c] = x[r];
}

// Upper triangular solve with the diagonal block U[k0:k0+nb, k0:k0+nb] on all columns of rows k0..k0+nb of B
// (registers, partial sums and block size as above; the reciprocals of the diagonal are formed once per block).
template <int LB>
__global__ void __launch_bounds__(TRSM_T) k_trsm_upper_block(const double2 *__restrict__ U, double2 *B, int n, int k0,
                                                             int nb, int64_t sU, int64_t sB) {
    U += blockIdx.y * sU;
    B += blockIdx.y * sB;
    __shared__ double2 Us[LB][LB];
    __shared__ double2 Ui[LB];
    for (int e = threadIdx.x; e < nb * nb; e += blockDim.x)
        Us[e / nb][e % nb] = U[(int64_t)(k0 + e / nb) * n + k0 + e % nb];
    __syncthreads();
    for (int r = threadIdx.x; r < nb; r += blockDim.x) {
        const double2 d = Us[r][r];
        const double dd = d.x * d.x + d.y * d.y;
        const double rdd = dd == 0.0 ? 0.0 : 1.0 / dd;
        Ui[r] = make_double2(d.x * rdd, -d.y * rdd);
    }
    __syncthreads();
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    double2 x[LB];
#pragma unroll
    for (int r = 0; r < LB; ++r)
        if (r < nb) x[r] = B[(int64_t)(k0 + r) * n + c];
#pragma unroll
    for (int r = LB - 1; r >= 0; --r) {
        if (r < nb) {
            double2 a[4] = {x[r], make_double2(0, 0), make_double2(0, 0), make_double2(0, 0)};
#pragma unroll
            for (int q = r + 1; q < LB; ++q)
                if (q < nb) csub_mul(a[q & 3], Us[r][q], x[q]);
            const double2 v = make_double2((a[0].x + a[1].x) + (a[2].x + a[3].x), (a[0].y + a[1].y) + (a[2].y + a[3].y));
            x[r] = cmul(v, Ui[r]);
        }
    }
#pragma unroll
    for (int r = 0; r < LB; ++r)
        if (r < nb) B[(int64_t)(k0 + r) * n + c] = x[r];
}

// out[t, x] = i * sum_k A_t[k, x] B_t[k, x] (the diagonal of A_t^T B_t) for every slice in one launch, with
// A_t = T[(t + 1) mod Nt] and B_t = P[t] for t < Nt - 1, B_{Nt-1} = G. A block covers 32 columns (one per lane,
// coalesced rows) of one slice; its CD_W warps split k and are summed in shared memory.
constexpr int CD_W = 8;

__global__ void __launch_bounds__(32 * CD_W) k_coldot_slices(const double2 *__restrict__ T, const double2 *__restrict__ P,
                                                             const double2 *__restrict__ G, double2 *__restrict__ out,
                                                             int n, int Nt) {
    const int t = blockIdx.y;
    const int64_t nn = (int64_t)n * n;
    const double2 *A = T + (int64_t)((t + 1) % Nt) * nn;
    const double2 *B = t == Nt - 1 ? G : P + (int64_t)t * nn;
    const int x = blockIdx.x * 32 + threadIdx.x;
    double2 acc = make_double2(0, 0);
    if (x < n)
        for (int k = threadIdx.y; k < n; k += CD_W) {
            const double2 a = A[(int64_t)k * n + x], b = B[(int64_t)k * n + x];
            acc.x += a.x * b.x - a.y * b.y;
            acc.y += a.x * b.y + a.y * b.x;
        }
    __shared__ double2 red[CD_W][32];
    red[threadIdx.y][threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.y == 0 && x < n) {
        double2 sum = red[0][threadIdx.x];
#pragma unroll
        for (int w = 1; w < CD_W; ++w) {
            sum.x += red[w][threadIdx.x].x;
            sum.y += red[w][threadIdx.x].y;
        }
        out[(int64_t)t * n + x] = make_double2(-sum.y, sum.x);  // i * sum
    }
}

// out[j, i] = E[j, i] * d[i]
__global__ void k_colscale(const double2 *__restrict__ E, const double2 *__restrict__ d, double2 *__restrict__ out,
                           int n) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)n * n) return;
    out[idx] = cmul(E[idx], d[idx % n]);
}

// out = T^T + 1
__global__ void k_transpose_plus_identity(const double2 *__restrict__ T, double2 *__restrict__ out, int n) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)n * n) return;
    const int i = (int)(idx / n), j = (int)(idx % n);
    double2 v = T[(int64_t)j * n + i];
    if (i == j) v.x += 1.0;
    out[idx] = v;
}

}  // namespace

// Factors nmat matrices at once (matrix g at A + g * mstride, mstride 0 = n * n): each panel step is one launch
// over the whole batch, so independent matrices (the two species, many configurations) factor side by side on
// different SMs. Pivots, log sums and swap counts are per matrix; the singular flag is shared.
// logsum[g] = sum_k (log|u_kk| + i arg u_kk) over matrix g's pivots (zero pivots, flagged singular, are skipped),
// one block per matrix, fixed-order tree sum.
__global__ void k_pivot_logsum(const double2 *__restrict__ pivots, int n, double2 *__restrict__ logsum) {
    __shared__ double2 red[256];
    const double2 *pv = pivots + (int64_t)blockIdx.x * n;
    double2 acc = make_double2(0, 0);
    for (int k = threadIdx.x; k < n; k += 256) {
        const double2 d = pv[k];
        if (d.x != 0.0 || d.y != 0.0) {
            acc.x += log(hypot(d.x, d.y));
            acc.y += atan2(d.y, d.x);
        }
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            red[threadIdx.x].x += red[threadIdx.x + w].x;
            red[threadIdx.x].y += red[threadIdx.x + w].y;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) logsum[blockIdx.x] = red[0];
}

namespace {
template <int NB>
int lu_factor_nb(nslg_fm *fm, double2 *A, int n, LuScratch &s, int nmat, int64_t mstride, bool pivoting) {
    cudaStream_t st = fm->ctx->stream;
    const double2 minus_one = make_double2(-1, 0);
    for (int k0 = 0; k0 < n; k0 += NB) {
        const int nb = std::min(NB, n - k0);
        const size_t smem = (size_t)(n - k0) * (NB + 1) * sizeof(double2);
        if (n - k0 <= 64)
            k_lu_panel_smem<128, NB><<<nmat, 128, smem, st>>>(A, n, k0, nb, s.piv, s.pivots, s.swaps, s.singular,
                                                              mstride, pivoting);
        else if (smem <= (size_t)PANEL_SMEM)
            k_lu_panel_smem<512, NB><<<nmat, 512, smem, st>>>(A, n, k0, nb, s.piv, s.pivots, s.swaps, s.singular,
                                                              mstride, pivoting);
        else
            k_lu_panel<<<nmat, LT, 0, st>>>(A, n, k0, nb, s.piv, s.pivots, s.swaps, s.singular, mstride, pivoting);
        note_launch(st);
        if (n > nb && pivoting) {
            k_lu_laswp<<<dim3((unsigned)ceil_div(n, 128), (unsigned)nmat), 128, 0, st>>>(A, n, k0, nb, s.piv, mstride);
            note_launch(st);
        }
        const int rest = n - k0 - nb;
        if (rest > 0) {
            // U12 = L11^{-1} A12, then A22 -= L21 U12
            k_trsm_lower_block<NB><<<dim3((unsigned)ceil_div(rest, TRSM_T), (unsigned)nmat), TRSM_T, 0, st>>>(
                A, A, n, k0, nb, k0 + nb, mstride, mstride);
            note_launch(st);
            const double2 *L21 = A + (int64_t)(k0 + nb) * n + k0, *U12 = A + (int64_t)k0 * n + k0 + nb;
            double2 *A22 = A + (int64_t)(k0 + nb) * n + k0 + nb;
            NSLG_TRY(zgemm(st, rest, rest, nb, minus_one, L21, n, mstride, U12, n, mstride, A22, n, mstride, nmat,
                           false, true));
        }
    }
    return NSLG_OK;
}

}  // namespace

// Factors nmat matrices at once (matrix g at A + g * mstride, mstride 0 = n * n): each panel step is one launch
// over the whole batch, so independent matrices (the two species, many configurations) factor side by side on
// different SMs. Pivots, log sums and swap counts are per matrix; the singular flag is shared.
int lu_factor(nslg_fm *fm, double2 *A, int n, LuScratch &s, int nmat, int64_t mstride, bool want_logsum,
              bool pivoting) {
    cudaStream_t st = fm->ctx->stream;
    if (mstride == 0) mstride = (int64_t)n * n;
    {
        // the panel kernels' shared-memory limit, raised once per device (first call is never inside a capture:
        // the captured trajectory runs eagerly first)
        static std::mutex mu;
        static std::set<int> done;
        std::lock_guard<std::mutex> lock(mu);
        if (!done.count(fm->ctx->device)) {
            NSLG_CUDA(cudaFuncSetAttribute(k_lu_panel_smem<512, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           PANEL_SMEM));
            NSLG_CUDA(cudaFuncSetAttribute(k_lu_panel_smem<128, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           PANEL_SMEM));
            NSLG_CUDA(cudaFuncSetAttribute(k_lu_panel_smem<512, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           PANEL_SMEM));
            NSLG_CUDA(cudaFuncSetAttribute(k_lu_panel_smem<128, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           PANEL_SMEM));
            done.insert(fm->ctx->device);
        }
    }
    NSLG_CUDA(cudaMemsetAsync(s.swaps, 0, (size_t)nmat * sizeof(int), st));
    if (!fm->defer_checks) NSLG_CUDA(cudaMemsetAsync(s.singular, 0, sizeof(int), st));
    if (panel_width(n) == 32) NSLG_TRY(lu_factor_nb<32>(fm, A, n, s, nmat, mstride, pivoting));
    else NSLG_TRY(lu_factor_nb<8>(fm, A, n, s, nmat, mstride, pivoting));
    if (want_logsum) {
        k_pivot_logsum<<<(unsigned)nmat, 256, 0, st>>>(s.pivots, n, s.logsum);
        note_launch(st);
    }
    NSLG_CUDA(cudaGetLastError());
    return NSLG_OK;
}

namespace {
template <int NB>
int lu_solve_nb(nslg_fm *fm, const double2 *LU, double2 *B, int n, int nmat, int64_t lu_stride, int64_t b_stride,
                bool backward = true) {
    cudaStream_t st = fm->ctx->stream;
    const double2 minus_one = make_double2(-1, 0);
    const dim3 gc((unsigned)ceil_div(n, TRSM_T), (unsigned)nmat);
    for (int k0 = 0; k0 < n; k0 += NB) {  // forward: L y = P b
        const int nb = std::min(NB, n - k0);
        k_trsm_lower_block<NB><<<gc, TRSM_T, 0, st>>>(LU, B, n, k0, nb, 0, lu_stride, b_stride);
        note_launch(st);
        const int rest = n - k0 - nb;
        if (rest > 0)
            NSLG_TRY(zgemm(st, rest, n, nb, minus_one, LU + (int64_t)(k0 + nb) * n + k0, n, lu_stride,
                           B + (int64_t)k0 * n, n, b_stride, B + (int64_t)(k0 + nb) * n, n, b_stride, nmat, false,
                           true));
    }
    if (!backward) return NSLG_OK;
    for (int k0 = ((n - 1) / NB) * NB; k0 >= 0; k0 -= NB) {  // backward: U x = y
        const int nb = std::min(NB, n - k0);
        k_trsm_upper_block<NB><<<gc, TRSM_T, 0, st>>>(LU, B, n, k0, nb, lu_stride, b_stride);
        note_launch(st);
        if (k0 > 0)
            NSLG_TRY(zgemm(st, k0, n, nb, minus_one, LU + k0, n, lu_stride, B + (int64_t)k0 * n, n, b_stride, B, n,
                           b_stride, nmat, false, true));
    }
    return NSLG_OK;
}

// B[g] = P_g I: the identity with the factorisation's row swaps applied in order (row k of the result is row
// perm[k] of I, perm the composition of the swaps). Each block rebuilds perm in shared memory with one thread, then
// its threads write rows [row0, row0 + rows_per_block) of matrix blockIdx.x.
__global__ void k_perm_identity(double2 *B, int n, const int *piv, int64_t bstride, int rows_per_block) {
    extern __shared__ int perm[];
    const int g = blockIdx.x;
    piv += (int64_t)g * n;
    B += g * bstride;
    if (threadIdx.x == 0) {
        for (int k = 0; k < n; ++k) perm[k] = k;
        for (int k = 0; k < n; ++k) {
            const int p = piv[k];
            const int a = perm[k];
            perm[k] = perm[p];
            perm[p] = a;
        }
    }
    __syncthreads();
    const int r0 = blockIdx.y * rows_per_block, r1 = min(n, r0 + rows_per_block);
    for (int64_t e = (int64_t)r0 * n + threadIdx.x; e < (int64_t)r1 * n; e += blockDim.x) {
        const int k = (int)(e / n), j = (int)(e % n);
        B[e] = make_double2(j == perm[k] ? 1.0 : 0.0, 0.0);
    }
}

// G[g] = A_g^{-1} for small matrices (n <= GJ_MAX) in one launch: Gauss-Jordan elimination with partial pivoting on
// [A | I] in shared memory, one CTA per matrix. The pivot of step k is chosen from the same Schur-complement column
// as in the LU with partial pivoting (same rule), so pivots (if given), swaps and singular mean the same as after
// lu_factor.
// Replaces the panel, triangular-solve and permutation launches of lu_factor + lu_inverse for the small lattices,
// where each of those launches is a chain of dependent FP64 steps.
constexpr int GJ_MAX = 32;
constexpr int GJ_T = 256;
constexpr int SCAN_MAX_MATRICES = 8;  // the small-lattice gradient uses scans up to this many matrices per call

__global__ void __launch_bounds__(GJ_T) k_gj_inverse(const double2 *__restrict__ A, int64_t astride,
                                                     double2 *__restrict__ G, int n, double2 *pivots, int *swaps,
                                                     int *singular) {
    __shared__ double2 W[GJ_MAX][2 * GJ_MAX + 1];
    __shared__ double2 f[GJ_MAX];
    __shared__ double2 inv_sh;
    __shared__ int pivot;
    const int g = blockIdx.x;
    A += g * astride;
    G += (int64_t)g * n * n;
    const int w = 2 * n;
    for (int e = threadIdx.x; e < n * w; e += GJ_T) {
        const int i = e / w, j = e % w;
        W[i][j] = j < n ? A[(int64_t)i * n + j] : make_double2(j - n == i ? 1.0 : 0.0, 0.0);
    }
    __syncthreads();
        int nswap = 0, sing = 0;
    for (int k = 0; k < n; ++k) {
        if (threadIdx.x < 32) {  // pivot: largest |a_ik|^2 over rows i >= k, first index on ties
            double bm = -1.0;
            int bi = n;
            const int i = k + threadIdx.x;
            if (i < n) {
                const double2 v = W[i][k];
                bm = v.x * v.x + v.y * v.y;
                bi = i;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const double om = __shfl_down_sync(0xffffffffu, bm, o);
                const int oi = __shfl_down_sync(0xffffffffu, bi, o);
                if (piv_better(om, oi, bm, bi)) {
                    bm = om;
                    bi = oi;
                }
            }
            if (threadIdx.x == 0) pivot = bi;
        }
        __syncthreads();
        const int p = pivot;
        if (p != k)
            for (int j = threadIdx.x; j < w; j += GJ_T) {
                const double2 a = W[k][j];
                W[k][j] = W[p][j];
                W[p][j] = a;
            }
        __syncthreads();
        if (threadIdx.x == 0) {
            const double2 d = W[k][k];
            const double dd = d.x * d.x + d.y * d.y;
            const double rdd = dd == 0.0 ? 0.0 : 1.0 / dd;
            inv_sh = make_double2(d.x * rdd, -d.y * rdd);
            if (pivots) pivots[(int64_t)g * n + k] = d;
            if (p != k) ++nswap;
            if (dd == 0.0) sing = 1;
        }
        __syncthreads();
        const double2 inv = inv_sh;
        for (int j = k + threadIdx.x; j < w; j += GJ_T) W[k][j] = cmul(W[k][j], inv);  // columns < k of row k are 0
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += GJ_T) f[i] = i == k ? make_double2(0, 0) : W[i][k];
        __syncthreads();
        const int wk = w - k;
        for (int e = threadIdx.x; e < n * wk; e += GJ_T) {
            const int i = e / wk, j = k + e % wk;
            if (i == k) continue;
            const double2 l = f[i], u = W[k][j];
            double2 a = W[i][j];
            a.x -= l.x * u.x - l.y * u.y;
            a.y -= l.x * u.y + l.y * u.x;
            W[i][j] = a;
        }
        __syncthreads();
    }
    for (int e = threadIdx.x; e < n * n; e += GJ_T) G[e] = W[e / n][n + e % n];
    if (threadIdx.x == 0) {
        swaps[g] = nswap;
        if (sing) *singular = 1;
    }
}

}  // namespace

// G[g] = A_g^{-1} for nmat factored matrices (LU of matrix g at LU + g * lu_stride, G dense (nmat, n, n)).
int lu_inverse(nslg_fm *fm, const double2 *LU, double2 *G, int n, const LuScratch &s, int nmat, int64_t lu_stride) {
    cudaStream_t st = fm->ctx->stream;
    const int64_t nn = (int64_t)n * n;
    if (lu_stride == 0) lu_stride = nn;
    const int rpb = 32;
    k_perm_identity<<<dim3((unsigned)nmat, (unsigned)ceil_div(n, rpb)), 256, (size_t)n * sizeof(int), st>>>(
        G, n, s.piv, nn, rpb);
    note_launch(st);
    if (panel_width(n) == 32) NSLG_TRY(lu_solve_nb<32>(fm, LU, G, n, nmat, lu_stride, nn));
    else NSLG_TRY(lu_solve_nb<8>(fm, LU, G, n, nmat, lu_stride, nn));
    NSLG_CUDA(cudaGetLastError());
    return NSLG_OK;
}

// Forward substitution only: B[g] = L_g^{-1} B[g] with the unit lower factor of an LU computed without pivoting.
int lu_forward(nslg_fm *fm, const double2 *LU, double2 *B, int n, int nmat, int64_t lu_stride, int64_t b_stride) {
    if (panel_width(n) == 32) return lu_solve_nb<32>(fm, LU, B, n, nmat, lu_stride, b_stride, false);
    return lu_solve_nb<8>(fm, LU, B, n, nmat, lu_stride, b_stride, false);
}

int get_lu_scratch(nslg_fm *fm, int n, LuScratch &s, int nmat, const char *tag) {
    const std::string t = tag ? tag : "lu";
    NSLG_TRY(ws_get(fm, (t + "_piv").c_str(), (size_t)n * nmat, &s.piv));
    NSLG_TRY(ws_get(fm, (t + "_logsum").c_str(), (size_t)nmat, &s.logsum));
    NSLG_TRY(ws_get(fm, (t + "_pivots").c_str(), (size_t)n * nmat, &s.pivots));
    NSLG_TRY(ws_get(fm, (t + "_swaps").c_str(), (size_t)nmat, &s.swaps));
    NSLG_TRY(ws_get(fm, "lu_singular", 1, &s.singular));
    return NSLG_OK;
}

namespace {

// In-place product tree over T matrices in buf (T, n, n): after the call buf[0] = M_{T-1} ... M_0.
int product_tree(nslg_fm *fm, double2 *buf, double2 *tmp, int T, int n) {
    cudaStream_t st = fm->ctx->stream;
    const int64_t nn = (int64_t)n * n;
    const double2 one = make_double2(1, 0);
    while (T > 1) {
        const int pairs = T / 2;
        // tmp[k] = buf[2k+1] @ buf[2k]
        NSLG_TRY(zgemm(st, n, n, n, one, buf + nn, n, 2 * nn, buf, n, 2 * nn, tmp, n, nn, pairs, false));
        NSLG_CUDA(cudaMemcpyAsync(buf, tmp, pairs * nn * sizeof(double2), cudaMemcpyDeviceToDevice, st));
        if (T & 1)
            NSLG_CUDA(cudaMemcpyAsync(buf + pairs * nn, buf + (T - 1) * nn, nn * sizeof(double2),
                                      cudaMemcpyDeviceToDevice, st));
        T = pairs + (T & 1);
    }
    return NSLG_OK;
}

}  // namespace

// log det M for the populated configuration and current species; result on the host.
int fm_logdet(nslg_fm *fm, double2 *out) {
    cudaStream_t st = fm->ctx->stream;
    const int Nt = (int)fm->Nt, n = (int)fm->Nx;
    const int64_t nn = (int64_t)n * n;
    const bool diag = fm->kind == NSLG_FM_DIAG;
    const double2 d = make_double2(fm->sgn * fm->delta.x, fm->sgn * fm->delta.y);
    if (use_stratified(fm)) {
        const ExpEntry *Ep, *Ed;
        NSLG_TRY(get_exp(fm, make_double2(-d.x, -d.y), &Ep));
        NSLG_TRY(get_exp(fm, d, &Ed));
        const int sg = fm->sgn;
        return logdet_strat(fm, 1, &Ep, &Ed, &sg, fm->phase, fm->phase_inv, out);
    }
    const ExpEntry *E;
    if (diag) NSLG_TRY(get_lin(fm, d, 1, &E));  // 1 - sgn delta K
    else NSLG_TRY(get_exp(fm, d, &E));
    double2 *B, *tmp, *phisum;
    NSLG_TRY(ws_get(fm, "ld_slices", (size_t)Nt * nn, &B));
    NSLG_TRY(ws_get(fm, "ld_tmp", (size_t)((Nt + 1) / 2) * nn, &tmp));
    NSLG_TRY(ws_get(fm, "ld_phisum", 1, &phisum));
    LuScratch s;
    NSLG_TRY(get_lu_scratch(fm, n, s));
    // Exp: B_t = exp(sgn delta K) diag(phiExp[t+1]), product B_{Nt-1} ... B_0 (hubbardExp.tpp:140-147).
    // Diag: fk_t = (1 - sgn delta K) diag(phiExpInv[t+1]), product fk_0 ... fk_{Nt-1} (hubbardDiag.tpp:176-187).
    k_slices<<<(unsigned)ceil_div(nn * Nt, 256), 256, 0, st>>>(E->full, diag ? fm->phase_inv : fm->phase, B, Nt, n,
                                                                1, false, diag);
    note_launch(st);
    NSLG_CUDA(cudaGetLastError());
    NSLG_TRY(product_tree(fm, B, tmp, Nt, n));
    k_add_identity<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(B, n);
    note_launch(st);
    NSLG_TRY(lu_factor(fm, B, n, s));
    double2 ls;
    int sw = 0, sing = 0;
    NSLG_CUDA(cudaMemcpyAsync(&ls, s.logsum, sizeof(double2), cudaMemcpyDeviceToHost, st));
    NSLG_CUDA(cudaMemcpyAsync(&sw, s.swaps, sizeof(int), cudaMemcpyDeviceToHost, st));
    NSLG_CUDA(cudaMemcpyAsync(&sing, s.singular, sizeof(int), cudaMemcpyDeviceToHost, st));
    NSLG_CUDA(cudaStreamSynchronize(st));
    if (sing) {
        *out = make_double2(-INFINITY, 0.0);
        return NSLG_OK;
    }
    double im = ls.y + (sw & 1 ? M_PI : 0.0);
    im = std::remainder(im, 2.0 * M_PI);  // principal branch, like log(det(.))
    if (im <= -M_PI) im += 2.0 * M_PI;
    *out = make_double2(ls.x, im);
    if (diag) {  // + i sgn sum(phi), not folded (hubbardDiag.tpp:189-191)
        k_sum_c128<<<1, 256, 0, st>>>(fm->phi, (int64_t)Nt * n, phisum);
        note_launch(st);
        double2 ps;
        NSLG_CUDA(cudaMemcpyAsync(&ps, phisum, sizeof(double2), cudaMemcpyDeviceToHost, st));
        NSLG_CUDA(cudaStreamSynchronize(st));
        out->x += -fm->sgn * ps.y;
        out->y += fm->sgn * ps.x;
    }
    return NSLG_OK;
}

namespace {

// Batched k_slices: B[g, t, i, j] = E_g[i, j] * ph[g, (t + shift) mod Nt, rowscale ? i : j] with
// E_g = (g & emask) ? E1 : E0.
__global__ void k_slices_many(const double2 *__restrict__ E0, const double2 *__restrict__ E1, int emask,
                              const double2 *__restrict__ ph, double2 *__restrict__ B, int nmat, int Nt, int n,
                              int shift, bool rowscale) {
    const int64_t nn = (int64_t)n * n;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nn * Nt * nmat) return;
    const int64_t gt = idx / nn;
    const int g = (int)(gt / Nt), t = (int)(gt % Nt);
    const int64_t ij = idx - gt * nn;
    const int i = (int)(ij / n), j = (int)(ij - (int64_t)i * n);
    const double2 *E = (g & emask) ? E1 : E0;
    const int ts = ((t + shift) % Nt + Nt) % Nt;
    B[idx] = cmul(E[ij], ph[((int64_t)g * Nt + ts) * n + (rowscale ? i : j)]);
}

// A[g] += 1 for nmat matrices at stride mstride
__global__ void k_add_identity_many(double2 *A, int n, int nmat, int64_t mstride) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)n * nmat) return;
    const int g = (int)(idx / n), i = (int)(idx % n);
    A[g * mstride + (int64_t)i * n + i].x += 1.0;
}

// out[g, t, x] = i * sum_k S[g, (t + 1) mod Nt][x, k] B[k, x] with B = P[g, t] (t < Nt - 1) or G[g] (t = Nt - 1):
// one warp per (g, t, x), lanes over k (row of S coalesced), shuffle reduction.
__global__ void k_diagprod_many(const double2 *__restrict__ S, const double2 *__restrict__ P,
                                const double2 *__restrict__ G, double2 *__restrict__ out, int n, int Nt, int nmat) {
    const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (wid >= (int64_t)nmat * Nt * n) return;
    const int x = (int)(wid % n);
    const int64_t gt = wid / n;
    const int g = (int)(gt / Nt), t = (int)(gt % Nt);
    const int64_t nn = (int64_t)n * n;
    const double2 *Sr = S + ((int64_t)g * Nt + (t + 1) % Nt) * nn + (int64_t)x * n;
    const double2 *B = t == Nt - 1 ? G + (int64_t)g * nn : P + ((int64_t)g * Nt + t) * nn;
    double2 acc = make_double2(0, 0);
    for (int k = lane; k < n; k += 32) {
        const double2 a = Sr[k], bv = B[(int64_t)k * n + x];
        acc.x += a.x * bv.x - a.y * bv.y;
        acc.y += a.x * bv.y + a.y * bv.x;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        acc.x += __shfl_down_sync(0xffffffffu, acc.x, o);
        acc.y += __shfl_down_sync(0xffffffffu, acc.y, o);
    }
    if (lane == 0) out[gt * n + x] = make_double2(-acc.y, acc.x);  // i * acc
}

}  // namespace

namespace {

// Tensor-core form of the gradient (force precision NSLG_PREC_BF16_SPLIT; exponential discretisation with a real
// exp(-sgn delta K), symmetric because K is real and Hermitian). Both chains become split-BF16 products Y E'^T with
// a diagonal scale, E' = exp(-sgn delta K), D_t = phiExpInv[(t - 1) mod Nt]:
//   T(t) = S(t)^T = T(t+1) E'^T D_t         (column scale of the product),  T(Nt-1) = E' D_{Nt-1}
//   P(t) = P(t-1) Fk(t) = (P(t-1) D_t) E'    (column scale of the operand),  P(-1) = G = (1 + S(0))^{-1} (FP64 LU)
//   pi_dot(t) = i diag(S(t+1) P(t)) = i sum_k T(t+1)[k, x] P(t)[k, x]
int grad_logdet_tc(nslg_fm *fm, const ExpEntry *E, double2 *out) {
    const ExpEntry *Es[1] = {E};
    return grad_logdet_tc_many(fm, 1, Es, fm->phase_inv, out);
}

}  // namespace

// The split-BF16 gradient for nmat matrices (matrix g: factor E[g], phase rows ph_inv + g * Nt * Nx, output
// out + g * Nt * Nx): the FP64 LU of the nmat matrices 1 + S(0) and the solves against the identity run as one
// batch, so the two species of a force share the single-SM LU launches; with two matrices the second one's
// tensor-core chains run on the handle's side stream, beside the first one's (each chain product fills only a
// few dozen SMs).
int grad_logdet_tc_many(nslg_fm *fm, int nmat, const ExpEntry *const *E, const double2 *ph_inv, double2 *out) {
    cudaStream_t st = fm->ctx->stream;
    const int Nt = (int)fm->Nt, n = (int)fm->Nx;
    const int64_t nn = (int64_t)n * n, ms = (int64_t)Nt * nn;
    NSLG_REQUIRE(nmat == 1 || nmat == 2, NSLG_ERR_ARG, "split-BF16 gradient: one or two matrices");
    std::vector<OzPlanes *> Pz(nmat);
    for (int g = 0; g < nmat; ++g) NSLG_TRY(oz_planes(fm, E[g], &Pz[g]));
    double2 *T, *P, *G;
    NSLG_TRY(ws_get(fm, "gr_S", (size_t)nmat * ms, &T));
    NSLG_TRY(ws_get(fm, "gr_P", (size_t)nmat * ms, &P));
    NSLG_TRY(ws_get(fm, "gr_G", (size_t)nmat * nn, &G));
    const size_t dg_elems = (size_t)oz_digits() * 2 * n * oz_ld(n) * 2;  // digit planes of one product (bytes/2)
    char *dg;
    int *rexp;
    NSLG_TRY(ws_get(fm, "fz_digits", dg_elems * nmat, &dg));
    NSLG_TRY(ws_get(fm, "fz_rexp", (size_t)2 * n * nmat, &rexp));
    cudaStream_t sg[2] = {st, st};
    if (nmat == 2) {
        if (!fm->side) NSLG_CUDA(cudaStreamCreateWithFlags(&fm->side, cudaStreamNonBlocking));
        if (!fm->ev_fork) NSLG_CUDA(cudaEventCreateWithFlags(&fm->ev_fork, cudaEventDisableTiming));
        if (!fm->ev_join) NSLG_CUDA(cudaEventCreateWithFlags(&fm->ev_join, cudaEventDisableTiming));
        sg[1] = fm->side;
    }
    auto fork = [&]() -> int {
        if (nmat == 2) {
            NSLG_CUDA(cudaEventRecord(fm->ev_fork, st));
            NSLG_CUDA(cudaStreamWaitEvent(fm->side, fm->ev_fork, 0));
        }
        return NSLG_OK;
    };
    auto join = [&]() -> int {
        if (nmat == 2) {
            NSLG_CUDA(cudaEventRecord(fm->ev_join, fm->side));
            NSLG_CUDA(cudaStreamWaitEvent(st, fm->ev_join, 0));
        }
        return NSLG_OK;
    };
    LuScratch s;
    NSLG_TRY(get_lu_scratch(fm, n, s, nmat));
    auto D = [&](int g, int t) { return ph_inv + ((int64_t)g * Nt + ((t - 1) % Nt + Nt) % Nt) * n; };
    auto Tg = [&](int g, int t) { return T + g * ms + (int64_t)t * nn; };
    auto Pg = [&](int g, int t) { return P + g * ms + (int64_t)t * nn; };
    auto dgg = [&](int g) { return (void *)(dg + g * dg_elems); };
    const unsigned g2 = (unsigned)ceil_div(nn, 256);
    NSLG_TRY(fork());
    for (int g = 0; g < nmat; ++g) {
        k_colscale<<<g2, 256, 0, sg[g]>>>(E[g]->full, D(g, Nt - 1), Tg(g, Nt - 1), n);
        note_launch(sg[g]);
        for (int t = Nt - 2; t >= 0; --t)
            NSLG_TRY(oz_gemm(Tg(g, t + 1), Tg(g, t), nullptr, D(g, t), *Pz[g], dgg(g), rexp + 2 * n * g, n, n,
                             fm->tc_err, sg[g]));
        k_transpose_plus_identity<<<g2, 256, 0, sg[g]>>>(Tg(g, 0), Pg(g, 0), n);  // 1 + S(0) in P[g, 0] as scratch
        note_launch(sg[g]);
    }
    NSLG_TRY(join());
    NSLG_TRY(lu_factor(fm, P, n, s, nmat, ms, false));
    NSLG_TRY(lu_inverse(fm, P, G, n, s, nmat, ms));
    NSLG_TRY(fork());
    for (int g = 0; g < nmat; ++g)
        for (int t = 0; t < Nt - 1; ++t) {
            const double2 *prev = t == 0 ? G + g * nn : Pg(g, t - 1);
            NSLG_TRY(oz_gemm(prev, Pg(g, t), D(g, t), nullptr, *Pz[g], dgg(g), rexp + 2 * n * g, n, n, fm->tc_err,
                             sg[g]));
        }
    NSLG_TRY(join());
    for (int g = 0; g < nmat; ++g) {
        k_coldot_slices<<<dim3((unsigned)ceil_div(n, 32), (unsigned)Nt), dim3(32, CD_W), 0, st>>>(
            T + g * ms, P + g * ms, G + g * nn, out + (int64_t)g * Nt * n, n, Nt);
        note_launch(st);
    }
    NSLG_CUDA(cudaGetLastError());
    return NSLG_OK;
}

// d log det M / d phi (Nt, Nx) into a device buffer.
int fm_grad_logdet(nslg_fm *fm, double2 *out) {
    cudaStream_t st = fm->ctx->stream;
    const int n = (int)fm->Nx;
    // Fk(t) = diag(phiExpInv[t-1]) exp(-sgn delta K) (Exp) or diag(phiExpInv[t-1]) (1 - sgn delta K) (Diag,
    // hubbardDiag.tpp:203-205)
    const ExpEntry *E;
    if (fm->kind == NSLG_FM_DIAG) NSLG_TRY(get_lin(fm, make_double2(fm->sgn * fm->delta.x, fm->sgn * fm->delta.y), 1, &E));
    else NSLG_TRY(get_exp(fm, make_double2(-fm->sgn * fm->delta.x, -fm->sgn * fm->delta.y), &E));
    if (use_stratified_grad(fm)) {
        const ExpEntry *Ed;
        NSLG_TRY(get_exp(fm, make_double2(fm->sgn * fm->delta.x, fm->sgn * fm->delta.y), &Ed));
        NSLG_TRY(grad_logdet_strat(fm, 1, &E, &Ed, fm->phase, fm->phase_inv, out));
    } else if (fm->force_precision == NSLG_PREC_BF16_SPLIT && fm->kind == NSLG_FM_EXP && E->is_real && n <= 2048) {
        NSLG_TRY(grad_logdet_tc(fm, E, out));
    } else {
        NSLG_TRY(grad_logdet_many(fm, 1, E->full, E->full, 0, fm->phase_inv, out));
    }
    if (fm->defer_checks) return NSLG_OK;  // the captured trajectory checks the sticky flag after its replay
    LuScratch s;
    NSLG_TRY(get_lu_scratch(fm, n, s));
    int sing = 0;
    NSLG_CUDA(cudaMemcpyAsync(&sing, s.singular, sizeof(int), cudaMemcpyDeviceToHost, st));
    NSLG_CUDA(cudaStreamSynchronize(st));
    NSLG_REQUIRE(!sing, NSLG_ERR_ARG, "gradLogDetM: 1 + A^{-1} is singular");
    return NSLG_OK;
}


// d log det M / d phi for nmat matrices at once (hubbardExp.tpp:153-211), FP64: matrix g has the time-slice factor
// E_g = (g & emask) ? E1 : E0 and the phase rows ph_inv[g] = phiExpInv (Nt, Nx); out is (nmat, Nt, Nx).
//   Fk(t) = diag(phiExpInv[(t - 1) mod Nt]) E,  S(t) = Fk(t) S(t+1), S(Nt-1) = Fk(Nt-1),
//   G = (1 + S(0))^{-1},  P(t) = P(t-1) Fk(t), P(-1) = G,  pi_dot(t) = i diag(S(t+1) P(t)), pi_dot(Nt-1) = i diag(S(0) G).
// Every chain step is one batched GEMM over the nmat matrices and the LU/solve factor them side by side, so the
// species of one configuration, or many configurations, share each launch.
int grad_logdet_many(nslg_fm *fm, int nmat, const double2 *E0, const double2 *E1, int emask, const double2 *ph_inv,
                     double2 *out) {
    cudaStream_t st = fm->ctx->stream;
    const int Nt = (int)fm->Nt, n = (int)fm->Nx;
    const int64_t nn = (int64_t)n * n, ms = (int64_t)Nt * nn;
    double2 *Fk, *S, *P, *G;
    NSLG_TRY(ws_get(fm, "gr_Fk", (size_t)nmat * ms, &Fk));
    NSLG_TRY(ws_get(fm, "gr_S", (size_t)nmat * ms, &S));
    NSLG_TRY(ws_get(fm, "gr_P", (size_t)nmat * ms, &P));
    NSLG_TRY(ws_get(fm, "gr_G", (size_t)nmat * nn, &G));
    LuScratch s;
    NSLG_TRY(get_lu_scratch(fm, n, s, nmat));
    const double2 one = make_double2(1, 0);
    k_slices_many<<<(unsigned)ceil_div(ms * nmat, 256), 256, 0, st>>>(E0, E1, emask, ph_inv, Fk, nmat, Nt, n, -1,
                                                                       true);
    note_launch(st);
    if (n <= GJ_MAX && Nt > 1 && nmat <= SCAN_MAX_MATRICES) {
        // Small matrices, few of them: the chains are latency-bound (each product is a few microseconds of dependent
        // FP64 steps on a handful of SMs), so they become scans with log2(Nt) levels of batched products
        // (Hillis-Steele: ~Nt log2 Nt products instead of 2 (Nt - 1), all of a level in one launch; with many
        // matrices the chains already fill the GPU and the scans' extra products would cost more than they save):
        //   Q(t) = Fk(0) ... Fk(t) (prefix), S(t) = Fk(t) ... Fk(Nt-1) (suffix), P(t) = G Q(t) (one launch),
        // and G = (1 + S(0))^{-1} comes from one Gauss-Jordan launch.
        double2 *Q0, *Q1, *S1, *Pm;
        NSLG_TRY(ws_get(fm, "gr_Q0", (size_t)nmat * ms, &Q0));
        NSLG_TRY(ws_get(fm, "gr_Q1", (size_t)nmat * ms, &Q1));
        NSLG_TRY(ws_get(fm, "gr_S1", (size_t)nmat * ms, &S1));
        NSLG_TRY(ws_get(fm, "gr_Pm", (size_t)nmat * nn, &Pm));
        const double2 *Qc = Fk, *Sc = Fk;
        double2 *Qbuf[2] = {Q0, Q1}, *Sbuf[2] = {S, S1};
        int lvl = 0;
        for (int o = 1; o < Nt; o <<= 1, ++lvl) {
            double2 *Qn = Qbuf[lvl & 1], *Sn = Sbuf[lvl & 1];
            // prefix: Qn(t) = Q(t - o) Q(t) for t >= o, Qn(t) = Q(t) below
            NSLG_TRY(zgemm2(st, n, n, n, one, Qc, n, ms, nn, Qc + o * nn, n, ms, nn, Qn + o * nn, n, ms, nn, nmat,
                            Nt - o));
            NSLG_CUDA(cudaMemcpy2DAsync(Qn, ms * sizeof(double2), Qc, ms * sizeof(double2), o * nn * sizeof(double2),
                                        nmat, cudaMemcpyDeviceToDevice, st));
            // suffix: Sn(t) = S(t) S(t + o) for t < Nt - o, Sn(t) = S(t) above
            NSLG_TRY(zgemm2(st, n, n, n, one, Sc, n, ms, nn, Sc + o * nn, n, ms, nn, Sn, n, ms, nn, nmat, Nt - o));
            NSLG_CUDA(cudaMemcpy2DAsync(Sn + (Nt - o) * nn, ms * sizeof(double2), Sc + (Nt - o) * nn,
                                        ms * sizeof(double2), o * nn * sizeof(double2), nmat, cudaMemcpyDeviceToDevice,
                                        st));
            Qc = Qn;
            Sc = Sn;
        }
        NSLG_CUDA(cudaMemcpy2DAsync(Pm, nn * sizeof(double2), Sc, ms * sizeof(double2), nn * sizeof(double2), nmat,
                                    cudaMemcpyDeviceToDevice, st));
        k_add_identity_many<<<(unsigned)ceil_div((int64_t)n * nmat, 256), 256, 0, st>>>(Pm, n, nmat, nn);
        note_launch(st);
        if (!fm->defer_checks) NSLG_CUDA(cudaMemsetAsync(s.singular, 0, sizeof(int), st));
        k_gj_inverse<<<(unsigned)nmat, GJ_T, 0, st>>>(Pm, nn, G, n, nullptr, s.swaps, s.singular);
        note_launch(st);
        NSLG_TRY(zgemm2(st, n, n, n, one, G, n, nn, 0, Qc, n, ms, nn, P, n, ms, nn, nmat, Nt - 1));
        const int64_t warps = (int64_t)nmat * Nt * n;
        k_diagprod_many<<<(unsigned)ceil_div(warps * 32, 256), 256, 0, st>>>(Sc, P, G, out, n, Nt, nmat);
        note_launch(st);
        NSLG_CUDA(cudaGetLastError());
        return NSLG_OK;
    }
    // S(Nt-1) = Fk(Nt-1), then the suffix chain
    NSLG_CUDA(cudaMemcpy2DAsync(S + (int64_t)(Nt - 1) * nn, ms * sizeof(double2), Fk + (int64_t)(Nt - 1) * nn,
                                ms * sizeof(double2), nn * sizeof(double2), nmat, cudaMemcpyDeviceToDevice, st));
    for (int t = Nt - 2; t >= 0; --t)
        NSLG_TRY(zgemm(st, n, n, n, one, Fk + t * nn, n, ms, S + (t + 1) * nn, n, ms, S + t * nn, n, ms, nmat, false));
    // 1 + S(0) in P[g, 0] as scratch, factor, G = (1 + S(0))^{-1}
    NSLG_CUDA(cudaMemcpy2DAsync(P, ms * sizeof(double2), S, ms * sizeof(double2), nn * sizeof(double2), nmat,
                                cudaMemcpyDeviceToDevice, st));
    k_add_identity_many<<<(unsigned)ceil_div((int64_t)n * nmat, 256), 256, 0, st>>>(P, n, nmat, ms);
    note_launch(st);
    if (n <= GJ_MAX) {
        if (!fm->defer_checks) NSLG_CUDA(cudaMemsetAsync(s.singular, 0, sizeof(int), st));
        k_gj_inverse<<<(unsigned)nmat, GJ_T, 0, st>>>(P, ms, G, n, nullptr, s.swaps, s.singular);
        note_launch(st);
    } else {
        NSLG_TRY(lu_factor(fm, P, n, s, nmat, ms, false));
        NSLG_TRY(lu_inverse(fm, P, G, n, s, nmat, ms));
    }
    // prefix chain P(t) = P(t-1) Fk(t), P(-1) = G
    for (int t = 0; t < Nt - 1; ++t) {
        const double2 *prev = t == 0 ? G : P + (t - 1) * nn;
        NSLG_TRY(zgemm(st, n, n, n, one, prev, n, t == 0 ? nn : ms, Fk + t * nn, n, ms, P + t * nn, n, ms, nmat,
                       false));
    }
    const int64_t warps = (int64_t)nmat * Nt * n;
    k_diagprod_many<<<(unsigned)ceil_div(warps * 32, 256), 256, 0, st>>>(S, P, G, out, n, Nt, nmat);
    note_launch(st);
    NSLG_CUDA(cudaGetLastError());
    return NSLG_OK;
}

// log det M for nmat matrices of the exponential discretisation at once (hubbardExp.tpp:129-150): matrix g has
// B_t = E_g diag(phiExp_g[(t + 1) mod Nt]) with E_g = (g & emask) ? E1 : E0 and phase rows ph[g] (Nt, Nx). The
// product B_{Nt-1} ... B_0 is a chain of batched GEMMs (one launch per t for all g), 1 + product is factored by the
// batched LU and log det = sum log u_kk + i pi (#swaps) on the principal branch; out[g] on the host (-inf for a
// singular matrix).
int logdet_many(nslg_fm *fm, int nmat, const double2 *E0, const double2 *E1, int emask, const double2 *ph,
                double2 *out) {
    cudaStream_t st = fm->ctx->stream;
    const int Nt = (int)fm->Nt, n = (int)fm->Nx;
    const int64_t nn = (int64_t)n * n, ms = (int64_t)Nt * nn;
    double2 *B, *R;
    NSLG_TRY(ws_get(fm, "ldm_slices", (size_t)nmat * ms, &B));
    NSLG_TRY(ws_get(fm, "ldm_prod", (size_t)2 * nmat * nn, &R));
    LuScratch s;
    NSLG_TRY(get_lu_scratch(fm, n, s, nmat));
    const double2 one = make_double2(1, 0);
    k_slices_many<<<(unsigned)ceil_div(ms * nmat, 256), 256, 0, st>>>(E0, E1, emask, ph, B, nmat, Nt, n, 1, false);
    note_launch(st);
    double2 *cur = R, *nxt = R + (int64_t)nmat * nn;
    NSLG_CUDA(cudaMemcpy2DAsync(cur, nn * sizeof(double2), B, ms * sizeof(double2), nn * sizeof(double2), nmat,
                                cudaMemcpyDeviceToDevice, st));
    for (int t = 1; t < Nt; ++t) {
        NSLG_TRY(zgemm(st, n, n, n, one, B + t * nn, n, ms, cur, n, nn, nxt, n, nn, nmat, false));
        std::swap(cur, nxt);
    }
    k_add_identity_many<<<(unsigned)ceil_div((int64_t)n * nmat, 256), 256, 0, st>>>(cur, n, nmat, nn);
    note_launch(st);
    NSLG_TRY(lu_factor(fm, cur, n, s, nmat, nn));
    std::vector<double2> ls(nmat);
    std::vector<int> sw(nmat);
    int sing = 0;
    NSLG_CUDA(cudaMemcpyAsync(ls.data(), s.logsum, nmat * sizeof(double2), cudaMemcpyDeviceToHost, st));
    NSLG_CUDA(cudaMemcpyAsync(sw.data(), s.swaps, nmat * sizeof(int), cudaMemcpyDeviceToHost, st));
    NSLG_CUDA(cudaMemcpyAsync(&sing, s.singular, sizeof(int), cudaMemcpyDeviceToHost, st));
    NSLG_CUDA(cudaStreamSynchronize(st));
    NSLG_REQUIRE(!sing, NSLG_ERR_ARG, "logDetM: 1 + prod B_t is singular for a configuration of the batch");
    for (int g = 0; g < nmat; ++g) {
        double im = ls[g].y + (sw[g] & 1 ? M_PI : 0.0);
        im = std::remainder(im, 2.0 * M_PI);
        if (im <= -M_PI) im += 2.0 * M_PI;
        out[g] = make_double2(ls[g].x, im);
    }
    return NSLG_OK;
}

}  // namespace nslg
