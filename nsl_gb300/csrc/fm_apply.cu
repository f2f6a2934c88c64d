// Fused fermion-matrix applications M psi and M^dagger psi (exponential discretisation) on CUDA cores.
//
// One launch evaluates, for every right-hand side r and time slice t (hubbardExp.tpp:13-75),
//   M:    out[r, t+1] = psi[r, t+1] - B_{t+1} * expK (phase[t] o psi[r, t])           (B_0 = -1)
//   Mdag: out[r, t-1] = psi[r, t-1] - conj(phase[t-1]) o B'_{t-1} * expK* psi[r, t]    (B'_{Nt-1} = -1)
// as one GEMM over the spatial index with the phase multiply in the operand load (prologue) and the time shift,
// the anti-periodic boundary sign and the "psi -" in the epilogue, so psi is read once and out written once.
// The GEMM rows are the (r, t) pairs, the columns the output site x and the reduction runs over the input site y:
//   Z[(r,t), x] = sum_y Y[(r,t), y] E[x, y].
// expK is real whenever delta and the hopping matrix are real (honeycomb, ring with real kappa); the kernel then
// does a complex-by-real product (2 real FMAs per term instead of 4).
//
// The diagonal discretisation (HubbardDiag, hubbardDiag.tpp:10-71) uses the same GEMM with E = sgn delta K on the
// unshifted slice and adds its phase term element-wise in the epilogue:
//   M:    out[r, t] = psi[r, t] - (sgn delta K psi[r, t]) - B_t phase[t-1] psi[r, t-1]               (B_0 = -1)
//   Mdag: out[r, t] = psi[r, t] - (sgn delta* K psi[r, t]) - conj(phase[t]) B'_t psi[r, t+1]     (B'_{Nt-1} = -1)
//
// A system mask (sys_mask, sys_rows consecutive rows per system) lets whole tiles of unflagged systems return at once:
// the reliable updates of a batched CG evaluate b - A x only for the systems that asked for one.
//
// Vectors are FP64 (Tio = double) in both forms. Tc = double is the FP64 drop-in (DFMA); Tc = float is the FP32
// operator of the mixed-precision solver (FFMA): psi is rounded to FP32 in the operand load, the product runs in FP32
// and the epilogue forms psi - s * z in FP64.

#include "fm_internal.cuh"

namespace nslg {

namespace {

constexpr int BM = 64;   // complex rows (r, t) per CTA
constexpr int BN = 64;   // output sites x per CTA
constexpr int BK = 16;   // reduction sites y per stage
constexpr int NTHREADS = 256;

template <typename Tio, typename T, bool CE, int MODE>
__global__ void __launch_bounds__(NTHREADS) k_fm_apply(const cplx_t<Tio> *__restrict__ psi,
                                                       cplx_t<Tio> *__restrict__ out,
                                                       const cplx_t<T> *__restrict__ phase,
                                                       const T *__restrict__ Ere, const T *__restrict__ Eim, int Nt,
                                                       int Nx, int64_t rows, const int *__restrict__ sys_mask,
                                                       int64_t sys_rows) {
    using C = cplx_t<T>;
    using Cio = cplx_t<Tio>;
    __shared__ C As[BK][BM + 1];
    __shared__ T Bs[BK][BN + 1];
    __shared__ T Bsi[CE ? BK : 1][BN + 1];

    const int tid = threadIdx.x;
    const int tx = tid % 16, ty = tid / 16;
    const int64_t m0 = (int64_t)blockIdx.x * BM;
    const int n0 = blockIdx.y * BN;
    if (sys_mask) {  // no row of this tile belongs to a flagged system: nothing to compute
        bool any = false;
        const int64_t last = min(rows, m0 + BM) - 1;
        for (int64_t s = m0 / sys_rows; s <= last / sys_rows; ++s) any |= sys_mask[s] != 0;
        if (!any) return;
    }

    C acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = cmake<C>(0, 0);

    for (int k0 = 0; k0 < Nx; k0 += BK) {
        // operand tile: 64 rows x 16 sites, 4 elements per thread, 16 consecutive threads read one row segment
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            const int idx = tid + l * NTHREADS;
            const int row = idx / BK, kk = idx % BK;
            const int64_t grow = m0 + row;
            const int y = k0 + kk;
            C v = cmake<C>(0, 0);
            if (grow < rows && y < Nx) {
                const Cio w = psi[grow * Nx + y];
                v.x = (T)w.x;
                v.y = (T)w.y;
                if (MODE == MODE_M) {  // the diagonal modes multiply psi by nothing before the GEMM
                    const int t = (int)(grow % Nt);
                    v = cmul(phase[(int64_t)t * Nx + y], v);
                }
            }
            As[kk][row] = v;
        }
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            const int idx = tid + l * NTHREADS;
            const int n = idx / BK, kk = idx % BK;
            const int x = n0 + n, y = k0 + kk;
            const bool ok = (x < Nx && y < Nx);
            Bs[kk][n] = ok ? Ere[(int64_t)x * Nx + y] : T(0);
            if (CE) Bsi[kk][n] = ok ? Eim[(int64_t)x * Nx + y] : T(0);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            C a[4];
            T b[4], bi[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                b[j] = Bs[kk][tx + 16 * j];
                if (CE) bi[j] = Bsi[kk][tx + 16 * j];
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    acc[i][j].x = fma(a[i].x, b[j], acc[i][j].x);
                    acc[i][j].y = fma(a[i].y, b[j], acc[i][j].y);
                    if (CE) {
                        acc[i][j].x = fma(-a[i].y, bi[j], acc[i][j].x);
                        acc[i][j].y = fma(a[i].x, bi[j], acc[i][j].y);
                    }
                }
        }
        __syncthreads();
    }

    // epilogue: time shift, boundary sign, phase (Mdag) and psi - .
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int64_t grow = m0 + ty + 16 * i;
        if (grow >= rows) continue;
        const int64_t r = grow / Nt;
        const int t = (int)(grow - r * Nt);
        int to;
        Tio s;
        if (MODE == MODE_M) {
            to = (t + 1 == Nt) ? 0 : t + 1;
            s = (to == 0) ? Tio(-1) : Tio(1);
        } else if (MODE == MODE_MDAG) {
            to = (t == 0) ? Nt - 1 : t - 1;
            s = (t == 0) ? Tio(-1) : Tio(1);
        } else {  // diagonal modes: the GEMM stays on its slice
            to = t;
            s = Tio(1);
        }
        const int64_t orow = (r * Nt + to) * Nx;
        // diagonal modes: the neighbouring slice of the element-wise phase term and its boundary sign
        const int tn = (MODE == MODE_DIAG_M) ? (t == 0 ? Nt - 1 : t - 1) : (t + 1 == Nt ? 0 : t + 1);
        const Tio sn = (MODE == MODE_DIAG_M) ? (t == 0 ? Tio(-1) : Tio(1)) : (t + 1 == Nt ? Tio(-1) : Tio(1));
        const int64_t nrow = (r * Nt + tn) * Nx;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int x = n0 + tx + 16 * j;
            if (x >= Nx) continue;
            C z = acc[i][j];
            if (MODE == MODE_MDAG) z = cmulc(phase[(int64_t)to * Nx + x], z);
            const Cio p = psi[orow + x];
            Cio o;
            o.x = p.x - s * (Tio)z.x;
            o.y = p.y - s * (Tio)z.y;
            if (MODE == MODE_DIAG_M || MODE == MODE_DIAG_MDAG) {
                const Cio q = psi[nrow + x];
                const C ph = phase[(int64_t)(MODE == MODE_DIAG_M ? tn : t) * Nx + x];
                const Tio phx = (Tio)ph.x, phy = (MODE == MODE_DIAG_M) ? (Tio)ph.y : -(Tio)ph.y;  // phase or conj
                o.x -= sn * (phx * q.x - phy * q.y);
                o.y -= sn * (phx * q.y + phy * q.x);
            }
            out[orow + x] = o;
        }
    }
}

template <typename T, bool CE>
int launch_mode(int mode, const double2 *psi, double2 *out, const cplx_t<T> *phase, const T *Ere, const T *Eim,
                int Nt, int Nx, int64_t rows, cudaStream_t st, const int *mask, int64_t sys_rows) {
    dim3 grid((unsigned)ceil_div(rows, BM), (unsigned)ceil_div(Nx, BN));
    if (mode == MODE_M)
        k_fm_apply<double, T, CE, MODE_M><<<grid, NTHREADS, 0, st>>>(psi, out, phase, Ere, Eim, Nt, Nx, rows, mask,
                                                                     sys_rows);
    else if (mode == MODE_MDAG)
        k_fm_apply<double, T, CE, MODE_MDAG><<<grid, NTHREADS, 0, st>>>(psi, out, phase, Ere, Eim, Nt, Nx, rows, mask,
                                                                        sys_rows);
    else if (mode == MODE_DIAG_M)
        k_fm_apply<double, T, CE, MODE_DIAG_M><<<grid, NTHREADS, 0, st>>>(psi, out, phase, Ere, Eim, Nt, Nx, rows,
                                                                          mask, sys_rows);
    else
        k_fm_apply<double, T, CE, MODE_DIAG_MDAG><<<grid, NTHREADS, 0, st>>>(psi, out, phase, Ere, Eim, Nt, Nx,
                                                                             rows, mask, sys_rows);
    note_launch(st);
    NSLG_CUDA(cudaGetLastError());
    return NSLG_OK;
}

}  // namespace

template <typename T>
int fm_apply_simt(int mode, const double2 *psi, double2 *out, const cplx_t<T> *phase, const T *Ere, const T *Eim,
                  int Nt, int Nx, int64_t rows, cudaStream_t st, const int *sys_mask, int64_t sys_rows) {
    if (rows == 0) return NSLG_OK;
    NSLG_REQUIRE(!sys_mask || sys_rows >= 1, NSLG_ERR_ARG, "operator row mask: rows per system must be positive");
    if (Eim) return launch_mode<T, true>(mode, psi, out, phase, Ere, Eim, Nt, Nx, rows, st, sys_mask, sys_rows);
    return launch_mode<T, false>(mode, psi, out, phase, Ere, nullptr, Nt, Nx, rows, st, sys_mask, sys_rows);
}

template int fm_apply_simt<double>(int, const double2 *, double2 *, const double2 *, const double *, const double *,
                                   int, int, int64_t, cudaStream_t, const int *, int64_t);
template int fm_apply_simt<float>(int, const double2 *, double2 *, const float2 *, const float *, const float *,
                                  int, int, int64_t, cudaStream_t, const int *, int64_t);

}  // namespace nslg
