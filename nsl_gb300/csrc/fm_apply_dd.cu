// M psi and M^dagger psi in double-double arithmetic, for residuals that FP64 cannot resolve.
//
// At low temperature the CG solutions of M M^dagger x = b have |A| |x| / |b| ~ 1e7..1e8, so rounding x to FP64 alone
// moves b - A x by ~1e-9 |b|, and evaluating A x in FP64 adds as much again: a true residual of 1e-10 can neither be
// held nor certified in FP64. Here vectors are unevaluated sums hi + lo of two FP64 numbers (~32 significant
// digits) and the operator (hubbardExp.tpp:13-75 with the FP64 exp(delta K) and phases of the handle) is applied with
// error-free transformations: products by FMA (a b = p + e exactly, e = fma(a, b, -p)), sums by Knuth's two-sum
// (Dekker 1971; Knuth, TAOCP vol. 2, 4.2.2), so A (x_hi + x_lo) is exact to ~1e-30 relative to |A| |x|.
//
// Layout and tiling follow the FP64 CUDA-core kernel (fm_apply.cu): GEMM rows are the (right-hand side, time slice)
// pairs, columns the output sites, the reduction runs over the input sites with the phase multiply in the operand
// load and the time shift, boundary sign, conj(phase) (M^dagger) and "psi -" in the epilogue. A row mask skips the
// right-hand sides that do not need a residual (the CG evaluates it only for systems due an update).

#include "fm_internal.cuh"

namespace nslg {

namespace {

struct dd {
    double hi, lo;
};

__device__ __forceinline__ dd two_sum(double a, double b) {
    const double s = a + b;
    const double bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ dd fast_two_sum(double a, double b) {  // |a| >= |b|
    const double s = a + b;
    return {s, b - (s - a)};
}
// a + b, both double-double (the sum of the high parts exactly, the low parts added in FP64, renormalised)
__device__ __forceinline__ dd dd_add(dd a, dd b) {
    dd s = two_sum(a.hi, b.hi);
    s.lo += a.lo + b.lo;
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ dd dd_neg(dd a) { return {-a.hi, -a.lo}; }
// a * b with b an FP64 number: the product of the high part exactly (FMA), the low part's in FP64
__device__ __forceinline__ dd dd_mul_d(dd a, double b) {
    const double p = a.hi * b;
    const double e = fma(a.hi, b, -p);
    return fast_two_sum(p, fma(a.lo, b, e));
}

struct ddc {
    dd re, im;
};
// (a_r + i a_i) * v with a FP64 complex, v double-double complex
__device__ __forceinline__ ddc cmul_d(double2 a, ddc v) {
    return {dd_add(dd_mul_d(v.re, a.x), dd_neg(dd_mul_d(v.im, a.y))), dd_add(dd_mul_d(v.im, a.x), dd_mul_d(v.re, a.y))};
}
// conj(a) * v
__device__ __forceinline__ ddc cmulc_d(double2 a, ddc v) {
    return {dd_add(dd_mul_d(v.re, a.x), dd_mul_d(v.im, a.y)), dd_add(dd_mul_d(v.im, a.x), dd_neg(dd_mul_d(v.re, a.y)))};
}

constexpr int DBM = 32;  // complex rows per CTA
constexpr int DBN = 32;  // output sites per CTA
constexpr int DBK = 16;  // reduction sites per stage
constexpr int DNT = 256; // 16 x 16 threads, 2 x 2 outputs each

// MODE_M / MODE_MDAG of the exponential discretisation, double-double. CE: complex exp(delta K).
template <bool CE, int MODE>
__global__ void __launch_bounds__(DNT) k_fm_apply_dd(const double2 *__restrict__ xh, const double2 *__restrict__ xl,
                                                    double2 *__restrict__ oh, double2 *__restrict__ ol,
                                                    const double2 *__restrict__ phase, const double *__restrict__ Ere,
                                                    const double *__restrict__ Eim, int Nt, int Nx, int64_t rows,
                                                    const int *__restrict__ sys_mask, int64_t sys_rows) {
    __shared__ ddc As[DBK][DBM + 1];
    __shared__ double Bs[DBK][DBN + 1];
    __shared__ double Bsi[CE ? DBK : 1][DBN + 1];
    const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
    const int64_t m0 = (int64_t)blockIdx.x * DBM;
    const int n0 = blockIdx.y * DBN;
    if (sys_mask) {  // every row of this tile belongs to systems without an update: nothing to do
        bool any = false;
        const int64_t last = min(rows, m0 + DBM) - 1;
        for (int64_t s = m0 / sys_rows; s <= last / sys_rows; ++s) any |= sys_mask[s] != 0;
        if (!any) return;
    }
    ddc acc[2][2];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) acc[i][j] = {{0, 0}, {0, 0}};

    for (int k0 = 0; k0 < Nx; k0 += DBK) {
        // operand tile: 32 rows x 16 sites, two per thread
#pragma unroll
        for (int l = 0; l < 2; ++l) {
            const int idx = tid + l * DNT;
            const int row = idx / DBK, kk = idx % DBK;
            const int64_t grow = m0 + row;
            const int y = k0 + kk;
            ddc v = {{0, 0}, {0, 0}};
            if (grow < rows && y < Nx) {
                const double2 h = xh[grow * Nx + y], lo = xl[grow * Nx + y];
                v = {fast_two_sum(h.x, lo.x), fast_two_sum(h.y, lo.y)};
                if (MODE == MODE_M) {
                    const int t = (int)(grow % Nt);
                    v = cmul_d(phase[(int64_t)t * Nx + y], v);
                }
            }
            As[kk][row] = v;
        }
        for (int idx = tid; idx < DBN * DBK; idx += DNT) {
            const int n = idx / DBK, kk = idx % DBK;
            const int x = n0 + n, y = k0 + kk;
            const bool ok = (x < Nx && y < Nx);
            Bs[kk][n] = ok ? Ere[(int64_t)x * Nx + y] : 0.0;
            if (CE) Bsi[kk][n] = ok ? Eim[(int64_t)x * Nx + y] : 0.0;
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < DBK; ++kk) {
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const ddc a = As[kk][ty + 16 * i];
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    const double b = Bs[kk][tx + 16 * j];
                    acc[i][j].re = dd_add(acc[i][j].re, dd_mul_d(a.re, b));
                    acc[i][j].im = dd_add(acc[i][j].im, dd_mul_d(a.im, b));
                    if (CE) {
                        const double bi = Bsi[kk][tx + 16 * j];
                        acc[i][j].re = dd_add(acc[i][j].re, dd_neg(dd_mul_d(a.im, bi)));
                        acc[i][j].im = dd_add(acc[i][j].im, dd_mul_d(a.re, bi));
                    }
                }
            }
        }
        __syncthreads();
    }
    // epilogue: time shift, boundary sign, conj(phase) (M^dagger), psi - s z
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const int64_t grow = m0 + ty + 16 * i;
        if (grow >= rows) continue;
        if (sys_mask && !sys_mask[grow / sys_rows]) continue;
        const int64_t r = grow / Nt;
        const int t = (int)(grow - r * Nt);
        int to;
        bool neg;  // s = -1 on the wrapped slice
        if (MODE == MODE_M) {
            to = (t + 1 == Nt) ? 0 : t + 1;
            neg = to == 0;
        } else {
            to = (t == 0) ? Nt - 1 : t - 1;
            neg = t == 0;
        }
        const int64_t orow = (r * Nt + to) * Nx;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int x = n0 + tx + 16 * j;
            if (x >= Nx) continue;
            ddc z = acc[i][j];
            if (MODE == MODE_MDAG) z = cmulc_d(phase[(int64_t)to * Nx + x], z);
            const double2 ph = xh[orow + x], pl = xl[orow + x];
            const dd pr = fast_two_sum(ph.x, pl.x), pi = fast_two_sum(ph.y, pl.y);
            const dd ore = neg ? dd_add(pr, z.re) : dd_add(pr, dd_neg(z.re));
            const dd oim = neg ? dd_add(pi, z.im) : dd_add(pi, dd_neg(z.im));
            oh[orow + x] = make_double2(ore.hi, oim.hi);
            ol[orow + x] = make_double2(ore.lo, oim.lo);
        }
    }
}

int launch_dd(int mode, const double2 *xh, const double2 *xl, double2 *oh, double2 *ol, const double2 *phase,
              const ExpEntry *e, int Nt, int Nx, int64_t rows, const int *sys_mask, int64_t sys_rows,
              cudaStream_t st) {
    const dim3 grid((unsigned)ceil_div(rows, DBM), (unsigned)ceil_div(Nx, DBN));
    const bool ce = !e->is_real;
    if (mode == MODE_M) {
        if (ce) k_fm_apply_dd<true, MODE_M><<<grid, DNT, 0, st>>>(xh, xl, oh, ol, phase, e->re, e->im, Nt, Nx, rows,
                                                                  sys_mask, sys_rows);
        else k_fm_apply_dd<false, MODE_M><<<grid, DNT, 0, st>>>(xh, xl, oh, ol, phase, e->re, nullptr, Nt, Nx, rows,
                                                                sys_mask, sys_rows);
    } else {
        if (ce) k_fm_apply_dd<true, MODE_MDAG><<<grid, DNT, 0, st>>>(xh, xl, oh, ol, phase, e->re, e->im, Nt, Nx,
                                                                     rows, sys_mask, sys_rows);
        else k_fm_apply_dd<false, MODE_MDAG><<<grid, DNT, 0, st>>>(xh, xl, oh, ol, phase, e->re, nullptr, Nt, Nx,
                                                                   rows, sys_mask, sys_rows);
    }
    note_launch(st);
    NSLG_CUDA(cudaGetLastError());
    return NSLG_OK;
}

}  // namespace

// (oh + ol) = op (xh + xl) in double-double for op in {M, M^dagger, M M^dagger, M^dagger M} (exponential
// discretisation), vectors (nbatch, Nt, Nx); with sys_mask, only the rows of systems s (sys_rows consecutive rows
// each) with sys_mask[s] != 0 are written.
int fm_apply_dd(nslg_fm *fm, int op, const double2 *xh, const double2 *xl, double2 *oh, double2 *ol, int64_t nbatch,
                const int *sys_mask, int64_t sys_rows) {
    NSLG_REQUIRE(fm->kind == NSLG_FM_EXP, NSLG_ERR_UNSUPPORTED,
                 "double-double residuals are implemented for the exponential discretisation");
    NSLG_REQUIRE(fm->populated, NSLG_ERR_STATE, "the fermion matrix has no configuration (call populate first)");
    cudaStream_t st = fm->ctx->stream;
    const int Nt = (int)fm->Nt, Nx = (int)fm->Nx;
    const int64_t rows = nbatch * fm->Nt;
    const double2 d = make_double2(fm->sgn * fm->delta.x, fm->sgn * fm->delta.y);
    const double2 dc = make_double2(fm->sgn * fm->delta.x, -fm->sgn * fm->delta.y);
    const ExpEntry *E = nullptr, *Ec = nullptr;
    if (op != NSLG_OP_MDAGGER) NSLG_TRY(get_exp(fm, d, &E));
    if (op != NSLG_OP_M) NSLG_TRY(get_exp(fm, dc, &Ec));
    if (!sys_mask) sys_rows = rows;
    switch (op) {
        case NSLG_OP_M: return launch_dd(MODE_M, xh, xl, oh, ol, fm->phase, E, Nt, Nx, rows, sys_mask, sys_rows, st);
        case NSLG_OP_MDAGGER:
            return launch_dd(MODE_MDAG, xh, xl, oh, ol, fm->phase, Ec, Nt, Nx, rows, sys_mask, sys_rows, st);
        default: break;
    }
    double2 *th, *tl;
    NSLG_TRY(ws_get(fm, "dd_tmp_h", rows * Nx, &th));
    NSLG_TRY(ws_get(fm, "dd_tmp_l", rows * Nx, &tl));
    if (op == NSLG_OP_MMDAGGER) {
        NSLG_TRY(launch_dd(MODE_MDAG, xh, xl, th, tl, fm->phase, Ec, Nt, Nx, rows, sys_mask, sys_rows, st));
        return launch_dd(MODE_M, th, tl, oh, ol, fm->phase, E, Nt, Nx, rows, sys_mask, sys_rows, st);
    }
    NSLG_TRY(launch_dd(MODE_M, xh, xl, th, tl, fm->phase, E, Nt, Nx, rows, sys_mask, sys_rows, st));
    return launch_dd(MODE_MDAG, th, tl, oh, ol, fm->phase, Ec, Nt, Nx, rows, sys_mask, sys_rows, st);
}

}  // namespace nslg
