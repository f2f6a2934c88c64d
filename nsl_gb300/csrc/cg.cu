// Conjugate gradient on the fermion operators, batched, with device-resident scalars.
//
// Restates src/NSL/LinAlg/Solver/Impl/CG.tpp:15-113 (x0 = b, alpha = |r|^2 / <p, A p>, stop when the recurrence
// |r|^2 <= eps^2, return x on exhaustion) for many systems at once. All scalars live on the device; an iteration is
//   apply (t = A p)  ->  k_dot (<p, t> partials)  ->  k_cg_xr (alpha; x += alpha p; r -= alpha t; |r|^2 partials)
//                    ->  k_cg_p (beta; p = r + beta p; convergence / exhaustion / reliable-update flags)
// and a chunk of iterations is captured once into a CUDA graph and replayed; the host reads the per-system
// status only between chunks. Each block re-sums the (few) partials it needs in a fixed order, so the reductions
// are deterministic and need no grid-wide barrier. With the split-BF16 operator on MM^dagger / M^dagger M the dot
// products and the r update move into the operator's epilogues (cg_iteration_fused): four kernels per iteration.
//
// Batch semantics: SHARED mode is the reference's (one CG over all right-hand sides with alpha/beta summed over the
// whole batch, inner_product.tpp:30-33), implemented as a single system of length nbatch*Nt*Nx; PER_RHS runs nbatch
// independent systems, each masked out once it has converged.
//
// Vectors x, r, p, t are FP64 in every form; the operator's products run in FP64 (the drop-in), FP32 or 3xTF32
// (FP32-class) or split-BF16 (FP64-class, tensor cores). With the true-residual stopping rule or a mixed precision
// the solver does FP64 reliable updates: when a system's recurrence |r|^2 has fallen 100x below its running
// maximum since the last update (or reached the target), the true residual r = b - A x is recomputed with the FP64
// operator and replaces that system's recurrence residual (the search direction is kept); the system stops when
// the true |r| <= eps. FP32-class operators also get periodic updates and stall detection with escalation to the
// FP64 operator; FP64-class systems stop, unconverged, once their true residual no longer improves (the accuracy
// FP64 can certify). Keeping the vectors in FP64 is what lets the low-precision operators reach that accuracy.

#include <algorithm>
#include <mutex>
#include <set>
#include <type_traits>
#include <typeinfo>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "fm_internal.cuh"
#include "oz_digits.cuh"

namespace nslg {

namespace {

struct CgState {
    double rsq;   // |r|^2 of the current recurrence residual (kept at its pre-trigger value during an update)
    double maxr;  // largest |r|^2 since the last reliable update
    double tgt;   // recurrence |r|^2 that hands over to a reliable update (starts at eps^2, shrinks if it was early)
    double trig;  // recurrence |r|^2 that triggered the pending update
    double best;  // smallest true |r|^2 seen at a reliable update
    int status;
    int iters;
    int last_upd;  // iteration of the last reliable update
    int stall;     // consecutive reliable updates without a 4x gain in the true |r|^2
    double base;   // |b_seg|^2: the residual of the double-double solution at the last rebase (double-double rule)
    double eps2;   // the system's target |r|^2 (eps^2 of its fermion matrix)
};
// CG_STALLED: the low-precision operator has stopped reducing this system's true residual; it waits until every
// running system is stalled or done, then the batch continues with the FP64 operator.
// CG_REBASE (double-double rule): the system's FP64 increment is folded into its double-double solution and its
// residual recomputed in double-double before it continues or stops.
// CG_RESIDENT: the system is being solved by the resident kernel (cg_resident.cuh), which keeps its own copy of the
// state; the launch-per-step kernels leave it alone until the state is handed back.
enum { CG_ACTIVE = 0, CG_CONVERGED = 1, CG_EXHAUSTED = 2, CG_UPDATE = 3, CG_STALLED = 4, CG_REBASE = 5,
       CG_RESIDENT = 6 };
constexpr int UPDATE_EVERY = 1000;  // forced reliable update after this many iterations without one
constexpr int STALL_LIMIT = 3;      // updates without progress before a system is stalled
// FP64-class operators: after this many reliable updates without a 4x gain in the true |r|^2 the system has reached
// the accuracy FP64 can certify (the rounding of b - A x itself) and stops unconverged instead of iterating on.
constexpr int FLOOR_LIMIT = 4;

constexpr int RT = 256;  // threads of the vector kernels

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum, result valid in every thread.
__device__ double block_sum(double v) {
    __shared__ double sh[RT / 32];
    __shared__ double total;
    v = warp_sum(v);
    const int w = threadIdx.x / 32, l = threadIdx.x % 32;
    if (l == 0) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        double u = (l < RT / 32) ? sh[l] : 0.0;
        u = warp_sum(u);
        if (l == 0) total = u;
    }
    __syncthreads();
    const double out = total;
    __syncthreads();
    return out;
}

__device__ __forceinline__ double2 block_sum2(double2 v) {
    double2 o;
    o.x = block_sum(v.x);
    o.y = block_sum(v.y);
    return o;
}

// Sum of partial[0..nblk) in a fixed order (deterministic), by warp 0 only: GB300 runs FP64 at ~2 operations per
// clock per SM, so the scalar work of a CG step is kept out of the other warps. Valid in lanes of warp 0.
__device__ __forceinline__ double warp0_sum_partials(const double *partial, int nblk) {
    double v = 0;
    for (int i = threadIdx.x; i < nblk; i += 32) v += partial[i];
    return warp_sum(v);
}
__device__ __forceinline__ double2 warp0_sum_partials2(const double2 *partial, int nblk) {
    double2 v = make_double2(0, 0);
    for (int i = threadIdx.x; i < nblk; i += 32) {
        v.x += partial[i].x;
        v.y += partial[i].y;
    }
    v.x = warp_sum(v.x);
    v.y = warp_sum(v.y);
    return v;
}

// Sum of partial[0..nblk) broadcast to every thread of the block.
__device__ double sum_partials(const double *partial, int nblk) {
    __shared__ double sh;
    if (threadIdx.x < 32) {
        const double v = warp0_sum_partials(partial, nblk);
        if (threadIdx.x == 0) sh = v;
    }
    __syncthreads();
    return sh;
}

__device__ __forceinline__ void chunk_range(int64_t n, int nblk, int blk, int64_t &lo, int64_t &hi) {
    const int64_t c = (n + nblk - 1) / nblk;
    lo = (int64_t)blk * c;
    hi = min(n, lo + c);
}

// The systems of a solve: system s is the contiguous range [off_s, off_s + len_s) of every vector. Equal systems
// (one fermion matrix) have off_s = s n and len_s = n (off and len null); a group of fermion matrices of different
// sizes solved together gives each instance's right-hand sides their own lengths through the tables.
struct Sys {
    int64_t n = 0;
    const int64_t *off = nullptr;
    const int64_t *len = nullptr;
    // block blk of nblk's share [o + lo, o + hi) of system s
    __device__ __forceinline__ void range(int s, int nblk, int blk, int64_t &o, int64_t &lo, int64_t &hi) const {
        o = off ? off[s] : (int64_t)s * n;
        chunk_range(len ? len[s] : n, nblk, blk, lo, hi);
    }
};

// partial[s, blk] = sum conj(a) b over the block's chunk of system s
__global__ void __launch_bounds__(RT) k_dot(const double2 *__restrict__ a, const double2 *__restrict__ b, Sys sy,
                                            int nblk, double2 *__restrict__ partial, const CgState *__restrict__ st) {
    const int s = blockIdx.y, blk = blockIdx.x;
    if (st && st[s].status != CG_ACTIVE) return;
    int64_t lo, hi;
    int64_t o;
    sy.range(s, nblk, blk, o, lo, hi);
    a += o;
    b += o;
    double2 acc = make_double2(0, 0);
    for (int64_t i = lo + threadIdx.x; i < hi; i += RT) {
        const double2 x = a[i], y = b[i];
        acc.x += x.x * y.x + x.y * y.y;
        acc.y += x.x * y.y - x.y * y.x;
    }
    acc = block_sum2(acc);
    if (threadIdx.x == 0) partial[(int64_t)s * nblk + blk] = acc;
}

// alpha = rsq / <p, t>;  x += alpha p;  r -= alpha t;  partial |r|^2
__global__ void __launch_bounds__(RT) k_cg_xr(double2 *__restrict__ x, double2 *__restrict__ r,
                                              const double2 *__restrict__ p, const double2 *__restrict__ t, Sys sy,
                                              int nblk, const double2 *__restrict__ p_pt,
                                              const CgState *__restrict__ st, double *__restrict__ p_rr) {
    const int s = blockIdx.y, blk = blockIdx.x;
    const CgState S = st[s];
    if (S.status != CG_ACTIVE) return;
    __shared__ double2 alpha;
    if (threadIdx.x < 32) {
        const double2 pt = warp0_sum_partials2(p_pt + (int64_t)s * nblk, nblk);
        if (threadIdx.x == 0) {
            const double den = pt.x * pt.x + pt.y * pt.y;
            alpha = make_double2(S.rsq * pt.x / den, -S.rsq * pt.y / den);
        }
    }
    __syncthreads();
    const double ar = alpha.x, ai = alpha.y;
    int64_t lo, hi;
    int64_t off;
    sy.range(s, nblk, blk, off, lo, hi);
    double acc = 0;
    for (int64_t i = off + lo + threadIdx.x; i < off + hi; i += RT) {
        const double2 pv = p[i], tv = t[i];
        double2 xv = x[i], rv = r[i];
        xv.x += ar * pv.x - ai * pv.y;
        xv.y += ar * pv.y + ai * pv.x;
        rv.x -= ar * tv.x - ai * tv.y;
        rv.y -= ar * tv.y + ai * tv.x;
        x[i] = xv;
        r[i] = rv;
        acc += rv.x * rv.x + rv.y * rv.y;
    }
    acc = block_sum(acc);
    if (threadIdx.x == 0) p_rr[(int64_t)s * nblk + blk] = acc;
}

// The state after an iteration whose recurrence |r|^2 is rn (beta set when the system runs on):
// reliable == 0: the reference's rule, converged when |r|^2 <= errSq (CG.tpp:70).
// reliable == 1: hand over to a reliable update when |r|^2 < update_frac * maxr or |r|^2 <= tgt;
// reliable == 2: also after UPDATE_EVERY iterations without one (FP32-class operators: stall detection).
__device__ __forceinline__ CgState cg_next_state(const CgState &S, double rn, int64_t max_iter, int reliable,
                                                 double update_frac, double &beta) {
    CgState N = S;
    N.iters = S.iters + 1;
    if (!reliable) {
        if (rn <= S.eps2) N.status = CG_CONVERGED;
        else if (N.iters >= max_iter) N.status = CG_EXHAUSTED;
    } else if (rn <= S.tgt || rn < update_frac * S.maxr || N.iters >= max_iter ||
               (reliable == 2 && N.iters - S.last_upd >= UPDATE_EVERY)) {
        N.status = CG_UPDATE;
        N.trig = rn;
    }
    if (N.status == CG_ACTIVE) {
        beta = rn / S.rsq;
        N.rsq = rn;
        N.maxr = fmax(S.maxr, rn);
    }
    return N;
}

// beta = |r_new|^2 / |r_old|^2; p = r + beta p; status update (cg_next_state). st_in and st_out are different buffers.
// With x_alpha (fused split-BF16 iteration) the same pass also applies x += alpha[s] p with the p of this iteration.
// With go, also go[s] = (the system runs the next iteration): the fused iteration's kernels skip the others.
__global__ void __launch_bounds__(RT) k_cg_p(const double2 *__restrict__ r, double2 *__restrict__ p,
                                             double2 *__restrict__ x, const double *__restrict__ x_alpha, Sys sy,
                                             int nblk, const double *__restrict__ p_rr, int npart,
                                             const CgState *__restrict__ st_in, CgState *__restrict__ st_out,
                                             double errSq, int64_t max_iter, int reliable, double update_frac,
                                             int *__restrict__ go) {
    const int s = blockIdx.y, blk = blockIdx.x;
    const CgState S = st_in[s];
    if (S.status != CG_ACTIVE) {
        if (blk == 0 && threadIdx.x == 0) {
            st_out[s] = S;
            if (go) go[s] = 0;
        }
        return;
    }
    __shared__ CgState Nsh;
    __shared__ double beta_sh;
    if (threadIdx.x < 32) {
        const double rn = warp0_sum_partials(p_rr + (int64_t)s * npart, npart);
        if (threadIdx.x == 0) Nsh = cg_next_state(S, rn, max_iter, reliable, update_frac, beta_sh);
    }
    __syncthreads();
    const CgState N = Nsh;
    int64_t lo, hi;
    int64_t off;
    sy.range(s, nblk, blk, off, lo, hi);
    if (x_alpha) {  // the system ran this iteration (it was ACTIVE): x += alpha p, then p as below
        const double alpha = x_alpha[s];
        const bool next = N.status == CG_ACTIVE;
        const double beta = next ? beta_sh : 0.0;
        for (int64_t i = off + lo + threadIdx.x; i < off + hi; i += RT) {
            double2 pv = p[i];
            double2 xv = x[i];
            xv.x = fma(alpha, pv.x, xv.x);
            xv.y = fma(alpha, pv.y, xv.y);
            x[i] = xv;
            if (next) {
                const double2 rv = r[i];
                pv.x = rv.x + beta * pv.x;
                pv.y = rv.y + beta * pv.y;
                p[i] = pv;
            }
        }
    } else if (N.status == CG_ACTIVE) {
        const double beta = beta_sh;
        for (int64_t i = off + lo + threadIdx.x; i < off + hi; i += RT) {
            const double2 rv = r[i];
            double2 pv = p[i];
            pv.x = rv.x + beta * pv.x;
            pv.y = rv.y + beta * pv.y;
            p[i] = pv;
        }
    }
    if (blk == 0 && threadIdx.x == 0) {
        st_out[s] = N;
        if (go) go[s] = N.status == CG_ACTIVE;
    }
}

// The fused split-BF16 iteration on M M^dagger: k_cg_p's update (beta, state, x += alpha p, p = r + beta p) one warp
// per complex row of Nx sites (a block's rows belong to one system of rows_per_sys rows), which also writes the digit
// planes and row scales of the new p for the next iteration's first factor M^dagger p, whose own digit pre-pass is
// then skipped. Systems that do not run the next iteration write no digits (the operator skips their rows).
__global__ void __launch_bounds__(RT) k_cg_p_oz(const double2 *__restrict__ r, double2 *__restrict__ p,
                                                double2 *__restrict__ x, const double *__restrict__ x_alpha, int Nx,
                                                int rows_per_sys, const double *__restrict__ p_rr, int npart,
                                                const CgState *__restrict__ st_in, CgState *__restrict__ st_out,
                                                int64_t max_iter, int reliable, double update_frac,
                                                int *__restrict__ go, __nv_bfloat16 *__restrict__ planes, int *__restrict__ rexp, int ld,
                                                int64_t rows) {
    constexpr int WPB = RT / 32;
    const int s = blockIdx.y, lane = threadIdx.x % 32, w = threadIdx.x / 32;
    const CgState S = st_in[s];
    if (S.status != CG_ACTIVE) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            st_out[s] = S;
            go[s] = 0;
        }
        return;
    }
    __shared__ CgState Nsh;
    __shared__ double beta_sh;
    if (threadIdx.x < 32) {
        const double rn = warp0_sum_partials(p_rr + (int64_t)s * npart, npart);
        if (threadIdx.x == 0) Nsh = cg_next_state(S, rn, max_iter, reliable, update_frac, beta_sh);
    }
    __syncthreads();
    const CgState N = Nsh;
    const bool next = N.status == CG_ACTIVE;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st_out[s] = N;
        go[s] = next;
    }
    const int lrow = blockIdx.x * WPB + w;
    if (lrow >= rows_per_sys) return;
    const int64_t grow = (int64_t)s * rows_per_sys + lrow;
    const double alpha = x_alpha[s], beta = next ? beta_sh : 0.0;
    double2 *pr = p + grow * Nx, *xr = x + grow * Nx;
    const double2 *rr = r + grow * Nx;
    constexpr int NP = OZ_CACHE / 2;  // site pairs kept in registers
    unsigned long long c[NP][4];
    unsigned long long mr = 0, mi = 0;
    auto step = [&](int y, unsigned long long (&b)[4]) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            b[2 * h] = b[2 * h + 1] = 0ull;
            if (y + h < Nx) {
                double2 pv = pr[y + h];
                double2 xv = xr[y + h];
                xv.x = fma(alpha, pv.x, xv.x);
                xv.y = fma(alpha, pv.y, xv.y);
                xr[y + h] = xv;
                if (next) {
                    const double2 rv = rr[y + h];
                    pv.x = fma(beta, pv.x, rv.x);
                    pv.y = fma(beta, pv.y, rv.y);
                    pr[y + h] = pv;
                    b[2 * h] = (unsigned long long)__double_as_longlong(pv.x);
                    b[2 * h + 1] = (unsigned long long)__double_as_longlong(pv.y);
                }
            }
        }
    };
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        step(2 * (lane + 32 * k), c[k]);
        mr = max(mr, max(c[k][0] & 0x7FFFFFFFFFFFFFFFull, c[k][2] & 0x7FFFFFFFFFFFFFFFull));
        mi = max(mi, max(c[k][1] & 0x7FFFFFFFFFFFFFFFull, c[k][3] & 0x7FFFFFFFFFFFFFFFull));
    }
    for (int y = 2 * (lane + 32 * NP); y < Nx; y += 64) {  // rows longer than the register cache
        unsigned long long b[4];
        step(y, b);
        mr = max(mr, max(b[0] & 0x7FFFFFFFFFFFFFFFull, b[2] & 0x7FFFFFFFFFFFFFFFull));
        mi = max(mi, max(b[1] & 0x7FFFFFFFFFFFFFFFull, b[3] & 0x7FFFFFFFFFFFFFFFull));
    }
    if (!next) return;  // warp-uniform
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mr = max(mr, __shfl_xor_sync(0xffffffffu, mr, o));
        mi = max(mi, __shfl_xor_sync(0xffffffffu, mi, o));
    }
    const int er = scale_exponent(mr), ei = scale_exponent(mi);
    if (lane == 0) {
        rexp[2 * grow] = er;
        rexp[2 * grow + 1] = ei;
    }
    const int64_t mreal = 2 * rows;
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        const int y = 2 * (lane + 32 * k);
        if (y < ld) write_digits2(planes, mreal, grow, ld, y, c[k], er, ei);
    }
    for (int y = 2 * (lane + 32 * NP); y < ld; y += 64) {
        unsigned long long b[4] = {0ull, 0ull, 0ull, 0ull};
#pragma unroll
        for (int h = 0; h < 2; ++h)
            if (y + h < Nx) {
                const double2 pv = pr[y + h];  // written by this thread above
                b[2 * h] = (unsigned long long)__double_as_longlong(pv.x);
                b[2 * h + 1] = (unsigned long long)__double_as_longlong(pv.y);
            }
        write_digits2(planes, mreal, grow, ld, y, b, er, ei);
    }
}

// go[s] = (system s runs): the first node of every captured chunk of the fused iteration, after the host's updates
__global__ void k_go_from_state(const CgState *__restrict__ st, int nsys, int *__restrict__ go) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < nsys) go[s] = st[s].status == CG_ACTIVE;
}

// Fused split-BF16 iteration: alpha = |r|^2 / |M^dagger p|^2 per running system from the npart curvature partial
// sums the first operator factor wrote (fixed summation order), and the activity flag the second factor reads.
__global__ void __launch_bounds__(RT) k_cg_alpha(const double *__restrict__ part, int npart,
                                                 const CgState *__restrict__ st, double *__restrict__ alpha,
                                                 int *__restrict__ active) {
    const int s = blockIdx.x;
    const CgState S = st[s];
    double v = 0;
    if (S.status == CG_ACTIVE)
        for (int i = threadIdx.x; i < npart; i += RT) v += part[(int64_t)s * npart + i];
    v = block_sum(v);
    if (threadIdx.x == 0) {
        active[s] = S.status == CG_ACTIVE;
        alpha[s] = S.status == CG_ACTIVE ? S.rsq / v : 0.0;
    }
}

// r = b - t and partial |r|^2, for every system (st == null) or only the systems due a reliable update (UPDATE: the
// update evaluates A x for those systems only).
__global__ void __launch_bounds__(RT) k_resid(const double2 *__restrict__ b, const double2 *__restrict__ t,
                                              double2 *__restrict__ r, Sys sy, int nblk,
                                              double *__restrict__ partial, const CgState *__restrict__ st) {
    const int s = blockIdx.y, blk = blockIdx.x;
    if (st && st[s].status != CG_UPDATE) return;
    int64_t lo, hi;
    int64_t off;
    sy.range(s, nblk, blk, off, lo, hi);
    double acc = 0;
    for (int64_t i = off + lo + threadIdx.x; i < off + hi; i += RT) {
        const double2 bv = b[i], tv = t[i];
        const double2 rv = make_double2(bv.x - tv.x, bv.y - tv.y);
        r[i] = rv;
        acc += rv.x * rv.x + rv.y * rv.y;
    }
    acc = block_sum(acc);
    if (threadIdx.x == 0) partial[(int64_t)s * nblk + blk] = acc;
}

// Initial state from the |r|^2 partials; p = r.
__global__ void __launch_bounds__(RT) k_start(const double2 *__restrict__ r, double2 *__restrict__ p, Sys sy,
                                              int nblk, const double *__restrict__ partial, CgState *__restrict__ st,
                                              double errSq, const double *__restrict__ eps2_sys, int64_t max_iter) {
    const int s = blockIdx.y, blk = blockIdx.x;
    const double rn = sum_partials(partial + (int64_t)s * nblk, nblk);
    int64_t lo, hi;
    int64_t off;
    sy.range(s, nblk, blk, off, lo, hi);
    for (int64_t i = off + lo + threadIdx.x; i < off + hi; i += RT) p[i] = r[i];
    if (blk == 0 && threadIdx.x == 0) {
        CgState S;
        S.rsq = rn;
        S.maxr = rn;
        S.tgt = errSq;
        S.trig = rn;
        S.best = rn;
        S.iters = 0;
        S.last_upd = 0;
        S.stall = 0;
        S.base = rn;
        S.eps2 = eps2_sys ? eps2_sys[s] : errSq;
        S.tgt = S.eps2;
        S.status = (rn <= S.eps2) ? CG_CONVERGED : (max_iter <= 0 ? CG_EXHAUSTED : CG_ACTIVE);
        st[s] = S;
    }
}

// Reliable update, second half. rt holds the true residual b - A x (FP64 operator) and partial its |rt|^2 for the
// systems that triggered the update (UPDATE, or REBASE under the double-double rule): each takes r = rt and
// converges, is exhausted, stalls or continues with p = r + beta p. Systems caught mid-recurrence (ACTIVE) are left
// untouched: replacing a residual after p = r + beta p was formed from the recurrence residual would break
// <r, p> = |r|^2, which alpha relies on, and made hard systems diverge.
// With dd (double-double rule) only a REBASE residual, evaluated in double-double, can certify convergence; a
// REBASE also starts a new FP64 segment (base, best and the stall count restart from its residual).
__global__ void __launch_bounds__(RT) k_rel_finish(double2 *__restrict__ r, const double2 *__restrict__ rt,
                                                   double2 *__restrict__ p, Sys sy, int nblk,
                                                   const double *__restrict__ partial,
                                                   const CgState *__restrict__ st_in, CgState *__restrict__ st_out,
                                                   double errSq, int64_t max_iter, int may_stall, int dd) {
    const int s = blockIdx.y, blk = blockIdx.x;
    const CgState S = st_in[s];
    if (S.status != CG_UPDATE && S.status != CG_REBASE) {
        if (blk == 0 && threadIdx.x == 0) st_out[s] = S;
        return;
    }
    const double rn = sum_partials(partial + (int64_t)s * nblk, nblk);
    CgState N = S;
    const bool rebase = S.status == CG_REBASE;
    const bool converged = rn <= S.eps2 && (!dd || rebase);
    int64_t lo, hi;
    int64_t off;
    sy.range(s, nblk, blk, off, lo, hi);
    N.rsq = rn;
    N.maxr = rn;
    N.last_upd = S.iters;
    if (rebase && rn < 0.25 * S.base) {  // a new segment: the FP64 floor restarts from this residual
        N.base = rn;
        N.best = rn;
        N.stall = 0;
    } else if (rn < 0.25 * S.best) {
        N.best = rn;
        N.stall = 0;
    } else {
        N.best = fmin(S.best, rn);
        N.stall = S.stall + 1;
    }
    if (rebase) N.base = rn;
    bool new_direction = false;
    if (converged) {
        N.status = CG_CONVERGED;
    } else if (S.iters >= max_iter) {
        N.status = CG_EXHAUSTED;
    } else if (may_stall && N.stall >= STALL_LIMIT) {
        N.status = CG_STALLED;  // p is reset when the system resumes
    } else if (!may_stall && N.stall >= FLOOR_LIMIT) {
        N.status = CG_EXHAUSTED;  // attainable accuracy reached: not converged, no further gain
    } else if (S.status == CG_UPDATE || rebase) {
        // the recurrence reached the target but the true residual did not: ask the recurrence for more next time
        if (S.trig <= S.tgt) N.tgt = 0.25 * S.tgt;
        new_direction = true;
        N.status = CG_ACTIVE;
    }
    const double beta = rn / S.rsq;
    for (int64_t i = off + lo + threadIdx.x; i < off + hi; i += RT) {
        const double2 rv = rt[i];
        r[i] = rv;
        if (new_direction) {
            double2 pv = p[i];
            pv.x = rv.x + beta * pv.x;
            pv.y = rv.y + beta * pv.y;
            p[i] = pv;
        }
    }
    if (blk == 0 && threadIdx.x == 0) st_out[s] = N;
}

// Escalation: stalled systems restart their direction (p = r) and run on with the FP64 operator.
__global__ void __launch_bounds__(RT) k_resume(const double2 *__restrict__ r, double2 *__restrict__ p, Sys sy,
                                               int nblk, CgState *__restrict__ st) {
    const int s = blockIdx.y, blk = blockIdx.x;
    const CgState S = st[s];
    if (S.status != CG_STALLED) return;
    int64_t lo, hi;
    int64_t off;
    sy.range(s, nblk, blk, off, lo, hi);
    for (int64_t i = off + lo + threadIdx.x; i < off + hi; i += RT) p[i] = r[i];
    __syncthreads();
    if (blk == 0 && threadIdx.x == 0) {
        CgState N = S;
        N.status = CG_ACTIVE;
        N.stall = 0;
        N.maxr = S.rsq;
        st[s] = N;
    }
}

// |v|^2 partials per system
__global__ void __launch_bounds__(RT) k_norm2(const double2 *__restrict__ v, Sys sy, int nblk,
                                              double *__restrict__ partial) {
    const int s = blockIdx.y, blk = blockIdx.x;
    int64_t lo, hi;
    int64_t off;
    sy.range(s, nblk, blk, off, lo, hi);
    double acc = 0;
    for (int64_t i = off + lo + threadIdx.x; i < off + hi; i += RT) acc += v[i].x * v[i].x + v[i].y * v[i].y;
    acc = block_sum(acc);
    if (threadIdx.x == 0) partial[(int64_t)s * nblk + blk] = acc;
}

// Double-double rule, after an FP64 reliable update: a system in UPDATE whose FP64 true |r|^2 has met the target,
// fallen below REBASE_FRAC of its segment's base, or stopped improving (the FP64 floor of its segment) is marked
// REBASE. One warp per system.
constexpr double REBASE_FRAC = 1e-10;  // |r| / |b_seg| = 1e-5: far above the ~1e-8 FP64 floor of a segment
__global__ void k_mark_rebase(const double *__restrict__ partial, int nblk, CgState *__restrict__ st, double errSq) {
    const int s = blockIdx.x;
    const double rn = warp0_sum_partials(partial + (int64_t)s * nblk, nblk);
    if (threadIdx.x != 0) return;
    CgState S = st[s];
    if (S.status != CG_UPDATE) return;
    const bool floor = !(rn < 0.25 * S.best) && S.stall >= 1;
    if (rn <= S.eps2 || rn <= REBASE_FRAC * S.base || floor) {
        S.status = CG_REBASE;
        st[s] = S;
    }
}

// flags[s] = 1 for the systems in `status`
__global__ void k_status_flags(const CgState *__restrict__ st, int nsys, int status, int *__restrict__ flags) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < nsys) flags[s] = st[s].status == status;
}

__device__ __forceinline__ void dd_add_d(double &hi, double &lo, double b) {
    const double s = hi + b;
    const double bb = s - hi;
    const double e = (hi - (s - bb)) + (b - bb);
    const double l = lo + e;
    hi = s + l;
    lo = l - (hi - s);
}

// X += x (double-double accumulation of the FP64 increment) and x = 0, for the flagged systems (all with null flags).
__global__ void __launch_bounds__(RT) k_dd_fold(double2 *__restrict__ Xh, double2 *__restrict__ Xl,
                                               double2 *__restrict__ x, Sys sy, int nblk,
                                               const int *__restrict__ flags) {
    const int s = blockIdx.y, blk = blockIdx.x;
    if (flags && !flags[s]) return;
    int64_t lo, hi;
    int64_t off;
    sy.range(s, nblk, blk, off, lo, hi);
    for (int64_t i = off + lo + threadIdx.x; i < off + hi; i += RT) {
        double2 h = Xh[i], l = Xl[i];
        const double2 v = x[i];
        dd_add_d(h.x, l.x, v.x);
        dd_add_d(h.y, l.y, v.y);
        Xh[i] = h;
        Xl[i] = l;
        x[i] = make_double2(0.0, 0.0);
    }
}

// r = b - (Th + Tl) rounded to FP64 (the double-double residual), b_seg = r and |r|^2 partials, for the flagged
// systems (every system with null flags).
__global__ void __launch_bounds__(RT) k_resid_dd(const double2 *__restrict__ b, const double2 *__restrict__ Th,
                                                const double2 *__restrict__ Tl, double2 *__restrict__ r,
                                                double2 *__restrict__ bseg, Sys sy, int nblk,
                                                double *__restrict__ partial, const int *__restrict__ flags) {
    const int s = blockIdx.y, blk = blockIdx.x;
    if (flags && !flags[s]) return;
    int64_t lo, hi;
    int64_t off;
    sy.range(s, nblk, blk, off, lo, hi);
    double acc = 0;
    for (int64_t i = off + lo + threadIdx.x; i < off + hi; i += RT) {
        const double2 bv = b[i], th = Th[i], tl = Tl[i];
        double rh = bv.x, rl = 0.0, ih = bv.y, il = 0.0;
        dd_add_d(rh, rl, -th.x);
        dd_add_d(rh, rl, -tl.x);
        dd_add_d(ih, il, -th.y);
        dd_add_d(ih, il, -tl.y);
        const double2 rv = make_double2(rh + rl, ih + il);
        r[i] = rv;
        if (bseg) bseg[i] = rv;
        acc += rv.x * rv.x + rv.y * rv.y;
    }
    acc = block_sum(acc);
    if (threadIdx.x == 0) partial[(int64_t)s * nblk + blk] = acc;
}

struct Plan {
    int64_t nsys, n, nbatch;  // n: the length of every system (one fermion matrix)
    int nblk;
    int64_t total = 0;        // elements of one vector (all systems)
    Sys sy;                   // the systems' ranges as the kernels read them
};

Plan make_plan(nslg_fm *fm, int64_t nbatch, int mode) {
    Plan P;
    P.nbatch = nbatch;
    const int64_t vol = fm->Nt * fm->Nx;
    if (mode == NSLG_CG_SHARED) {
        P.nsys = 1;
        P.n = nbatch * vol;
    } else {
        P.nsys = nbatch;
        P.n = vol;
    }
    // ~8 blocks of 256 threads per SM over all systems, at least 1024 elements per block
    const int64_t target = 8 * (int64_t)std::max(fm->ctx->num_sms, 1);
    int64_t nb = std::max<int64_t>(1, target / P.nsys);
    nb = std::min<int64_t>(nb, std::max<int64_t>(1, P.n / 1024));
    P.nblk = (int)std::min<int64_t>(nb, 1024);
    P.total = P.nsys * P.n;
    P.sy.n = P.n;
    return P;
}

struct CgBufs {
    double2 *x = nullptr, *r = nullptr, *p = nullptr, *t = nullptr;
};

struct CgRun {
    nslg_fm *fm;
    int op;
    Plan P;
    CgBufs v;
    double2 *p_pt;
    double *p_rr;
    CgState *states;  // 2 * nsys (double buffer)
    double errSq;
    int64_t max_iter;
    int reliable;
    const double2 *half = nullptr;  // M^dagger p (MMdag) or M p (MdagM): the operator's intermediate vector
    // fused split-BF16 iteration (MMdag / MdagM on the tensor cores): the CG dot products and updates run in the
    // operator's epilogues
    bool fused = false;
    const OzPlanes *oz_first = nullptr, *oz_second = nullptr;
    void *oz_dg = nullptr;
    int *oz_rexp = nullptr;
    double2 *tmp = nullptr;
    double2 *u = nullptr;  // MMdag: phase o tmp, written by the first factor's epilogue (the second factor's operand)
    double *part_c = nullptr, *part_r = nullptr, *alpha = nullptr;
    int *active = nullptr;
    int npart = 0;  // partial sums per system in part_c / part_r
    // double-double rule: the solution is Xh + Xl + x (x the FP64 increment since the system's last rebase) and the
    // FP64 reliable updates evaluate bseg - A x, bseg = b - A (Xh + Xl) from the last rebase
    bool dd = false;
    double2 *Xh = nullptr, *Xl = nullptr, *Th = nullptr, *Tl = nullptr, *bseg = nullptr;
    int *flags = nullptr;
    // the fermion matrices of the solve: one, or a group of different sizes whose right-hand sides are packed one
    // instance after the other (instance i: nbatch right-hand sides from element voff, systems [s0, s0 + nsys))
    struct Inst {
        nslg_fm *fm;
        int64_t nbatch, voff, s0, nsys, rows_per_sys;
        bool resident = false;  // its systems run in the resident kernel
        bool idle = false;      // none of its systems runs in the launch-per-step loop (all final, or resident)
    };
    std::vector<Inst> inst;
    std::string key;  // identity of the instances in graph keys
    // while the launch-per-step loop runs, its operator applications leave out the idle instances (a group whose
    // instances converge at different times stops paying for the finished ones)
    bool skip_idle = false;
    std::string idle_mask() const {
        std::string m;
        for (auto &I : inst) m += I.idle ? '1' : '0';
        return m;
    }
};

// op on the packed vectors of every instance, products in T (one launch sequence per instance); with flags (FP64
// products) only the rows of the flagged systems are computed.
template <typename T> int apply_all(CgRun &R, const double2 *in, double2 *out, const int *flags = nullptr) {
    for (auto &I : R.inst)
        if (!(R.skip_idle && I.idle))
            NSLG_TRY(fm_apply_dev<T>(I.fm, R.op, in + I.voff, out + I.voff, I.nbatch, flags ? flags + I.s0 : nullptr,
                                     I.rows_per_sys));
    return NSLG_OK;
}
// op in double-double on the packed pairs, only for the flagged systems when flags is given.
int apply_dd_all(CgRun &R, const double2 *xh, const double2 *xl, double2 *oh, double2 *ol, const int *flags) {
    for (auto &I : R.inst)
        if (!(R.skip_idle && I.idle))
            NSLG_TRY(fm_apply_dd(I.fm, R.op, xh + I.voff, xl + I.voff, oh + I.voff, ol + I.voff, I.nbatch,
                                 flags ? flags + I.s0 : nullptr, I.rows_per_sys));
    return NSLG_OK;
}

// Reliable update once |r|^2 fell this far below its running maximum: 100x for the FP32-class operators (their
// recurrence drifts from the true residual quickly), 1e4x for FP64-class products (split-BF16, FP64 with the
// true-residual rule), whose recurrence stays close to the true residual and for which each FP64 update costs
// about a dozen split-BF16 iterations.
constexpr double UPDATE_FRAC = 0.01;
constexpr double UPDATE_FRAC_FP64_CLASS = 1e-4;
constexpr int CHUNK = 16;  // iterations per captured graph (even: the state double buffer returns to slot 0)

// One fused split-BF16 iteration on A = M M^dagger (M^dagger M):
//   first factor  tmp = M^dagger p (M p), epilogue: curvature partials |tmp|^2
//   k_cg_alpha    alpha = |r|^2 / |tmp|^2 per running system
//   second factor A p = M tmp (M^dagger tmp), epilogue: r -= alpha A p, partials |r|^2
//   k_cg_p        beta, status; x += alpha p, p = r + beta p
//   (M M^dagger, all but a chunk's last iteration: k_cg_p_oz also writes the digits of the new p, and the next
//   iteration's first factor skips its digit pre-pass)
int cg_iteration_fused(CgRun &R, CgState *st_a, CgState *st_b, int j) {
    nslg_fm *fm = R.fm;
    cudaStream_t st = fm->ctx->stream;
    const int Nt = (int)fm->Nt, Nx = (int)fm->Nx;
    const int64_t rows = R.P.nbatch * fm->Nt;
    const int first = R.op == NSLG_OP_MMDAGGER ? MODE_MDAG : MODE_M;
    const int second = R.op == NSLG_OP_MMDAGGER ? MODE_M : MODE_MDAG;
    OzEpi e1;
    e1.mode = 1;
    e1.part = R.part_c;
    e1.go = R.active;  // finished systems skip both factors (go is maintained by k_cg_p and each chunk's first node)
    e1.sys_rows = R.P.n / fm->Nx;
    e1.u = R.u;  // MMdag: the M factor's operand phase o tmp comes from the M^dagger epilogue
    const bool mmdag = R.op == NSLG_OP_MMDAGGER;
    e1.digits_ready = mmdag && j > 0;  // written by the previous iteration's k_cg_p_oz
    NSLG_TRY(fm_apply_oz(first, R.v.p, R.tmp, fm->phase, *R.oz_first, R.oz_dg, R.oz_rexp, Nt, Nx, rows, fm->tc_err,
                         st, &e1));
    k_cg_alpha<<<(unsigned)R.P.nsys, RT, 0, st>>>(R.part_c, R.npart, st_a, R.alpha, R.active);
    note_launch(st);
    OzEpi e2;
    e2.mode = 2;
    e2.part = R.part_r;
    e2.alpha = R.alpha;
    e2.active = R.active;
    e2.r = R.v.r;
    e2.sys_rows = R.P.n / fm->Nx;
    e2.go = R.active;
    e2.operand = R.u;
    NSLG_TRY(fm_apply_oz(second, R.tmp, nullptr, fm->phase, *R.oz_second, R.oz_dg, R.oz_rexp, Nt, Nx, rows,
                         fm->tc_err, st, &e2));
    if (mmdag && j + 1 < CHUNK) {
        const int rps = (int)(R.P.n / fm->Nx);
        dim3 grid((unsigned)ceil_div(rps, RT / 32), (unsigned)R.P.nsys);
        k_cg_p_oz<<<grid, RT, 0, st>>>(R.v.r, R.v.p, R.v.x, R.alpha, Nx, rps, R.part_r, R.npart, st_a, st_b,
                                       R.max_iter, R.reliable, UPDATE_FRAC_FP64_CLASS, R.active,
                                       static_cast<__nv_bfloat16 *>(R.oz_dg), R.oz_rexp, oz_ld(Nx), rows);
    } else {
        dim3 grid(R.P.nblk, (unsigned)R.P.nsys);
        k_cg_p<<<grid, RT, 0, st>>>(R.v.r, R.v.p, R.v.x, R.alpha, R.P.sy, R.P.nblk, R.part_r, R.npart, st_a, st_b,
                                    R.errSq, R.max_iter, R.reliable, UPDATE_FRAC_FP64_CLASS, R.active);
    }
    note_launch(st);
    NSLG_CUDA(cudaGetLastError());
    return NSLG_OK;
}

// One CG iteration (captured into the chunk graph).
template <typename Top> int cg_iteration(CgRun &R, CgState *st_a, CgState *st_b, int j) {
    if constexpr (std::is_same_v<Top, BF16Split>)
        if (R.fused) return cg_iteration_fused(R, st_a, st_b, j);
    cudaStream_t st = R.fm->ctx->stream;
    NSLG_TRY(apply_all<Top>(R, R.v.p, R.v.t));
    dim3 grid(R.P.nblk, (unsigned)R.P.nsys);
    // <p, A p>; for A = M M^dagger (M^dagger M) in the mixed forms as |M^dagger p|^2 (|M p|^2), equal in exact
    // arithmetic but positive by construction when the two factors carry independent rounding
    if (R.half) k_dot<<<grid, RT, 0, st>>>(R.half, R.half, R.P.sy, R.P.nblk, R.p_pt, st_a);
    else k_dot<<<grid, RT, 0, st>>>(R.v.p, R.v.t, R.P.sy, R.P.nblk, R.p_pt, st_a);
    note_launch(st);
    k_cg_xr<<<grid, RT, 0, st>>>(R.v.x, R.v.r, R.v.p, R.v.t, R.P.sy, R.P.nblk, R.p_pt, st_a, R.p_rr);
    note_launch(st);
    // FP32-class operators also force an update every UPDATE_EVERY iterations (stall detection, mode 2)
    constexpr bool fp32_class = std::is_same_v<Top, float> || std::is_same_v<Top, TF32x3>;
    const int rule = (R.reliable && fp32_class) ? 2 : R.reliable;
    k_cg_p<<<grid, RT, 0, st>>>(R.v.r, R.v.p, nullptr, nullptr, R.P.sy, R.P.nblk, R.p_rr, R.P.nblk, st_a, st_b,
                                R.errSq, R.max_iter, rule, fp32_class ? UPDATE_FRAC : UPDATE_FRAC_FP64_CLASS, nullptr);
    note_launch(st);
    NSLG_CUDA(cudaGetLastError());
    return NSLG_OK;
}

#include "cg_resident.cuh"


template <typename Top> int run_chunk(CgRun &R) {
    nslg_fm *fm = R.fm;
    cudaStream_t st = fm->ctx->stream;
    char keybuf[256];
    // R.key holds, per instance, the handle, its species sign (it selects the exp(+-delta K) entry the captured
    // applications read), its batch and its workspace generation
    std::snprintf(keybuf, sizeof keybuf, "cg:%s:%d:%lld:%lld:%lld:%d:%d:", typeid(Top).name(), R.op,
                  (long long)R.P.nsys, (long long)R.P.n, (long long)R.max_iter, R.reliable,
                  (R.half ? 1 : 0) + (R.fused ? 2 : 0));
    std::string key = std::string(keybuf) + R.key + (R.inst.size() > 1 ? "|" + R.idle_mask() : std::string());
    auto it = fm->graphs.find(key);
    if (it == fm->graphs.end()) {
        // every batch composition of a group and every idle set captures its own graph: keep the cache bounded
        size_t ncg = 0;
        for (auto &g : fm->graphs) ncg += g.first.compare(0, 3, "cg:") == 0;
        if (ncg >= 256) {
            for (auto g = fm->graphs.begin(); g != fm->graphs.end();) {
                if (g->first.compare(0, 3, "cg:") == 0) {
                    cudaGraphExecDestroy(g->second);
                    fm->graph_kernels.erase(g->first);
                    g = fm->graphs.erase(g);
                } else {
                    ++g;
                }
            }
        }
        cudaGraph_t g;
        NSLG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        int rc = NSLG_OK;
        if (std::is_same_v<Top, BF16Split> && R.fused) {
            k_go_from_state<<<(unsigned)ceil_div(R.P.nsys, 256), 256, 0, st>>>(R.states, (int)R.P.nsys, R.active);
            note_launch(st);
        }
        for (int j = 0; j < CHUNK && rc == NSLG_OK; ++j)
            rc = cg_iteration<Top>(R, R.states + (j & 1) * R.P.nsys, R.states + ((j + 1) & 1) * R.P.nsys, j);
        cudaError_t ce = cudaStreamEndCapture(st, &g);
        if (rc != NSLG_OK) {
            if (ce == cudaSuccess) cudaGraphDestroy(g);
            return rc;
        }
        NSLG_CUDA(ce);
        size_t nodes = 0;
        cudaGraphGetNodes(g, nullptr, &nodes);
        cudaGraphExec_t ex;
        cudaError_t ie = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        NSLG_CUDA(ie);
        it = fm->graphs.emplace(key, ex).first;
        fm->graph_kernels[key] = nodes;
    }
    NSLG_CUDA(cudaGraphLaunch(it->second, st));
    note_launch(st, fm->graph_kernels[key]);
    return NSLG_OK;
}

// ----- resident systems -----------------------------------------------------------------------------------------
// Systems of at most RES_MAX_LEN elements on lattices of at most RES_MAX_NX sites whose shared-memory need fits
// RES_MAX_SMEM, with a mixed-precision request, run in the resident kernel (cg_resident.cuh, float-float iteration);
// NSLG_CG_RESIDENT=0 keeps every system on the launch-per-step solver.
constexpr int64_t RES_MAX_LEN = 2048;
constexpr int RES_MAX_NX = 64;
constexpr size_t RES_MAX_SMEM = 220 * 1024;

struct ResRun {
    std::vector<RSys> sys;
    std::vector<int> list;  // the resident systems
    RSys *d_sys = nullptr;
    int *d_list = nullptr, *d_prec = nullptr, *d_cnt = nullptr;
    CgState *d_st = nullptr;
    size_t smem = 0;
    int budget = 0;
    RArgs args;
};

// Marks the instances whose systems go to the resident kernel; true if any.
int plan_resident(CgRun &R, int precision, bool *any) {
    *any = false;
    const char *env = std::getenv("NSLG_CG_RESIDENT");
    if (env && env[0] == '0') return NSLG_OK;
    if (precision == NSLG_PREC_FP64 || (R.op != NSLG_OP_MMDAGGER && R.op != NSLG_OP_MDAGGERM)) return NSLG_OK;
    for (auto &I : R.inst) {
        nslg_fm *f = I.fm;
        const int64_t len = I.rows_per_sys * f->Nx;
        if (f->kind != NSLG_FM_EXP || f->delta.y != 0.0 || f->Nx > RES_MAX_NX || len > RES_MAX_LEN ||
            res_smem_bytes(len, (int)f->Nx) > RES_MAX_SMEM)
            continue;
        const ExpEntry *E;
        NSLG_TRY(get_exp(f, make_double2(f->sgn * f->delta.x, 0.0), &E));
        if (!E->is_real) continue;
        I.resident = true;
        *any = true;
    }
    return NSLG_OK;
}

// Hands the resident systems over (their states move to the kernel's own array, CG_RESIDENT in the solver's) and
// launches the resident kernel on the first handle's side stream, after everything queued on the solver's stream.
int resident_start(CgRun &R, const double2 *b, ResRun &Q) {
    nslg_fm *fm = R.fm;
    cudaStream_t st = fm->ctx->stream;
    const Plan &P = R.P;
    Q.sys.assign((size_t)P.nsys, RSys{});
    double cost = 1;
    for (auto &I : R.inst) {
        if (!I.resident) continue;
        nslg_fm *f = I.fm;
        const ExpEntry *E;
        NSLG_TRY(get_exp(f, make_double2(f->sgn * f->delta.x, 0.0), &E));
        const int64_t len = I.rows_per_sys * f->Nx;
        for (int64_t k = 0; k < I.nsys; ++k) {
            RSys &y = Q.sys[(size_t)(I.s0 + k)];
            y.ph = f->phase;
            y.E = E->re;
            y.Nt = (int)f->Nt;
            y.Nx = (int)f->Nx;
            y.off = I.voff + k * len;
            y.len = (int)len;
            Q.list.push_back((int)(I.s0 + k));
        }
        Q.smem = std::max(Q.smem, res_smem_bytes(len, (int)f->Nx));
        cost = std::max(cost, 3.3 * (double)len * (double)f->Nx + 10.0 * (double)len);
    }
    // iterations per launch: ~1e9 cycles of the slowest (FP64-escalated) system, so that one launch stays well
    // under a second
    Q.budget = (int)std::min(100000.0, std::max(64.0, 1e9 / cost));
    {
        static std::mutex mu;
        static std::set<int> done;
        std::lock_guard<std::mutex> lock(mu);
        if (!done.count(fm->ctx->device)) {
            NSLG_CUDA(cudaFuncSetAttribute(k_cg_resident, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)RES_MAX_SMEM));
            done.insert(fm->ctx->device);
        }
    }
    const int count = (int)Q.list.size();
    NSLG_TRY(ws_get(fm, "cgr_sys", Q.sys.size(), &Q.d_sys));
    NSLG_TRY(ws_get(fm, "cgr_list", (size_t)count, &Q.d_list));
    NSLG_TRY(ws_get(fm, "cgr_prec", (size_t)P.nsys, &Q.d_prec));
    NSLG_TRY(ws_get(fm, "cgr_cnt", (size_t)(3 * P.nsys), &Q.d_cnt));
    NSLG_TRY(ws_get(fm, "cgr_st", (size_t)P.nsys, &Q.d_st));
    NSLG_CUDA(cudaMemcpyAsync(Q.d_sys, Q.sys.data(), Q.sys.size() * sizeof(RSys), cudaMemcpyHostToDevice, st));
    NSLG_CUDA(cudaMemcpyAsync(Q.d_list, Q.list.data(), count * sizeof(int), cudaMemcpyHostToDevice, st));
    NSLG_CUDA(cudaMemsetAsync(Q.d_prec, 0, P.nsys * sizeof(int), st));
    NSLG_CUDA(cudaMemsetAsync(Q.d_cnt, 0, 3 * P.nsys * sizeof(int), st));
    k_resident_handover<<<(unsigned)ceil_div(count, 256), 256, 0, st>>>(R.states, Q.d_st, Q.d_list, count, 0);
    note_launch(st);
    RArgs &A = Q.args;
    A.sys = Q.d_sys;
    A.list = Q.d_list;
    A.b = b;
    A.bseg = R.bseg;
    A.x = R.v.x;
    A.r = R.v.r;
    A.p = R.v.p;
    A.Xh = R.Xh;
    A.Xl = R.Xl;
    A.st = Q.d_st;
    A.prec64 = Q.d_prec;
    A.counts = Q.d_cnt;
    A.max_iter = R.max_iter;
    A.op = R.op;
    A.reliable = R.reliable;
    A.dd = R.dd ? 1 : 0;
    A.budget = Q.budget;
    if (!fm->side) NSLG_CUDA(cudaStreamCreateWithFlags(&fm->side, cudaStreamNonBlocking));
    if (!fm->ev_fork) NSLG_CUDA(cudaEventCreateWithFlags(&fm->ev_fork, cudaEventDisableTiming));
    if (!fm->ev_join) NSLG_CUDA(cudaEventCreateWithFlags(&fm->ev_join, cudaEventDisableTiming));
    NSLG_CUDA(cudaEventRecord(fm->ev_fork, st));
    NSLG_CUDA(cudaStreamWaitEvent(fm->side, fm->ev_fork, 0));
    k_cg_resident<<<(unsigned)count, RT, Q.smem, fm->side>>>(A);
    note_launch(fm->side);
    NSLG_CUDA(cudaGetLastError());
    return NSLG_OK;
}

// Waits for the resident kernel, launches it again for systems that ran out of their per-launch budget, hands the
// states back to the solver's array and adds the resident systems' update counts (maximum over systems).
int resident_finish(CgRun &R, ResRun &Q, int64_t *updates, int64_t *rebases, int64_t *escalations) {
    nslg_fm *fm = R.fm;
    cudaStream_t st = fm->ctx->stream;
    const Plan &P = R.P;
    std::vector<CgState> rs((size_t)P.nsys);
    std::vector<int> all = Q.list;
    for (;;) {
        NSLG_CUDA(cudaMemcpyAsync(rs.data(), Q.d_st, rs.size() * sizeof(CgState), cudaMemcpyDeviceToHost, fm->side));
        NSLG_CUDA(cudaStreamSynchronize(fm->side));
        std::vector<int> again;
        for (int s : Q.list)
            if (rs[s].status == CG_ACTIVE || rs[s].status == CG_UPDATE) again.push_back(s);
        if (again.empty()) break;
        Q.list = again;
        NSLG_CUDA(cudaMemcpyAsync(Q.d_list, Q.list.data(), Q.list.size() * sizeof(int), cudaMemcpyHostToDevice,
                                  fm->side));
        k_cg_resident<<<(unsigned)Q.list.size(), RT, Q.smem, fm->side>>>(Q.args);
        note_launch(fm->side);
        NSLG_CUDA(cudaGetLastError());
    }
    NSLG_CUDA(cudaEventRecord(fm->ev_join, fm->side));
    NSLG_CUDA(cudaStreamWaitEvent(st, fm->ev_join, 0));
    // the full list again: every resident system's state goes back
    NSLG_CUDA(cudaMemcpyAsync(Q.d_list, all.data(), all.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    k_resident_handover<<<(unsigned)ceil_div((int64_t)all.size(), 256), 256, 0, st>>>(R.states, Q.d_st, Q.d_list,
                                                                                    (int)all.size(), 1);
    note_launch(st);
    std::vector<int> cnt((size_t)(3 * P.nsys));
    NSLG_CUDA(cudaMemcpyAsync(cnt.data(), Q.d_cnt, cnt.size() * sizeof(int), cudaMemcpyDeviceToHost, st));
    NSLG_CUDA(cudaStreamSynchronize(st));
    int mu = 0, mr = 0, me = 0;
    for (int s : all) {
        mu = std::max(mu, cnt[3 * s]);
        mr = std::max(mr, cnt[3 * s + 1]);
        me = std::max(me, cnt[3 * s + 2]);
    }
    *updates += mu;
    *rebases += mr;
    *escalations += me;
    return NSLG_OK;
}

int read_states(nslg_fm *fm, const CgState *d, int64_t nsys, std::vector<CgState> &h) {
    h.resize(nsys);
    NSLG_CUDA(cudaMemcpyAsync(h.data(), d, nsys * sizeof(CgState), cudaMemcpyDeviceToHost, fm->ctx->stream));
    NSLG_CUDA(cudaStreamSynchronize(fm->ctx->stream));
    return NSLG_OK;
}

// Final statistics per instance: the true residual |b - A x| / |b| of every system (FP64, or double-double of the
// pair under the double-double rule), aggregated over the instance's systems.
int finish_stats(CgRun &R, const double2 *b, double2 *tmp, double2 *rtmp, const std::vector<CgState> &hs,
                 nslg_cg_stats *const *stats) {
    bool any = false;
    for (size_t i = 0; i < R.inst.size(); ++i) any |= stats[i] != nullptr;
    if (!any) return NSLG_OK;
    nslg_fm *fm = R.fm;
    const Plan &P = R.P;
    cudaStream_t st = fm->ctx->stream;
    dim3 grid(P.nblk, (unsigned)P.nsys);
    if (R.dd) {  // |b - A (Xh + Xl)| in double-double (the increment is folded in already)
        NSLG_TRY(apply_dd_all(R, R.Xh, R.Xl, R.Th, R.Tl, nullptr));
        k_resid_dd<<<grid, RT, 0, st>>>(b, R.Th, R.Tl, rtmp, nullptr, P.sy, P.nblk, R.p_rr, nullptr);
    } else {
        NSLG_TRY(apply_all<double>(R, R.v.x, tmp));
        k_resid<<<grid, RT, 0, st>>>(b, tmp, rtmp, P.sy, P.nblk, R.p_rr, nullptr);
    }
    note_launch(st);
    double *pb = R.p_rr + P.nsys * P.nblk;
    k_norm2<<<grid, RT, 0, st>>>(b, P.sy, P.nblk, pb);
    note_launch(st);
    NSLG_CUDA(cudaGetLastError());
    std::vector<double> h(2 * P.nsys * P.nblk);
    NSLG_CUDA(cudaMemcpyAsync(h.data(), R.p_rr, h.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    NSLG_CUDA(cudaStreamSynchronize(st));
    for (size_t i = 0; i < R.inst.size(); ++i) {
        nslg_cg_stats *out = stats[i];
        if (!out) continue;
        const auto &I = R.inst[i];
        double worst = 0, worst_rec = 0;
        int64_t iters = 0, conv = 0;
        for (int64_t s = I.s0; s < I.s0 + I.nsys; ++s) {
            double rr = 0, bb = 0;
            for (int k = 0; k < P.nblk; ++k) {
                rr += h[s * P.nblk + k];
                bb += h[P.nsys * P.nblk + s * P.nblk + k];
            }
            worst = std::max(worst, bb > 0 ? std::sqrt(rr / bb) : std::sqrt(rr));
            worst_rec = std::max(worst_rec, std::sqrt(std::max(hs[s].rsq, 0.0)));
            iters = std::max<int64_t>(iters, hs[s].iters);
            conv += (hs[s].status == CG_CONVERGED);
        }
        out->true_residual = worst;
        out->recurrence_residual = worst_rec;
        out->iterations = iters;
        out->converged = conv;
        out->systems = I.nsys;
    }
    return NSLG_OK;
}

}  // namespace

namespace {

// The CG loop over R's instances (R.fm, R.op, R.P, R.inst, R.key, R.errSq / eps2_sys and R.max_iter set by the
// caller). b, x0, x and x_lo are packed device buffers of R.P.total elements (x0 may equal b; x must not overlap b).
int cg_run(CgRun &R, const double2 *b, const double2 *x0, double2 *x, double2 *x_lo, const double *eps2_sys,
           int precision, int stop, nslg_cg_stats *const *stats) {
    nslg_fm *fm = R.fm;
    const int op = R.op;
    const int64_t max_iter = R.max_iter;
    cudaStream_t st = fm->ctx->stream;
    R.dd = stop == NSLG_STOP_TRUE_RESIDUAL_DD;
    R.reliable = (stop != NSLG_STOP_RECURRENCE || precision != NSLG_PREC_FP64) ? 1 : 0;
    const Plan &P = R.P;
    const int64_t total = P.total;
    // one fermion matrix with equal systems (the group front end packs systems through tables, P.n = 0, even for one
    // instance): only then do the fused split-BF16 iteration and the curvature from the intermediate vector apply,
    // both index systems as rows / (P.n / Nx)
    const bool single_matrix = R.inst.size() == 1 && P.n > 0;
    const int64_t nbatch = P.nbatch;
    bool resident = false;
    NSLG_TRY(plan_resident(R, precision, &resident));
    bool all_resident = resident;
    for (auto &I : R.inst) all_resident &= I.resident;
    // (the launch-per-step forms below are set up only when some system runs there)
    const bool single = single_matrix && !all_resident;
    NSLG_TRY(ws_get(fm, "cg_flags", (size_t)P.nsys, &R.flags));
    if (R.dd) {
        NSLG_TRY(ws_get(fm, "cg_Xh", total, &R.Xh));
        NSLG_TRY(ws_get(fm, "cg_Xl", total, &R.Xl));
        NSLG_TRY(ws_get(fm, "cg_Th", total, &R.Th));
        NSLG_TRY(ws_get(fm, "cg_Tl", total, &R.Tl));
        NSLG_TRY(ws_get(fm, "cg_bseg", total, &R.bseg));
    }
    double2 *tmp, *rtmp;
    NSLG_TRY(ws_get(fm, "cg_r", total, &R.v.r));
    NSLG_TRY(ws_get(fm, "cg_p", total, &R.v.p));
    NSLG_TRY(ws_get(fm, "cg_t", total, &R.v.t));
    NSLG_TRY(ws_get(fm, "cg_tmp", total, &tmp));
    NSLG_TRY(ws_get(fm, "cg_rtmp", total, &rtmp));
    NSLG_TRY(ws_get(fm, "cg_ppt", P.nsys * P.nblk, &R.p_pt));
    NSLG_TRY(ws_get(fm, "cg_prr", 2 * P.nsys * P.nblk, &R.p_rr));
    NSLG_TRY(ws_get(fm, "cg_state", 2 * P.nsys, &R.states));
    if (single && R.reliable && precision != NSLG_PREC_FP64 && (op == NSLG_OP_MMDAGGER || op == NSLG_OP_MDAGGERM)) {
        double2 *h;
        NSLG_TRY(ws_get(fm, "apply_tmp", total, &h));  // the buffer the two-factor applications write first
        R.half = h;
    }
    if (single && precision == NSLG_PREC_BF16_SPLIT && (op == NSLG_OP_MMDAGGER || op == NSLG_OP_MDAGGERM) &&
        fm->Nx <= 2048 && fm->kind == NSLG_FM_EXP) {
        const double2 d = make_double2(fm->sgn * fm->delta.x, fm->sgn * fm->delta.y);
        const double2 dc = make_double2(fm->sgn * fm->delta.x, -fm->sgn * fm->delta.y);
        const ExpEntry *E, *Ec;
        NSLG_TRY(get_exp(fm, d, &E));
        NSLG_TRY(get_exp(fm, dc, &Ec));
        const int64_t ntn = oz_ntiles((int)fm->Nx);
        const int64_t npart = (P.n / fm->Nx) * 2 * ntn;
        if (E->is_real && Ec->is_real && npart >= 1 && npart <= (int64_t)1 << 30) {
            OzPlanes *Pm, *Pd;
            NSLG_TRY(oz_planes(fm, E, &Pm));
            NSLG_TRY(oz_planes(fm, Ec, &Pd));
            R.oz_first = op == NSLG_OP_MMDAGGER ? Pd : Pm;
            R.oz_second = op == NSLG_OP_MMDAGGER ? Pm : Pd;
            const int64_t rows = nbatch * fm->Nt;
            NSLG_TRY(ws_get(fm, "oz_rexp", (size_t)2 * rows, &R.oz_rexp));
            NSLG_TRY(ws_get(fm, "oz_digits", (size_t)oz_digits() * 2 * rows * oz_ld((int)fm->Nx) * 2, &R.oz_dg));
            R.npart = (int)npart;
            NSLG_TRY(ws_get(fm, "cg_partc", (size_t)(P.nsys * npart), &R.part_c));
            NSLG_TRY(ws_get(fm, "cg_partr", (size_t)(P.nsys * npart), &R.part_r));
            NSLG_TRY(ws_get(fm, "cg_alpha", (size_t)P.nsys, &R.alpha));
            NSLG_TRY(ws_get(fm, "cg_active", (size_t)P.nsys, &R.active));
            NSLG_TRY(ws_get(fm, "apply_tmp", total, &R.tmp));
            if (op == NSLG_OP_MMDAGGER) NSLG_TRY(ws_get(fm, "apply_u", total, &R.u));
            R.fused = true;
        }
    }
    // The iterate lives in a workspace buffer: the captured chunk graph bakes in its address, and the caller's x
    // may be a different buffer on every call.
    double2 *xw;
    NSLG_TRY(ws_get(fm, "cg_x", total, &xw));
    R.v.x = xw;
    dim3 grid(P.nblk, (unsigned)P.nsys);
    if (R.dd) {
        // X = x0 (double-double), x = 0, r = bseg = b - A X in double-double
        NSLG_CUDA(cudaMemcpyAsync(R.Xh, x0, total * sizeof(double2), cudaMemcpyDeviceToDevice, st));
        NSLG_CUDA(cudaMemsetAsync(R.Xl, 0, total * sizeof(double2), st));
        NSLG_CUDA(cudaMemsetAsync(xw, 0, total * sizeof(double2), st));
        NSLG_TRY(apply_dd_all(R, R.Xh, R.Xl, R.Th, R.Tl, nullptr));
        k_resid_dd<<<grid, RT, 0, st>>>(b, R.Th, R.Tl, R.v.r, R.bseg, P.sy, P.nblk, R.p_rr, nullptr);
    } else {
        // t = A x ; r = b - t ; p = r
        NSLG_CUDA(cudaMemcpyAsync(xw, x0, total * sizeof(double2), cudaMemcpyDeviceToDevice, st));
        NSLG_TRY(apply_all<double>(R, xw, R.v.t));
        k_resid<<<grid, RT, 0, st>>>(b, R.v.t, R.v.r, P.sy, P.nblk, R.p_rr, nullptr);
    }
    note_launch(st);
    k_start<<<grid, RT, 0, st>>>(R.v.r, R.v.p, P.sy, P.nblk, R.p_rr, R.states, R.errSq, eps2_sys, max_iter);
    note_launch(st);
    NSLG_CUDA(cudaGetLastError());
    ResRun Q;
    if (resident) {  // the small systems leave for the resident kernel, which runs beside the loop below
        NSLG_TRY(resident_start(R, b, Q));
        for (auto &I : R.inst) I.idle = I.resident;
        R.skip_idle = true;
    }
    std::vector<CgState> hs;
    NSLG_TRY(read_states(fm, R.states, P.nsys, hs));
    int64_t updates = 0, chunks = 0, escalations = 0, rebases = 0;
    const double2 *b_upd = R.dd ? R.bseg : b;  // what the FP64 reliable updates subtract A x from
    int cur_prec = precision;
    const bool trace = std::getenv("NSLG_CG_TRACE") != nullptr;
    for (;;) {
        bool active = false, pending = false;
        for (auto &s : hs) {
            active |= (s.status == CG_ACTIVE);
            pending |= (s.status == CG_UPDATE);
        }
        if (pending) {  // r = b - A64 x for the systems in CG_UPDATE, then continue / stop them
            k_status_flags<<<(unsigned)ceil_div(P.nsys, 256), 256, 0, st>>>(R.states, (int)P.nsys, CG_UPDATE,
                                                                           R.flags);
            note_launch(st);
            NSLG_TRY(apply_all<double>(R, xw, tmp, R.flags));
            k_resid<<<grid, RT, 0, st>>>(b_upd, tmp, rtmp, P.sy, P.nblk, R.p_rr, R.states);
            note_launch(st);
            if (R.dd) {
                // systems at the FP64 floor of their segment (or at the target): fold x into X and recompute their
                // residual in double-double
                k_mark_rebase<<<(unsigned)P.nsys, 32, 0, st>>>(R.p_rr, P.nblk, R.states, R.errSq);
                note_launch(st);
                NSLG_TRY(read_states(fm, R.states, P.nsys, hs));
                bool any = false;
                for (auto &sv : hs) any |= sv.status == CG_REBASE;
                if (any) {
                    k_status_flags<<<(unsigned)ceil_div(P.nsys, 256), 256, 0, st>>>(R.states, (int)P.nsys, CG_REBASE,
                                                                                   R.flags);
                    k_dd_fold<<<grid, RT, 0, st>>>(R.Xh, R.Xl, xw, P.sy, P.nblk, R.flags);
                    note_launch(st, 2);
                    NSLG_TRY(apply_dd_all(R, R.Xh, R.Xl, R.Th, R.Tl, R.flags));
                    k_resid_dd<<<grid, RT, 0, st>>>(b, R.Th, R.Tl, rtmp, R.bseg, P.sy, P.nblk, R.p_rr, R.flags);
                    note_launch(st);
                    ++rebases;
                }
            }
            k_rel_finish<<<grid, RT, 0, st>>>(R.v.r, rtmp, R.v.p, P.sy, P.nblk, R.p_rr, R.states, R.states + P.nsys,
                                              R.errSq, max_iter, (cur_prec == NSLG_PREC_FP32 || cur_prec == NSLG_PREC_TF32X3) ? 1 : 0,
                                              R.dd ? 1 : 0);
            note_launch(st);
            NSLG_CUDA(cudaGetLastError());
            NSLG_CUDA(cudaMemcpyAsync(R.states, R.states + P.nsys, P.nsys * sizeof(CgState),
                                      cudaMemcpyDeviceToDevice, st));
            ++updates;
            NSLG_TRY(read_states(fm, R.states, P.nsys, hs));
            continue;
        }
        if (!active) {
            bool stalled = false;
            for (auto &s : hs) stalled |= (s.status == CG_STALLED);
            if (!stalled) break;
            // every running system has stopped gaining with the low-precision operator: finish them in FP64
            cur_prec = NSLG_PREC_FP64;
            ++escalations;
            k_resume<<<grid, RT, 0, st>>>(R.v.r, R.v.p, P.sy, P.nblk, R.states);
            note_launch(st);
            NSLG_CUDA(cudaGetLastError());
            NSLG_TRY(read_states(fm, R.states, P.nsys, hs));
            if (trace) std::fprintf(stderr, "[nslg cg] escalating to the FP64 operator\n");
            continue;
        }
        if (cur_prec == NSLG_PREC_FP64) NSLG_TRY(run_chunk<double>(R));
        else if (cur_prec == NSLG_PREC_FP32) NSLG_TRY(run_chunk<float>(R));
        else if (cur_prec == NSLG_PREC_TF32X3) NSLG_TRY(run_chunk<TF32x3>(R));
        else NSLG_TRY(run_chunk<BF16Split>(R));
        NSLG_TRY(read_states(fm, R.states, P.nsys, hs));
        if (R.inst.size() > 1) {  // instances whose systems are all final leave the applications
            R.skip_idle = true;
            for (auto &I : R.inst) {
                bool running = false;
                for (int64_t k = I.s0; k < I.s0 + I.nsys && !running; ++k) {
                    const int stt = hs[(size_t)k].status;
                    running = stt == CG_ACTIVE || stt == CG_UPDATE || stt == CG_STALLED || stt == CG_REBASE;
                }
                I.idle = !running;
            }
        }
        if (trace && (++chunks % 256) == 0) {
            double worst = 0;
            int it = 0;
            for (auto &s : hs) {
                if (s.status == CG_ACTIVE || s.status == CG_UPDATE) worst = std::max(worst, std::sqrt(s.rsq));
                it = std::max(it, s.iters);
            }
            std::fprintf(stderr, "[nslg cg] iters=%d updates=%lld max running |r|=%.3e\n", it, (long long)updates,
                         worst);
        }
    }
    if (resident) {
        NSLG_TRY(resident_finish(R, Q, &updates, &rebases, &escalations));
        NSLG_TRY(read_states(fm, R.states, P.nsys, hs));
    }
    R.skip_idle = false;
    for (auto &I : R.inst) I.idle = false;
    if (R.dd) {  // x = X + x rounded; the low part to x_lo
        k_dd_fold<<<grid, RT, 0, st>>>(R.Xh, R.Xl, xw, P.sy, P.nblk, nullptr);
        note_launch(st);
        NSLG_CUDA(cudaMemcpyAsync(x, R.Xh, total * sizeof(double2), cudaMemcpyDeviceToDevice, st));
        if (x_lo) NSLG_CUDA(cudaMemcpyAsync(x_lo, R.Xl, total * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    } else {
        NSLG_CUDA(cudaMemcpyAsync(x, xw, total * sizeof(double2), cudaMemcpyDeviceToDevice, st));
        if (x_lo) NSLG_CUDA(cudaMemsetAsync(x_lo, 0, total * sizeof(double2), st));
    }
    if (trace)
        std::fprintf(stderr, "[nslg cg] op=%d prec=%d systems=%lld updates=%lld iters(max)=%d\n", op, precision,
                     (long long)P.nsys, (long long)updates,
                     std::max_element(hs.begin(), hs.end(), [](const CgState &a, const CgState &b) {
                         return a.iters < b.iters;
                     })->iters);
    NSLG_TRY(finish_stats(R, b, tmp, rtmp, hs, stats));
    for (size_t i = 0; i < R.inst.size(); ++i)
        if (stats[i]) {
            stats[i]->reliable_updates = updates;
            stats[i]->escalated = escalations;
            stats[i]->dd_rebases = rebases;
        }
    for (auto &s : hs)
        if (s.status != CG_CONVERGED) {
            set_error("CG did not converge within max_iter iterations");
            return NSLG_NOT_CONVERGED;
        }
    return NSLG_OK;
}

}  // namespace

// One fermion matrix: b, x0 and x are device buffers of nbatch*Nt*Nx (x0 may equal b; x must not overlap b).
int cg_solve(nslg_fm *fm, int op, const double2 *b, const double2 *x0, double2 *x, int64_t nbatch, double eps,
             int64_t max_iter, int mode, int precision, int stop, nslg_cg_stats *stats, double2 *x_lo) {
    CgRun R;
    R.fm = fm;
    R.op = op;
    R.P = make_plan(fm, nbatch, mode);
    R.errSq = eps * eps;
    R.max_iter = max_iter;
    R.inst.push_back({fm, nbatch, 0, 0, R.P.nsys, R.P.n / fm->Nx});
    R.key = std::to_string(reinterpret_cast<uintptr_t>(fm)) + ":" + std::to_string(fm->sgn) + ":" +
            std::to_string(nbatch) + ":" + std::to_string(fm->ws_generation);
    nslg_cg_stats *sp[1] = {stats};
    return cg_run(R, b, x0, x, x_lo, nullptr, precision, stop, sp);
}

// A group of fermion matrices on one context, every right-hand side an independent system (per-RHS), packed one
// instance after the other in the workspaces of the first handle. b[i], x0[i] (or null), x[i], x_lo[i] (or null)
// are buffers (host or device) of handle i; eps[i] its absolute tolerance; stats[i] (or null) its statistics.
int cg_solve_group(int nfm, nslg_fm *const *fms, int op, const double2 *const *b, const double2 *const *x0,
                   double2 *const *x, double2 *const *x_lo, const int64_t *nbatch, const double *eps,
                   int64_t max_iter, int precision, int stop, nslg_cg_stats *const *stats) {
    nslg_fm *fm = fms[0];
    cudaStream_t st = fm->ctx->stream;
    CgRun R;
    R.fm = fm;
    R.op = op;
    R.max_iter = max_iter;
    R.errSq = 0;
    std::vector<int64_t> off, len;
    std::vector<double> eps2;
    int64_t voff = 0, s0 = 0, maxlen = 0;
    for (int i = 0; i < nfm; ++i) {
        nslg_fm *f = fms[i];
        const int64_t vol = f->Nt * f->Nx;
        R.inst.push_back({f, nbatch[i], voff, s0, nbatch[i], f->Nt});
        for (int64_t r = 0; r < nbatch[i]; ++r) {
            off.push_back(voff + r * vol);
            len.push_back(vol);
            eps2.push_back(eps[i] * eps[i]);
        }
        R.key += std::to_string(reinterpret_cast<uintptr_t>(f)) + ":" + std::to_string(f->sgn) + ":" +
                 std::to_string(nbatch[i]) + ":" + std::to_string(f->ws_generation) + ";";
        voff += nbatch[i] * vol;
        s0 += nbatch[i];
        maxlen = std::max(maxlen, vol);
    }
    Plan &P = R.P;
    if (nfm == 1) {  // one matrix: the equal-systems plan (and with it the fused split-BF16 iteration)
        P = make_plan(fm, nbatch[0], NSLG_CG_PER_RHS);
        R.errSq = eps[0] * eps[0];
        R.inst[0].rows_per_sys = fm->Nt;
    } else {
        P.nsys = s0;
        P.nbatch = s0;
        P.n = 0;  // systems of different lengths: the tables
        P.total = voff;
    }
    // ~8 blocks of 256 threads per SM over all systems, at least 1024 elements per block of the longest system
    const int64_t target = 8 * (int64_t)std::max(fm->ctx->num_sms, 1);
    int64_t nb = std::max<int64_t>(1, target / P.nsys);
    nb = std::min<int64_t>(nb, std::max<int64_t>(1, maxlen / 1024));
    P.nblk = (int)std::min<int64_t>(nb, 1024);
    double *deps = nullptr;
    if (nfm > 1) {
        int64_t *doff, *dlen;
        NSLG_TRY(ws_get(fm, "cgg_off", (size_t)P.nsys, &doff));
        NSLG_TRY(ws_get(fm, "cgg_len", (size_t)P.nsys, &dlen));
        NSLG_TRY(ws_get(fm, "cgg_eps2", (size_t)P.nsys, &deps));
        NSLG_CUDA(cudaMemcpyAsync(doff, off.data(), off.size() * sizeof(int64_t), cudaMemcpyHostToDevice, st));
        NSLG_CUDA(cudaMemcpyAsync(dlen, len.data(), len.size() * sizeof(int64_t), cudaMemcpyHostToDevice, st));
        NSLG_CUDA(cudaMemcpyAsync(deps, eps2.data(), eps2.size() * sizeof(double), cudaMemcpyHostToDevice, st));
        P.sy.n = 0;
        P.sy.off = doff;
        P.sy.len = dlen;
    }
    // packed right-hand sides, starting vectors and solutions
    double2 *pb, *px0, *px, *plo = nullptr;
    NSLG_TRY(ws_get(fm, "cgg_b", (size_t)P.total, &pb));
    NSLG_TRY(ws_get(fm, "cgg_x0", (size_t)P.total, &px0));
    NSLG_TRY(ws_get(fm, "cgg_x", (size_t)P.total, &px));
    bool want_lo = false;
    for (int i = 0; i < nfm; ++i) want_lo |= x_lo && x_lo[i];
    if (want_lo) NSLG_TRY(ws_get(fm, "cgg_xlo", (size_t)P.total, &plo));
    for (int i = 0; i < nfm; ++i) {
        const size_t bytes = (size_t)nbatch[i] * fms[i]->Nt * fms[i]->Nx * sizeof(double2);
        const int64_t o = R.inst[i].voff;
        NSLG_CUDA(cudaMemcpyAsync(pb + o, b[i], bytes, cudaMemcpyDefault, st));
        NSLG_CUDA(cudaMemcpyAsync(px0 + o, (x0 && x0[i]) ? x0[i] : b[i], bytes, cudaMemcpyDefault, st));
    }
    const int rc = cg_run(R, pb, px0, px, plo, deps, precision, stop, stats);
    if (rc != NSLG_OK && rc != NSLG_NOT_CONVERGED) return rc;
    for (int i = 0; i < nfm; ++i) {
        const size_t bytes = (size_t)nbatch[i] * fms[i]->Nt * fms[i]->Nx * sizeof(double2);
        const int64_t o = R.inst[i].voff;
        NSLG_CUDA(cudaMemcpyAsync(x[i], px + o, bytes, cudaMemcpyDefault, st));
        if (want_lo && x_lo[i]) NSLG_CUDA(cudaMemcpyAsync(x_lo[i], plo + o, bytes, cudaMemcpyDefault, st));
    }
    NSLG_CUDA(cudaStreamSynchronize(st));  // the caller's buffers may be host memory
    return rc;
}

}  // namespace nslg
