// Conjugate gradient on the fermion operators, batched, with device-resident scalars.
//
// Restates src/NSL/LinAlg/Solver/Impl/CG.tpp:15-113 (x0 = b, alpha = |r|^2 / <p, A p>, stop when the recurrence
// |r|^2 <= eps^2, return x on exhaustion) for many systems at once. All scalars live on the device; an iteration is
//   apply (t = A p)  ->  k_dot (<p, t> partials)  ->  k_cg_xr (alpha; x += alpha p; r -= alpha t; |r|^2 partials)
//                    ->  k_cg_p (beta; p = r + beta p; convergence / exhaustion / reliable-update flags)
// and a chunk of iterations is captured once into a CUDA graph and replayed; the host reads the per-system
// status only between chunks. Each block re-sums the (few) partials it needs in a fixed order, so the reductions
// are deterministic and need no grid-wide barrier.
//
// Batch semantics: SHARED mode is the reference's (one CG over all right-hand sides with alpha/beta summed over the
// whole batch, inner_product.tpp:30-33), implemented as a single system of length nbatch*Nt*Nx; PER_RHS runs nbatch
// independent systems, each masked out once it has converged.
//
// Mixed precision (precision FP32): the iteration runs in FP32 (vectors and operator) with an FP64 solution and
// FP64 reliable updates: when a system's recurrence residual has dropped by 10x since its last update, or reached
// the target, x64 += x32, the true residual r64 = b - A64 x64 is recomputed in FP64 and replaces r32; the system
// stops when |r64| <= eps.

#include <algorithm>
#include <cmath>
#include <vector>

#include "fm_internal.cuh"

namespace nslg {

namespace {

struct CgState {
    double rsq;   // |r|^2 of the current recurrence residual
    double maxr;  // largest |r|^2 since the last reliable update
    int status;
    int iters;
};
enum { CG_ACTIVE = 0, CG_CONVERGED = 1, CG_EXHAUSTED = 2, CG_UPDATE = 3 };

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

// Sum of partial[0..nblk) in a fixed order (deterministic), valid in every thread.
__device__ double sum_partials(const double *partial, int nblk) {
    double v = 0;
    for (int i = threadIdx.x; i < nblk; i += RT) v += partial[i];
    return block_sum(v);
}
__device__ double2 sum_partials2(const double2 *partial, int nblk) {
    double2 v = make_double2(0, 0);
    for (int i = threadIdx.x; i < nblk; i += RT) {
        v.x += partial[i].x;
        v.y += partial[i].y;
    }
    return block_sum2(v);
}

__device__ __forceinline__ void chunk_range(int64_t n, int nblk, int blk, int64_t &lo, int64_t &hi) {
    const int64_t c = (n + nblk - 1) / nblk;
    lo = (int64_t)blk * c;
    hi = min(n, lo + c);
}

template <typename C> __device__ __forceinline__ double2 to_d2(C v) { return make_double2((double)v.x, (double)v.y); }

// partial[s, blk] = sum conj(a) b over the block's chunk of system s
template <typename T>
__global__ void __launch_bounds__(RT) k_dot(const cplx_t<T> *__restrict__ a, const cplx_t<T> *__restrict__ b,
                                            int64_t n, int nblk, double2 *__restrict__ partial,
                                            const CgState *__restrict__ st) {
    const int s = blockIdx.y, blk = blockIdx.x;
    if (st && st[s].status != CG_ACTIVE) return;
    int64_t lo, hi;
    chunk_range(n, nblk, blk, lo, hi);
    a += (int64_t)s * n;
    b += (int64_t)s * n;
    double2 acc = make_double2(0, 0);
    for (int64_t i = lo + threadIdx.x; i < hi; i += RT) {
        const double2 x = to_d2(a[i]), y = to_d2(b[i]);
        acc.x += x.x * y.x + x.y * y.y;
        acc.y += x.x * y.y - x.y * y.x;
    }
    acc = block_sum2(acc);
    if (threadIdx.x == 0) partial[(int64_t)s * nblk + blk] = acc;
}

// alpha = rsq / <p, t>;  x += alpha p;  r -= alpha t;  partial |r|^2
template <typename T>
__global__ void __launch_bounds__(RT) k_cg_xr(cplx_t<T> *__restrict__ x, cplx_t<T> *__restrict__ r,
                                              const cplx_t<T> *__restrict__ p, const cplx_t<T> *__restrict__ t,
                                              int64_t n, int nblk, const double2 *__restrict__ p_pt,
                                              const CgState *__restrict__ st, double *__restrict__ p_rr) {
    const int s = blockIdx.y, blk = blockIdx.x;
    const CgState S = st[s];
    if (S.status != CG_ACTIVE) return;
    const double2 pt = sum_partials2(p_pt + (int64_t)s * nblk, nblk);
    // alpha = rsq / pt
    const double den = pt.x * pt.x + pt.y * pt.y;
    const double ar = S.rsq * pt.x / den, ai = -S.rsq * pt.y / den;
    const T alr = (T)ar, ali = (T)ai;
    int64_t lo, hi;
    chunk_range(n, nblk, blk, lo, hi);
    const int64_t off = (int64_t)s * n;
    double acc = 0;
    for (int64_t i = off + lo + threadIdx.x; i < off + hi; i += RT) {
        const cplx_t<T> pv = p[i], tv = t[i];
        cplx_t<T> xv = x[i], rv = r[i];
        xv.x += alr * pv.x - ali * pv.y;
        xv.y += alr * pv.y + ali * pv.x;
        rv.x -= alr * tv.x - ali * tv.y;
        rv.y -= alr * tv.y + ali * tv.x;
        x[i] = xv;
        r[i] = rv;
        acc += (double)rv.x * rv.x + (double)rv.y * rv.y;
    }
    acc = block_sum(acc);
    if (threadIdx.x == 0) p_rr[(int64_t)s * nblk + blk] = acc;
}

// beta = |r_new|^2 / |r_old|^2; p = r + beta p; status update. st_in and st_out are different buffers.
template <typename T>
__global__ void __launch_bounds__(RT) k_cg_p(const cplx_t<T> *__restrict__ r, cplx_t<T> *__restrict__ p, int64_t n,
                                             int nblk, const double *__restrict__ p_rr,
                                             const CgState *__restrict__ st_in, CgState *__restrict__ st_out,
                                             double errSq, int64_t max_iter, double update_frac, double targetSq) {
    const int s = blockIdx.y, blk = blockIdx.x;
    const CgState S = st_in[s];
    if (S.status != CG_ACTIVE) {
        if (blk == 0 && threadIdx.x == 0) st_out[s] = S;
        return;
    }
    const double rn = sum_partials(p_rr + (int64_t)s * nblk, nblk);
    CgState N = S;
    N.iters = S.iters + 1;
    if (update_frac == 0.0) {  // FP64: the reference's rule (CG.tpp:70)
        if (rn <= errSq) N.status = CG_CONVERGED;
        else if (N.iters >= max_iter) N.status = CG_EXHAUSTED;
    } else {  // mixed: hand over to an FP64 reliable update
        if (rn <= targetSq || rn < update_frac * S.maxr) N.status = CG_UPDATE;
        else if (N.iters >= max_iter) N.status = CG_UPDATE;
    }
    if (N.status == CG_ACTIVE) {
        const T beta = (T)(rn / S.rsq);
        int64_t lo, hi;
        chunk_range(n, nblk, blk, lo, hi);
        const int64_t off = (int64_t)s * n;
        for (int64_t i = off + lo + threadIdx.x; i < off + hi; i += RT) {
            const cplx_t<T> rv = r[i];
            cplx_t<T> pv = p[i];
            pv.x = rv.x + beta * pv.x;
            pv.y = rv.y + beta * pv.y;
            p[i] = pv;
        }
        N.rsq = rn;
        N.maxr = fmax(S.maxr, rn);
    }
    // On CG_UPDATE the old rsq is kept: the reliable update forms beta from it.
    if (blk == 0 && threadIdx.x == 0) st_out[s] = N;
}

// r64 = b - t64;  rlow = r64;  plow = rlow;  xlow = 0 (if given);  partial |r64|^2. Only systems whose status is
// `only_status` (or all when only_status < 0).
template <typename T>
__global__ void __launch_bounds__(RT) k_resid(const double2 *__restrict__ b, const double2 *__restrict__ t64,
                                              double2 *__restrict__ r64, int64_t n, int nblk,
                                              double *__restrict__ partial, const CgState *__restrict__ st,
                                              int only_status) {
    const int s = blockIdx.y, blk = blockIdx.x;
    if (st && only_status >= 0 && st[s].status != only_status) return;
    int64_t lo, hi;
    chunk_range(n, nblk, blk, lo, hi);
    const int64_t off = (int64_t)s * n;
    double acc = 0;
    for (int64_t i = off + lo + threadIdx.x; i < off + hi; i += RT) {
        const double2 bv = b[i], tv = t64[i];
        const double2 rv = make_double2(bv.x - tv.x, bv.y - tv.y);
        r64[i] = rv;
        acc += rv.x * rv.x + rv.y * rv.y;
    }
    acc = block_sum(acc);
    if (threadIdx.x == 0) partial[(int64_t)s * nblk + blk] = acc;
}

// Initial state from |r|^2 partials; copies r into p (and the low-precision r, p; zeroes xlow).
template <typename T>
__global__ void __launch_bounds__(RT) k_start(const double2 *__restrict__ r64, cplx_t<T> *__restrict__ rlow,
                                              cplx_t<T> *__restrict__ plow, cplx_t<T> *__restrict__ xlow, int64_t n,
                                              int nblk, const double *__restrict__ partial, CgState *__restrict__ st,
                                              double errSq, int64_t max_iter) {
    const int s = blockIdx.y, blk = blockIdx.x;
    const double rn = sum_partials(partial + (int64_t)s * nblk, nblk);
    int64_t lo, hi;
    chunk_range(n, nblk, blk, lo, hi);
    const int64_t off = (int64_t)s * n;
    for (int64_t i = off + lo + threadIdx.x; i < off + hi; i += RT) {
        const double2 v = r64[i];
        cplx_t<T> w;
        w.x = (T)v.x;
        w.y = (T)v.y;
        if (rlow) rlow[i] = w;
        plow[i] = w;
        if (xlow) {
            cplx_t<T> z;
            z.x = 0;
            z.y = 0;
            xlow[i] = z;
        }
    }
    if (blk == 0 && threadIdx.x == 0) {
        CgState S;
        S.rsq = rn;
        S.maxr = rn;
        S.iters = 0;
        S.status = (rn <= errSq) ? CG_CONVERGED : (max_iter <= 0 ? CG_EXHAUSTED : CG_ACTIVE);
        st[s] = S;
    }
}

// Reliable update, part 1: x64 += xlow; xlow = 0 (systems in CG_UPDATE).
__global__ void __launch_bounds__(RT) k_rel_accum(double2 *__restrict__ x64, float2 *__restrict__ xlow, int64_t n,
                                                  int nblk, const CgState *__restrict__ st) {
    const int s = blockIdx.y, blk = blockIdx.x;
    if (st[s].status != CG_UPDATE) return;
    int64_t lo, hi;
    chunk_range(n, nblk, blk, lo, hi);
    const int64_t off = (int64_t)s * n;
    for (int64_t i = off + lo + threadIdx.x; i < off + hi; i += RT) {
        const float2 v = xlow[i];
        double2 x = x64[i];
        x.x += (double)v.x;
        x.y += (double)v.y;
        x64[i] = x;
        xlow[i] = make_float2(0.f, 0.f);
    }
}

// Reliable update, part 2: with the true |r64|^2 partials: converged, or r32 = r64 and p = r32 + beta p.
__global__ void __launch_bounds__(RT) k_rel_finish(const double2 *__restrict__ r64, float2 *__restrict__ r32,
                                                   float2 *__restrict__ p32, int64_t n, int nblk,
                                                   const double *__restrict__ partial, const CgState *__restrict__ st_in,
                                                   CgState *__restrict__ st_out, double errSq, int64_t max_iter) {
    const int s = blockIdx.y, blk = blockIdx.x;
    const CgState S = st_in[s];
    if (S.status != CG_UPDATE) {
        if (blk == 0 && threadIdx.x == 0) st_out[s] = S;
        return;
    }
    const double rn = sum_partials(partial + (int64_t)s * nblk, nblk);
    CgState N = S;
    if (rn <= errSq) {
        N.status = CG_CONVERGED;
        N.rsq = rn;
    } else if (S.iters >= max_iter) {
        N.status = CG_EXHAUSTED;
        N.rsq = rn;
    } else {
        const float beta = (float)(rn / S.rsq);
        int64_t lo, hi;
        chunk_range(n, nblk, blk, lo, hi);
        const int64_t off = (int64_t)s * n;
        for (int64_t i = off + lo + threadIdx.x; i < off + hi; i += RT) {
            const double2 v = r64[i];
            const float2 rv = make_float2((float)v.x, (float)v.y);
            float2 pv = p32[i];
            pv.x = rv.x + beta * pv.x;
            pv.y = rv.y + beta * pv.y;
            r32[i] = rv;
            p32[i] = pv;
        }
        N.status = CG_ACTIVE;
        N.rsq = rn;
        N.maxr = rn;
    }
    if (blk == 0 && threadIdx.x == 0) st_out[s] = N;
}

// |b|^2 per system (for the relative true residual in the statistics)
__global__ void __launch_bounds__(RT) k_norm2(const double2 *__restrict__ v, int64_t n, int nblk,
                                              double *__restrict__ partial) {
    const int s = blockIdx.y, blk = blockIdx.x;
    int64_t lo, hi;
    chunk_range(n, nblk, blk, lo, hi);
    const int64_t off = (int64_t)s * n;
    double acc = 0;
    for (int64_t i = off + lo + threadIdx.x; i < off + hi; i += RT) acc += v[i].x * v[i].x + v[i].y * v[i].y;
    acc = block_sum(acc);
    if (threadIdx.x == 0) partial[(int64_t)s * nblk + blk] = acc;
}

struct Plan {
    int64_t nsys, n, nbatch;
    int nblk;
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
    const int64_t target = 4 * (int64_t)std::max(fm->ctx->num_sms, 1);
    int64_t nb = std::max<int64_t>(1, target / P.nsys);
    nb = std::min<int64_t>(nb, std::max<int64_t>(1, P.n / 2048));
    P.nblk = (int)std::min<int64_t>(nb, 1024);
    return P;
}

template <typename T> struct CgBufs {
    cplx_t<T> *x = nullptr, *r = nullptr, *p = nullptr, *t = nullptr;
};

// One CG iteration on the low-precision vectors (captured into the chunk graph).
template <typename T>
int cg_iteration(nslg_fm *fm, int op, const Plan &P, CgBufs<T> &v, double2 *p_pt, double *p_rr, CgState *st_a,
                 CgState *st_b, double errSq, int64_t max_iter, double update_frac, double targetSq) {
    cudaStream_t st = fm->ctx->stream;
    NSLG_TRY(fm_apply_dev<T>(fm, op, v.p, v.t, P.nbatch));
    dim3 grid(P.nblk, (unsigned)P.nsys);
    k_dot<T><<<grid, RT, 0, st>>>(v.p, v.t, P.n, P.nblk, p_pt, st_a);
    note_launch(st);
    k_cg_xr<T><<<grid, RT, 0, st>>>(v.x, v.r, v.p, v.t, P.n, P.nblk, p_pt, st_a, p_rr);
    note_launch(st);
    k_cg_p<T><<<grid, RT, 0, st>>>(v.r, v.p, P.n, P.nblk, p_rr, st_a, st_b, errSq, max_iter, update_frac, targetSq);
    note_launch(st);
    NSLG_CUDA(cudaGetLastError());
    return NSLG_OK;
}

constexpr int CHUNK = 16;  // iterations per captured graph (even: the state double buffer returns to slot 0)

template <typename T>
int run_chunk(nslg_fm *fm, int op, const Plan &P, CgBufs<T> &v, double2 *p_pt, double *p_rr, CgState *states,
              double errSq, int64_t max_iter, double update_frac, double targetSq, bool use_graph) {
    cudaStream_t st = fm->ctx->stream;
    if (!use_graph) {
        for (int j = 0; j < CHUNK; ++j) {
            CgState *a = states + (j & 1) * P.nsys, *b = states + ((j + 1) & 1) * P.nsys;
            NSLG_TRY(cg_iteration<T>(fm, op, P, v, p_pt, p_rr, a, b, errSq, max_iter, update_frac, targetSq));
        }
        return NSLG_OK;
    }
    char keybuf[256];
    std::snprintf(keybuf, sizeof keybuf, "cg:%d:%d:%lld:%lld:%lld:%llu:%.17g:%lld:%.17g:%.17g", (int)sizeof(T), op,
                  (long long)P.nsys, (long long)P.n, (long long)P.nbatch, (unsigned long long)fm->ws_generation,
                  errSq, (long long)max_iter, update_frac, targetSq);
    std::string key(keybuf);
    auto it = fm->graphs.find(key);
    if (it == fm->graphs.end()) {
        cudaGraph_t g;
        NSLG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        int rc = NSLG_OK;
        for (int j = 0; j < CHUNK && rc == NSLG_OK; ++j) {
            CgState *a = states + (j & 1) * P.nsys, *b = states + ((j + 1) & 1) * P.nsys;
            rc = cg_iteration<T>(fm, op, P, v, p_pt, p_rr, a, b, errSq, max_iter, update_frac, targetSq);
        }
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

int read_states(nslg_fm *fm, const CgState *d, int64_t nsys, std::vector<CgState> &h) {
    h.resize(nsys);
    NSLG_CUDA(cudaMemcpyAsync(h.data(), d, nsys * sizeof(CgState), cudaMemcpyDeviceToHost, fm->ctx->stream));
    NSLG_CUDA(cudaStreamSynchronize(fm->ctx->stream));
    return NSLG_OK;
}

// Final statistics: FP64 true residual |b - A x| / |b| per system.
int finish_stats(nslg_fm *fm, int op, const Plan &P, const double2 *b, const double2 *x64, double *partial,
                 const std::vector<CgState> &hs, nslg_cg_stats *stats) {
    if (!stats) return NSLG_OK;
    cudaStream_t st = fm->ctx->stream;
    double2 *t64, *r64;
    const int64_t total = P.nsys * P.n;
    NSLG_TRY(ws_get(fm, "cg_t64", total, &t64));
    NSLG_TRY(ws_get(fm, "cg_r64", total, &r64));
    NSLG_TRY(fm_apply_dev<double>(fm, op, x64, t64, P.nbatch));
    dim3 grid(P.nblk, (unsigned)P.nsys);
    k_resid<double><<<grid, RT, 0, st>>>(b, t64, r64, P.n, P.nblk, partial, nullptr, -1);
    note_launch(st);
    double *pb = partial + P.nsys * P.nblk;
    k_norm2<<<grid, RT, 0, st>>>(b, P.n, P.nblk, pb);
    note_launch(st);
    NSLG_CUDA(cudaGetLastError());
    std::vector<double> h(2 * P.nsys * P.nblk);
    NSLG_CUDA(cudaMemcpyAsync(h.data(), partial, h.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    NSLG_CUDA(cudaStreamSynchronize(st));
    double worst = 0, worst_rec = 0;
    int64_t iters = 0, conv = 0;
    for (int64_t s = 0; s < P.nsys; ++s) {
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
    stats->true_residual = worst;
    stats->recurrence_residual = worst_rec;
    stats->iterations = iters;
    stats->converged = conv;
    stats->systems = P.nsys;
    return NSLG_OK;
}

}  // namespace

// FP64 CG with the reference's semantics. b, x0 and x are device buffers of nbatch*Nt*Nx.
int cg_solve_fp64(nslg_fm *fm, int op, const double2 *b, const double2 *x0, double2 *x, int64_t nbatch, double eps,
                  int64_t max_iter, int mode, nslg_cg_stats *stats) {
    cudaStream_t st = fm->ctx->stream;
    const Plan P = make_plan(fm, nbatch, mode);
    const int64_t total = P.nsys * P.n;
    CgBufs<double> v;
    double2 *p_pt;
    double *p_rr;
    CgState *states;
    NSLG_TRY(ws_get(fm, "cg_r", total, &v.r));
    NSLG_TRY(ws_get(fm, "cg_p", total, &v.p));
    NSLG_TRY(ws_get(fm, "cg_t", total, &v.t));
    NSLG_TRY(ws_get(fm, "cg_ppt", P.nsys * P.nblk, &p_pt));
    NSLG_TRY(ws_get(fm, "cg_prr", 2 * P.nsys * P.nblk, &p_rr));
    NSLG_TRY(ws_get(fm, "cg_state", 2 * P.nsys, &states));
    double2 *t64, *r64;  // reserved up front for the exit statistics (no reallocation between solves)
    NSLG_TRY(ws_get(fm, "cg_t64", total, &t64));
    NSLG_TRY(ws_get(fm, "cg_r64", total, &r64));
    v.x = x;
    if (x0 != x) NSLG_CUDA(cudaMemcpyAsync(x, x0, total * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    const double errSq = eps * eps;
    // t = A x ; r = b - t ; p = r
    NSLG_TRY(fm_apply_dev<double>(fm, op, x, v.t, nbatch));
    dim3 grid(P.nblk, (unsigned)P.nsys);
    k_resid<double><<<grid, RT, 0, st>>>(b, v.t, v.r, P.n, P.nblk, p_rr, nullptr, -1);
    note_launch(st);
    k_start<double><<<grid, RT, 0, st>>>(v.r, nullptr, v.p, nullptr, P.n, P.nblk, p_rr, states, errSq, max_iter);
    note_launch(st);
    NSLG_CUDA(cudaGetLastError());
    std::vector<CgState> hs;
    NSLG_TRY(read_states(fm, states, P.nsys, hs));
    auto all_done = [&]() {
        for (auto &s : hs)
            if (s.status == CG_ACTIVE) return false;
        return true;
    };
    while (!all_done()) {
        NSLG_TRY(run_chunk<double>(fm, op, P, v, p_pt, p_rr, states, errSq, max_iter, 0.0, 0.0, true));
        NSLG_TRY(read_states(fm, states, P.nsys, hs));
    }
    NSLG_TRY(finish_stats(fm, op, P, b, x, p_rr, hs, stats));
    if (stats) stats->reliable_updates = 0;
    for (auto &s : hs)
        if (s.status != CG_CONVERGED) {
            set_error("CG did not converge within max_iter iterations");
            return NSLG_NOT_CONVERGED;
        }
    return NSLG_OK;
}

// Mixed precision: FP32 iterations, FP64 solution and reliable updates; stops on the FP64 true residual <= eps.
int cg_solve_mixed(nslg_fm *fm, int op, const double2 *b, const double2 *x0, double2 *x, int64_t nbatch, double eps,
                   int64_t max_iter, int mode, nslg_cg_stats *stats) {
    cudaStream_t st = fm->ctx->stream;
    const Plan P = make_plan(fm, nbatch, mode);
    const int64_t total = P.nsys * P.n;
    CgBufs<float> v;
    double2 *p_pt, *t64, *r64;
    double *p_rr;
    CgState *states;
    NSLG_TRY(ws_get(fm, "cgm_x", total, &v.x));
    NSLG_TRY(ws_get(fm, "cgm_r", total, &v.r));
    NSLG_TRY(ws_get(fm, "cgm_p", total, &v.p));
    NSLG_TRY(ws_get(fm, "cgm_t", total, &v.t));
    NSLG_TRY(ws_get(fm, "cg_t64", total, &t64));
    NSLG_TRY(ws_get(fm, "cg_r64", total, &r64));
    NSLG_TRY(ws_get(fm, "cg_ppt", P.nsys * P.nblk, &p_pt));
    NSLG_TRY(ws_get(fm, "cg_prr", 2 * P.nsys * P.nblk, &p_rr));
    NSLG_TRY(ws_get(fm, "cg_state", 2 * P.nsys, &states));
    if (x0 != x) NSLG_CUDA(cudaMemcpyAsync(x, x0, total * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    const double errSq = eps * eps;
    const double update_frac = 0.01;  // reliable update once |r|^2 fell 100x (|r| 10x) below its running maximum
    const double targetSq = errSq;
    dim3 grid(P.nblk, (unsigned)P.nsys);
    NSLG_TRY(fm_apply_dev<double>(fm, op, x, t64, nbatch));
    k_resid<float><<<grid, RT, 0, st>>>(b, t64, r64, P.n, P.nblk, p_rr, nullptr, -1);
    note_launch(st);
    k_start<float><<<grid, RT, 0, st>>>(r64, v.r, v.p, v.x, P.n, P.nblk, p_rr, states, errSq, max_iter);
    note_launch(st);
    NSLG_CUDA(cudaGetLastError());
    std::vector<CgState> hs;
    NSLG_TRY(read_states(fm, states, P.nsys, hs));
    int64_t updates = 0;
    for (;;) {
        bool active = false, pending = false;
        for (auto &s : hs) {
            active |= (s.status == CG_ACTIVE);
            pending |= (s.status == CG_UPDATE);
        }
        if (pending) {
            // x64 += x32; r64 = b - A64 x64; then converged or continue with r32 = r64
            k_rel_accum<<<grid, RT, 0, st>>>(x, v.x, P.n, P.nblk, states);
            note_launch(st);
            NSLG_CUDA(cudaGetLastError());
            NSLG_TRY(fm_apply_dev<double>(fm, op, x, t64, nbatch));
            k_resid<float><<<grid, RT, 0, st>>>(b, t64, r64, P.n, P.nblk, p_rr, states, CG_UPDATE);
            note_launch(st);
            k_rel_finish<<<grid, RT, 0, st>>>(r64, v.r, v.p, P.n, P.nblk, p_rr, states, states + P.nsys, errSq,
                                              max_iter);
            note_launch(st);
            NSLG_CUDA(cudaGetLastError());
            NSLG_CUDA(cudaMemcpyAsync(states, states + P.nsys, P.nsys * sizeof(CgState), cudaMemcpyDeviceToDevice,
                                      st));
            ++updates;
            NSLG_TRY(read_states(fm, states, P.nsys, hs));
            continue;
        }
        if (!active) break;
        NSLG_TRY(run_chunk<float>(fm, op, P, v, p_pt, p_rr, states, errSq, max_iter, update_frac, targetSq, true));
        NSLG_TRY(read_states(fm, states, P.nsys, hs));
    }
    NSLG_TRY(finish_stats(fm, op, P, b, x, p_rr, hs, stats));
    if (stats) stats->reliable_updates = updates;
    for (auto &s : hs)
        if (s.status != CG_CONVERGED) {
            set_error("CG did not converge within max_iter iterations");
            return NSLG_NOT_CONVERGED;
        }
    return NSLG_OK;
}

}  // namespace nslg
