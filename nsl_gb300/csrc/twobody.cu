// Two-body correlators from momentum wall sources on the device (TwoBodyCorrelator::measure(NumberTimeSources),
// src/NSL/Measurements/Hubbard/twoBodyCorrelationFunction.tpp:188-306, and its twelve channel functions :481-1001).
//
// For every source time tsrc = 0, Nt/Ntsrc, 2 Nt/Ntsrc, ... < Nt the wall sources W[k, s, :] (momentum k, band s)
// are placed on slice tsrc. Per species: CG on MM^dagger solves for the sources and M^dagger maps the solutions to
// columns of M^{-1}; CG on M^dagger M solves for the conjugated sources and M maps them to columns of M^{-dagger}.
// Both are shifted t -> t - tsrc with the anti-periodic sign on the wrapped slices and projected on the wall sources:
//   C[kSink, kSrc, t, sSink, sSrc] = sum_x conj(W[kSink, sSink, x]) M^{-1}(...)[kSrc, sSrc, t, x]          (corrPool)
//   D[kSink, kSrc, t, sSink, sSrc] = conj(sum_x W[kSink, sSink, x] M^{-dagger}(...)[kSrc, sSrc, t, x])     (corrPoolDag)
// For every momentum tuple (w, x, P, Q) of the caller's list the twelve isospin/spin channels are sums of
// products of two such pool entries, "direct" X(w, P)[i, l] Y(x, Q)[j, k] and "exchange" X(w, Q)[i, k] Y(x, P)[j, l],
// written to out[channel, tuple, t, i * nb + j, l * nb + k] and averaged with 1 / Ntsrc.
//
// GB300 layout of the work: all source times of a chunk go into one batched solve per (species, operator) (the
// reference runs one CG per source time); the projections are one kernel per pool (wall vectors transposed so a
// warp reads 32 consecutive sink indices); the contraction accumulates the 24 distinct pool products over the
// chunk's source times in registers and forms the twelve channels once, instead of the reference's
// 12 * nb^4 * tuples tensor-slice operations per source time.

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "fm_internal.cuh"

namespace nslg {


namespace {

// src[(s * nk + k) * nb + b, t, x] = W[k, b, x] if t == tsrc(s) else 0 (conjugated when conj_src), for the
// chunk's source times s = 0 .. ns-1 with tsrc(s) = (s0 + s) * step.
__global__ void k_wall_sources(const double2 *__restrict__ W, double2 *__restrict__ src, int nkb, int Nt, int Nx,
                               int s0, int step, int64_t total, bool conj_src) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const int x = (int)(idx % Nx);
    const int t = (int)((idx / Nx) % Nt);
    const int64_t r = idx / ((int64_t)Nx * Nt);
    const int s = (int)(r / nkb), kb = (int)(r % nkb);
    double2 v = make_double2(0, 0);
    if (t == (s0 + s) * step) {
        v = W[(int64_t)kb * Nx + x];
        if (conj_src) v.y = -v.y;
    }
    src[idx] = v;
}

// Wt[x, j] = conj(W[j, x]) (j = k * nb + b): the wall vectors transposed so that consecutive sink indices are
// consecutive in memory.
__global__ void k_wall_conj_transpose(const double2 *__restrict__ W, double2 *__restrict__ Wt, int nkb, int Nx) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)nkb * Nx) return;
    const int j = (int)(idx / Nx), x = (int)(idx % Nx);
    const double2 w = W[idx];
    Wt[(int64_t)x * nkb + j] = make_double2(w.x, -w.y);
}

// Projection of one pool. Block (r, time tile): r = (s * nk + kSrc) * nb + bSrc is a solution column, the tile
// covers PT_T slices of its time-shifted rows G'[t] = sign * G[(t + tsrc) mod Nt] (sign -1 where t + tsrc >= Nt),
// conjugated when conj_g; each thread owns sink indices j = kSink * nb + bSink and accumulates
//   pool[s, kSink, kSrc, t, bSink, bSrc] = sum_x Wt[x, j] G'[t, x]
// over x in chunks staged in shared memory. pool has strides (4 pools per source time, see below).
constexpr int PT_T = 8;    // time slices per block
constexpr int PT_X = 32;   // x chunk
constexpr int PT_J = 128;  // threads per block

__global__ void __launch_bounds__(PT_J) k_wall_pool(const double2 *__restrict__ G, const double2 *__restrict__ Wt,
                                                    double2 *__restrict__ pool, int nk, int nb, int Nt, int Nx,
                                                    int s0, int step, bool conj_g, int64_t pool_s_stride) {
    __shared__ double2 Gs[PT_T][PT_X];
    const int nkb = nk * nb;
    const int64_t r = blockIdx.x;
    const int s = (int)(r / nkb), kbSrc = (int)(r % nkb);
    const int kSrc = kbSrc / nb, bSrc = kbSrc % nb;
    const int tsrc = (s0 + s) * step;
    const int t0 = blockIdx.y * PT_T;
    const double2 *Gr = G + r * Nt * Nx;
    for (int j0 = 0; j0 < nkb; j0 += PT_J) {
        const int j = j0 + threadIdx.x;
        double2 acc[PT_T];
#pragma unroll
        for (int tt = 0; tt < PT_T; ++tt) acc[tt] = make_double2(0, 0);
        for (int x0 = 0; x0 < Nx; x0 += PT_X) {
            __syncthreads();
            for (int e = threadIdx.x; e < PT_T * PT_X; e += PT_J) {
                const int tt = e / PT_X, xx = e % PT_X;
                const int t = t0 + tt, x = x0 + xx;
                double2 g = make_double2(0, 0);
                if (t < Nt && x < Nx) {
                    const int ts = t + tsrc;
                    g = Gr[(int64_t)(ts % Nt) * Nx + x];
                    if (ts >= Nt) g = make_double2(-g.x, -g.y);
                    if (conj_g) g.y = -g.y;
                }
                Gs[tt][xx] = g;
            }
            __syncthreads();
            if (j < nkb) {
                const int xe = min(PT_X, Nx - x0);
                for (int xx = 0; xx < xe; ++xx) {
                    const double2 w = Wt[(int64_t)(x0 + xx) * nkb + j];
#pragma unroll
                    for (int tt = 0; tt < PT_T; ++tt) {
                        const double2 g = Gs[tt][xx];
                        acc[tt].x += w.x * g.x - w.y * g.y;
                        acc[tt].y += w.x * g.y + w.y * g.x;
                    }
                }
            }
        }
        if (j < nkb) {
            const int kSink = j / nb, bSink = j % nb;
            double2 *dst = pool + (int64_t)s * pool_s_stride + (((int64_t)kSink * nk + kSrc) * Nt) * nb * nb;
#pragma unroll
            for (int tt = 0; tt < PT_T; ++tt) {
                const int t = t0 + tt;
                if (t < Nt) dst[((int64_t)t * nb + bSink) * nb + bSrc] = acc[tt];
            }
        }
    }
}

// Pools of one source time: [Cp, Ch, Dp, Dh], each (nk, nk, Nt, nb, nb).
enum { POOL_CP = 0, POOL_CH = 1, POOL_DP = 2, POOL_DH = 3 };

// Ordered pool pairs (A, B) whose products the channels use; direct = A(w, P)[i, l] B(x, Q)[j, k], exchange =
// A(w, Q)[i, k] B(x, P)[j, l].
enum {
    PR_DPDP, PR_DPCH, PR_CHDP, PR_CHCH, PR_DPDH, PR_DHDP, PR_CPCH, PR_CHCP, PR_DHDH, PR_CPDH, PR_DHCP, PR_CPCP, NPAIR
};
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }

// One thread per (tuple u, t, o = (i nb + j) nb^2 + (l nb + k)); the 24 products summed over the chunk's source
// times, then the channels (in the reference's order I1S1Iz1Sz1, I1S1Iz1Sz0, I1S1Iz1Szn1, I1S1Iz0Sz1, I1S1Iz0Szn1,
// I1S1Izn1Sz1, I1S1Izn1Sz0, I1S1Izn1Szn1, I0S1Iz0Sz1, I0S1Iz0Szn1, I1S0Iz1Sz0, I1S0Izn1Sz0) scaled by `scale` and
// written (or added, accumulate) to out[ch, u, t, o].
__global__ void k_twobody_contract(const double2 *__restrict__ pools, const int *__restrict__ tuples,
                                   double2 *__restrict__ out, int64_t ntuple, int nk, int nb, int Nt, int ns,
                                   int64_t pool_s_stride, double scale, bool accumulate) {
    const int nb2 = nb * nb, nb4 = nb2 * nb2;
    const int64_t total = ntuple * Nt * nb4;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= total) return;
    const int o = (int)(idx % nb4);
    const int t = (int)((idx / nb4) % Nt);
    const int64_t u = idx / ((int64_t)nb4 * Nt);
    const int i = (o / nb2) / nb, j = (o / nb2) % nb, l = (o % nb2) / nb, k = (o % nb2) % nb;
    const int w = tuples[4 * u + 0], x = tuples[4 * u + 1], P = tuples[4 * u + 2], Q = tuples[4 * u + 3];
    const int64_t pool_n = (int64_t)nk * nk * Nt * nb2;  // one pool
    auto at = [&](int a, int b, int s1, int s2) { return (((int64_t)a * nk + b) * Nt + t) * nb2 + s1 * nb + s2; };
    const int64_t o_wP = at(w, P, i, l), o_xQ = at(x, Q, j, k), o_wQ = at(w, Q, i, k), o_xP = at(x, P, j, l);
    double2 dir[NPAIR], exc[NPAIR];
#pragma unroll
    for (int p = 0; p < NPAIR; ++p) dir[p] = exc[p] = make_double2(0, 0);
    for (int s = 0; s < ns; ++s) {
        const double2 *ps = pools + (int64_t)s * pool_s_stride;
        double2 wP[4], xQ[4], wQ[4], xP[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            wP[q] = ps[q * pool_n + o_wP];
            xQ[q] = ps[q * pool_n + o_xQ];
            wQ[q] = ps[q * pool_n + o_wQ];
            xP[q] = ps[q * pool_n + o_xP];
        }
#define NSLG_TB_PAIR(p, a, b)                               \
    dir[p] = cadd(dir[p], cmul(wP[a], xQ[b]));              \
    exc[p] = cadd(exc[p], cmul(wQ[a], xP[b]));
        NSLG_TB_PAIR(PR_DPDP, POOL_DP, POOL_DP)
        NSLG_TB_PAIR(PR_DPCH, POOL_DP, POOL_CH)
        NSLG_TB_PAIR(PR_CHDP, POOL_CH, POOL_DP)
        NSLG_TB_PAIR(PR_CHCH, POOL_CH, POOL_CH)
        NSLG_TB_PAIR(PR_DPDH, POOL_DP, POOL_DH)
        NSLG_TB_PAIR(PR_DHDP, POOL_DH, POOL_DP)
        NSLG_TB_PAIR(PR_CPCH, POOL_CP, POOL_CH)
        NSLG_TB_PAIR(PR_CHCP, POOL_CH, POOL_CP)
        NSLG_TB_PAIR(PR_DHDH, POOL_DH, POOL_DH)
        NSLG_TB_PAIR(PR_CPDH, POOL_CP, POOL_DH)
        NSLG_TB_PAIR(PR_DHCP, POOL_DH, POOL_CP)
        NSLG_TB_PAIR(PR_CPCP, POOL_CP, POOL_CP)
#undef NSLG_TB_PAIR
    }
    // the twelve channels as signed sums of the direct and exchange products
    double2 ch[12];
    ch[0] = csub(dir[PR_DPDP], exc[PR_DPDP]);
    ch[1] = cscale(csub(cadd(dir[PR_DPCH], dir[PR_CHDP]), cadd(exc[PR_DPCH], exc[PR_CHDP])), -0.5);
    ch[2] = csub(dir[PR_CHCH], exc[PR_CHCH]);
    ch[3] = cscale(csub(cadd(dir[PR_DPDH], dir[PR_DHDP]), cadd(exc[PR_DPDH], exc[PR_DHDP])), 0.5);
    ch[4] = cscale(csub(cadd(dir[PR_CPCH], dir[PR_CHCP]), cadd(exc[PR_CPCH], exc[PR_CHCP])), 0.5);
    ch[5] = csub(dir[PR_DHDH], exc[PR_DHDH]);
    ch[6] = cscale(csub(cadd(dir[PR_CPDH], dir[PR_DHCP]), cadd(exc[PR_CPDH], exc[PR_DHCP])), -0.5);
    ch[7] = csub(dir[PR_CPCP], exc[PR_CPCP]);
    ch[8] = cscale(cadd(cadd(dir[PR_DPDH], dir[PR_DHDP]), cadd(exc[PR_DPDH], exc[PR_DHDP])), 0.5);
    ch[9] = cscale(cadd(cadd(dir[PR_CPCH], dir[PR_CHCP]), cadd(exc[PR_CPCH], exc[PR_CHCP])), 0.5);
    ch[10] = cscale(cadd(cadd(dir[PR_DPCH], dir[PR_CHDP]), cadd(exc[PR_DPCH], exc[PR_CHDP])), -0.5);
    ch[11] = cscale(cadd(cadd(dir[PR_CPDH], dir[PR_DHCP]), cadd(exc[PR_CPDH], exc[PR_DHCP])), -0.5);
#pragma unroll
    for (int c = 0; c < 12; ++c) {
        double2 *dst = out + (int64_t)c * total + idx;
        const double2 v = cscale(ch[c], scale);
        *dst = accumulate ? cadd(*dst, v) : v;
    }
}

}  // namespace

// Device buffers: phi (Nt, Nx), W (nk, nb, Nx), tuples (ntuple, 4) int32 validated by the caller, out
// (12, ntuple, Nt, nb^2, nb^2). Source times are processed in chunks (at most 65535 systems and 2^28 vector
// elements per batched solve; the environment variable NSLG_TB_CHUNK lowers the number of source times per chunk
// to bound the memory). Leaves fm populated with the hole species, like the reference's last populate.
int twobody_measure(nslg_fm *fm, const double2 *phi, const double2 *W, int nk, int nb, const int *tuples,
                    int64_t ntuple, int nts, double eps, int64_t max_iter, int precision, double2 *out,
                    nslg_cg_stats *stats) {
    cudaStream_t st = fm->ctx->stream;
    const int Nt = (int)fm->Nt, Nx = (int)fm->Nx;
    const int nkb = nk * nb;
    const int step = Nt / nts;
    const int nsrc = (Nt + step - 1) / step;  // the reference's loop tsrc = 0, step, ... < Nt
    const int64_t per_src = (int64_t)nkb * Nt * Nx;
    int chunk = (int)std::max<int64_t>(1, std::min<int64_t>(65535 / nkb, ((int64_t)1 << 28) / per_src));
    if (const char *e = std::getenv("NSLG_TB_CHUNK")) chunk = std::max(1, std::min(chunk, std::atoi(e)));
    chunk = std::min(chunk, nsrc);
    const int64_t rmax = (int64_t)chunk * nkb;
    const int64_t vec = rmax * Nt * Nx;
    const int64_t pool_n = (int64_t)nk * nk * Nt * nb * nb;
    const int64_t pool_s_stride = 4 * pool_n;

    double2 *src, *x1, *g1, *wt, *pools;
    NSLG_TRY(ws_get(fm, "tb_src", (size_t)vec, &src));
    NSLG_TRY(ws_get(fm, "tb_x", (size_t)vec, &x1));
    NSLG_TRY(ws_get(fm, "tb_g", (size_t)vec, &g1));
    NSLG_TRY(ws_get(fm, "tb_wt", (size_t)nkb * Nx, &wt));
    NSLG_TRY(ws_get(fm, "tb_pools", (size_t)chunk * pool_s_stride, &pools));
    k_wall_conj_transpose<<<(unsigned)ceil_div((int64_t)nkb * Nx, 256), 256, 0, st>>>(W, wt, nkb, Nx);
    note_launch(st);

    nslg_cg_stats agg{};
    agg.true_residual = 0;
    int rc_all = NSLG_OK;
    auto merge = [&](const nslg_cg_stats &s) {
        agg.iterations = std::max(agg.iterations, s.iterations);
        agg.reliable_updates += s.reliable_updates;
        agg.converged += s.converged;
        agg.systems += s.systems;
        agg.recurrence_residual = std::max(agg.recurrence_residual, s.recurrence_residual);
        agg.true_residual = std::max(agg.true_residual, s.true_residual);
        agg.escalated = std::max(agg.escalated, s.escalated);
    };
    const int species[2] = {NSLG_PARTICLE, NSLG_HOLE};
    for (int s0 = 0; s0 < nsrc; s0 += chunk) {
        const int ns = std::min(chunk, nsrc - s0);
        const int64_t R = (int64_t)ns * nkb;
        const int64_t total = R * Nt * Nx;
        for (int sp = 0; sp < 2; ++sp) {
            NSLG_TRY(populate_dev(fm, phi, species[sp]));
            for (int which = 0; which < 2; ++which) {
                // which 0: C from M^dagger (MM^dagger)^{-1} src; which 1: D from M (M^dagger M)^{-1} conj(src)
                const int op = which == 0 ? NSLG_OP_MMDAGGER : NSLG_OP_MDAGGERM;
                k_wall_sources<<<(unsigned)ceil_div(total, 256), 256, 0, st>>>(W, src, nkb, Nt, Nx, s0, step, total,
                                                                               which == 1);
                note_launch(st);
                NSLG_TRY(prepare_apply(fm, op, R, precision));
                nslg_cg_stats cs{};
                const int rc = cg_solve(fm, op, src, src, x1, R, eps, max_iter, NSLG_CG_PER_RHS, precision,
                                        NSLG_STOP_TRUE_RESIDUAL, &cs);
                if (rc != NSLG_OK && rc != NSLG_NOT_CONVERGED) return rc;
                if (rc == NSLG_NOT_CONVERGED) rc_all = NSLG_NOT_CONVERGED;
                merge(cs);
                const int back = which == 0 ? NSLG_OP_MDAGGER : NSLG_OP_M;
                if (precision == NSLG_PREC_BF16_SPLIT) NSLG_TRY(fm_apply_dev<BF16Split>(fm, back, x1, g1, R));
                else NSLG_TRY(fm_apply_dev<double>(fm, back, x1, g1, R));
                const int q = which == 0 ? (sp == 0 ? POOL_CP : POOL_CH) : (sp == 0 ? POOL_DP : POOL_DH);
                k_wall_pool<<<dim3((unsigned)R, (unsigned)ceil_div(Nt, PT_T)), PT_J, 0, st>>>(
                    g1, wt, pools + q * pool_n, nk, nb, Nt, Nx, s0, step, which == 1, pool_s_stride);
                note_launch(st);
            }
        }
        const int64_t ctot = ntuple * Nt * (int64_t)nb * nb * nb * nb;
        if (ctot > 0) {
            k_twobody_contract<<<(unsigned)ceil_div(ctot, 128), 128, 0, st>>>(
                pools, tuples, out, ntuple, nk, nb, Nt, ns, pool_s_stride, 1.0 / nts, s0 > 0);
            note_launch(st);
        }
    }
    NSLG_CUDA(cudaGetLastError());
    if (stats) *stats = agg;
    return rc_all;
}

}  // namespace nslg
