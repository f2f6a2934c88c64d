// Hubbard actions, forces and the leapfrog trajectory on the device (FP64).
//
//   gauge action  S_g = sum phi^2 / (2 U~),  force_g = -phi / U~                 (hubbardGaugeAction.tpp:55-67)
//   fermion action S_f = -(log det M_P + log det M_H),
//                 force_f = -(grad log det M_P - grad log det M_H)              (hubbardFermiAction.tpp:68-113)
//   leapfrog: p += eps/2 F(q); q += eps p; (Nmd-1) x {p += eps F(q); q += eps p}; p += eps/2 F(q)
//                                                                               (leapfrog.tpp:35-58)
//   LeapfrogRealForce zeroes Im F before every kick (leapfrogRealForce.tpp:44-70).
// A force evaluation is two gradient evaluations (particle, hole) plus one fused elementwise kernel that forms the
// total force and applies the momentum kick and the following drift.

#include <cmath>

#include <cstdio>
#include <string>
#include <vector>

#include "fm_internal.cuh"

namespace nslg {

int fm_logdet(nslg_fm *fm, double2 *out);
int fm_grad_logdet(nslg_fm *fm, double2 *out);

namespace {

// F = [gauge] -phi / Ut  +  [fermion] -(gP - gH);  optional Re projection.
// Then p += ckick F and, if cdrift != 0, q += cdrift p (the drift that follows a kick in leapfrog).
__global__ void k_kick_drift(const double2 *__restrict__ gP, const double2 *__restrict__ gH, double2 *q, double2 *p,
                             double2 *F_out, double2 Ut_inv_neg, int terms, int real_force, double ckick,
                             double cdrift, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double2 phi = q[i];
    double2 F = make_double2(0, 0);
    if (terms & 1) F = cmul(phi, Ut_inv_neg);
    if (terms & 2) {
        F.x -= gP[i].x - gH[i].x;
        F.y -= gP[i].y - gH[i].y;
    }
    if (real_force) F.y = 0.0;
    if (F_out) F_out[i] = F;
    if (p) {
        double2 pv = p[i];
        pv.x += ckick * F.x;
        pv.y += ckick * F.y;
        p[i] = pv;
        if (cdrift != 0.0) {
            double2 qv = phi;
            qv.x += cdrift * pv.x;
            qv.y += cdrift * pv.y;
            q[i] = qv;
        }
    }
}

// Phases of both species of nconf configurations: g = 2 b + s (s = 0 particle, sgn +1; s = 1 hole, sgn -1),
// ph[g] = exp(i sgn phi_b + sgn mu~), ph_inv[g] = exp(-i sgn phi_b - sgn mu~) (the populate formulas,
// hubbardExp.hpp:95-144); ph may be null.
__global__ void k_phases_species(const double2 *__restrict__ phi, double2 *__restrict__ ph, double2 *__restrict__ ph_inv,
                                 double2 mu, int64_t nconf, int64_t m) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 2 * nconf * m) return;
    const int64_t g = idx / m, i = idx % m;
    const int sgn = (g & 1) ? -1 : 1;
    const double2 f = phi[(g >> 1) * m + i];
    const double a = sgn * (mu.x - f.y);
    const double b = sgn * (f.x + mu.y);
    double sb, cb;
    sincos(b, &sb, &cb);
    const double ea = exp(a), eia = exp(-a);
    if (ph) ph[idx] = make_double2(ea * cb, ea * sb);
    ph_inv[idx] = make_double2(eia * cb, -eia * sb);
}

// kick_drift for nconf configurations with the gradients laid out g = 2 b + s: F_b = -phi_b / U~ - (g_2b - g_2b+1).
// With uin_cfg the gauge coupling is per configuration: -1 / U~_b = uin_cfg[b].
__global__ void k_kick_drift_many(const double2 *__restrict__ g2, double2 *q, double2 *p, double2 Ut_inv_neg,
                                  const double2 *__restrict__ uin_cfg, int terms, int real_force, double ckick,
                                  double cdrift, int64_t m, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t b = i / m, j = i % m;
    const double2 phi = q[i];
    double2 F = make_double2(0, 0);
    if (terms & 1) F = cmul(phi, uin_cfg ? uin_cfg[b] : Ut_inv_neg);
    if (terms & 2) {
        const double2 gp = g2[2 * b * m + j], gh = g2[(2 * b + 1) * m + j];
        F.x -= gp.x - gh.x;
        F.y -= gp.y - gh.y;
    }
    if (real_force) F.y = 0.0;
    double2 pv = p[i];
    pv.x += ckick * F.x;
    pv.y += ckick * F.y;
    p[i] = pv;
    if (cdrift != 0.0) {
        double2 qv = phi;
        qv.x += cdrift * pv.x;
        qv.y += cdrift * pv.y;
        q[i] = qv;
    }
}

// S_b = sum phi_b^2 (complex square) per configuration, one block each
__global__ void k_sumsq_many(const double2 *a, int64_t m, double2 *out) {
    __shared__ double2 red[256];
    const double2 *v = a + (int64_t)blockIdx.x * m;
    double2 acc = make_double2(0, 0);
    for (int64_t i = threadIdx.x; i < m; i += 256) {
        const double2 x = v[i];
        acc.x += x.x * x.x - x.y * x.y;
        acc.y += 2.0 * x.x * x.y;
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
    if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

__global__ void k_drift(double2 *q, const double2 *p, double c, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    q[i].x += c * p[i].x;
    q[i].y += c * p[i].y;
}

// sum a*a (complex square, not |a|^2) in one block, deterministic.
__global__ void k_sumsq(const double2 *a, int64_t n, double2 *out) {
    __shared__ double2 red[256];
    double2 acc = make_double2(0, 0);
    for (int64_t i = threadIdx.x; i < n; i += 256) {
        const double2 v = a[i];
        acc.x += v.x * v.x - v.y * v.y;
        acc.y += 2.0 * v.x * v.y;
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
    if (threadIdx.x == 0) *out = red[0];
}

double2 cdivd(double2 a, double2 b) {
    const double d = b.x * b.x + b.y * b.y;
    return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}

}  // namespace

// populate(phi, species) from a device buffer (phi may be fm->phi itself)
int populate_dev(nslg_fm *fm, const double2 *phi, int species) {
    fm->species = species;
    fm->sgn = species == NSLG_PARTICLE ? 1 : -1;
    if (phi != fm->phi)
        NSLG_CUDA(cudaMemcpyAsync(fm->phi, phi, (size_t)fm->Nt * fm->Nx * sizeof(double2), cudaMemcpyDeviceToDevice,
                                  fm->ctx->stream));
    NSLG_TRY(compute_phases(fm));
    fm->populated = true;
    return NSLG_OK;
}

namespace {

// The time-slice factors of the gradient for both species: exp(-sgn delta K) (Exp) or 1 - sgn delta K (Diag).
int grad_factors(nslg_fm *fm, const double2 **EP, const double2 **EH) {
    const ExpEntry *e[2];
    for (int s = 0; s < 2; ++s) {
        const int sgn = s == 0 ? 1 : -1;
        if (fm->kind == NSLG_FM_DIAG) NSLG_TRY(get_lin(fm, make_double2(sgn * fm->delta.x, sgn * fm->delta.y), 1, &e[s]));
        else NSLG_TRY(get_exp(fm, make_double2(-sgn * fm->delta.x, -sgn * fm->delta.y), &e[s]));
    }
    *EP = e[0]->full;
    *EH = e[1]->full;
    return NSLG_OK;
}

// The FP64 gradients of both species of nconf configurations phi (nconf, Nt, Nx) in one batched pass:
// g2 = (nconf, 2, Nt, Nx), species particle then hole per configuration.
int fermion_grads_many(nslg_fm *fm, const double2 *phi, int64_t nconf, double2 *g2) {
    const int64_t m = fm->Nt * fm->Nx;
    double2 *ph_inv, *ph = nullptr;
    NSLG_TRY(ws_get(fm, "hmc_phinv2", (size_t)(2 * nconf * m), &ph_inv));
    const bool strat = use_stratified_grad(fm);
    if (strat) NSLG_TRY(ws_get(fm, "hmc_ph2", (size_t)(2 * nconf * m), &ph));
    k_phases_species<<<(unsigned)ceil_div(2 * nconf * m, 256), 256, 0, fm->ctx->stream>>>(phi, ph, ph_inv,
                                                                                         fm->mu_tilde, nconf, m);
    note_launch(fm->ctx->stream);
    if (strat) {
        // stratified: matrix 2b + s has E' = exp(-sgn_s delta K) and E = exp(sgn_s delta K)
        const ExpEntry *e[2][2];
        for (int sp = 0; sp < 2; ++sp) {
            const int sgn = sp == 0 ? 1 : -1;
            NSLG_TRY(get_exp(fm, make_double2(-sgn * fm->delta.x, -sgn * fm->delta.y), &e[sp][0]));
            NSLG_TRY(get_exp(fm, make_double2(sgn * fm->delta.x, sgn * fm->delta.y), &e[sp][1]));
        }
        std::vector<const ExpEntry *> Ep(2 * nconf), Ed(2 * nconf);
        for (int64_t g = 0; g < 2 * nconf; ++g) {
            Ep[g] = e[g & 1][0];
            Ed[g] = e[g & 1][1];
        }
        NSLG_TRY(grad_logdet_strat(fm, (int)(2 * nconf), Ep.data(), Ed.data(), ph, ph_inv, g2));
    } else {
        const double2 *EP, *EH;
        NSLG_TRY(grad_factors(fm, &EP, &EH));
        NSLG_TRY(grad_logdet_many(fm, (int)(2 * nconf), EP, EH, 1, ph_inv, g2));
    }
    if (fm->defer_checks) return NSLG_OK;  // the captured trajectory checks the sticky flag after its replay
    int *sing;
    NSLG_TRY(ws_get(fm, "lu_singular", 1, &sing));
    int h = 0;
    NSLG_CUDA(cudaMemcpyAsync(&h, sing, sizeof(int), cudaMemcpyDeviceToHost, fm->ctx->stream));
    NSLG_CUDA(cudaStreamSynchronize(fm->ctx->stream));
    NSLG_REQUIRE(!h, NSLG_ERR_ARG, "gradLogDetM: 1 + A^{-1} is singular");
    return NSLG_OK;
}

// The split-BF16 gradients of both species of phi (exponential discretisation, real factors, Nx <= 2048) into
// g2 = (2, Nt, Nx): tensor-core chains per species, one batched FP64 LU and solve for the pair. Returns
// NSLG_ERR_UNSUPPORTED (nothing launched) when the form does not apply.
int fermion_grads_tc_pair(nslg_fm *fm, const double2 *phi, double2 *g2) {
    const int64_t m = fm->Nt * fm->Nx;
    if (fm->kind != NSLG_FM_EXP || fm->Nx > 2048) return NSLG_ERR_UNSUPPORTED;
    const ExpEntry *E[2];
    for (int s = 0; s < 2; ++s) {
        const int sgn = s == 0 ? 1 : -1;
        NSLG_TRY(get_exp(fm, make_double2(-sgn * fm->delta.x, -sgn * fm->delta.y), &E[s]));
        if (!E[s]->is_real) return NSLG_ERR_UNSUPPORTED;
    }
    double2 *ph_inv;
    NSLG_TRY(ws_get(fm, "hmc_phinv2", (size_t)(2 * m), &ph_inv));
    k_phases_species<<<(unsigned)ceil_div(2 * m, 256), 256, 0, fm->ctx->stream>>>(phi, nullptr, ph_inv, fm->mu_tilde,
                                                                                 1, m);
    note_launch(fm->ctx->stream);
    NSLG_TRY(grad_logdet_tc_many(fm, 2, E, ph_inv, g2));
    if (fm->defer_checks) return NSLG_OK;
    int *sing;
    NSLG_TRY(ws_get(fm, "lu_singular", 1, &sing));
    int h = 0;
    NSLG_CUDA(cudaMemcpyAsync(&h, sing, sizeof(int), cudaMemcpyDeviceToHost, fm->ctx->stream));
    NSLG_CUDA(cudaStreamSynchronize(fm->ctx->stream));
    NSLG_REQUIRE(!h, NSLG_ERR_ARG, "gradLogDetM: 1 + A^{-1} is singular");
    return NSLG_OK;
}

// gP = grad log det M_P(phi), gH = grad log det M_H(phi); leaves fm populated with the hole species. When
// gH = gP + Nt * Nx both species are computed as a pair: in FP64 as one batch of two matrices, in split-BF16 with
// the LU of the pair batched; otherwise one species after the other.
int fermion_grads(nslg_fm *fm, const double2 *phi, double2 *gP, double2 *gH) {
    if (gH == gP + fm->Nt * fm->Nx) {
        // small lattices (Nx <= 32) take the FP64 pair whatever the force precision: their gradient is a few
        // latency-bound launches (scans, one Gauss-Jordan inverse) that tensor-core products would not shorten
        if (fm->force_precision == NSLG_PREC_FP64 || fm->Nx <= 32 || use_stratified_grad(fm)) {
            NSLG_TRY(fermion_grads_many(fm, phi, 1, gP));
            return populate_dev(fm, phi, NSLG_HOLE);
        }
        if (fm->force_precision == NSLG_PREC_BF16_SPLIT) {
            const int rc = fermion_grads_tc_pair(fm, phi, gP);
            if (rc == NSLG_OK) return populate_dev(fm, phi, NSLG_HOLE);
            if (rc != NSLG_ERR_UNSUPPORTED) return rc;
        }
    }
    NSLG_TRY(populate_dev(fm, phi, NSLG_PARTICLE));
    NSLG_TRY(fm_grad_logdet(fm, gP));
    NSLG_TRY(populate_dev(fm, phi, NSLG_HOLE));
    NSLG_TRY(fm_grad_logdet(fm, gH));
    return NSLG_OK;
}

}  // namespace

int hubbard_force_dev(nslg_fm *fm, const double2 *phi, double2 Ut, int terms, int real_force, double2 *F) {
    const int64_t n = fm->Nt * fm->Nx;
    double2 *gP = nullptr, *gH = nullptr;
    if (terms & 2) {
        NSLG_TRY(ws_get(fm, "hmc_g2", 2 * n, &gP));
        gH = gP + n;
        NSLG_TRY(fermion_grads(fm, phi, gP, gH));
    }
    const double2 uin = cdivd(make_double2(-1, 0), Ut);
    k_kick_drift<<<(unsigned)ceil_div(n, 256), 256, 0, fm->ctx->stream>>>(
        gP, gH, const_cast<double2 *>(phi), nullptr, F, uin, terms, real_force, 0.0, 0.0, n);
    note_launch(fm->ctx->stream);
    NSLG_CUDA(cudaGetLastError());
    return NSLG_OK;
}

int hubbard_eval_dev(nslg_fm *fm, const double2 *phi, double2 Ut, int terms, double2 *S) {
    double2 total = make_double2(0, 0);
    cudaStream_t st = fm->ctx->stream;
    if (terms & 1) {
        double2 *d;
        NSLG_TRY(ws_get(fm, "hmc_red", 1, &d));
        k_sumsq<<<1, 256, 0, st>>>(phi, fm->Nt * fm->Nx, d);
        note_launch(st);
        double2 h;
        NSLG_CUDA(cudaMemcpyAsync(&h, d, sizeof(double2), cudaMemcpyDeviceToHost, st));
        NSLG_CUDA(cudaStreamSynchronize(st));
        const double2 g = cdivd(h, make_double2(2 * Ut.x, 2 * Ut.y));
        total.x += g.x;
        total.y += g.y;
    }
    if (terms & 2) {
        double2 lp, lh;
        NSLG_TRY(populate_dev(fm, phi, NSLG_PARTICLE));
        NSLG_TRY(fm_logdet(fm, &lp));
        NSLG_TRY(populate_dev(fm, phi, NSLG_HOLE));
        NSLG_TRY(fm_logdet(fm, &lh));
        total.x -= lp.x + lh.x;
        total.y -= lp.y + lh.y;
    }
    *S = total;
    return NSLG_OK;
}

// q[b] = q_new[b] for every configuration b whose accept[b] is non-zero (the Metropolis selection of many chains).
__global__ void k_accept_select(const int *__restrict__ accept, const double2 *__restrict__ q_new,
                                double2 *__restrict__ q, int64_t m, int64_t nconf) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m * nconf) return;
    if (accept[i / m]) q[i] = q_new[i];
}

// out[b] = 1/2 sum p_b^2 (complex square) for nconf momenta p (nconf, Nt, Nx) on the device; out on the host.
int kinetic_batch_dev(nslg_fm *fm, const double2 *p, int64_t nconf, double2 *out) {
    cudaStream_t st = fm->ctx->stream;
    double2 *d;
    NSLG_TRY(ws_get(fm, "hmc_kinb", (size_t)nconf, &d));
    k_sumsq_many<<<(unsigned)nconf, 256, 0, st>>>(p, fm->Nt * fm->Nx, d);
    note_launch(st);
    NSLG_CUDA(cudaGetLastError());
    NSLG_CUDA(cudaMemcpyAsync(out, d, nconf * sizeof(double2), cudaMemcpyDeviceToHost, st));
    NSLG_CUDA(cudaStreamSynchronize(st));
    for (int64_t b = 0; b < nconf; ++b) out[b] = make_double2(0.5 * out[b].x, 0.5 * out[b].y);
    return NSLG_OK;
}

// q[b] = q_new[b] where accept[b] (host array of nconf flags) is non-zero; q and q_new on the device.
int accept_batch_dev(nslg_fm *fm, int64_t nconf, const int *accept, const double2 *q_new, double2 *q) {
    cudaStream_t st = fm->ctx->stream;
    const int64_t m = fm->Nt * fm->Nx;
    int *d;
    NSLG_TRY(ws_get(fm, "hmc_accept", (size_t)nconf, &d));
    NSLG_CUDA(cudaMemcpyAsync(d, accept, nconf * sizeof(int), cudaMemcpyHostToDevice, st));
    k_accept_select<<<(unsigned)ceil_div(m * nconf, 256), 256, 0, st>>>(d, q_new, q, m, nconf);
    note_launch(st);
    NSLG_CUDA(cudaGetLastError());
    // the flags' host buffer belongs to the caller: the copy has to finish before the call returns
    NSLG_CUDA(cudaStreamSynchronize(st));
    return NSLG_OK;
}

double2 sum_squares_host(nslg_fm *fm, const double2 *a, int *rc) {
    double2 *d;
    *rc = ws_get(fm, "hmc_red", 1, &d);
    double2 h = make_double2(0, 0);
    if (*rc != NSLG_OK) return h;
    k_sumsq<<<1, 256, 0, fm->ctx->stream>>>(a, fm->Nt * fm->Nx, d);
    note_launch(fm->ctx->stream);
    if (cudaMemcpyAsync(&h, d, sizeof(double2), cudaMemcpyDeviceToHost, fm->ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(fm->ctx->stream) != cudaSuccess) {
        set_error("sum of squares: CUDA failure");
        *rc = NSLG_ERR_CUDA;
    }
    return h;
}

// Full leapfrog trajectory on device buffers q, p (updated in place).
namespace {

// The Nmd + 1 force evaluations with their fused kicks and drifts, enqueued on the handle's stream; nconf
// configurations (q, p of shape (nconf, Nt, Nx)) advance together, their gradients batched (FP64 for nconf > 1).
// uin_cfg (device, nconf values, nconf > 1 only): -1 / U~ per configuration instead of the common Ut.
int leapfrog_steps(nslg_fm *fm, double2 *q, double2 *p, double2 Ut, const double2 *uin_cfg, double traj,
                   int64_t nmd, int backward, int real_force, int terms, int64_t nconf) {
    const int64_t m = fm->Nt * fm->Nx, n = nconf * m;
    cudaStream_t st = fm->ctx->stream;
    double eps = traj / (double)nmd;
    if (backward) eps = -eps;
    double2 *gP = nullptr, *gH = nullptr;
    NSLG_TRY(ws_get(fm, "hmc_g2", 2 * n, &gP));
    gH = gP + m;
    const double2 uin = cdivd(make_double2(-1, 0), Ut);
    const unsigned grid = (unsigned)ceil_div(n, 256);
    for (int64_t step = 0; step <= nmd; ++step) {
        const double ck = (step == 0 || step == nmd) ? 0.5 * eps : eps;
        const double cd = (step == nmd) ? 0.0 : eps;
        if (nconf == 1) {
            if (terms & 2) NSLG_TRY(fermion_grads(fm, q, gP, gH));
            k_kick_drift<<<grid, 256, 0, st>>>(gP, gH, q, p, nullptr, uin, terms, real_force, ck, cd, n);
        } else {
            if (terms & 2) NSLG_TRY(fermion_grads_many(fm, q, nconf, gP));
            k_kick_drift_many<<<grid, 256, 0, st>>>(gP, q, p, uin, uin_cfg, terms, real_force, ck, cd, m, n);
        }
        note_launch(st);
    }
    NSLG_CUDA(cudaGetLastError());
    return NSLG_OK;
}

}  // namespace

// A trajectory on the workspace buffers q, p. The first call for a given (Nmd, length, direction, terms, U~) runs
// eagerly, which builds every workspace and exp(delta K) entry; the second captures the same launches into a CUDA
// graph (thousands of small kernels on small lattices, so launch latency would dominate) and later calls replay it.
// Inside the graph the gradients' singularity checks are deferred: the LU's singular flag stays sticky over the
// trajectory and is read once after the replay. With uin_cfg (a device buffer of nconf couplings -1 / U~_b whose
// address the graph bakes in and whose values the caller sets before each call) U~ is per configuration.
namespace {

std::string lf_key(const nslg_fm *fm, const double2 *q, const double2 *p, double2 Ut, const double2 *uin_cfg,
                   double traj, int64_t nmd, int backward, int real_force, int terms, int64_t nconf) {
    char keybuf[320];
    if (uin_cfg) Ut = make_double2(0, 0);
    std::snprintf(keybuf, sizeof keybuf, "lf:%lld:%.17g:%d:%d:%d:%.17g:%.17g:%llu:%p:%p:%p:%d:%lld", (long long)nmd,
                  traj, backward, real_force, terms, Ut.x, Ut.y, (unsigned long long)fm->ws_generation, (void *)q,
                  (void *)p, (void *)uin_cfg, fm->force_precision, (long long)nconf);
    return std::string(keybuf);
}

// After a trajectory (eager or replayed) of one configuration: the last populate was the hole species.
void after_trajectory(nslg_fm *fm, int terms, int64_t nconf) {
    if ((terms & 2) && nconf == 1) {
        fm->species = NSLG_HOLE;
        fm->sgn = -1;
        fm->populated = true;
    }
}

}  // namespace

int leapfrog_dev(nslg_fm *fm, double2 *q, double2 *p, double2 Ut, double traj, int64_t nmd, int backward,
                 int real_force, int terms, int64_t nconf, const double2 *uin_cfg) {
    cudaStream_t st = fm->ctx->stream;
    auto make_key = [&]() { return lf_key(fm, q, p, Ut, uin_cfg, traj, nmd, backward, real_force, terms, nconf); };
    std::string key = make_key();
    auto it = fm->graphs.find(key);
    if (it == fm->graphs.end() && !fm->lf_seen.count(key)) {
        NSLG_TRY(leapfrog_steps(fm, q, p, Ut, uin_cfg, traj, nmd, backward, real_force, terms, nconf));
        fm->lf_seen[make_key()] = 1;  // the key after the eager run's allocations
        return NSLG_OK;
    }
    int *sing = nullptr;
    if (terms & 2) NSLG_TRY(ws_get(fm, "lu_singular", 1, &sing));
    if (it == fm->graphs.end()) {
        cudaGraph_t g;
        NSLG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        fm->defer_checks = true;
        const int rc = leapfrog_steps(fm, q, p, Ut, uin_cfg, traj, nmd, backward, real_force, terms, nconf);
        fm->defer_checks = false;
        const cudaError_t ce = cudaStreamEndCapture(st, &g);
        if (rc != NSLG_OK) {
            if (ce == cudaSuccess) cudaGraphDestroy(g);
            return rc;
        }
        NSLG_CUDA(ce);
        if (make_key() != key) {
            cudaGraphDestroy(g);
            NSLG_REQUIRE(false, NSLG_ERR_STATE, "leapfrog: a workspace moved while the trajectory was captured");
        }
        size_t nodes = 0;
        cudaGraphGetNodes(g, nullptr, &nodes);
        cudaGraphExec_t ex;
        const cudaError_t ie = cudaGraphInstantiate(&ex, g, 0);
        if (ie != cudaSuccess) cudaGraphDestroy(g);
        NSLG_CUDA(ie);
        it = fm->graphs.emplace(key, ex).first;
        fm->graph_kernels[key] = nodes;
        fm->graph_defs[key] = g;
    }
    if (sing) NSLG_CUDA(cudaMemsetAsync(sing, 0, sizeof(int), st));
    NSLG_CUDA(cudaGraphLaunch(it->second, st));
    note_launch(st, fm->graph_kernels[key]);
    after_trajectory(fm, terms, nconf);
    if (sing) {
        int h = 0;
        NSLG_CUDA(cudaMemcpyAsync(&h, sing, sizeof(int), cudaMemcpyDeviceToHost, st));
        NSLG_CUDA(cudaStreamSynchronize(st));
        NSLG_REQUIRE(!h, NSLG_ERR_ARG, "gradLogDetM: 1 + A^{-1} is singular");
    }
    return NSLG_OK;
}

// Trajectories of a group of handles on one context (each its own lattice shape, nconf[g] configurations on its
// workspace buffers q[g], p[g], couplings Ut[g] for one configuration or uin_cfg[g] for several). Once every member
// has a captured trajectory graph, the members' graphs become the independent branches of one parent graph (one
// launch; the branches run concurrently); until then each member runs (eagerly, then captured) on its own.
int leapfrog_group_dev(int ng, nslg_fm *const *fms, const int64_t *nconf, double2 *const *q, double2 *const *p,
                       const double2 *Ut, const double2 *const *uin_cfg, double traj, int64_t nmd, int backward,
                       int real_force, int terms) {
    nslg_fm *f0 = fms[0];
    cudaStream_t st = f0->ctx->stream;
    std::vector<std::string> keys(ng);
    bool ready = true;
    for (int g = 0; g < ng; ++g) {
        keys[g] = lf_key(fms[g], q[g], p[g], Ut[g], uin_cfg[g], traj, nmd, backward, real_force, terms, nconf[g]);
        ready &= fms[g]->graph_defs.count(keys[g]) > 0;
    }
    if (!ready || ng == 1) {
        for (int g = 0; g < ng; ++g)
            NSLG_TRY(leapfrog_dev(fms[g], q[g], p[g], Ut[g], traj, nmd, backward, real_force, terms, nconf[g],
                                  uin_cfg[g]));
        return NSLG_OK;
    }
    std::string pk = "lfg";
    for (int g = 0; g < ng; ++g) pk += "|" + std::to_string(fms[g]->uid) + "#" + keys[g];
    auto it = f0->graphs.find(pk);
    if (it == f0->graphs.end()) {
        cudaGraph_t parent;
        NSLG_CUDA(cudaGraphCreate(&parent, 0));
        uint64_t nodes = 0;
        for (int g = 0; g < ng; ++g) {
            cudaGraphNode_t node;
            const cudaError_t e = cudaGraphAddChildGraphNode(&node, parent, nullptr, 0, fms[g]->graph_defs[keys[g]]);
            if (e != cudaSuccess) cudaGraphDestroy(parent);
            NSLG_CUDA(e);
            nodes += fms[g]->graph_kernels[keys[g]];
        }
        cudaGraphExec_t ex;
        const cudaError_t ie = cudaGraphInstantiate(&ex, parent, 0);
        cudaGraphDestroy(parent);
        NSLG_CUDA(ie);
        it = f0->graphs.emplace(pk, ex).first;
        f0->graph_kernels[pk] = nodes;
    }
    std::vector<int *> sing(ng, nullptr);
    if (terms & 2)
        for (int g = 0; g < ng; ++g) {
            NSLG_TRY(ws_get(fms[g], "lu_singular", 1, &sing[g]));
            NSLG_CUDA(cudaMemsetAsync(sing[g], 0, sizeof(int), st));
        }
    NSLG_CUDA(cudaGraphLaunch(it->second, st));
    note_launch(st, f0->graph_kernels[pk]);
    std::vector<int> h(ng, 0);
    for (int g = 0; g < ng; ++g) {
        after_trajectory(fms[g], terms, nconf[g]);
        if (sing[g]) NSLG_CUDA(cudaMemcpyAsync(&h[g], sing[g], sizeof(int), cudaMemcpyDeviceToHost, st));
    }
    NSLG_CUDA(cudaStreamSynchronize(st));
    for (int g = 0; g < ng; ++g) NSLG_REQUIRE(!h[g], NSLG_ERR_ARG, "gradLogDetM: 1 + A^{-1} is singular");
    return NSLG_OK;
}

// S_b for nconf configurations phi (nconf, Nt, Nx) on the device into S (host, nconf values): the gauge term per
// configuration from one reduction launch, the fermion term -(log det M_P + log det M_H) from one batched log det of
// all 2 nconf matrices (exponential discretisation; the diagonal one evaluates configuration by configuration).
// Ut_cfg (host, nconf values, or null for Ut): U~ per configuration.
int hubbard_eval_batch_dev(nslg_fm *fm, const double2 *phi, int64_t nconf, double2 Ut, int terms, double2 *S,
                           const double2 *Ut_cfg) {
    cudaStream_t st = fm->ctx->stream;
    const int64_t m = fm->Nt * fm->Nx;
    std::vector<double2> total(nconf, make_double2(0, 0));
    if (terms & 1) {
        double2 *d;
        NSLG_TRY(ws_get(fm, "hmc_redb", (size_t)nconf, &d));
        k_sumsq_many<<<(unsigned)nconf, 256, 0, st>>>(phi, m, d);
        note_launch(st);
        std::vector<double2> h(nconf);
        NSLG_CUDA(cudaMemcpyAsync(h.data(), d, nconf * sizeof(double2), cudaMemcpyDeviceToHost, st));
        NSLG_CUDA(cudaStreamSynchronize(st));
        for (int64_t b = 0; b < nconf; ++b) {
            const double2 u = Ut_cfg ? Ut_cfg[b] : Ut;
            total[b] = cdivd(h[b], make_double2(2 * u.x, 2 * u.y));
        }
    }
    if (terms & 2) {
        std::vector<double2> ld(2 * nconf);
        if (fm->kind == NSLG_FM_EXP) {
            double2 *ph, *ph_inv;
            NSLG_TRY(ws_get(fm, "hmc_ph2", (size_t)(2 * nconf * m), &ph));
            NSLG_TRY(ws_get(fm, "hmc_phinv2", (size_t)(2 * nconf * m), &ph_inv));
            k_phases_species<<<(unsigned)ceil_div(2 * nconf * m, 256), 256, 0, st>>>(phi, ph, ph_inv, fm->mu_tilde,
                                                                                    nconf, m);
            note_launch(st);
            const ExpEntry *EP, *EH;  // B_t = exp(sgn delta K) diag(phiExp[t + 1])
            NSLG_TRY(get_exp(fm, fm->delta, &EP));
            NSLG_TRY(get_exp(fm, make_double2(-fm->delta.x, -fm->delta.y), &EH));
            if (use_stratified(fm)) {
                std::vector<const ExpEntry *> Ep(2 * nconf), Ed(2 * nconf);
                std::vector<int> sg(2 * nconf);
                for (int64_t g = 0; g < 2 * nconf; ++g) {
                    Ep[g] = (g & 1) ? EP : EH;  // exp(-sgn delta K)
                    Ed[g] = (g & 1) ? EH : EP;  // exp(sgn delta K)
                    sg[g] = (g & 1) ? -1 : 1;
                }
                NSLG_TRY(logdet_strat(fm, (int)(2 * nconf), Ep.data(), Ed.data(), sg.data(), ph, ph_inv, ld.data()));
            } else {
                NSLG_TRY(logdet_many(fm, (int)(2 * nconf), EP->full, EH->full, 1, ph, ld.data()));
            }
        } else {
            for (int64_t b = 0; b < nconf; ++b) {
                NSLG_TRY(populate_dev(fm, phi + b * m, NSLG_PARTICLE));
                NSLG_TRY(fm_logdet(fm, &ld[2 * b]));
                NSLG_TRY(populate_dev(fm, phi + b * m, NSLG_HOLE));
                NSLG_TRY(fm_logdet(fm, &ld[2 * b + 1]));
            }
        }
        for (int64_t b = 0; b < nconf; ++b) {
            total[b].x -= ld[2 * b].x + ld[2 * b + 1].x;
            total[b].y -= ld[2 * b].y + ld[2 * b + 1].y;
        }
    }
    for (int64_t b = 0; b < nconf; ++b) S[b] = total[b];
    return NSLG_OK;
}

}  // namespace nslg
