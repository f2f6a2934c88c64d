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

// gP = grad log det M_P(phi), gH = grad log det M_H(phi); leaves fm populated with the hole species.
int fermion_grads(nslg_fm *fm, const double2 *phi, double2 *gP, double2 *gH) {
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
        NSLG_TRY(ws_get(fm, "hmc_gP", n, &gP));
        NSLG_TRY(ws_get(fm, "hmc_gH", n, &gH));
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

// The Nmd + 1 force evaluations with their fused kicks and drifts, enqueued on the handle's stream.
int leapfrog_steps(nslg_fm *fm, double2 *q, double2 *p, double2 Ut, double traj, int64_t nmd, int backward,
                   int real_force, int terms) {
    const int64_t n = fm->Nt * fm->Nx;
    cudaStream_t st = fm->ctx->stream;
    double eps = traj / (double)nmd;
    if (backward) eps = -eps;
    double2 *gP = nullptr, *gH = nullptr;
    NSLG_TRY(ws_get(fm, "hmc_gP", n, &gP));
    NSLG_TRY(ws_get(fm, "hmc_gH", n, &gH));
    const double2 uin = cdivd(make_double2(-1, 0), Ut);
    const unsigned grid = (unsigned)ceil_div(n, 256);
    for (int64_t step = 0; step <= nmd; ++step) {
        if (terms & 2) NSLG_TRY(fermion_grads(fm, q, gP, gH));
        const double ck = (step == 0 || step == nmd) ? 0.5 * eps : eps;
        const double cd = (step == nmd) ? 0.0 : eps;
        k_kick_drift<<<grid, 256, 0, st>>>(gP, gH, q, p, nullptr, uin, terms, real_force, ck, cd, n);
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
// trajectory and is read once after the replay.
int leapfrog_dev(nslg_fm *fm, double2 *q, double2 *p, double2 Ut, double traj, int64_t nmd, int backward,
                 int real_force, int terms) {
    cudaStream_t st = fm->ctx->stream;
    char keybuf[256];
    auto make_key = [&]() {
        std::snprintf(keybuf, sizeof keybuf, "lf:%lld:%.17g:%d:%d:%d:%.17g:%.17g:%llu:%p:%p:%d", (long long)nmd, traj,
                      backward, real_force, terms, Ut.x, Ut.y, (unsigned long long)fm->ws_generation, (void *)q,
                      (void *)p, fm->force_precision);
        return std::string(keybuf);
    };
    std::string key = make_key();
    auto it = fm->graphs.find(key);
    if (it == fm->graphs.end() && !fm->lf_seen.count(key)) {
        NSLG_TRY(leapfrog_steps(fm, q, p, Ut, traj, nmd, backward, real_force, terms));
        fm->lf_seen[make_key()] = 1;  // the key after the eager run's allocations
        return NSLG_OK;
    }
    int *sing = nullptr;
    if (terms & 2) NSLG_TRY(ws_get(fm, "lu_singular", 1, &sing));
    if (it == fm->graphs.end()) {
        cudaGraph_t g;
        NSLG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        fm->defer_checks = true;
        const int rc = leapfrog_steps(fm, q, p, Ut, traj, nmd, backward, real_force, terms);
        fm->defer_checks = false;
        const cudaError_t ce = cudaStreamEndCapture(st, &g);
        if (rc != NSLG_OK) {
            if (ce == cudaSuccess) cudaGraphDestroy(g);
            return rc;
        }
        NSLG_CUDA(ce);
        NSLG_REQUIRE(make_key() == key, NSLG_ERR_STATE, "leapfrog: a workspace moved while the trajectory was captured");
        size_t nodes = 0;
        cudaGraphGetNodes(g, nullptr, &nodes);
        cudaGraphExec_t ex;
        const cudaError_t ie = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        NSLG_CUDA(ie);
        it = fm->graphs.emplace(key, ex).first;
        fm->graph_kernels[key] = nodes;
    }
    if (sing) NSLG_CUDA(cudaMemsetAsync(sing, 0, sizeof(int), st));
    NSLG_CUDA(cudaGraphLaunch(it->second, st));
    note_launch(st, fm->graph_kernels[key]);
    if (terms & 2) {  // as after the eager run: the last populate is the hole species
        fm->species = NSLG_HOLE;
        fm->sgn = -1;
        fm->populated = true;
    }
    if (sing) {
        int h = 0;
        NSLG_CUDA(cudaMemcpyAsync(&h, sing, sizeof(int), cudaMemcpyDeviceToHost, st));
        NSLG_CUDA(cudaStreamSynchronize(st));
        NSLG_REQUIRE(!h, NSLG_ERR_ARG, "gradLogDetM: 1 + A^{-1} is singular");
    }
    return NSLG_OK;
}

}  // namespace nslg
