// extern "C" entry points of libnslgpu (declared in include/nsl_gb300.h) and the handle plumbing behind them:
// pointer staging, workspaces, operator dispatch.

#include <algorithm>
#include <atomic>
#include <type_traits>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "fm_internal.cuh"

namespace nslg {

int fm_logdet(nslg_fm *fm, double2 *out);
int fm_grad_logdet(nslg_fm *fm, double2 *out);
int hubbard_force_dev(nslg_fm *fm, const double2 *phi, double2 Ut, int terms, int real_force, double2 *F);
int hubbard_eval_dev(nslg_fm *fm, const double2 *phi, double2 Ut, int terms, double2 *S);
int leapfrog_dev(nslg_fm *fm, double2 *q, double2 *p, double2 Ut, double traj, int64_t nmd, int backward,
                 int real_force, int terms, int64_t nconf = 1, const double2 *uin_cfg = nullptr);
int leapfrog_group_dev(int ng, nslg_fm *const *fms, const int64_t *nconf, double2 *const *q, double2 *const *p,
                       const double2 *Ut, const double2 *const *uin_cfg, double traj, int64_t nmd, int backward,
                       int real_force, int terms);
int hubbard_eval_batch_dev(nslg_fm *fm, const double2 *phi, int64_t nconf, double2 Ut, int terms, double2 *S,
                           const double2 *Ut_cfg = nullptr);
double2 sum_squares_host(nslg_fm *fm, const double2 *a, int *rc);
int kinetic_batch_dev(nslg_fm *fm, const double2 *p, int64_t nconf, double2 *out);
int accept_batch_dev(nslg_fm *fm, int64_t nconf, const int *accept, const double2 *q_new, double2 *q);

int twobody_measure(nslg_fm *fm, const double2 *phi, const double2 *W, int nk, int nb, const int *tuples,
                    int64_t ntuple, int nts, double eps, int64_t max_iter, int precision, double2 *out,
                    nslg_cg_stats *stats);

namespace {
thread_local std::string g_last_error;

double2 cdiv(double2 a, double2 b) {
    const double d = b.x * b.x + b.y * b.y;
    return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}

// Device view of a caller buffer: the pointer itself when it is device-accessible, else a workspace copy.
int stage_in(nslg_fm *fm, const char *name, const void *p, size_t bytes, const void **dev) {
    bool on_device;
    NSLG_TRY(device_ptr(fm, p, &on_device));
    if (on_device) {
        *dev = p;
        return NSLG_OK;
    }
    void *w;
    NSLG_TRY(ws_get(fm, name, bytes, &w));
    NSLG_CUDA(cudaMemcpyAsync(w, p, bytes, cudaMemcpyHostToDevice, fm->ctx->stream));
    *dev = w;
    return NSLG_OK;
}

bool overlaps(const void *a, size_t na, const void *b, size_t nb) {
    const char *x = static_cast<const char *>(a), *y = static_cast<const char *>(b);
    return x < y + nb && y < x + na;
}

int check_fm(nslg_fm *fm) {
    NSLG_REQUIRE(fm != nullptr, NSLG_ERR_ARG, "null fermion-matrix handle");
    return NSLG_OK;
}

}  // namespace

void set_error(const std::string &msg) { g_last_error = msg; }

int device_ptr(const nslg_fm *fm, const void *p, bool *dev) {
    cudaPointerAttributes a;
    *dev = false;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return NSLG_OK;  // unregistered host memory
    }
    const int c = nslg_ptr_class(a.type == cudaMemoryTypeDevice, a.type == cudaMemoryTypeManaged, a.device,
                                 fm->ctx->device);
    NSLG_REQUIRE(c != NSLG_PTR_FOREIGN, NSLG_ERR_ARG,
                 "buffer is device memory of GPU " + std::to_string(a.device) + " but the handle runs on GPU " +
                     std::to_string(fm->ctx->device));
    *dev = c == NSLG_PTR_DEVICE;
    return NSLG_OK;
}

int ws_get(nslg_fm *fm, const char *name, size_t bytes, void **out) {
    auto &b = fm->ws[name];
    if (b.bytes < bytes) {
        if (b.p) NSLG_CUDA(cudaFree(b.p));
        b.p = nullptr;
        b.bytes = 0;
        const size_t want = std::max<size_t>(bytes, 256);
        if (cudaMalloc(&b.p, want) != cudaSuccess) {
            cudaGetLastError();
            set_error("device allocation of " + std::to_string(want) + " bytes for workspace '" + name + "' failed");
            return NSLG_ERR_OOM;
        }
        b.bytes = want;
        ++fm->ws_generation;
        drop_graphs(fm);
    }
    *out = b.p;
    return NSLG_OK;
}

void drop_graphs(nslg_fm *fm) {
    for (auto &g : fm->graphs) cudaGraphExecDestroy(g.second);
    fm->graphs.clear();
    for (auto &g : fm->graph_defs) cudaGraphDestroy(g.second);
    fm->graph_defs.clear();
}

namespace {
std::atomic<uint64_t> g_launches{0};
}

void note_launch(cudaStream_t st, uint64_t n) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) cudaGetLastError();
    if (cs == cudaStreamCaptureStatusNone) g_launches.fetch_add(n, std::memory_order_relaxed);
}

uint64_t launches() { return g_launches.load(); }

int num_sms() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n;
}

// Makes sure the exp(d K) entries and temporaries an operator needs exist (so graph capture allocates nothing).
int prepare_apply(nslg_fm *fm, int op, int64_t nbatch, int precision) {
    NSLG_REQUIRE(fm->kind == NSLG_FM_EXP || precision == NSLG_PREC_FP64 || precision == NSLG_PREC_FP32,
                 NSLG_ERR_UNSUPPORTED, "the diagonal discretisation applies its operators in FP64 or FP32 only");
    const double2 d = make_double2(fm->sgn * fm->delta.x, fm->sgn * fm->delta.y);
    const double2 dc = make_double2(fm->sgn * fm->delta.x, -fm->sgn * fm->delta.y);
    const ExpEntry *e;
    TcPlanes *P;
    OzPlanes *Q;
    for (int which = 0; which < 2; ++which) {
        if ((which == 0 && op == NSLG_OP_MDAGGER) || (which == 1 && op == NSLG_OP_M)) continue;
        NSLG_TRY(get_factor(fm, which == 0 ? d : dc, &e));
        if (precision == NSLG_PREC_TF32X3 && e->is_real) NSLG_TRY(tc_planes(fm, e, &P));
        if (precision == NSLG_PREC_BF16_SPLIT && e->is_real && fm->Nx <= 2048) NSLG_TRY(oz_planes(fm, e, &Q));
    }
    if (precision == NSLG_PREC_BF16_SPLIT) {
        int *rexp;
        void *dg;
        const int64_t rows = nbatch * fm->Nt;
        NSLG_TRY(ws_get(fm, "oz_rexp", (size_t)2 * rows, &rexp));
        NSLG_TRY(ws_get(fm, "oz_digits", (size_t)oz_digits() * 2 * rows * oz_ld((int)fm->Nx) * 2, &dg));
    }
    if (op == NSLG_OP_MMDAGGER || op == NSLG_OP_MDAGGERM) {
        void *w;
        const int64_t n = nbatch * fm->Nt * fm->Nx;
        NSLG_TRY(ws_get(fm, "apply_tmp", n * sizeof(double2), &w));
    }
    return NSLG_OK;
}

// One fused M (mode MODE_M) or M^dagger (MODE_MDAG) application with exp(d K) entry e, products in T. The
// tensor-core form needs a real exp(d K); with a complex one it runs the FP32 CUDA-core kernel of equal accuracy.
template <typename T>
int apply_one(nslg_fm *fm, int mode, const ExpEntry *e, const double2 *in, double2 *out, int64_t rows,
              const int *mask = nullptr, int64_t sys_rows = 1) {
    cudaStream_t st = fm->ctx->stream;
    const int Nt = (int)fm->Nt, Nx = (int)fm->Nx;
    if (fm->kind == NSLG_FM_DIAG) {  // e = sgn delta K (M) or sgn delta* K (M^dagger): CUDA-core kernel
        const int dmode = mode == MODE_M ? MODE_DIAG_M : MODE_DIAG_MDAG;
        if constexpr (std::is_same_v<T, double>)
            return fm_apply_simt<double>(dmode, in, out, fm->phase, e->re, e->is_real ? nullptr : e->im, Nt, Nx,
                                         rows, st);
        else if constexpr (std::is_same_v<T, float>)
            return fm_apply_simt<float>(dmode, in, out, fm->phase32, e->re32, e->is_real ? nullptr : e->im32, Nt, Nx,
                                        rows, st);
        else
            NSLG_REQUIRE(false, NSLG_ERR_UNSUPPORTED,
                         "the diagonal discretisation applies its operators in FP64 or FP32 only");
    }
    if constexpr (std::is_same_v<T, BF16Split>) {
        if (e->is_real && Nx <= 2048) {
            OzPlanes *P;
            NSLG_TRY(oz_planes(fm, e, &P));
            int *rexp;
            void *dg;
            NSLG_TRY(ws_get(fm, "oz_rexp", (size_t)2 * rows, &rexp));
            NSLG_TRY(ws_get(fm, "oz_digits", (size_t)oz_digits() * 2 * rows * oz_ld(Nx) * 2, &dg));
            return fm_apply_oz(mode, in, out, fm->phase, *P, dg, rexp, Nt, Nx, rows, fm->tc_err, st);
        }
        return fm_apply_simt<double>(mode, in, out, fm->phase, e->re, e->is_real ? nullptr : e->im, Nt, Nx, rows, st);
    } else if constexpr (std::is_same_v<T, TF32x3>) {
        if (e->is_real) {
            TcPlanes *P;
            NSLG_TRY(tc_planes(fm, e, &P));
            return fm_apply_tc(mode, in, out, fm->phase, *P, Nt, Nx, rows, fm->tc_err, st);
        }
        return fm_apply_simt<float>(mode, in, out, fm->phase32, e->re32, e->im32, Nt, Nx, rows, st);
    } else if constexpr (std::is_same_v<T, float>) {
        return fm_apply_simt<float>(mode, in, out, fm->phase32, e->re32, e->is_real ? nullptr : e->im32, Nt, Nx,
                                    rows, st);
    } else {
        return fm_apply_simt<double>(mode, in, out, fm->phase, e->re, e->is_real ? nullptr : e->im, Nt, Nx, rows,
                                     st, mask, sys_rows);
    }
}

template <typename T>
int fm_apply_dev(nslg_fm *fm, int op, const double2 *psi, double2 *out, int64_t nbatch, const int *mask,
                 int64_t sys_rows) {
    NSLG_REQUIRE(fm->populated, NSLG_ERR_STATE, "the fermion matrix has no configuration (call populate first)");
    const double2 d = make_double2(fm->sgn * fm->delta.x, fm->sgn * fm->delta.y);
    const double2 dc = make_double2(fm->sgn * fm->delta.x, -fm->sgn * fm->delta.y);
    const ExpEntry *E = nullptr, *Ec = nullptr;
    if (op != NSLG_OP_MDAGGER) NSLG_TRY(get_factor(fm, d, &E));
    if (op != NSLG_OP_M) NSLG_TRY(get_factor(fm, dc, &Ec));
    const int64_t rows = nbatch * fm->Nt;
    switch (op) {
        case NSLG_OP_M: return apply_one<T>(fm, MODE_M, E, psi, out, rows, mask, sys_rows);
        case NSLG_OP_MDAGGER: return apply_one<T>(fm, MODE_MDAG, Ec, psi, out, rows, mask, sys_rows);
        default: break;
    }
    double2 *tmp;
    NSLG_TRY(ws_get(fm, "apply_tmp", rows * fm->Nx, &tmp));
    if (op == NSLG_OP_MMDAGGER) {  // M (M^dagger psi)
        NSLG_TRY(apply_one<T>(fm, MODE_MDAG, Ec, psi, tmp, rows, mask, sys_rows));
        return apply_one<T>(fm, MODE_M, E, tmp, out, rows, mask, sys_rows);
    }
    // M^dagger (M psi)
    NSLG_TRY(apply_one<T>(fm, MODE_M, E, psi, tmp, rows, mask, sys_rows));
    return apply_one<T>(fm, MODE_MDAG, Ec, tmp, out, rows, mask, sys_rows);
}

template int fm_apply_dev<double>(nslg_fm *, int, const double2 *, double2 *, int64_t, const int *, int64_t);
template int fm_apply_dev<float>(nslg_fm *, int, const double2 *, double2 *, int64_t, const int *, int64_t);
template int fm_apply_dev<TF32x3>(nslg_fm *, int, const double2 *, double2 *, int64_t, const int *, int64_t);
template int fm_apply_dev<BF16Split>(nslg_fm *, int, const double2 *, double2 *, int64_t, const int *, int64_t);

// Reports (and clears) a timeout recorded by a tensor-core kernel's bounded waits.
int check_tc_error(nslg_fm *fm) {
    int h = 0;
    NSLG_CUDA(cudaMemcpyAsync(&h, fm->tc_err, sizeof(int), cudaMemcpyDeviceToHost, fm->ctx->stream));
    NSLG_CUDA(cudaStreamSynchronize(fm->ctx->stream));
    if (h != 0) {
        NSLG_CUDA(cudaMemsetAsync(fm->tc_err, 0, sizeof(int), fm->ctx->stream));
        if (h == 31)  // the split-BF16 digit sums of this exp(delta K) are not provably exact
            set_error("split-BF16 operator: exp(delta K) is too delocalised for exact digit sums (delta too large); "
                      "use the FP64 operator");
        else
            set_error("tensor-core operator: a pipeline wait timed out (code " + std::to_string(h) + ")");
        return NSLG_ERR_CUDA;
    }
    return NSLG_OK;
}

}  // namespace nslg

using namespace nslg;

extern "C" {

NSLG_API int nslg_version(void) { return 1; }

NSLG_API const char *nslg_last_error(void) { return g_last_error.c_str(); }

NSLG_API uint64_t nslg_kernel_launches(void) { return launches(); }

NSLG_API int nslg_ctx_create(int device, void *stream, nslg_ctx **out) {
    NSLG_REQUIRE(out != nullptr, NSLG_ERR_ARG, "nslg_ctx_create: out is null");
    int n = 0;
    NSLG_CUDA(cudaGetDeviceCount(&n));
    NSLG_REQUIRE(device >= 0 && device < n, NSLG_ERR_ARG, "nslg_ctx_create: no such CUDA device");
    NSLG_CUDA(cudaSetDevice(device));
    auto *c = new nslg_ctx;
    c->device = device;
    if (stream) {
        c->stream = static_cast<cudaStream_t>(stream);
    } else {
        if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete c;
            set_error("nslg_ctx_create: cudaStreamCreate failed");
            return NSLG_ERR_CUDA;
        }
        c->own_stream = true;
    }
    c->num_sms = num_sms();
    *out = c;
    return NSLG_OK;
}

// Drops one reference; the last one synchronises and destroys the owned stream and frees the context.
static void ctx_release(nslg_ctx *ctx) {
    if (ctx->refs.fetch_sub(1) != 1) return;
    if (ctx->own_stream) {
        cudaStreamSynchronize(ctx->stream);
        cudaStreamDestroy(ctx->stream);
    }
    delete ctx;
}

NSLG_API int nslg_ctx_destroy(nslg_ctx *ctx) {
    if (!ctx) return NSLG_OK;
    ctx_release(ctx);
    return NSLG_OK;
}

NSLG_API int nslg_ctx_synchronize(nslg_ctx *ctx) {
    NSLG_REQUIRE(ctx != nullptr, NSLG_ERR_ARG, "null context");
    NSLG_CUDA(cudaStreamSynchronize(ctx->stream));
    return NSLG_OK;
}

NSLG_API void *nslg_ctx_stream(nslg_ctx *ctx) { return ctx ? static_cast<void *>(ctx->stream) : nullptr; }

NSLG_API int nslg_fm_create(nslg_ctx *ctx, int64_t Nx, int64_t Nt, const nslg_c128 *hops, nslg_c128 beta,
                            nslg_c128 mu, int species, nslg_fm **out) {
    return nslg_fm_create_kind(ctx, NSLG_FM_EXP, Nx, Nt, hops, beta, mu, species, out);
}

NSLG_API int nslg_fm_create_kind(nslg_ctx *ctx, int kind, int64_t Nx, int64_t Nt, const nslg_c128 *hops,
                                 nslg_c128 beta, nslg_c128 mu, int species, nslg_fm **out) {
    NSLG_REQUIRE(ctx && hops && out, NSLG_ERR_ARG, "nslg_fm_create: null argument");
    NSLG_REQUIRE(kind == NSLG_FM_EXP || kind == NSLG_FM_DIAG, NSLG_ERR_ARG, "nslg_fm_create: unknown discretisation");
    NSLG_REQUIRE(Nx >= 1 && Nx <= 16384 && Nt >= 1 && Nt <= 65536, NSLG_ERR_SHAPE,
                 "nslg_fm_create: Nx must be in [1, 16384] and Nt in [1, 65536]");
    NSLG_REQUIRE(species == NSLG_PARTICLE || species == NSLG_HOLE, NSLG_ERR_ARG, "nslg_fm_create: bad species");
    NSLG_CUDA(cudaSetDevice(ctx->device));
    static std::atomic<uint64_t> next_uid{1};
    auto *fm = new nslg_fm;
    fm->uid = next_uid.fetch_add(1);
    fm->ctx = ctx;
    ctx->refs.fetch_add(1);  // released by nslg_fm_destroy
    fm->kind = kind;
    fm->Nx = Nx;
    fm->Nt = Nt;
    fm->delta = cdiv(make_double2(beta.re, beta.im), make_double2((double)Nt, 0));
    fm->mu_tilde = cmul(fm->delta, make_double2(mu.re, mu.im));
    fm->species = species;
    fm->sgn = species == NSLG_PARTICLE ? 1 : -1;
    const size_t mat = (size_t)Nx * Nx * sizeof(double2), fld = (size_t)Nt * Nx;
    auto fail = [&](int rc) {
        nslg_fm_destroy(fm);
        return rc;
    };
    if (cudaMalloc(&fm->hops, mat) != cudaSuccess || cudaMalloc(&fm->phi, fld * sizeof(double2)) != cudaSuccess ||
        cudaMalloc(&fm->phase, fld * sizeof(double2)) != cudaSuccess ||
        cudaMalloc(&fm->phase_inv, fld * sizeof(double2)) != cudaSuccess ||
        cudaMalloc(&fm->phase32, fld * sizeof(float2)) != cudaSuccess ||
        cudaMalloc(&fm->tc_err, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        set_error("nslg_fm_create: device allocation failed");
        return fail(NSLG_ERR_OOM);
    }
    if (cudaMemcpyAsync(fm->hops, hops, mat, cudaMemcpyDefault, ctx->stream) != cudaSuccess) {
        set_error("nslg_fm_create: copying the hopping matrix failed");
        return fail(NSLG_ERR_CUDA);
    }
    if (cudaMemsetAsync(fm->tc_err, 0, sizeof(int), ctx->stream) != cudaSuccess) return fail(NSLG_ERR_CUDA);
    int rc = compute_hops_norm(fm);
    if (rc != NSLG_OK) return fail(rc);
    *out = fm;
    return NSLG_OK;
}

NSLG_API int nslg_fm_destroy(nslg_fm *fm) {
    if (!fm) return NSLG_OK;
    cudaStreamSynchronize(fm->ctx->stream);
    drop_graphs(fm);
    for (auto &kv : fm->lin) {
        cudaFree(kv.second.full);
        cudaFree(kv.second.re);
        cudaFree(kv.second.im);
        cudaFree(kv.second.re32);
        cudaFree(kv.second.im32);
    }
    for (auto &kv : fm->memo) {
        cudaFree(kv.second.full);
        cudaFree(kv.second.re);
        cudaFree(kv.second.im);
        cudaFree(kv.second.re32);
        cudaFree(kv.second.im32);
        if (kv.second.tc) {
            cudaFree(kv.second.tc->hi);
            cudaFree(kv.second.tc->lo);
            delete kv.second.tc;
        }
        if (kv.second.oz) {
            cudaFree(kv.second.oz->planes);
            cudaFree(kv.second.oz->col_exp);
            delete kv.second.oz;
        }
    }
    cudaFree(fm->tc_err);
    if (fm->side) {
        cudaStreamSynchronize(fm->side);
        cudaStreamDestroy(fm->side);
    }
    if (fm->ev_fork) cudaEventDestroy(fm->ev_fork);
    if (fm->ev_join) cudaEventDestroy(fm->ev_join);
    for (auto &kv : fm->ws) cudaFree(kv.second.p);
    cudaFree(fm->hops);
    cudaFree(fm->phi);
    cudaFree(fm->phase);
    cudaFree(fm->phase_inv);
    cudaFree(fm->phase32);
    nslg_ctx *ctx = fm->ctx;
    delete fm;
    ctx_release(ctx);
    return NSLG_OK;
}

NSLG_API int nslg_fm_set_exp_hopping(nslg_fm *fm, nslg_c128 delta, const nslg_c128 *expK) {
    NSLG_TRY(check_fm(fm));
    NSLG_REQUIRE(expK != nullptr, NSLG_ERR_ARG, "nslg_fm_set_exp_hopping: expK is null");
    const void *dev;
    NSLG_TRY(stage_in(fm, "io_exp", expK, (size_t)fm->Nx * fm->Nx * sizeof(double2), &dev));
    NSLG_TRY(install_exp(fm, make_double2(delta.re, delta.im), static_cast<const double2 *>(dev)));
    NSLG_CUDA(cudaStreamSynchronize(fm->ctx->stream));
    return NSLG_OK;
}

NSLG_API int nslg_fm_get_exp_hopping(nslg_fm *fm, nslg_c128 delta, nslg_c128 *out) {
    NSLG_TRY(check_fm(fm));
    NSLG_REQUIRE(out != nullptr, NSLG_ERR_ARG, "nslg_fm_get_exp_hopping: out is null");
    const ExpEntry *e;
    NSLG_TRY(get_exp(fm, make_double2(delta.re, delta.im), &e));
    NSLG_CUDA(cudaMemcpyAsync(out, e->full, (size_t)fm->Nx * fm->Nx * sizeof(double2), cudaMemcpyDefault,
                              fm->ctx->stream));
    NSLG_CUDA(cudaStreamSynchronize(fm->ctx->stream));
    return NSLG_OK;
}

NSLG_API int nslg_fm_populate(nslg_fm *fm, const nslg_c128 *phi, int species) {
    NSLG_TRY(check_fm(fm));
    NSLG_REQUIRE(phi != nullptr, NSLG_ERR_ARG, "nslg_fm_populate: phi is null");
    NSLG_REQUIRE(species < 0 || species == NSLG_PARTICLE || species == NSLG_HOLE, NSLG_ERR_ARG,
                 "nslg_fm_populate: bad species");
    bool phi_dev;
    NSLG_TRY(device_ptr(fm, phi, &phi_dev));
    if (species >= 0) {
        fm->species = species;
        fm->sgn = species == NSLG_PARTICLE ? 1 : -1;
    }
    NSLG_CUDA(cudaMemcpyAsync(fm->phi, phi, (size_t)fm->Nt * fm->Nx * sizeof(double2), cudaMemcpyDefault,
                              fm->ctx->stream));
    NSLG_TRY(compute_phases(fm));
    fm->populated = true;
    if (!phi_dev) NSLG_CUDA(cudaStreamSynchronize(fm->ctx->stream));
    return NSLG_OK;
}

NSLG_API int nslg_fm_get_phases(nslg_fm *fm, nslg_c128 *out) {
    NSLG_TRY(check_fm(fm));
    NSLG_REQUIRE(out != nullptr, NSLG_ERR_ARG, "nslg_fm_get_phases: out is null");
    NSLG_REQUIRE(fm->populated, NSLG_ERR_STATE, "nslg_fm_get_phases: populate() has not been called");
    bool dev;
    NSLG_TRY(device_ptr(fm, out, &dev));
    NSLG_CUDA(cudaMemcpyAsync(out, fm->phase, (size_t)fm->Nt * fm->Nx * sizeof(double2), cudaMemcpyDefault,
                              fm->ctx->stream));
    if (!dev) NSLG_CUDA(cudaStreamSynchronize(fm->ctx->stream));
    return NSLG_OK;
}

NSLG_API int nslg_fm_apply(nslg_fm *fm, int op, const nslg_c128 *psi, nslg_c128 *out, int64_t nbatch,
                           int precision) {
    NSLG_TRY(check_fm(fm));
    NSLG_REQUIRE(psi && out, NSLG_ERR_ARG, "nslg_fm_apply: null buffer");
    NSLG_REQUIRE(op >= NSLG_OP_M && op <= NSLG_OP_MDAGGERM, NSLG_ERR_ARG, "nslg_fm_apply: unknown operator");
    NSLG_REQUIRE(precision >= NSLG_PREC_FP64 && precision <= NSLG_PREC_BF16_SPLIT, NSLG_ERR_ARG,
                 "nslg_fm_apply: unknown precision");
    NSLG_REQUIRE(nbatch >= 0, NSLG_ERR_SHAPE, "nslg_fm_apply: negative batch");
    NSLG_REQUIRE(fm->populated, NSLG_ERR_STATE, "nslg_fm_apply: populate() has not been called");
    const int64_t n = nbatch * fm->Nt * fm->Nx;
    const size_t bytes = n * sizeof(double2);
    NSLG_REQUIRE(!overlaps(psi, bytes, out, bytes), NSLG_ERR_ARG, "nslg_fm_apply: psi and out overlap");
    if (n == 0) return NSLG_OK;
    cudaStream_t st = fm->ctx->stream;
    NSLG_TRY(prepare_apply(fm, op, nbatch, precision));
    const void *din;
    NSLG_TRY(stage_in(fm, "io_in", psi, bytes, &din));
    bool out_dev, in_dev;
    NSLG_TRY(device_ptr(fm, out, &out_dev));
    NSLG_TRY(device_ptr(fm, psi, &in_dev));
    double2 *dout;
    if (out_dev) dout = reinterpret_cast<double2 *>(out);
    else NSLG_TRY(ws_get(fm, "io_out", n, &dout));
    const double2 *pin = static_cast<const double2 *>(din);
    if (precision == NSLG_PREC_FP64) NSLG_TRY(fm_apply_dev<double>(fm, op, pin, dout, nbatch));
    else if (precision == NSLG_PREC_FP32) NSLG_TRY(fm_apply_dev<float>(fm, op, pin, dout, nbatch));
    else if (precision == NSLG_PREC_TF32X3) NSLG_TRY(fm_apply_dev<TF32x3>(fm, op, pin, dout, nbatch));
    else NSLG_TRY(fm_apply_dev<BF16Split>(fm, op, pin, dout, nbatch));
    if (!out_dev) NSLG_CUDA(cudaMemcpyAsync(out, dout, bytes, cudaMemcpyDeviceToHost, st));
    if (!out_dev || !in_dev) {
        NSLG_CUDA(cudaStreamSynchronize(st));
        NSLG_TRY(check_tc_error(fm));
    }
    // device-buffer calls stay asynchronous: a tensor-core pipeline timeout is reported by the next call on this
    // handle that synchronises
    return NSLG_OK;
}

NSLG_API int nslg_fm_apply_dd(nslg_fm *fm, int op, const nslg_c128 *psi_hi, const nslg_c128 *psi_lo,
                              nslg_c128 *out_hi, nslg_c128 *out_lo, int64_t nbatch) {
    NSLG_TRY(check_fm(fm));
    NSLG_REQUIRE(psi_hi && out_hi && out_lo, NSLG_ERR_ARG, "nslg_fm_apply_dd: null buffer");
    NSLG_REQUIRE(op >= NSLG_OP_M && op <= NSLG_OP_MDAGGERM, NSLG_ERR_ARG, "nslg_fm_apply_dd: unknown operator");
    NSLG_REQUIRE(nbatch >= 0, NSLG_ERR_SHAPE, "nslg_fm_apply_dd: negative batch");
    NSLG_REQUIRE(fm->kind == NSLG_FM_EXP, NSLG_ERR_UNSUPPORTED,
                 "nslg_fm_apply_dd: implemented for the exponential discretisation");
    NSLG_REQUIRE(fm->populated, NSLG_ERR_STATE, "nslg_fm_apply_dd: populate() has not been called");
    const int64_t n = nbatch * fm->Nt * fm->Nx;
    const size_t bytes = n * sizeof(double2);
    for (const void *o : {(const void *)out_hi, (const void *)out_lo})
        for (const void *i : {(const void *)psi_hi, (const void *)psi_lo})
            NSLG_REQUIRE(!i || !overlaps(i, bytes, o, bytes), NSLG_ERR_ARG, "nslg_fm_apply_dd: outputs overlap inputs");
    NSLG_REQUIRE(!overlaps(out_hi, bytes, out_lo, bytes), NSLG_ERR_ARG, "nslg_fm_apply_dd: out_hi and out_lo overlap");
    if (n == 0) return NSLG_OK;
    cudaStream_t st = fm->ctx->stream;
    const void *dh, *dl;
    NSLG_TRY(stage_in(fm, "io_ddh", psi_hi, bytes, &dh));
    if (psi_lo) {
        NSLG_TRY(stage_in(fm, "io_ddl", psi_lo, bytes, &dl));
    } else {
        double2 *z;
        NSLG_TRY(ws_get(fm, "io_ddz", n, &z));
        NSLG_CUDA(cudaMemsetAsync(z, 0, bytes, st));
        dl = z;
    }
    bool hd, ld;
    NSLG_TRY(device_ptr(fm, out_hi, &hd));
    NSLG_TRY(device_ptr(fm, out_lo, &ld));
    double2 *oh, *ol;
    if (hd) oh = reinterpret_cast<double2 *>(out_hi);
    else NSLG_TRY(ws_get(fm, "io_ddoh", n, &oh));
    if (ld) ol = reinterpret_cast<double2 *>(out_lo);
    else NSLG_TRY(ws_get(fm, "io_ddol", n, &ol));
    NSLG_TRY(fm_apply_dd(fm, op, static_cast<const double2 *>(dh), static_cast<const double2 *>(dl), oh, ol, nbatch,
                         nullptr, 0));
    if (!hd) NSLG_CUDA(cudaMemcpyAsync(out_hi, oh, bytes, cudaMemcpyDeviceToHost, st));
    if (!ld) NSLG_CUDA(cudaMemcpyAsync(out_lo, ol, bytes, cudaMemcpyDeviceToHost, st));
    bool ih;
    NSLG_TRY(device_ptr(fm, psi_hi, &ih));
    if (!hd || !ld || !ih) NSLG_CUDA(cudaStreamSynchronize(st));
    return NSLG_OK;
}

NSLG_API int nslg_fm_set_force_precision(nslg_fm *fm, int precision) {
    NSLG_TRY(check_fm(fm));
    NSLG_REQUIRE(precision == NSLG_PREC_FP64 || precision == NSLG_PREC_BF16_SPLIT, NSLG_ERR_ARG,
                 "nslg_fm_set_force_precision: NSLG_PREC_FP64 or NSLG_PREC_BF16_SPLIT");
    fm->force_precision = precision;
    return NSLG_OK;
}

NSLG_API int nslg_fm_set_stabilisation(nslg_fm *fm, int mode) {
    NSLG_TRY(check_fm(fm));
    NSLG_REQUIRE(mode == NSLG_STAB_AUTO || mode == NSLG_STAB_PLAIN || mode == NSLG_STAB_STRATIFIED, NSLG_ERR_ARG,
                 "nslg_fm_set_stabilisation: unknown mode");
    if (mode != fm->stabilisation) {  // captured trajectories bake in the form
        drop_graphs(fm);
        fm->lf_seen.clear();
    }
    fm->stabilisation = mode;
    return NSLG_OK;
}

NSLG_API int nslg_fm_logdet(nslg_fm *fm, nslg_c128 *out) {
    NSLG_TRY(check_fm(fm));
    NSLG_REQUIRE(out != nullptr, NSLG_ERR_ARG, "nslg_fm_logdet: out is null");
    NSLG_REQUIRE(fm->populated, NSLG_ERR_STATE, "nslg_fm_logdet: populate() has not been called");
    double2 v;
    NSLG_TRY(fm_logdet(fm, &v));
    out->re = v.x;
    out->im = v.y;
    return NSLG_OK;
}

NSLG_API int nslg_fm_grad_logdet(nslg_fm *fm, nslg_c128 *out) {
    NSLG_TRY(check_fm(fm));
    NSLG_REQUIRE(out != nullptr, NSLG_ERR_ARG, "nslg_fm_grad_logdet: out is null");
    NSLG_REQUIRE(fm->populated, NSLG_ERR_STATE, "nslg_fm_grad_logdet: populate() has not been called");
    const int64_t n = fm->Nt * fm->Nx;
    bool dev;
    NSLG_TRY(device_ptr(fm, out, &dev));
    double2 *d;
    if (dev) d = reinterpret_cast<double2 *>(out);
    else NSLG_TRY(ws_get(fm, "io_grad", n, &d));
    NSLG_TRY(fm_grad_logdet(fm, d));
    if (!dev) NSLG_CUDA(cudaMemcpyAsync(out, d, n * sizeof(double2), cudaMemcpyDeviceToHost, fm->ctx->stream));
    NSLG_CUDA(cudaStreamSynchronize(fm->ctx->stream));
    if (fm->force_precision != NSLG_PREC_FP64) NSLG_TRY(check_tc_error(fm));
    return NSLG_OK;
}

NSLG_API int nslg_hubbard_eval(nslg_fm *fm, const nslg_c128 *phi, nslg_c128 Utilde, int terms, nslg_c128 *S) {
    NSLG_TRY(check_fm(fm));
    NSLG_REQUIRE(phi && S, NSLG_ERR_ARG, "nslg_hubbard_eval: null argument");
    NSLG_REQUIRE(terms >= 1 && terms <= 3, NSLG_ERR_ARG, "nslg_hubbard_eval: terms must be a mask of 1 and 2");
    const int64_t n = fm->Nt * fm->Nx;
    const void *d;
    NSLG_TRY(stage_in(fm, "io_phi", phi, n * sizeof(double2), &d));
    double2 v;
    NSLG_TRY(hubbard_eval_dev(fm, static_cast<const double2 *>(d), make_double2(Utilde.re, Utilde.im), terms, &v));
    S->re = v.x;
    S->im = v.y;
    return NSLG_OK;
}

NSLG_API int nslg_hubbard_force(nslg_fm *fm, const nslg_c128 *phi, nslg_c128 Utilde, int terms, int real_force,
                                nslg_c128 *force) {
    NSLG_TRY(check_fm(fm));
    NSLG_REQUIRE(phi && force, NSLG_ERR_ARG, "nslg_hubbard_force: null argument");
    NSLG_REQUIRE(terms >= 1 && terms <= 3, NSLG_ERR_ARG, "nslg_hubbard_force: terms must be a mask of 1 and 2");
    const int64_t n = fm->Nt * fm->Nx;
    const size_t bytes = n * sizeof(double2);
    NSLG_REQUIRE(!overlaps(phi, bytes, force, bytes), NSLG_ERR_ARG, "nslg_hubbard_force: phi and force overlap");
    const void *d;
    NSLG_TRY(stage_in(fm, "io_phi", phi, bytes, &d));
    bool dev;
    NSLG_TRY(device_ptr(fm, force, &dev));
    double2 *f;
    if (dev) f = reinterpret_cast<double2 *>(force);
    else NSLG_TRY(ws_get(fm, "io_force", n, &f));
    NSLG_TRY(hubbard_force_dev(fm, static_cast<const double2 *>(d), make_double2(Utilde.re, Utilde.im), terms,
                               real_force, f));
    if (!dev) NSLG_CUDA(cudaMemcpyAsync(force, f, bytes, cudaMemcpyDeviceToHost, fm->ctx->stream));
    NSLG_CUDA(cudaStreamSynchronize(fm->ctx->stream));
    if (fm->force_precision != NSLG_PREC_FP64) NSLG_TRY(check_tc_error(fm));
    return NSLG_OK;
}

NSLG_API int nslg_leapfrog(nslg_fm *fm, const nslg_c128 *q0, const nslg_c128 *p0, nslg_c128 *q1, nslg_c128 *p1,
                           nslg_c128 Utilde, double traj_length, int64_t nmd, int backward, int real_force,
                           int terms) {
    NSLG_TRY(check_fm(fm));
    NSLG_REQUIRE(q0 && p0 && q1 && p1, NSLG_ERR_ARG, "nslg_leapfrog: null argument");
    NSLG_REQUIRE(nmd >= 1, NSLG_ERR_ARG, "nslg_leapfrog: Nmd must be >= 1");
    NSLG_REQUIRE(terms >= 1 && terms <= 3, NSLG_ERR_ARG, "nslg_leapfrog: terms must be a mask of 1 and 2");
    NSLG_REQUIRE(std::isfinite(traj_length), NSLG_ERR_ARG, "nslg_leapfrog: trajectory length must be finite");
    const int64_t n = fm->Nt * fm->Nx;
    const size_t bytes = n * sizeof(double2);
    cudaStream_t st = fm->ctx->stream;
    double2 *q, *p;
    NSLG_TRY(ws_get(fm, "lf_q", n, &q));
    NSLG_TRY(ws_get(fm, "lf_p", n, &p));
    NSLG_CUDA(cudaMemcpyAsync(q, q0, bytes, cudaMemcpyDefault, st));
    NSLG_CUDA(cudaMemcpyAsync(p, p0, bytes, cudaMemcpyDefault, st));
    NSLG_TRY(leapfrog_dev(fm, q, p, make_double2(Utilde.re, Utilde.im), traj_length, nmd, backward, real_force,
                          terms));
    NSLG_CUDA(cudaMemcpyAsync(q1, q, bytes, cudaMemcpyDefault, st));
    NSLG_CUDA(cudaMemcpyAsync(p1, p, bytes, cudaMemcpyDefault, st));
    NSLG_CUDA(cudaStreamSynchronize(st));
    if (fm->force_precision != NSLG_PREC_FP64) NSLG_TRY(check_tc_error(fm));
    return NSLG_OK;
}

NSLG_API int nslg_leapfrog_batch(nslg_fm *fm, int64_t nconf, const nslg_c128 *q0, const nslg_c128 *p0,
                                 nslg_c128 *q1, nslg_c128 *p1, nslg_c128 Utilde, double traj_length, int64_t nmd,
                                 int backward, int real_force, int terms) {
    NSLG_TRY(check_fm(fm));
    NSLG_REQUIRE(q0 && p0 && q1 && p1, NSLG_ERR_ARG, "nslg_leapfrog_batch: null argument");
    NSLG_REQUIRE(nconf >= 1 && 2 * nconf <= 65535, NSLG_ERR_SHAPE, "nslg_leapfrog_batch: need 1 <= nconf <= 32767");
    NSLG_REQUIRE(nmd >= 1, NSLG_ERR_ARG, "nslg_leapfrog_batch: Nmd must be >= 1");
    NSLG_REQUIRE(terms >= 1 && terms <= 3, NSLG_ERR_ARG, "nslg_leapfrog_batch: terms must be a mask of 1 and 2");
    NSLG_REQUIRE(std::isfinite(traj_length), NSLG_ERR_ARG, "nslg_leapfrog_batch: trajectory length must be finite");
    if (nconf == 1) return nslg_leapfrog(fm, q0, p0, q1, p1, Utilde, traj_length, nmd, backward, real_force, terms);
    const int64_t n = nconf * fm->Nt * fm->Nx;
    const size_t bytes = n * sizeof(double2);
    cudaStream_t st = fm->ctx->stream;
    double2 *q, *p;
    NSLG_TRY(ws_get(fm, "lfb_q", n, &q));
    NSLG_TRY(ws_get(fm, "lfb_p", n, &p));
    NSLG_CUDA(cudaMemcpyAsync(q, q0, bytes, cudaMemcpyDefault, st));
    NSLG_CUDA(cudaMemcpyAsync(p, p0, bytes, cudaMemcpyDefault, st));
    NSLG_TRY(leapfrog_dev(fm, q, p, make_double2(Utilde.re, Utilde.im), traj_length, nmd, backward, real_force,
                          terms, nconf));
    NSLG_CUDA(cudaMemcpyAsync(q1, q, bytes, cudaMemcpyDefault, st));
    NSLG_CUDA(cudaMemcpyAsync(p1, p, bytes, cudaMemcpyDefault, st));
    NSLG_CUDA(cudaStreamSynchronize(st));
    return NSLG_OK;
}

NSLG_API int nslg_leapfrog_group(int ngroups, nslg_fm *const *fms, const int64_t *nconf,
                                 const nslg_c128 *const *q0, const nslg_c128 *const *p0, nslg_c128 *const *q1,
                                 nslg_c128 *const *p1, const nslg_c128 *const *Utilde, double traj_length,
                                 int64_t nmd, int backward, int real_force, int terms) {
    NSLG_REQUIRE(ngroups >= 1 && ngroups <= 4096, NSLG_ERR_ARG, "nslg_leapfrog_group: need 1 <= ngroups <= 4096");
    NSLG_REQUIRE(fms && nconf && q0 && p0 && q1 && p1 && Utilde, NSLG_ERR_ARG, "nslg_leapfrog_group: null argument");
    NSLG_REQUIRE(nmd >= 1, NSLG_ERR_ARG, "nslg_leapfrog_group: Nmd must be >= 1");
    NSLG_REQUIRE(terms >= 1 && terms <= 3, NSLG_ERR_ARG, "nslg_leapfrog_group: terms must be a mask of 1 and 2");
    NSLG_REQUIRE(std::isfinite(traj_length), NSLG_ERR_ARG, "nslg_leapfrog_group: trajectory length must be finite");
    for (int g = 0; g < ngroups; ++g) {
        NSLG_TRY(check_fm(fms[g]));
        NSLG_REQUIRE(fms[g]->ctx == fms[0]->ctx, NSLG_ERR_ARG, "nslg_leapfrog_group: the handles must share one context");
        for (int h = 0; h < g; ++h)
            NSLG_REQUIRE(fms[h] != fms[g], NSLG_ERR_ARG, "nslg_leapfrog_group: a handle appears twice");
        NSLG_REQUIRE(nconf[g] >= 1 && 2 * nconf[g] <= 65535, NSLG_ERR_SHAPE,
                     "nslg_leapfrog_group: need 1 <= nconf <= 32767 per group");
        NSLG_REQUIRE(q0[g] && p0[g] && q1[g] && p1[g] && Utilde[g], NSLG_ERR_ARG, "nslg_leapfrog_group: null argument");
        for (int64_t b = 0; b < nconf[g]; ++b)
            NSLG_REQUIRE(std::isfinite(Utilde[g][b].re) && std::isfinite(Utilde[g][b].im) &&
                             (Utilde[g][b].re != 0 || Utilde[g][b].im != 0),
                         NSLG_ERR_ARG, "nslg_leapfrog_group: U~ must be finite and nonzero");
    }
    cudaStream_t st = fms[0]->ctx->stream;
    std::vector<double2 *> q(ngroups), p(ngroups);
    std::vector<const double2 *> uin(ngroups, nullptr);
    std::vector<double2> Ut(ngroups);
    for (int g = 0; g < ngroups; ++g) {
        nslg_fm *fm = fms[g];
        const int64_t n = nconf[g] * fm->Nt * fm->Nx;
        NSLG_TRY(ws_get(fm, "lfb_q", n, &q[g]));
        NSLG_TRY(ws_get(fm, "lfb_p", n, &p[g]));
        Ut[g] = make_double2(Utilde[g][0].re, Utilde[g][0].im);
        if (nconf[g] > 1) {  // -1 / U~ per configuration, in a buffer the captured trajectory reads
            double2 *d;
            NSLG_TRY(ws_get(fm, "lfb_uin", (size_t)nconf[g], &d));
            uin[g] = d;
        }
    }
    // staging after every workspace exists (a later allocation would move none of these, but keep them together)
    std::vector<std::vector<double2>> uh(ngroups);
    for (int g = 0; g < ngroups; ++g) {
        const size_t bytes = (size_t)nconf[g] * fms[g]->Nt * fms[g]->Nx * sizeof(double2);
        NSLG_CUDA(cudaMemcpyAsync(q[g], q0[g], bytes, cudaMemcpyDefault, st));
        NSLG_CUDA(cudaMemcpyAsync(p[g], p0[g], bytes, cudaMemcpyDefault, st));
        if (uin[g]) {
            uh[g].resize(nconf[g]);
            for (int64_t b = 0; b < nconf[g]; ++b)
                uh[g][b] = cdiv(make_double2(-1, 0), make_double2(Utilde[g][b].re, Utilde[g][b].im));
            NSLG_CUDA(cudaMemcpyAsync(const_cast<double2 *>(uin[g]), uh[g].data(), nconf[g] * sizeof(double2),
                                      cudaMemcpyHostToDevice, st));
        }
    }
    NSLG_TRY(leapfrog_group_dev(ngroups, fms, nconf, q.data(), p.data(), Ut.data(), uin.data(), traj_length, nmd,
                                backward, real_force, terms));
    for (int g = 0; g < ngroups; ++g) {
        const size_t bytes = (size_t)nconf[g] * fms[g]->Nt * fms[g]->Nx * sizeof(double2);
        NSLG_CUDA(cudaMemcpyAsync(q1[g], q[g], bytes, cudaMemcpyDefault, st));
        NSLG_CUDA(cudaMemcpyAsync(p1[g], p[g], bytes, cudaMemcpyDefault, st));
    }
    NSLG_CUDA(cudaStreamSynchronize(st));
    for (int g = 0; g < ngroups; ++g)
        if (fms[g]->force_precision != NSLG_PREC_FP64 && nconf[g] == 1) NSLG_TRY(check_tc_error(fms[g]));
    return NSLG_OK;
}

NSLG_API int nslg_hubbard_eval_batch_u(nslg_fm *fm, int64_t nconf, const nslg_c128 *phi, const nslg_c128 *Utilde,
                                       int terms, nslg_c128 *S) {
    NSLG_TRY(check_fm(fm));
    NSLG_REQUIRE(phi && S && Utilde, NSLG_ERR_ARG, "nslg_hubbard_eval_batch_u: null argument");
    NSLG_REQUIRE(nconf >= 1 && 2 * nconf <= 65535, NSLG_ERR_SHAPE,
                 "nslg_hubbard_eval_batch_u: need 1 <= nconf <= 32767");
    NSLG_REQUIRE(terms >= 1 && terms <= 3, NSLG_ERR_ARG, "nslg_hubbard_eval_batch_u: terms must be a mask of 1 and 2");
    std::vector<double2> ut(nconf);
    for (int64_t b = 0; b < nconf; ++b) {
        NSLG_REQUIRE(std::isfinite(Utilde[b].re) && std::isfinite(Utilde[b].im) &&
                         (Utilde[b].re != 0 || Utilde[b].im != 0),
                     NSLG_ERR_ARG, "nslg_hubbard_eval_batch_u: U~ must be finite and nonzero");
        ut[b] = make_double2(Utilde[b].re, Utilde[b].im);
    }
    const void *d;
    NSLG_TRY(stage_in(fm, "io_phib", phi, (size_t)nconf * fm->Nt * fm->Nx * sizeof(double2), &d));
    std::vector<double2> v(nconf);
    NSLG_TRY(hubbard_eval_batch_dev(fm, static_cast<const double2 *>(d), nconf, ut[0], terms, v.data(), ut.data()));
    for (int64_t b = 0; b < nconf; ++b) S[b] = nslg_c128{v[b].x, v[b].y};
    return NSLG_OK;
}

NSLG_API int nslg_hubbard_eval_batch(nslg_fm *fm, int64_t nconf, const nslg_c128 *phi, nslg_c128 Utilde, int terms,
                                     nslg_c128 *S) {
    NSLG_TRY(check_fm(fm));
    NSLG_REQUIRE(phi && S, NSLG_ERR_ARG, "nslg_hubbard_eval_batch: null argument");
    NSLG_REQUIRE(nconf >= 1 && 2 * nconf <= 65535, NSLG_ERR_SHAPE, "nslg_hubbard_eval_batch: need 1 <= nconf <= 32767");
    NSLG_REQUIRE(terms >= 1 && terms <= 3, NSLG_ERR_ARG, "nslg_hubbard_eval_batch: terms must be a mask of 1 and 2");
    const void *d;
    NSLG_TRY(stage_in(fm, "io_phib", phi, (size_t)nconf * fm->Nt * fm->Nx * sizeof(double2), &d));
    std::vector<double2> v(nconf);
    NSLG_TRY(hubbard_eval_batch_dev(fm, static_cast<const double2 *>(d), nconf, make_double2(Utilde.re, Utilde.im),
                                    terms, v.data()));
    for (int64_t b = 0; b < nconf; ++b) S[b] = nslg_c128{v[b].x, v[b].y};
    return NSLG_OK;
}

NSLG_API int nslg_kinetic(nslg_fm *fm, const nslg_c128 *p, nslg_c128 *out) {
    NSLG_TRY(check_fm(fm));
    NSLG_REQUIRE(p && out, NSLG_ERR_ARG, "nslg_kinetic: null argument");
    const void *d;
    NSLG_TRY(stage_in(fm, "io_p", p, (size_t)fm->Nt * fm->Nx * sizeof(double2), &d));
    int rc = NSLG_OK;
    const double2 s = sum_squares_host(fm, static_cast<const double2 *>(d), &rc);
    NSLG_TRY(rc);
    out->re = 0.5 * s.x;
    out->im = 0.5 * s.y;
    return NSLG_OK;
}

NSLG_API int nslg_kinetic_batch(nslg_fm *fm, int64_t nconf, const nslg_c128 *p, nslg_c128 *out) {
    NSLG_TRY(check_fm(fm));
    NSLG_REQUIRE(p && out, NSLG_ERR_ARG, "nslg_kinetic_batch: null argument");
    NSLG_REQUIRE(nconf >= 1 && nconf <= 2147483647, NSLG_ERR_SHAPE, "nslg_kinetic_batch: need nconf >= 1");
    const void *d;
    NSLG_TRY(stage_in(fm, "io_pb", p, (size_t)nconf * fm->Nt * fm->Nx * sizeof(double2), &d));
    return kinetic_batch_dev(fm, static_cast<const double2 *>(d), nconf, reinterpret_cast<double2 *>(out));
}

NSLG_API int nslg_accept_batch(nslg_fm *fm, int64_t nconf, const int32_t *accept, const nslg_c128 *q_new,
                               nslg_c128 *q) {
    NSLG_TRY(check_fm(fm));
    NSLG_REQUIRE(accept && q_new && q, NSLG_ERR_ARG, "nslg_accept_batch: null argument");
    NSLG_REQUIRE(nconf >= 1 && nconf <= 2147483647, NSLG_ERR_SHAPE, "nslg_accept_batch: need nconf >= 1");
    const size_t bytes = (size_t)nconf * fm->Nt * fm->Nx * sizeof(double2);
    NSLG_REQUIRE(q_new == q || !overlaps(q_new, bytes, q, bytes), NSLG_ERR_ARG,
                 "nslg_accept_batch: q_new and q overlap");
    if (q_new == q) return NSLG_OK;
    const void *dn;
    NSLG_TRY(stage_in(fm, "io_qnew", q_new, bytes, &dn));
    bool q_dev;
    NSLG_TRY(device_ptr(fm, q, &q_dev));
    double2 *dq;
    if (q_dev) {
        dq = reinterpret_cast<double2 *>(q);
    } else {
        NSLG_TRY(ws_get(fm, "io_q", bytes, reinterpret_cast<void **>(&dq)));
        NSLG_CUDA(cudaMemcpyAsync(dq, q, bytes, cudaMemcpyHostToDevice, fm->ctx->stream));
    }
    NSLG_TRY(accept_batch_dev(fm, nconf, accept, static_cast<const double2 *>(dn), dq));
    if (!q_dev) {
        NSLG_CUDA(cudaMemcpyAsync(q, dq, bytes, cudaMemcpyDeviceToHost, fm->ctx->stream));
        NSLG_CUDA(cudaStreamSynchronize(fm->ctx->stream));
    }
    return NSLG_OK;
}

namespace {
int cg_solve_abi(nslg_fm *fm, int op, const nslg_c128 *b, const nslg_c128 *x0, nslg_c128 *x, nslg_c128 *x_lo,
                 int64_t nbatch, double eps, int64_t max_iter, int mode, int precision, int stop, nslg_cg_stats *stats);
}

NSLG_API int nslg_cg_solve(nslg_fm *fm, int op, const nslg_c128 *b, const nslg_c128 *x0, nslg_c128 *x,
                           int64_t nbatch, double eps, int64_t max_iter, int mode, int precision, int stop,
                           nslg_cg_stats *stats) {
    return cg_solve_abi(fm, op, b, x0, x, nullptr, nbatch, eps, max_iter, mode, precision, stop, stats);
}

NSLG_API int nslg_cg_solve_dd(nslg_fm *fm, int op, const nslg_c128 *b, const nslg_c128 *x0, nslg_c128 *x,
                              nslg_c128 *x_lo, int64_t nbatch, double eps, int64_t max_iter, int mode, int precision,
                              nslg_cg_stats *stats) {
    return cg_solve_abi(fm, op, b, x0, x, x_lo, nbatch, eps, max_iter, mode, precision, NSLG_STOP_TRUE_RESIDUAL_DD,
                        stats);
}

namespace {
int cg_solve_abi(nslg_fm *fm, int op, const nslg_c128 *b, const nslg_c128 *x0, nslg_c128 *x, nslg_c128 *x_lo,
                 int64_t nbatch, double eps, int64_t max_iter, int mode, int precision, int stop, nslg_cg_stats *stats) {
    NSLG_TRY(check_fm(fm));
    NSLG_REQUIRE(b && x, NSLG_ERR_ARG, "nslg_cg_solve: null buffer");
    NSLG_REQUIRE(op >= NSLG_OP_M && op <= NSLG_OP_MDAGGERM, NSLG_ERR_ARG, "nslg_cg_solve: unknown operator");
    NSLG_REQUIRE(mode == NSLG_CG_SHARED || mode == NSLG_CG_PER_RHS, NSLG_ERR_ARG, "nslg_cg_solve: unknown mode");
    NSLG_REQUIRE(precision >= NSLG_PREC_FP64 && precision <= NSLG_PREC_BF16_SPLIT, NSLG_ERR_ARG,
                 "nslg_cg_solve: unknown precision");
    NSLG_REQUIRE(stop == NSLG_STOP_RECURRENCE || stop == NSLG_STOP_TRUE_RESIDUAL || stop == NSLG_STOP_TRUE_RESIDUAL_DD,
                 NSLG_ERR_ARG, "nslg_cg_solve: unknown stopping rule");
    NSLG_REQUIRE(stop != NSLG_STOP_TRUE_RESIDUAL_DD || fm->kind == NSLG_FM_EXP, NSLG_ERR_UNSUPPORTED,
                 "nslg_cg_solve: the double-double rule is implemented for the exponential discretisation");
    NSLG_REQUIRE(nbatch >= 1, NSLG_ERR_SHAPE, "nslg_cg_solve: nbatch must be >= 1");
    NSLG_REQUIRE(mode == NSLG_CG_SHARED || nbatch <= 65535, NSLG_ERR_SHAPE,
                 "nslg_cg_solve: at most 65535 independent systems per call");
    NSLG_REQUIRE(eps >= 0 && std::isfinite(eps), NSLG_ERR_ARG, "nslg_cg_solve: eps must be finite and >= 0");
    NSLG_REQUIRE(fm->populated, NSLG_ERR_STATE, "nslg_cg_solve: populate() has not been called");
    const int64_t n = nbatch * fm->Nt * fm->Nx;
    const size_t bytes = n * sizeof(double2);
    cudaStream_t st = fm->ctx->stream;
    NSLG_TRY(prepare_apply(fm, op, nbatch, precision));
    const void *db, *dx0;
    NSLG_TRY(stage_in(fm, "io_b", b, bytes, &db));
    if (x0) NSLG_TRY(stage_in(fm, "io_x0", x0, bytes, &dx0));
    else dx0 = db;
    bool out_dev;
    NSLG_TRY(device_ptr(fm, x, &out_dev));
    double2 *dx;
    if (out_dev && !overlaps(x, bytes, db, bytes)) dx = reinterpret_cast<double2 *>(x);
    else NSLG_TRY(ws_get(fm, "io_x", n, &dx));
    double2 *dlo = nullptr;
    if (x_lo) {
        NSLG_REQUIRE(!overlaps(x_lo, bytes, b, bytes) && !overlaps(x_lo, bytes, x, bytes) &&
                         !(x0 && overlaps(x_lo, bytes, x0, bytes)),
                     NSLG_ERR_ARG, "nslg_cg_solve_dd: x_lo overlaps b, x0 or x");
        bool lo_dev;
        NSLG_TRY(device_ptr(fm, x_lo, &lo_dev));
        if (lo_dev) dlo = reinterpret_cast<double2 *>(x_lo);
        else NSLG_TRY(ws_get(fm, "io_xlo", n, &dlo));
    }
    int rc = cg_solve(fm, op, static_cast<const double2 *>(db), static_cast<const double2 *>(dx0), dx, nbatch, eps,
                      max_iter, mode, precision, stop, stats, dlo);
    if (rc != NSLG_OK && rc != NSLG_NOT_CONVERGED) return rc;
    if (dx != reinterpret_cast<double2 *>(x)) NSLG_CUDA(cudaMemcpyAsync(x, dx, bytes, cudaMemcpyDefault, st));
    if (dlo && dlo != reinterpret_cast<double2 *>(x_lo))
        NSLG_CUDA(cudaMemcpyAsync(x_lo, dlo, bytes, cudaMemcpyDefault, st));
    NSLG_CUDA(cudaStreamSynchronize(st));
    if (precision >= NSLG_PREC_TF32X3) NSLG_TRY(check_tc_error(fm));
    return rc;
}
}  // namespace

NSLG_API int nslg_cg_solve_group(int nfm, nslg_fm *const *fms, int op, const nslg_c128 *const *b,
                                 const nslg_c128 *const *x0, nslg_c128 *const *x, nslg_c128 *const *x_lo,
                                 const int64_t *nbatch, const double *eps, int64_t max_iter, int precision, int stop,
                                 nslg_cg_stats *stats) {
    NSLG_REQUIRE(nfm >= 1 && fms && b && x && nbatch && eps, NSLG_ERR_ARG, "nslg_cg_solve_group: null argument");
    NSLG_REQUIRE(op >= NSLG_OP_M && op <= NSLG_OP_MDAGGERM, NSLG_ERR_ARG, "nslg_cg_solve_group: unknown operator");
    NSLG_REQUIRE(precision >= NSLG_PREC_FP64 && precision <= NSLG_PREC_BF16_SPLIT, NSLG_ERR_ARG,
                 "nslg_cg_solve_group: unknown precision");
    NSLG_REQUIRE(stop == NSLG_STOP_RECURRENCE || stop == NSLG_STOP_TRUE_RESIDUAL || stop == NSLG_STOP_TRUE_RESIDUAL_DD,
                 NSLG_ERR_ARG, "nslg_cg_solve_group: unknown stopping rule");
    int64_t systems = 0;
    for (int i = 0; i < nfm; ++i) {
        nslg_fm *f = fms[i];
        NSLG_REQUIRE(f != nullptr && b[i] && x[i], NSLG_ERR_ARG, "nslg_cg_solve_group: null handle or buffer");
        NSLG_REQUIRE(f->ctx == fms[0]->ctx, NSLG_ERR_ARG, "nslg_cg_solve_group: handles on different contexts");
        NSLG_REQUIRE(f->populated, NSLG_ERR_STATE, "nslg_cg_solve_group: populate() has not been called");
        NSLG_REQUIRE(nbatch[i] >= 1, NSLG_ERR_SHAPE, "nslg_cg_solve_group: nbatch[i] must be >= 1");
        NSLG_REQUIRE(eps[i] >= 0 && std::isfinite(eps[i]), NSLG_ERR_ARG, "nslg_cg_solve_group: eps must be finite");
        NSLG_REQUIRE(stop != NSLG_STOP_TRUE_RESIDUAL_DD || f->kind == NSLG_FM_EXP, NSLG_ERR_UNSUPPORTED,
                     "nslg_cg_solve_group: the double-double rule is implemented for the exponential discretisation");
        const size_t bytes = (size_t)nbatch[i] * f->Nt * f->Nx * sizeof(double2);
        NSLG_REQUIRE(!overlaps(x[i], bytes, b[i], bytes), NSLG_ERR_ARG, "nslg_cg_solve_group: x[i] overlaps b[i]");
        for (const void *pp : {(const void *)b[i], (const void *)x[i]}) {
            bool d;
            NSLG_TRY(device_ptr(f, pp, &d));
        }
        systems += nbatch[i];
    }
    NSLG_REQUIRE(systems <= 65535, NSLG_ERR_SHAPE, "nslg_cg_solve_group: at most 65535 systems");
    for (int i = 0; i < nfm; ++i) NSLG_TRY(prepare_apply(fms[i], op, nbatch[i], precision));
    std::vector<nslg_cg_stats *> sp(nfm, nullptr);
    if (stats)
        for (int i = 0; i < nfm; ++i) sp[i] = stats + i;
    const int rc = cg_solve_group(nfm, fms, op, reinterpret_cast<const double2 *const *>(b),
                                  reinterpret_cast<const double2 *const *>(x0), reinterpret_cast<double2 *const *>(x),
                                  reinterpret_cast<double2 *const *>(x_lo), nbatch, eps, max_iter, precision, stop,
                                  sp.data());
    if (rc != NSLG_OK && rc != NSLG_NOT_CONVERGED) return rc;
    if (precision >= NSLG_PREC_TF32X3)
        for (int i = 0; i < nfm; ++i) NSLG_TRY(check_tc_error(fms[i]));
    return rc;
}

NSLG_API int nslg_twobody_measure(nslg_fm *fm, const nslg_c128 *phi, const nslg_c128 *wall, int64_t nk, int64_t nb,
                                  const int64_t *tuples, int64_t ntuple, int64_t n_time_sources, double eps,
                                  int64_t max_iter, int precision, nslg_c128 *out, nslg_cg_stats *stats) {
    NSLG_TRY(check_fm(fm));
    NSLG_REQUIRE(phi && wall && out, NSLG_ERR_ARG, "nslg_twobody_measure: null buffer");
    NSLG_REQUIRE(nk >= 1 && nb >= 1 && nk * nb <= 65535, NSLG_ERR_SHAPE,
                 "nslg_twobody_measure: need 1 <= nk * nb <= 65535 wall sources");
    NSLG_REQUIRE(ntuple >= 0 && (ntuple == 0 || tuples), NSLG_ERR_ARG, "nslg_twobody_measure: bad tuple list");
    NSLG_REQUIRE(n_time_sources >= 1 && n_time_sources <= fm->Nt, NSLG_ERR_ARG,
                 "nslg_twobody_measure: need 1 <= n_time_sources <= Nt");
    NSLG_REQUIRE(eps >= 0 && std::isfinite(eps), NSLG_ERR_ARG, "nslg_twobody_measure: eps must be finite and >= 0");
    NSLG_REQUIRE(max_iter >= 1, NSLG_ERR_ARG, "nslg_twobody_measure: max_iter must be >= 1");
    NSLG_REQUIRE(precision >= NSLG_PREC_FP64 && precision <= NSLG_PREC_BF16_SPLIT, NSLG_ERR_ARG,
                 "nslg_twobody_measure: unknown precision");
    cudaStream_t st = fm->ctx->stream;
    const int64_t Nt = fm->Nt, Nx = fm->Nx;
    // the tuple list, checked on the host and uploaded as int32
    std::vector<int64_t> th((size_t)ntuple * 4);
    bool tuples_dev = false;
    if (ntuple > 0) NSLG_TRY(device_ptr(fm, tuples, &tuples_dev));
    if (ntuple > 0 && tuples_dev) {  // ordered on the context's stream like the call's other inputs
        NSLG_CUDA(cudaMemcpyAsync(th.data(), tuples, th.size() * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        NSLG_CUDA(cudaStreamSynchronize(st));
    } else if (ntuple > 0) {
        std::memcpy(th.data(), tuples, th.size() * sizeof(int64_t));
    }
    std::vector<int> t32(th.size());
    for (size_t i = 0; i < th.size(); ++i) {
        NSLG_REQUIRE(th[i] >= 0 && th[i] < nk, NSLG_ERR_ARG, "nslg_twobody_measure: momentum index out of range");
        t32[i] = (int)th[i];
    }
    int *dt = nullptr;
    if (ntuple > 0) {
        NSLG_TRY(ws_get(fm, "tb_tuples", t32.size(), &dt));
        NSLG_CUDA(cudaMemcpyAsync(dt, t32.data(), t32.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    }
    const void *dphi, *dwall;
    NSLG_TRY(stage_in(fm, "io_phi", phi, (size_t)Nt * Nx * sizeof(double2), &dphi));
    NSLG_TRY(stage_in(fm, "tb_wall", wall, (size_t)nk * nb * Nx * sizeof(double2), &dwall));
    const int64_t nout = (int64_t)NSLG_TB_NCHANNELS * ntuple * Nt * nb * nb * nb * nb;
    bool out_dev;
    NSLG_TRY(device_ptr(fm, out, &out_dev));
    double2 *dout;
    if (out_dev) dout = reinterpret_cast<double2 *>(out);
    else NSLG_TRY(ws_get(fm, "tb_out", (size_t)std::max<int64_t>(nout, 1), &dout));
    const int rc = twobody_measure(fm, static_cast<const double2 *>(dphi), static_cast<const double2 *>(dwall),
                                   (int)nk, (int)nb, dt, ntuple, (int)n_time_sources, eps, max_iter, precision, dout,
                                   stats);
    if (rc != NSLG_OK && rc != NSLG_NOT_CONVERGED) return rc;
    if (!out_dev && nout > 0)
        NSLG_CUDA(cudaMemcpyAsync(out, dout, (size_t)nout * sizeof(double2), cudaMemcpyDeviceToHost, st));
    NSLG_CUDA(cudaStreamSynchronize(st));
    if (precision >= NSLG_PREC_TF32X3) NSLG_TRY(check_tc_error(fm));
    return rc;
}

}  // extern "C"
