// Allocation-free operator application, for callers that cannot allocate device memory at the point of the call.
//
// Who needs it: latency-critical loops that forbid allocator traffic once they run, and hosts whose device memory
// is handed out up front by an external pool the library cannot draw from. nslg_fm_apply only allocates a workspace
// the first time it meets a shape, but it may; nslg_fm_apply_noalloc never does.
//
// The two-factor operators (M M^dagger and M^dagger M) need one intermediate vector (M^dagger psi, resp. M psi).
// Here it lives in a fixed device array of this file, g_noalloc_scratch, sized for NSLG_NOALLOC_MAX_ELEMS complex128
// values (2^21 values, 32 MiB), which every GPU that loads the library holds until the process exits. In host code
// the array's name is only a host-side stand-in, so its device address is looked up with cudaGetSymbolAddress, once
// per device, with that device current, on the first call on that device (the CUDA runtime may load this file's
// device code then, so that first call belongs in the caller's setup). Every call shares the array and the next
// call overwrites it: calls that overlap on the GPU (different streams, or concurrent host threads on one device)
// race. The intermediate is fully written by the first factor before the second reads it, so nothing in it needs
// clearing. The looked-up address is cached per device ordinal for the life of the process: a cudaDeviceReset
// unloads the module and makes it stale, so a device on which this entry point ran must not be reset (no handle of
// the library survives a reset either).
#include <mutex>

#include "fm_internal.cuh"

namespace nslg {
namespace {

constexpr int64_t NOALLOC_MAX_ELEMS = NSLG_NOALLOC_MAX_ELEMS;

static __device__ __align__(256) double2 g_noalloc_scratch[NOALLOC_MAX_ELEMS];

std::mutex g_noalloc_mu;
double2 *g_noalloc_ptr[128] = {};

// Device address of the scratch array on `device` (looked up once per device, with that device current).
int noalloc_scratch(int device, double2 **out) {
    NSLG_REQUIRE(device >= 0 && device < 128, NSLG_ERR_ARG, "nslg_fm_apply_noalloc: device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[device]) {
        int cur = -1;
        NSLG_CUDA(cudaGetDevice(&cur));
        if (cur != device) NSLG_CUDA(cudaSetDevice(device));
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (cur != device) cudaSetDevice(cur);
        NSLG_CUDA(e);
        g_noalloc_ptr[device] = static_cast<double2 *>(p);
    }
    *out = g_noalloc_ptr[device];
    return NSLG_OK;
}

// The memoised factor matrix (exp(d K), or d K for the diagonal discretisation), or null (a lookup only: computing
// it would allocate).
const ExpEntry *resident_exp(nslg_fm *fm, double2 d) {
    if (fm->kind == NSLG_FM_DIAG) {
        auto it = fm->lin.find(std::make_tuple(d.x, d.y, 0));
        return it == fm->lin.end() ? nullptr : &it->second;
    }
    auto it = fm->memo.find(std::make_pair(d.x, d.y));
    return it == fm->memo.end() ? nullptr : &it->second;
}

template <typename T>
int apply_factor(nslg_fm *fm, int mode, const ExpEntry *e, const double2 *in, double2 *out, int64_t rows) {
    const int Nt = (int)fm->Nt, Nx = (int)fm->Nx;
    if (fm->kind == NSLG_FM_DIAG) mode = mode == MODE_M ? MODE_DIAG_M : MODE_DIAG_MDAG;
    if constexpr (sizeof(T) == 8)
        return fm_apply_simt<double>(mode, in, out, fm->phase, e->re, e->is_real ? nullptr : e->im, Nt, Nx, rows,
                                     fm->ctx->stream);
    else
        return fm_apply_simt<float>(mode, in, out, fm->phase32, e->re32, e->is_real ? nullptr : e->im32, Nt, Nx,
                                    rows, fm->ctx->stream);
}

template <typename T>
int apply_noalloc(nslg_fm *fm, int op, const double2 *psi, double2 *out, int64_t nbatch, const ExpEntry *E,
                  const ExpEntry *Ec, double2 *scratch) {
    const int64_t rows = nbatch * fm->Nt;
    switch (op) {
        case NSLG_OP_M: return apply_factor<T>(fm, MODE_M, E, psi, out, rows);
        case NSLG_OP_MDAGGER: return apply_factor<T>(fm, MODE_MDAG, Ec, psi, out, rows);
        case NSLG_OP_MMDAGGER:
            NSLG_TRY(apply_factor<T>(fm, MODE_MDAG, Ec, psi, scratch, rows));
            return apply_factor<T>(fm, MODE_M, E, scratch, out, rows);
        default:
            NSLG_TRY(apply_factor<T>(fm, MODE_M, E, psi, scratch, rows));
            return apply_factor<T>(fm, MODE_MDAG, Ec, scratch, out, rows);
    }
}

}  // namespace
}  // namespace nslg

using namespace nslg;

extern "C" NSLG_API int nslg_fm_apply_noalloc(nslg_fm *fm, int op, const nslg_c128 *psi, nslg_c128 *out,
                                              int64_t nbatch, int precision) {
    NSLG_REQUIRE(fm != nullptr, NSLG_ERR_ARG, "nslg_fm_apply_noalloc: null handle");
    NSLG_REQUIRE(psi && out, NSLG_ERR_ARG, "nslg_fm_apply_noalloc: null buffer");
    NSLG_REQUIRE(op >= NSLG_OP_M && op <= NSLG_OP_MDAGGERM, NSLG_ERR_ARG, "nslg_fm_apply_noalloc: unknown operator");
    NSLG_REQUIRE(precision == NSLG_PREC_FP64 || precision == NSLG_PREC_FP32, NSLG_ERR_ARG,
                 "nslg_fm_apply_noalloc: precision must be NSLG_PREC_FP64 or NSLG_PREC_FP32");
    NSLG_REQUIRE(nbatch >= 0, NSLG_ERR_SHAPE, "nslg_fm_apply_noalloc: negative batch");
    NSLG_REQUIRE(fm->populated, NSLG_ERR_STATE, "nslg_fm_apply_noalloc: populate() has not been called");
    const int64_t n = nbatch * fm->Nt * fm->Nx;
    const size_t bytes = (size_t)n * sizeof(double2);
    if (n == 0) return NSLG_OK;
    NSLG_REQUIRE(n <= NSLG_NOALLOC_MAX_ELEMS || op == NSLG_OP_M || op == NSLG_OP_MDAGGER, NSLG_ERR_SHAPE,
                 "nslg_fm_apply_noalloc: nbatch*Nt*Nx = " + std::to_string(n) + " exceeds the scratch of " +
                     std::to_string((long long)NSLG_NOALLOC_MAX_ELEMS) + " complex values");
    bool psi_dev, out_dev;
    NSLG_TRY(device_ptr(fm, psi, &psi_dev));
    NSLG_TRY(device_ptr(fm, out, &out_dev));
    NSLG_REQUIRE(psi_dev && out_dev, NSLG_ERR_ARG,
                 "nslg_fm_apply_noalloc: psi and out must be device memory (host buffers would need staging)");
    const char *a = reinterpret_cast<const char *>(psi), *b = reinterpret_cast<const char *>(out);
    NSLG_REQUIRE(!(a < b + bytes && b < a + bytes), NSLG_ERR_ARG, "nslg_fm_apply_noalloc: psi and out overlap");
    const double2 d = make_double2(fm->sgn * fm->delta.x, fm->sgn * fm->delta.y);
    const double2 dc = make_double2(fm->sgn * fm->delta.x, -fm->sgn * fm->delta.y);
    const ExpEntry *E = resident_exp(fm, d), *Ec = resident_exp(fm, dc);
    NSLG_REQUIRE((op == NSLG_OP_MDAGGER || E) && (op == NSLG_OP_M || Ec), NSLG_ERR_STATE,
                 "nslg_fm_apply_noalloc: exp(delta K) is not resident yet; create it once with an allocating call "
                 "(nslg_fm_get_exp_hopping or nslg_fm_apply) before the first allocation-free call");
    double2 *scratch;
    NSLG_TRY(noalloc_scratch(fm->ctx->device, &scratch));
    const double2 *in = reinterpret_cast<const double2 *>(psi);
    double2 *o = reinterpret_cast<double2 *>(out);
    return precision == NSLG_PREC_FP64 ? apply_noalloc<double>(fm, op, in, o, nbatch, E, Ec, scratch)
                                       : apply_noalloc<float>(fm, op, in, o, nbatch, E, Ec, scratch);
}
