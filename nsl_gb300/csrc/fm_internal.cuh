// Internal state of the context and fermion-matrix handles, and the kernels' host-side launchers.
#pragma once

#include <cuda.h>

#include <atomic>
#include <map>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "nslg_common.cuh"
#include "ptr_class.h"

namespace nslg {

// Operator modes of the CUDA-core kernel: the exponential discretisation (M, M^dagger) and the diagonal one
// (HubbardDiag: the hopping acts within a time slice, the phase term is the shifted element-wise one).
enum { MODE_M = 0, MODE_MDAG = 1, MODE_DIAG_M = 2, MODE_DIAG_MDAG = 3 };
// Split-BF16 kernel only: a plain product out = (Y o pro) E^T (o epi), Y complex (rows, Nx), E real (Nx, Nx).
enum { MODE_OZ_GEMM = 4 };

// TF32 hi/lo planes of a real exp(d K) and their TMA descriptors (B operand of the tensor-core operator).
struct TcPlanes {
    float *hi = nullptr, *lo = nullptr;  // (Nx, ld) row-major, ld = Nx rounded up to 32, zero padded
    int ld = 0;
    int bn = 0;  // tile width in output sites
    CUtensorMap map_hi, map_lo;
};

// Split-BF16 digit planes of a real exp(d K) (S planes stacked along rows), per-row scale exponents and the TMA
// descriptor (B operand of the exact-accumulation tensor-core operator).
struct OzPlanes {
    void *planes = nullptr;  // BF16, (S * Nx, ld)
    int *col_exp = nullptr;  // (Nx)
    int ld = 0;
    CUtensorMap map;
};

// exp(d K) memo entry (SpatialLattice::exp_hopping_matrix, lattice.tpp:52-58), kept in the layouts the kernels read.
struct ExpEntry {
    double2 *full = nullptr;  // complex (Nx, Nx) row-major
    double *re = nullptr;     // real plane, FP64
    double *im = nullptr;     // imaginary plane, FP64 (null when exp(d K) is exactly real)
    float *re32 = nullptr;    // FP32 copies for the mixed-precision inner operator
    float *im32 = nullptr;
    bool is_real = true;
    TcPlanes *tc = nullptr;   // built on first tensor-core use
    OzPlanes *oz = nullptr;   // built on first split-BF16 use
};

// Operator-arithmetic tags for the tensor-core operators (3xTF32; split BF16 with exact accumulation).
struct TF32x3 {};
struct BF16Split {};

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

}  // namespace nslg

struct nslg_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int num_sms = 0;
    // One reference for the caller's handle and one per fermion matrix created on it: the context (and its stream)
    // is released when the last of them goes, so handles may be destroyed in any order.
    std::atomic<int> refs{1};
};

struct nslg_fm {
    nslg_ctx *ctx = nullptr;
    int64_t Nx = 0, Nt = 0;
    double2 delta{0, 0};     // beta / Nt
    double2 mu_tilde{0, 0};  // delta * mu
    int species = NSLG_PARTICLE;
    int sgn = 1;
    double2 *hops = nullptr;  // K (Nx, Nx)
    double hops_norm1 = 0;    // max column sum of |K| (bounds its spectral radius)
    double2 hops_trace{0, 0}; // tr K
    int stabilisation = NSLG_STAB_AUTO;  // log det / gradient form (nslg_stabilisation)
    std::map<std::pair<double, double>, nslg::ExpEntry> memo;
    int kind = NSLG_FM_EXP;  // discretisation (nslg_fm_kind)
    // HubbardDiag matrices: d K (one_minus = 0) and 1 - d K (one_minus = 1), keyed by (d, one_minus)
    std::map<std::tuple<double, double, int>, nslg::ExpEntry> lin;
    double2 *phi = nullptr;        // (Nt, Nx)
    double2 *phase = nullptr;      // exp(i sgn phi + sgn mu_tilde)
    double2 *phase_inv = nullptr;  // exp(-i sgn phi - sgn mu_tilde)
    float2 *phase32 = nullptr;
    bool populated = false;
    int *tc_err = nullptr;  // device flag a tensor-core kernel sets if one of its bounded waits gives up
    // a second stream for independent work of one call (the hole species' tensor-core chains of a force), forked
    // from and joined back to ctx->stream with the two events; created on first use
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    std::map<std::string, nslg::DevBuf> ws;
    uint64_t ws_generation = 0;  // bumped whenever a workspace buffer moves (invalidates captured graphs)
    std::map<std::string, cudaGraphExec_t> graphs;
    std::map<std::string, uint64_t> graph_kernels;  // kernel nodes per captured graph
    // the captured (not instantiated) trajectory graphs, kept so that a group of handles can launch the trajectories
    // of all its members as the branches of one graph
    std::map<std::string, cudaGraph_t> graph_defs;
    uint64_t uid = 0;  // unique per handle over the process (keys of graphs that span several handles)
    // leapfrog trajectories run eagerly once per shape (to build every workspace and exp(delta K) entry), are
    // captured into a CUDA graph on the next call and replayed after that
    std::map<std::string, int> lf_seen;
    // set while a trajectory is captured: the gradient skips its host-side singularity check (it would synchronise)
    // and the LU keeps its singular flag sticky, so the trajectory checks it once after the replay
    bool defer_checks = false;
    // arithmetic of the log-det gradient (the HMC force): NSLG_PREC_FP64 or NSLG_PREC_BF16_SPLIT (tensor cores)
    int force_precision = NSLG_PREC_FP64;
};

namespace nslg {

// ----- workspace -------------------------------------------------------------------------------------------------
// Returns a device buffer of at least `bytes` kept in the handle under `name` (grown on demand, freed with the
// handle).
int ws_get(nslg_fm *fm, const char *name, size_t bytes, void **out);
template <typename P> int ws_get(nslg_fm *fm, const char *name, size_t count, P **out) {
    return ws_get(fm, name, count * sizeof(P), reinterpret_cast<void **>(out));
}

// Destroys every captured graph of the handle (a workspace moved, or a setting the graphs bake in changed).
void drop_graphs(nslg_fm *fm);

// ----- pointer staging -------------------------------------------------------------------------------------------
// *dev = whether p is device memory the handle's GPU can address (device memory of that GPU, or managed memory);
// unregistered or pinned host memory gives false. Device memory of another GPU is NSLG_ERR_ARG: the library enables
// no peer access, so a kernel on the handle's GPU could not read it.
int device_ptr(const nslg_fm *fm, const void *p, bool *dev);

// ----- exp(d K) -----------------------------------------------------------------------------------------------------
int get_exp(nslg_fm *fm, double2 d, const ExpEntry **out);
// d K (one_minus = 0) or 1 - d K (one_minus = 1) for the diagonal discretisation, memoised like exp(d K).
int get_lin(nslg_fm *fm, double2 d, int one_minus, const ExpEntry **out);
// The matrix of one operator factor for the handle's discretisation: exp(d K) or d K.
int get_factor(nslg_fm *fm, double2 d, const ExpEntry **out);
int install_exp(nslg_fm *fm, double2 d, const double2 *E_dev);

// ----- kernels (launchers) ---------------------------------------------------------------------------------------
// Fused M / Mdag application on FP64 vectors with the product in T (double: FP64 drop-in; float: FP32 operator).
// With sys_mask only tiles holding rows of systems s (sys_rows consecutive rows each) with sys_mask[s] != 0 compute.
template <typename T>
int fm_apply_simt(int mode, const double2 *psi, double2 *out, const cplx_t<T> *phase, const T *Ere, const T *Eim,
                  int Nt, int Nx, int64_t rows, cudaStream_t st, const int *sys_mask = nullptr,
                  int64_t sys_rows = 1);

// out = op(psi) for op in {M, Mdag, MMdag, MdagM} on FP64 device buffers (nbatch, Nt, Nx), products in T. sys_mask
// (FP64 products only) restricts the work to the rows of flagged systems (sys_rows rows each); the other rows of
// out are left unspecified.
template <typename T>
int fm_apply_dev(nslg_fm *fm, int op, const double2 *psi, double2 *out, int64_t nbatch,
                 const int *sys_mask = nullptr, int64_t sys_rows = 1);

// C[b] = alpha * A[b] @ B[b] (+ I if add_identity), complex FP64, row-major, batched with element strides.
int zgemm(cudaStream_t st, int M, int N, int K, double2 alpha, const double2 *A, int64_t lda, int64_t sA,
          const double2 *B, int64_t ldb, int64_t sB, double2 *C, int64_t ldc, int64_t sC, int batch,
          bool add_identity, bool accumulate = false);
// Two-level batched product (batch x batch2 products, element offsets z1 * s + z2 * s2); real: 1 = A holds real
// numbers, 2 = B does (imaginary parts zero: half the FMAs).
int zgemm2(cudaStream_t st, int M, int N, int K, double2 alpha, const double2 *A, int64_t lda, int64_t sA,
           int64_t sA2, const double2 *B, int64_t ldb, int64_t sB, int64_t sB2, double2 *C, int64_t ldc, int64_t sC,
           int64_t sC2, int batch, int batch2, int real = 0);

int compute_phases(nslg_fm *fm);
int populate_dev(nslg_fm *fm, const double2 *phi, int species);  // phi: device buffer (Nt, Nx)
// Batched FP64 gradient / log det over nmat matrices (logdet.cu): matrix g uses (g & emask) ? E1 : E0 and the
// phase rows at ph + g * Nt * Nx; grad out (nmat, Nt, Nx) on the device, log det out[nmat] on the host.
int grad_logdet_many(nslg_fm *fm, int nmat, const double2 *E0, const double2 *E1, int emask, const double2 *ph_inv,
                     double2 *out);
int logdet_many(nslg_fm *fm, int nmat, const double2 *E0, const double2 *E1, int emask, const double2 *ph,
                double2 *out);
// Split-BF16 (tensor-core) gradient for nmat matrices with factors E[g] (real, Nx <= 2048); LU and solves batched.
int grad_logdet_tc_many(nslg_fm *fm, int nmat, const ExpEntry *const *E, const double2 *ph_inv, double2 *out);
int prepare_apply(nslg_fm *fm, int op, int64_t nbatch, int precision);
// CG on op (cg.cu); x_lo (optional) receives the low part of the solution under the double-double rule.
int cg_solve(nslg_fm *fm, int op, const double2 *b, const double2 *x0, double2 *x, int64_t nbatch, double eps,
             int64_t max_iter, int mode, int precision, int stop, nslg_cg_stats *stats, double2 *x_lo = nullptr);
// CG on a group of fermion matrices of different sizes (cg.cu), per-RHS systems, one launch sequence.
int cg_solve_group(int nfm, nslg_fm *const *fms, int op, const double2 *const *b, const double2 *const *x0,
                   double2 *const *x, double2 *const *x_lo, const int64_t *nbatch, const double *eps,
                   int64_t max_iter, int precision, int stop, nslg_cg_stats *const *stats);
// (oh + ol) = op (xh + xl) in double-double arithmetic (fm_apply_dd.cu, exponential discretisation); with sys_mask
// only the rows of systems s (sys_rows rows each) with sys_mask[s] != 0 are written.
int fm_apply_dd(nslg_fm *fm, int op, const double2 *xh, const double2 *xl, double2 *oh, double2 *ol, int64_t nbatch,
                const int *sys_mask, int64_t sys_rows);
// Stratified (UDT) log det and gradient (stable.cu): whether the handle uses them, and the batched forms over nmat
// matrices with factors Ep[g] = exp(-sgn_g delta K), E[g] = exp(sgn_g delta K) and phase rows ph / pinv
// (nmat, Nt, Nx).
bool use_stratified(const nslg_fm *fm);
bool use_stratified_grad(const nslg_fm *fm);
int grad_logdet_strat(nslg_fm *fm, int nmat, const ExpEntry *const *Ep, const ExpEntry *const *E, const double2 *ph,
                      const double2 *pinv, double2 *out);
int logdet_strat(nslg_fm *fm, int nmat, const ExpEntry *const *Ep, const ExpEntry *const *E, const int *sgn,
                 const double2 *ph, const double2 *pinv, double2 *out);

// ----- batched dense LU (logdet.cu) --------------------------------------------------------------------------------
struct LuScratch {
    int *piv;
    double2 *pivots;  // u_kk per matrix (n each)
    double2 *logsum;  // sum of log u_kk per matrix (principal logs)
    int *swaps;       // row swaps per matrix
    int *singular;    // set if a zero pivot occurred (shared by the batch)
};
// Scratch of a batch of nmat LU factorisations of size n; `tag` names an independent set (two factorisations whose
// pivots are both needed later take different tags).
int get_lu_scratch(nslg_fm *fm, int n, LuScratch &s, int nmat = 1, const char *tag = nullptr);
// Right-looking blocked LU of nmat matrices at A + g * mstride (mstride 0: n * n), in place. With pivoting: partial
// pivoting (largest modulus, first index on ties); without: the diagonal is the pivot (Hermitian positive definite
// matrices, where it is the Cholesky factorisation with U = diag(U) L^H).
int lu_factor(nslg_fm *fm, double2 *A, int n, LuScratch &s, int nmat = 1, int64_t mstride = 0,
              bool want_logsum = true, bool pivoting = true);
// G[g] = A_g^{-1} from the factors (G dense (nmat, n, n)).
int lu_inverse(nslg_fm *fm, const double2 *LU, double2 *G, int n, const LuScratch &s, int nmat = 1,
               int64_t lu_stride = 0);
// B[g] = L_g^{-1} B[g] (n x n right-hand sides) with the unit lower factor of an unpivoted LU.
int lu_forward(nslg_fm *fm, const double2 *LU, double2 *B, int n, int nmat, int64_t lu_stride, int64_t b_stride);
int compute_hops_norm(nslg_fm *fm);

// Tensor-core operator: planes of a real exp(d K) (built once per entry) and the fused M / Mdag launch.
int tc_planes(nslg_fm *fm, const ExpEntry *e, TcPlanes **out);
int fm_apply_tc(int mode, const double2 *psi, double2 *out, const double2 *phase, const TcPlanes &P, int Nt, int Nx,
                int64_t rows, int *err, cudaStream_t st);
int oz_planes(nslg_fm *fm, const ExpEntry *e, OzPlanes **out);
int oz_ld(int Nx);   // digit-plane row length (Nx rounded up to the 32-site k-block)
int oz_digits();     // digits per operand
// Epilogue extensions of the split-BF16 kernel for the CG on MM^dagger / M^dagger M (mode 0: plain application).
// mode 1 (first factor): out is written and part[(2 row + c) * oz_ntiles(Nx) + n-tile] = sum of out^2 over the
//   tile's sites, the curvature partial sums |M^dagger p|^2.
// mode 2 (second factor): out is not written; for systems with active[s] the CG residual update
//   r -= alpha[s] (A p) is applied in place and part holds the partial sums of the new |r|^2. A system is the
//   sys_rows consecutive complex rows s * sys_rows ...
struct OzEpi {
    int mode = 0;
    double *part = nullptr;
    const double *alpha = nullptr;
    const int *active = nullptr;
    double2 *r = nullptr;
    int64_t sys_rows = 1;
    // with go: rows of systems s with go[s] == 0 are skipped (their digits are not written, tiles of such rows only
    // return at once); their outputs and partial sums are left unwritten
    const int *go = nullptr;
    // mode 1 with M^dagger: also u = phase o out, the operand of a following M application, from the epilogue
    double2 *u = nullptr;
    // with operand: the digit pre-pass reads this vector as it is (for M: phase o psi already formed, e.g. the u of
    // the preceding M^dagger) instead of forming phase o psi; psi is still the epilogue's psi
    const double2 *operand = nullptr;
    // the operand's digit planes and row scales are already in digits / rexp (written by the CG kernel that formed
    // the operand): the pre-pass is skipped
    bool digits_ready = false;
};
int oz_ntiles(int Nx);  // output-site tiles of the split-BF16 kernel (partial sums per row)
// out[j, i] = sum_k Y[j, k] pro[k] E[i, k] epi[i] on the tensor cores (split-BF16, FP64-class), Y and out complex
// (rows, Nx), E the real matrix of the planes P; pro / epi may be null (no scale). digits / rexp as fm_apply_oz.
int oz_gemm(const double2 *Y, double2 *out, const double2 *pro_scale, const double2 *epi_scale, const OzPlanes &P,
            void *digits, int *rexp, int Nx, int64_t rows, int *err, cudaStream_t st);
// digits: workspace of oz_digits() * 2 * rows * oz_ld(Nx) BF16; rexp: 2 * rows ints (per-row scale exponents).
int fm_apply_oz(int mode, const double2 *psi, double2 *out, const double2 *phase, const OzPlanes &P, void *digits,
                int *rexp, int Nt, int Nx, int64_t rows, int *err, cudaStream_t st, const OzEpi *epi = nullptr);

}  // namespace nslg
