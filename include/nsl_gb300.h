/* C ABI of libnslgpu: the GB300 (sm_103a) implementation of NSL's fermion-matrix hot path.
 *
 * Every entry point replaces one member of the reference NSL C++ API (paths inside the NSL source tree):
 * the HubbardExp fermion matrix (src/NSL/FermionMatrix/Impl/hubbardExp.{hpp,tpp}), the CG solver
 * (src/NSL/LinAlg/Solver/Impl/CG.{hpp,tpp}), the Hubbard gauge and fermion actions
 * (src/NSL/Action/Implementations/hubbard{Gauge,Fermi}Action.tpp) and the leapfrog integrators
 * (src/NSL/Integrator/Impl/leapfrog{,RealForce}.tpp).
 *
 * Conventions
 *  - Tensors are complex128, interleaved (re, im), row-major and contiguous: exactly the storage behind
 *    NSL::Tensor<NSL::complex<double>>::data() (src/NSL/Tensor/Impl/randomAccess.tpp:97-99). Fields phi and
 *    momenta are (Nt, Nx); pseudo-fermion vectors are (nbatch, Nt, Nx) with any leading batch dims flattened.
 *  - Pointers may be host or device memory (cudaPointerGetAttributes decides). Host buffers are staged through
 *    the handle's device workspace and the call returns when the result is in host memory. Device buffers must
 *    be memory of the context's GPU (or managed memory); another GPU's memory is NSLG_ERR_ARG. Calls on device
 *    buffers are ordered on the context's stream; nslg_ctx_synchronize() waits for them.
 *  - The caller owns every buffer it passes. The library owns only handle-resident state (exp(delta K), phases,
 *    workspaces).
 *  - Every function returns an nslg_status; nslg_last_error() gives the message of the last failure on the calling
 *    host thread. Argument errors are reported, never aborted on. CG non-convergence is NSLG_NOT_CONVERGED with
 *    the best iterate written to x (the reference logs an error and returns x, CG.tpp:90-93).
 *  - A handle is used by one host thread at a time (the reference objects hold mutable workspaces,
 *    hubbardExp.hpp:201-212).
 */
#ifndef NSL_GB300_H
#define NSL_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NSLG_API __attribute__((visibility("default")))

typedef struct {
    double re, im;
} nslg_c128;

typedef struct nslg_ctx nslg_ctx;
typedef struct nslg_fm nslg_fm;

typedef enum {
    NSLG_OK = 0,
    NSLG_ERR_ARG = 1,         /* invalid argument (null pointer, unknown enum, aliasing) */
    NSLG_ERR_SHAPE = 2,       /* sizes out of range */
    NSLG_ERR_OOM = 3,         /* device allocation failed */
    NSLG_ERR_CUDA = 4,        /* a CUDA runtime call failed */
    NSLG_NOT_CONVERGED = 5,   /* CG reached max_iter; x holds the last iterate */
    NSLG_ERR_UNSUPPORTED = 7, /* valid request the library does not support */
    NSLG_ERR_STATE = 8        /* call order violated (e.g. apply before populate) */
} nslg_status;

/* NSL::FermionMatrix::MatrixCombination, same order (src/NSL/LinAlg/Solver/applicationType.tpp:18). */
typedef enum { NSLG_OP_M = 0, NSLG_OP_MDAGGER = 1, NSLG_OP_MMDAGGER = 2, NSLG_OP_MDAGGERM = 3 } nslg_op;

/* NSL::Hubbard::Species (src/NSL/Action/Implementations/hubbard.tpp:7). */
typedef enum { NSLG_PARTICLE = 0, NSLG_HOLE = 1 } nslg_species;
/* Discretisation of the fermion matrix: HubbardExp (src/NSL/FermionMatrix/Impl/hubbardExp.hpp) or HubbardDiag
 * (src/NSL/FermionMatrix/Impl/hubbardDiag.hpp: (M psi)_t = psi_t - sgn delta K psi_t - B_t e^{i sgn phi_{t-1} +
 * sgn mu~} psi_{t-1}). */
typedef enum { NSLG_FM_EXP = 0, NSLG_FM_DIAG = 1 } nslg_fm_kind;

/* Arithmetic of the operator applications (vectors are FP64 in every form). FP64 is the drop-in; FP32 runs the
 * products on CUDA cores in FP32; TF32X3 runs them on the tensor cores as three TF32 MMAs (hi*hi + hi*lo + lo*hi)
 * with FP32 accumulation in TMEM, as accurate as FP32 (a complex exp(delta K) uses the FP32 CUDA-core kernel).
 * BF16_SPLIT is FP64-class on the tensor cores: operand and exp(delta K) rows rounded to 53-bit integers at per-row
 * power-of-two scales and cut into six balanced 9-bit digits (exact in BF16), 21 BF16 digit products per K step
 * accumulated exactly in FP32 TMEM and recombined in 64-bit integers (~1e-15 relative to the output's maximum, an
 * FP64 product's error; complex exp(delta K) or Nx > 2048 use the FP64 CUDA-core kernel). Exactness is proven per
 * exp(delta K) from its own digits; a matrix that fails the bound (delta >= 2 on lattices of ~300 sites and up) makes
 * every split-BF16 application report NSLG_ERR_CUDA ("too delocalised") instead of an inexact result. */
typedef enum { NSLG_PREC_FP64 = 0, NSLG_PREC_FP32 = 1, NSLG_PREC_TF32X3 = 2, NSLG_PREC_BF16_SPLIT = 3 } nslg_precision;

/* CG batch semantics. SHARED is the reference's: one CG over the whole batch with alpha/beta summed over every
 * element (src/NSL/LinAlg/inner_product.tpp:30-33). PER_RHS runs an independent CG per right-hand side (per-instance
 * convergence masking). */
typedef enum { NSLG_CG_SHARED = 0, NSLG_CG_PER_RHS = 1 } nslg_cg_mode;

/* CG stopping rule. RECURRENCE is the reference's: |r|^2 <= eps^2 on the recurrence residual (CG.tpp:70), FP64
 * operator only. TRUE_RESIDUAL stops on the FP64 true residual |b - A x| <= eps, with FP64 reliable updates (r is
 * recomputed as b - A x in FP64 whenever the recurrence residual has dropped below its running maximum by 1e4 for
 * FP64-class operators, 100 for FP32-class ones); it is always used for FP32 operators. Its accuracy ends where FP64
 * can represent x and evaluate A x: ~1e-16 |A| |x|, i.e. 1e-9..1e-8 |b| at beta = 8 on honeycomb 12x12.
 * TRUE_RESIDUAL_DD certifies below that: the solution is accumulated as a double-double pair x + x_lo, the FP64
 * reliable updates work on the increment since the last rebase, and a rebase (when the FP64 residual of the increment
 * has fallen 1e5 below the last rebase's, stops improving, or meets eps) folds the increment into the pair and
 * evaluates b - A (x + x_lo) in double-double arithmetic (~1e-30 relative to |A| |x|); only that residual can meet eps.
 * Exponential discretisation only. No counterpart in the reference. */
typedef enum { NSLG_STOP_RECURRENCE = 0, NSLG_STOP_TRUE_RESIDUAL = 1, NSLG_STOP_TRUE_RESIDUAL_DD = 2 } nslg_cg_stop;

typedef struct {
    int64_t iterations;         /* inner iterations of the slowest system */
    int64_t reliable_updates;   /* FP64 true-residual recomputations (mixed precision) */
    int64_t converged;          /* systems that met the stopping rule */
    int64_t systems;            /* systems solved (1 in SHARED mode, nbatch in PER_RHS mode) */
    double recurrence_residual; /* max over systems of |r| of the recurrence at exit */
    double true_residual;       /* max over systems of |b - A x| / |b| at exit (FP64; double-double, of x + x_lo,
                                   under NSLG_STOP_TRUE_RESIDUAL_DD) */
    int64_t escalated;          /* 1 if the low-precision operator stalled and the solve finished in FP64 */
    int64_t dd_rebases;         /* double-double residual evaluations (NSLG_STOP_TRUE_RESIDUAL_DD) */
} nslg_cg_stats;

/* ----- library and context --------------------------------------------------------------------------------- */
NSLG_API int nslg_version(void);
NSLG_API const char *nslg_last_error(void);
/* Number of kernels this library has launched in the process so far (graph replays count each kernel node). */
NSLG_API uint64_t nslg_kernel_launches(void);
/* device: CUDA ordinal; stream: a cudaStream_t to order work on, or NULL for a stream the context creates.
 * Replaces NSL::Device selection (src/NSL/device.tpp:22-143). */
NSLG_API int nslg_ctx_create(int device, void *stream, nslg_ctx **out);
/* Releases the caller's handle. Fermion matrices created on the context keep it (and its stream) alive until the
 * last of them is destroyed, so the handles may be destroyed in any order. */
NSLG_API int nslg_ctx_destroy(nslg_ctx *ctx);
NSLG_API int nslg_ctx_synchronize(nslg_ctx *ctx);
/* The cudaStream_t the context orders its work on (for event-based ordering with other stream users). */
NSLG_API void *nslg_ctx_stream(nslg_ctx *ctx);

/* ----- HubbardExp ------------------------------------------------------------------------------------------ */
/* Replaces HubbardExp(Species, LatticeType&, Nt, beta, mu) (src/NSL/FermionMatrix/Impl/hubbardExp.hpp:48-76).
 * hops is the lattice hopping matrix K (Nx, Nx) (SpatialLattice::hopping_matrix, src/NSL/Lattice/lattice.tpp:47-49).
 * delta = beta/Nt and mu_tilde = delta*mu as in hubbardExp.hpp:51-52. exp(d K) for the deltas the operators need
 * is computed on the device on first use and memoised per handle, like SpatialLattice::exp_hopping_matrix
 * (lattice.tpp:52-58); nslg_fm_set_exp_hopping() installs a caller-provided one instead. */
NSLG_API int nslg_fm_create(nslg_ctx *ctx, int64_t Nx, int64_t Nt, const nslg_c128 *hops, nslg_c128 beta,
                            nslg_c128 mu, int species, nslg_fm **out);
/* As nslg_fm_create for a chosen discretisation: replaces the HubbardDiag constructors (hubbardDiag.hpp:44-93)
 * when kind is NSLG_FM_DIAG. HubbardDiag applies its operators in FP64 or FP32 (NSLG_PREC_TF32X3 and
 * NSLG_PREC_BF16_SPLIT give NSLG_ERR_UNSUPPORTED); log det, its gradient, actions, leapfrog and CG work as for
 * HubbardExp. */
NSLG_API int nslg_fm_create_kind(nslg_ctx *ctx, int kind, int64_t Nx, int64_t Nt, const nslg_c128 *hops,
                                 nslg_c128 beta, nslg_c128 mu, int species, nslg_fm **out);
NSLG_API int nslg_fm_destroy(nslg_fm *fm);
/* Installs exp(delta K) (Nx, Nx) for the key delta (the reference memo entry, lattice.tpp:52-58). */
NSLG_API int nslg_fm_set_exp_hopping(nslg_fm *fm, nslg_c128 delta, const nslg_c128 *expK);
/* Copies exp(delta K) for the key delta into out (Nx, Nx), computing it if it is not memoised yet. */
NSLG_API int nslg_fm_get_exp_hopping(nslg_fm *fm, nslg_c128 delta, nslg_c128 *out);
/* Replaces HubbardExp::populate(phi[, species]) (hubbardExp.hpp:103-128). species < 0 keeps the current one. */
NSLG_API int nslg_fm_populate(nslg_fm *fm, const nslg_c128 *phi, int species);
/* Copies the phase factors phiExp = exp(i sgn phi + sgn mu~) (Nt, Nx) of the populated configuration (the member
 * phiExp_ of hubbardExp.hpp:116-128) into out: with exp(delta K) (nslg_fm_get_exp_hopping) they define the FP64
 * operator exactly, e.g. for checking a double-double residual elsewhere. */
NSLG_API int nslg_fm_get_phases(nslg_fm *fm, nslg_c128 *out);
/* Replaces HubbardExp::M / Mdagger / MMdagger / MdaggerM (hubbardExp.tpp:39-125). psi and out are
 * (nbatch, Nt, Nx) and must not overlap. With device buffers the call is asynchronous on the context's stream; a
 * timeout inside a tensor-core kernel (NSLG_PREC_TF32X3, NSLG_PREC_BF16_SPLIT) is then reported as NSLG_ERR_CUDA by
 * the next call on this handle that synchronises (host buffers, nslg_cg_solve). */
NSLG_API int nslg_fm_apply(nslg_fm *fm, int op, const nslg_c128 *psi, nslg_c128 *out, int64_t nbatch,
                           int precision);

/* op applied in double-double arithmetic (~1e-30 relative to |op| |psi|): (out_hi + out_lo) = op (psi_hi + psi_lo)
 * with the handle's FP64 exp(delta K) and phases, the residual evaluation of NSLG_STOP_TRUE_RESIDUAL_DD. psi_lo may
 * be NULL (zero). Exponential discretisation only; buffers (nbatch, Nt, Nx), host or device, the outputs not
 * overlapping the inputs. No counterpart in the reference. */
NSLG_API int nslg_fm_apply_dd(nslg_fm *fm, int op, const nslg_c128 *psi_hi, const nslg_c128 *psi_lo,
                              nslg_c128 *out_hi, nslg_c128 *out_lo, int64_t nbatch);

/* Replaces HubbardExp::logDetM (hubbardExp.tpp:129-150): log det M = log det(1 + B_{Nt-1} ... B_0) for the
 * populated phi and current species, FP64, on the principal branch (Im in (-pi, pi]) like log(det(.))
 * (src/NSL/LinAlg/det.tpp:15-20); evaluated as a sum of logs of LU pivots, so it stays finite where det overflows. */
NSLG_API int nslg_fm_logdet(nslg_fm *fm, nslg_c128 *out);
/* Replaces HubbardExp::gradLogDetM (hubbardExp.tpp:153-211): out (Nt, Nx) = d log det M / d phi, FP64. */
NSLG_API int nslg_fm_grad_logdet(nslg_fm *fm, nslg_c128 *out);
/* Arithmetic of gradLogDetM and therefore of the action force and the leapfrog: NSLG_PREC_FP64 (default, the
 * reference's) or NSLG_PREC_BF16_SPLIT, where the two matrix chains run as split-BF16 tensor-core products
 * (FP64-class, ~1e-13 per product; the LU stays FP64). Applies to the exponential discretisation with a real
 * exp(delta K) and Nx <= 2048, otherwise the FP64 path runs. log det M (the action value, Delta H) is always FP64. */
NSLG_API int nslg_fm_set_force_precision(nslg_fm *fm, int precision);

/* Form of log det M and its gradient (the action, the force, the leapfrog and Delta H). PLAIN is the reference's
 * algorithm (hubbardExp.tpp:129-211): one product of the Nt time slices, LU of 1 + product; in FP64 it loses about
 * log10(e^{beta rho}) - 16 digits (rho = the largest |eigenvalue| of K): ~1e-7 relative at beta = 8 and no correct digit
 * at beta = 12 on the honeycomb lattices. STRATIFIED keeps the slice products as U D T factorisations (unitary U
 * from Cholesky-QR, graded scales D, well-conditioned T) at chunk boundaries, evaluates the equal-time Green
 * function (1 + C(s))^{-1} there without mixing the scales, and carries it between boundaries by similarity
 * transforms: ~1e-13 relative at any beta (FP64, whatever nslg_fm_set_force_precision selected). AUTO (default)
 * takes STRATIFIED when beta * rho > 14, where PLAIN's error would exceed ~1e-12. The diagonal discretisation always
 * runs PLAIN. No counterpart in the reference. */
typedef enum { NSLG_STAB_AUTO = 0, NSLG_STAB_PLAIN = 1, NSLG_STAB_STRATIFIED = 2 } nslg_stabilisation;
NSLG_API int nslg_fm_set_stabilisation(nslg_fm *fm, int mode);

/* Allocation-free variant of nslg_fm_apply; it has no counterpart in the reference. It is for callers that must not
 * allocate device memory at the point of the call: latency-critical loops that forbid allocator traffic once they
 * run, and hosts whose device memory is handed out up front by a pool the library cannot draw from. nslg_fm_apply
 * allocates a workspace the first time it meets a shape; this call never allocates. Limits: psi and out must be
 * device memory (no host staging); precision is NSLG_PREC_FP64 or NSLG_PREC_FP32 (the tensor-core forms need
 * workspaces), else NSLG_ERR_ARG; every factor matrix the operator reads must already be resident on the handle,
 * else NSLG_ERR_STATE: one nslg_fm_apply with the same op, the same species and this handle's discretisation has
 * run (M reads exp(sgn delta K), M^dagger exp(sgn delta* K), the two-factor operators both; switching species with
 * populate selects other entries, and HubbardDiag's factors are sgn delta K and sgn delta* K, which
 * nslg_fm_get_exp_hopping does not create). MM^dagger and M^dagger M keep their
 * intermediate vector in one fixed device array of the library, so for those nbatch * Nt * Nx may be at most
 * NSLG_NOALLOC_MAX_ELEMS (32 MiB of complex128, held on every device the library runs on), else NSLG_ERR_SHAPE. The
 * array is shared by all handles and streams: calls that overlap on the GPU (two streams, or two host threads on one
 * device) race on it, so order them. The first call on a device looks the array up (the CUDA runtime may load the
 * library's device code then): make it during setup. The address is kept per device ordinal for the life of the
 * process; after cudaDeviceReset on that device it is stale, so reset no device on which this call has run (the
 * library's handles do not survive a reset either). */
#define NSLG_NOALLOC_MAX_ELEMS 2097152
NSLG_API int nslg_fm_apply_noalloc(nslg_fm *fm, int op, const nslg_c128 *psi, nslg_c128 *out, int64_t nbatch,
                                   int precision);

/* ----- Hubbard actions and leapfrog --------------------------------------------------------------------------- */
/* Action terms (bit mask): the gauge term S = sum phi^2 / (2 U~) (src/NSL/Action/Implementations/
 * hubbardGaugeAction.tpp:55-67) and the fermion term S = -(log det M_P + log det M_H) (hubbardFermiAction.tpp:68-113),
 * U~ = delta U (hubbard.tpp:9-19). The fermion term uses fm (its species is switched to particle, then hole, as the
 * reference's HubbardFermionAction does with its hfm_). */
typedef enum { NSLG_TERM_GAUGE = 1, NSLG_TERM_FERMION = 2 } nslg_term;
/* Replaces Action<...>::eval / operator() (src/NSL/Action/action.tpp:103-139) for the selected terms. */
NSLG_API int nslg_hubbard_eval(nslg_fm *fm, const nslg_c128 *phi, nslg_c128 Utilde, int terms, nslg_c128 *S);
/* Replaces Action<...>::force (action.tpp:78-88): force (Nt, Nx); real_force zeroes Im (LeapfrogRealForce). */
NSLG_API int nslg_hubbard_force(nslg_fm *fm, const nslg_c128 *phi, nslg_c128 Utilde, int terms, int real_force,
                                nslg_c128 *force);
/* Replaces Leapfrog(action, trajLength, Nmd, backward)::operator()(q, p) (src/NSL/Integrator/Impl/leapfrog.tpp:18-58)
 * and, with real_force, LeapfrogRealForce (leapfrogRealForce.tpp:18-74): the whole trajectory runs on the device
 * (Nmd + 1 force evaluations, fused kick/drift kernels). q1/p1 may alias q0/p0. */
NSLG_API int nslg_leapfrog(nslg_fm *fm, const nslg_c128 *q0, const nslg_c128 *p0, nslg_c128 *q1, nslg_c128 *p1,
                           nslg_c128 Utilde, double traj_length, int64_t nmd, int backward, int real_force, int terms);
/* 1/2 sum p^2 (complex square), the kinetic term of H in HMC::generate_ (src/NSL/MarkovChain/HMC.tpp:204-215). */
NSLG_API int nslg_kinetic(nslg_fm *fm, const nslg_c128 *p, nslg_c128 *out);

/* Many independent configurations (chains) in one call; no counterpart in the reference, which runs one chain per
 * HMC object (src/NSL/MarkovChain/HMC.tpp). q, p are (nconf, Nt, Nx) (host or device); each configuration follows
 * the trajectory nslg_leapfrog would give it (to rounding: the order of the force's matrix products may differ), with
 * the particle and hole gradients of all configurations batched into the same launches (FP64 force whatever
 * nslg_fm_set_force_precision selected). 1 <= nconf <= 32767. */
NSLG_API int nslg_leapfrog_batch(nslg_fm *fm, int64_t nconf, const nslg_c128 *q0, const nslg_c128 *p0, nslg_c128 *q1,
                                 nslg_c128 *p1, nslg_c128 Utilde, double traj_length, int64_t nmd, int backward,
                                 int real_force, int terms);
/* Chains of different lattice shapes in one launch (no reference counterpart; per chain it is the
 * Leapfrog::integrate of leapfrog.tpp:35-58 that nslg_leapfrog replaces). Group g is the handle fms[g] (its own
 * lattice, Nt, beta, mu) with nconf[g] configurations q0[g], p0[g] of shape (nconf[g], Nt_g, Nx_g) and one coupling
 * U~ per configuration in Utilde[g][0..nconf[g]); results go to q1[g], p1[g]. Every handle belongs to the same
 * context and appears once; 1 <= ngroups <= 4096, 1 <= nconf[g] <= 32767. Each group advances exactly as
 * nslg_leapfrog_batch would with its couplings (nslg_leapfrog for nconf[g] = 1). The first two calls with a given
 * set of groups and parameters run the groups one after the other (eagerly, then while capturing each group's
 * trajectory); from the third on, every group's trajectory is a branch of one CUDA graph and the call is one graph
 * launch whose branches run concurrently. Returns once the results are written. */
NSLG_API int nslg_leapfrog_group(int ngroups, nslg_fm *const *fms, const int64_t *nconf,
                                 const nslg_c128 *const *q0, const nslg_c128 *const *p0, nslg_c128 *const *q1,
                                 nslg_c128 *const *p1, const nslg_c128 *const *Utilde, double traj_length,
                                 int64_t nmd, int backward, int real_force, int terms);
/* S[b] = the action of configuration b of phi (nconf, Nt, Nx), as nslg_hubbard_eval; S is a host array of nconf. */
NSLG_API int nslg_hubbard_eval_batch(nslg_fm *fm, int64_t nconf, const nslg_c128 *phi, nslg_c128 Utilde, int terms,
                                     nslg_c128 *S);
/* As nslg_hubbard_eval_batch with a coupling per configuration: Utilde is a host array of nconf values. */
NSLG_API int nslg_hubbard_eval_batch_u(nslg_fm *fm, int64_t nconf, const nslg_c128 *phi, const nslg_c128 *Utilde,
                                       int terms, nslg_c128 *S);
/* out[b] = 1/2 sum p_b^2 (complex square) for momenta p (nconf, Nt, Nx): nslg_kinetic for many chains, the kinetic
 * term of H in HMC::generate_ (HMC.tpp:204-215). out is a host array of nconf. */
NSLG_API int nslg_kinetic_batch(nslg_fm *fm, int64_t nconf, const nslg_c128 *p, nslg_c128 *out);
/* The Metropolis selection of many chains (HMC.tpp:223-226 per chain): q[b] = q_new[b] for every b whose accept[b]
 * (host array of nconf flags) is non-zero, q[b] unchanged otherwise; q and q_new are (nconf, Nt, Nx). The call
 * returns once the flags have been read. */
NSLG_API int nslg_accept_batch(nslg_fm *fm, int64_t nconf, const int32_t *accept, const nslg_c128 *q_new,
                               nslg_c128 *q);

/* ----- CG ---------------------------------------------------------------------------------------------------- */
/* Replaces CG<Type>(FermionMatrix&, MatrixCombination, eps, maxIter)::operator()(b[, x0])
 * (src/NSL/LinAlg/Solver/Impl/CG.hpp:142-186, CG.tpp:15-113). x0 may be NULL (then x0 = b, CG.tpp:98-103).
 * Vectors are FP64; precision selects the operator's arithmetic (FP32 = mixed precision). stop selects the rule
 * (nslg_cg_stop); with FP64 and NSLG_STOP_RECURRENCE the iteration is the reference's exactly. eps is absolute, in
 * the norm of the reference's rule. x may alias x0 but not b. stats may be NULL. */
NSLG_API int nslg_cg_solve(nslg_fm *fm, int op, const nslg_c128 *b, const nslg_c128 *x0, nslg_c128 *x,
                           int64_t nbatch, double eps, int64_t max_iter, int mode, int precision, int stop,
                           nslg_cg_stats *stats);
/* nslg_cg_solve with the stopping rule NSLG_STOP_TRUE_RESIDUAL_DD, returning the solution as the double-double pair
 * x + x_lo (x_lo may be NULL: then x alone, the pair rounded to FP64, whose own residual is only FP64-accurate).
 * The pair is what meets |b - A (x + x_lo)| <= eps below FP64's floor; x_lo must not overlap b, x0 or x. */
NSLG_API int nslg_cg_solve_dd(nslg_fm *fm, int op, const nslg_c128 *b, const nslg_c128 *x0, nslg_c128 *x,
                              nslg_c128 *x_lo, int64_t nbatch, double eps, int64_t max_iter, int mode, int precision,
                              nslg_cg_stats *stats);

/* Independent CG solves on several fermion matrices at once: instances of different Nx, Nt, beta and phi (and
 * species, discretisation) solved together, every right-hand side its own system, masked out as it converges. No
 * counterpart in the reference, which solves one CG per object (CG.tpp:15-113). Handle i (populated, all on one
 * context) has nbatch[i] >= 1 right-hand sides b[i] (nbatch[i], Nt_i, Nx_i), starting vectors x0[i] (x0 or x0[i] NULL:
 * x0 = b), solutions x[i] and, under NSLG_STOP_TRUE_RESIDUAL_DD, low parts x_lo[i] (x_lo or x_lo[i] may be NULL),
 * absolute tolerance eps[i]; stats (NULL or an array of nfm) receives each instance's statistics (iterations,
 * converged systems, true residual of its systems; the reliable-update and rebase counts are the group's). The
 * iteration's vector kernels run once for all instances and the operator once per instance, all captured in the same
 * CUDA graphs; buffers may be host or device memory. At most 65535 systems in all. */
NSLG_API int nslg_cg_solve_group(int nfm, nslg_fm *const *fms, int op, const nslg_c128 *const *b,
                                 const nslg_c128 *const *x0, nslg_c128 *const *x, nslg_c128 *const *x_lo,
                                 const int64_t *nbatch, const double *eps, int64_t max_iter, int precision, int stop,
                                 nslg_cg_stats *stats);

/* ----- two-body correlators ---------------------------------------------------------------------------------- */
/* Channels of the two-body correlator, in the order the reference computes them
 * (src/NSL/Measurements/Hubbard/twoBodyCorrelationFunction.tpp:290-303). */
typedef enum {
    NSLG_TB_I1S1IZ1SZ1 = 0, NSLG_TB_I1S1IZ1SZ0, NSLG_TB_I1S1IZ1SZN1, NSLG_TB_I1S1IZ0SZ1, NSLG_TB_I1S1IZ0SZN1,
    NSLG_TB_I1S1IZN1SZ1, NSLG_TB_I1S1IZN1SZ0, NSLG_TB_I1S1IZN1SZN1, NSLG_TB_I0S1IZ0SZ1, NSLG_TB_I0S1IZ0SZN1,
    NSLG_TB_I1S0IZ1SZ0, NSLG_TB_I1S0IZN1SZ0, NSLG_TB_NCHANNELS
} nslg_twobody_channel;

/* Replaces TwoBodyCorrelator<Type, LatticeType, FermionMatrixType>::measure(NumberTimeSources)
 * (twoBodyCorrelationFunction.tpp:188-306 and the channel functions :481-1001) on one configuration phi (Nt, Nx),
 * with fm built for the lattice, Nt, beta and mu of params. wall is params["wallSources"] (nk, nb, Nx). tuples
 * (ntuple, 4) lists the momentum keys (w, x, P, Q) to evaluate: the reference allocates every key with
 * k_w + k_x = k_P + k_Q modulo the reciprocal lattice (:196-226) and stores map[w][x][P][Q] under the HDF5 node
 * "w-x-P-Q". Source times are 0, s, 2s, ... < Nt with s = Nt / n_time_sources (1 <= n_time_sources <= Nt), each
 * contribution divided by n_time_sources. out is (NSLG_TB_NCHANNELS, ntuple, Nt, nb*nb, nb*nb): channel, tuple
 * and the reference tensor's entry [t, i*nb + j, l*nb + k]. The solves run as independent CGs per source vector
 * (MM^dagger, then M^dagger M on the conjugated sources) with the true-residual rule |b - A x| <= eps at
 * `precision`; NSLG_NOT_CONVERGED is returned with out filled when a system did not converge in max_iter (the
 * reference's CG logs and continues, CG.tpp:90-93). fm is left populated with phi and the hole species. phi, wall,
 * tuples and out may be host or device pointers; stats (may be NULL) aggregates the solves. */
NSLG_API int nslg_twobody_measure(nslg_fm *fm, const nslg_c128 *phi, const nslg_c128 *wall, int64_t nk, int64_t nb,
                                  const int64_t *tuples, int64_t ntuple, int64_t n_time_sources, double eps,
                                  int64_t max_iter, int precision, nslg_c128 *out, nslg_cg_stats *stats);

#ifdef __cplusplus
}
#endif

#endif /* NSL_GB300_H */
