// Stratified (UDT) log det M and d log det M / d phi for the exponential discretisation, in FP64.
//
// HubbardExp::logDetM and gradLogDetM (hubbardExp.tpp:129-211) multiply all Nt time-slice matrices into one product
// whose singular values spread over ~e^{2 beta |K|}; in FP64 that loses about log10(e^{beta |K|}) - 16 digits
// (the reference's log(det(.)) is NaN at beta >= 8; its gradient is off by 1e-7 at beta = 8 and has no correct digit
// at beta = 12 on the 24x24 lattice). Here the same quantities are evaluated from stratified products, the standard
// stabilisation of long chains of matrix multiplications:
//
//   Fk(t) = diag(phiExpInv[(t-1) mod Nt]) E',  E' = exp(-sgn delta K),  Fk(t)^{-1} = E diag(phiExp[(t-1) mod Nt]),
//   C(s)  = Fk(s) ... Fk(Nt-1) Fk(0) ... Fk(s-1),   G(s) = (1 + C(s))^{-1},
//   gradLogDetM[t] = i (1 - diag G(t+1))   (the reference's pi_dot by the push-through identity; G(t+1) = 1 - M^-1_tt),
//   logDetM = log det(1 + C(0)) + sum_t log det Fk(t)^{-1}   (principal branch of the imaginary part).
//
// The slices are grouped into J chunks of k consecutive factors (k chosen so that a chunk product's condition
// number stays below ~1e4). Two stacks hold, at every chunk boundary s_j, the suffix product
// L_j = Fk(s_j) ... Fk(Nt-1) = U_L D_L T_L and the adjoint of the prefix product R_j = Fk(0) ... Fk(s_j - 1),
// R_j^H = U_R D_R T_R, each as a unitary U, graded positive scales D (sorted descending) and a well-conditioned T.
// A stack step multiplies the next chunk product into U (Z = C U, condition number that of C), takes the QR
// factorisation Z = Q R by two Cholesky-QR passes (Gram matrix, unpivoted LU of the Hermitian positive definite Gram
// = Cholesky, forward substitution with the Cholesky factor: all batched GEMMs and the batched LU), and folds R into
// D and T:
// D' = diag(R) D, T' = D'^{-1} R D T, followed by a sort of D' (permuting U's columns and T's rows).
// At a boundary, with D = D_b D_s split into the parts above and below 1,
//   1 + L R = U_L D_Lb X D_Rb U_R^H,   X = D_Lb^{-1} (U_L^H U_R) D_Rb^{-1} + D_Ls (T_L T_R^H) D_Rs,
// and X is well conditioned, so G(s_j) = U_R D_Rb^{-1} X^{-1} D_Lb^{-1} U_L^H (pivoted LU of X) never adds O(e^{beta|K|})
// to O(1) numbers. Inside a chunk G is carried from both neighbouring boundaries by the similarity
// G(s+1) = Fk(s)^{-1} G(s) Fk(s) (forward) and G(s) = Fk(s) G(s+1) Fk(s)^{-1} (backward), at most k/2 steps each,
// which amplifies the boundary error by at most the square root of a chunk's condition number.
// Both stacks, all boundaries and all wraps are batched over the matrices of a call (both species of a force).

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <string>
#include <vector>

#include "fm_internal.cuh"

namespace nslg {

namespace {

constexpr int TR = 32;  // transpose tile
constexpr int EW = 256; // threads of the element-wise kernels

// Matrix z of a two-level batch sits at base + (z / per) * outer + (z % per) * inner (elements).
struct Bat {
    int per = 1;
    int64_t outer = 0, inner = 0;
    __host__ __device__ int64_t off(int64_t z) const { return (z / per) * outer + (z % per) * inner; }
};
Bat flat(int64_t stride) {
    Bat b;
    b.per = 1;
    b.outer = stride;
    return b;
}
Bat two(int per, int64_t outer, int64_t inner) {
    Bat b;
    b.per = per;
    b.outer = outer;
    b.inner = inner;
    return b;
}

// out[z] = A[z]^H for the n x n matrices of a batch (blockIdx.z), through a shared-memory tile.
__global__ void k_ctrans(const double2 *__restrict__ A, Bat ba, double2 *__restrict__ out, Bat bo, int n) {
    __shared__ double2 tile[TR][TR + 1];
    A += ba.off(blockIdx.z);
    out += bo.off(blockIdx.z);
    const int c0 = blockIdx.x * TR, r0 = blockIdx.y * TR;
    for (int yy = threadIdx.y; yy < TR; yy += blockDim.y) {
        const int r = r0 + yy, c = c0 + threadIdx.x;
        if (r < n && c < n) tile[yy][threadIdx.x] = A[(int64_t)r * n + c];
    }
    __syncthreads();
    for (int yy = threadIdx.y; yy < TR; yy += blockDim.y) {
        const int r = c0 + yy, c = r0 + threadIdx.x;  // out[r][c] = conj(A[c][r])
        if (r < n && c < n) {
            const double2 v = tile[threadIdx.x][yy];
            out[(int64_t)r * n + c] = make_double2(v.x, -v.y);
        }
    }
}

// Identity matrices / unit scales for the first stack entries.
__global__ void k_eye(double2 *A, Bat b, int n, int nmat) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nn = (int64_t)n * n;
    if (idx >= nn * nmat) return;
    const int64_t z = idx / nn, e = idx % nn;
    A[b.off(z) + e] = make_double2((e / n) == (e % n) ? 1.0 : 0.0, 0.0);
}
__global__ void k_ones(double *d, Bat b, int n, int nmat) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)n * nmat) return;
    d[b.off(idx / n) + idx % n] = 1.0;
}

// After the unpivoted LU of a Hermitian positive definite Gram matrix G = L U (U = D L^H, D = diag(U) > 0), the
// Cholesky factor R = D^{-1/2} U (upper triangle, real diagonal sqrt(D)). Q^H = R^{-H} Z^H is then solved with R
// itself, not with the LU's L: L and U carry independent rounding, and pairing one with the other loses
// ~cond(Z)^2 eps in Q R = Z. R^H = L'' diag(R) with the unit lower L''_ij = conj(R_ji) / R_jj, written into the LU
// matrix's strictly lower part (k_chol_lower) so that the batched unit-lower forward substitution applies, and the
// rows are divided by R_ii afterwards (k_rows_div_rdiag).
__global__ void k_chol_r(const double2 *__restrict__ LU, double2 *__restrict__ R, int n, int nmat) {
    const int64_t nn = (int64_t)n * n;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nn * nmat) return;
    const int64_t z = idx / nn, e = idx % nn;
    const int i = (int)(e / n), j = (int)(e % n);
    const double dii = LU[z * nn + (int64_t)i * n + i].x;
    const double s = dii > 0.0 ? 1.0 / sqrt(dii) : 0.0;
    if (j > i) {
        const double2 u = LU[idx];
        R[idx] = make_double2(u.x * s, u.y * s);
    } else {
        R[idx] = make_double2(j == i ? sqrt(fmax(dii, 0.0)) : 0.0, 0.0);
    }
}
__global__ void k_chol_lower(const double2 *__restrict__ R, double2 *__restrict__ LU, int n, int nmat) {
    const int64_t nn = (int64_t)n * n;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nn * nmat) return;
    const int64_t z = idx / nn, e = idx % nn;
    const int i = (int)(e / n), j = (int)(e % n);
    if (i <= j) return;
    const double rjj = R[z * nn + (int64_t)j * n + j].x;
    const double2 rji = R[z * nn + (int64_t)j * n + i];
    LU[idx] = rjj > 0.0 ? make_double2(rji.x / rjj, -rji.y / rjj) : make_double2(0.0, 0.0);
}
__global__ void k_rows_div_rdiag(double2 *__restrict__ Y, const double2 *__restrict__ R, int n, int nmat) {
    const int64_t nn = (int64_t)n * n;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nn * nmat) return;
    const int64_t z = idx / nn, e = idx % nn;
    const int i = (int)(e / n);
    const double rii = R[z * nn + (int64_t)i * n + i].x;
    const double s = rii > 0.0 ? 1.0 / rii : 0.0;
    Y[idx] = make_double2(Y[idx].x * s, Y[idx].y * s);
}

// UDT step, scales: dn[z][i] = R[z]_ii * d[z][i] (R_ii real positive), then R[z]_ij *= d_j / dn_i.
__global__ void k_udt_scales(const double2 *__restrict__ R, const double *__restrict__ d, Bat bd,
                             double *__restrict__ dn, int n, int nmat) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)n * nmat) return;
    const int64_t z = idx / n;
    const int i = (int)(idx % n);
    dn[idx] = R[z * n * n + (int64_t)i * n + i].x * d[bd.off(z) + i];
}
__global__ void k_udt_scale_r(double2 *__restrict__ R, const double *__restrict__ d, Bat bd,
                              const double *__restrict__ dn, int n, int nmat) {
    const int64_t nn = (int64_t)n * n;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nn * nmat) return;
    const int64_t z = idx / nn, e = idx % nn;
    const int i = (int)(e / n), j = (int)(e % n);
    if (j < i) return;  // lower triangle is zero
    const double f = d[bd.off(z) + j] / dn[z * n + i];
    const double2 r = R[idx];
    R[idx] = make_double2(r.x * f, r.y * f);
}

// rank[z][i] = position of dn[z][i] in descending order (ties: lower index first).
__global__ void k_rank_desc(const double *__restrict__ dn, int *__restrict__ rank, int n, int nmat) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)n * nmat) return;
    const int64_t z = idx / n;
    const int i = (int)(idx % n);
    const double *v = dn + z * n;
    const double di = v[i];
    int r = 0;
    for (int j = 0; j < n; ++j) {
        const double dj = v[j];
        r += (dj > di) || (dj == di && j < i);
    }
    rank[idx] = r;
}

// U[z][:, rank_j] = Q[z][:, j], T[z][rank_i, :] = Tn[z][i, :], d[z][rank_i] = dn[z][i].
__global__ void k_udt_permute(const double2 *__restrict__ Q, const double2 *__restrict__ Tn,
                              const double *__restrict__ dn, const int *__restrict__ rank, double2 *__restrict__ U,
                              double2 *__restrict__ T, Bat bm, double *__restrict__ d, Bat bd, int n, int nmat) {
    const int64_t nn = (int64_t)n * n;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nn * nmat) return;
    const int64_t z = idx / nn, e = idx % nn;
    const int i = (int)(e / n), j = (int)(e % n);
    const int *rk = rank + z * n;
    const int64_t o = bm.off(z);
    U[o + (int64_t)i * n + rk[j]] = Q[idx];
    T[o + (int64_t)rk[i] * n + j] = Tn[idx];
    if (j == 0) d[bd.off(z) + rk[i]] = dn[z * n + i];
}

// Chunk products: C[g, j] starts as Fk(s_j) = diag(pinv[g][(s_j - 1) mod Nt]) E'[g] (step < 0), or is column-scaled
// by phase row (s_j + step - 1) mod Nt before the next product with E' (C <- C Fk(s_j + step)).
__device__ __forceinline__ int chunk_start(int j, int q, int r) { return j * q + min(j, r); }

__global__ void k_chunk_scale(double2 *__restrict__ C, const double2 *__restrict__ Ep, const double2 *__restrict__ pinv,
                              int n, int Nt, int J, int q, int r, int nmat, int step) {
    const int64_t nn = (int64_t)n * n;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nn * J * nmat) return;
    const int64_t z = idx / nn, e = idx % nn;
    const int g = (int)(z / J), j = (int)(z % J);
    const int i = (int)(e / n), c = (int)(e % n);
    if (step >= q + (j < r ? 1 : 0)) return;  // this chunk has no factor `step`
    const int s = chunk_start(j, q, r) + max(step, 0);
    const double2 *ph = pinv + ((int64_t)g * Nt + ((s - 1) % Nt + Nt) % Nt) * n;
    if (step < 0) C[idx] = cmul(ph[i], Ep[(int64_t)g * nn + e]);
    else C[idx] = cmul(C[idx], ph[c]);
}

// Boundary matrix X[z] = D_Lb^{-1} M1 D_Rb^{-1} + D_Ls M2 D_Rs and right-hand side W[z] = D_Lb^{-1} U_L^H.
__global__ void k_boundary_x(const double2 *__restrict__ M1, const double2 *__restrict__ M2, Bat b2,
                             const double *__restrict__ dL, Bat bl, const double *__restrict__ dR, Bat br,
                             const double2 *__restrict__ ULH, double2 *__restrict__ X, double2 *__restrict__ W, int n,
                             int nmat) {
    const int64_t nn = (int64_t)n * n;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nn * nmat) return;
    const int64_t z = idx / nn, e = idx % nn;
    const int i = (int)(e / n), k = (int)(e % n);
    const double li = dL[bl.off(z) + i], rk = dR[br.off(z) + k];
    const double lb = fmax(li, 1.0), ls = fmin(li, 1.0), rb = fmax(rk, 1.0), rs = fmin(rk, 1.0);
    const double2 a = M1[idx], b = M2[b2.off(z) + e];
    const double fa = 1.0 / (lb * rb), fb = ls * rs;
    X[idx] = make_double2(a.x * fa + b.x * fb, a.y * fa + b.y * fb);
    if (W) {
        const double2 u = ULH[idx];
        W[idx] = make_double2(u.x / lb, u.y / lb);
    }
}

// Y[z] rows divided by D_Rb.
__global__ void k_rows_div_big(double2 *__restrict__ Y, const double *__restrict__ dR, Bat bd, int n, int nmat) {
    const int64_t nn = (int64_t)n * n;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nn * nmat) return;
    const int64_t z = idx / nn, e = idx % nn;
    const int i = (int)(e / n);
    const double f = 1.0 / fmax(dR[bd.off(z) + i], 1.0);
    Y[idx] = make_double2(Y[idx].x * f, Y[idx].y * f);
}

// Wrap scaling of G[g, j] at slice s = s_j + ofs (forward) or s_{j+1} - ofs (backward):
// forward   G_ik *= ph[s-1]_i pinv[s-1]_k      (before E G E')
// backward  G_ik *= pinv[s-1]_i ph[s-1]_k      (after E' G E)
__global__ void k_wrap_scale(double2 *__restrict__ G, const double2 *__restrict__ ph, const double2 *__restrict__ pinv,
                             int n, int Nt, int J, int q, int r, int nmat, int ofs, bool forward) {
    const int64_t nn = (int64_t)n * n;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nn * J * nmat) return;
    const int64_t z = idx / nn, e = idx % nn;
    const int g = (int)(z / J), j = (int)(z % J);
    const int i = (int)(e / n), k = (int)(e % n);
    const int s = forward ? chunk_start(j, q, r) + ofs : chunk_start(j + 1, q, r) - ofs;
    const int64_t row = ((int64_t)g * Nt + ((s - 1) % Nt + Nt) % Nt) * n;
    const double2 *a = forward ? ph + row : pinv + row;
    const double2 *b = forward ? pinv + row : ph + row;
    G[idx] = cmul(cmul(a[i], G[idx]), b[k]);
}

// out[g, t] = i (1 - diag G[g, j]) with t = (s - 1) mod Nt, s = s_j + ofs (forward) / s_{j+1} - ofs (backward), for
// the chunks where the step exists: ofs <= (len_j - 1) / 2 forward, ofs <= len_j - 1 - (len_j - 1) / 2 backward;
// ofs = 0 (forward) writes the boundary rows.
__global__ void k_grad_rows(const double2 *__restrict__ G, double2 *__restrict__ out, int n, int Nt, int J, int q,
                            int r, int nmat, int ofs, bool forward) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)n * J * nmat) return;
    const int64_t z = idx / n;
    const int x = (int)(idx % n);
    const int g = (int)(z / J), j = (int)(z % J);
    const int len = chunk_start(j + 1, q, r) - chunk_start(j, q, r);
    const int f = (len - 1) / 2, b = len - 1 - f;
    if (forward ? ofs > f : (ofs < 1 || ofs > b)) return;
    const int s = forward ? chunk_start(j, q, r) + ofs : chunk_start(j + 1, q, r) - ofs;
    const int t = ((s - 1) % Nt + Nt) % Nt;
    const double2 v = G[z * n * n + (int64_t)x * n + x];
    out[((int64_t)g * Nt + t) * n + x] = make_double2(v.y, 1.0 - v.x);  // i (1 - v)
}

// sum over z of log(max(d, 1)) (the big scales of the suffix stack at s = 0), per matrix; and the log of the phase
// rows sum_{t,x} Log(phiExp) (principal logs), one block per matrix.
__global__ void k_logdet_terms(const double *__restrict__ dL, Bat bd, const double2 *__restrict__ ph, int n, int Nt,
                               double2 *__restrict__ out) {
    __shared__ double2 red[256];
    const int g = blockIdx.x;
    double2 acc = make_double2(0, 0);
    for (int i = threadIdx.x; i < n; i += 256) acc.x += log(fmax(dL[bd.off(g) + i], 1.0));
    const double2 *p = ph + (int64_t)g * Nt * n;
    for (int64_t e = threadIdx.x; e < (int64_t)Nt * n; e += 256) {
        const double2 v = p[e];
        acc.x += log(hypot(v.x, v.y));
        acc.y += atan2(v.y, v.x);
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
    if (threadIdx.x == 0) out[g] = red[0];
}

inline unsigned blocks(int64_t n) { return (unsigned)ceil_div(n, EW); }

int ctrans(cudaStream_t st, const double2 *A, Bat ba, double2 *out, Bat bo, int n, int nmat) {
    const dim3 grid((unsigned)ceil_div(n, TR), (unsigned)ceil_div(n, TR), (unsigned)nmat);
    k_ctrans<<<grid, dim3(TR, 8), 0, st>>>(A, ba, out, bo, n);
    note_launch(st);
    return NSLG_OK;
}

// Workspace of one stratified evaluation (names are handle workspaces).
struct Strat {
    int n = 0, Nt = 0, nmat = 0, k = 1, J = 1, q = 1, r = 0;
    bool real = false;                          // every E' and E real: their products skip the imaginary parts
    double2 *Ep = nullptr, *E = nullptr;        // E' = exp(-sgn delta K), E = exp(sgn delta K) per matrix
    double2 *C = nullptr, *CH = nullptr;        // chunk products and their adjoints (nmat, J, n, n)
    double2 *SU = nullptr, *ST = nullptr;       // suffix stack (nmat, J + 1, n, n)
    double2 *PU = nullptr, *PT = nullptr;       // prefix stack (adjoint) (nmat, J + 1, n, n)
    double *Sd = nullptr, *Pd = nullptr;        // (nmat, J + 1, n)
    double2 *Z, *Q, *R, *ZH, *Gm, *Y, *YH, *R1, *R2, *Tn;  // QR work (2 nmat, n, n)
    double *dn = nullptr;
    int *rank = nullptr;
};

// Number of factors per chunk. A chunk product of k slices has a condition number of at most exp(2 k |delta| rho)
// (rho >= the spectral radius of K: its max column sum), and the wraps inside a chunk multiply the boundary's error
// by up to exp(|delta| rho k / 2). k keeps that factor at 3: measured against the oracle's stratified forms, the
// gradient's error grows with k as 4e-13 (k = 4), 5e-13 (6), 1.7e-12 (8), 4.4e-12 (12) at honeycomb 12x12, Nt = 64,
// beta = 8 and 1.7e-12 (6), 4.4e-12 (8), 2.7e-11 (16) at 24x24, Nt = 128, beta = 12.
int chunk_len(const nslg_fm *fm) {
    if (const char *e = std::getenv("NSLG_STRAT_CHUNK")) {  // tuning and accuracy studies
        const int k = std::atoi(e);
        if (k >= 1) return std::min<int>(k, (int)fm->Nt);
    }
    const double a = std::fabs(fm->delta.x) * std::max(fm->hops_norm1, 1e-300);
    const int k = a > 0 ? (int)std::floor(2.0 * std::log(3.0) / a) : (int)fm->Nt;
    return std::max(1, std::min<int>(k, (int)fm->Nt));
}

int strat_setup(nslg_fm *fm, int nmat, const ExpEntry *const *Ep, const ExpEntry *const *E, bool need_prefix,
                Strat &S) {
    cudaStream_t st = fm->ctx->stream;
    S.n = (int)fm->Nx;
    S.Nt = (int)fm->Nt;
    S.nmat = nmat;
    S.k = chunk_len(fm);
    S.J = (int)ceil_div(S.Nt, S.k);
    S.q = S.Nt / S.J;
    S.r = S.Nt % S.J;
    const int64_t nn = (int64_t)S.n * S.n;
    const int64_t J = S.J;
    NSLG_TRY(ws_get(fm, "st_Ep", (size_t)nmat * nn, &S.Ep));
    NSLG_TRY(ws_get(fm, "st_E", (size_t)nmat * nn, &S.E));
    S.real = true;
    for (int g = 0; g < nmat; ++g) {
        S.real = S.real && Ep[g]->is_real && E[g]->is_real;
        NSLG_CUDA(cudaMemcpyAsync(S.Ep + g * nn, Ep[g]->full, nn * sizeof(double2), cudaMemcpyDeviceToDevice, st));
        NSLG_CUDA(cudaMemcpyAsync(S.E + g * nn, E[g]->full, nn * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    }
    NSLG_TRY(ws_get(fm, "st_C", (size_t)nmat * J * nn, &S.C));
    NSLG_TRY(ws_get(fm, "st_SU", (size_t)nmat * (J + 1) * nn, &S.SU));
    NSLG_TRY(ws_get(fm, "st_ST", (size_t)nmat * (J + 1) * nn, &S.ST));
    NSLG_TRY(ws_get(fm, "st_Sd", (size_t)nmat * (J + 1) * S.n, &S.Sd));
    const int side = need_prefix ? 2 : 1;
    if (need_prefix) {
        NSLG_TRY(ws_get(fm, "st_CH", (size_t)nmat * J * nn, &S.CH));
        NSLG_TRY(ws_get(fm, "st_PU", (size_t)nmat * (J + 1) * nn, &S.PU));
        NSLG_TRY(ws_get(fm, "st_PT", (size_t)nmat * (J + 1) * nn, &S.PT));
        NSLG_TRY(ws_get(fm, "st_Pd", (size_t)nmat * (J + 1) * S.n, &S.Pd));
    }
    const size_t qn = (size_t)side * nmat * nn;
    NSLG_TRY(ws_get(fm, "st_Z", qn, &S.Z));
    NSLG_TRY(ws_get(fm, "st_Q", qn, &S.Q));
    NSLG_TRY(ws_get(fm, "st_R", qn, &S.R));
    NSLG_TRY(ws_get(fm, "st_ZH", qn, &S.ZH));
    NSLG_TRY(ws_get(fm, "st_Gm", qn, &S.Gm));
    NSLG_TRY(ws_get(fm, "st_Y", qn, &S.Y));
    NSLG_TRY(ws_get(fm, "st_YH", qn, &S.YH));
    NSLG_TRY(ws_get(fm, "st_R1", qn, &S.R1));
    NSLG_TRY(ws_get(fm, "st_R2", qn, &S.R2));
    NSLG_TRY(ws_get(fm, "st_Tn", qn, &S.Tn));
    NSLG_TRY(ws_get(fm, "st_dn", (size_t)side * nmat * S.n, &S.dn));
    NSLG_TRY(ws_get(fm, "st_rank", (size_t)side * nmat * S.n, &S.rank));
    return NSLG_OK;
}

// Chunk products C[g, j] = Fk(s_j) ... Fk(s_{j+1} - 1) for every matrix and chunk (and their adjoints).
int strat_chunks(nslg_fm *fm, Strat &S, const double2 *pinv) {
    cudaStream_t st = fm->ctx->stream;
    const int n = S.n, J = S.J;
    const int64_t nn = (int64_t)n * n, tot = nn * J * S.nmat;
    const double2 one = make_double2(1, 0);
    double2 *buf;
    NSLG_TRY(ws_get(fm, "st_Cbuf", (size_t)tot, &buf));
    k_chunk_scale<<<blocks(tot), EW, 0, st>>>(S.C, S.Ep, pinv, n, S.Nt, J, S.q, S.r, S.nmat, -1);
    note_launch(st);
    const int maxlen = S.q + (S.r > 0 ? 1 : 0);
    for (int m = 1; m < maxlen; ++m) {
        // C <- (C diag(pinv[s_j + m - 1])) E' for the chunks longer than m (all of them while m < q, the first r
        // chunks of every matrix at m = q)
        k_chunk_scale<<<blocks(tot), EW, 0, st>>>(S.C, S.Ep, pinv, n, S.Nt, J, S.q, S.r, S.nmat, m);
        note_launch(st);
        const int nch = m < S.q ? J : S.r;
        NSLG_TRY(zgemm2(st, n, n, n, one, S.C, n, (int64_t)J * nn, nn, S.Ep, n, nn, 0, buf, n, (int64_t)J * nn, nn,
                        S.nmat, nch, S.real ? 2 : 0));
        NSLG_CUDA(cudaMemcpy2DAsync(S.C, (size_t)J * nn * sizeof(double2), buf, (size_t)J * nn * sizeof(double2),
                                    (size_t)nch * nn * sizeof(double2), S.nmat, cudaMemcpyDeviceToDevice, st));
    }
    if (S.CH) NSLG_TRY(ctrans(st, S.C, flat(nn), S.CH, flat(nn), n, S.nmat * J));
    NSLG_CUDA(cudaGetLastError());
    return NSLG_OK;
}

// Z (cnt matrices, contiguous) = Q R by two Cholesky-QR passes.
int cholqr2(nslg_fm *fm, Strat &S, int cnt) {
    cudaStream_t st = fm->ctx->stream;
    const int n = S.n;
    const int64_t nn = (int64_t)n * n, tot = nn * cnt;
    const double2 one = make_double2(1, 0);
    LuScratch ls;
    NSLG_TRY(get_lu_scratch(fm, n, ls, cnt, "st_chol"));
    // pass 1: G = Z^H Z = L U, R1 = D^{-1/2} U, Y = R1^{-H} Z^H = Q1^H
    NSLG_TRY(ctrans(st, S.Z, flat(nn), S.ZH, flat(nn), n, cnt));
    NSLG_TRY(zgemm(st, n, n, n, one, S.ZH, n, nn, S.Z, n, nn, S.Gm, n, nn, cnt, false));
    NSLG_TRY(lu_factor(fm, S.Gm, n, ls, cnt, nn, false, false));
    k_chol_r<<<blocks(tot), EW, 0, st>>>(S.Gm, S.R1, n, cnt);
    k_chol_lower<<<blocks(tot), EW, 0, st>>>(S.R1, S.Gm, n, cnt);
    note_launch(st, 2);
    NSLG_CUDA(cudaMemcpyAsync(S.Y, S.ZH, tot * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    NSLG_TRY(lu_forward(fm, S.Gm, S.Y, n, cnt, nn, nn));
    k_rows_div_rdiag<<<blocks(tot), EW, 0, st>>>(S.Y, S.R1, n, cnt);
    note_launch(st);
    // pass 2 on Q1: G = Q1^H Q1 = Y Y^H
    NSLG_TRY(ctrans(st, S.Y, flat(nn), S.YH, flat(nn), n, cnt));
    NSLG_TRY(zgemm(st, n, n, n, one, S.Y, n, nn, S.YH, n, nn, S.Gm, n, nn, cnt, false));
    NSLG_TRY(lu_factor(fm, S.Gm, n, ls, cnt, nn, false, false));
    k_chol_r<<<blocks(tot), EW, 0, st>>>(S.Gm, S.R2, n, cnt);
    k_chol_lower<<<blocks(tot), EW, 0, st>>>(S.R2, S.Gm, n, cnt);
    note_launch(st, 2);
    NSLG_TRY(lu_forward(fm, S.Gm, S.Y, n, cnt, nn, nn));
    k_rows_div_rdiag<<<blocks(tot), EW, 0, st>>>(S.Y, S.R2, n, cnt);
    note_launch(st);
    NSLG_TRY(zgemm(st, n, n, n, one, S.R2, n, nn, S.R1, n, nn, S.R, n, nn, cnt, false));
    NSLG_TRY(ctrans(st, S.Y, flat(nn), S.Q, flat(nn), n, cnt));
    NSLG_CUDA(cudaGetLastError());
    return NSLG_OK;
}

// Folds (Q, R) of matrices [z0, z0 + nmat) of the QR work into the stack entry (Uo, To, do) from the previous entry
// (d_prev, T_prev): D' = diag(R) D, T' = D'^{-1} R D T, sorted by D'.
int udt_fold(nslg_fm *fm, Strat &S, int z0, const double *d_prev, const double2 *T_prev, double2 *Uo, double2 *To,
             double *d_out, int64_t mstride, int64_t dstride) {
    cudaStream_t st = fm->ctx->stream;
    const int n = S.n, nmat = S.nmat;
    const int64_t nn = (int64_t)n * n;
    const double2 one = make_double2(1, 0);
    double2 *R = S.R + z0 * nn, *Q = S.Q + z0 * nn, *Tn = S.Tn + z0 * nn;
    double *dn = S.dn + (int64_t)z0 * n;
    int *rank = S.rank + (int64_t)z0 * n;
    k_udt_scales<<<blocks((int64_t)n * nmat), EW, 0, st>>>(R, d_prev, flat(dstride), dn, n, nmat);
    note_launch(st);
    k_udt_scale_r<<<blocks(nn * nmat), EW, 0, st>>>(R, d_prev, flat(dstride), dn, n, nmat);
    note_launch(st);
    NSLG_TRY(zgemm(st, n, n, n, one, R, n, nn, T_prev, n, mstride, Tn, n, nn, nmat, false));
    k_rank_desc<<<blocks((int64_t)n * nmat), EW, 0, st>>>(dn, rank, n, nmat);
    note_launch(st);
    k_udt_permute<<<blocks(nn * nmat), EW, 0, st>>>(Q, Tn, dn, rank, Uo, To, flat(mstride), d_out, flat(dstride), n,
                                                    nmat);
    note_launch(st);
    NSLG_CUDA(cudaGetLastError());
    return NSLG_OK;
}

// Both stacks (the prefix one only when S.PU is set), one batched step per chunk.
int strat_stacks(nslg_fm *fm, Strat &S) {
    cudaStream_t st = fm->ctx->stream;
    const int n = S.n, J = S.J, nmat = S.nmat;
    const int64_t nn = (int64_t)n * n, ms = (int64_t)(J + 1) * nn, ds = (int64_t)(J + 1) * n;
    const double2 one = make_double2(1, 0);
    const bool prefix = S.PU != nullptr;
    // identities: suffix entry J, prefix entry 0
    k_eye<<<blocks(nn * nmat), EW, 0, st>>>(S.SU + J * nn, flat(ms), n, nmat);
    k_eye<<<blocks(nn * nmat), EW, 0, st>>>(S.ST + J * nn, flat(ms), n, nmat);
    k_ones<<<blocks((int64_t)n * nmat), EW, 0, st>>>(S.Sd + (int64_t)J * n, flat(ds), n, nmat);
    note_launch(st, 3);
    if (prefix) {
        k_eye<<<blocks(nn * nmat), EW, 0, st>>>(S.PU, flat(ms), n, nmat);
        k_eye<<<blocks(nn * nmat), EW, 0, st>>>(S.PT, flat(ms), n, nmat);
        k_ones<<<blocks((int64_t)n * nmat), EW, 0, st>>>(S.Pd, flat(ds), n, nmat);
        note_launch(st, 3);
    }
    for (int i = 0; i < J; ++i) {
        const int js = J - 1 - i;  // suffix: L_js = C_js L_{js+1}
        NSLG_TRY(zgemm(st, n, n, n, one, S.C + js * nn, n, (int64_t)J * nn, S.SU + (js + 1) * nn, n, ms, S.Z, n, nn,
                       nmat, false));
        if (prefix)  // prefix (adjoint): R_{i+1}^H = C_i^H R_i^H
            NSLG_TRY(zgemm(st, n, n, n, one, S.CH + i * nn, n, (int64_t)J * nn, S.PU + i * nn, n, ms,
                           S.Z + nmat * nn, n, nn, nmat, false));
        NSLG_TRY(cholqr2(fm, S, prefix ? 2 * nmat : nmat));
        NSLG_TRY(udt_fold(fm, S, 0, S.Sd + (int64_t)(js + 1) * n, S.ST + (js + 1) * nn, S.SU + js * nn,
                          S.ST + js * nn, S.Sd + (int64_t)js * n, ms, ds));
        if (prefix)
            NSLG_TRY(udt_fold(fm, S, nmat, S.Pd + (int64_t)i * n, S.PT + i * nn, S.PU + (i + 1) * nn,
                              S.PT + (i + 1) * nn, S.Pd + (int64_t)(i + 1) * n, ms, ds));
    }
    return NSLG_OK;
}

}  // namespace

// True when the stratified forms are used for this handle: the exponential discretisation with a product whose
// dynamic range exp(beta rho) exceeds e^14 (beyond it the direct product loses digits below 1e-12; measured against
// dense inverses of M), unless nslg_fm_set_stabilisation forced one form.
bool use_stratified(const nslg_fm *fm) {
    if (fm->kind != NSLG_FM_EXP) return false;
    if (fm->stabilisation == NSLG_STAB_PLAIN) return false;
    if (fm->stabilisation == NSLG_STAB_STRATIFIED) return true;
    const double beta_rho = std::fabs(fm->delta.x) * (double)fm->Nt * fm->hops_norm1;
    return beta_rho > 14.0;
}

// The gradient (the HMC force) follows use_stratified, except that the split-BF16 force setting
// (nslg_fm_set_force_precision(NSLG_PREC_BF16_SPLIT): a fast force whose error is stated, not the FP64 one) keeps the
// direct product under AUTO while beta rho <= 28: there the split-BF16 direct-product gradient is within ~2e-7 of the
// stratified FP64 one (honeycomb 12x12, Nt = 64, beta = 8: beta rho = 24), while at beta rho = 36 (honeycomb 24x24,
// Nt = 128, beta = 12) the direct product has no correct digit. Log det (Delta H, the Metropolis step) always
// follows use_stratified.
bool use_stratified_grad(const nslg_fm *fm) {
    if (!use_stratified(fm)) return false;
    const double beta_rho = std::fabs(fm->delta.x) * (double)fm->Nt * fm->hops_norm1;
    return !(fm->force_precision == NSLG_PREC_BF16_SPLIT && fm->stabilisation == NSLG_STAB_AUTO && beta_rho <= 28.0);
}

// d log det M / d phi for nmat matrices (matrix g: factors E'[g] = exp(-sgn_g delta K) and E[g] = exp(sgn_g delta K),
// phase rows ph[g] = phiExp and pinv[g] = phiExpInv (Nt, Nx)); out (nmat, Nt, Nx) on the device.
int grad_logdet_strat(nslg_fm *fm, int nmat, const ExpEntry *const *Ep, const ExpEntry *const *E, const double2 *ph,
                      const double2 *pinv, double2 *out) {
    cudaStream_t st = fm->ctx->stream;
    Strat S;
    NSLG_TRY(strat_setup(fm, nmat, Ep, E, true, S));
    NSLG_TRY(strat_chunks(fm, S, pinv));
    NSLG_TRY(strat_stacks(fm, S));
    const int n = S.n, J = S.J, Nt = S.Nt;
    const int64_t nn = (int64_t)n * n, ms = (int64_t)(J + 1) * nn, ds = (int64_t)(J + 1) * n;
    const int64_t nb = (int64_t)nmat * J, tot = nb * nn;
    const double2 one = make_double2(1, 0);
    // boundary Green functions G(s_j) for every matrix and chunk
    double2 *ULH, *THH, *M1, *M2, *X, *W, *Xi, *G0, *Gf, *Gb, *Wt;
    NSLG_TRY(ws_get(fm, "stb_ULH", (size_t)tot, &ULH));
    NSLG_TRY(ws_get(fm, "stb_THH", (size_t)tot, &THH));
    NSLG_TRY(ws_get(fm, "stb_M1", (size_t)tot, &M1));
    NSLG_TRY(ws_get(fm, "stb_M2", (size_t)tot, &M2));
    NSLG_TRY(ws_get(fm, "stb_X", (size_t)tot, &X));
    NSLG_TRY(ws_get(fm, "stb_W", (size_t)tot, &W));
    NSLG_TRY(ws_get(fm, "stb_Xi", (size_t)tot, &Xi));
    NSLG_TRY(ws_get(fm, "stb_G0", (size_t)tot, &G0));
    NSLG_TRY(ws_get(fm, "stb_Gf", (size_t)tot, &Gf));
    NSLG_TRY(ws_get(fm, "stb_Gb", (size_t)tot, &Gb));
    NSLG_TRY(ws_get(fm, "stb_Wt", (size_t)tot, &Wt));
    const Bat stack = two(J, ms, nn), dstack = two(J, ds, n);
    NSLG_TRY(ctrans(st, S.SU, stack, ULH, flat(nn), n, (int)nb));
    NSLG_TRY(ctrans(st, S.PT, stack, THH, flat(nn), n, (int)nb));
    // M1 = U_L^H U_R, M2 = T_L T_R^H
    NSLG_TRY(zgemm2(st, n, n, n, one, ULH, n, (int64_t)J * nn, nn, S.PU, n, ms, nn, M1, n, (int64_t)J * nn, nn, nmat,
                    J));
    NSLG_TRY(zgemm2(st, n, n, n, one, S.ST, n, ms, nn, THH, n, (int64_t)J * nn, nn, M2, n, (int64_t)J * nn, nn, nmat,
                    J));
    k_boundary_x<<<blocks(tot), EW, 0, st>>>(M1, M2, flat(nn), S.Sd, dstack, S.Pd, dstack, ULH, X, W, n, (int)nb);
    note_launch(st);
    LuScratch ls;
    NSLG_TRY(get_lu_scratch(fm, n, ls, (int)nb, "st_x"));
    if (!fm->defer_checks) NSLG_CUDA(cudaMemsetAsync(ls.singular, 0, sizeof(int), st));
    NSLG_TRY(lu_factor(fm, X, n, ls, (int)nb, nn, false, true));
    NSLG_TRY(lu_inverse(fm, X, Xi, n, ls, (int)nb, nn));
    // Y = X^{-1} W, rows / D_Rb, G = U_R Y
    NSLG_TRY(zgemm(st, n, n, n, one, Xi, n, nn, W, n, nn, M1, n, nn, (int)nb, false));
    k_rows_div_big<<<blocks(tot), EW, 0, st>>>(M1, S.Pd, dstack, n, (int)nb);
    note_launch(st);
    NSLG_TRY(zgemm2(st, n, n, n, one, S.PU, n, ms, nn, M1, n, (int64_t)J * nn, nn, G0, n, (int64_t)J * nn, nn, nmat,
                    J));
    k_grad_rows<<<blocks((int64_t)n * nb), EW, 0, st>>>(G0, out, n, Nt, J, S.q, S.r, nmat, 0, true);
    note_launch(st);
    // wraps inside the chunks: forward from s_j, backward from s_{j+1} (= s_0 after the last chunk)
    const int maxlen = S.q + (S.r > 0 ? 1 : 0);
    const int fmax = (maxlen - 1) / 2, bmax = maxlen - 1 - (maxlen - 1) / 2;
    if (maxlen > 1) {
        NSLG_CUDA(cudaMemcpyAsync(Gf, G0, tot * sizeof(double2), cudaMemcpyDeviceToDevice, st));
        for (int j = 0; j < J; ++j)  // Gb[g, j] = G0[g, (j + 1) mod J]
            NSLG_CUDA(cudaMemcpy2DAsync(Gb + (int64_t)j * nn, (size_t)J * nn * sizeof(double2),
                                        G0 + (int64_t)((j + 1) % J) * nn, (size_t)J * nn * sizeof(double2),
                                        nn * sizeof(double2), nmat, cudaMemcpyDeviceToDevice, st));
    }
    for (int m = 1; m <= fmax; ++m) {  // G(s+1) = E diag(ph[s-1]) G(s) diag(pinv[s-1]) E', s = s_j + m - 1
        k_wrap_scale<<<blocks(tot), EW, 0, st>>>(Gf, ph, pinv, n, Nt, J, S.q, S.r, nmat, m - 1, true);
        note_launch(st);
        NSLG_TRY(zgemm2(st, n, n, n, one, S.E, n, nn, 0, Gf, n, (int64_t)J * nn, nn, Wt, n, (int64_t)J * nn, nn,
                        nmat, J, S.real ? 1 : 0));
        NSLG_TRY(zgemm2(st, n, n, n, one, Wt, n, (int64_t)J * nn, nn, S.Ep, n, nn, 0, Gf, n, (int64_t)J * nn, nn,
                        nmat, J, S.real ? 2 : 0));
        k_grad_rows<<<blocks((int64_t)n * nb), EW, 0, st>>>(Gf, out, n, Nt, J, S.q, S.r, nmat, m, true);
        note_launch(st);
    }
    for (int m = 1; m <= bmax; ++m) {  // G(s) = diag(pinv[s-1]) E' G(s+1) E diag(ph[s-1]), s = s_{j+1} - m
        NSLG_TRY(zgemm2(st, n, n, n, one, S.Ep, n, nn, 0, Gb, n, (int64_t)J * nn, nn, Wt, n, (int64_t)J * nn, nn,
                        nmat, J, S.real ? 1 : 0));
        NSLG_TRY(zgemm2(st, n, n, n, one, Wt, n, (int64_t)J * nn, nn, S.E, n, nn, 0, Gb, n, (int64_t)J * nn, nn,
                        nmat, J, S.real ? 2 : 0));
        k_wrap_scale<<<blocks(tot), EW, 0, st>>>(Gb, ph, pinv, n, Nt, J, S.q, S.r, nmat, m, false);
        note_launch(st);
        k_grad_rows<<<blocks((int64_t)n * nb), EW, 0, st>>>(Gb, out, n, Nt, J, S.q, S.r, nmat, m, false);
        note_launch(st);
    }
    NSLG_CUDA(cudaGetLastError());
    return NSLG_OK;
}

// log det M for nmat matrices (as above; ph[g] = phiExp rows, sgn_g the species sign of matrix g): the suffix stack
// to s = 0, then log det(1 + C(0)) = log det U_L + sum log D_Lb + log det X with X = D_Lb^{-1} U_L^H + D_Ls T_L,
// plus log det of the slices' inverses, Nt sgn delta tr K + sum Log phiExp. out[g] on the host, imaginary part on
// the principal branch; -inf for a singular X.
int logdet_strat(nslg_fm *fm, int nmat, const ExpEntry *const *Ep, const ExpEntry *const *E, const int *sgn,
                 const double2 *ph, const double2 *pinv, double2 *out) {
    cudaStream_t st = fm->ctx->stream;
    Strat S;
    NSLG_TRY(strat_setup(fm, nmat, Ep, E, false, S));
    NSLG_TRY(strat_chunks(fm, S, pinv));
    NSLG_TRY(strat_stacks(fm, S));
    const int n = S.n, J = S.J;
    const int64_t nn = (int64_t)n * n, ms = (int64_t)(J + 1) * nn, ds = (int64_t)(J + 1) * n;
    double2 *ULH, *X, *Uc, *terms;
    NSLG_TRY(ws_get(fm, "stl_ULH", (size_t)nmat * nn, &ULH));
    NSLG_TRY(ws_get(fm, "stl_X", (size_t)nmat * nn, &X));
    NSLG_TRY(ws_get(fm, "stl_U", (size_t)nmat * nn, &Uc));
    NSLG_TRY(ws_get(fm, "stl_terms", (size_t)nmat, &terms));
    NSLG_TRY(ctrans(st, S.SU, flat(ms), ULH, flat(nn), n, nmat));
    // X = D_Lb^{-1} U_L^H + D_Ls T_L (the boundary formula with an identity prefix)
    double *ones;
    NSLG_TRY(ws_get(fm, "stl_ones", (size_t)n, &ones));
    k_ones<<<blocks(n), EW, 0, st>>>(ones, flat(0), n, 1);
    note_launch(st);
    k_boundary_x<<<blocks(nn * nmat), EW, 0, st>>>(ULH, S.ST, flat(ms), S.Sd, flat(ds), ones, flat(0), nullptr, X,
                                                   nullptr, n, nmat);
    note_launch(st);
    NSLG_CUDA(cudaGetLastError());
    NSLG_CUDA(cudaMemcpy2DAsync(Uc, nn * sizeof(double2), S.SU, ms * sizeof(double2), nn * sizeof(double2), nmat,
                                cudaMemcpyDeviceToDevice, st));
    LuScratch lx, lu;
    NSLG_TRY(get_lu_scratch(fm, n, lx, nmat, "stl_x"));
    NSLG_TRY(get_lu_scratch(fm, n, lu, nmat, "stl_u"));
    NSLG_CUDA(cudaMemsetAsync(lx.singular, 0, sizeof(int), st));
    NSLG_TRY(lu_factor(fm, X, n, lx, nmat, nn, true, true));
    std::vector<double2> lsx(nmat), lsu(nmat), tm(nmat);
    std::vector<int> swx(nmat), swu(nmat);
    int sing = 0;
    NSLG_CUDA(cudaMemcpyAsync(lsx.data(), lx.logsum, nmat * sizeof(double2), cudaMemcpyDeviceToHost, st));
    NSLG_CUDA(cudaMemcpyAsync(swx.data(), lx.swaps, nmat * sizeof(int), cudaMemcpyDeviceToHost, st));
    NSLG_CUDA(cudaMemcpyAsync(&sing, lx.singular, sizeof(int), cudaMemcpyDeviceToHost, st));
    NSLG_TRY(lu_factor(fm, Uc, n, lu, nmat, nn, true, true));  // det U_L (unitary: its phase)
    k_logdet_terms<<<(unsigned)nmat, 256, 0, st>>>(S.Sd, flat(ds), ph, n, (int)fm->Nt, terms);
    note_launch(st);
    NSLG_CUDA(cudaGetLastError());
    NSLG_CUDA(cudaMemcpyAsync(lsu.data(), lu.logsum, nmat * sizeof(double2), cudaMemcpyDeviceToHost, st));
    NSLG_CUDA(cudaMemcpyAsync(swu.data(), lu.swaps, nmat * sizeof(int), cudaMemcpyDeviceToHost, st));
    NSLG_CUDA(cudaMemcpyAsync(tm.data(), terms, nmat * sizeof(double2), cudaMemcpyDeviceToHost, st));
    NSLG_CUDA(cudaStreamSynchronize(st));
    for (int g = 0; g < nmat; ++g) {
        if (sing) {
            out[g] = make_double2(-INFINITY, 0.0);
            continue;
        }
        // Nt sgn delta tr K
        const double2 dtr = make_double2(sgn[g] * fm->delta.x * fm->hops_trace.x - sgn[g] * fm->delta.y * fm->hops_trace.y,
                                         sgn[g] * fm->delta.x * fm->hops_trace.y + sgn[g] * fm->delta.y * fm->hops_trace.x);
        double re = lsx[g].x + lsu[g].x + tm[g].x + (double)fm->Nt * dtr.x;
        double im = lsx[g].y + lsu[g].y + tm[g].y + (double)fm->Nt * dtr.y + ((swx[g] + swu[g]) & 1 ? M_PI : 0.0);
        im = std::remainder(im, 2.0 * M_PI);
        if (im <= -M_PI) im += 2.0 * M_PI;
        out[g] = make_double2(re, im);
    }
    return NSLG_OK;
}

}  // namespace nslg
