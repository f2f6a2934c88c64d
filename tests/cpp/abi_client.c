/* A plain C client of libnslgpu (include/nsl_gb300.h): what a caller without C++ or Python does through the C ABI.
 * Test infrastructure (built and run by tests/test_gpu_abi_c.py on a GPU host).
 *
 * Usage: abi_client <dir>. <dir>/params.txt holds "Nx Nt nrhs beta mu"; hops.bin (Nx, Nx), phi.bin (Nt, Nx) and
 * psi.bin (nrhs, Nt, Nx) are raw complex128. Writes M.bin (nrhs, Nt, Nx, particle species), x.bin (CG on MM^dagger
 * per right-hand side, b = psi, split-BF16 mixed precision to 1e-10 relative true residual), logdet.bin (1) and
 * grad.bin (Nt, Nx); prints the CG statistics. Exit status 0 on success, the failing call's status otherwise. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "nsl_gb300.h"

static nslg_c128 *read_c128(const char *dir, const char *name, size_t n) {
    char path[4096];
    snprintf(path, sizeof path, "%s/%s", dir, name);
    FILE *f = fopen(path, "rb");
    if (!f) return NULL;
    nslg_c128 *v = (nslg_c128 *)malloc(n * sizeof(nslg_c128));
    size_t got = fread(v, sizeof(nslg_c128), n, f);
    fclose(f);
    if (got != n) {
        free(v);
        return NULL;
    }
    return v;
}

static int write_c128(const char *dir, const char *name, const nslg_c128 *v, size_t n) {
    char path[4096];
    snprintf(path, sizeof path, "%s/%s", dir, name);
    FILE *f = fopen(path, "wb");
    if (!f) return 1;
    size_t put = fwrite(v, sizeof(nslg_c128), n, f);
    fclose(f);
    return put != n;
}

#define CHECK(call)                                                                  \
    do {                                                                             \
        int rc_ = (call);                                                            \
        if (rc_ != NSLG_OK) {                                                        \
            fprintf(stderr, "%s failed: %d (%s)\n", #call, rc_, nslg_last_error()); \
            return rc_;                                                              \
        }                                                                            \
    } while (0)

int main(int argc, char **argv) {
    if (argc != 2) {
        fprintf(stderr, "usage: %s <dir>\n", argv[0]);
        return 2;
    }
    const char *dir = argv[1];
    char path[4096];
    snprintf(path, sizeof path, "%s/params.txt", dir);
    FILE *pf = fopen(path, "r");
    long long Nx, Nt, R;
    double beta, mu;
    if (!pf || fscanf(pf, "%lld %lld %lld %lf %lf", &Nx, &Nt, &R, &beta, &mu) != 5) return 2;
    fclose(pf);
    nslg_c128 *hops = read_c128(dir, "hops.bin", (size_t)(Nx * Nx));
    nslg_c128 *phi = read_c128(dir, "phi.bin", (size_t)(Nt * Nx));
    nslg_c128 *psi = read_c128(dir, "psi.bin", (size_t)(R * Nt * Nx));
    if (!hops || !phi || !psi) return 2;
    const size_t n = (size_t)(R * Nt * Nx);
    nslg_c128 *out = (nslg_c128 *)malloc(n * sizeof(nslg_c128));
    nslg_c128 *x = (nslg_c128 *)malloc(n * sizeof(nslg_c128));
    nslg_c128 *grad = (nslg_c128 *)malloc((size_t)(Nt * Nx) * sizeof(nslg_c128));

    nslg_ctx *ctx = NULL;
    nslg_fm *fm = NULL;
    nslg_c128 b = {beta, 0.0}, m = {mu, 0.0};
    CHECK(nslg_ctx_create(0, NULL, &ctx));
    CHECK(nslg_fm_create(ctx, Nx, Nt, hops, b, m, NSLG_PARTICLE, &fm));
    CHECK(nslg_fm_populate(fm, phi, NSLG_PARTICLE));
    CHECK(nslg_fm_apply(fm, NSLG_OP_M, psi, out, R, NSLG_PREC_FP64));
    double bnorm = 0.0;
    for (size_t i = 0; i < (size_t)(Nt * Nx); ++i) bnorm += psi[i].re * psi[i].re + psi[i].im * psi[i].im;
    nslg_cg_stats st;
    memset(&st, 0, sizeof st);
    const int rc = nslg_cg_solve(fm, NSLG_OP_MMDAGGER, psi, NULL, x, R, 1e-10 * __builtin_sqrt(bnorm), 100000,
                                 NSLG_CG_PER_RHS, NSLG_PREC_BF16_SPLIT, NSLG_STOP_TRUE_RESIDUAL, &st);
    if (rc != NSLG_OK && rc != NSLG_NOT_CONVERGED) {
        fprintf(stderr, "nslg_cg_solve failed: %d (%s)\n", rc, nslg_last_error());
        return rc;
    }
    nslg_c128 ld;
    CHECK(nslg_fm_logdet(fm, &ld));
    CHECK(nslg_fm_grad_logdet(fm, grad));
    printf("cg iterations %lld converged %lld/%lld true_residual %.3e\n", (long long)st.iterations,
           (long long)st.converged, (long long)st.systems, st.true_residual);
    if (write_c128(dir, "M.bin", out, n) || write_c128(dir, "x.bin", x, n) || write_c128(dir, "logdet.bin", &ld, 1) ||
        write_c128(dir, "grad.bin", grad, (size_t)(Nt * Nx)))
        return 3;
    CHECK(nslg_fm_destroy(fm));
    CHECK(nslg_ctx_destroy(ctx));
    free(hops);
    free(phi);
    free(psi);
    free(out);
    free(x);
    free(grad);
    return 0;
}
