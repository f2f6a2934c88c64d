// Resident CG: the whole solve of one small system in one CTA, its vectors in shared memory.
//
// Included by cg.cu (it uses the solver's CgState, status codes and block reductions). For systems of at most a
// thousand or so elements an iteration of the launch-per-step solver is 4-6 launches of almost no work each: launch
// latency bounds it. Here one CTA owns one system (one right-hand side of one fermion matrix, or the whole batch of
// a matrix in the reference's shared mode) and runs the iteration of CG.tpp:15-95 on A = M M^dagger (M^dagger M)
// with every step in registers and shared memory: the two operator factors (hubbardExp.tpp:13-75, real
// exp(delta K) staged transposed in shared memory), the dot products as block reductions (warp shuffles), the
// x / r / p updates and the solver's state machine (reliable updates, double-double rebases, stall escalation) in
// the same loop. One launch carries every small system of a solve, each CTA until its system converges or is
// exhausted, or for a bounded number of iterations after which the host launches it again (the state, r and p are
// written back).
//
// Arithmetic. The iteration's operator products run in float-float (each operand and exp(delta K) as an unevaluated
// sum hi + lo of two FP32 numbers; products by the FMA two-product, sums by Knuth's two-sum, ~44 significant bits):
// FP64-class accuracy on the FP32 pipe, which does 128 FMA per clock per SM against FP64's ~2 on this part (the
// mixed-precision requests map here). Vectors are FP64, the curvature |M^dagger p|^2 is summed in FP64, and FP64
// reliable updates recompute r = b - A x with the FP64 operator when |r|^2 fell 1e4x below its running maximum or
// reached the target. A system whose iteration stops gaining escalates to the FP64 operator in the same kernel (the
// launch-per-step solver escalates all systems together). Under the double-double rule the rebase (fold x into
// X = Xh + Xl, r = b - A X in double-double) also runs in the kernel.
//
// Shared memory per CTA (n = system elements, Nx sites): r, p, t (FP64, 48 n bytes), a 32 n byte scratch region
// (two float-float operand vectors, or two FP64 vectors), exp(delta K) transposed as float-float and in FP64
// (16 Nx^2 bytes).
//
// (Included inside cg.cu's anonymous namespace.)

struct RSys {
    const double2 *ph;  // phases exp(i sgn phi + sgn mu~) (Nt, Nx) of the system's fermion matrix
    const double *E;    // exp(sgn delta K), real (delta real), row-major (Nx, Nx)
    int Nt, Nx;
    int64_t off;        // the system's first element in the packed vectors
    int len;            // its elements: rhs * Nt * Nx
};

struct RArgs {
    const RSys *sys;
    const int *list;  // the systems this launch runs (blockIdx.x -> system index)
    const double2 *b;
    double2 *bseg;    // double-double rule: b - A X at the last rebase (the FP64 updates subtract A x from it)
    double2 *x, *r, *p;
    double2 *Xh, *Xl;
    CgState *st;      // the resident systems' own states (not the launch-per-step solver's)
    int *prec64;      // per system: 1 once it runs the FP64 operator (escalated)
    int *counts;      // per system: reliable updates, double-double rebases, escalations
    int64_t max_iter;
    int op;           // NSLG_OP_MMDAGGER or NSLG_OP_MDAGGERM
    int reliable;     // 0: the reference's recurrence rule (FP64 only); 1: reliable updates
    int dd;
    int budget;       // iterations per launch
};

__host__ __device__ constexpr size_t res_smem_bytes(int64_t len, int Nx) {
    return (size_t)len * 80 + (size_t)Nx * Nx * 16;
}

// ----- complex helpers ---------------------------------------------------------------------------------------------
__device__ __forceinline__ double2 r_cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 r_cmulc(double2 a, double2 b) {  // conj(a) b
    return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}

// Element i of a system of rhs blocks of (Nt, Nx): its slice to, site x, and the element offset of the input row
// that feeds it in M (slice to - 1) and M^dagger (slice to + 1), with the boundary signs.
struct RIdx {
    int x, v;            // site, and element of the phases (slice to, site x)
    int rowM, rowD;      // element offsets of the input rows
    double sM, sD;       // -1 on the anti-periodic wrap
};
__device__ __forceinline__ RIdx r_index(int i, int Nt, int Nx) {
    RIdx q;
    const int row = i / Nx;
    q.x = i - row * Nx;
    const int blk = row / Nt;
    const int to = row - blk * Nt;
    const int tm = to == 0 ? Nt - 1 : to - 1;
    const int tp = to == Nt - 1 ? 0 : to + 1;
    q.v = to * Nx + q.x;
    q.rowM = (blk * Nt + tm) * Nx;
    q.rowD = (blk * Nt + tp) * Nx;
    q.sM = to == 0 ? -1.0 : 1.0;
    q.sD = to == Nt - 1 ? -1.0 : 1.0;
    return q;
}

// sum_y E[x, y] v[row + y] with E staged transposed (Et[y Nx + x]): a warp reads consecutive x (no bank conflicts)
// and one broadcast v element per step.
__device__ __forceinline__ double2 r_rowdot(const double *Et, const double2 *v, int Nx, int x) {
    double2 a = make_double2(0, 0);
    for (int y = 0; y < Nx; ++y) {
        const double e = Et[y * Nx + x];
        const double2 w = v[y];
        a.x = fma(e, w.x, a.x);
        a.y = fma(e, w.y, a.y);
    }
    return a;
}
// Float-float: a value is hi + lo with |lo| <= ulp(hi) / 2; a complex operand element is float4 {re hi, im hi,
// re lo, im lo}, an exp(delta K) element float2 {hi, lo}. The _rn intrinsics keep the compiler from contracting the
// error-free steps into FMAs.
__device__ __forceinline__ float4 r_ff_split(double2 v) {
    const float rh = (float)v.x, ih = (float)v.y;
    return make_float4(rh, ih, (float)(v.x - (double)rh), (float)(v.y - (double)ih));
}
// S + C += a * b with a = ah + al, b = bh + bl: the product of the high parts exactly (two-product), the cross terms in
// FP32, the sum into S by two-sum, every error into C.
__device__ __forceinline__ void r_ff_mac(float &S, float &C, float ah, float al, float bh, float bl) {
    const float p = __fmul_rn(ah, bh);
    float e = fmaf(ah, bh, -p);
    e = fmaf(ah, bl, e);
    e = fmaf(al, bh, e);
    const float s = __fadd_rn(S, p);
    const float bb = __fsub_rn(s, S);
    const float err = __fadd_rn(__fsub_rn(S, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    S = s;
    C = __fadd_rn(C, __fadd_rn(err, e));
}
// sum_y E[x, y] v[row + y] in float-float, returned in FP64
__device__ __forceinline__ double2 r_rowdot_ff(const float2 *Et, const float4 *v, int Nx, int x) {
    float Sr = 0.f, Cr = 0.f, Si = 0.f, Ci = 0.f;
    for (int y = 0; y < Nx; ++y) {
        const float2 e = Et[y * Nx + x];
        const float4 w = v[y];
        r_ff_mac(Sr, Cr, e.x, e.y, w.x, w.z);
        r_ff_mac(Si, Ci, e.x, e.y, w.y, w.w);
    }
    return make_double2((double)Sr + (double)Cr, (double)Si + (double)Ci);
}

// ----- double-double (error-free transformations: FMA two-product, Knuth two-sum) -------------------------------------
struct rdd {
    double hi, lo;
};
__device__ __forceinline__ rdd r_two_sum(double a, double b) {
    const double s = a + b;
    const double bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ rdd r_fast_two_sum(double a, double b) {
    const double s = a + b;
    return {s, b - (s - a)};
}
__device__ __forceinline__ rdd r_dd_add(rdd a, rdd b) {
    rdd s = r_two_sum(a.hi, b.hi);
    s.lo += a.lo + b.lo;
    return r_fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ rdd r_dd_neg(rdd a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ rdd r_dd_mul_d(rdd a, double b) {
    const double p = a.hi * b;
    const double e = fma(a.hi, b, -p);
    return r_fast_two_sum(p, fma(a.lo, b, e));
}
struct rddc {
    rdd re, im;
};
__device__ __forceinline__ rddc r_ddc(double2 h, double2 l) { return {r_fast_two_sum(h.x, l.x), r_fast_two_sum(h.y, l.y)}; }
__device__ __forceinline__ rddc r_cmul_dd(double2 a, rddc v) {  // a v, a FP64
    return {r_dd_add(r_dd_mul_d(v.re, a.x), r_dd_neg(r_dd_mul_d(v.im, a.y))),
            r_dd_add(r_dd_mul_d(v.im, a.x), r_dd_mul_d(v.re, a.y))};
}
__device__ __forceinline__ rddc r_cmulc_dd(double2 a, rddc v) {  // conj(a) v
    return {r_dd_add(r_dd_mul_d(v.re, a.x), r_dd_mul_d(v.im, a.y)),
            r_dd_add(r_dd_mul_d(v.im, a.x), r_dd_neg(r_dd_mul_d(v.re, a.y)))};
}
__device__ __forceinline__ rddc r_axpy_dd(rddc acc, double e, rddc w) {
    return {r_dd_add(acc.re, r_dd_mul_d(w.re, e)), r_dd_add(acc.im, r_dd_mul_d(w.im, e))};
}
// a - s z (s = +-1)
__device__ __forceinline__ rddc r_sub_dd(rddc a, double s, rddc z) {
    if (s < 0) return {r_dd_add(a.re, z.re), r_dd_add(a.im, z.im)};
    return {r_dd_add(a.re, r_dd_neg(z.re)), r_dd_add(a.im, r_dd_neg(z.im))};
}

// ----- the kernel --------------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(RT) k_cg_resident(RArgs A) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int s = A.list[blockIdx.x];
    const RSys Y = A.sys[s];
    const int Nt = Y.Nt, Nx = Y.Nx, n = Y.len;
    const int64_t off = Y.off;
    const int tid = threadIdx.x;
    double2 *r = reinterpret_cast<double2 *>(smem);
    double2 *p = r + n;
    double2 *t = p + n;
    // scratch (32 n bytes): two float-float vectors fa, fb, or two FP64 vectors u64, w64
    float4 *fa = reinterpret_cast<float4 *>(t + n);
    float4 *fb = fa + n;
    double2 *u64 = reinterpret_cast<double2 *>(fa);
    double2 *w64 = u64 + n;
    float2 *Eff = reinterpret_cast<float2 *>(fb + n);  // exp(delta K) transposed, float-float
    double *Et = reinterpret_cast<double *>(Eff + Nx * Nx);  // and in FP64

    __shared__ CgState S;
    __shared__ int prec64, status_sh, newdir_sh;
    __shared__ double beta_sh, alpha_re, alpha_im;
    __shared__ int n_upd, n_reb, n_esc;
    if (tid == 0) {
        S = A.st[s];
        prec64 = A.prec64[s];
        n_upd = A.counts[3 * s];
        n_reb = A.counts[3 * s + 1];
        n_esc = A.counts[3 * s + 2];
    }
    __syncthreads();
    if (S.status != CG_ACTIVE && S.status != CG_UPDATE) return;

    const double2 *bg = A.b + off;
    const double2 *bupd = (A.dd ? A.bseg : A.b) + off;
    double2 *xg = A.x + off;
    const double2 *ph = Y.ph;
    for (int i = tid; i < n; i += RT) {
        r[i] = A.r[off + i];
        p[i] = A.p[off + i];
    }
    for (int i = tid; i < Nx * Nx; i += RT) {
        const int xx = i / Nx, yy = i - xx * Nx;  // E[xx, yy] -> [yy Nx + xx]
        const double e = Y.E[i];
        const float eh = (float)e;
        Et[yy * Nx + xx] = e;
        Eff[yy * Nx + xx] = make_float2(eh, (float)(e - (double)eh));
    }
    const bool mmdag = A.op == NSLG_OP_MMDAGGER;

    // the operands derived from p: float-float p (M M^dagger) or phased p (M^dagger M); FP64 phased p when
    // escalated (M^dagger M)
    auto refresh = [&]() {
        __syncthreads();
        if (!prec64) {
            for (int i = tid; i < n; i += RT) {
                if (mmdag) fa[i] = r_ff_split(p[i]);
                else fb[i] = r_ff_split(r_cmul(ph[i % (Nt * Nx)], p[i]));
            }
        } else if (!mmdag) {
            for (int i = tid; i < n; i += RT) u64[i] = r_cmul(ph[i % (Nt * Nx)], p[i]);
        }
        __syncthreads();
    };

    // t = A p; alpha = |r|^2 / curvature into alpha_re / alpha_im
    auto apply_iter = [&]() {
        double2 acc = make_double2(0, 0);
        if (!prec64) {  // float-float products, curvature |h|^2 of the first factor h
            for (int i = tid; i < n; i += RT) {
                const RIdx q = r_index(i, Nt, Nx);
                const double2 ph_i = ph[q.v];
                double2 h;
                if (mmdag) {  // h = M^dagger p; fb = phase o h
                    const double2 z = r_cmulc(ph_i, r_rowdot_ff(Eff, fa + q.rowD, Nx, q.x));
                    h = make_double2(p[i].x - q.sD * z.x, p[i].y - q.sD * z.y);
                    fb[i] = r_ff_split(r_cmul(ph_i, h));
                } else {  // h = M p; fa = h
                    const double2 z = r_rowdot_ff(Eff, fb + q.rowM, Nx, q.x);
                    h = make_double2(p[i].x - q.sM * z.x, p[i].y - q.sM * z.y);
                    fa[i] = r_ff_split(h);
                }
                t[i] = h;
                acc.x += h.x * h.x + h.y * h.y;
            }
            __syncthreads();
            for (int i = tid; i < n; i += RT) {
                const RIdx q = r_index(i, Nt, Nx);
                double2 z;
                double sg;
                if (mmdag) {  // t = M h
                    z = r_rowdot_ff(Eff, fb + q.rowM, Nx, q.x);
                    sg = q.sM;
                } else {  // t = M^dagger h
                    z = r_cmulc(ph[q.v], r_rowdot_ff(Eff, fa + q.rowD, Nx, q.x));
                    sg = q.sD;
                }
                const double2 h = t[i];
                t[i] = make_double2(h.x - sg * z.x, h.y - sg * z.y);
            }
            const double c = block_sum(acc.x);
            if (tid == 0) {
                alpha_re = S.rsq / c;
                alpha_im = 0.0;
            }
            __syncthreads();
            return;
        }
        // FP64 operator (escalated), alpha = |r|^2 / <p, A p> (CG.tpp:45-52)
        for (int i = tid; i < n; i += RT) {
            const RIdx q = r_index(i, Nt, Nx);
            const double2 ph_i = ph[q.v];
            if (mmdag) {
                const double2 z = r_cmulc(ph_i, r_rowdot(Et, p + q.rowD, Nx, q.x));
                const double2 h = make_double2(p[i].x - q.sD * z.x, p[i].y - q.sD * z.y);
                t[i] = h;
                w64[i] = r_cmul(ph_i, h);
            } else {
                const double2 z = r_rowdot(Et, u64 + q.rowM, Nx, q.x);
                w64[i] = make_double2(p[i].x - q.sM * z.x, p[i].y - q.sM * z.y);
            }
        }
        __syncthreads();
        for (int i = tid; i < n; i += RT) {
            const RIdx q = r_index(i, Nt, Nx);
            double2 o;
            if (mmdag) {
                const double2 z = r_rowdot(Et, w64 + q.rowM, Nx, q.x);
                o = make_double2(t[i].x - q.sM * z.x, t[i].y - q.sM * z.y);
            } else {
                const double2 z = r_cmulc(ph[q.v], r_rowdot(Et, w64 + q.rowD, Nx, q.x));
                o = make_double2(w64[i].x - q.sD * z.x, w64[i].y - q.sD * z.y);
            }
            const double2 pv = p[i];
            acc.x += pv.x * o.x + pv.y * o.y;
            acc.y += pv.x * o.y - pv.y * o.x;
            t[i] = o;
        }
        const double2 pt = block_sum2(acc);
        if (tid == 0) {
            const double den = pt.x * pt.x + pt.y * pt.y;
            alpha_re = S.rsq * pt.x / den;
            alpha_im = -S.rsq * pt.y / den;
        }
        __syncthreads();
    };

    // r = b_upd - A x with the FP64 operator (x from global memory); returns |r|^2
    auto true_residual = [&]() -> double {
        double acc = 0;
        __syncthreads();
        if (!mmdag) {
            for (int i = tid; i < n; i += RT) u64[i] = r_cmul(ph[i % (Nt * Nx)], xg[i]);
            __syncthreads();
        }
        for (int i = tid; i < n; i += RT) {
            const RIdx q = r_index(i, Nt, Nx);
            const double2 ph_i = ph[q.v];
            const double2 xv = xg[i];
            if (mmdag) {
                const double2 z = r_cmulc(ph_i, r_rowdot(Et, xg + q.rowD, Nx, q.x));
                const double2 h = make_double2(xv.x - q.sD * z.x, xv.y - q.sD * z.y);
                t[i] = h;
                w64[i] = r_cmul(ph_i, h);
            } else {
                const double2 z = r_rowdot(Et, u64 + q.rowM, Nx, q.x);
                w64[i] = make_double2(xv.x - q.sM * z.x, xv.y - q.sM * z.y);
            }
        }
        __syncthreads();
        for (int i = tid; i < n; i += RT) {
            const RIdx q = r_index(i, Nt, Nx);
            double2 o;
            if (mmdag) {
                const double2 z = r_rowdot(Et, w64 + q.rowM, Nx, q.x);
                o = make_double2(t[i].x - q.sM * z.x, t[i].y - q.sM * z.y);
            } else {
                const double2 z = r_cmulc(ph[q.v], r_rowdot(Et, w64 + q.rowD, Nx, q.x));
                o = make_double2(w64[i].x - q.sD * z.x, w64[i].y - q.sD * z.y);
            }
            const double2 bv = bupd[i];
            const double2 rv = make_double2(bv.x - o.x, bv.y - o.y);
            r[i] = rv;
            acc += rv.x * rv.x + rv.y * rv.y;
        }
        return block_sum(acc);
    };

    // Double-double rebase: X += x, x = 0, r = b_seg = b - A X in double-double; returns |r|^2
    auto rebase = [&]() -> double {
        double2 *Xh = A.Xh + off, *Xl = A.Xl + off;
        double2 *Tl = u64;  // the intermediate's low part; its high part goes to t
        __syncthreads();
        for (int i = tid; i < n; i += RT) {
            const double2 h = Xh[i], l = Xl[i];
            const double2 v = xg[i];
            const rdd a = r_dd_add({h.x, l.x}, {v.x, 0.0});
            const rdd c = r_dd_add({h.y, l.y}, {v.y, 0.0});
            Xh[i] = make_double2(a.hi, c.hi);
            Xl[i] = make_double2(a.lo, c.lo);
            xg[i] = make_double2(0, 0);
        }
        __syncthreads();
        for (int i = tid; i < n; i += RT) {
            const RIdx q = r_index(i, Nt, Nx);
            rddc z = {{0, 0}, {0, 0}};
            rddc o;
            const rddc xi = r_ddc(Xh[i], Xl[i]);
            if (mmdag) {  // M^dagger X
                for (int y = 0; y < Nx; ++y)
                    z = r_axpy_dd(z, Et[y * Nx + q.x], r_ddc(Xh[q.rowD + y], Xl[q.rowD + y]));
                o = r_sub_dd(xi, q.sD, r_cmulc_dd(ph[q.v], z));
            } else {  // M X
                for (int y = 0; y < Nx; ++y) {
                    const int j = q.rowM + y;
                    z = r_axpy_dd(z, Et[y * Nx + q.x], r_cmul_dd(ph[j % (Nt * Nx)], r_ddc(Xh[j], Xl[j])));
                }
                o = r_sub_dd(xi, q.sM, z);
            }
            t[i] = make_double2(o.re.hi, o.im.hi);
            Tl[i] = make_double2(o.re.lo, o.im.lo);
        }
        __syncthreads();
        double acc = 0;
        for (int i = tid; i < n; i += RT) {
            const RIdx q = r_index(i, Nt, Nx);
            rddc z = {{0, 0}, {0, 0}};
            rddc o;
            const rddc ti = r_ddc(t[i], Tl[i]);
            if (mmdag) {  // M T
                for (int y = 0; y < Nx; ++y) {
                    const int j = q.rowM + y;
                    z = r_axpy_dd(z, Et[y * Nx + q.x], r_cmul_dd(ph[j % (Nt * Nx)], r_ddc(t[j], Tl[j])));
                }
                o = r_sub_dd(ti, q.sM, z);
            } else {  // M^dagger T
                for (int y = 0; y < Nx; ++y) z = r_axpy_dd(z, Et[y * Nx + q.x], r_ddc(t[q.rowD + y], Tl[q.rowD + y]));
                o = r_sub_dd(ti, q.sD, r_cmulc_dd(ph[q.v], z));
            }
            const double2 bv = bg[i];
            const rdd rr = r_dd_add({bv.x, 0.0}, r_dd_neg(o.re));
            const rdd ri = r_dd_add({bv.y, 0.0}, r_dd_neg(o.im));
            const double2 rv = make_double2(rr.hi + rr.lo, ri.hi + ri.lo);
            r[i] = rv;
            acc += rv.x * rv.x + rv.y * rv.y;
        }
        __syncthreads();
        for (int i = tid; i < n; i += RT) A.bseg[off + i] = r[i];
        return block_sum(acc);
    };

    refresh();
    int steps = 0;
    while (steps < A.budget) {
        if (S.status == CG_ACTIVE) {
            ++steps;
            apply_iter();
            const double ar = alpha_re, ai = alpha_im;
            double acc = 0;
            for (int i = tid; i < n; i += RT) {
                const double2 pv = p[i], tv = t[i];
                double2 xv = xg[i], rv = r[i];
                xv.x += ar * pv.x - ai * pv.y;
                xv.y += ar * pv.y + ai * pv.x;
                rv.x -= ar * tv.x - ai * tv.y;
                rv.y -= ar * tv.y + ai * tv.x;
                xg[i] = xv;
                r[i] = rv;
                acc += rv.x * rv.x + rv.y * rv.y;
            }
            const double rn = block_sum(acc);
            if (tid == 0) {  // the transitions of k_cg_p (both operators are FP64-class here)
                CgState N = S;
                N.iters = S.iters + 1;
                if (!A.reliable) {
                    if (rn <= S.eps2) N.status = CG_CONVERGED;
                    else if (N.iters >= A.max_iter) N.status = CG_EXHAUSTED;
                } else if (rn <= S.tgt || rn < UPDATE_FRAC_FP64_CLASS * S.maxr || N.iters >= A.max_iter) {
                    N.status = CG_UPDATE;
                    N.trig = rn;
                }
                if (N.status == CG_ACTIVE) {
                    beta_sh = rn / S.rsq;
                    N.rsq = rn;
                    N.maxr = fmax(S.maxr, rn);
                }
                S = N;
            }
            __syncthreads();
            if (S.status == CG_ACTIVE) {
                const double beta = beta_sh;
                for (int i = tid; i < n; i += RT) {
                    double2 pv = p[i];
                    const double2 rv = r[i];
                    pv.x = rv.x + beta * pv.x;
                    pv.y = rv.y + beta * pv.y;
                    p[i] = pv;
                }
                refresh();
            }
            continue;
        }
        if (S.status != CG_UPDATE) break;
        // reliable update (and, under the double-double rule, a rebase): the transitions of k_mark_rebase and
        // k_rel_finish
        double rn = true_residual();
        bool reb = false;
        if (A.dd) {
            if (tid == 0) {
                const bool floor = !(rn < 0.25 * S.best) && S.stall >= 1;
                status_sh = (rn <= S.eps2 || rn <= REBASE_FRAC * S.base || floor) ? 1 : 0;
            }
            __syncthreads();
            reb = status_sh != 0;
            if (reb) rn = rebase();
        }
        if (tid == 0) {
            ++n_upd;
            if (reb) ++n_reb;
            CgState N = S;
            const bool may_stall = !prec64;  // float-float escalates to FP64; FP64 stops at its floor
            const bool converged = rn <= S.eps2 && (!A.dd || reb);
            N.rsq = rn;
            N.maxr = rn;
            N.last_upd = S.iters;
            if (reb && rn < 0.25 * S.base) {
                N.base = rn;
                N.best = rn;
                N.stall = 0;
            } else if (rn < 0.25 * S.best) {
                N.best = rn;
                N.stall = 0;
            } else {
                N.best = fmin(S.best, rn);
                N.stall = S.stall + 1;
            }
            if (reb) N.base = rn;
            int newdir = 0;
            if (converged) {
                N.status = CG_CONVERGED;
            } else if (S.iters >= A.max_iter) {
                N.status = CG_EXHAUSTED;
            } else if (may_stall && N.stall >= STALL_LIMIT) {
                // escalation (k_resume): this system continues with the FP64 operator from p = r
                prec64 = 1;
                ++n_esc;
                N.status = CG_ACTIVE;
                N.stall = 0;
                N.maxr = rn;
                newdir = 2;
            } else if (!may_stall && N.stall >= FLOOR_LIMIT) {
                N.status = CG_EXHAUSTED;
            } else {
                if (S.trig <= S.tgt) N.tgt = 0.25 * S.tgt;
                newdir = 1;
                N.status = CG_ACTIVE;
            }
            beta_sh = rn / S.rsq;
            newdir_sh = newdir;
            S = N;
        }
        __syncthreads();
        if (newdir_sh == 1) {
            const double beta = beta_sh;
            for (int i = tid; i < n; i += RT) {
                double2 pv = p[i];
                const double2 rv = r[i];
                pv.x = rv.x + beta * pv.x;
                pv.y = rv.y + beta * pv.y;
                p[i] = pv;
            }
        } else if (newdir_sh == 2) {
            for (int i = tid; i < n; i += RT) p[i] = r[i];
        }
        if (S.status == CG_ACTIVE) refresh();
    }
    __syncthreads();
    for (int i = tid; i < n; i += RT) {
        A.r[off + i] = r[i];
        A.p[off + i] = p[i];
    }
    if (tid == 0) {
        A.st[s] = S;
        A.prec64[s] = prec64;
        A.counts[3 * s] = n_upd;
        A.counts[3 * s + 1] = n_reb;
        A.counts[3 * s + 2] = n_esc;
    }
}

// status of the flagged systems <- CG_RESIDENT (their own copy in rst), or back from rst
__global__ void k_resident_handover(CgState *__restrict__ st, CgState *__restrict__ rst, const int *__restrict__ list,
                                    int count, int back) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const int s = list[k];
    if (back) {
        st[s] = rst[s];
    } else {
        rst[s] = st[s];
        CgState S = st[s];
        S.status = CG_RESIDENT;
        st[s] = S;
    }
}
