/*
 * Body of the CPU oracle, instantiated twice by fluid_oracle.c: once with
 * REAL = float (the reference's arithmetic, bit-for-bit) and once with
 * REAL = double (the FP64 run of the same method, used to measure error).
 *
 * TEST INFRASTRUCTURE ONLY: this restatement is the checker for the CUDA
 * path. Nothing in the product links it.
 *
 * Each routine follows one function of the reference's src/fluid.cpp; the
 * citation sits above it. Every float expression keeps the reference's
 * evaluation order (the file is compiled with -ffp-contract=off), so the
 * float instantiation reproduces src/fluid.cpp exactly.
 */

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(name, SFX)

/* Interleaved HWC index: src/fluid.cpp:15-17. */
static inline long FN(cell)(int i, int j, int w, int ch) { return ((long)j * w + i) * ch; }

/* Periodic wrap of a backtraced coordinate, src/fluid.cpp:48-49,105-106:
 * fmod(fmod(x, n) + n, n), evaluated in REAL. */
static inline REAL FN(wrap)(REAL x, REAL n) { return FMOD(FMOD(x, n) + n, n); }

/* Boundary modes of the backtrace: 0 periodic (the reference's wrapping
 * mode); 1 clamp, the reference's commented-out alternative
 * (src/fluid.cpp:43-45,100-102): std::max(0.5f, std::min<float>(n - 1.5, x)),
 * after which i0 + 1 stays inside the grid; 2 walls: clamp, and zero velocity
 * on the boundary cells after advection and after projection. */
static inline REAL FN(clampc)(REAL x, REAL n)
{
    const REAL hi = (REAL)((double)n - 1.5);
    const REAL m = (x < hi) ? x : hi;     /* std::min<float>(hi, x): x when x < hi */
    return ((REAL)0.5 < m) ? m : (REAL)0.5; /* std::max(0.5f, m) */
}
static inline REAL FN(bound)(REAL x, REAL n, int bc) { return bc ? FN(clampc)(x, n) : FN(wrap)(x, n); }
static inline int FN(on_edge)(int i, int j, int w, int h) { return i == 0 || j == 0 || i == w - 1 || j == h - 1; }

/* Bilinear weights and sum in the reference's order, src/fluid.cpp:62-66. */
static inline REAL FN(bilerp)(REAL sx, REAL sy, REAL f00, REAL f10, REAL f01, REAL f11)
{
    REAL a = (1 - sx) * (1 - sy) * f00;
    REAL b = sx * (1 - sy) * f10;
    REAL c = (1 - sx) * sy * f01;
    REAL d = sx * sy * f11;
    return ((a + b) + c) + d;
}

/* Velocity advection, src/fluid.cpp:24-70: channels 0-1 of `in` are
 * backtraced by dt*u/width cells (S3), wrapped, and bilinearly sampled into
 * channels 0-1 of `out`; channels 2-3 of `out` are untouched. */
static void FN(advect)(const REAL *in, REAL *out, int w, int h, REAL dt, int bc)
{
    const REAL fw = (REAL)w, fh = (REAL)h;
    OMP_FOR
    for (int j = 0; j < h; j++) {
        for (int i = 0; i < w; i++) {
            const long c = FN(cell)(i, j, w, 4);
            if (bc == 2 && FN(on_edge)(i, j, w, h)) {
                out[c + 0] = 0;
                out[c + 1] = 0;
                continue;
            }
            REAL xp = (REAL)i - dt * in[c + 0] / fw;
            REAL yp = (REAL)j - dt * in[c + 1] / fh;
            xp = FN(bound)(xp, fw, bc);
            yp = FN(bound)(yp, fh, bc);
            const int i0 = (int)xp, j0 = (int)yp;
            const int i1 = (i0 + 1) % w, j1 = (j0 + 1) % h;
            const REAL sx = xp - (REAL)i0, sy = yp - (REAL)j0;
            const long c00 = FN(cell)(i0, j0, w, 4), c10 = FN(cell)(i1, j0, w, 4);
            const long c01 = FN(cell)(i0, j1, w, 4), c11 = FN(cell)(i1, j1, w, 4);
            for (int k = 0; k < 2; k++)
                out[c + k] = FN(bilerp)(sx, sy, in[c00 + k], in[c10 + k], in[c01 + k], in[c11 + k]);
        }
    }
}

/* Image advection, src/fluid.cpp:72-127: each pixel reads the velocity of
 * the nearest velocity cell (S4), backtraces by (dt/viw)*u/iwidth, wraps and
 * samples all `ic` channels bilinearly. */
static void FN(advect_color)(const REAL *img, REAL *out, int iw, int ih, int ic,
                             const REAL *vel, int vw, int vh, REAL dt, int bc)
{
    const REAL fiw = (REAL)iw, fih = (REAL)ih, fvw = (REAL)vw, fvh = (REAL)vh;
    const REAL viw = fvw / fiw, vih = fvh / fih;
    OMP_FOR
    for (int j = 0; j < ih; j++) {
        for (int i = 0; i < iw; i++) {
            const int vi = (int)((REAL)i * viw);
            const int vj = (int)((REAL)j * vih);
            const long vc = FN(cell)(vi, vj, vw, 4);
            REAL xp = (REAL)i - (dt / viw) * vel[vc + 0] / fiw;
            REAL yp = (REAL)j - (dt / vih) * vel[vc + 1] / fih;
            xp = FN(bound)(xp, fiw, bc);
            yp = FN(bound)(yp, fih, bc);
            const int i0 = (int)xp, j0 = (int)yp;
            const int i1 = (i0 + 1) % iw, j1 = (j0 + 1) % ih;
            const REAL sx = xp - (REAL)i0, sy = yp - (REAL)j0;
            const long o = FN(cell)(i, j, iw, ic);
            const long c00 = FN(cell)(i0, j0, iw, ic), c10 = FN(cell)(i1, j0, iw, ic);
            const long c01 = FN(cell)(i0, j1, iw, ic), c11 = FN(cell)(i1, j1, iw, ic);
            for (int k = 0; k < ic; k++)
                out[o + k] = FN(bilerp)(sx, sy, img[c00 + k], img[c10 + k], img[c01 + k], img[c11 + k]);
        }
    }
}

/* One diffusion sweep, src/fluid.cpp:151-186: the centre term is the
 * current iterate (S8); alpha = visc*dt in REAL, beta = 1 + 4*alpha in double. */
static void FN(diffuse_sweep)(const REAL *in, REAL *out, int w, int h, REAL alpha, REAL beta)
{
    OMP_FOR
    for (int j = 0; j < h; j++) {
        const int jm = (j + h - 1) % h, jp = (j + 1) % h;
        for (int i = 0; i < w; i++) {
            const int im = (i + w - 1) % w, ip = (i + 1) % w;
            for (int k = 0; k < 2; k++) {
                REAL l = alpha * in[FN(cell)(im, j, w, 4) + k];
                REAL r = alpha * in[FN(cell)(ip, j, w, 4) + k];
                REAL t = alpha * in[FN(cell)(i, jm, w, 4) + k];
                REAL b = alpha * in[FN(cell)(i, jp, w, 4) + k];
                REAL centre = (REAL)1.0 * in[FN(cell)(i, j, w, 4) + k];
                out[FN(cell)(i, j, w, 4) + k] = ((((l + r) + t) + b) + centre) / beta;
            }
        }
    }
}

/* Divergence into channel 3 of both buffers, src/fluid.cpp:218-237 (S5):
 * b = gamma*((u[i+1]-u[i-1]) + (v[j+1]-v[j-1])), gamma = -1/dt in double,
 * rounded to REAL. */
static void FN(divergence)(REAL *x, REAL *y, int w, int h, REAL gamma)
{
    OMP_FOR
    for (int j = 0; j < h; j++) {
        const int jm = (j + h - 1) % h, jp = (j + 1) % h;
        for (int i = 0; i < w; i++) {
            const int im = (i + w - 1) % w, ip = (i + 1) % w;
            REAL du = x[FN(cell)(ip, j, w, 4) + 0] - x[FN(cell)(im, j, w, 4) + 0];
            REAL dv = x[FN(cell)(i, jp, w, 4) + 1] - x[FN(cell)(i, jm, w, 4) + 1];
            REAL b = gamma * (du + dv);
            x[FN(cell)(i, j, w, 4) + 3] = b;
            y[FN(cell)(i, j, w, 4) + 3] = b;
        }
    }
}

/* One pressure Jacobi sweep on channel 2, src/fluid.cpp:239-257 (S6):
 * p' = (((pL+pR)+pT)+pB + 1*b)/4, periodic neighbours. */
static void FN(pressure_sweep)(const REAL *in, REAL *out, int w, int h)
{
    OMP_FOR
    for (int j = 0; j < h; j++) {
        const int jm = (j + h - 1) % h, jp = (j + 1) % h;
        for (int i = 0; i < w; i++) {
            const int im = (i + w - 1) % w, ip = (i + 1) % w;
            REAL pl = in[FN(cell)(im, j, w, 4) + 2];
            REAL pr = in[FN(cell)(ip, j, w, 4) + 2];
            REAL pt = in[FN(cell)(i, jm, w, 4) + 2];
            REAL pb = in[FN(cell)(i, jp, w, 4) + 2];
            REAL b = in[FN(cell)(i, j, w, 4) + 3];
            out[FN(cell)(i, j, w, 4) + 2] = ((((pl + pr) + pt) + pb) + (REAL)1.0 * b) / (REAL)4.0;
        }
    }
}

/* Residual of the pressure system of src/fluid.cpp:239-257, 4p - sum(nb) = b,
 * evaluated in double per cell as ((((b+pL)+pR)+pT)+pB) - 4p; returns
 * sum r^2 and (through *bb) sum b^2. Rows are summed into per-row partials
 * first and the partials added in row order, so the result does not depend
 * on the thread count. */
static double FN(residual_sq)(const REAL *x, int w, int h, double *bb, double *rowbuf)
{
    OMP_FOR
    for (int j = 0; j < h; j++) {
        const int jm = (j + h - 1) % h, jp = (j + 1) % h;
        double rs = 0.0, bs = 0.0;
        for (int i = 0; i < w; i++) {
            const int im = (i + w - 1) % w, ip = (i + 1) % w;
            double b = (double)x[FN(cell)(i, j, w, 4) + 3];
            double r = b + (double)x[FN(cell)(im, j, w, 4) + 2];
            r = r + (double)x[FN(cell)(ip, j, w, 4) + 2];
            r = r + (double)x[FN(cell)(i, jm, w, 4) + 2];
            r = r + (double)x[FN(cell)(i, jp, w, 4) + 2];
            r = r - 4.0 * (double)x[FN(cell)(i, j, w, 4) + 2];
            rs += r * r;
            bs += b * b;
        }
        rowbuf[2 * j] = rs;
        rowbuf[2 * j + 1] = bs;
    }
    double rsum = 0.0, bsum = 0.0;
    for (int j = 0; j < h; j++) {
        rsum += rowbuf[2 * j];
        bsum += rowbuf[2 * j + 1];
    }
    *bb = bsum;
    return rsum;
}

/* Projection, src/fluid.cpp:269-296 (S7): u -= (pR-pL)*dt/2, v -= (pB-pT)*dt/2,
 * reading pressure and velocity from `in`, writing channels 0-1 of `out`. */
static void FN(project)(const REAL *in, REAL *out, int w, int h, REAL dt, int bc)
{
    OMP_FOR
    for (int j = 0; j < h; j++) {
        const int jm = (j + h - 1) % h, jp = (j + 1) % h;
        for (int i = 0; i < w; i++) {
            const int im = (i + w - 1) % w, ip = (i + 1) % w;
            REAL pl = in[FN(cell)(im, j, w, 4) + 2];
            REAL pr = in[FN(cell)(ip, j, w, 4) + 2];
            REAL pt = in[FN(cell)(i, jm, w, 4) + 2];
            REAL pb = in[FN(cell)(i, jp, w, 4) + 2];
            REAL gx = (pr - pl) * dt / (REAL)2.0;
            REAL gy = (pb - pt) * dt / (REAL)2.0;
            const long c = FN(cell)(i, j, w, 4);
            out[c + 0] = in[c + 0] - gx;
            out[c + 1] = in[c + 1] - gy;
            if (bc == 2 && FN(on_edge)(i, j, w, h)) { /* walls: zero velocity on the boundary cells */
                out[c + 0] = 0;
                out[c + 1] = 0;
            }
        }
    }
}

static void FN(swap)(REAL **a, REAL **b) { REAL *t = *a; *a = *b; *b = t; }

/*
 * One timestep, src/fluid.cpp:298-310, with the buffer ping-pong of the
 * reference kept literally (S9): the caller's two pointers are swapped by
 * diffusion and by the pressure loop exactly as src/fluid.cpp:188-194 and
 * :260-266 swap vp->data / vp_out->data.
 *
 * Generalisation beyond the reference (which fixes both counts to
 * NUM_JACOBI_ITERS): `diffuse_iters` diffusion sweeps, and a pressure solve
 * that either runs exactly `max_iters` sweeps (tol <= 0) or stops at the
 * first check point k (k a multiple of `check_every`, or k == max_iters)
 * where ||b - A p_k||_2 / ||b||_2 <= tol (||r||_2 alone when b == 0).
 * With diffuse_iters == max_iters == NUM_JACOBI_ITERS and tol <= 0 this is
 * src/fluid.cpp:298-310 exactly.
 */
int FN(pfso_step_bc)(REAL **vp, REAL **tmp, int w, int h, REAL dt, REAL visc,
                     int diffuse_iters, int max_iters, double tol, int check_every,
                     int want_residual, int bc, pfso_stats *st)
{
    if (w <= 0 || h <= 0 || diffuse_iters < 0 || max_iters < 0 || bc < 0 || bc > 2) return -1;
    if (bc && (w < 2 || h < 2)) return -1;
    double *rowbuf = (double *)malloc(sizeof(double) * 2 * (size_t)h);
    if (!rowbuf) return -2;

    /* advect(vp, tmp): src/fluid.cpp:300 */
    FN(advect)(*vp, *tmp, w, h, dt, bc);

    /* diffuse(tmp, vp): src/fluid.cpp:301,144-195 */
    {
        REAL alpha = visc * dt;
        REAL beta = (REAL)(1.0 + 4.0 * (double)alpha);
        REAL **src = tmp, **dst = vp;
        for (int it = 0; it < diffuse_iters; it++) {
            FN(diffuse_sweep)(*src, *dst, w, h, alpha, beta);
            if (it != diffuse_iters - 1) FN(swap)(src, dst);
        }
    }

    /* computePressure(vp, tmp): src/fluid.cpp:303,210-267 */
    int sweeps = 0, checks = 0;
    double rel = -1.0, bnorm = -1.0;
    {
        REAL gamma = (REAL)(-1.0 / (double)dt);
        REAL **src = vp, **dst = tmp;
        FN(divergence)(*src, *dst, w, h, gamma);
        for (int it = 0; it < max_iters; it++) {
            FN(pressure_sweep)(*src, *dst, w, h);
            FN(swap)(src, dst); /* *src now holds iterate it+1 */
            sweeps = it + 1;
            int last = (sweeps == max_iters);
            if (tol > 0.0 && (last || (check_every > 0 && sweeps % check_every == 0))) {
                double bb, rr = FN(residual_sq)(*src, w, h, &bb, rowbuf);
                checks++;
                bnorm = sqrt(bb);
                rel = bb > 0.0 ? sqrt(rr) / bnorm : sqrt(rr);
                if (rel <= tol) break;
            }
        }
        if (sweeps > 0) FN(swap)(src, dst); /* the reference skips the last swap */
        if (want_residual && !(tol > 0.0)) {
            double bb, rr = FN(residual_sq)(*dst, w, h, &bb, rowbuf);
            bnorm = sqrt(bb);
            rel = bb > 0.0 ? sqrt(rr) / bnorm : sqrt(rr);
        }
    }

    /* subtractPressureGradient(tmp, vp): src/fluid.cpp:304,269-296 */
    FN(project)(*tmp, *vp, w, h, dt, bc);

    free(rowbuf);
    if (st) {
        st->sweeps = sweeps;
        st->checks = checks;
        st->rel_residual = rel;
        st->bnorm = bnorm;
        st->capped = (tol > 0.0 && sweeps == max_iters && !(rel <= tol)) ? 1 : 0;
    }
    return 0;
}

int FN(pfso_step)(REAL **vp, REAL **tmp, int w, int h, REAL dt, REAL visc,
                  int diffuse_iters, int max_iters, double tol, int check_every,
                  int want_residual, pfso_stats *st)
{
    return FN(pfso_step_bc)(vp, tmp, w, h, dt, visc, diffuse_iters, max_iters, tol, check_every, want_residual, 0,
                            st);
}

/* advect_color_step, src/fluid.cpp:312-320: advect, then swap image/itmp. */
int FN(pfso_advect_color_step_bc)(REAL **image, REAL **itmp, int iw, int ih, int ic,
                                  const REAL *vel, int vw, int vh, REAL dt, int bc)
{
    if (iw <= 0 || ih <= 0 || ic <= 0 || vw <= 0 || vh <= 0 || bc < 0 || bc > 2) return -1;
    if (bc && (iw < 2 || ih < 2)) return -1;
    FN(advect_color)(*image, *itmp, iw, ih, ic, vel, vw, vh, dt, bc);
    FN(swap)(image, itmp);
    return 0;
}

int FN(pfso_advect_color_step)(REAL **image, REAL **itmp, int iw, int ih, int ic,
                               const REAL *vel, int vw, int vh, REAL dt)
{
    return FN(pfso_advect_color_step_bc)(image, itmp, iw, ih, ic, vel, vw, vh, dt, 0);
}

/* Single operators, exposed for unit tests of each stage. */
void FN(pfso_advect)(const REAL *in, REAL *out, int w, int h, REAL dt) { FN(advect)(in, out, w, h, dt, 0); }
void FN(pfso_pressure_sweep)(const REAL *in, REAL *out, int w, int h) { FN(pressure_sweep)(in, out, w, h); }
void FN(pfso_divergence)(REAL *x, REAL *y, int w, int h, REAL dt)
{
    FN(divergence)(x, y, w, h, (REAL)(-1.0 / (double)dt));
}
double FN(pfso_residual)(const REAL *x, int w, int h, double *bnorm_out)
{
    double *rowbuf = (double *)malloc(sizeof(double) * 2 * (size_t)h);
    double bb, rr = FN(residual_sq)(x, w, h, &bb, rowbuf);
    free(rowbuf);
    if (bnorm_out) *bnorm_out = sqrt(bb);
    return bb > 0.0 ? sqrt(rr) / sqrt(bb) : sqrt(rr);
}

#undef FN
