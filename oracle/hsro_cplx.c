/*
 * hsro_cplx.c -- complex-conjugate shifts for the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the library's complex-shift
 * path.  The product never links or calls this file.  It is compiled inside
 * hsro.c's translation unit so that it shares the real scalar kernels
 * (protect_sum, protect_update, protect_real_division), the partition, the
 * tile norms and the scaling-factor algebra.
 *
 * The reference declares complex eigenvalues (problemgenerator.h:12-19 returns
 * wi; main.c:95-97 asserts wi == 0 because "only real eigenvalues are
 * supported") and ships the robust kernels a complex shift needs -- complex
 * division (robust.c:486-675), the complex 1x1 solve (robust.c:677-773) and
 * one scaling factor per pair of columns (robust.c:370-417) -- but its driver
 * stops at real shifts.  This file restates the natural extension: the same
 * tiled Givens RQ factorisation of H - mu I, overflow-protected tiled
 * back-substitution, level-3 tile updates and scale reconciliation, for
 * mu = wr + i*wi, in complex arithmetic.  There is no reference output to pin
 * the whole path against; its scalar kernels are pinned bit for bit against
 * the reference's own robust.c (tests/test_oracle_cplx.py), and the vectors
 * are checked against LAPACK dhsein and by their residuals.
 *
 * Conventions (the LAPACK dhsein/dtrevc layout):
 *   - pair k occupies columns 2k (real part) and 2k+1 (imaginary part) of vr;
 *     the eigenvector of wr - i*wi is the conjugate;
 *   - one scaling factor per pair (robust.c:370-417 gives both columns of a
 *     pair the same factor);
 *   - magnitude bounds use cabs1(z) = |Re z| + |Im z| (LAPACK's CABS1), an
 *     upper bound of |z| that also bounds each component, so every real
 *     overflow decision of the reference applies unchanged to complex
 *     operands; the products in a bound may exceed |t||x| by at most a factor
 *     2 (cabs1(ab) <= cabs1(a) cabs1(b), cabs1(sigma) <= sqrt(2)), which the
 *     margin between Omega = 1e300 and DBL_MAX absorbs;
 *   - the Givens rotation of a complex f against a real g is
 *         [col_j', col_{j-1}'] = [col_j, col_{j-1}] [ c  sigma ; -conj(sigma)  c ]
 *     with c real >= 0, |c|^2 + |sigma|^2 = 1 and sigma*f + c*g = 0, so for a
 *     real f it is reduce.c:14-24's rotation (sigma = s after the negation);
 *   - the bound of y(0:j-2) in the diagonal solve is its largest cabs1 at the
 *     start of step j, times the step's scaling factors -- for real vectors
 *     this equals the reference's recomputed infnorm, for complex ones it is
 *     the same bound up to rounding, and it is what the kernels carry;
 *   - every complex product and update is spelled with explicit fma() in one
 *     fixed shape (the helpers below); the CUDA kernels spell the same shapes,
 *     so the device reproduces this file bit for bit.
 */

/* ------------------------------------------------------------------------ */
/* Complex helpers, fixed expression shapes.                                 */
/* ------------------------------------------------------------------------ */
typedef struct { double re, im; } hcplx;

static inline hcplx cmk(double re, double im) { hcplx z; z.re = re; z.im = im; return z; }
static inline double cabs1(double re, double im) { return fabs(re) + fabs(im); }
/* a * b */
static inline hcplx cmul(hcplx a, hcplx b)
{ return cmk(fma(a.re, b.re, -(a.im * b.im)), fma(a.re, b.im, a.im * b.re)); }
/* conj(a) * b */
static inline hcplx cmulc(hcplx a, hcplx b)
{ return cmk(fma(a.re, b.re, a.im * b.im), fma(a.re, b.im, -(a.im * b.re))); }
/* y + a * b */
static inline hcplx cfma(hcplx a, hcplx b, hcplx y)
{ return cmk(fma(a.re, b.re, fma(-a.im, b.im, y.re)), fma(a.re, b.im, fma(a.im, b.re, y.im))); }
/* y - a * b */
static inline hcplx cfnma(hcplx a, hcplx b, hcplx y)
{ return cmk(fma(-a.re, b.re, fma(a.im, b.im, y.re)), fma(-a.re, b.im, fma(-a.im, b.re, y.im))); }
/* y + a * h, h real */
static inline hcplx cfmar(hcplx a, double h, hcplx y)
{ return cmk(fma(a.re, h, y.re), fma(a.im, h, y.im)); }
static inline hcplx cscal(double c, hcplx a) { return cmk(c * a.re, c * a.im); }
/* Rotation pair of the back-transform and of Ytilde2:
 *   out = c*t1 - conj(s)*t2,   next = c*t2 + s*t1                           */
static inline hcplx crot_out(double c, hcplx s, hcplx t1, hcplx t2)
{ const hcplx q = cmulc(s, t2); return cmk(fma(c, t1.re, -q.re), fma(c, t1.im, -q.im)); }
static inline hcplx crot_next(double c, hcplx s, hcplx t1, hcplx t2)
{ const hcplx p = cmul(s, t1); return cmk(fma(c, t2.re, p.re), fma(c, t2.im, p.im)); }

/* Largest cabs1 over n entries; NaN never wins (vector_infnorm, utils.h:75-85). */
static inline double cinfnorm(int n, const double *re, const double *im)
{
    double nrm = 0.0;
    for (int i = 0; i < n; i++) {
        const double a = cabs1(re[i], im[i]);
        if (a > nrm) nrm = a;
    }
    return nrm;
}
static inline void c_scale(int n, double *re, double *im, double a)
{
    if (a != 1.0)
        for (int i = 0; i < n; i++) { re[i] = a * re[i]; im[i] = a * im[i]; }
}
static inline void c_scale_except(int n, int skip, double *re, double *im, double a)
{
    if (a != 1.0)
        for (int i = 0; i < n; i++)
            if (i != skip) { re[i] = a * re[i]; im[i] = a * im[i]; }
}

/* ------------------------------------------------------------------------ */
/* Robust complex division (robust.c:486-675), restated.                     */
/* ------------------------------------------------------------------------ */
/* protect_mul (robust.c:194-212): alpha with t*(alpha*x) safe. */
static double protect_mul(double tnorm, double xnorm)
{
    double scale = 1.0;
    if (fabs(xnorm) <= 1.0) {
        if (fabs(tnorm) * fabs(xnorm) > g_omega) scale = 0.5;
    } else {
        if (fabs(tnorm) > g_omega / fabs(xnorm)) scale = 0.5 / fabs(xnorm);
    }
    return scale;
}

/* dladiv2 (robust.c:486-568): (alpha, res) with res = alpha * the LAPACK
 * dladiv2 quantity, every intermediate protected. */
static void c_dladiv2(double a, double b, double c, double d, double r, double t,
                      double *ret, double *scale)
{
    double res, alpha = 1.0;
    (void)c;
    if (r != 0.0) {
        const double br = b * r;
        if (br != 0.0) {
            /* (a + b r) t */
            double s = protect_sum(a, br);
            res = (s * a) + (s * br);
            alpha = s * alpha;
            s = protect_mul(fabs(t), fabs(res));
            res = (s * res) * t;
            alpha = s * alpha;
        } else {
            /* a t + (b t) r */
            const double s1 = protect_mul(fabs(t), fabs(a));
            double tmp1 = (s1 * a) * t;
            const double s2 = protect_mul(fabs(t), fabs(b));
            double tmp2 = (s2 * b) * t;
            tmp2 = tmp2 * r;
            const double smin = fmin(s1, s2);
            tmp1 = tmp1 * (s1 / smin);
            tmp2 = tmp2 * (s2 / smin);
            alpha = smin * alpha;
            const double s = protect_sum(tmp1, tmp2);
            res = (s * tmp1) + (s * tmp2);
            alpha = s * alpha;
        }
    } else {
        /* (a + d (b / c)) t */
        const double s1 = protect_real_division(b, c);
        alpha = s1 * alpha;
        double tmp = (s1 * b) / c;
        const double s2 = protect_mul(fabs(d), fabs(tmp));
        alpha = s2 * alpha;
        tmp = d * (s2 * tmp);
        a = (s1 * s2) * a;
        double s = protect_sum(a, tmp);
        alpha = s * alpha;
        tmp = (s * a) + (s * tmp);
        s = protect_mul(fabs(tmp), fabs(t));
        alpha = s * alpha;
        res = (s * tmp) * t;
    }
    *scale = alpha;
    *ret = res;
}

/* dladiv1 (robust.c:571-620): p + i q = (a + i b) / (c + i d), |d| < |c|. */
static void c_dladiv1(double a, double b, double c, double d, double *p, double *q,
                      double *scale)
{
    const double r = d / c;
    const double dr = d * r;
    const double s1 = protect_sum(c, dr);
    const double sum = (s1 * c) + (s1 * dr);
    const double s2 = protect_real_division(1.0, sum);
    const double t = 1.0 / (s2 * sum);
    const double alpha = 1.0 / (s1 * s2);
    double beta1 = 1.0, beta2 = 1.0;
    c_dladiv2(a, b, c, d, r, t, p, &beta1);
    c_dladiv2(b, -a, c, d, r, t, q, &beta2);
    double beta = 1.0;
    /* Opposite-direction factors cannot be consolidated; the reference prints
     * an error there and keeps both parts unscaled (robust.c:601-607). */
    if (!((beta1 > 1.0 && beta2 < 1.0) || (beta1 < 1.0 && beta2 > 1.0))) {
        beta = fmin(beta1, beta2);
        *p = (*p) * (beta / beta1);
        *q = (*q) * (beta / beta2);
    }
    *scale = alpha * beta;
}

/* dladiv (robust.c:623-636). */
static void c_dladiv(double a, double b, double c, double d, double *xr, double *xi,
                     double *scale)
{
    if (fabs(d) < fabs(c)) {
        c_dladiv1(a, b, c, d, xr, xi, scale);
    } else {
        c_dladiv1(b, a, d, c, xr, xi, scale);
        *xi = -(*xi);
    }
}

/* robust_cmplx_div (robust.c:639-675): x = (alpha (a + i b)) / (c + i d)
 * with |c| + |d| lifted to smin when smaller (returns 1 then). */
int hsro_robust_cmplx_div(double smin, double a, double b, double c, double d,
                          double *xr, double *xi, double *scale, int is)
{
    int info = 0;
    if (fabs(c) + fabs(d) < smin) {
        c = smin;
        d = 0.0;
        info = 1;
    }
    double alpha = 1.0;
    c_dladiv(a, b, c, d, xr, xi, &alpha);
    *scale = is ? (double)ilogb(alpha) : alpha;
    return info;
}

/* Complex 1x1 solve: x := (scale x) / (t - l) for complex t and l.  With
 * t = t_re (real) and l = lambda it is solve_1x1_cmplx_system
 * (robust.c:677-773) operation for operation: protect_sum of the real part,
 * the same scale on the imaginary part, the smin lift on |Re| + |Im|, the
 * robust division, and the factor (1/s) * alpha. */
int hsro_csolve_1x1(double smin, double tr, double ti, double lr, double li,
                    double *xr, double *xi, double *scale, int is)
{
    int info = 0;
    const double s = fmin(protect_sum(tr, -lr), protect_sum(ti, -li));
    double csr = (s * tr) - (s * lr);
    double csi = (s * ti) - (s * li);
    if (fabs(csr) + fabs(csi) < smin) {
        csr = smin;
        csi = 0.0;
        info = 1;
    }
    double alpha = 1.0;
    c_dladiv(*xr, *xi, csr, csi, xr, xi, &alpha);
    *scale = is ? (double)ilogb((1.0 / s) * alpha) : (1.0 / s) * alpha;
    return info;
}

/* ------------------------------------------------------------------------ */
/* Complex Givens rotation: c real, sigma complex with                       */
/*   sigma*f + c*g = 0,  c*f - conj(sigma)*g = sign(f) sqrt(|f|^2 + g^2).    */
/* Safe scaling by powers of two (exact; E. Anderson, "Algorithm 978: Safe   */
/* scaling in the Level 1 BLAS", 2017): the phase f/|f| is taken from f      */
/* scaled by its own exponent, |f| and g from both scaled by the exponent of */
/* the larger.  When |f| < 2^-600 |g|, c = 0 (the rotation swaps columns).  */
/* ------------------------------------------------------------------------ */
static inline int exp_clamped(double m)
{
    uint64_t bits;
    memcpy(&bits, &m, sizeof bits);
    int e = (int)((bits >> 52) & 0x7ff) - 1023;
    if (e > 1000) e = 1000;
    if (e < -1000) e = -1000;
    return e;
}
static inline double pow2(int e)
{
    const uint64_t bits = (uint64_t)(1023 + e) << 52;
    double r;
    memcpy(&r, &bits, sizeof r);
    return r;
}

void hsro_cgivens(double fr, double fi, double g, double *c, double *sr, double *si)
{
    if (g == 0.0) {
        *c = 1.0; *sr = 0.0; *si = 0.0;
        return;
    }
    if (fr == 0.0 && fi == 0.0) {
        *c = 0.0; *sr = -copysign(1.0, g); *si = 0.0;
        return;
    }
    const int ef = exp_clamped(fmax(fabs(fr), fabs(fi)));
    const int eg = exp_clamped(fabs(g));
    const int e = ef > eg ? ef : eg;
    /* phase of f */
    const double uf = pow2(-ef);
    const double fsr = fr * uf, fsi = fi * uf;
    const double af1 = sqrt(fma(fsr, fsr, fsi * fsi));
    const double pr = fsr / af1, pi = fsi / af1;
    /* |f| and g on the common scale */
    const double af = (ef - e < -600) ? 0.0 : af1 * pow2(ef - e);
    const double gs = g * pow2(-e);
    const double d = sqrt(fma(af, af, gs * gs));
    *c = af / d;
    const double t = gs / d;
    *sr = -(t * pr);
    *si = t * pi;
}

/* ------------------------------------------------------------------------ */
/* Diagonal tile, complex shift: Givens generation fused with the robust     */
/* back-substitution (reduceDiag reduce.c:27-68 + solve solve-task.c:19-119; */
/* J = 0: factor_and_solve_R11 solve-task.c:123-225).                        */
/* ------------------------------------------------------------------------ */
static int cdiag_tile(const prob_t *P, int J, hcplx mu, double *vre, double *vim,
                      double *yre, double *yim, double *beta, double *c,
                      double *sr, double *si, cnt_t *cn)
{
    const int is = P->is;
    const int l = P->fr[J];
    const int b = P->fr[J + 1] - l;
    const double Hnorm = P->Hn[J + (size_t)J * P->T];
    const double smin = fmax(DBL_EPSILON / 2 * cabs1(mu.re, mu.im), P->smlnum);
    int info = 0;
    double phi;

    for (int j = b - 1; j >= 1; j--) {
        /* Bounds of y(0:j-2), v(0:j-2) as they enter the step. */
        double ynorm = cinfnorm(j - 1, yre, yim);
        const double vnorm = cinfnorm(j - 1, vre, vim);
        const double hsub = HH(l + j, l + j - 1);
        hsro_cgivens(vre[j], vim[j], hsub, &c[j], &sr[j], &si[j]);
        const hcplx sg = cmk(sr[j], si[j]);

        /* y(j) := y(j) / R(j,j), R(j,j) = c v(j) - conj(sigma) H(j,j-1). */
        phi = sc_one(is);
        const int pj = hsro_csolve_1x1(smin, c[j] * vre[j], c[j] * vim[j], sr[j] * hsub,
                                       (-si[j]) * hsub, &yre[j], &yim[j], &phi, is);
        info |= pj;
        cn->pert += pj;
        const double a1 = sc_value(phi, is);
        if (a1 != 1.0) { cn->divr++; ynorm = a1 * ynorm; }
        *beta = sc_combine(*beta, phi, is);
        c_scale_except(b, j, yre, yim, a1);

        /* y(j-1), protected (solve-task.c:84-90). */
        const hcplx hd = cmk(HH(l + j - 1, l + j - 1) - mu.re, -mu.im);
        phi = protect_double_update(cabs1(vre[j - 1], vim[j - 1]), cabs1(yre[j], yim[j]),
                                    cabs1(hd.re, hd.im), cabs1(yre[j], yim[j]),
                                    cabs1(yre[j - 1], yim[j - 1]), is);
        const double a2 = sc_value(phi, is);
        if (a2 != 1.0) { cn->solr++; ynorm = a2 * ynorm; }
        c_scale(b, yre, yim, a2);
        *beta = sc_combine(*beta, phi, is);
        {
            const hcplx yj = cmk(yre[j], yim[j]);
            const hcplx yc = cscal(c[j], yj), ys = cmulc(sg, yj);
            hcplx t = cfnma(yc, cmk(vre[j - 1], vim[j - 1]), cmk(yre[j - 1], yim[j - 1]));
            t = cfma(ys, hd, t);
            yre[j - 1] = t.re;
            yim[j - 1] = t.im;
        }

        /* y(0:j-2), protected by the tile norm (solve-task.c:92-100). */
        phi = protect_double_update(vnorm, cabs1(yre[j], yim[j]), Hnorm,
                                    cabs1(yre[j], yim[j]), ynorm, is);
        const double a3 = sc_value(phi, is);
        if (a3 != 1.0) cn->solr++;
        c_scale(b, yre, yim, a3);
        *beta = sc_combine(*beta, phi, is);
        {
            const hcplx yj = cmk(yre[j], yim[j]);
            const hcplx yc = cscal(c[j], yj), ys = cmulc(sg, yj);
            for (int i = 0; i < j - 1; i++) {
                hcplx t = cfnma(yc, cmk(vre[i], vim[i]), cmk(yre[i], yim[i]));
                t = cfmar(ys, HH(l + i, l + j - 1), t);
                yre[i] = t.re;
                yim[i] = t.im;
            }
        }

        /* Next annihilation column (solve-task.c:105-108): c H(:,j-1) + sigma v. */
        {
            const hcplx sv = cmul(sg, cmk(vre[j - 1], vim[j - 1]));
            vre[j - 1] = fma(c[j], hd.re, sv.re);
            vim[j - 1] = fma(c[j], hd.im, sv.im);
        }
        for (int i = 0; i < j - 1; i++) {
            const hcplx sv = cmul(sg, cmk(vre[i], vim[i]));
            vre[i] = fma(c[j], HH(l + i, l + j - 1), sv.re);
            vim[i] = sv.im;
        }
    }

    double v0r = vre[0], v0i = vim[0];
    if (J > 0) {
        /* Final rotation with the entry left of the tile (reduce.c:53-61). */
        const double hleft = HH(l, l - 1);
        if (hleft != 0) {
            hsro_cgivens(v0r, v0i, hleft, &c[0], &sr[0], &si[0]);
        } else {
            c[0] = 1.0; sr[0] = 0.0; si[0] = 0.0;
        }
        const double nr = fma(v0r, c[0], -(hleft * sr[0]));
        const double ni = fma(v0i, c[0], hleft * si[0]);
        v0r = nr;
        v0i = ni;
    }
    phi = sc_one(is);
    {
        const int p0 = hsro_csolve_1x1(smin, v0r, v0i, 0.0, 0.0, &yre[0], &yim[0], &phi, is);
        info |= p0;
        cn->pert += p0;
    }
    const double a = sc_value(phi, is);
    if (a != 1.0) cn->divr++;
    *beta = sc_combine(*beta, phi, is);
    c_scale(b - 1, yre + 1, yim + 1, a);
    return info;
}

/* ------------------------------------------------------------------------ */
/* Crossover propagation of tile J's rotations into tile I < J, prefix-      */
/* product form: R := H(I, J^-) w + pi R, w_q = c_q prod_{p<q} sigma_p      */
/* (reduceOffdiagBlocked, reduce.c:73-143).                                  */
/* ------------------------------------------------------------------------ */
static void coffdiag_reduce(const prob_t *P, int I, int J, hcplx mu, const double *c,
                            const double *sr, const double *si, double *rre, double *rim,
                            double *wre, double *wim)
{
    const int m = P->fr[I + 1] - P->fr[I];
    const int nc = P->fr[J + 1] - P->fr[J];
    const int r0 = P->fr[I], c0 = P->fr[J] - 1;
    hcplx pk = cmk(1.0, 0.0);
    for (int k = 0; k < nc; k++) {
        const hcplx w = cscal(c[k], pk);
        wre[k] = w.re;
        wim[k] = w.im;
        pk = cmul(pk, cmk(sr[k], si[k]));
    }
    /* Per row the sums over k run in k order; columns of H outermost. */
    double ar[m], ai[m];
    for (int i = 0; i < m; i++) ar[i] = ai[i] = 0.0;
    for (int k = 0; k < nc; k++)
        for (int i = 0; i < m; i++) {
            const double h = HH(r0 + i, c0 + k);
            ar[i] = fma(h, wre[k], ar[i]);
            ai[i] = fma(h, wim[k], ai[i]);
        }
    for (int i = 0; i < m; i++) {
        const hcplx r = cfma(pk, cmk(rre[i], rim[i]), cmk(ar[i], ai[i]));
        rre[i] = r.re;
        rim[i] = r.im;
    }
    if (I == J - 1) {
        const hcplx r = cfnma(mu, cmk(wre[0], wim[0]), cmk(rre[m - 1], rim[m - 1]));
        rre[m - 1] = r.re;
        rim[m - 1] = r.im;
    }
}

/* ------------------------------------------------------------------------ */
/* Robust tile update Y(I) -= R(I, J-columns) X(J) for ns pairs              */
/* (update-task.c:16-262).  Y: pair k at columns 2k, 2k+1 (ldY).             */
/* ------------------------------------------------------------------------ */
static void ctile_update(const prob_t *P, int I, int J, int ns, const double *wr,
                         const double *wi, double *Y, int ldY, double *Yn, double *Ys,
                         const double *X, int ldX, const double *Xs, const double *c,
                         const double *sr, const double *si, const double *Rtr,
                         const double *Rti, double *zr, double *zi, double *tmp,
                         cnt_t *cn)
{
    const int is = P->is;
    const int m = P->fr[I + 1] - P->fr[I];
    const int kb = P->fr[J + 1] - P->fr[J];
    const int r0 = P->fr[I];
    const int applyShift = (I == J - 1);
    const double Hnorm = P->Hn[I + (size_t)J * P->T];
    const double *h = &HH(r0, P->fr[J] - 1);
    double *tscale = tmp, *z2n = tmp + ns;
#define YR(k) (Y + (size_t)(2 * (k)) * ldY)
#define YI(k) (Y + (size_t)(2 * (k) + 1) * ldY)
#define XR(k) (X + (size_t)(2 * (k)) * ldX)
#define XI(k) (X + (size_t)(2 * (k) + 1) * ldX)

    /* Part 0: consistent scaling (update-task.c:68-88). */
    for (int k = 0; k < ns; k++) {
        if (Xs[k] < Ys[k]) {
            const double a = sc_upscale(Xs[k], Ys[k], is);
            c_scale(m, YR(k), YI(k), a);
            Yn[k] = a * Yn[k];
            Ys[k] = Xs[k];
            cn->p0r++;
        }
    }

    /* Part 1: the column left of tile J (update-task.c:103-151). */
    const double hnrm = infnorm(m, h);
    for (int k = 0; k < ns; k++) {
        const hcplx mu = cmk(wr[k], wi[k]);
        hcplx x0 = cmk(XR(k)[0], XI(k)[0]);
        if (Ys[k] < Xs[k]) x0 = cscal(sc_upscale(Ys[k], Xs[k], is), x0);
        const hcplx q = cmulc(cmk(sr[(size_t)k * kb], si[(size_t)k * kb]), x0);
        const hcplx yt = cmk(-q.re, -q.im);
        const double alpha = hsro_protect_update(fmax(hnrm, cabs1(mu.re, mu.im)),
                                                 cabs1(yt.re, yt.im), Yn[k], is);
        const double a = sc_value(alpha, is);
        double *yr = YR(k), *yi = YI(k);
        if (a != 1.0) {
            cn->p1r++;
            const hcplx at = cscal(a, yt);
            for (int i = 0; i < m; i++) {
                yr[i] = fma(-h[i], at.re, a * yr[i]);
                yi[i] = fma(-h[i], at.im, a * yi[i]);
            }
            if (applyShift) {
                const hcplx t = cfma(mu, at, cmk(yr[m - 1], yi[m - 1]));
                yr[m - 1] = t.re;
                yi[m - 1] = t.im;
            }
        } else {
            for (int i = 0; i < m; i++) {
                yr[i] = fma(-h[i], yt.re, yr[i]);
                yi[i] = fma(-h[i], yt.im, yi[i]);
            }
            if (applyShift) {
                const hcplx t = cfma(mu, yt, cmk(yr[m - 1], yi[m - 1]));
                yr[m - 1] = t.re;
                yi[m - 1] = t.im;
            }
        }
        Ys[k] = sc_combine(Ys[k], alpha, is);
        Yn[k] = cinfnorm(m, yr, yi);
    }

    /* Part 2: rotate X(J) into Ytilde2 (update-task.c:170-198). */
    for (int k = 0; k < ns; k++) {
        double *wr_ = zr + (size_t)k * kb, *wi_ = zi + (size_t)k * kb;
        const double *xr = XR(k), *xi = XI(k);
        const double *ck = c + (size_t)k * kb, *srk = sr + (size_t)k * kb, *sik = si + (size_t)k * kb;
        const double a = (Ys[k] < Xs[k]) ? sc_upscale(Ys[k], Xs[k], is) : 1.0;
        const int scaled = Ys[k] < Xs[k];
        hcplx z = scaled ? cscal(a, cmk(xr[0], xi[0])) : cmk(xr[0], xi[0]);
        z = cscal(ck[0], z);
        for (int q = 1; q < kb; q++) {
            const hcplx t2 = scaled ? cscal(a, cmk(xr[q], xi[q])) : cmk(xr[q], xi[q]);
            const hcplx s = cmk(srk[q], sik[q]);
            const hcplx out = crot_out(ck[q], s, z, t2);
            z = crot_next(ck[q], s, z, t2);
            wr_[q - 1] = out.re;
            wi_[q - 1] = out.im;
        }
        wr_[kb - 1] = z.re;
        wi_[kb - 1] = z.im;
        z2n[k] = cinfnorm(kb, wr_, wi_);
    }

    /* Bounds (update-task.c:206-226). */
    int status = 0;
    for (int k = 0; k < ns; k++) {
        tscale[k] = hsro_protect_update(Hnorm, z2n[k], Yn[k], is);
        if (sc_value(tscale[k], is) != 1.0) status = 1;
    }
    if (status) {
        for (int k = 0; k < ns; k++) {
            const double a = sc_value(tscale[k], is);
            if (a != 1.0) cn->p2r++;
            c_scale(kb, zr + (size_t)k * kb, zi + (size_t)k * kb, a);
            c_scale(m, YR(k), YI(k), a);
            Ys[k] = sc_combine(Ys[k], tscale[k], is);
        }
    }

    /* Y -= H(I, J .. J+kb-2) Ytilde2(0:kb-2), then the rank-1 term with the
     * crossover column (update-task.c:233-243). */
    const double *Hs = &HH(r0, P->fr[J]);
    double ar[m], ai[m];
    for (int k = 0; k < ns; k++) {
        const double *wr_ = zr + (size_t)k * kb, *wi_ = zi + (size_t)k * kb;
        const double *rtr = Rtr + (size_t)k * m, *rti = Rti + (size_t)k * m;
        double *yr = YR(k), *yi = YI(k);
        const hcplx zl = cmk(wr_[kb - 1], wi_[kb - 1]);
        /* Per row the sums over q run in q order; columns of H outermost. */
        for (int i = 0; i < m; i++) ar[i] = ai[i] = 0.0;
        for (int q = 0; q < kb - 1; q++) {
            const double *hq = Hs + (size_t)q * P->ldH;
            for (int i = 0; i < m; i++) {
                ar[i] = fma(hq[i], wr_[q], ar[i]);
                ai[i] = fma(hq[i], wi_[q], ai[i]);
            }
        }
        for (int i = 0; i < m; i++) {
            hcplx t = cmk(yr[i] - ar[i], yi[i] - ai[i]);
            t = cfnma(cmk(rtr[i], rti[i]), zl, t);
            yr[i] = t.re;
            yi[i] = t.im;
        }
        Yn[k] = cinfnorm(m, yr, yi);
    }
#undef YR
#undef YI
#undef XR
#undef XI
}

/* ------------------------------------------------------------------------ */
/* 2-norm with three accumulators, fused squares (shifted_Hessenberg_solve.c */
/* :135-229).                                                                */
/* ------------------------------------------------------------------------ */
static inline void cnrm3_add(nrm3_t *a, double x)
{
    const double ax = fabs(x);
    if (ax > NRM_TBIG) { const double t = ax * NRM_SBIG; a->abig = fma(t, t, a->abig); }
    else if (ax < NRM_TSML) { const double t = ax * NRM_SSML; a->asml = fma(t, t, a->asml); }
    else a->amed = fma(ax, ax, a->amed);
}

/* ------------------------------------------------------------------------ */
/* One tile of ns pairs through the sweep, the reconciliation, the back-     */
/* transform, the norm, the convergence test and the normalisation           */
/* (shifted_Hessenberg_solve.c:43-394, reduce.c:201-356).                    */
/*   vr: n x 2ns (ldvr), pair k at columns 2k, 2k+1                          */
/*   vrn: bounds [T][ns] in/out; vrn[0][k] gets the convergence flag        */
/* ------------------------------------------------------------------------ */
typedef struct {
    double *Rr, *Ri, *C, *Sr, *Si, *scales, *zr, *zi, *tmp, *vre, *vim, *wre, *wim;
} cws_t;

static void cshift_tile(const prob_t *P, int ns, const double *wr, const double *wi,
                        double *vr, int ldvr, double *vrn, double *sc_out,
                        unsigned char *pert, cws_t *w, cnt_t *cn)
{
    const int n = P->n, T = P->T, is = P->is;
    const int *fr = P->fr;
#define RR(I) (w->Rr + (size_t)fr[I] * ns)
#define RI(I) (w->Ri + (size_t)fr[I] * ns)
#define CT(I) (w->C + (size_t)fr[I] * ns)
#define SRT(I) (w->Sr + (size_t)fr[I] * ns)
#define SIT(I) (w->Si + (size_t)fr[I] * ns)
#define SC(I) (w->scales + (size_t)(I) * ns)
#define VRN(I) (vrn + (size_t)(I) * ns)
#define YRE(I, k) (vr + (size_t)fr[I] + (size_t)(2 * (k)) * ldvr)
#define YIM(I, k) (vr + (size_t)fr[I] + (size_t)(2 * (k) + 1) * ldvr)

    for (int i = 0; i < T * ns; i++) w->scales[i] = sc_one(is);
    memset(w->C, 0, (size_t)n * ns * sizeof(double));
    memset(w->Sr, 0, (size_t)n * ns * sizeof(double));
    memset(w->Si, 0, (size_t)n * ns * sizeof(double));

    /* Initial crossover columns: H(:, n-1) - mu e_n (reduce.c:276-308). */
    for (int I = 0; I < T; I++) {
        const int m = fr[I + 1] - fr[I];
        for (int k = 0; k < ns; k++) {
            double *rr = RR(I) + (size_t)k * m, *ri = RI(I) + (size_t)k * m;
            for (int i = 0; i < m; i++) {
                rr[i] = HH(fr[I] + i, n - 1);
                ri[i] = 0.0;
            }
            if (I == T - 1) {
                rr[m - 1] = rr[m - 1] - wr[k];
                ri[m - 1] = -wi[k];
            }
        }
    }

    for (int J = T - 1; J >= 0; J--) {
        const int b = fr[J + 1] - fr[J];
        for (int k = 0; k < ns; k++) {
            memcpy(w->vre, RR(J) + (size_t)k * b, (size_t)b * sizeof(double));
            memcpy(w->vim, RI(J) + (size_t)k * b, (size_t)b * sizeof(double));
            const int pk = cdiag_tile(P, J, cmk(wr[k], wi[k]), w->vre, w->vim, YRE(J, k),
                                      YIM(J, k), SC(J) + k, CT(J) + (size_t)k * b,
                                      SRT(J) + (size_t)k * b, SIT(J) + (size_t)k * b, cn);
            if (pert && pk) pert[k] = 1;
        }
        if (J == 0) break;
        for (int I = J - 1; I >= 0; I--) {
            ctile_update(P, I, J, ns, wr, wi, YRE(I, 0), ldvr, VRN(I), SC(I), YRE(J, 0), ldvr,
                         SC(J), CT(J), SRT(J), SIT(J), RR(I), RI(I), w->zr, w->zi, w->tmp, cn);
        }
        for (int I = J - 1; I >= 0; I--) {
            const int m = fr[I + 1] - fr[I];
            for (int k = 0; k < ns; k++)
                coffdiag_reduce(P, I, J, cmk(wr[k], wi[k]), CT(J) + (size_t)k * b,
                                SRT(J) + (size_t)k * b, SIT(J) + (size_t)k * b,
                                RR(I) + (size_t)k * m, RI(I) + (size_t)k * m, w->wre, w->wim);
        }
    }

    for (int k = 0; k < ns; k++) {
        double smin = SC(0)[k];
        for (int I = 1; I < T; I++) smin = sc_min(smin, SC(I)[k], is);
        if (sc_out) sc_out[k] = smin;
        nrm3_t acc = {0.0, 0.0, 0.0};
        hcplx tau1 = cmk(0.0, 0.0);
        for (int I = 0; I < T; I++) {
            const int m = fr[I + 1] - fr[I];
            double *yr = YRE(I, k), *yi = YIM(I, k);
            const double *ck = CT(I) + (size_t)k * m;
            const double *srk = SRT(I) + (size_t)k * m, *sik = SIT(I) + (size_t)k * m;
            const double alpha = sc_upscale(smin, SC(I)[k], is);
            int start = 0;
            if (I == 0) {
                start = 1;
                tau1 = cscal(alpha, cmk(yr[0], yi[0]));
            }
            for (int i = start; i < m; i++) {
                const hcplx tau2 = cscal(alpha, cmk(yr[i], yi[i]));
                const hcplx s = cmk(srk[i], sik[i]);
                const hcplx out = crot_out(ck[i], s, tau1, tau2);
                tau1 = crot_next(ck[i], s, tau1, tau2);
                yr[i - 1] = out.re;
                yi[i - 1] = out.im;
                cnrm3_add(&acc, out.re);
                cnrm3_add(&acc, out.im);
            }
        }
        vr[(size_t)(n - 1) + (size_t)(2 * k) * ldvr] = tau1.re;
        vr[(size_t)(n - 1) + (size_t)(2 * k + 1) * ldvr] = tau1.im;
        cnrm3_add(&acc, tau1.re);
        cnrm3_add(&acc, tau1.im);
        const double ynrm = nrm3_finish(acc);
        if (!(ynrm > 0.1 / sqrt(n))) {
            VRN(0)[k] = 0.0;
        } else {
            double *yr = vr + (size_t)(2 * k) * ldvr, *yi = vr + (size_t)(2 * k + 1) * ldvr;
            for (int i = 0; i < n; i++) { yr[i] /= ynrm; yi[i] /= ynrm; }
            VRN(0)[k] = 1.0;
        }
    }
#undef RR
#undef RI
#undef CT
#undef SRT
#undef SIT
#undef SC
#undef VRN
#undef YRE
#undef YIM
}

/* All pairs [0, np) in shift tiles of rhs_tlsz pairs (OpenMP over tiles). */
static int csolve_all(const prob_t *P, int np, const double *wr, const double *wi,
                      double *vr, int ldvr, double *vrnorms, int rhs_tlsz,
                      unsigned char *pert, double *colscale, cnt_t *total)
{
    const int n = P->n, T = P->T;
    const int ntiles = (np + rhs_tlsz - 1) / rhs_tlsz;
    int bmax = 0;
    for (int I = 0; I < T; I++)
        if (P->fr[I + 1] - P->fr[I] > bmax) bmax = P->fr[I + 1] - P->fr[I];
    int err = 0;
#pragma omp parallel
    {
        cnt_t cn = {0, 0, 0, 0, 0, 0};
        cws_t w;
        const size_t smax = (size_t)rhs_tlsz;
        w.Rr = (double *)malloc(sizeof(double) * (size_t)n * smax);
        w.Ri = (double *)malloc(sizeof(double) * (size_t)n * smax);
        w.C = (double *)malloc(sizeof(double) * (size_t)n * smax);
        w.Sr = (double *)malloc(sizeof(double) * (size_t)n * smax);
        w.Si = (double *)malloc(sizeof(double) * (size_t)n * smax);
        w.scales = (double *)malloc(sizeof(double) * (size_t)T * smax);
        w.zr = (double *)malloc(sizeof(double) * (size_t)bmax * smax);
        w.zi = (double *)malloc(sizeof(double) * (size_t)bmax * smax);
        w.tmp = (double *)malloc(sizeof(double) * 2 * smax);
        w.vre = (double *)malloc(sizeof(double) * (size_t)bmax);
        w.vim = (double *)malloc(sizeof(double) * (size_t)bmax);
        w.wre = (double *)malloc(sizeof(double) * (size_t)bmax);
        w.wim = (double *)malloc(sizeof(double) * (size_t)bmax);
        double *vrn = (double *)malloc(sizeof(double) * (size_t)T * smax);
        const int ok = w.Rr && w.Ri && w.C && w.Sr && w.Si && w.scales && w.zr && w.zi &&
                       w.tmp && w.vre && w.vim && w.wre && w.wim && vrn;
        if (!ok) {
#pragma omp atomic write
            err = -2;
        }
#pragma omp for schedule(dynamic, 1)
        for (int q = 0; q < ntiles; q++) {
            if (!ok) continue;
            const int k0 = q * rhs_tlsz;
            const int ns = np - k0 < rhs_tlsz ? np - k0 : rhs_tlsz;
            for (int I = 0; I < T; I++)
                for (int k = 0; k < ns; k++)
                    vrn[(size_t)I * ns + k] = vrnorms[(size_t)(k0 + k) + (size_t)I * np];
            cshift_tile(P, ns, wr + k0, wi + k0, vr + (size_t)(2 * k0) * ldvr, ldvr, vrn,
                        colscale ? colscale + k0 : NULL, pert ? pert + k0 : NULL, &w, &cn);
            for (int I = 0; I < T; I++)
                for (int k = 0; k < ns; k++)
                    vrnorms[(size_t)(k0 + k) + (size_t)I * np] = vrn[(size_t)I * ns + k];
        }
        free(w.Rr); free(w.Ri); free(w.C); free(w.Sr); free(w.Si); free(w.scales);
        free(w.zr); free(w.zi); free(w.tmp); free(w.vre); free(w.vim); free(w.wre);
        free(w.wim); free(vrn);
#pragma omp critical
        {
            total->pert += cn.pert; total->divr += cn.divr; total->solr += cn.solr;
            total->p1r += cn.p1r; total->p2r += cn.p2r; total->p0r += cn.p0r;
        }
    }
    return err;
}

int hsro_inverse_iteration_cplx(int n, const double *H, int ldH, int npairs,
                                const double *wr, const double *wi, int tlsz,
                                int rhs_tlsz, double *vr, int ldvr, int intscale,
                                int max_restarts, unsigned char *perturbed,
                                double *colscale, int *status, hsro_stats *stats)
{
    if (n <= 0 || ldH < n || npairs < 0 || tlsz <= 0 || tlsz % 4 != 0 ||
        rhs_tlsz <= 0 || ldvr < n || !H || (npairs && (!wr || !wi || !vr)))
        return -1;
    if (stats) memset(stats, 0, sizeof(*stats));
    if (npairs == 0) return 0;
#ifdef HSRO_BLAS_THREADS
    HSRO_BLAS_THREADS(1);
#endif
    prob_t P;
    int *fr = NULL;
    if (setup(&P, n, H, ldH, tlsz, intscale, &fr) != 0) return -2;
    const int T = P.T;
    cnt_t total = {0, 0, 0, 0, 0, 0};
    const double eps3 = hsro_dlange_inf(n, n, H, ldH) * (DBL_EPSILON / 2);
    double *vrnorms = (double *)malloc(sizeof(double) * (size_t)T * npairs);
    int *conv = (int *)malloc(sizeof(int) * (size_t)npairs);
    int *idx = (int *)malloc(sizeof(int) * (size_t)npairs);
    if (!vrnorms || !conv || !idx) {
        free(vrnorms); free(conv); free(idx); free(fr); free((void *)P.Hn);
        return -2;
    }
    if (perturbed) memset(perturbed, 0, (size_t)npairs);

    /* Start vector: eps3 in the real part (inverse_iteration.c:19-34). */
    for (int k = 0; k < npairs; k++)
        for (int i = 0; i < n; i++) {
            vr[(size_t)i + (size_t)(2 * k) * ldvr] = eps3;
            vr[(size_t)i + (size_t)(2 * k + 1) * ldvr] = 0.0;
        }
    for (int i = 0; i < T * npairs; i++) vrnorms[i] = eps3;
    int rc = csolve_all(&P, npairs, wr, wi, vr, ldvr, vrnorms, rhs_tlsz, perturbed,
                        colscale, &total);
    for (int k = 0; k < npairs; k++) conv[k] = vrnorms[k] != 0.0;

    /* Restarts in place: the pairs that did not converge are solved again
     * with the dlaein-style start vector of round `its`
     * (inverse_iteration.c:36-57), their positions unchanged. */
    const int max_its = max_restarts < 0 ? n : (max_restarts < n ? max_restarts : n);
    long restarts = 0;
    for (int its = 0; rc == 0 && its < max_its; its++) {
        int m = 0;
        for (int k = 0; k < npairs; k++)
            if (!conv[k]) idx[m++] = k;
        if (m == 0) break;
        double *swr = (double *)malloc(sizeof(double) * (size_t)m);
        double *swi = (double *)malloc(sizeof(double) * (size_t)m);
        double *svr = (double *)malloc(sizeof(double) * (size_t)n * 2 * m);
        double *svn = (double *)malloc(sizeof(double) * (size_t)T * m);
        unsigned char *sp = (unsigned char *)calloc((size_t)m, 1);
        double *ssc = (double *)malloc(sizeof(double) * (size_t)m);
        if (!swr || !swi || !svr || !svn || !sp || !ssc) {
            free(swr); free(swi); free(svr); free(svn); free(sp); free(ssc);
            rc = -2;
            break;
        }
        const double tmp = eps3 / (sqrt(n) + 1.0);
        const double ub = fmax(fmax(eps3, tmp), fabs(tmp - eps3 / sqrt(n)));
        for (int q = 0; q < m; q++) {
            swr[q] = wr[idx[q]];
            swi[q] = wi[idx[q]];
            double *v = svr + (size_t)(2 * q) * n, *vi = v + n;
            v[0] = eps3;
            for (int i = 1; i < n; i++) v[i] = tmp;
            v[n - 1 - its] -= eps3 * sqrt(n);
            for (int i = 0; i < n; i++) vi[i] = 0.0;
        }
        for (int i = 0; i < T * m; i++) svn[i] = ub;
        rc = csolve_all(&P, m, swr, swi, svr, n, svn, rhs_tlsz, sp, ssc, &total);
        for (int q = 0; q < m; q++) {
            const int k = idx[q];
            memcpy(vr + (size_t)(2 * k) * ldvr, svr + (size_t)(2 * q) * n, sizeof(double) * (size_t)n);
            memcpy(vr + (size_t)(2 * k + 1) * ldvr, svr + (size_t)(2 * q + 1) * n, sizeof(double) * (size_t)n);
            conv[k] = svn[q] != 0.0;
            if (perturbed) perturbed[k] = sp[q];
            if (colscale) colscale[k] = ssc[q];
        }
        free(swr); free(swi); free(svr); free(svn); free(sp); free(ssc);
        restarts++;
    }
    int nonconv = 0;
    for (int k = 0; k < npairs; k++) {
        if (status) status[k] = conv[k];
        nonconv += !conv[k];
    }
    stats_out(stats, &total);
    if (stats) { stats->restarts = restarts; stats->nonconverged = nonconv; }
    free(vrnorms); free(conv); free(idx); free(fr); free((void *)P.Hn);
    return rc;
}
