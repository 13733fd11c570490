/*
 * hsro.h -- CPU oracle for hsrq3in's robust level-3 inverse iteration.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm (tiled Givens RQ of H - mu*I, overflow-protected tiled
 * back-substitution, level-3 tile updates, scale reconciliation and
 * normalisation).  It is used as the checker in tests/, by smoke() and as the
 * timed CPU port in bench.py.  The product library never links, loads or
 * calls it.
 *
 * Every routine cites the reference file:line it restates.  Two arithmetic
 * modes are compiled from the same source:
 *   - "ref" (default, built with -ffp-contract=off): every expression is
 *     evaluated exactly as the reference's C source spells it, so the result
 *     is bit-identical to the reference compiled with the same flags and the
 *     same dgemm;
 *   - "fma" (-DHSRO_FMA): the expression shapes of the CUDA kernels (fused
 *     multiply-adds where the kernels fuse them, prefix-product coefficients
 *     for the crossover-column propagation, an ordered dot product in place of
 *     dgemm), so that single-tile problems agree bit for bit with the device.
 */
#ifndef HSRO_H
#define HSRO_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct hsro_stats {
    long perturbations;   /* solve_1x1 calls that lifted |t-lambda| to smin   */
    long div_rescales;    /* solve_1x1 calls whose scale factor was != 1     */
    long solve_rescales;  /* protect_double_update in diagonal solves != 1   */
    long part1_rescales;  /* tile_update Part 1 protect_update != 1          */
    long part2_rescales;  /* tile_update Part 2 per-column factors != 1      */
    long consistency_rescales; /* tile_update Part 0 Y rescales            */
    long restarts;        /* restart rounds with a new starting vector      */
    int  nonconverged;    /* columns not converged on exit                  */
} hsro_stats;

/* Drop-in twin of tiled_inverse_iteration (inverse_iteration.h:19-22).
 *   intscale   0: scaling factors are doubles (the reference default build);
 *              1: scaling factors are base-2 exponents (-DINTSCALING).
 *   perturbed  optional [nrhs]: 1 where any 1x1 solve of that column was
 *              perturbed (robust.c:432-435), else 0.
 *   colscale   optional [nrhs]: the reconciled scaling factor smin of each
 *              column (robust.c:58-82) before normalisation, as a double
 *              (an exponent in intscale mode).
 *   status     optional [nrhs]: 1 converged, 0 not converged.
 *   stats      optional counters.
 * Returns 0 on success, <0 on invalid arguments or allocation failure.      */
int hsro_inverse_iteration(int n, const double *H, int ldH,
                           int nrhs, double *wr, int tlsz, int rhs_tlsz,
                           double *vr, int ldvr, int intscale,
                           unsigned char *perturbed, double *colscale,
                           int *status, hsro_stats *stats);

/* Same as above, but the right-hand sides are supplied by the caller in vr
 * (one solve, no convergence restart, no normalisation skipped).  Used by
 * the _ex parity tests with uniform[0,1] right-hand sides.                  */
int hsro_solve_rhs(int n, const double *H, int ldH,
                   int nrhs, const double *wr, int tlsz, int rhs_tlsz,
                   double *vr, int ldvr, int intscale,
                   unsigned char *perturbed, double *colscale,
                   int *status, hsro_stats *stats);

/* LAPACK-3.10-style Givens rotation (dlartg, Anderson 2017), transposed as
 * in reduce.c:14-24: [c s; -s c]^T convention, s negated.                   */
void hsro_givens(double f, double g, double *c, double *s);
/* Plain dlartg (not negated), exposed for pinning against LAPACK.           */
void hsro_dlartg(double f, double g, double *c, double *s, double *r);
/* dlange('I') restated (row-sum order of LAPACK).                           */
double hsro_dlange_inf(int m, int n, const double *A, int ldA);

/* Robust scalar kernels, real subset of robust.c, exposed for unit tests.   */
double hsro_protect_update(double t, double x, double y, int intscale);
int    hsro_solve_1x1(double smin, double t, double lambda, double *x,
                      double *scale, int intscale);

/* ---- Complex-conjugate shifts (hsro_cplx.c) ---------------------------- */
/* Eigenvectors for npairs complex shifts mu_k = wr[k] + i*wi[k].  vr is
 * n x 2*npairs (ldvr): pair k's vector has its real part in column 2k and its
 * imaginary part in column 2k+1 (the LAPACK dhsein layout), unit 2-norm.
 * Pairs that do not converge are solved again in place, up to max_restarts
 * rounds (< 0: n).  perturbed/colscale/status are per pair.                 */
int hsro_inverse_iteration_cplx(int n, const double *H, int ldH, int npairs,
                                const double *wr, const double *wi, int tlsz,
                                int rhs_tlsz, double *vr, int ldvr, int intscale,
                                int max_restarts, unsigned char *perturbed,
                                double *colscale, int *status, hsro_stats *stats);
/* Complex Givens rotation of (f_re + i f_im, g): c, sigma = sr + i si with
 * sigma f + c g = 0.                                                        */
void hsro_cgivens(double fr, double fi, double g, double *c, double *sr, double *si);
/* robust_cmplx_div (robust.c:639-675) restated. */
int hsro_robust_cmplx_div(double smin, double a, double b, double c, double d,
                          double *xr, double *xi, double *scale, int intscale);
/* x := (scale x) / (t - l), complex t and l (solve_1x1_cmplx_system,
 * robust.c:677-773, for t real).                                            */
int hsro_csolve_1x1(double smin, double tr, double ti, double lr, double li,
                    double *xr, double *xi, double *scale, int intscale);

/* Pivot log for the decision tests: while buf is set, hsro_inverse_iteration
 * stores in buf[k] (nrhs entries) the smallest |t - lambda| / smin over the
 * 1x1 solves of output column k (< 1 where the solve was perturbed).  NULL
 * switches it off.  Not thread-safe across concurrent calls.               */
void hsro_set_pivot_log(double *buf);

/* Number of OpenMP threads the oracle may use (0 = runtime default).        */
void hsro_set_threads(int nthreads);
/* Arithmetic mode the library was compiled for: 0 ref, 1 fma.              */
int  hsro_mode(void);

#ifdef __cplusplus
}
#endif
#endif
