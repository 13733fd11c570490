/*
 * ref_shim.c -- decision recorder linked around the unmodified reference.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/build.py links the reference's own object
 * files with -Wl,--wrap for the robust kernels that the task kernels call
 * across translation units (solve-task.c -> solve_1x1_real_system,
 * protect_double_update; update-task.c -> protect_update,
 * protect_multi_rhs_update_real).  Each wrapper calls the reference's own
 * routine (__real_*) and records the decision it returned, so the parity
 * tests can compare the reference's overflow-protection decisions with the
 * oracle's and the CUDA library's.  No reference source is copied here.
 */
#include <stdatomic.h>
#include <string.h>

#ifdef SHIM_INTSCALING
typedef int scaling_t;
#define ONE 0
#else
typedef double scaling_t;
#define ONE 1.0
#endif

enum { EV_PERTURB = 1, EV_DIV_RESCALE = 2, EV_SOLVE_RESCALE = 3,
       EV_PART1_RESCALE = 4, EV_PART2_RESCALE = 5 };

#define MAX_EVENTS (1 << 20)
static atomic_long g_counts[8];
static atomic_long g_nev;
static double g_ev_key[MAX_EVENTS];
static double g_ev_val[MAX_EVENTS];
static int g_ev_kind[MAX_EVENTS];

static void record(int kind, double key, double val)
{
    atomic_fetch_add(&g_counts[kind], 1);
    const long i = atomic_fetch_add(&g_nev, 1);
    if (i < MAX_EVENTS) {
        g_ev_key[i] = key;
        g_ev_val[i] = val;
        g_ev_kind[i] = kind;
    }
}

extern int __real_solve_1x1_real_system(double smin, double t, double lambda,
                                        double *x, scaling_t *scale);
int __wrap_solve_1x1_real_system(double smin, double t, double lambda,
                                 double *x, scaling_t *scale)
{
    const int info = __real_solve_1x1_real_system(smin, t, lambda, x, scale);
    atomic_fetch_add(&g_counts[0], 1);
    if (info) record(EV_PERTURB, smin, (double)info);
    if (*scale != ONE) record(EV_DIV_RESCALE, smin, (double)*scale);
    return info;
}

extern scaling_t __real_protect_double_update(double t1, double x1, double t2,
                                              double x2, double y);
scaling_t __wrap_protect_double_update(double t1, double x1, double t2,
                                       double x2, double y)
{
    const scaling_t a = __real_protect_double_update(t1, x1, t2, x2, y);
    if (a != ONE) record(EV_SOLVE_RESCALE, y, (double)a);
    return a;
}

extern scaling_t __real_protect_update(double t, double x, double y);
scaling_t __wrap_protect_update(double t, double x, double y)
{
    const scaling_t a = __real_protect_update(t, x, y);
    if (a != ONE) record(EV_PART1_RESCALE, t, (double)a);
    return a;
}

extern int __real_protect_multi_rhs_update_real(const double *Xnorms, int num_rhs,
                                                double tnorm, const double *Ynorms,
                                                scaling_t *scales);
int __wrap_protect_multi_rhs_update_real(const double *Xnorms, int num_rhs,
                                         double tnorm, const double *Ynorms,
                                         scaling_t *scales)
{
    const int st = __real_protect_multi_rhs_update_real(Xnorms, num_rhs, tnorm,
                                                        Ynorms, scales);
    for (int k = 0; k < num_rhs; k++)
        if (scales[k] != ONE) record(EV_PART2_RESCALE, tnorm, (double)scales[k]);
    return st;
}

/* Control API (ctypes). */
void hsr_ref_shim_reset(void)
{
    for (int i = 0; i < 8; i++) atomic_store(&g_counts[i], 0);
    atomic_store(&g_nev, 0);
}

/* out[0] = 1x1 solves, out[1..5] = events by kind. */
void hsr_ref_shim_counts(long *out)
{
    for (int i = 0; i < 6; i++) out[i] = atomic_load(&g_counts[i]);
}

long hsr_ref_shim_events(int *kind, double *key, double *val, long max)
{
    long n = atomic_load(&g_nev);
    if (n > MAX_EVENTS) n = MAX_EVENTS;
    if (n > max) n = max;
    memcpy(kind, g_ev_kind, sizeof(int) * (size_t)n);
    memcpy(key, g_ev_key, sizeof(double) * (size_t)n);
    memcpy(val, g_ev_val, sizeof(double) * (size_t)n);
    return n;
}

extern void scipy_openblas_set_num_threads(int);
void hsr_ref_set_blas_threads(int n) { scipy_openblas_set_num_threads(n); }
