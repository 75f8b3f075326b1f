/*
 * CPU oracle (TEST INFRASTRUCTURE ONLY) -- see oracle.h.
 *
 * Compiled with -O2 -ffp-contract=off so that every + - * / is a separately
 * rounded IEEE double operation, in the order written in the reference.
 *
 * Reference files followed (paths within the NumbaCS project):
 *   src/numbacs/flows.py:1146-1158     double gyre RHS, defaults :1162-1172
 *   src/numbacs/flows.py:1182-1213     Bickley jet RHS, defaults :1217-1238
 *   src/numbacs/flows.py:9-46          get_interp_arrays_2D (cubic prefilter)
 *   src/numbacs/flows.py:154-254       get_flow_2D RHS (planar / spherical 1 / 2)
 *   src/numbacs/integration.py:123-182 flowmap_grid_2D (t_eval scaling, mask, loop)
 *   src/numbacs/diagnostics.py:21-65   ftle_grid_2D (+ utils.py:41-44, :185-189)
 *   src/numbacs/diagnostics.py:200-269 C_eig_2D, ftle_from_eig
 *   src/numbacs/extraction/ridges.py:9-154 ftle_ridge_pts / _ftle_ridges
 *
 * Third-party algorithms restated (not present in the reference tree):
 *   numbalsoda.dop853 -- Hairer & Wanner's dop853 (Dormand-Prince 8(5,3) with
 *     the dop853 step-size controller and HINIT initial step, default
 *     constants safe=0.9, fac1=0.333, fac2=6, beta=0, uround=2.3e-16);
 *   interpolation (EconForge) >= 2.2.6 prefilter/eval_spline -- uniform cubic
 *     B-spline with natural (zero second derivative) boundary conditions;
 *   numba's np.percentile -- rank = 1 + (n-1)*q/100, value
 *     lower*(1-m) + upper*m of the two bracketing order statistics.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../numbacs_gb300/csrc/dop853_tableau.h"
#include "../numbacs_gb300/csrc/detmath.h"

#define PI_D 3.141592653589793

/* ------------------------------------------------------------------ flows */

/* Python float modulo (result has the sign of the divisor). */
static double py_fmod(double a, double b)
{
    double m = fmod(a, b);
    if (m != 0.0) {
        if ((b < 0.0) != (m < 0.0)) m += b;
    } else {
        m = copysign(0.0, b);
    }
    return m;
}

/* flows.py:1146-1158 */
static void rhs_double_gyre(double t, const double* y, double* dy, const double* p)
{
    double tt = p[0] * t;
    double a = p[2] * sin(p[4] * tt + p[5]);
    double b = 1.0 - 2.0 * a;
    double f = a * (y[0] * y[0]) + b * y[0];
    double df = 2.0 * a * y[0] + b;
    dy[0] = p[0] * (-PI_D * p[1] * sin(PI_D * f) * cos(PI_D * y[1]) - p[3] * y[0]);
    dy[1] = p[0] * (PI_D * p[1] * cos(PI_D * f) * sin(PI_D * y[1]) * df - p[3] * y[1]);
}

/* flows.py:1182-1213 */
static void rhs_bickley(double t, const double* y, double* dy, const double* p)
{
    double tt = p[0] * t;
    double Y = y[1] / p[2];
    double ch = cosh(Y);
    double sech2 = 1.0 / (ch * ch);
    double s1 = y[0] - p[9] * tt, s2 = y[0] - p[10] * tt, s3 = y[0] - p[11] * tt;
    dy[0] = p[0] * (p[1] * sech2
                    + 2.0 * p[1] * tanh(Y) * sech2
                          * (p[3] * cos(p[6] * s1) + p[4] * cos(p[7] * s2) + p[5] * cos(p[8] * s3)));
    dy[1] = -p[0] * (p[1] * p[2] * sech2
                     * (p[3] * p[6] * sin(p[6] * s1) + p[4] * p[7] * sin(p[7] * s2)
                        + p[5] * p[8] * sin(p[8] * s3)));
}

/* uniform cubic B-spline basis at fractional offset t (rows of the
 * standard B-spline matrix applied to [t^3, t^2, t, 1]) */
static void bspline_weights(double t, double w[4])
{
    double t3 = t * t * t, t2 = t * t;
    w[0] = (-1.0 / 6.0) * t3 + (3.0 / 6.0) * t2 + (-3.0 / 6.0) * t + (1.0 / 6.0);
    w[1] = (3.0 / 6.0) * t3 + (-6.0 / 6.0) * t2 + (0.0 / 6.0) * t + (4.0 / 6.0);
    w[2] = (-3.0 / 6.0) * t3 + (3.0 / 6.0) * t2 + (3.0 / 6.0) * t + (1.0 / 6.0);
    w[3] = (1.0 / 6.0) * t3 + (0.0 / 6.0) * t2 + (0.0 / 6.0) * t + (0.0 / 6.0);
}

/* derivative of the basis with respect to the offset t (the rows above
 * differentiated: [3t^2, 2t, 1] times the t^3, t^2, t coefficients) */
static void bspline_dweights(double t, double w[4])
{
    double t2 = t * t;
    w[0] = (-3.0 / 6.0) * t2 + (6.0 / 6.0) * t + (-3.0 / 6.0);
    w[1] = (9.0 / 6.0) * t2 + (-12.0 / 6.0) * t + (0.0 / 6.0);
    w[2] = (-9.0 / 6.0) * t2 + (6.0 / 6.0) * t + (3.0 / 6.0);
    w[3] = (3.0 / 6.0) * t2 + (0.0 / 6.0) * t + (0.0 / 6.0);
}

/* cell index and fractional offset along one axis (a, b, n) of a coordinate
 * on or inside [a, b]; a NaN coordinate takes cell 0 (and a NaN offset) */
static int spline_locate(double a, double b, int n, double x, double* t)
{
    double dinv = (double)(n - 1) / (b - a);
    double u = (x - a) * dinv;
    double fu = floor(u);
    int i;
    if (fu > (double)(n - 2)) i = n - 2;
    else if (!(fu >= 0.0)) i = 0;
    else i = (int)fu;
    *t = u - (double)i;
    return i;
}

/* sum_a w0[a] sum_b w1[b] sum_c w2[c] C[it+a, ix+b, iy+c] */
static double spline_sum(const double* c, int st, int sx, int it, int ix, int iy,
                         const double* w0, const double* w1, const double* w2)
{
    double acc = 0.0;
    for (int a = 0; a < 4; ++a) {
        double sa = 0.0;
        for (int b = 0; b < 4; ++b) {
            const double* row = c + (size_t)(it + a) * st + (size_t)(ix + b) * sx + iy;
            double sb = w2[0] * row[0] + w2[1] * row[1] + w2[2] * row[2] + w2[3] * row[3];
            sa += w1[b] * sb;
        }
        acc += w0[a] * sa;
    }
    return acc;
}

/* Tricubic B-spline value at (t, x, y) with the extrapolation modes of the
 * interpolation package's eval_spline (flows.py:121 passes extrap_mode
 * through unchanged):
 *   0 "constant": 0 strictly outside the grid box.  Pinned through
 *     flowmap_composition's fixtures (integration.py:630-640 evaluate
 *     eval_linear(..., xto.CONSTANT); wall points that a map leaves 1 ulp
 *     outside [0, 2] compose to 0 there); eval_spline takes the same option.
 *   1 "nearest": each coordinate clamped into its axis' [a, b], then
 *     evaluated there.
 *   2 "linear": the value at that clamped point plus, for every axis whose
 *     coordinate was clamped (t, then x, then y), the spline's derivative
 *     along that axis at the clamped point times the distance beyond the
 *     box (first-order continuation from the box surface).
 * No fixture of the reference pins modes 1 and 2; this definition is the
 * behaviour the GPU path is tested against. */
double orc_eval_spline_3d(const double* g, const double* c, int extrap,
                          double t, double x, double y)
{
    int n[3] = {(int)g[2], (int)g[5], (int)g[8]};
    int sx = n[2] + 2, st = (n[1] + 2) * (n[2] + 2);
    if (extrap == 0 && (t < g[0] || t > g[1] || x < g[3] || x > g[4] || y < g[6] || y > g[7]))
        return 0.0;
    double v[3] = {t, x, y}, cl[3], dl[3], f[3], w[3][4];
    int i[3];
    for (int d = 0; d < 3; ++d) {
        double a = g[3 * d], b = g[3 * d + 1];
        cl[d] = v[d] < a ? a : (v[d] > b ? b : v[d]);
        dl[d] = v[d] - cl[d];
        i[d] = spline_locate(a, b, n[d], cl[d], &f[d]);
        bspline_weights(f[d], w[d]);
    }
    double acc = spline_sum(c, st, sx, i[0], i[1], i[2], w[0], w[1], w[2]);
    if (extrap == 2) {
        for (int d = 0; d < 3; ++d) {
            if (dl[d] == 0.0 || dl[d] != dl[d]) continue;
            double dw[4], dinv = (double)(n[d] - 1) / (g[3 * d + 1] - g[3 * d]);
            bspline_dweights(f[d], dw);
            double gd = spline_sum(c, st, sx, i[0], i[1], i[2], d == 0 ? dw : w[0],
                                   d == 1 ? dw : w[1], d == 2 ? dw : w[2]);
            acc = acc + (dl[d] * dinv) * gd;
        }
    }
    return acc;
}

/* flows.py:154-254 */
static void rhs_spline(const orc_flow* fl, double t, const double* y, double* dy, const double* p)
{
    double tt = p[0] * t;
    if (fl->spherical == 1 || fl->spherical == 2) {
        double xx = fl->spherical == 1 ? py_fmod(y[0] - 180.0, 360.0) - 180.0 : py_fmod(y[0], 360.0);
        double yy = y[1];
        double u = orc_eval_spline_3d(fl->grid, fl->cu, fl->extrap, tt, xx, yy);
        double v = orc_eval_spline_3d(fl->grid, fl->cv, fl->extrap, tt, xx, yy);
        double cy = fl->libm ? cos(yy * PI_D / 180.0) : nbcs_cos_deg(yy);
        dy[0] = p[0] * u * 180.0 / (PI_D * fl->r * cy);
        dy[1] = p[0] * v * 180.0 / (PI_D * fl->r);
    } else {
        double u = orc_eval_spline_3d(fl->grid, fl->cu, fl->extrap, tt, y[0], y[1]);
        double v = orc_eval_spline_3d(fl->grid, fl->cv, fl->extrap, tt, y[0], y[1]);
        dy[0] = p[0] * u;
        dy[1] = p[0] * v;
    }
}

double orc_cos_deg(double d) { return nbcs_cos_deg(d); }
double orc_root8(double x) { return nbcs_root8(x); }

void orc_rhs(const orc_flow* flow, double t, const double* y, double* dy, const double* p)
{
    switch (flow->kind) {
    case ORC_FLOW_DOUBLE_GYRE: rhs_double_gyre(t, y, dy, p); break;
    case ORC_FLOW_BICKLEY: rhs_bickley(t, y, dy, p); break;
    default: rhs_spline(flow, t, y, dy, p); break;
    }
}

/* ------------------------------------------------------- spline prefilter */

/* Natural-BC interpolation along one line of n samples (stride s):
 *   c[-1] - 2c[0] + c[1] = 0,  (c[i-1] + 4c[i] + c[i+1])/6 = f[i],
 *   c[n-2] - 2c[n-1] + c[n] = 0.
 * The end rows give c[0] = f[0], c[n-1] = f[n-1]; the interior is a
 * (1,4,1) tridiagonal system solved by forward elimination / back
 * substitution.  `cw` is scratch of length n. */
static void prefilter_line(const double* f, long fs, int n, double* c, long cs, double* cw)
{
    /* c has n+2 entries, c[0] <-> node -1 */
    if (n == 1) {
        c[0] = c[cs] = c[2 * cs] = f[0];
        return;
    }
    double c0 = f[0], cn1 = f[(long)(n - 1) * fs];
    /* unknowns c_1..c_{n-2}; rhs_i = 6 f_i minus known neighbours */
    int m = n - 2;
    double* d = cw; /* modified diagonal */
    double* r = cw + n; /* modified rhs */
    for (int k = 0; k < m; ++k) {
        int i = k + 1;
        double rhs = 6.0 * f[(long)i * fs];
        if (k == 0) rhs -= c0;
        if (k == m - 1) rhs -= cn1;
        if (k == 0) {
            d[k] = 4.0;
            r[k] = rhs;
        } else {
            double w = 1.0 / d[k - 1];
            d[k] = 4.0 - w;
            r[k] = rhs - w * r[k - 1];
        }
    }
    double next = 0.0;
    for (int k = m - 1; k >= 0; --k) {
        double v = (k == m - 1) ? r[k] / d[k] : (r[k] - next) / d[k];
        c[(long)(k + 2) * cs] = v;
        next = v;
    }
    c[1 * cs] = c0;
    c[(long)n * cs] = cn1;
    double c1 = (n > 2) ? c[2 * cs] : cn1;
    double cn2 = (n > 2) ? c[(long)(n - 1) * cs] : c0;
    c[0] = 2.0 * c0 - c1;
    c[(long)(n + 1) * cs] = 2.0 * cn1 - cn2;
}

int orc_prefilter_3d(const double* f, int nt, int nx, int ny, double* coef)
{
    if (nt < 1 || nx < 1 || ny < 1) return -1;
    int NT = nt + 2, NX = nx + 2, NY = ny + 2;
    size_t nmax = (size_t)(NT > NX ? (NT > NY ? NT : NY) : (NX > NY ? NX : NY));
    double* cw = (double*)malloc(sizeof(double) * 2 * nmax);
    double* tmp = (double*)malloc(sizeof(double) * (size_t)NT * nx * ny);
    double* tmp2 = (double*)malloc(sizeof(double) * (size_t)NT * NX * ny);
    if (!cw || !tmp || !tmp2) { free(cw); free(tmp); free(tmp2); return -2; }
    /* axis t: f (nt,nx,ny) -> tmp (NT,nx,ny) */
    for (int ix = 0; ix < nx; ++ix)
        for (int iy = 0; iy < ny; ++iy)
            prefilter_line(f + (size_t)ix * ny + iy, (long)nx * ny, nt,
                           tmp + (size_t)ix * ny + iy, (long)nx * ny, cw);
    /* axis x: tmp (NT,nx,ny) -> tmp2 (NT,NX,ny) */
    for (int it = 0; it < NT; ++it)
        for (int iy = 0; iy < ny; ++iy)
            prefilter_line(tmp + (size_t)it * nx * ny + iy, ny, nx,
                           tmp2 + (size_t)it * NX * ny + iy, ny, cw);
    /* axis y: tmp2 (NT,NX,ny) -> coef (NT,NX,NY) */
    for (int it = 0; it < NT; ++it)
        for (int ix = 0; ix < NX; ++ix)
            prefilter_line(tmp2 + ((size_t)it * NX + ix) * ny, 1, ny,
                           coef + ((size_t)it * NX + ix) * NY, 1, cw);
    free(cw); free(tmp); free(tmp2);
    return 0;
}

/* ------------------------------------------------------------- DOP853 */

static double dmax(double a, double b) { return a > b ? a : b; }
static double dmin(double a, double b) { return a < b ? a : b; }
static double dsign(double a, double b) { return b >= 0.0 ? fabs(a) : -fabs(a); }

#define N2 2

/* HINIT of dop853 (initial step-size guess, iord = 8). */
static double hinit(const orc_flow* fl, const double* p, double x, const double* y,
                    double posneg, const double* f0, double* f1, double hmax,
                    double rtol, double atol)
{
    double dnf = 0.0, dny = 0.0, sk, sqr, h, der2, der12, h1, y1[N2];
    for (int i = 0; i < N2; ++i) {
        sk = atol + rtol * fabs(y[i]);
        sqr = f0[i] / sk;
        dnf += sqr * sqr;
        sqr = y[i] / sk;
        dny += sqr * sqr;
    }
    if (dnf <= 1.0e-10 || dny <= 1.0e-10) h = 1.0e-6;
    else h = sqrt(dny / dnf) * 0.01;
    h = dmin(h, hmax);
    h = dsign(h, posneg);
    for (int i = 0; i < N2; ++i) y1[i] = y[i] + h * f0[i];
    orc_rhs(fl, x + h, y1, f1, p);
    der2 = 0.0;
    for (int i = 0; i < N2; ++i) {
        sk = atol + rtol * fabs(y[i]);
        sqr = (f1[i] - f0[i]) / sk;
        der2 += sqr * sqr;
    }
    der2 = sqrt(der2) / h;
    der12 = dmax(fabs(der2), sqrt(dnf));
    if (der12 <= 1.0e-15) h1 = dmax(1.0e-6, fabs(h) * 1.0e-3);
    else if (fl->libm) h1 = pow(0.01 / der12, 1.0 / 8.0); /* (0.01/der12)^(1/iord), iord = 8 */
    else h1 = nbcs_root8(0.01 / der12);
    h = dmin(100.0 * fabs(h), dmin(h1, hmax));
    return dsign(h, posneg);
}

/* Dense output of dop853 (its contd8 and the three extra stages, as
 * numbalsoda.dop853 evaluates a t_eval grid inside one run): after the
 * accepted step [xold, xold + h] from y0 to y1 with stages k1, k6..k12 and
 * the derivative k13 at the end, the interpolant at every due output time
 * teval[*m] (up to the step's end) is written to out[2 * m ..]. */
static void dense_output(const orc_flow* fl, const double* p, double xold, double h,
                         const double* y0, const double* y1, const double* k1, const double* k6,
                         const double* k7, const double* k8, const double* k9, const double* k10,
                         const double* k11, const double* k12, const double* k13,
                         const double* teval, int n, int* m, double posneg, double* out)
{
    double k14[N2], k15[N2], k16[N2], yy[N2], F[7][N2];
    for (int i = 0; i < N2; ++i)
        yy[i] = y0[i] + h * (DP853_A_14_1 * k1[i] + DP853_A_14_7 * k7[i] + DP853_A_14_8 * k8[i]
                             + DP853_A_14_9 * k9[i] + DP853_A_14_10 * k10[i] + DP853_A_14_11 * k11[i]
                             + DP853_A_14_12 * k12[i] + DP853_A_14_13 * k13[i]);
    orc_rhs(fl, xold + DP853_C_14 * h, yy, k14, p);
    for (int i = 0; i < N2; ++i)
        yy[i] = y0[i] + h * (DP853_A_15_1 * k1[i] + DP853_A_15_6 * k6[i] + DP853_A_15_7 * k7[i]
                             + DP853_A_15_8 * k8[i] + DP853_A_15_11 * k11[i] + DP853_A_15_12 * k12[i]
                             + DP853_A_15_13 * k13[i] + DP853_A_15_14 * k14[i]);
    orc_rhs(fl, xold + DP853_C_15 * h, yy, k15, p);
    for (int i = 0; i < N2; ++i)
        yy[i] = y0[i] + h * (DP853_A_16_1 * k1[i] + DP853_A_16_6 * k6[i] + DP853_A_16_7 * k7[i]
                             + DP853_A_16_8 * k8[i] + DP853_A_16_9 * k9[i] + DP853_A_16_13 * k13[i]
                             + DP853_A_16_14 * k14[i] + DP853_A_16_15 * k15[i]);
    orc_rhs(fl, xold + DP853_C_16 * h, yy, k16, p);
    for (int i = 0; i < N2; ++i) {
        double d = y1[i] - y0[i];
        F[0][i] = d;
        F[1][i] = h * k1[i] - d;
        F[2][i] = 2.0 * d - h * (k13[i] + k1[i]);
#define DENSE_ROW(r) \
        (DP853_D_##r##_1 * k1[i] + DP853_D_##r##_6 * k6[i] + DP853_D_##r##_7 * k7[i] \
         + DP853_D_##r##_8 * k8[i] + DP853_D_##r##_9 * k9[i] + DP853_D_##r##_10 * k10[i] \
         + DP853_D_##r##_11 * k11[i] + DP853_D_##r##_12 * k12[i] + DP853_D_##r##_13 * k13[i] \
         + DP853_D_##r##_14 * k14[i] + DP853_D_##r##_15 * k15[i] + DP853_D_##r##_16 * k16[i])
        F[3][i] = h * DENSE_ROW(4);
        F[4][i] = h * DENSE_ROW(5);
        F[5][i] = h * DENSE_ROW(6);
        F[6][i] = h * DENSE_ROW(7);
#undef DENSE_ROW
    }
    while (*m < n && (teval[*m] - (xold + h)) * posneg <= 0.0) {
        double th = (teval[*m] - xold) / h, th1 = 1.0 - th;
        for (int i = 0; i < N2; ++i) {
            double v = F[6][i] * th;
            v = (F[5][i] + v) * th1;
            v = (F[4][i] + v) * th;
            v = (F[3][i] + v) * th1;
            v = (F[2][i] + v) * th;
            v = (F[1][i] + v) * th1;
            v = (F[0][i] + v) * th;
            out[2 * *m + i] = v + y0[i];
        }
        ++*m;
    }
}

static int dop853_run(const orc_flow* fl, const double* p, double x, double xend, double* y,
                      double rtol, double atol, int nmax, int32_t* stats3, const double* teval,
                      int n, double* dense);

int orc_dop853(const orc_flow* fl, const double* p, double x, double xend,
               double* y, double rtol, double atol, int nmax, int32_t* stats3)
{
    return dop853_run(fl, p, x, xend, y, rtol, atol, nmax, stats3, 0, 0, 0);
}

/* dop853 with dense output at teval[0..n) (teval[0] = x, then in the
 * direction of integration up to xend): out (n, 2); entries past a failure
 * stay 0. */
int orc_dop853_dense(const orc_flow* fl, const double* p, const double* teval, int n, double* y,
                     double rtol, double atol, int nmax, int32_t* stats3, double* out)
{
    memset(out, 0, sizeof(double) * 2 * (size_t)n);
    if (n < 1) return ORC_OK;
    return dop853_run(fl, p, teval[0], teval[n - 1], y, rtol, atol, nmax, stats3, teval, n, out);
}

static int dop853_run(const orc_flow* fl, const double* p, double x, double xend, double* y,
                      double rtol, double atol, int nmax, int32_t* stats3, const double* teval,
                      int n, double* dense)
{
    const double uround = 2.3e-16, safe = 0.9, fac1 = 0.333, fac2 = 6.0, beta = 0.0;
    double k1[N2], k2[N2], k3[N2], k4[N2], k5[N2], k6[N2], k7[N2], k8[N2], k9[N2], k10[N2];
    double yy1[N2];
    double facold = 1.0e-4, expo1 = 1.0 / 8.0 - beta * 0.2;
    double facc1 = 1.0 / fac1, facc2 = 1.0 / fac2;
    double posneg = dsign(1.0, xend - x);
    double hmax, h, hnew, xph, err, err2, deno, fac, fac11, sk, erri, sqr;
    int last = 0, reject = 0, nstep = 0, naccpt = 0, nrejct = 0, nfcn = 0, status = ORC_OK;
    int m = 1;  /* next dense output */

    if (dense) { dense[0] = y[0]; dense[1] = y[1]; }
    if (xend == x) {
        if (stats3) { stats3[0] = 0; stats3[1] = 0; stats3[2] = 0; }
        for (; dense && m < n; ++m) { dense[2 * m] = y[0]; dense[2 * m + 1] = y[1]; }
        return ORC_OK;
    }
    orc_rhs(fl, x, y, k1, p);
    hmax = fabs(xend - x);
    h = hinit(fl, p, x, y, posneg, k1, k2, hmax, rtol, atol);
    nfcn += 2;

    for (;;) {
        if (nstep > nmax) { status = ORC_MAX_STEPS; break; }
        if (0.1 * fabs(h) <= fabs(x) * uround) { status = ORC_STEP_UNDERFLOW; break; }
        if ((x + 1.01 * h - xend) * posneg > 0.0) {
            h = xend - x;
            last = 1;
        }
        nstep++;
        for (int i = 0; i < N2; ++i) yy1[i] = y[i] + h * DP853_A_2_1 * k1[i];
        orc_rhs(fl, x + DP853_C_2 * h, yy1, k2, p);
        for (int i = 0; i < N2; ++i) yy1[i] = y[i] + h * (DP853_A_3_1 * k1[i] + DP853_A_3_2 * k2[i]);
        orc_rhs(fl, x + DP853_C_3 * h, yy1, k3, p);
        for (int i = 0; i < N2; ++i) yy1[i] = y[i] + h * (DP853_A_4_1 * k1[i] + DP853_A_4_3 * k3[i]);
        orc_rhs(fl, x + DP853_C_4 * h, yy1, k4, p);
        for (int i = 0; i < N2; ++i)
            yy1[i] = y[i] + h * (DP853_A_5_1 * k1[i] + DP853_A_5_3 * k3[i] + DP853_A_5_4 * k4[i]);
        orc_rhs(fl, x + DP853_C_5 * h, yy1, k5, p);
        for (int i = 0; i < N2; ++i)
            yy1[i] = y[i] + h * (DP853_A_6_1 * k1[i] + DP853_A_6_4 * k4[i] + DP853_A_6_5 * k5[i]);
        orc_rhs(fl, x + DP853_C_6 * h, yy1, k6, p);
        for (int i = 0; i < N2; ++i)
            yy1[i] = y[i] + h * (DP853_A_7_1 * k1[i] + DP853_A_7_4 * k4[i] + DP853_A_7_5 * k5[i]
                                 + DP853_A_7_6 * k6[i]);
        orc_rhs(fl, x + DP853_C_7 * h, yy1, k7, p);
        for (int i = 0; i < N2; ++i)
            yy1[i] = y[i] + h * (DP853_A_8_1 * k1[i] + DP853_A_8_4 * k4[i] + DP853_A_8_5 * k5[i]
                                 + DP853_A_8_6 * k6[i] + DP853_A_8_7 * k7[i]);
        orc_rhs(fl, x + DP853_C_8 * h, yy1, k8, p);
        for (int i = 0; i < N2; ++i)
            yy1[i] = y[i] + h * (DP853_A_9_1 * k1[i] + DP853_A_9_4 * k4[i] + DP853_A_9_5 * k5[i]
                                 + DP853_A_9_6 * k6[i] + DP853_A_9_7 * k7[i] + DP853_A_9_8 * k8[i]);
        orc_rhs(fl, x + DP853_C_9 * h, yy1, k9, p);
        for (int i = 0; i < N2; ++i)
            yy1[i] = y[i] + h * (DP853_A_10_1 * k1[i] + DP853_A_10_4 * k4[i] + DP853_A_10_5 * k5[i]
                                 + DP853_A_10_6 * k6[i] + DP853_A_10_7 * k7[i] + DP853_A_10_8 * k8[i]
                                 + DP853_A_10_9 * k9[i]);
        orc_rhs(fl, x + DP853_C_10 * h, yy1, k10, p);
        for (int i = 0; i < N2; ++i)
            yy1[i] = y[i] + h * (DP853_A_11_1 * k1[i] + DP853_A_11_4 * k4[i] + DP853_A_11_5 * k5[i]
                                 + DP853_A_11_6 * k6[i] + DP853_A_11_7 * k7[i] + DP853_A_11_8 * k8[i]
                                 + DP853_A_11_9 * k9[i] + DP853_A_11_10 * k10[i]);
        orc_rhs(fl, x + DP853_C_11 * h, yy1, k2, p);
        xph = x + h;
        for (int i = 0; i < N2; ++i)
            yy1[i] = y[i] + h * (DP853_A_12_1 * k1[i] + DP853_A_12_4 * k4[i] + DP853_A_12_5 * k5[i]
                                 + DP853_A_12_6 * k6[i] + DP853_A_12_7 * k7[i] + DP853_A_12_8 * k8[i]
                                 + DP853_A_12_9 * k9[i] + DP853_A_12_10 * k10[i] + DP853_A_12_11 * k2[i]);
        orc_rhs(fl, xph, yy1, k3, p);
        nfcn += 11;
        for (int i = 0; i < N2; ++i) {
            k4[i] = DP853_B_1 * k1[i] + DP853_B_6 * k6[i] + DP853_B_7 * k7[i] + DP853_B_8 * k8[i]
                    + DP853_B_9 * k9[i] + DP853_B_10 * k10[i] + DP853_B_11 * k2[i] + DP853_B_12 * k3[i];
            k5[i] = y[i] + h * k4[i];
        }
        /* error estimation: 5th-order estimate combined with the 3rd-order one */
        err = 0.0;
        err2 = 0.0;
        for (int i = 0; i < N2; ++i) {
            sk = atol + rtol * dmax(fabs(y[i]), fabs(k5[i]));
            erri = k4[i] - DP853_BHH1 * k1[i] - DP853_BHH2 * k9[i] - DP853_BHH3 * k3[i];
            sqr = erri / sk;
            err2 += sqr * sqr;
            erri = DP853_E5_1 * k1[i] + DP853_E5_6 * k6[i] + DP853_E5_7 * k7[i] + DP853_E5_8 * k8[i]
                   + DP853_E5_9 * k9[i] + DP853_E5_10 * k10[i] + DP853_E5_11 * k2[i]
                   + DP853_E5_12 * k3[i];
            sqr = erri / sk;
            err += sqr * sqr;
        }
        deno = err + 0.01 * err2;
        if (deno <= 0.0) deno = 1.0;
        err = fabs(h) * err * sqrt(1.0 / (deno * (double)N2));
        if (isnan(err)) { status = ORC_NONFINITE; break; }
        /* new step size, fac1 <= hnew/h <= fac2 */
        /* err^expo1 with expo1 = 1/8 (beta = 0, so facold^beta = 1) */
        fac11 = fl->libm ? pow(err, 0.125) : nbcs_root8(err);
        fac = fac11;
        fac = dmax(facc2, dmin(facc1, fac / safe));
        hnew = h / fac;
        if (err <= 1.0) {
            facold = dmax(err, 1.0e-4);
            naccpt++;
            orc_rhs(fl, xph, k5, k4, p);
            nfcn++;
            /* stages 11 and 12 are in k2 and k3, the end derivative in k4 */
            if (dense && m < n && (teval[m] - xph) * posneg <= 0.0) {
                dense_output(fl, p, x, h, y, k5, k1, k6, k7, k8, k9, k10, k2, k3, k4, teval, n,
                             &m, posneg, dense);
                nfcn += 3;
            }
            for (int i = 0; i < N2; ++i) {
                k1[i] = k4[i];
                y[i] = k5[i];
            }
            x = xph;
            if (last) break;
            if (fabs(hnew) > hmax) hnew = posneg * hmax;
            if (reject) hnew = posneg * dmin(fabs(hnew), fabs(h));
            reject = 0;
        } else {
            hnew = h / dmin(facc1, fac11 / safe);
            reject = 1;
            if (naccpt >= 1) nrejct++;
            last = 0;
        }
        h = hnew;
    }
    if (stats3) { stats3[0] = naccpt; stats3[1] = nrejct; stats3[2] = nfcn; }
    return status;
}

int orc_flowmap_grid_2d(const orc_flow* fl, double t0, double T,
                        const double* x, int nx, const double* y, int ny,
                        const double* params, int np, double rtol, double atol,
                        const uint8_t* mask, double* out, int32_t* status,
                        int32_t* stats, int nmax, int nthreads)
{
    (void)np;
    /* t_eval = params[0] * linspace(t0, t0 + T, 2)   (integration.py:164) */
    double ts = params[0] * t0;
    double te = params[0] * (t0 + T);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int i = 0; i < nx; ++i) {
        for (int j = 0; j < ny; ++j) {
            size_t k = (size_t)i * ny + j;
            if (mask && mask[k]) {
                out[2 * k] = 0.0;
                out[2 * k + 1] = 0.0;
                if (status) status[k] = ORC_MASKED;
                if (stats) { stats[3 * k] = 0; stats[3 * k + 1] = 0; stats[3 * k + 2] = 0; }
                continue;
            }
            double yv[2] = {x[i], y[j]};
            int st = orc_dop853(fl, params, ts, te, yv, rtol, atol, nmax, stats ? stats + 3 * k : 0);
            out[2 * k] = yv[0];
            out[2 * k + 1] = yv[1];
            if (status) status[k] = st;
        }
    }
    return 0;
}

/* integration.py:8-62 (flowmap, method "dop853"): the same integration for
 * a list of points pts (npts, 2); masked points are left 0. */
int orc_flowmap_pts(const orc_flow* fl, double t0, double T, const double* pts, long npts,
                    const double* params, double rtol, double atol, const uint8_t* mask,
                    double* out, int32_t* status, int nmax, int nthreads)
{
    double ts = params[0] * t0;
    double te = params[0] * (t0 + T);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
    for (long k = 0; k < npts; ++k) {
        if (mask && mask[k]) {
            out[2 * k] = 0.0;
            out[2 * k + 1] = 0.0;
            if (status) status[k] = ORC_MASKED;
            continue;
        }
        double yv[2] = {pts[2 * k], pts[2 * k + 1]};
        int st = orc_dop853(fl, params, ts, te, yv, rtol, atol, nmax, 0);
        out[2 * k] = yv[0];
        out[2 * k + 1] = yv[1];
        if (status) status[k] = st;
    }
    return 0;
}

/* integration.py:65-121 (flowmap_n, method "dop853"): each point's positions
 * at the n times teval (params[0] * linspace(t0, t0 + T, n), built by the
 * caller) from one dense-output run; out (npts, n, 2); masked points and
 * entries past a failure stay 0. */
int orc_flowmap_n_pts(const orc_flow* fl, const double* pts, long npts, const double* teval,
                      int n, const double* params, double rtol, double atol,
                      const uint8_t* mask, double* out, int32_t* status, int nmax, int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
    for (long k = 0; k < npts; ++k) {
        double* o = out + 2 * (size_t)n * k;
        if (mask && mask[k]) {
            memset(o, 0, sizeof(double) * 2 * (size_t)n);
            if (status) status[k] = ORC_MASKED;
            continue;
        }
        double yv[2] = {pts[2 * k], pts[2 * k + 1]};
        int st = orc_dop853_dense(fl, params, teval, n, yv, rtol, atol, nmax, 0, o);
        if (status) status[k] = st;
    }
    return 0;
}

/* ------------------------------------------------------------ FTLE */

/* diagnostics.py:21-65 with utils.gradF_stencil_2D (:41-44) and
 * utils.eigvalsh_max_2D (:185-189) */
void orc_ftle_grid_2d(const double* F, int nx, int ny, double T, double dx, double dy,
                      const uint8_t* mask, double* ftle)
{
    double scaling = 1.0 / (2.0 * fabs(T));
    memset(ftle, 0, sizeof(double) * (size_t)nx * ny);
#ifdef _OPENMP
#pragma omp parallel for
#endif
    for (int i = 1; i < nx - 1; ++i) {
        for (int j = 1; j < ny - 1; ++j) {
            size_t k = (size_t)i * ny + j;
            if (mask && mask[k]) continue;
            double dxdx = (F[2 * (k + ny)] - F[2 * (k - ny)]) / (2.0 * dx);
            double dxdy = (F[2 * (k + 1)] - F[2 * (k - 1)]) / (2.0 * dy);
            double dydx = (F[2 * (k + ny) + 1] - F[2 * (k - ny) + 1]) / (2.0 * dx);
            double dydy = (F[2 * (k + 1) + 1] - F[2 * (k - 1) + 1]) / (2.0 * dy);
            double off = dxdx * dxdy + dydx * dydy;
            double a = dxdx * dxdx + dydx * dydx;
            double d = dxdy * dxdy + dydy * dydy;
            double tr = a + d;
            double disc = sqrt((a - d) * (a - d) + 4.0 * (off * off));
            double lmax = 0.5 * (tr + disc);
            if (lmax > 1.0) ftle[k] = scaling * log(lmax);
        }
    }
}

/* Symmetric 2x2 eigen-decomposition [[a,b],[b,d]], ascending eigenvalues.
 * lmax uses the same closed form as eigvalsh_max_2D; lmin is taken from the
 * product of the eigenvalues in the cancellation-free form used by LAPACK's
 * dlaev2 (the reference calls LAPACK through np.linalg.eigh).  The unit
 * eigenvector of lmax is built from the larger of the two stable
 * expressions; its sign is normalised to a non-negative x component. */
static void sym2_eig(double a, double b, double d, double* lmin, double* lmax,
                     double* vx, double* vy)
{
    double tr = a + d;
    double disc = sqrt((a - d) * (a - d) + 4.0 * (b * b));
    double l1 = 0.5 * (tr + disc);
    double acmx = fabs(a) > fabs(d) ? a : d;
    double acmn = fabs(a) > fabs(d) ? d : a;
    double l2 = (l1 != 0.0) ? (acmx / l1) * acmn - (b / l1) * b : 0.5 * (tr - disc);
    double ex, ey;
    if (b == 0.0) {
        if (a >= d) { ex = 1.0; ey = 0.0; }
        else { ex = 0.0; ey = 1.0; }
    } else if (a >= d) {
        ex = l1 - d;
        ey = b;
    } else {
        ex = b;
        ey = l1 - a;
    }
    double nrm = sqrt(ex * ex + ey * ey);
    ex /= nrm;
    ey /= nrm;
    if (ex < 0.0 || (ex == 0.0 && ey < 0.0)) { ex = -ex; ey = -ey; }
    *lmin = l2;
    *lmax = l1;
    *vx = ex;
    *vy = ey;
}

/* diagnostics.py:200-244: evals (nx,ny,2) ascending, evecs (nx,ny,2,2) with
 * eigenvectors in columns (evecs[...,:,1] belongs to the larger eigenvalue) */
void orc_c_eig_2d(const double* F, int nx, int ny, double dx, double dy,
                  const uint8_t* mask, double* evals, double* evecs)
{
    memset(evals, 0, sizeof(double) * (size_t)nx * ny * 2);
    memset(evecs, 0, sizeof(double) * (size_t)nx * ny * 4);
#ifdef _OPENMP
#pragma omp parallel for
#endif
    for (int i = 1; i < nx - 1; ++i) {
        for (int j = 1; j < ny - 1; ++j) {
            size_t k = (size_t)i * ny + j;
            if (mask && mask[k]) continue;
            double dxdx = (F[2 * (k + ny)] - F[2 * (k - ny)]) / (2.0 * dx);
            double dxdy = (F[2 * (k + 1)] - F[2 * (k - 1)]) / (2.0 * dy);
            double dydx = (F[2 * (k + ny) + 1] - F[2 * (k - ny) + 1]) / (2.0 * dx);
            double dydy = (F[2 * (k + 1) + 1] - F[2 * (k - 1) + 1]) / (2.0 * dy);
            double off = dxdx * dxdy + dydx * dydy;
            double a = dxdx * dxdx + dydx * dydx;
            double d = dxdy * dxdy + dydy * dydy;
            double l0, l1, vx, vy;
            sym2_eig(a, off, d, &l0, &l1, &vx, &vy);
            evals[2 * k] = l0;
            evals[2 * k + 1] = l1;
            /* columns: v_min = (-vy, vx), v_max = (vx, vy) */
            evecs[4 * k + 0] = -vy; /* [0][0] */
            evecs[4 * k + 1] = vx;  /* [0][1] */
            evecs[4 * k + 2] = vx;  /* [1][0] */
            evecs[4 * k + 3] = vy;  /* [1][1] */
        }
    }
}

/* diagnostics.py:247-269 */
void orc_ftle_from_eig(const double* ev, int64_t n, double T, double* ftle)
{
    double den = 2.0 * fabs(T);
    for (int64_t k = 0; k < n; ++k) ftle[k] = ev[k] > 1.0 ? log(ev[k]) / den : 0.0;
}

/* -------------------------------------------------------- percentile */

static int cmp_double(const void* a, const void* b)
{
    double x = *(const double*)a, y = *(const double*)b;
    return (x > y) - (x < y);
}

/* numba's np.percentile for a NaN-free input and 0 < q < 100:
 * rank = 1 + (n-1)*(q/100); f = floor(rank); m = rank - f;
 * lower/upper = order statistics k = f-1 and f; value = lower*(1-m) + upper*m.
 * q == 100 returns the maximum, q == 0 the minimum; any NaN -> NaN. */
double orc_percentile(const double* f, int64_t n, double q)
{
    if (n <= 0) return NAN;
    for (int64_t k = 0; k < n; ++k)
        if (isnan(f[k])) return NAN;
    if (n == 1) return f[0];
    double* s = (double*)malloc(sizeof(double) * (size_t)n);
    memcpy(s, f, sizeof(double) * (size_t)n);
    qsort(s, (size_t)n, sizeof(double), cmp_double);
    double val;
    int64_t pinf = 0, ninf = 0;
    for (int64_t k = 0; k < n; ++k) {
        if (s[k] == INFINITY) ++pinf;
        else if (s[k] == -INFINITY) ++ninf;
    }
    if (q == 100.0) {
        val = s[n - 1];
        if (pinf + ninf > 0 && !isfinite(val)) val = NAN;
    } else if (q == 0.0) {
        val = s[0];
        if (pinf + ninf > 0) {
            int64_t finite = n - (pinf + ninf);
            if (finite == 0) val = NAN;
            if (pinf == 1 && n == 2) val = NAN;
            if (ninf > 1) val = NAN;
            if (finite == 1 && pinf > 1 && ninf != 1) val = NAN;
        }
    } else {
        double rank = 1.0 + (double)(n - 1) * (q / 100.0);
        double fl = floor(rank);
        double m = rank - fl;
        int64_t k = (int64_t)(fl - 1.0);
        double lower = s[k], upper = s[k + 1 < n ? k + 1 : n - 1];
        val = lower * (1.0 - m) + upper * m;
    }
    free(s);
    return val;
}

/* ------------------------------------------------------------ ridges */

/* extraction/ridges.py:79-154 (_ftle_ridges); ftle_ridge_pts (:9-76) is the
 * row-major compaction of rpts_full over mask_out. */
void orc_ridge_field_d(const double* f, const double* ev, const double* x, int nx,
                       const double* y, int ny, double dx, double dy, double sdd_thresh,
                       double f_min, uint8_t* mask_out, double* rpts);

void orc_ridge_field(const double* f, const double* ev, const double* x, int nx,
                     const double* y, int ny, double sdd_thresh, double f_min,
                     uint8_t* mask_out, double* rpts)
{
    orc_ridge_field_d(f, ev, x, nx, y, ny, x[1] - x[0], y[1] - y[0], sdd_thresh, f_min,
                      mask_out, rpts);
}

/* the same with the grid spacing given (a row block of a sharded field) */
void orc_ridge_field_d(const double* f, const double* ev, const double* x, int nx,
                       const double* y, int ny, double dx, double dy, double sdd_thresh,
                       double f_min, uint8_t* mask_out, double* rpts)
{
    memset(mask_out, 0, (size_t)nx * ny);
    memset(rpts, 0, sizeof(double) * 2 * (size_t)nx * ny);
#ifdef _OPENMP
#pragma omp parallel for
#endif
    for (int i = 2; i < nx - 2; ++i) {
        for (int j = 2; j < ny - 2; ++j) {
            size_t k = (size_t)i * ny + j;
            double f0 = f[k];
            if (!(f0 > f_min)) continue;
            double fx = (f[k + ny] - f[k - ny]) / (2.0 * dx);
            double fy = (f[k + 1] - f[k - 1]) / (2.0 * dy);
            double fxx = (f[k + ny] - 2.0 * f[k] + f[k - ny]) / (dx * dx);
            double fyy = (f[k + 1] - 2.0 * f[k] + f[k - 1]) / (dy * dy);
            double fxy = (f[k + ny + 1] - f[k + ny - 1] - f[k - ny + 1] + f[k - ny - 1])
                         / (4.0 * dx * dy);
            double ex = ev[2 * k], ey = ev[2 * k + 1];
            double c2 = ex * (fxx * ex + fxy * ey) + ey * (fxy * ex + fyy * ey);
            if (c2 < -sdd_thresh) {
                double t = -(fx * ex + fy * ey) / c2;
                if (fabs(t * ex) <= dx / 2.0 && fabs(t * ey) <= dy / 2.0) {
                    rpts[2 * k] = x[i] + t * ex;
                    rpts[2 * k + 1] = y[j] + t * ey;
                    mask_out[k] = 1;
                }
            }
        }
    }
}

/* ------------------------------------------------------ auxiliary grid */

/* Which particles flowmap_aux_grid_2D integrates (integration.py:320-464,
 * method "dop853"): with eig_main (n_aux = 5) an edge point integrates only
 * its centre particle (k = 4) when compute_edge is set; without eig_main
 * (n_aux = 4) every point integrates all four when compute_edge is set; with
 * compute_edge off the edge points are skipped. */
static int aux_active(int i, int j, int k, int nx, int ny, int n_aux, int compute_edge)
{
    const int edge = (i == 0 || i == nx - 1 || j == 0 || j == ny - 1);
    if (!edge) return 1;
    if (!compute_edge) return 0;
    return n_aux == 4 || k == 4;
}

/* integration.py:249-464: particle k of grid point (i, j) starts at
 * (x_i, y_j) + aux_k with aux = (h,0), (-h,0), (0,h), (0,-h) [, (0,0)];
 * out (nx,ny,n_aux,2); masked and skipped entries stay 0 (status MASKED). */
int orc_flowmap_aux_grid_2d(const orc_flow* fl, double t0, double T, const double* x, int nx,
                            const double* y, int ny, const double* params, double h,
                            int eig_main, int compute_edge, double rtol, double atol,
                            const uint8_t* mask, double* out, int32_t* status, int32_t* stats,
                            int nmax, int nthreads)
{
    const int n_aux = eig_main ? 5 : 4;
    const double aux[5][2] = {{h, 0.0}, {-h, 0.0}, {0.0, h}, {0.0, -h}, {0.0, 0.0}};
    double ts = params[0] * t0;
    double te = params[0] * (t0 + T);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int i = 0; i < nx; ++i) {
        for (int j = 0; j < ny; ++j) {
            for (int k = 0; k < n_aux; ++k) {
                size_t q = ((size_t)i * ny + j) * n_aux + k;
                if ((mask && mask[(size_t)i * ny + j]) || !aux_active(i, j, k, nx, ny, n_aux, compute_edge)) {
                    out[2 * q] = 0.0;
                    out[2 * q + 1] = 0.0;
                    if (status) status[q] = ORC_MASKED;
                    if (stats) { stats[3 * q] = 0; stats[3 * q + 1] = 0; stats[3 * q + 2] = 0; }
                    continue;
                }
                double yv[2] = {x[i] + aux[k][0], y[j] + aux[k][1]};
                int st = orc_dop853(fl, params, ts, te, yv, rtol, atol, nmax, stats ? stats + 3 * q : 0);
                out[2 * q] = yv[0];
                out[2 * q + 1] = yv[1];
                if (status) status[q] = st;
            }
        }
    }
    return 0;
}

/* diagnostics.py:69-111 (C_tensor_2D) with utils.gradF_aux_stencil_2D
 * (:50-84): C11, C12, C22 of the aux-particle tensor for 2 <= i < nx-2,
 * 2 <= j < ny-2 (unmasked), 0 elsewhere; F is (nx, ny, na, 2). */
void orc_c_tensor_2d(const double* F, int nx, int ny, int na, double h, const uint8_t* mask,
                     double* C)
{
    memset(C, 0, sizeof(double) * 3 * (size_t)nx * ny);
    for (int i = 2; i < nx - 2; ++i) {
        for (int j = 2; j < ny - 2; ++j) {
            size_t k = (size_t)i * ny + j;
            if (mask && mask[k]) continue;
            const double* A = F + k * na * 2;
            double dxdx = (A[0] - A[2]) / (2.0 * h);
            double dxdy = (A[4] - A[6]) / (2.0 * h);
            double dydx = (A[1] - A[3]) / (2.0 * h);
            double dydy = (A[5] - A[7]) / (2.0 * h);
            C[3 * k] = dxdx * dxdx + dydx * dydx;
            C[3 * k + 1] = dxdx * dxdy + dydx * dydy;
            C[3 * k + 2] = dxdy * dxdy + dydy * dydy;
        }
    }
}

/* diagnostics.py:113-197 (C_eig_aux_2D) with utils.gradF_aux_stencil_2D
 * (:50-84) and gradF_main_stencil_2D (:88-124).  eig_main: eigenvectors from
 * the aux-grid tensor, eigenvalues from the main-grid tensor (centre
 * particles, spacing dx, dy), for 2 <= i < nx-2, 2 <= j < ny-2; otherwise both
 * from the aux-grid tensor for 1 <= i < nx-1, 1 <= j < ny-1. */
void orc_c_eig_aux_2d(const double* F, int nx, int ny, double dx, double dy, double h,
                      int eig_main, const uint8_t* mask, double* evals, double* evecs)
{
    const int n_aux = eig_main ? 5 : 4, b = eig_main ? 2 : 1;
    memset(evals, 0, sizeof(double) * (size_t)nx * ny * 2);
    memset(evecs, 0, sizeof(double) * (size_t)nx * ny * 4);
#ifdef _OPENMP
#pragma omp parallel for
#endif
    for (int i = b; i < nx - b; ++i) {
        for (int j = b; j < ny - b; ++j) {
            size_t k = (size_t)i * ny + j;
            if (mask && mask[k]) continue;
            const double* A = F + 2 * n_aux * k;  /* A[2*m + c]: particle m, component c */
            double dxdx = (A[0] - A[2]) / (2.0 * h);
            double dxdy = (A[4] - A[6]) / (2.0 * h);
            double dydx = (A[1] - A[3]) / (2.0 * h);
            double dydy = (A[5] - A[7]) / (2.0 * h);
            double off = dxdx * dxdy + dydx * dydy;
            double l0, l1, vx, vy;
            sym2_eig(dxdx * dxdx + dydx * dydx, off, dxdy * dxdy + dydy * dydy, &l0, &l1, &vx, &vy);
            if (eig_main) {
                const int c = 2 * (n_aux - 1);  /* centre particle */
                const double* xp = F + 2 * n_aux * (k + ny) + c;
                const double* xm = F + 2 * n_aux * (k - ny) + c;
                const double* yp = F + 2 * n_aux * (k + 1) + c;
                const double* ym = F + 2 * n_aux * (k - 1) + c;
                double mxdx = (xp[0] - xm[0]) / (2.0 * dx);
                double mxdy = (yp[0] - ym[0]) / (2.0 * dy);
                double mydx = (xp[1] - xm[1]) / (2.0 * dx);
                double mydy = (yp[1] - ym[1]) / (2.0 * dy);
                double moff = mxdx * mxdy + mydx * mydy;
                double wx, wy;
                sym2_eig(mxdx * mxdx + mydx * mydx, moff, mxdy * mxdy + mydy * mydy, &l0, &l1,
                         &wx, &wy);
            }
            evals[2 * k] = l0;
            evals[2 * k + 1] = l1;
            evecs[4 * k + 0] = -vy;
            evecs[4 * k + 1] = vx;
            evecs[4 * k + 2] = vx;
            evecs[4 * k + 3] = vy;
        }
    }
}

/* --------------------------------------------------- flow-map composition */

/* Cell and offset of x on the uniform axis (a, n; dinv = (n-1)/(b-a)) for
 * multilinear interpolation of a point inside [a, b]. */
static int lin_locate(double a, double dinv, int n, double x, double* lam)
{
    if (x != x) { *lam = x; return 0; }
    double u = (x - a) * dinv;
    int i = (int)floor(u);
    if (i > n - 2) i = n - 2;
    if (i < 0) i = 0;
    *lam = u - (double)i;
    return i;
}

/* eval_linear(grid, f[..., c], (px, py)) on f (nx, ny, 2) */
static void bilinear2(const double* f, const double* g, int nx, int ny, double px, double py,
                      double* r)
{
    if (px < g[0] || px > g[1] || py < g[3] || py > g[4]) {  /* xto.CONSTANT: 0 outside */
        r[0] = r[1] = 0.0;
        return;
    }
    double l0, l1;
    int i = lin_locate(g[0], ((double)nx - 1.0) / (g[1] - g[0]), nx, px, &l0);
    int j = lin_locate(g[3], ((double)ny - 1.0) / (g[4] - g[3]), ny, py, &l1);
    const double* f00 = f + 2 * ((size_t)i * ny + j);
    const double* f10 = f00 + 2 * (size_t)ny;
    /* lerp along y in both rows, then along x (explicit FMAs) */
    for (int c = 0; c < 2; ++c) {
        double a = fma(l1, f00[2 + c] - f00[c], f00[c]);
        double b = fma(l1, f10[2 + c] - f10[c], f10[c]);
        r[c] = fma(l0, b - a, a);
    }
}

/* integration.py:609-641 (flowmap_composition): the points start at the
 * first map's values, pass through maps 1 .. nT-2 by bilinear interpolation
 * on the grid (x0, x1, nx, y0, y1, ny; 0 outside it, xto.CONSTANT) and end
 * at the last map (nT = 1
 * therefore interpolates the single map at its own values, as the reference
 * does).  Map j of the sequence is fms[(first + j) % nT] (a ring buffer). */
void orc_flowmap_compose(const double* fms, int nT, int first, int nx, int ny, const double* grid,
                         double* out)
{
    const size_t m = (size_t)nx * ny * 2;
#ifdef _OPENMP
#pragma omp parallel for
#endif
    for (long p = 0; p < (long)nx * ny; ++p) {
        const double* f0 = fms + m * (size_t)(first % nT);
        double pt[2] = {f0[2 * p], f0[2 * p + 1]}, r[2];
        for (int k = 1; k < nT - 1; ++k) {
            bilinear2(fms + m * (size_t)((first + k) % nT), grid, nx, ny, pt[0], pt[1], r);
            pt[0] = r[0];
            pt[1] = r[1];
        }
        bilinear2(fms + m * (size_t)((first + nT - 1) % nT), grid, nx, ny, pt[0], pt[1], r);
        out[2 * p] = r[0];
        out[2 * p + 1] = r[1];
    }
}
