/*
 * CPU oracle for the flow-map -> FTLE -> ridge path (TEST INFRASTRUCTURE ONLY).
 *
 * This is a plain-C restatement of the reference NumbaCS algorithms, used as the
 * checker for the CUDA library and as the timed CPU baseline.  It is never linked
 * into, imported by, or called from the product library; only the tests, the
 * smoke check and the benchmark's CPU-baseline leg load it.
 *
 * Parity pin: the restatement reproduces the reference's own golden fixtures
 * (tests/testing_data/fm.npy, ftle.npy, Cevals.npy/Cevecs.npy, ridge_pts.npy,
 * ridges.pkl and the spline / RHS literals in tests/test_flows.py), copied into
 * tests/golden/ by tests/golden/make_golden.py.
 */
#ifndef NBCS_ORACLE_H
#define NBCS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* flow kinds (same numbering as the CUDA library) */
enum { ORC_FLOW_DOUBLE_GYRE = 0, ORC_FLOW_BICKLEY = 1, ORC_FLOW_SPLINE2D = 2 };

/* per-particle status codes (same as the CUDA library) */
enum {
    ORC_OK = 0,
    ORC_MASKED = 1,
    ORC_MAX_STEPS = -2,
    ORC_STEP_UNDERFLOW = -3,
    ORC_NONFINITE = -4
};

typedef struct {
    int kind;          /* ORC_FLOW_* */
    int spherical;     /* spline only: 0 planar, 1 lon in [-180,180), 2 lon in [0,360) */
    int extrap;        /* spline only, outside the grid box: 0 constant (zero), 1 nearest,
                          2 linear (orc_eval_spline_3d) */
    double r;          /* spline only: sphere radius used for the km -> degree conversion */
    double grid[9];    /* spline only: t0,t1,nt, x0,x1,nx, y0,y1,ny */
    const double* cu;  /* spline only: coefficients (nt+2, nx+2, ny+2), C order */
    const double* cv;
    /* 0: the deterministic helpers the GPU library also uses (err^(1/8) as
     * three square roots, the Taylor-series cos of the spherical metric), so
     * that GPU and oracle can be compared bit for bit; 1: the reference's
     * literal libm calls (pow(err, 1/8) as in Hairer's dop853, cos(lat*pi/180)
     * as in flows.py:180), to measure how far those helpers move results */
    int libm;
} orc_flow;

/* the deterministic helpers of detmath.h (exposed for their accuracy test) */
double orc_cos_deg(double d);
double orc_root8(double x);

/* velocity fields (one RHS evaluation, reference direction convention) */
void orc_rhs(const orc_flow* flow, double t, const double* y, double* dy, const double* p);

/* natural-BC cubic B-spline prefilter of f (nt,nx,ny) -> coef (nt+2,nx+2,ny+2) */
int orc_prefilter_3d(const double* f, int nt, int nx, int ny, double* coef);
/* tricubic spline evaluation at (t,x,y) with the grid tuple above */
double orc_eval_spline_3d(const double* grid, const double* coef, int extrap,
                          double t, double x, double y);

/* DOP853 integration of one particle over [x, xend] (solver time). */
int orc_dop853(const orc_flow* flow, const double* p, double x, double xend,
               double* y, double rtol, double atol, int nmax, int32_t* stats3);

/* flowmap_grid_2D: out (nx,ny,2); status (nx,ny) nullable; stats (nx,ny,3) nullable */
int orc_flowmap_grid_2d(const orc_flow* flow, double t0, double T,
                        const double* x, int nx, const double* y, int ny,
                        const double* params, int np, double rtol, double atol,
                        const uint8_t* mask, double* out, int32_t* status,
                        int32_t* stats, int nmax, int nthreads);

/* dop853 with dense output at teval[0..n): out (n,2) */
int orc_dop853_dense(const orc_flow* flow, const double* p, const double* teval, int n, double* y,
                     double rtol, double atol, int nmax, int32_t* stats3, double* out);

/* flowmap_n: pts (npts,2), teval (n) -> out (npts,n,2); mask, status nullable */
int orc_flowmap_n_pts(const orc_flow* flow, const double* pts, long npts, const double* teval,
                      int n, const double* params, double rtol, double atol,
                      const uint8_t* mask, double* out, int32_t* status, int nmax, int nthreads);

/* flowmap: pts (npts,2) -> out (npts,2); mask, status (npts,) nullable */
int orc_flowmap_pts(const orc_flow* flow, double t0, double T, const double* pts, long npts,
                    const double* params, double rtol, double atol, const uint8_t* mask,
                    double* out, int32_t* status, int nmax, int nthreads);

/* C_tensor_2D: F (nx,ny,na,2) -> C (nx,ny,3) */
void orc_c_tensor_2d(const double* F, int nx, int ny, int na, double h, const uint8_t* mask,
                     double* C);

void orc_ftle_grid_2d(const double* fm, int nx, int ny, double T, double dx, double dy,
                      const uint8_t* mask, double* ftle);
void orc_c_eig_2d(const double* fm, int nx, int ny, double dx, double dy,
                  const uint8_t* mask, double* evals, double* evecs);
void orc_ftle_from_eig(const double* evmax, int64_t n, double T, double* ftle);

/* np.percentile as evaluated inside the reference's numba-jitted code */
double orc_percentile(const double* f, int64_t n, double q);

/* _ftle_ridges: ridge mask (nx,ny) u8 and the full r_pts (nx*ny,2) array */
void orc_ridge_field(const double* f, const double* evec, const double* x, int nx,
                     const double* y, int ny, double sdd_thresh, double f_min,
                     uint8_t* mask_out, double* rpts_full);
void orc_ridge_field_d(const double* f, const double* evec, const double* x, int nx,
                       const double* y, int ny, double dx, double dy, double sdd_thresh,
                       double f_min, uint8_t* mask_out, double* rpts_full);

/* flowmap_aux_grid_2D: out (nx,ny,n_aux,2), n_aux = 5 (eig_main) or 4 */
int orc_flowmap_aux_grid_2d(const orc_flow* flow, double t0, double T, const double* x, int nx,
                            const double* y, int ny, const double* params, double h,
                            int eig_main, int compute_edge, double rtol, double atol,
                            const uint8_t* mask, double* out, int32_t* status, int32_t* stats,
                            int nmax, int nthreads);
/* C_eig_aux_2D: evals (nx,ny,2), evecs (nx,ny,2,2) */
void orc_c_eig_aux_2d(const double* fm_aux, int nx, int ny, double dx, double dy, double h,
                      int eig_main, const uint8_t* mask, double* evals, double* evecs);
/* flowmap_composition over nT maps (nT,nx,ny,2) read in ring order from `first`;
 * grid = x0, x1, nx, y0, y1, ny */
void orc_flowmap_compose(const double* fms, int nT, int first, int nx, int ny,
                         const double* grid, double* out);

#ifdef __cplusplus
}
#endif
#endif
