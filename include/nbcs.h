/*
 * nbcs.h -- C ABI of the GB300 (sm_103a) flow-map -> FTLE -> ridge library
 * (libnbcs.so).  Plain pointers and sizes only; every array argument is a
 * DEVICE pointer unless marked "host".  All calls are asynchronous on the
 * given CUDA stream (cudaStream_t passed as void*), allocate no memory, and
 * return an int status (NBCS_OK = 0, negative on error; see nbcs_last_error).
 *
 * Each entry point names the reference NumbaCS interface it replaces
 * (path:line within the NumbaCS project).  In the reference those are
 * numba-jitted Python functions; the "plugin" is a numba @cfunc RHS whose
 * address is handed to numbalsoda's dop853.  A host function pointer cannot
 * run on the GPU, so the RHS is described by the nbcs_flow struct instead and
 * the right-hand sides are compiled device functions selected by `kind`.
 */
#ifndef NBCS_H
#define NBCS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NBCS_ABI_VERSION 3

/* return codes */
#define NBCS_OK 0
#define NBCS_ERR_INVALID (-1)     /* bad argument (size, pointer, flow, ...) */
#define NBCS_ERR_CUDA (-2)        /* a CUDA runtime call failed */
#define NBCS_ERR_SCRATCH (-3)     /* scratch buffer missing or too small */
#define NBCS_ERR_UNSUPPORTED (-4) /* option not supported (e.g. method="lsoda") */

/* per-particle status written by the integrators (int32) */
#define NBCS_PARTICLE_OK 0
#define NBCS_PARTICLE_MASKED 1
#define NBCS_PARTICLE_MAX_STEPS (-2)      /* more than max_steps attempted steps */
#define NBCS_PARTICLE_STEP_UNDERFLOW (-3) /* 0.1|h| <= |t| * 2.3e-16 */
#define NBCS_PARTICLE_NONFINITE (-4)      /* error estimate became NaN */

/* flow kinds */
#define NBCS_FLOW_DOUBLE_GYRE 0 /* flows.py:1144-1178, params[6]  */
#define NBCS_FLOW_BICKLEY 1     /* flows.py:1180-1245, params[12] */
#define NBCS_FLOW_SPLINE2D 2    /* flows.py:121-258, params[1]    */

/* integrator precision */
#define NBCS_PREC_FP64 0  /* every operation in IEEE double, no FMA contraction */
#define NBCS_PREC_MIXED 1 /* FP32 stages / interpolation, compensated FP32-pair positions */

#define NBCS_MAX_PARAMS 16

/* Replaces the funcptr returned by get_predefined_flow (flows.py:1104-1295)
 * and get_flow_2D (flows.py:121-258).  For SPLINE2D the coefficient arrays
 * are the (nt+2, nx+2, ny+2) cubic B-spline coefficients of u and v
 * interleaved per node: coef_uv[2*node + 0] = u, [2*node + 1] = v. */
typedef struct nbcs_flow {
    int32_t kind;      /* NBCS_FLOW_* */
    int32_t spherical; /* SPLINE2D: 0 planar, 1 lon in [-180,180), 2 lon in [0,360) */
    int32_t extrap;    /* SPLINE2D, outside the grid box: 0 "constant" (zero velocity),
                          1 "nearest" (value at the nearest box point), 2 "linear"
                          (that value plus derivative x distance along each clamped
                          axis); eval_spline's extrap_mode, flows.py:121 */
    int32_t reserved;
    double r;          /* SPLINE2D spherical: radius (km) for km/h -> deg/h */
    double grid[9];    /* SPLINE2D: t0,t1,nt, x0,x1,nx, y0,y1,ny (UCGrid tuple) */
    const double* coef_uv;  /* SPLINE2D FP64 coefficients (device), required */
    /* SPLINE2D FP32 copy (device), required for NBCS_PREC_MIXED, in the "quad"
     * layout: entry k (32 bytes) holds u_j, v_j for j = k .. k+3 (zeros past the
     * end); n entries, 32-byte aligned; n < 2^32 (the mixed path indexes
     * entries with 32-bit integers). */
    const float* coef_uv32;
} nbcs_flow;

/* integrator options; a NULL opts pointer means all defaults */
typedef struct nbcs_opts {
    int32_t precision;     /* NBCS_PREC_* (default FP64) */
    int32_t max_steps;     /* attempted-step limit per particle (default 100000) */
    int32_t threads_per_block; /* FP64 path: 0 = library default (128) */
    int32_t blocks_per_sm;     /* grid cap in blocks per SM; 0 = one block per particle tile */
    int32_t lanes_per_particle; /* mixed spline path: 1, 2 or 4 lanes share a particle; 0 = auto */
    int32_t step_model_mode;    /* how a step_model proposal h_m meets the controller's h_c.
                                   At every fresh step: 0 = h_m, 1 = min(h_m, h_c),
                                   2 = sqrt(h_m h_c).  Only at the first step and after a
                                   rejection: 3 = min(h_m, h_c); 4 = h_m replaces HINIT's
                                   initial step (no probe evaluation), then min(h_m, h_c)
                                   after a rejection */
    int32_t* stats;        /* optional device (n,3) int32: accepted, rejected, RHS evals */
    const void* step_model; /* optional learned step-size proposer (device blob, see nbcs_mlp_*);
                               mixed precision, spline flows */
} nbcs_opts;

/* Library version / last error message of the calling host thread. */
int nbcs_abi_version(void);
const char* nbcs_last_error(void);

/* ---------------------------------------------------------------- flows */

/* get_interp_arrays_2D prefilter (flows.py:9-46 -> interpolation.splines.prefilter,
 * k=3): natural-BC cubic B-spline coefficients of f (nt,nx,ny) into coef
 * (nt+2,nx+2,ny+2).  scratch >= nbcs_spline_prefilter_scratch_bytes(). */
size_t nbcs_spline_prefilter_scratch_bytes(int32_t nt, int32_t nx, int32_t ny);
int nbcs_spline_prefilter_3d(const double* f, int32_t nt, int32_t nx, int32_t ny,
                             double* coef, void* scratch, size_t scratch_bytes, void* stream);

/* get_flow_2D coefficient capture (flows.py:156-254 closes over C_eval_u /
 * C_eval_v): interleave cu, cv (n nodes each) into coef_uv (2n doubles) and,
 * if coef_uv32 != NULL, an FP32 copy in the quad layout (8n floats, 32-byte
 * aligned; coef_uv 16-byte aligned). */
int nbcs_spline_pack_uv(const double* cu, const double* cv, int64_t n, double* coef_uv,
                        float* coef_uv32, void* stream);

/* One RHS evaluation per point, as the reference @cfunc computes it
 * (flows.py:1146-1213 and :154-254): ty (n,3) rows (t, x, y) -> dy (n,2).
 * params: host array of np doubles. */
int nbcs_eval_rhs(const nbcs_flow* flow, const double* params, int32_t np, const double* ty,
                  int64_t n, double* dy, int32_t precision, void* stream);

/* ----------------------------------------------------------- integration */

/* flowmap_grid_2D (integration.py:123-182) with method="dop853":
 * integrate every particle (x[i], y[j]) over solver time
 * params[0]*[t0, t0+T] with DOP853 (rtol, atol) and write its end position to
 * flowmap (nx,ny,2).  mask (nx,ny) u8 may be NULL; masked particles are left
 * 0 with status MASKED.  status (nx,ny) int32 may be NULL. */
int nbcs_flowmap_grid_2d(const nbcs_flow* flow, double t0, double T,
                         const double* x, int32_t nx, const double* y, int32_t ny,
                         const double* params, int32_t np, double rtol, double atol,
                         const uint8_t* mask, double* flowmap, int32_t* status,
                         const nbcs_opts* opts, void* stream);

/* flowmap_n (integration.py:65-121) and flowmap_n_grid_2D (:468-534) with
 * method="dop853": the positions of each point pts (npts,2) at the n output
 * times teval (device, params[0] * linspace(t0, t0 + T, n), teval[0] the
 * start) from one DOP853 run with dop853's dense output, as numbalsoda.dop853
 * fills a t_eval grid -> out (npts, n, 2); masked points and outputs past a
 * failure stay 0; status (npts,) may be NULL.  FP64 only (opts may be NULL). */
int nbcs_flowmap_n_pts(const nbcs_flow* flow, const double* pts, int64_t npts, const double* teval,
                       int32_t n, const double* params, int32_t np, double rtol, double atol,
                       const uint8_t* mask, double* out, int32_t* status, const nbcs_opts* opts,
                       void* stream);

/* flowmap (integration.py:8-62) and flowmap_grid_ND with ndims = 2
 * (:186-247), method="dop853": the same integration for a list of points,
 * pts (npts,2) C-order -> flowmap (npts,2); mask (npts,) u8 and status
 * (npts,) int32 may be NULL; npts < 2^31; no step_model. */
int nbcs_flowmap_pts(const nbcs_flow* flow, double t0, double T, const double* pts,
                     int64_t npts, const double* params, int32_t np, double rtol, double atol,
                     const uint8_t* mask, double* flowmap, int32_t* status,
                     const nbcs_opts* opts, void* stream);

/* flowmap_aux_grid_2D (integration.py:249-464) with method="dop853": every
 * grid point (x[i], y[j]) integrates the particles started at (x[i], y[j]) +
 * (h,0), (-h,0), (0,h), (0,-h) and, with eig_main, (0,0), into flowmap_aux
 * (nx, ny, 5 or 4, 2).  compute_edge != 0: edge points integrate only their
 * centre particle (eig_main) or all four; compute_edge == 0: edge points are
 * skipped.  Masked and skipped entries are left 0 with status MASKED;
 * status (nx, ny, 5 or 4) int32 may be NULL.  opts as for
 * nbcs_flowmap_grid_2d (no step_model; the mixed path's FP32 stage rounding
 * is amplified 1/(2h)-fold by C_eig_aux_2D's differences, so FP64 is the
 * path for this one). */
int nbcs_flowmap_aux_grid_2d(const nbcs_flow* flow, double t0, double T,
                             const double* x, int32_t nx, const double* y, int32_t ny,
                             const double* params, int32_t np, double h, int32_t eig_main,
                             int32_t compute_edge, double rtol, double atol,
                             const uint8_t* mask, double* flowmap_aux, int32_t* status,
                             const nbcs_opts* opts, void* stream);

/* flowmap_composition (integration.py:609-641): compose nT flow maps
 * (nT, nx, ny, 2) on the grid `grid` (host, 6 doubles: x0, x1, nx, y0, y1, ny
 * -- the UCGrid tuple) into out (nx, ny, 2).  Map j of the sequence is
 * flowmaps[(first + j) % nT] (pass first = 0 for the reference's order; a
 * ring buffer advanced by one map per step needs no shifting).  Bilinear
 * interpolation, 0 outside the grid box (interpolation's xto.CONSTANT); nT = 1
 * interpolates the map at its own values, as the reference does.  The
 * callers flowmap_composition_initial / _step (:644-737) are host loops over
 * nbcs_flowmap_grid_2d and this call. */
int nbcs_flowmap_compose(const double* flowmaps, int32_t nT, int32_t first, const double* grid,
                         double* out, void* stream);

/* -------------------------------------------------------- batched fields */

/* One FTLE field of a batched launch: what one flowmap_grid_2D call (plus an
 * optional ftle_evec_2d) takes.  Replaces the reference's Python loop over t0
 * values (examples/time_series/*.py) that calls flowmap_grid_2D and
 * ftle_grid_2D once per field.  All pointers are device pointers. */
typedef struct nbcs_field {
    int32_t flow;      /* index into the batch's flows array */
    int32_t nx, ny;
    int32_t np;        /* number of params */
    double params[NBCS_MAX_PARAMS];
    double t0, T, rtol, atol;
    double dx, dy;     /* grid spacing for the FTLE stencil */
    const double* x;
    const double* y;
    const uint8_t* mask; /* nullable */
    double* flowmap;     /* (nx, ny, 2) */
    int32_t* status;     /* nullable */
    double* ftle;        /* (nx, ny); NULL: no FTLE for this field */
    double* evec_max;    /* (nx, ny, 2); used when ftle != NULL */
} nbcs_field;

/* The fields of a batch that share one integrator instantiation (flow kind;
 * for spline flows also the spherical mode and whether the grid nodes are
 * floats): one launch of the class's tile kernel integrates all of them. */
#define NBCS_BATCH_MAX_CLASSES 8
typedef struct nbcs_batch_class {
    int32_t kind, spherical, exact_nodes, lanes; /* lanes per particle */
    int32_t field0, nfields;  /* a contiguous range of the plan's field table */
    int64_t tiles;            /* 256-thread particle tiles of the class's fields */
    int32_t flow, reserved;   /* the flow every field of the class uses, else -1 */
    double r, grid[9];        /* that flow's radius and spline grid (kernel arguments) */
    const float* coef_uv32;   /* and its FP32 coefficients */
} nbcs_batch_class;

/* Host-side handle of a prepared batch (filled by nbcs_batch_prepare). */
typedef struct nbcs_batch {
    void* scratch;       /* device memory holding the batch description */
    int32_t nflows, nfields, precision, reserved;
    int64_t total_chunks; /* 32-particle work units over all fields */
    int64_t ftle_blocks;  /* 256-point FTLE work units */
    int64_t tiles;        /* particle tiles of one 256-thread block over all fields */
    int32_t nclasses, reserved2;
    nbcs_batch_class classes[NBCS_BATCH_MAX_CLASSES];
} nbcs_batch;

size_t nbcs_batch_scratch_bytes(int32_t nflows, int32_t nfields);
/* Copy the flows and fields (host arrays) into `scratch` and fill `plan`.
 * Reads host memory: not capturable; call once per batch layout. */
int nbcs_batch_prepare(const nbcs_flow* flows, int32_t nflows, const nbcs_field* fields,
                       int32_t nfields, int32_t precision, void* scratch, size_t scratch_bytes,
                       nbcs_batch* plan, void* stream);
/* Integrate every particle of every field, then run the FTLE/eigvec stencil
 * of all fields in one launch.  Kernel launches only: capturable in a CUDA
 * graph.  Two schedules, chosen by opts->blocks_per_sm:
 *   >= 0  one persistent grid of blocks_per_sm blocks per SM (0 = full
 *         occupancy) whose warps take 32-particle chunks of any field from a
 *         shared counter;
 *   <  0  (mixed precision) per flow class one launch of that class's tile
 *         kernel -- the single-field integrator's block shape and register
 *         budget -- with one block per particle tile of the class's fields,
 *         fields ordered longest first (|T|, then size), the hardware block
 *         scheduler balancing the tiles; the classes run one after another
 *         on `stream` (nbcs_batch_run_class launches one class, so a caller
 *         can put the classes on parallel streams).
 * Either way fields of different sizes and lengths share the GPU instead of
 * each leaving it idle at the end of its own launch.  opts: precision is
 * taken from the plan; stats/step_model unused. */
int nbcs_batch_run(const nbcs_batch* plan, const nbcs_opts* opts, void* stream);
/* The tile kernel of class k of a mixed-precision plan (no FTLE). */
int nbcs_batch_run_class(const nbcs_batch* plan, int32_t k, const nbcs_opts* opts, void* stream);
/* The FTLE/eigvec stencil of every field of the plan (after its flow maps). */
int nbcs_batch_run_ftle(const nbcs_batch* plan, void* stream);

/* ------------------------------------------------------------ diagnostics */

/* ftle_grid_2D (diagnostics.py:21-65): flowmap (nx,ny,2) -> ftle (nx,ny). */
int nbcs_ftle_grid_2d(const double* flowmap, int32_t nx, int32_t ny, double T, double dx,
                      double dy, const uint8_t* mask, double* ftle, void* stream);

/* C_eig_2D (diagnostics.py:200-244): evals (nx,ny,2) ascending, evecs
 * (nx,ny,2,2) eigenvectors in columns. */
int nbcs_c_eig_2d(const double* flowmap, int32_t nx, int32_t ny, double dx, double dy,
                  const uint8_t* mask, double* evals, double* evecs, void* stream);

/* C_tensor_2D (diagnostics.py:69-111): flowmap_aux (nx, ny, naux >= 4, 2) from
 * nbcs_flowmap_aux_grid_2d -> C (nx,ny,3) = C11, C12, C22 of the Cauchy-Green
 * tensor of the +-h particles for 2 <= i < nx-2, 2 <= j < ny-2 (unmasked),
 * 0 elsewhere. */
int nbcs_c_tensor_2d(const double* flowmap_aux, int32_t nx, int32_t ny, int32_t naux, double h,
                     const uint8_t* mask, double* C, void* stream);

/* C_eig_aux_2D (diagnostics.py:113-197): flowmap_aux (nx, ny, 5 or 4, 2) from
 * nbcs_flowmap_aux_grid_2d -> evals (nx,ny,2) ascending, evecs (nx,ny,2,2)
 * eigenvectors in columns.  eig_main: eigenvectors from the aux-particle
 * differences (spacing h), eigenvalues from the centre particles' main-grid
 * differences (dx, dy), at 2 <= i < nx-2, 2 <= j < ny-2; otherwise both from
 * the aux differences at 1 <= i < nx-1, 1 <= j < ny-1; 0 elsewhere. */
int nbcs_c_eig_aux_2d(const double* flowmap_aux, int32_t nx, int32_t ny, int32_t eig_main,
                      double dx, double dy, double h, const uint8_t* mask, double* evals,
                      double* evecs, void* stream);

/* ftle_from_eig (diagnostics.py:247-269) on a strided eigenvalue array:
 * ftle[k] = log(ev[k*stride]) / (2|T|) if ev > 1 else 0. */
int nbcs_ftle_from_eig(const double* eigval, int64_t n, int64_t stride, double T,
                       double* ftle, void* stream);

/* Fused C_eig_2D + ftle_from_eig(eigvals[...,1]) + eigvecs[...,:,1]:
 * flowmap -> ftle (nx,ny) and evec_max (nx,ny,2) in one pass (the inputs of
 * ftle_ridge_pts).  The scaling divisions (1/(2dx), 1/(2dy), 1/(2|T|)) are
 * products with reciprocals, the eigenvector is normalised by a reciprocal
 * square root and the log's mantissa part is an FP32 log1p, so the
 * eigenvector is within a few ulp and the FTLE within ~3e-7 relative of
 * nbcs_c_eig_2d + nbcs_ftle_from_eig rather than bit-identical (those two
 * keep the reference's IEEE arithmetic). */
int nbcs_ftle_evec_2d(const double* flowmap, int32_t nx, int32_t ny, double T, double dx,
                      double dy, const uint8_t* mask, double* ftle, double* evec_max,
                      void* stream);

/* ------------------------------------------------------------- extraction */

/* np.percentile(f, q) as evaluated in the reference's jitted ftle_ridge_pts
 * (ridges.py:48-51; numba's linear-rank rule), written to *out (device). */
size_t nbcs_percentile_scratch_bytes(int64_t n);
int nbcs_percentile(const double* f, int64_t n, double q, double* out, void* scratch,
                    size_t scratch_bytes, void* stream);

/* ftle_ridge_pts (ridges.py:9-76) and the _ftle_ridges mask (ridges.py:79-154).
 * Writes mask_out (nx,ny) u8 if not NULL, rpts_full (nx*ny,2) if not NULL
 * (zeros off the ridge, as _ftle_ridges returns), the row-major compacted
 * points to pts_out (capacity nx*ny rows) and their count to *n_out
 * (device int64).  percentile == 0 means threshold 0 (ridges.py:48-49). */
size_t nbcs_ridge_scratch_bytes(int32_t nx, int32_t ny);
int nbcs_ridge_pts(const double* f, const double* evec_max, const double* x, int32_t nx,
                   const double* y, int32_t ny, double sdd_thresh, double percentile,
                   uint8_t* mask_out, double* rpts_full, double* pts_out, int64_t* n_out,
                   void* scratch, size_t scratch_bytes, void* stream);

/* nbcs_ridge_pts with the threshold f_min and the grid spacing dx, dy given
 * instead of a percentile of f and x[1] - x[0], y[1] - y[0] (no reference
 * counterpart: a row block of a field sharded over several GPUs takes the
 * global field's percentile, reduced on the host, and the global spacing).
 * Same arguments and scratch otherwise. */
int nbcs_ridge_pts_fmin(const double* f, const double* evec_max, const double* x, int32_t nx,
                        const double* y, int32_t ny, double dx, double dy, double sdd_thresh,
                        double f_min, uint8_t* mask_out, double* rpts_full, double* pts_out,
                        int64_t* n_out, void* scratch, size_t scratch_bytes, void* stream);

/* ftle_ordered_ridges (ridges.py:720-1054), host side: link the ridge points
 * of a ridge test (ridge_mask (nx, ny) u8 and r_pts (nx*ny, 2) as
 * nbcs_ridge_pts writes them, copied to the host) into curves, strongest
 * ridge first, and join curves whose endpoints lie within dist_tol with
 * tangents within ep_tan_ang; drops ridges shorter than min_ridge_pts as the
 * reference does.  All arrays are HOST memory (f (nx, ny), evec_max (nx, ny,
 * 2), x, y).  Output: the points of every ridge, one after another, in
 * pts_out (max_pts x 2) and each ridge's point count in ridge_len_out
 * (max_ridges); *n_pts, *n_ridges receive the totals (also when the buffers
 * are too small, which returns NBCS_ERR_SCRATCH).  Every ridge point belongs
 * to at most one ridge, so max_pts = max_ridges = number of mask points
 * always suffices. */
int nbcs_order_ridges(const double* f, const double* evec_max, const double* x, int32_t nx,
                      const double* y, int32_t ny, const uint8_t* ridge_mask, const double* r_pts,
                      double dist_tol, double ep_tan_ang, int64_t min_ridge_pts, double sdd_thresh,
                      double c, double* pts_out, int64_t max_pts, int64_t* ridge_len_out,
                      int64_t max_ridges, int64_t* n_pts, int64_t* n_ridges);

/* 8-connected component labels of a mask (nx, ny) u8 -> labels (nx, ny)
 * int32: 0 background, 1..n numbered by each component's first pixel in
 * row-major order, exactly as scipy.ndimage.label with a 3x3 structure
 * (the labelling step of ftle_ridges, ridges.py:219-222).  *nlabels (device
 * int32) receives n, or -1 if the union-find gave up (error flag). */
size_t nbcs_label8_scratch_bytes(int32_t nx, int32_t ny);
int nbcs_label8(const uint8_t* mask, int32_t nx, int32_t ny, int32_t* labels, int32_t* nlabels,
                void* scratch, size_t scratch_bytes, void* stream);

/* --------------------------------------------- learned step-size proposer */
/* No counterpart in the reference.  An 8 -> 64 -> 64 -> 1 ReLU MLP with BF16
 * weights and FP32 accumulation (tensor cores, mma.sync m16n8k16) that
 * proposes log h for the next DOP853 step from local flow features
 * (lon, lat, t, u, v, du/dx, du/dy, dv/dx); the embedded error estimate still
 * accepts or rejects every step.
 *   master parameters: float[nbcs_mlp_param_count()] =
 *     W1[64][8], b1[64], W2[64][64], b2[64], w3[64], b3
 *   blob (device, nbcs_mlp_blob_bytes(), 16-byte aligned): header of
 *     feature mean[8], feature 1/std[8], target mean, target std, b3, pad,
 *     b1[64], b2[64], w3[64] (floats), then W1 bf16[64][16] (inputs padded
 *     to 16 with zeros) and W2 bf16[64][64].  nbcs_mlp_pack fills everything
 *     but the normalisation constants, which the caller writes. */
size_t nbcs_mlp_blob_bytes(void);
int nbcs_mlp_param_count(void);
int nbcs_mlp_pack(const float* params, void* blob, void* stream);
/* predictions (target units) for n feature rows (n, 8) */
int nbcs_mlp_predict(const void* blob, const float* feats, int64_t n, float* out, void* stream);
/* gradient (float[param_count], overwritten) of sum_i (net_i - standardised
 * target_i)^2 / n with respect to the master parameters, and the unscaled
 * sum of squares in *loss; both device pointers */
int nbcs_mlp_grad(const void* blob, const float* feats, const float* targets, int64_t n,
                  float* grad, float* loss, void* stream);
/* one Adam step (bias-corrected, step >= 1) on the master parameters; if
 * blob != NULL it is repacked from them */
int nbcs_mlp_adam(float* params, float* m, float* v, const float* grad, float lr, float beta1,
                  float beta2, float eps, int32_t step, void* blob, void* stream);
/* Training data: integrate the grid with the mixed-precision plain
 * controller and, for a sampled fraction of the accepted steps that start
 * and end inside the velocity grid (a hash of particle and step, `sample` in
 * [0, 1]), write the features at the step start to
 * feats (capacity, 8) and the step that would have met the error target,
 * log(|h| * 0.9 * err^(-1/8)), to targets; *count (device uint64, caller
 * zeroes it) counts the samples offered, including any beyond capacity.
 * Spline flows only. */
int nbcs_flowmap_log_steps(const nbcs_flow* flow, double t0, double T, const double* x,
                           int32_t nx, const double* y, int32_t ny, const double* params,
                           int32_t np, double rtol, double atol, float sample, uint32_t seed,
                           float* feats, float* targets, int64_t capacity,
                           unsigned long long* count, void* stream);

/* Allocation-free variant of nbcs_ridge_pts.  No counterpart in the
 * reference: it exists for callers that cannot allocate device memory -- a
 * plugin whose host program keeps all cudaMalloc calls to itself, or a caller
 * binding this library through a thin FFI with no device allocator of its
 * own.  Same arguments and results as nbcs_ridge_pts, minus the scratch: the
 * scratch is a fixed array compiled into the library (about 8.4 MB, see
 * nbcs_ridge_noalloc_scratch_bytes), which every GPU that loads the library
 * holds until the process exits.  Grids above NBCS_RIDGE_NOALLOC_MAX_POINTS
 * points are rejected with NBCS_ERR_INVALID.  The first call on a device looks
 * up the array's device address with that device current; make it before any
 * stream capture.  The address is kept per device ordinal for the life of the
 * process: it belongs to the device's primary context (the one the CUDA
 * runtime uses) and is not looked up again after cudaDeviceReset, so do not
 * call this entry point after resetting the device or from another context
 * on it.  All calls share the array, so calls whose work overlaps on the GPU
 * race on it. */
#define NBCS_RIDGE_NOALLOC_MAX_POINTS (1L << 23)
size_t nbcs_ridge_noalloc_scratch_bytes(void);
int nbcs_ridge_pts_noalloc(const double* f, const double* evec_max, const double* x, int32_t nx,
                           const double* y, int32_t ny, double sdd_thresh, double percentile,
                           uint8_t* mask_out, double* rpts_full, double* pts_out, int64_t* n_out,
                           void* stream);

/* ------------------------------------------------------------ measurement */
/* No counterpart in the reference (which has no GPU path). */

/* Bounds-checked build (libnbcs_check.so, built with -DNBCS_CHECK by
 * `python -m numbacs_gb300.build --check`): the accesses whose index comes
 * from data -- the spline coefficient gathers of both integrators (the cell
 * of a particle's position), the composition's bilinear gathers, the
 * labelling's parent links -- test it against their buffer, skip the access
 * and set a bit instead of faulting.  nbcs_check_enabled() is 1 in that
 * build, 0 in the normal one (where nbcs_check_bits always reports 0).
 * nbcs_check_bits ORs the bits set since the last reset into *bits
 * (synchronous; reset != 0 clears them).  No counterpart in the reference. */
#define NBCS_CHECK_SPLINE_GATHER 0x1u
#define NBCS_CHECK_COMPOSE_GATHER 0x2u
#define NBCS_CHECK_LABEL_LINK 0x4u
int nbcs_check_enabled(void);
int nbcs_check_bits(uint32_t* bits, int32_t reset);

/* Number of kernels this library has launched in the process so far. */
unsigned long long nbcs_launch_count(void);

/* FMA throughput probe for the compute roofline: one launch of 8*SMs blocks
 * of 256 threads, 8 FMA chains each, `iters` iterations, in FP64 (precision
 * NBCS_PREC_FP64) or FP32.  `sink` is a device buffer of >= 64 KiB; *flops
 * (host) receives the flop count of the launch (an FMA counts 2). */
int nbcs_probe_fma(int32_t precision, int64_t iters, void* sink, double* flops, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* NBCS_H */
