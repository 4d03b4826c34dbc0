/*
 * rtg.h -- C ABI of the GB300 radiative-transfer DG solve (librtg.so).
 *
 * The library applies the reference's steady monochromatic RT system
 *     A = (BC - IC) + (M - S)
 * matrix-free on one GPU and solves the interior/inflow split system of
 * rt/solve.py:81-132 with device-resident Krylov methods.  All entry points
 * take plain pointers and sizes; no exceptions cross the ABI.  Every function
 * returns RTG_OK (0) or a positive error code; rtg_last_error() gives the
 * message of the calling thread's last failure.  Vectors passed as "device"
 * live in GPU memory in the reference's global DOF order (sorted column keys,
 * sorted cell keys, beta = nth*ny*i + nth*j + a: dg/matrix/get_idxs.py:11-80).
 *
 * Reference interfaces replaced (src/ of jasonltorchinsky/radiative-transfer-amr):
 *   rtg_create            -- the per-call mesh walks of every rt builder
 *                            (rt/mass_matrix.py:23-106 and siblings); the mesh
 *                            arrives flattened (dg/mesh/class_Mesh.py:12-61)
 *   rtg_apply             -- rt.Problem.mass_matrix / scattering_matrix /
 *                            preconditioner_matrix / interior_convection_matrix /
 *                            boundary_convection_matrix followed by Mat.mult
 *                            (rt/mass_matrix.py:23, rt/scattering_matrix.py:22,
 *                            rt/preconditioner_matrix.py:22,
 *                            rt/interior_convection_matrix.py:25,
 *                            rt/boundary_convection_matrix.py:27)
 *   rtg_interior_mask     -- dg.matrix.get_intr_mask (dg/matrix/get_masks.py:22-129)
 *   rtg_split_vector /    -- dg.matrix.split_vector / merge_vectors
 *   rtg_merge_vectors        (dg/matrix/split_vector.py:15-48, merge_vectors.py:14-56)
 *   rtg_weight_forcing    -- the quadrature weighting of rt.Problem.forcing_vector
 *                            (rt/forcing_vector.py:103-155)
 *   rtg_solve             -- rt.Problem.solve (rt/solve.py:21-149)
 *   rtg_quad_nodes        -- dg.quadrature.quad_xyth (dg/quadrature/quad_xyth.py:22-86)
 */
#ifndef RTG_H
#define RTG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RTG_ABI_VERSION 1

/* status codes */
#define RTG_OK            0
#define RTG_ERR_ARG       1  /* bad argument (null pointer, size, flag) */
#define RTG_ERR_MESH      2  /* mesh description inconsistent */
#define RTG_ERR_CUDA      3  /* CUDA runtime error */
#define RTG_ERR_TIMEOUT   4  /* a bounded device wait gave up */
#define RTG_ERR_NONFINITE 5  /* NaN/Inf in an input or iterate */
#define RTG_ERR_SIZE      6  /* request exceeds a stated maximum */

/* rtg_apply component flags.  A plain combination adds the selected
 * reference matrices; RTG_SYSTEM selects A = (BC - IC) + (M - S) with the
 * (M - S) block and its |entry| <= 1e-14 drop rule taken from
 * rt/preconditioner_matrix.py:363-514. */
#define RTG_MASS      1u   /* + M   (rt/mass_matrix.py:108-180)                     */
#define RTG_SCAT      2u   /* + S   (reference sign: entries <= 0,
                                      rt/scattering_matrix.py:106-247)              */
#define RTG_IC        4u   /* + IC  (rt/interior_convection_matrix.py:110-250)      */
#define RTG_BC        8u   /* + BC  (rt/boundary_convection_matrix.py:160-540)      */
#define RTG_SYSTEM   16u   /* BC - IC + (M - S)                                      */
#define RTG_MASK_ROWS 32u  /* zero the rows of inflow-boundary DOFs in the output   */

/* precisions of rtg_apply / solver inner iterations */
#define RTG_FP64 0
#define RTG_FP32 1

/* learned correction of the sweep: network shape and training layouts */
#define RTG_NN_IN 16           /* physics features per row                      */
#define RTG_NN_HIDDEN 128      /* width of the two hidden layers                */
#define RTG_NN_MOM 8           /* moments of z per row (7 used, 1 pad)          */
#define RTG_NN_OUT 24          /* coefficients per row: C[3][RTG_NN_MOM]        */
#define RTG_NN_STATS 12        /* training statistics per row (10 used, 2 pad)  */
/* W1[16][128] b1[128] W2[128][128] b2[128] W3[128][24] b3[24] (FP32, row-major) */
#define RTG_NN_NPARAM 21784

typedef struct rtg_handle rtg_handle;

/* Flattened hp mesh.  Columns in sorted-key order; elements (leaf cells) in
 * global order: for each column, its cells in sorted-key order. */
typedef struct rtg_mesh_desc {
    int32_t ncols;
    int32_t nelem;
    const double*  col_pos;        /* [ncols*4] x0, y0, x1, y1                      */
    const int32_t* col_ndofs;      /* [ncols*2] nx, ny (nodes per direction)        */
    const int32_t* col_lv;         /* [ncols]   spatial refinement level            */
    const int32_t* col_nbr;        /* [ncols*8] neighbour column index per face F
                                      (0 right, 1 top, 2 left, 3 bottom) and slot
                                      (2 per face), -1 for none                      */
    const int32_t* col_elem_start; /* [ncols+1] first element of each column        */
    const double*  cell_pos;       /* [nelem*2] th0, th1                            */
    const int32_t* cell_ndof;      /* [nelem]   nth                                 */
    const int32_t* cell_lv;        /* [nelem]   angular refinement level            */
    const int32_t* cell_idx;       /* [nelem]   angular index at that level         */
    const int32_t* cell_quadrant;  /* [nelem]   0..3, or -1 for none                */
} rtg_mesh_desc;

/* Coefficients sampled at the nodes.  kappa/sigma: per column, nx*ny values at
 * (x_i, y_j), index i*ny + j, columns concatenated in order.  Phi: per
 * distinct column angular mesh ("signature"), the dense block
 * Phi(th_r, th'_a) over all angular nodes of the column in column order
 * (cells sorted, nodes ascending), row-major; col_sig maps columns to blocks. */
typedef struct rtg_coeffs {
    const double*  kappa;
    const double*  sigma;
    int32_t        nsig;
    const int64_t* sig_off;        /* [nsig+1] offsets into phi (in doubles)        */
    const double*  phi;
    const int32_t* col_sig;        /* [ncols]                                        */
} rtg_coeffs;

typedef struct rtg_info {
    int64_t ndof;          /* N                                  */
    int64_t ndof_interior; /* unknowns of the split system       */
    int32_t ncols;
    int32_t nelem;
    int32_t ncoupling;     /* face couplings to neighbour cells  */
    int32_t nsig;          /* distinct column angular meshes     */
    int32_t max_col_ndof;
    int32_t max_nth_col;
    int64_t table_bytes;   /* device bytes of operator tables    */
    int64_t bytes_per_apply_fp64; /* algorithmic bytes of one FP64 apply */
    int64_t bytes_per_apply_fp32;
    int64_t flops_per_apply;
} rtg_info;

typedef struct rtg_solve_opts {
    int32_t method;        /* 0: GMRES(restart) in FP64 (the plain method)
                              1: FP32 inner GMRES + FP64 iterative refinement   */
    int32_t restart;       /* Krylov subspace size (reference: 50)              */
    int32_t max_it;        /* total inner iterations cap (reference: 5000)      */
    double  rtol;          /* relative residual target on ||r||/||b||           */
    double  atol;          /* absolute residual target                           */
    int32_t precond;       /* 0 none, 1 upwind transport sweep (right precond.),
                              2 sweep + column diffusion correction (two-level,
                              FGMRES), 3 sweep + learned correction (FGMRES;
                              needs rtg_nn_set_params): once per handle and
                              inner precision, two timed 8-step cycles from
                              the first residual (sweep alone, then with the
                              correction) decide whether the correction stays;
                              it also falls back to 1 on a stall */
    int32_t nonzero_guess; /* 1: start from x (reference: x0 = f_I)             */
    double  inner_rtol;    /* method 1: inner FP32 reduction per outer step     */
    int32_t max_outer;     /* method 1: cap on refinement steps                 */
    int32_t verbose;
} rtg_solve_opts;

typedef struct rtg_solve_info {
    int32_t converged;     /* 1 converged, 0 hit max_it, <0 breakdown         */
    int32_t iterations;    /* inner Krylov iterations                          */
    int32_t outer;         /* refinement steps (method 1)                      */
    int32_t fp64_applies;
    int32_t fp32_applies;
    double  res0;          /* ||b - A x0||                                     */
    double  res_f;         /* final true residual ||b - A x|| (FP64)           */
    double  rhs_norm;      /* ||b||                                            */
    double  seconds;       /* wall time inside rtg_solve                       */
    int32_t hist_len;      /* residual history entries written                 */
    int32_t sweeps;        /* preconditioner (sweep) applications              */
    int32_t learned;       /* applications of the learned correction           */
    int32_t fallbacks;     /* precond 3: switches to the sweep alone (stalls)  */
    int32_t coarse;        /* applications of the diffusion correction         */
    int32_t trial_its;     /* precond 3: iterations of the learned-correction
                              trial run by this solve (0: decided earlier)    */
    int32_t learned_kept;  /* precond 3: 1 the trial kept the learned
                              correction, 0 the sweep alone was faster        */
} rtg_solve_info;

/* library / quadrature ------------------------------------------------------ */
int         rtg_abi_version(void);
const char* rtg_last_error(void);
/* Kernels the library has launched since it was loaded (host-side count of
 * launch statements, all handles and streams; a replay of a captured graph
 * counts the kernels it holds). */
int64_t rtg_launch_count(void);
/* kind 0: Legendre-Gauss-Lobatto (x, y), 1: Legendre-Gauss (th); ascending on
 * [-1, 1]; n in [1, 16]. */
int rtg_quad_nodes(int kind, int n, double* nodes, double* weights);

/* handle ---------------------------------------------------------------- */
int  rtg_create(const rtg_mesh_desc* mesh, const rtg_coeffs* coeffs, int device,
                rtg_handle** out);
void rtg_destroy(rtg_handle* h);
int  rtg_get_info(const rtg_handle* h, rtg_info* info);

/* operator -------------------------------------------------------------- */
/* y = Op(flags) x on `stream` (cudaStream_t, NULL = legacy default).
 * x, y: device arrays of N doubles (RTG_FP64) or floats (RTG_FP32); x and y
 * must not alias. */
int rtg_apply(rtg_handle* h, uint32_t flags, int prec, const void* x, void* y,
              void* stream);
/* Each precision's apply is autotuned on its first use: every plan shape of
 * the candidate list (16, 32 or 64 angular rows per work item; one CTA per
 * column or per work item; one launch, or one launch per shared-memory class
 * of the CTAs; FP32 also, with one CTA per column and 32 or 64 rows, with the
 * scattering product on the tensor cores, the scattering CTAs of one angular
 * mesh next to each other) is built and the whole apply timed; the fastest
 * is kept.  This returns the FP32 table (host, cap_rows rows of 9 int32: rows
 * per item, items per CTA (0: the whole column), split launches (0/1),
 * tensor-core scattering (0: none; 1: scattering CTAs heaviest first; 2:
 * grouped by angular mesh),
 * chosen (0/1), time in ns (-1: not timed), work items, CTAs, launches) and
 * the number of shapes, tuning first if needed. */
int rtg_apply_tuning(rtg_handle* h, int32_t* table, int cap_rows, int* nclasses, void* stream);
/* Fixes the apply plan of one precision to a shape instead of the autotuned
 * one: shape = {rows per item, items per CTA (0: whole column), split
 * launches (0/1), tensor-core scattering (0, 1 or 2 as above, FP32 only)}; NULL returns to
 * autotuning on the next apply.  Synchronizes the device and drops the
 * solver's captured graphs (they hold the old plan's launches). */
int rtg_apply_shape(rtg_handle* h, int prec, const int32_t* shape);
/* mask[N] (device, uint8): 1 for unknowns, 0 for inflow-boundary DOFs. */
int rtg_interior_mask(rtg_handle* h, uint8_t* mask, void* stream);
/* out = x with the entries of one part zeroed: part 0 keeps the unknowns,
 * part 1 keeps the inflow-boundary DOFs (device, doubles, in place allowed). */
int rtg_mask_vector(rtg_handle* h, int part, const double* x, double* out, void* stream);
/* Compact a full vector to its interior part (length ndof_interior) and back:
 * merge writes x_int at the unknowns and g at the inflow-boundary DOFs. */
int rtg_split_vector(rtg_handle* h, const double* x, double* x_int, void* stream);
int rtg_merge_vectors(rtg_handle* h, const double* x_int, const double* g, double* x,
                      void* stream);
/* z = P^{-1} r: the upwind transport sweep rtg_solve uses as its right
 * preconditioner (the GPU counterpart of the PETSc PC of rt/solve.py:125-127).
 * r, z: device arrays of N doubles (RTG_FP64) or floats (RTG_FP32); entries
 * of z at inflow-boundary DOFs are zero.  The first call builds the element
 * block inverses (device memory owned by the handle). */
int rtg_precondition(rtg_handle* h, int prec, const void* r, void* z, void* stream);
/* The sweep's wavefront levels, the couplings it lags (cycles of the upwind
 * graph) and the entries of its element block inverses (each held in FP32
 * and FP64); builds the sweep if needed.  Any output may be NULL. */
int rtg_sweep_info(rtg_handle* h, int* levels, int* lagged, int64_t* inverse_entries, void* stream);
/* The sweep's one-phase elements in precision prec (those whose upwind map
 * G_e = -B_e C_e, from upwind face values to the element's values, is applied
 * in one step after the inputs arrive: the elements with a map that fits the
 * launch shape the first sweep in that precision chose, or before it every
 * element with a map), and the map entries (BF16 in the FP32 sweep, FP64 in
 * the FP64 one) and upwind value indices one sweep in that precision reads;
 * builds the sweep if needed.  Any output may be NULL. */
int rtg_sweep_maps(rtg_handle* h, int prec, int* onephase, int64_t* map_entries, int64_t* upwind_entries,
                   void* stream);
/* One sweep as rtg_precondition, recording for every element e
 * trace[8e .. 8e+7] = {claimed, independent work done, published (GPU
 * global-timer nanoseconds), CTA, then SM clock cycles spent waiting for the
 * upwind face lines, forming T = Et z_upwind, forming the face couplings, and
 * applying the face columns of the block inverse with the stores} (device
 * array of 8*nelem uint64) and, when level (host, nelem int32) is not NULL,
 * each element's wavefront level.  A profiling aid: the sweep's cost is its
 * level count times the per-level latency these records resolve. */
int rtg_sweep_trace(rtg_handle* h, int prec, const void* r, void* z, uint64_t* trace, int32_t* level,
                    void* stream);
/* out_beta = (dx dy dth / 8) wx_i wy_j wth_a * fvals_beta (device doubles). */
int rtg_weight_forcing(rtg_handle* h, const double* fvals, double* out, void* stream);

/* solve ------------------------------------------------------------------ */
/* Solve A_II u_I = f_I - A_IB g_B (f, g full-length device vectors), writing
 * the merged solution u (device, N doubles).  With opts->nonzero_guess the
 * interior of u on entry is the initial guess.  hist (host, may be NULL)
 * receives up to hist_cap residual norms. */
int rtg_solve(rtg_handle* h, const double* f, const double* g, double* u,
              const rtg_solve_opts* opts, rtg_solve_info* info,
              double* hist, int hist_cap, void* stream);

/* The triangular factor R of the last Arnoldi cycle of the handle's last
 * rtg_solve (its Hessenberg after the Givens rotations), written column-major
 * into R (host, n*n doubles, zeros below the diagonal); *n = the cycle's
 * steps (0: no cycle ran; R untouched).  R may be NULL to query n.  The
 * singular values of R are those of the cycle's (n+1) x n Hessenberg: the
 * estimates of the preconditioned operator's extreme singular values that the
 * reference reads after its solve (rt/solve.py:110-115,
 * ksp.computeExtremeSingularValues(), which PETSc's GMRES computes from the
 * same factor).  For method 1 the cycle is the last FP32 inner cycle. */
int rtg_solve_hessenberg(rtg_handle* h, double* R, int cap, int32_t* n, void* stream);

/* Batched solve of independent problems held by one handle.  The handle's mesh
 * is the concatenation of nbatch instances' meshes (no couplings between
 * them; each instance with its own coefficients), instance b owning DOFs
 * [inst_off[b], inst_off[b+1]) (inst_off: host array of nbatch+1 offsets,
 * inst_off[0] = 0, inst_off[nbatch] = N).  Every operator apply and sweep
 * covers all instances in one launch; the Krylov state (inner products,
 * Hessenberg, Givens, convergence) is per instance and lives on the device;
 * one GMRES restart cycle is captured in a CUDA graph and replayed.
 * opts->method must be 1 (FP32 sweep-preconditioned GMRES inside FP64
 * iterative refinement); rtol/atol apply per instance.  infos (host, may be
 * NULL) receives nbatch entries.  Counterpart in the reference: a loop of
 * rt.Problem.solve calls (rt/solve.py:21-181), one per instance. */
int rtg_solve_batched(rtg_handle* h, int nbatch, const int64_t* inst_off, const double* f,
                      const double* g, double* u, const rtg_solve_opts* opts,
                      rtg_solve_info* infos, void* stream);

/* learned correction of the sweep --------------------------------------------
 * No counterpart in the reference.  rtg_solve with precond 2 runs FGMRES with
 * M(r) = z + L z, z = P^{-1} r (the sweep), L linear in z:
 *   a row is one (element, spatial node ij) pair, rows in element order then
 *   ij = i*ny + j;  m(z) = [m0, m1c, m1s, phi, em, cm, nm, 0] per row (angular
 *   moments of z at the node, the column's angular mean phi, the element mean
 *   of m0, the column mean of phi, its mean over the neighbour columns);
 *   o = C m with C (3 x 8) from a 16-128-128-24 ReLU network of 16 physics
 *   features of the row;  (L z) = o0 + o1 cos th + o2 sin th at the unknowns.
 * The coefficients C are computed when the network is set.  Training uses
 * per-row statistics of a target error e with t = (e - z)/s, s = rms(z):
 *   loss = sum_rows o^T G o - 2 q^T o + c,  o = C m(z)/s.
 * All array arguments are device pointers (params may also be host memory in
 * rtg_nn_set_params); prec selects double (RTG_FP64) or float (RTG_FP32)
 * vectors. */
int rtg_nn_rows(rtg_handle* h, int64_t* rows);
/* set the handle's network (RTG_NN_NPARAM floats) and compute its coefficients */
int rtg_nn_set_params(rtg_handle* h, const float* params, void* stream);
/* feat[rows][16]: the physics features of the handle's rows */
int rtg_nn_features(rtg_handle* h, float* feat, void* stream);
/* mom[rows][8] = m(z)/s and scale[0] = s = rms(z) */
int rtg_nn_moments(rtg_handle* h, int prec, const void* z, float* mom, float* scale, void* stream);
/* coef[rows][24] = network(feat); weights rounded to BF16, FP32 accumulation */
int rtg_nn_forward(const float* params, const float* feat, int64_t rows, float* coef, void* stream);
/* z += L z with the given coefficients (coef[rows][24]) */
int rtg_nn_correct(rtg_handle* h, int prec, const float* coef, void* z, void* stream);
/* stats[rows][12] of t = (e - z)/s times weight: G00 G01 G02 G11 G12 G22 q0 q1 q2 c 0 0 */
int rtg_nn_targets(rtg_handle* h, int prec, const void* z, const void* e, const float* scale, float weight,
                   float* stats, void* stream);
/* floats of scratch rtg_nn_loss_grad needs */
int64_t rtg_nn_work_floats(void);
/* loss (device double, may be NULL) and grad[RTG_NN_NPARAM] over `rows` rows */
int rtg_nn_loss_grad(const float* params, const float* feat, const float* mom, const float* stats, int64_t rows,
                     float* work, float* grad, double* loss, void* stream);
/* one Adam step (bias-corrected, decoupled weight decay wd) on all parameters */
int rtg_nn_adam(float* params, const float* grad, float* m, float* v, int step, float lr, float beta1,
                float beta2, float eps, float wd, void* stream);
/* z = M r = (I + L) P^{-1} r with the handle's network (the preconditioner of precond 3) */
int rtg_nn_precondition(rtg_handle* h, int prec, const void* r, void* z, void* stream);

/* error indicators and hp steering of the AMR loop -------------------------
 * Replace the reference's Error_Indicator methods (src/amr/Error_Indicator).
 * u: device FP64 solution, full length N in the global DOF order.  Outputs
 * are device FP64 arrays; errors are returned squared (the reference stores
 * their square roots).  The first call builds the indicator tables (angular
 * neighbours, face pairs with their interpolation matrices) on the handle. */
/* angular jump (error/error_angular_jump.py:14-98): per element
 * cell_err2[e] = 1/4 sum_ij wx_i wy_j (jl^2 + ju^2)/2, with jl, ju the jumps of
 * u at theta pull-back -1 and +1 against the lower and upper angular neighbour
 * cells of the column; col_err2[ncols] (may be NULL): sums over each column's
 * cells in order. */
int rtg_error_angular_jump(rtg_handle* h, const double* u, double* cell_err2, double* col_err2, void* stream);
/* spatial jump (error/error_spatial_jump.py:17-247): col_err2[ncols] = the
 * squared jumps of the column's face traces against every facing neighbour
 * cell, projected on the finer face interval's LGL rule (the larger node
 * count) times the smaller angular cell's LG rule and integrated, summed and
 * divided by perimeter * 2 pi. */
int rtg_error_spatial_jump(rtg_handle* h, const double* u, double* col_err2, void* stream);
/* hp-steering estimates (col_hp_steer.py:14-64, cell_hp_steer.py:15-48):
 * col_lp[ncols] from the Legendre coefficients of the angle-integrated
 * solution, cell_lp[nelem] from those of the space-integrated solution (either
 * may be NULL).  The reference refines a column in p when col_lp - 0.5 >=
 * (nx + ny)/2 and a cell when cell_lp - 0.5 >= nth, else in h. */
int rtg_hp_steer(rtg_handle* h, const double* u, double* col_lp, double* cell_lp, void* stream);

/* allocation-free inner products --------------------------------------------
 * No counterpart in the reference: the kind of reduction rtg_solve uses for
 * its Arnoldi inner products and residual norms (per-CTA partial sums added
 * in a fixed order; its own grid, so the last bits can differ), offered to callers
 * that may not allocate device memory (a host whose memory manager owns every
 * device allocation, or a caller running its own Krylov loop around
 * rtg_apply where a cudaMalloc would stall or break the surrounding work).
 * out[q] = sum_{i<n} V[q*ldv + i] * w[i] for q < k, written to the caller's
 * device array out (k doubles) on `stream`.  V, w, out: device pointers; ldv
 * >= n when k > 1 (ignored for k == 1).  k must be in [1, 64]: the per-CTA
 * partial sums live in one static device array of 296 x 64 doubles
 * (151,552 bytes) that every GPU loading the library holds until exit; k > 64
 * returns RTG_ERR_SIZE.  Nothing is allocated.  The first call on a device
 * looks up that array's device address (cudaGetSymbolAddress) with the device
 * current, so make the first call on each device before any stream capture.
 * All calls share the array: calls that overlap on the GPU race and must be
 * serialised by the caller; each call overwrites every partial sum it reads.
 * The array's address is cached per device: do not use the library across a
 * cudaDeviceReset. */
int rtg_dots_noalloc(int k, const double* V, int64_t ldv, const double* w, int64_t n,
                     double* out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* RTG_H */
