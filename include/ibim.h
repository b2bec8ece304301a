/*
 * ibim-levelset GB300 — C ABI of the implicit-boundary-integral Poisson–Boltzmann path.
 *
 * One shared library (libibim_gb300.so, sm_103a) implements the reference's hot path
 * (GaZ3ll3/ibim-levelset) on one GPU: level-set tube quadrature (levelset.h/.cpp),
 * the black-box Chebyshev FMM (bbfmm.h/.cpp), restarted GMRES (gmres.h/.cpp) and the BIE
 * operator and solvation energy (electric.h/.cpp).  The C++ headers under include/ibim/
 * keep the reference's class interfaces on top of these entry points.
 *
 * Conventions
 *   - every entry point returns an int status (IBIM_OK = 0); ibim_last_error() gives text;
 *   - no exception crosses the ABI; no CPU fallback: a missing GPU is IBIM_ERR_CUDA;
 *   - handles are owned by the caller and released with the matching *_destroy;
 *   - "host" pointers are ordinary host memory; "_dev" entry points take device pointers;
 *   - lengths in Angstrom (the reference's electric() with rescale s = 1);
 *   - one CUDA stream per context; calls on one context are serialised by the caller.
 */
#ifndef IBIM_GB300_H
#define IBIM_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define IBIM_OK 0
#define IBIM_ERR_INVALID_ARGUMENT 1 /* bad size, null pointer, inconsistent handles */
#define IBIM_ERR_CUDA 2             /* CUDA runtime error (includes "no GPU") */
#define IBIM_ERR_OUT_OF_MEMORY 3    /* device allocation refused or above the context budget */
#define IBIM_ERR_UNSUPPORTED_KERNEL 4 /* kernel id outside the reference's kernel set */
#define IBIM_ERR_LIMIT 5            /* a bounded device loop (flood fill) hit its iteration cap */
#define IBIM_ERR_IO 6               /* unreadable or malformed input file */
#define IBIM_ERR_CALLBACK 7         /* a caller-supplied operator callback returned non-zero */

/* ---- kernel ids: the 16 kernels of electric.cpp:67-291, plus the fused forms ---- */
#define IBIM_K1X 0
#define IBIM_K1Y 1
#define IBIM_K1Z 2
#define IBIM_K2 3
#define IBIM_K3XX 4
#define IBIM_K3YY 5
#define IBIM_K3ZZ 6
#define IBIM_K3XY 7
#define IBIM_K3YZ 8
#define IBIM_K3ZX 9
#define IBIM_K3YX 10
#define IBIM_K3ZY 11
#define IBIM_K3XZ 12
#define IBIM_K4X 13
#define IBIM_K4Y 14
#define IBIM_K4Z 15
/* 4 densities (phi n_x w, phi n_y w, phi n_z w, dphi w) -> 4 fields
 * (F = K1.m - K2 dphi, G = H m - K4 dphi, H the K3 block): all 16 FMMs of one matvec
 * (electric.cpp:333-367) in one pass. */
#define IBIM_KERNEL_BIE_FUSED 16

/* ---- precision modes ---- */
#define IBIM_PRECISION_FP64 0  /* reference-exact FP64 path */
#define IBIM_PRECISION_MIXED 1 /* FP32-class far/near field inside FP64-class iterative refinement */
/* FP64 operator whose V-list M2L runs on the tensor cores as exact products of BF16 integer
 * digits (Ozaki scheme, a 42-bit cut into 6 digits of 7 bits, or 7 of 6 bits from order 6 up,
 * under power-of-two row/column scales; ~1e-11 of the
 * FP64 product): the operator of the mixed path's refinement residual.  Accepted by
 * ibim_fmm_plan (hence ibim_fmm_apply / ibim_bie_matvec), ibim_gmres_solve, and as a whole-solve
 * mode (ibim_config.precision: FP64 level set, plain FP64 GMRES on this operator). */
#define IBIM_PRECISION_FP64_TC 2

typedef struct ibim_ctx_s *ibim_ctx;
typedef struct ibim_grid_s *ibim_grid;
typedef struct ibim_tube_s *ibim_tube;
typedef struct ibim_plan_s *ibim_plan;

/* Solvent / kernel parameters (electric.cpp:52-58: solvent_kappa, solvent_dE, solvent_dI, tau).
 * k3_scaled (opt-in, 0 = the reference): 1 divides the K3 kernels by 4 pi like K1, K2 and K4
 * (electric.cpp:103-268 writes K3 without the factor; the difference vanishes at kappa = 0). */
typedef struct {
    double kappa, dE, dI, tau;
    int k3_scaled;
} ibim_kernel_params;

/* Everything input.cfg carries for this path, with the geometry explicit. */
typedef struct {
    double lo[3];      /* grid origin (levelset sx, sy, sz) */
    double h;          /* grid spacing (levelset dx) */
    int n[3];          /* grid size (Nx, Ny, Nz) */
    int band;          /* expand band in cells (main.cpp:45: 8) */
    double init;       /* initial grid value (main.cpp:47: -2 * size) */
    double probe;      /* probe radius (main.cpp:35: 1.4) */
    double reinit_t;   /* reinit pseudo-time, input.cfg `reinit_step` (main.cpp:56,60) */
    int thickness;     /* lvlset_thickness */
    double thres;      /* lvlset_thres */
    int np;            /* fmm_np (Chebyshev order) */
    int maxpoint;      /* fmm_maxpoint */
    int maxlevel;      /* fmm_maxlevel */
    ibim_kernel_params kp;
    int restart;       /* gmres_restart */
    int maxiter;       /* gmres_maxiter */
    double tol;        /* gmres_tol */
    int precision;     /* IBIM_PRECISION_* */
    int jacobian;      /* opt-in, 0 = the reference: 1 multiplies each tube weight by the surface
                          Jacobian 1 - phi (k1 + k2) + phi^2 k1 k2 of the level set through the
                          grid point (levelset.cpp:576 has no Jacobian) */
} ibim_config;

typedef struct {
    double energy;        /* polarized (solvation) energy, e^2/A (electric.cpp:499-505) */
    double area;          /* sum of quadrature weights, A^2 (electric.cpp:60) */
    long n_points;        /* tube points (POINTS NUM) */
    long inclusion;       /* cavity cells removed (INCLUSION) */
    int reinit_steps[2];  /* pseudo-time steps taken by the two reinitialisations */
    int gmres_iters;      /* Arnoldi steps */
    int matvecs;          /* operator applications (all precisions) */
    int matvecs_fp64;     /* FP64 operator applications */
    int gmres_status;     /* 0 converged, 1 not (gmres.cpp:186) */
    int refinements;      /* outer iterative-refinement passes (mixed precision) */
    double residual;      /* final relative residual ||b - A x|| / ||b|| */
    double t_levelset_ms, t_surface_ms, t_plan_ms, t_solve_ms, t_energy_ms;
    long grid_cells;      /* level-set grid cells */
    int levelset_stages;  /* TVD-RK3 stage sweeps (evolve + both reinitialisations) */
    long fmm_nodes, fmm_v_pairs, fmm_x_pairs, fmm_near_pairs, fmm_operators; /* tree work counts */
    double t_tree_ms;      /* part of t_plan_ms: octree, lists and work lists (host) with their uploads */
    double t_operators_ms; /* part of t_plan_ms: M2L operators and their tensor-core images (device) */
} ibim_result;

/* ---- context ---- */
int ibim_ctx_create(int device, ibim_ctx *out);
int ibim_ctx_destroy(ibim_ctx ctx);
const char *ibim_last_error(void);
const char *ibim_status_string(int status);
/* Fill a config with the reference defaults (data/input.cfg, main.cpp). */
void ibim_config_default(ibim_config *cfg);
/* The context's CUDA stream (cudaStream_t), for callers that record events on it. */
void *ibim_ctx_stream(ibim_ctx ctx);
/* Device memory freed by finished solves stays reserved in the device's stream-ordered pool
 * for the next solve; this returns it to the driver (no counterpart in the reference). */
int ibim_ctx_trim(ibim_ctx ctx);
/* Kernels this library has launched since load (all contexts). */
long ibim_launch_count(void);
/* Per-category kernel timing with CUDA events on the stream each launch runs on.  mask bit k
 * enables category k: 0 expand, 1 WENO stage, 2 gradient count, 3 flood fill, 4 tube extraction,
 * 5 M2L operators, 6 P2M, 7 M2M, 8 M2L (V list), 9 M2L (X list), 10 L2L, 11 near field (+ L2P
 * when it runs after the far field), 12 right-hand side, 13 GMRES vector kernels; FP64 versions of
 * 8, 9 and 11 are categories 14, 15 and 16 (categories 6-11 then count the mixed-precision
 * kernels); 17 is the V-list M2L of the mixed path's refinement residual (BF16 integer slices on
 * the tensor cores, FP64-class); 18 and 19 are the separate L2P of the mixed and FP64 paths when
 * the near field runs beside the far field (the default; IBIM_NEAR_OVERLAP=0 fuses them again),
 * in which case the near-field times overlap the far-field ones; 20 is the FP64-class near field
 * in float-float arithmetic on the FP32 pipes (IBIM_PRECISION_FP64_TC; IBIM_NEAR_FF=0 keeps the
 * native FP64 near field, category 16).
 * ibim_profile_read returns (and clears) the summed milliseconds and launch counts of the first
 * ncat categories. */
int ibim_profile_enable(ibim_ctx ctx, unsigned mask);
int ibim_profile_read(ibim_ctx ctx, double *ms, long *launches, int ncat);
/* Algorithmic flops and bytes of the profiled launches per category since the last read (call
 * before ibim_profile_read, which clears them). */
int ibim_profile_work(ibim_ctx ctx, double *flops, double *bytes, int ncat);
/* Measured FMA issue rate of the device: kind 0 = FP64, 1 = FP32 (TFLOP/s, 2 flops per FMA). */
int ibim_measure_peak(ibim_ctx ctx, int kind, double *tflops);

/* ---- level set: replaces Grid and levelset (levelset.h:12-60, levelset.cpp:9-432) ---- */
int ibim_grid_create(ibim_ctx ctx, int nx, int ny, int nz, double sx, double sy, double sz, double dx,
                     double value, ibim_grid *out);                          /* Grid(val, Nx, Ny, Nz) */
int ibim_grid_destroy(ibim_grid g);
int ibim_grid_upload(ibim_grid g, const double *host);                       /* row-major, k fastest */
int ibim_grid_download(ibim_grid g, double *host);
/* The grid's origin and spacing.  The reference keeps them on the levelset object
 * (levelset.h:35-38), not on Grid; the C++ drop-in sets them from its levelset before each call. */
int ibim_grid_set_geometry(ibim_grid g, double sx, double sy, double sz, double dx);
int ibim_grid_scale(ibim_grid g, double s);                                  /* Grid::operator*= */
int ibim_grid_copy(ibim_grid dst, ibim_grid src);                            /* Grid::operator= */
int ibim_levelset_expand(ibim_grid g, const double *centers, const double *radii, int natoms,
                         double probe, int band);                            /* levelset::expand */
int ibim_levelset_evolve(ibim_grid g, double final_t, double vel, double cfl); /* levelset::evolve */
int ibim_levelset_reinitialize(ibim_grid g, ibim_grid phi0, double final_t, double vel, double cfl,
                               int thickness, double thres, int *steps);    /* levelset::reinitialize */
int ibim_levelset_count_gradient(ibim_grid g, double thickness, double thres, long *bad, long *total,
                                 double *accum_error);                      /* levelset::countGradient */
/* main.cpp:45-60 in one call: expand, evolve inward by the probe, flip sign, reinit twice.
 * cfg->precision selects an FP64 grid or (IBIM_PRECISION_MIXED) an FP32 grid. */
int ibim_levelset_build(ibim_ctx ctx, const double *centers, const double *radii, int natoms,
                        const ibim_config *cfg, ibim_grid *out, int steps[2]);

/* Level-set evolution (as ibim_levelset_evolve) on a caller-owned FP64 device grid
 * (row-major, k fastest), enqueued on `stream` (a cudaStream_t; NULL = default stream), that
 * allocates no device memory.  No counterpart in the reference: it serves callers that cannot
 * let a library allocate (a fixed HBM budget in the caller's own pool, or a loop that must not
 * enter cudaMalloc/cudaFree).  Its two stage buffers live in one fixed array of
 * 2 x 524,288 doubles (8 MiB) that every GPU loading the library keeps until exit; grids of
 * more than 524,288 cells are rejected with IBIM_ERR_INVALID_ARGUMENT.  The first call on a
 * device looks up the array's device address with that device current.  All calls share the
 * array, so calls that overlap on the GPU race. */
int ibim_levelset_evolve_static(double *grid_dev, int nx, int ny, int nz, double dx, double final_t, double vel,
                                double cfl, void *stream);

/* ---- tube quadrature: replaces Surface (levelset.h:62-72, levelset.cpp:437-586) ---- */
int ibim_surface_extract(ibim_grid g, int thickness, ibim_tube *out, long *n_points, long *inclusion);
/* Surface extraction with the opt-in surface Jacobian (jacobian = 1, see ibim_config.jacobian;
 * no counterpart in the reference: its weights stop at levelset.cpp:576). */
int ibim_surface_extract_jacobian(ibim_grid g, int thickness, int jacobian, ibim_tube *out, long *n_points,
                                  long *inclusion);
/* A tube from host arrays (points (n,3), normals (n,3), raw cosine weights (n)) on spacing h. */
int ibim_tube_create(ibim_ctx ctx, const double *points, const double *normals, const double *weights, long n,
                     double h, ibim_tube *out);
int ibim_tube_destroy(ibim_tube t);
long ibim_tube_size(ibim_tube t);
/* Download in the reference's (i, j, k) order; any pointer may be NULL. */
int ibim_tube_download(ibim_tube t, double *points, double *normals, double *weights);

/* ---- black-box FMM: replaces bbfmm::tree / bbfmm::kernel (bbfmm.h:149-270) ---- */
/* Tree and interaction lists over the tube points (sources); targets = the tube points when
 * `targets` is NULL, else the nt host points given (e.g. atom centres, electric.cpp:432-489). */
int ibim_fmm_plan(ibim_tube src, const double *targets, long nt, int order, int maxpoint, int maxlevel,
                  int precision, ibim_plan *out);
int ibim_plan_destroy(ibim_plan p);
/* counts: nodes, levels, leaves, V pairs, X pairs, near-field pairs (source-target) */
int ibim_plan_stats(ibim_plan p, long stats[8]);
/* The tree and its U/V/W/X lists in the reference's node numbering (bbfmm.cpp:88-91), for
 * inspection: buf gets nnodes, then per node level, parent, leaf, empty, nsrc, and for each
 * list its length followed by its sorted node ids.  *needed receives the int count; call with
 * cap = 0 first to size buf.  `which` is reserved (0). */
int ibim_plan_lists(ibim_plan p, int which, int *buf, long cap, long *needed);
/* The same tree and lists built on the host from n points (n, 3), without a GPU. */
int ibim_tree_lists_host(const double *points, long n, int maxpoint, int maxlevel, int *buf, long cap, long *needed);
/* One FMM in the plan's precision.  kernel in [IBIM_K1X, IBIM_K4Z]: in is (ns), out is (nt);
 * IBIM_KERNEL_BIE_FUSED: in is (4, ns), out is (4, nt).  Host buffers, caller point order. */
int ibim_fmm_apply(ibim_plan p, int kernel, const ibim_kernel_params *kp, const double *in, double *out);

/* ---- BIE operator, GMRES, energy: replaces GMRES (gmres.h:20-21) and electric (electric.h:13) ---- */
/* y = dmapping(x) (electric.cpp:294-388) in the plan's precision, x, y of length 2N, host buffers,
 * reference order. */
int ibim_bie_matvec(ibim_plan p, const ibim_kernel_params *kp, const double *x, double *y);
/* load (electric.cpp:395-412): b of length 2N. */
int ibim_bie_rhs(ibim_plan p, const ibim_kernel_params *kp, const double *centers, const double *charges,
                 int natoms, double *b);
/* GMRES(m, max_iter, tol) on the BIE operator from x (in/out, 2N) (gmres.cpp:50-164). */
int ibim_gmres_solve(ibim_plan p, const ibim_kernel_params *kp, const double *b, double *x, int restart,
                     int maxiter, double tol, int precision, int *iters, int *gmres_status, double *residual);
/* A linear operator applied by the caller on host vectors: y = A x, both of length n.  Return 0
 * to continue; any other value stops the solve that called it. */
typedef int (*ibim_apply_fn)(void *user, const double *x, double *y, long n);
/* GMRES(m, max_iter, tol) on an arbitrary operator: the reference's
 * int GMRES(std::function<Vector(Vector&)> A, Vector& x, Vector& b, int m, int max_iter, scalar_t tol)
 * (gmres.h:20-21, gmres.cpp:50-164).  The Krylov basis, modified Gram-Schmidt and the updates run
 * on the context's GPU in FP64 with the reference's Givens rotations and restarts; each product
 * goes to the host, through `apply`, and back.  b and x (in/out, the initial guess) are host
 * vectors of length n; the first product is A x, as in the reference, so *matvecs counts the
 * same operator applications as the reference's GMRES makes.  A callback returning non-zero
 * ends the solve with IBIM_ERR_CALLBACK and x unchanged. */
int ibim_gmres_host(ibim_ctx ctx, long n, ibim_apply_fn apply, void *user, const double *b, double *x, int restart,
                    int maxiter, double tol, int *iters, int *matvecs, int *gmres_status, double *residual);
/* electric() after Surface: RHS, GMRES, polarizeMap, energy (electric.cpp:9-505).
 * x (2N) and atom_potential (natoms) may be NULL. */
int ibim_electric(ibim_tube tube, const double *centers, const double *charges, int natoms,
                  const ibim_config *cfg, double *x, double *atom_potential, ibim_result *res);

/* ---- whole path: main.cpp:45-77 for explicit geometry ---- */
/* Host atom arrays (centers (n,3), charges, radii). */
int ibim_solve(ibim_ctx ctx, const double *centers, const double *charges, const double *radii, int natoms,
               const ibim_config *cfg, ibim_result *res);
/* Same with the atoms already resident on the device (centers (n,3), charges, radii). */
int ibim_solve_dev(ibim_ctx ctx, const double *centers_dev, const double *charges_dev, const double *radii_dev,
                   int natoms, const ibim_config *cfg, ibim_result *res);
/* PQR file (molecule.h:21-50: ATOM lines, tokens 5..9 = x y z q r). */
int ibim_solve_pqr(ibim_ctx ctx, const char *pqr_path, const ibim_config *cfg, ibim_result *res);

/* ---- many molecules in one launch per FMM stage (no counterpart in the reference: main.cpp solves
 * one molecule per run; the operator batched is dmapping, electric.cpp:294-388) ----
 * Solves nmol molecules on the mixed-precision path.  Worker threads (`workers`, each with its own
 * context) prepare molecules in order (level set, tube, right-hand side, plan, operator images)
 * while the device bytes of prepared molecules stay within hbm_budget_bytes (<= 0: 150e9).  Up to
 * max_wave prepared molecules form a wave: their plans are merged into one (sources, nodes,
 * operators, pairs and near-field work concatenated), so each FMM stage of a matvec is one launch
 * over the wave, and GMRES advances every molecule of the wave in lock-step (one merged matvec per
 * Arnoldi step, one host synchronisation per step for all molecules' Givens rotations), inside
 * the FP64 iterative refinement of IBIM_PRECISION_MIXED with one merged FP64-class residual per
 * pass.  wave_slots (1..4) waves run at once, each on its own stream.  Molecules must share h, fmm_np, eps_in/eps_out, tau, k3_scaled, restart and jacobian;
 * kappa, geometry, atoms and tolerances may differ; precision must be IBIM_PRECISION_MIXED.
 * Atoms of molecule i are rows aoff_i .. aoff_i + natoms[i] - 1 of centers (n, 3), charges and
 * radii, aoff_i = natoms[0] + ... + natoms[i-1].  results[i] and statuses[i] per molecule; the
 * call returns the first failing molecule's status (others still solved).  done_ms (may be NULL)
 * receives when each molecule's result was final, in ms since the call began (its latency when
 * all are submitted at once).  info (may be NULL, 9 doubles): waves, largest wave, peak budgeted
 * bytes, merged mixed matvecs, merged FP64-class matvecs, mean fraction of a wave's molecules
 * still iterating per merged matvec, ms spent in waves (merge, solve, energy), device bytes the
 * prepared molecules held, and the FMM-phase estimates they were admitted with. */
int ibim_batch_solve(ibim_ctx ctx, int nmol, const int *natoms, const double *centers, const double *charges,
                     const double *radii, const ibim_config *cfgs, int max_wave, int wave_slots,
                     double hbm_budget_bytes, int workers, ibim_result *results, int *statuses, double *done_ms,
                     double *info);

/* ---- launch-parameter table and autotuner (no counterpart in the reference) ----
 * A plan of Chebyshev order p with N sources takes its launch parameters from the row of order p
 * with the largest min_points <= N: pairs per work segment of the FP32 and the float-float near
 * fields, and the tensor-core M2L's launch form (2 = two CTAs of two row tiles per SM, 4 = one CTA
 * of four, 0 = persistent, 6 / 7 = CTA pairs of 2-SM MMAs with one / two row-tile pairs per CTA;
 * 0, 6 and 7 in the scaled FP16 operand form).  They change the partition of the same work only.
 * Without a row the defaults hold (2^17, 2^14, 2). */
int ibim_tuning_set(int order, long min_points, long near_seg_pairs, long nearff_seg_pairs, int tc_form);
int ibim_tuning_clear(void);
/* out: near_seg_pairs, nearff_seg_pairs, tc_form for order and npoints */
int ibim_tuning_get(int order, long npoints, long out[3]);
/* Rows "order min_points near_seg_pairs nearff_seg_pairs tc_form" ('#' starts a comment). */
int ibim_tuning_load(const char *path);
/* Times candidate launch parameters on this molecule (mixed path): for each, a plan prepared under
 * it and the CUDA-event time of a solve's mix of products (25 mixed, one FP64-class residual),
 * one coordinate at a time (launch form, FP32 segments, float-float segments), each over at least
 * reps and about 30 ms of products; a best other than the defaults is kept only when a second
 * measurement of both confirms it by 2 %.  report (7 doubles): tube points, best near_seg_pairs,
 * nearff_seg_pairs, tc_form, best cost ms, default cost ms, candidates timed.
 * install_min_points >= 0 adds the best as the row (order, it). */
int ibim_autotune(ibim_ctx ctx, const double *centers, const double *charges, const double *radii, int natoms,
                  const ibim_config *cfg, int reps, long install_min_points, double *report);

/* ---- request loop (no counterpart in the reference: main.cpp solves one molecule per run) ----
 * Solve requests queue in arrival order and are admitted by device memory in two phases: the
 * head of the queue starts (its level set) when its grids fit in hbm_budget_bytes beside what the
 * requests in flight hold; once its octree and lists are built, its FMM phase (operator images,
 * expansions, Krylov basis) waits until the bytes its exact operator, node and point counts need
 * fit.  A phase is always admitted when no other request holds memory of that phase.  Each
 * request keeps its level set, tree, operators and Krylov basis resident until it finishes.
 * ibim_server_create: `slots` worker threads, each with its own context and stream, run whole
 * solves concurrently on the device. */
typedef struct ibim_server_s *ibim_server;
int ibim_server_create(int device, int slots, double hbm_budget_bytes, ibim_server *out);
/* Lock-step request loop (mixed-precision requests): `workers` threads prepare admitted requests
 * (level set, tube, right-hand side, plan, operator images) while two solver threads, each on its
 * own stream, take the prepared ones in waves of up to max_wave requests of one shape (h, fmm_np,
 * eps, tau, restart):
 * a wave's plans are merged so that each FMM stage is one launch for all of them, and their GMRES
 * iterations advance together (as ibim_batch_solve).  Requests arriving while a wave runs are
 * prepared meanwhile and join the next wave.  Same submit / poll / wait / stats / destroy. */
int ibim_server_create_lockstep(int device, int workers, int max_wave, double hbm_budget_bytes, ibim_server *out);
/* Waits for every queued and running request, then stops the workers. */
int ibim_server_destroy(ibim_server s);
/* Queue one whole solve (as ibim_solve; inputs are copied); *id identifies it. */
int ibim_server_submit(ibim_server s, const double *centers, const double *charges, const double *radii, int natoms,
                       const ibim_config *cfg, long *id);
/* *done = 1 once finished, with the solve's status, result, latency (submit to finish) and run
 * time (start to finish) in ms; a finished request is collected by the call that reports it. */
int ibim_server_poll(ibim_server s, long id, int *done, int *status, ibim_result *res, double *latency_ms,
                     double *run_ms);
int ibim_server_wait(ibim_server s, long id, int *status, ibim_result *res, double *latency_ms, double *run_ms);
/* submitted, completed, in flight, queued, bytes admitted in flight, peak bytes admitted, budget,
 * waves run (lock-step loop; 0 for the pool) */
int ibim_server_stats(ibim_server s, double stats[8]);
/* A solve's device footprint estimated from its configuration alone (before its level set). */
double ibim_request_bytes_estimate(const ibim_config *cfg);
/* The FMM phase's device footprint for a tube of npoints points, estimated before the tree is
 * built (the request loops admit that phase with the built tree's exact counts). */
double ibim_fmm_bytes_estimate(const ibim_config *cfg, long npoints);

#ifdef __cplusplus
}
#endif
#endif
