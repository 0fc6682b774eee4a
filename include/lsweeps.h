/*
 * lsweeps.h -- C ABI of the GB300 L-sweeps library (liblsweeps_gb300.so).
 *
 * The library solves the 2D Helmholtz equation  -Lap u - omega^2 m(x) u = f
 * (5-point finite differences, cubic PML) with GMRES preconditioned by the
 * checkerboard L-sweep domain-decomposition preconditioner, on one GB300 GPU.
 * It replaces the hot path of the reference (paths relative to its root):
 *   DDCheckerboard            src/DDCheckerboard.cpp, include/DD.h:14-114
 *   SubdomainStructured       src/SubdomainStructured.cpp, include/Subdomain.h:20-227
 *   LocalLinearSolver         include/LocalLinearSolver.h:8-41 (EigenSparseLU ->
 *                             batched block-tridiagonal factorisation on the GPU)
 *   GlobalIterativeSolverGMRES src/GlobalIterativeSolverGMRES.cpp:65-348
 *   AssemblerHelmholtz2DFD / PMLCubic2D  src/AssemblerHelmholtz2DFD.cpp:371-457,
 *                             src/PMLCubic2D.cpp:35-236
 *
 * Conventions
 *   - The domain is [0, n_g h]^2 with n_g = N m + N - 1 elements per side
 *     (DDCheckerboard.cpp:119); the global DOF grid has n_dof = n_g + 2p - 1
 *     nodes per side (PML included), node G at coordinate (G + 1 - p) h.
 *   - Global vectors are complex128, interleaved (re, im), x-major with y
 *     fastest: index = Gx * n_dof + Gy (the reference's DOF order,
 *     AssemblerHelmholtz2DFD.cpp:166-177, applied globally).  A batch of nrhs
 *     vectors is stored back to back.
 *   - Pointers named *_dev are device pointers owned by the caller; *_host are
 *     host pointers.  `stream` is a cudaStream_t (NULL = legacy default stream).
 *   - Every call returns an lsw_status instead of exiting the process (the
 *     reference prints to cerr and calls exit(1)).  One context per host thread,
 *     or external locking; the library keeps no global state except the
 *     library-wide status strings, the sweep-front tuner's cache of measured
 *     launch shapes (per GPU and problem shape, behind a lock) and the fixed
 *     scratch array of lsw_local_solve_noalloc.
 */
#ifndef LSWEEPS_H
#define LSWEEPS_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum lsw_status {
  LSW_OK = 0,
  LSW_ERR_INVALID_ARGUMENT = 1,
  LSW_ERR_CUDA = 2,
  LSW_ERR_OUT_OF_MEMORY = 3,
  LSW_ERR_NOT_SET_UP = 4,
  LSW_ERR_NOT_FACTORIZED = 5,
  LSW_ERR_SINGULAR_BLOCK = 6,
  LSW_ERR_NOT_CONVERGED = 7,
  LSW_ERR_UNSUPPORTED = 8
} lsw_status;

/* Arithmetic of the subdomain factors and preconditioner applies.  The DD
 * matvec, Krylov vectors, Arnoldi and Hessenberg work are always FP64. */
typedef enum lsw_precision {
  LSW_PREC_C128 = 0, /* complex double factors and applies (reference arithmetic) */
  LSW_PREC_C64 = 1,  /* complex float factors and applies, FP32 accumulation */
  LSW_PREC_SPLIT = 2 /* complex float applies whose factor products run on the tensor cores:
                        every factor entry stored as two bf16 terms (hi + lo, 8 bytes per
                        complex value like complex float), three bf16 products per entry
                        (hi*hi + hi*lo + lo*hi) accumulated in FP32 */
} lsw_precision;

typedef enum lsw_gmres_mode {
  /* GlobalIterativeSolverGMRES::solve as written: left preconditioning, no
   * restart, x0 = M^-1 b, conjugate-first MGS dot, the reference's Givens
   * bookkeeping and a square solve of H (GlobalIterativeSolverGMRES.cpp:65-348).
   * Its logged residual is the parity quantity; it is not a true residual. */
  LSW_GMRES_REFERENCE = 0,
  /* Right-preconditioned flexible GMRES(restart), MGS, complex Givens; stops on
   * the true FP64 residual ||b - A x|| / ||b|| <= tol. */
  LSW_GMRES_FLEXIBLE = 1
} lsw_gmres_mode;

typedef struct lsw_ctx lsw_ctx;

/* DDCheckerboard::setUp arguments (DDCheckerboard.cpp:87-94) restricted to the
 * square case NCellsX == NCellsY, NX == NY, with the PML given in cells. */
typedef struct lsw_geom {
  int n_cells;       /* cells per side, N >= 1 */
  int n_els_in_cell; /* interior elements per cell side, m > 4 (DDCheckerboard.cpp:106-111) */
  int pml;           /* PML thickness in cells, p >= 1 */
  int order;         /* finite-difference order; only 2 (5-point) is supported */
  double h;          /* mesh size */
} lsw_geom;

typedef struct lsw_problem_info {
  int n_g;            /* elements per side of the physical domain */
  int n_dof;          /* DOFs per side of the global grid (PML included) */
  int n_cells_total;  /* N * N */
  int max_cell_side;  /* largest cell DOF count per side */
  int precision;      /* lsw_precision */
  int factorized;     /* 1 after lsw_factorize */
  long long factor_bytes;  /* bytes of the resident subdomain factors */
  long long device_bytes;  /* all device memory held by the problem */
  double omega;
  double pml_C;       /* PML absorption C = ln(omega) (Input.cpp:836) */
  long long kernel_launches; /* kernels launched by this context so far */
} lsw_problem_info;

/* Per-apply measurement of the sweep-front kernels (CUDA events around each
 * front launch on the caller's stream). */
typedef struct lsw_apply_profile {
  int fronts;            /* front launches per apply */
  int items;             /* front items (a cell and up to 16 of its right-hand sides) per apply */
  int slots;             /* right-hand sides over all cell solves */
  double front_ms;       /* summed device time of the front kernels */
  double total_ms;       /* device time of the whole apply */
  double alg_bytes;      /* algorithmic bytes of the front kernels: per cell and front
                            2 F + 4 R nx ny s, F = nx ny^2 s the factor, R its slots */
  double alg_flops;      /* 2 x 8 nx ny^2 R real flops per cell and front */
  double streamed_bytes; /* bytes the items stream: a cell whose slots are split over
                            several items reads its (padded) factor once per item */
} lsw_apply_profile;

/* One subdomain (SubdomainStructured) in local DOF coordinates:
 * local DOF (i, j) <-> global DOF (lo_x + i, lo_y + j). */
typedef struct lsw_cell_info {
  int I, J;            /* cell row (y) and column (x) */
  int nx, ny;          /* DOFs per side of the cell (x-lines, points per line) */
  int lo_x, lo_y;      /* global DOF index of local DOF 0 */
  int lines_x[2][4];   /* local x of trace0, trace1, traceN, traceNP; [0] non-shifted,
                          [1] shifted; -1 where the cell has no such trace */
  int lines_y[2][4];
  int own_x[2][2];     /* owned local range [lo, hi] along x (mValsToKeep*) */
  int own_y[2][2];
} lsw_cell_info;

typedef struct lsw_gmres_opts {
  int mode;        /* lsw_gmres_mode */
  double tol;      /* relative tolerance (reference default 1e-6) */
  int max_iter;    /* iteration cap (reference default 40) */
  int restart;     /* FGMRES restart length; ignored in reference mode */
  int verbose;     /* print the residual log to stdout */
} lsw_gmres_opts;

typedef struct lsw_gmres_report {
  int iterations;      /* iterations taken (max over the right-hand sides) */
  int converged;       /* 1 if every right-hand side met tol */
  double final_log;    /* last logged relative residual (max over rhs) */
  double true_rel_res; /* ||b - A x|| / ||b|| after the solve, FP64, max over rhs */
  double seconds;      /* wall time of the solve */
  int precond_applies; /* batched preconditioner applications (summed over sub-batches) */
  double* log;         /* optional caller buffer for the residual log of rhs 0 */
  int log_capacity;
  int log_len;
} lsw_gmres_report;

/* ---- context ------------------------------------------------------------- */
lsw_status lsw_ctx_create(lsw_ctx** ctx, int device);
lsw_status lsw_ctx_destroy(lsw_ctx* ctx);
const char* lsw_status_string(lsw_status s);
const char* lsw_ctx_last_error(const lsw_ctx* ctx);

/* Replay each preconditioner apply as a CUDA graph (enable = 1, the default;
 * LSW_GRAPHS=0 in the environment at context creation turns it off) or launch
 * its kernels one by one (enable = 0).  One graph per batch size is captured
 * on first use and captured again when the context's sweep pools are
 * reallocated or released; both ways run the same kernels on the same data and
 * give identical results.  A capture can be invalidated by CUDA calls that
 * other host threads make while it runs (allocations, frees, synchronous
 * copies) and can make such calls fail: callers that drive the library from
 * several threads at once turn graphs off.  A capture that fails is not an
 * error: the context then launches every apply's kernels directly.  No
 * counterpart in the reference (its applies are host loops over MPI ranks,
 * DDCheckerboard.cpp:687-739). */
lsw_status lsw_ctx_set_graphs(lsw_ctx* ctx, int enable);

/* Sweep-front launch shapes.  Each front (one launch per stage step, every
 * cell of the step, all four shifted decompositions and every right-hand side)
 * is cut into items of at most `slots_cap` right-hand-side slots of one cell,
 * each item a thread-block cluster of 2 x `cluster` CTAs (the two half chains
 * of the cell's twisted block solve).  With tuning on (enable = 1, the default;
 * LSW_TUNE=0 in the environment at context creation turns it off) the first
 * apply of a batch size measures every shape (slots 4, 8, 16 x CTAs 1, 2, 4
 * per half) on every front where it fits, with CUDA events on the call's
 * stream, and keeps each front's fastest; the choice is cached per GPU (UUID)
 * and problem shape for the process, and appended to the file named by
 * LSW_TUNE_CACHE when that is set (read back by later processes).  With
 * tuning off a cost model chooses.  Changing the setting drops the context's
 * schedules (rebuilt on next use; waits for the device).  No counterpart in the
 * reference (its sweeps are host loops, DDCheckerboard.cpp:812-880). */
lsw_status lsw_ctx_set_tuning(lsw_ctx* ctx, int enable);

/* Per-sweep launches for batches of at most `max_rhs` right-hand sides (2,
 * the default; LSW_SWEEP_LANES=<n> in the environment at context creation
 * sets it; 0 turns them off).  Such a batch runs every stage-2 sweep and every
 * L-sweep of the preconditioner as its own chain of launches on its own
 * stream, an L-sweep's step dd after its two producing stage-2 sweeps have
 * passed column / row dd + 1, so the L-sweeps start while stage 2 still runs
 * and the sweeps fill the GPU between one another's launches; their outputs go
 * to one plane per stage-2 sweep, summed at the end (four times the output
 * pool of one launch per step).  Results equal those of one launch per step up
 * to the order of the final sums.  Their launch shapes come from the cost
 * model, with each launch assumed to share the GPU with 2, 4 or 8 others of
 * its size (launches timed alone do not show that sharing): with tuning on
 * (lsw_ctx_set_tuning) the first apply of a batch size times one whole apply
 * per assumption and keeps the fastest, cached like the per-front shapes;
 * with tuning off the assumption is 4.  Changing the setting drops the
 * context's schedules (rebuilt on next use; waits for the device).  No counterpart in the reference (its sweeps are host loops,
 * DDCheckerboard.cpp:812-880). */
lsw_status lsw_ctx_set_sweep_lanes(lsw_ctx* ctx, int max_rhs);

typedef struct {
  int items;        /* items (cluster launches) in the front */
  int max_slots;    /* slots of the largest item */
  int slots_cap;    /* slots per item at most */
  int cluster;      /* CTAs per half chain */
  float tuned_ms;   /* the tuner's time for this front's shape; -1 when the cost model chose it */
  int tensor_cores; /* 1: the line products run on the tensor cores (complex64, tcgen05) */
} lsw_front_shape;

/* The launch shapes of the sweep fronts of a batch of nrhs right-hand sides
 * (building, and with tuning on measuring, the schedule if this batch size has
 * none yet, on `stream`): up to `capacity` entries in `out` (in launch order;
 * with per-sweep launches stage 1, then per stage-2 column the four sweeps,
 * then per stage-3 anti-diagonal the four L-sweeps), the launch count in
 * *n_fronts, the context's total tuning time so far in *tune_seconds (may be
 * NULL).  Requires a factorised problem. */
lsw_status lsw_front_shapes(lsw_ctx* ctx, int nrhs, lsw_front_shape* out, int capacity, int* n_fronts,
                            double* tune_seconds, void* stream);

/* Limit of every bounded wait inside the context's kernels (default ~2 s).
 * A wait that runs out makes its kernel give up and return normally; the call
 * that launched it then returns LSW_ERR_CUDA (results invalid).  No
 * counterpart in the reference (its blocking MPI_Recv waits without limit,
 * DDCheckerboard.cpp:976-1164). */
lsw_status lsw_ctx_set_wait_limit(lsw_ctx* ctx, double seconds);

/* Runs one bounded wait of the kernels' kind on a barrier that nothing
 * completes, with the context's limit: returns LSW_ERR_CUDA once the limit
 * has run out, and the context stays usable.  A check of the failure path for
 * deployments; no counterpart in the reference. */
lsw_status lsw_selftest_bounded_wait(lsw_ctx* ctx, void* stream);

/* Geometry of cell `cell` (index I*N + J) of a decomposition, computed on the
 * host without a GPU (DDCheckerboard::setUp trace limits, DDCheckerboard.cpp:214-419,
 * and SubdomainStructured::assignIndexSets, SubdomainStructured.cpp:1019-1116). */
lsw_status lsw_geometry_cell(const lsw_geom* geom, int cell, lsw_cell_info* out);

/* ---- problem ------------------------------------------------------------- */
/* DDCheckerboard::setUp (DDCheckerboard.cpp:87-645) + the assembler set-up of
 * Input::readAssemblerHelmholtz2DFD (Input.cpp:795-857): builds the cells,
 * trace geometry, sweep schedules and the device-resident operator.
 * m_grid_host: squared slowness on the n_dof x n_dof global grid (x-major). */
lsw_status lsw_problem_setup(lsw_ctx* ctx, const lsw_geom* geom, const double* m_grid_host,
                             double omega, int precision);
lsw_status lsw_problem_info_get(const lsw_ctx* ctx, lsw_problem_info* out);
lsw_status lsw_cell_info_get(const lsw_ctx* ctx, int cell, lsw_cell_info* out);

/* DDCheckerboard::factorize (DDCheckerboard.cpp:648-665) ->
 * LocalLinearSolverEigenSparseLU::factorize (LocalLinearSolverEigenSparseLU.cpp:40-62):
 * every cell factorised in one batched launch; idempotent. */
lsw_status lsw_factorize(lsw_ctx* ctx, void* stream);

/* DDCheckerboard::applyPrecond (DDCheckerboard.cpp:687-739): y = M^-1 x for a
 * batch of nrhs global vectors.  Asynchronous: it returns launch errors only;
 * a kernel that gave up on a bounded wait is reported (once) by the next call
 * that synchronises (lsw_apply_precond_profiled, lsw_gmres, lsw_local_solve). */
lsw_status lsw_apply_precond(lsw_ctx* ctx, const void* x_dev, void* y_dev, int nrhs, void* stream);

/* lsw_apply_precond with the front kernels timed by CUDA events; synchronises
 * the stream.  No counterpart in the reference (its only timers are
 * gettimeofday around factorize and GMRES, Problem.cpp:101-145). */
lsw_status lsw_apply_precond_profiled(lsw_ctx* ctx, const void* x_dev, void* y_dev, int nrhs, void* stream,
                                      lsw_apply_profile* prof);

/* DDCheckerboard::applySystemMatrix (DDCheckerboard.cpp:2611-2635): y = A x,
 * the global 5-point operator, FP64. */
lsw_status lsw_apply_A(lsw_ctx* ctx, const void* x_dev, void* y_dev, int nrhs, void* stream);

/* DDCheckerboard::assembleRHS (DDCheckerboard.cpp:668-684) with RHSSrcPts
 * (RHSSrcPts.cpp:87-112): Gaussian point sources of width = DD mesh size.
 * src_xy_host: nsrc (x, y) pairs; amp_host: nsrc amplitudes or NULL (= 1).
 * Writes one global vector. */
lsw_status lsw_assemble_rhs(lsw_ctx* ctx, const double* src_xy_host, const double* amp_host,
                            int nsrc, void* b_dev, void* stream);

/* GlobalIterativeSolverGMRES::solve (GlobalIterativeSolverGMRES.cpp:65-203)
 * on device vectors; every right-hand side of the batch is iterated in
 * lockstep and shares each preconditioner launch.  A batch whose Krylov bases
 * do not fit in free device memory is solved as consecutive sub-batches
 * (report: iterations and residuals are the maxima over all right-hand sides,
 * precond_applies the sum over the sub-batches). */
lsw_status lsw_gmres(lsw_ctx* ctx, const void* b_dev, void* x_dev, int nrhs,
                     const lsw_gmres_opts* opts, lsw_gmres_report* report, void* stream);

/* GlobalIterativeSolver::solve(rhs, res) (include/GlobalIterativeSolver.h:48)
 * on host buffers: copies b to the device, solves, copies x back. */
lsw_status lsw_solve_host(lsw_ctx* ctx, const double* b_host, double* x_host, int nrhs,
                          const lsw_gmres_opts* opts, lsw_gmres_report* report, void* stream);

/* Frees the context's solve workspaces: Krylov bases, sweep schedules and
 * their trace, output and scratch pools, lsw_solve_host's device copies of b
 * and x (they are rebuilt by the next call that needs them).  Factors and the problem stay resident.  No counterpart
 * in the reference (its workspaces are per-call Eigen vectors); a serving loop
 * calls it on idle operators to return device memory. */
lsw_status lsw_release_workspace(lsw_ctx* ctx);

/* LocalLinearSolver::solve (include/LocalLinearSolver.h:40) for one cell:
 * x = A_cell^-1 b on full cell vectors (nx*ny complex128, local order i*ny+j),
 * nrhs vectors back to back. */
lsw_status lsw_local_solve(lsw_ctx* ctx, int cell, const void* b_dev, void* x_dev, int nrhs,
                           void* stream);

/* Allocation-free variant of lsw_local_solve.  No counterpart in the reference.
 * For callers that cannot call cudaMalloc: processes whose device memory is
 * owned by their own pool under a fixed budget (a serving process that reserves
 * HBM up front), and latency-bound loops that cannot afford the device-wide
 * synchronisation an allocation may cause.  The caller passes only inputs and
 * outputs (same layout as lsw_local_solve); the call allocates nothing.  Its
 * scratch (descriptors and forward-substitution storage, ~nx*ny*8 bytes per
 * right-hand side in complex64, twice that in complex128) lives in one fixed
 * 8 MiB device array inside the library, which every GPU that loads the
 * library holds until the process exits; a request that does not fit returns
 * LSW_ERR_INVALID_ARGUMENT with the sizes in lsw_ctx_last_error.
 * lsw_ctx_create looks up that array's device address once, on the context's
 * device, and keeps it with the context.
 * All calls share the array: calls that overlap on the GPU (other streams,
 * other contexts on the same device) race and must be serialised by the
 * caller.  Nothing in the array needs clearing between calls: every element
 * is written before it is read.  Like lsw_local_solve, the call reads the
 * kernels' error word back and synchronises `stream` before it returns, so it
 * cannot be recorded into a CUDA graph (stream capture). */
lsw_status lsw_local_solve_noalloc(lsw_ctx* ctx, int cell, const void* b_dev, void* x_dev, int nrhs,
                                   void* stream);

#ifdef __cplusplus
}
#endif
#endif /* LSWEEPS_H */
