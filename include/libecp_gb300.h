/*
 * libecp_gb300.h -- entry points beside the drop-in interface.
 *
 * These have no counterpart in chrr/libECP; they expose what the GPU engine
 * adds: every block at once with a per-unit status, a device-resident job
 * that can be re-run without host traffic (benchmarks, serving), and the
 * pipe-throughput probe the roofline figures are quoted against.
 *
 * A "unit" is one (shell pair, ECP centre) combination.  Units are numbered
 * u = c * nPairs + p, c the rank of the ECP centre among atoms with an ECP,
 * p the rank of the shell pair in the reference's loop order (atom A, atom
 * B >= A, shell s1 of A, shell s2 of B, s2 >= s1 when A == B).  Each unit owns
 * two blocks (type 1 then type 2) of IJK(la) x IJK(lb) doubles.
 */
#ifndef LIBECP_GB300_H
#define LIBECP_GB300_H 1

#ifdef __cplusplus
extern "C" {
#endif

/* The arrays of getIntegrals (src/getIntegrals.h:7-13) in one struct. */
typedef struct {
  int nrAtoms;
  const double *geometry;
  const int *shellsECP, *KECP, *lECP;
  const double *nECP, *dECP, *aECP;
  const int *shellsBS, *lBS, *KBS;
  const double *dBS, *aBS;
  int largeGridOrder;
  double tolerance, accuracy;
  /* nuclear-derivative order n of libECP_init (src/libecp.h:15-21): 0, 1 or
   * 2.  With n > 0 every (shell pair, centre) carries the shifted blocks of
   * the reference's derivative scheme (src/libecp.c:240-248): (shifta,
   * shiftb) from {(0,0)} for n = 0, {(+1,0),(-1,0),(0,+1),(0,-1)} for n = 1,
   * {(+2,0),(-2,0),(+1,+1),(+1,-1),(-1,+1),(-1,-1),(0,+2),(0,-2),(+1,0),
   * (0,+1)} for n = 2, each a type-1 and a type-2 block of the shifted
   * Cartesian shells with coefficients times zeta^max(0, shift).  The AO
   * matrix (getIntegrals, ecpgb_getIntegrals) exists for n = 0 only. */
  int derivative;
  /* libECP_init's Cartesian order (src/libecp.h:15-21): NULL for libint's,
   * else the exponent triples of every Cartesian function of shells
   * l = 0..orderingLmax, shell by shell, in the caller's order within each
   * shell; blocks and the matrix then come out in that order.  The reference
   * requires orderingLmax >= maxL_ECP + 2 (max basis l + n) (src/libecp.c:159). */
  const int *shellOrdering;
  int orderingLmax;
} ecpgb_system;

enum {
  ECPGB_FP64 = 0,   /* plain FP64 kernels, one unit per CTA (the drop-in path) */
  ECPGB_FAST = 1,   /* batched FP64 path: a warp per primitive pair, quadrature
                       points tabulated level by level until convergence,
                       Horner-form Bessel rows, table-driven exp; same
                       schedules and decisions, rounding-level differences */
  ECPGB_MIXED = 2,  /* the batched path with the bulk radial arithmetic in
                       FP32: Bessel rows below the large-argument branch
                       (Horner in FP32 over FP32 Taylor coefficients) and the
                       ECP channel terms d r^n exp(-a r^2) (FP32 exp).  FP64
                       stays for the large-argument Bessel rows, the Gaussian
                       product exp prefactors, the quadrature sums and their
                       convergence tests, and every accumulation.  Errors are
                       those of FP32 (about 1e-7 relative to a block's
                       largest element): it does not meet the FP64 bar */
};

/* Unit status.  A large-grid (PSM92) quadrature that exhausts its levels keeps
 * its full-grid estimate and flags the unit; the reference frees its radial
 * table there and carries on with a dangling pointer (src/type2.c:612-617,
 * src/type1.c:245-247), which aborts the process in practice. */
enum {
  ECPGB_UNIT_DONE = 0,
  ECPGB_UNIT_SKIPPED = 1,     /* screened out: no callback in the reference   */
  ECPGB_UNIT_WARN_TYPE1 = 2,  /* blocks written; a type-1 large-grid
                                 quadrature did not meet its convergence test */
  ECPGB_UNIT_WARN_TYPE2 = 3,  /* blocks written; the same for type 2 only     */
};

typedef struct {
  long long units;        /* (pair, centre) units                        */
  long long emitted;      /* units that produced blocks                  */
  long long firstFailed;  /* first unit with a warning status, -1 if none */
  long long values;       /* doubles in the block layout                 */
  double msGpu;           /* device time of the last run (CUDA events)   */
  double msUnitKernel;    /* of which the per-unit kernel                */
  long long h2dBytes, d2hBytes;
} ecpgb_info;

/* Sizes of the block layout: units and doubles.  0 ok. */
int ecpgb_layout(const ecpgb_system *s, long long *nUnits, long long *nValues);

/* All blocks.  values[nValues] receives unit u's two blocks at
 * offsets[u] (type 1) and offsets[u] + IJK(la)*IJK(lb) (type 2); status[u]
 * one of ECPGB_UNIT_*.  offsets / status may be NULL.  0 ok, nonzero on set-up
 * errors (see ecpgb_last_error). */
int ecpgb_blocks(const ecpgb_system *s, int mode, double *values, long long *offsets,
                 int *status, ecpgb_info *info);

/* getIntegrals with a precision mode, a status and timings: returns 0 ok,
 * 1 set-up failed, 2 some unit carries a warning status (the matrix holds
 * every block; see ECPGB_UNIT_WARN_*). */
int ecpgb_getIntegrals(const ecpgb_system *s, int mode, int rowdim, double *I,
                       ecpgb_info *info);

/* Blocks in real spherical harmonics: both blocks of every emitted unit as
 * T(la) B T(lb)^T, T the reference's Cartesian -> real spherical matrices
 * (src/transformations.c:29-87, Schlegel and Frisch; rows m = -l..l) in the
 * job's Cartesian order, computed on the GPU.  T assumes Cartesian functions
 * each normalised on its own, so the caller's contraction coefficients must
 * carry those norms for the result to be the spherical functions' integrals.
 * Layout as ecpgb_blocks with 2 (2 la + 1)(2 lb + 1) values per unit
 * (ecpgb_layout_sph gives the sizes); ecpgb_cart2sph gives T(l),
 * (2l+1) x ncart(l), libint order.  No host CPU transform. */
int ecpgb_layout_sph(const ecpgb_system *s, long long *nUnits, long long *nValues);
int ecpgb_blocks_sph(const ecpgb_system *s, int mode, double *values, long long *offsets, int *status);
int ecpgb_cart2sph(int l, double *out);

/* Device-side consumers of the blocks.  With a symmetric density matrix D
 * (dim x dim, row stride ldD, the Cartesian AO order of getIntegrals):
 * *energy = sum_{mu nu} D_{mu nu} V_{mu nu} of the ECP matrix V, and
 * grad[3 * atom + k] = d energy / d R_{atom, k}, assembled on the GPU from the
 * derivative-order-1 blocks (d/dA of a Cartesian Gaussian = 2 zeta g(a + 1_k)
 * - a_k g(a - 1_k); the ECP centre by translational invariance), so only the
 * 3 nAtoms numbers come back.  Either output may be NULL.  s->derivative is
 * ignored.  0 ok, 1 error. */
int ecpgb_gradient(const ecpgb_system *s, int mode, const double *D, int ldD, double *energy, double *grad);

/* Device-resident job: inputs are copied to HBM once; ecpgb_job_run then
 * re-runs the whole pipeline (all kernels) nRuns times without host traffic,
 * writing one device-time per run (CUDA events on the engine's stream) to
 * msRun and the per-unit kernel's time to msUnit (either may be NULL).  With
 * flushL2 != 0 a 256 MiB buffer is written between runs, outside the timed
 * spans, so no run starts with a warm L2. */
typedef struct ecpgb_job ecpgb_job;
ecpgb_job *ecpgb_job_create(const ecpgb_system *s, int mode);
int ecpgb_job_run(ecpgb_job *j, int nRuns, int flushL2, float *msRun, float *msUnit);
int ecpgb_job_matrix(ecpgb_job *j, int rowdim, double *I); /* += last run's matrix */
long long ecpgb_job_units(const ecpgb_job *j, long long *emitted);
int ecpgb_job_kernel_launches(const ecpgb_job *j);           /* kernels per run */
void ecpgb_job_free(ecpgb_job *j);

/* Launch configuration of the batched path (ECPGB_FAST).  queue: 1 = a
 * persistent launch whose CTAs pull units from a work queue, 0 = one CTA per
 * unit; sorted: 1 = the queue holds the units by descending estimated cost
 * (primitive pairs x (la + lb + 2) x (L + 2)), 2 = grouped by (la, lb, L)
 * class (largest la + lb first), by that cost within a class, 0 = the
 * reference's order;
 * gcap: width cap of the type-1 step table in doubles per slot, which sets
 * the primitive pairs per warp and the CTAs per SM; balance: 1 = a unit with
 * few primitive pairs gets narrower type-1 groups so that all its warps
 * work; screen: 1 = with the queue launch, a screening stage first compacts
 * the queue to the units that compute blocks.  perClass: 1 = the autotuner
 * chose the type-1 cap and balance per (la, lb) class (see
 * ecpgb_job_class_config; gcap is then the cap the shared memory is sized
 * for); configurations set with ecpgb_job_config have none.  msUnit: the
 * unit kernel's time when the autotuner measured it, else 0. */
typedef struct {
  int queue, sorted, gcap, balance, screen, perClass;
  float msUnit;
} ecpgb_launch_config;

/* Autotuner: times each candidate configuration on the job (one untimed and
 * two timed runs each, unit kernel only), keeps the fastest for this job and
 * for later jobs of the same (max basis l, max ECP L) in this process, and
 * reports it in *chosen.  trials (may be NULL) receives up to maxTrials
 * candidates with their times; *nTrials the number written.  queue and sorted
 * leave every result bit for bit unchanged; gcap and balance regroup the
 * primitive pairs of the type-1 sums over warps, which moves results at
 * rounding level only.
 * 0 ok, 1 error, 3 the job is not a batched-path job. */
int ecpgb_job_tune(ecpgb_job *j, ecpgb_launch_config *chosen, ecpgb_launch_config *trials, int maxTrials,
                   int *nTrials);
/* The per-class type-1 settings of the job's configuration: for class
 * c = la * (max basis l + 1) + lb, c < n (at most 25), gcap[c] and
 * balance[c], or 0 and -1 where the class uses the job-wide gcap and balance.
 * 0 ok, 1 error. */
int ecpgb_job_class_config(ecpgb_job *j, int n, int *gcap, int *balance);
/* Sets (cfg != NULL) and/or reads (out != NULL) the job's configuration. */
int ecpgb_job_config(ecpgb_job *j, const ecpgb_launch_config *cfg, ecpgb_launch_config *out);
/* 1: ecpgb_job_run replays the pipeline as one captured CUDA graph (the
 * default); 0: plain stream launches. */
int ecpgb_job_use_graph(ecpgb_job *j, int on);
/* The last run's unit values (layout of ecpgb_blocks: unit u's blocks at
 * offset (u / nPairs) * centre stride + the pair's offset) and unit statuses;
 * either pointer may be NULL. */
int ecpgb_job_blocks(ecpgb_job *j, double *values, int *status);

/* Request server (continuous batching).  A worker thread admits submitted
 * jobs in arrival order as slots and device memory free up: each admitted
 * job is staged and run on its own CUDA stream while earlier ones are still
 * on the GPU, so their kernels overlap; the device-resident tables are shared
 * by all of them.  hbmBudgetBytes caps the device bytes the slots hold (a job
 * larger than the budget fails); slots caps the jobs in flight (1..64).  mode
 * is ECPGB_FP64 or ECPGB_FAST for every job of the server.  Results are those
 * of ecpgb_getIntegrals for the same system, mode and launch configuration,
 * bit for bit: a job runs the same kernels in the mix as alone. */
typedef struct ecpgb_server ecpgb_server;
typedef struct {
  long long units, values;  /* (pair, centre) units and block values of the job */
  double msQueued;          /* submit -> admitted (host clock) */
  double msLatency;         /* submit -> result ready (host clock) */
  double msGpu;             /* CUDA events around the job's stream work */
  long long deviceBytes;    /* device bytes of the job's slot while it ran */
  int slot, firstFailed;    /* firstFailed: first unit with a warning, -1 none */
} ecpgb_request_info;
typedef struct {
  long long submitted, completed, failed, queued, inflight;
  long long deviceBytesHeld, budget;
  int slots, maxInflight; /* maxInflight: most jobs seen on the GPU at once */
} ecpgb_server_stats;
ecpgb_server *ecpgb_server_create(int mode, long long hbmBudgetBytes, int slots);
/* Copies the system; returns the request id (>= 0) or -1 (see ecpgb_last_error). */
long long ecpgb_server_submit(ecpgb_server *sv, const ecpgb_system *s);
/* 0 queued or running, 1 done, -1 unknown id or failed. */
int ecpgb_server_poll(ecpgb_server *sv, long long id);
/* Blocks until the request is done, then I += its upper triangle (row stride
 * rowdim) and the request is released.  Returns like ecpgb_getIntegrals. */
int ecpgb_server_wait(ecpgb_server *sv, long long id, int rowdim, double *I, ecpgb_request_info *info);
int ecpgb_server_get_stats(ecpgb_server *sv, ecpgb_server_stats *st);
/* Finishes the jobs in flight and queued, then frees the server. */
void ecpgb_server_free(ecpgb_server *sv);

/* Readers for the text inputs of the reference's example program
 * (example/ex1.c:12-123): an xyz file (count, comment, "symbol x y z" lines,
 * coordinates used as given), an ECP file (per atom "index nCore nShells",
 * per shell "l K", per term "index a d n" -- or "d a n", the three-number
 * layout of the example's own ECP file, which the example's reader
 * misparses) and a basis file (per atom "index nShells", per shell "l K", per
 * primitive "index a d").  Every atom has an entry in both files.  The
 * system gets largeGridOrder 1024, tolerance 1e-12, accuracy 1e-14 (the
 * example's values, which the caller may change).  No GPU is needed.
 * Returns NULL on a missing file or a malformed line (ecpgb_last_error). */
typedef struct ecpgb_loaded ecpgb_loaded;
ecpgb_loaded *ecpgb_load_system(const char *xyzPath, const char *ecpPath, const char *basisPath);
const ecpgb_system *ecpgb_loaded_system(const ecpgb_loaded *L);
const char *ecpgb_loaded_symbol(const ecpgb_loaded *L, int atom);
void ecpgb_loaded_free(ecpgb_loaded *L);

/* Pipe-throughput probe on the current device: out[0] FP64 FMA TFLOP/s,
 * out[1] FP32 FMA TFLOP/s, out[2] MUFU ex2 Gop/s, out[3] FP64 exp() Gop/s.
 * Takes about 0.5 s.  0 ok. */
int ecpgb_measure_peaks(double *out);

/* getIntegrals for callers that cannot allocate device memory.  No
 * counterpart in the reference.  Meant for host programs that keep all GPU
 * memory in their own pool or arena, or that must not pay for (or risk the
 * failure of) an allocation inside a request.  Same arguments and result as
 * getIntegrals (accumulates into the upper triangle of I), computed by the
 * same kernels, but every device buffer comes from one fixed array of
 * ecpgb_noalloc_capacity() bytes (64 MiB) that each GPU loading the library
 * holds until the process exits; no CUDA allocation happens.  The first call
 * on a device looks up that array's address (make it before any stream
 * capture).  Calls share the array, so calls that overlap on the GPU race.
 * Returns 0 ok, 1 error (for instance a job larger than the array -- the
 * message gives the bytes needed), 2 some unit carries a warning status. */
int ecpgb_getIntegrals_noalloc(const ecpgb_system *s, int rowdim, double *I);
long long ecpgb_noalloc_capacity(void);

/* Selects the CUDA device this process's engine uses; call before any other
 * ecpgb_* or drop-in call (one process per GPU).  0 ok. */
int ecpgb_set_device(int device);

/* Text of the last error on this thread ("" if none). */
const char *ecpgb_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* LIBECP_GB300_H */
