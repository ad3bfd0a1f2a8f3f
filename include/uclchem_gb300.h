/*
 * uclchem_gb300 — C ABI of the GB300 batched chemistry solver.
 *
 * This is the drop-in seam for UCLCHEM's chemistry integration hot path: the
 * calls that UCLCHEM's Fortran makes inside updateChemistry /
 * integrateODESystem (rate coefficients, the generated RHS, DVODE) are
 * replaced by batched calls that run many grid points at once on one GPU.
 *
 * Conventions
 *  - plain C types only; every array is caller-owned host memory unless the
 *    name says "_dev" (device pointer, caller-owned, on the context's device);
 *  - abundance vectors are NEQ = nspec+1 doubles (species then density), the
 *    layout of abund(:,dstep) in src/fortran_src/chemistry.f90:40;
 *  - batched arrays are system-major: system s occupies [s*NEQ, (s+1)*NEQ);
 *  - every function returns 0 on success or a negative UCL_E_* code, never
 *    aborts; per-system status words reuse UCLCHEM/DVODE numbering;
 *  - one context per host thread; calls on one context are serialised; each
 *    context owns one CUDA stream.
 */
#ifndef UCLCHEM_GB300_H
#define UCLCHEM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* Error codes (library level).                                              */
#define UCL_OK 0
#define UCL_E_ARG (-101)      /* invalid argument / size                     */
#define UCL_E_CUDA (-102)     /* CUDA runtime error                          */
#define UCL_E_NOMEM (-103)    /* device allocation failed / over budget      */
#define UCL_E_NET (-104)      /* network file unreadable or inconsistent     */
#define UCL_E_UNSUPPORTED (-105) /* option outside the supported path        */
#define UCL_E_TIMEOUT (-106)  /* a bounded device wait expired               */
#define UCL_E_AGAIN (-107)    /* not now: take finished requests first         */

/* Per-model status words: UCLCHEM's error codes, constants.f90:22-27. */
#define UCL_PARAMETER_READ_ERROR (-1)
#define UCL_PHYSICS_INIT_ERROR (-2)
#define UCL_CHEM_INIT_ERROR (-3)
#define UCL_INT_UNRECOVERABLE_ERROR (-4)
#define UCL_INT_TOO_MANY_FAILS_ERROR (-5)
#define UCL_NOT_ENOUGH_TIMEPOINTS_ERROR (-6)

/* Number of physics columns per output row (io.f90:74-81):
 * time [yr], density, gasTemp, dustTemp, Av, radfield, zeta, point. */
#define UCL_N_PHYS 8

/* ------------------------------------------------------------------------ */
/* Model parameters: the fields of UCLCHEM's parameter dictionary that the
 * chemistry path reads (src/fortran_src/defaultparameters.f90:18-119).
 * Defaults (including the single-precision rounding of the reference's
 * default-REAL literals) are filled by ucl_params_default().               */
typedef struct ucl_model_params {
  double initialTemp, initialDens, finalDens, finalTime;
  double radfield, zeta, rout, rin, baseAv;
  double freezeFactor, freefallFactor;
  double metallicity;
  double fh, fhe, fc, fo, fn, fs, fmg, fsi, fcl, fp, ff, fd, fli, fna, fpah,
      f15n, f13c, f18o;
  double reltol, abstol_factor, abstol_min;
  double ebmaxh2, ebmaxcr, ebmaxuvcr, epsilon, uv_yield, phi, uvcreff, omega;
  int32_t freefall, endAtFinalDensity;
  int32_t desorb, h2desorb, crdesorb, uvdesorb, thermdesorb;
  int32_t ion, points, mxstep;
  int32_t enforceChargeConservation, improvedH2CRPDissociation;
  int32_t cosmicRayAttenuation; /* column-density CR attenuation, physics-core.f90:121-157 */
  int32_t ionModel;             /* 'L' or 'H' (character code), defaultparameters.f90:47 */
  /* physics module: 0 = the static/freefall CLOUD of cloud.f90; 1-4 = the
   * parameterised prestellar-core collapse of collapse.f90 (Priestley et al.
   * 2018): 1 'BE1.1', 2 'BE4', 3 'filament', 4 'ambipolar', the collapse
   * argument of uclchem.model.collapse (model.py:355, wrap.f90:83-152) */
  int32_t collapse;
  /* hot-core physics module (hotcore.f90): the temp_indx 1-6 of
   * uclchem.model.hot_core (model.py:429-524; the protostar mass 1, 5, 10,
   * 15, 25, 60 Msun of the temperature ramp), 0 = off */
  int32_t hotcore;
  double maxTemperature; /* the ramp's final temperature (K), max_temperature */
} ucl_model_params;

/* Fill *p with the reference defaults (defaultparameters.f90:18-119). */
void ucl_params_default(ucl_model_params* p);

/* ------------------------------------------------------------------------ */
/* Network tables (compiled from MakeRates' network.f90 + odes.f90).         */
typedef struct ucl_network ucl_network;

/* Load a compiled network blob ("UCLNET01", written by
 * uclchem_gb300/network.py).  Replaces the compile-time PARAMETER arrays of
 * src/fortran_src/network.f90:4-5169 and the generated odes.f90. */
int ucl_network_load(const char* path, ucl_network** out);
void ucl_network_free(ucl_network* net);
int ucl_network_nspec(const ucl_network* net);
int ucl_network_nreac(const ucl_network* net);

/* ------------------------------------------------------------------------ */
/* Context: device tables + workspace on one GPU.                            */
typedef struct ucl_ctx ucl_ctx;

/* Solver precision for the Newton matrix: FP64 LU (plain path) or FP32 LU
 * of the error-weight-equilibrated matrix refined by the FP64 Newton
 * iteration (mixed path).  Rates, RHS, Nordsieck history, error norms and
 * step control are FP64 in both. */
#define UCL_PREC_FP64 0
#define UCL_PREC_MIXED 1

/* Create a context on CUDA device `device` for network `net` (copied to the
 * device).  `hbm_budget` bounds the bytes of per-system workspace the
 * context may hold (0 = library default).  Replaces the one-time set-up of
 * initializeChemistry (src/fortran_src/chemistry.f90:46-141). */
int ucl_ctx_create(const ucl_network* net, int device, size_t hbm_budget,
                   ucl_ctx** out);

/* A context holding several networks (e.g. networks of different sizes), so
 * that one launch can integrate models of all of them
 * (ucl_solve_models_nets_device).  Network k is nets[k].  Every per-model
 * array of every entry point then uses the strides of the largest network:
 * ucl_ctx_nspec() species columns, ucl_ctx_nspec()+1 start-vector entries and
 * ucl_ctx_nreac() rate columns per row; a smaller network fills the leading
 * part.  The single-system probes (ucl_rates_batch, ucl_rhs_batch,
 * ucl_jac_batch) evaluate network 0.  No counterpart in the reference,
 * whose network is fixed at compile time. */
int ucl_ctx_create_multi(const ucl_network* const* nets, int nnets, int device,
                         size_t hbm_budget, ucl_ctx** out);
int ucl_ctx_nspec(const ucl_ctx* ctx); /* largest nspec of the context's networks */
int ucl_ctx_nreac(const ucl_ctx* ctx); /* largest reaction count */
void ucl_ctx_destroy(ucl_ctx* ctx);

/* Rate coefficients for `nsys` systems.  Replaces calculateReactionRates
 * (src/fortran_src/rates.f90:21-343) as called from updateChemistry
 * (chemistry.f90:179-203): the surface/bulk totals of abund are refreshed
 * (chemistry.f90:192-199) before the rates are evaluated.
 *   params   [nsys]           model parameters
 *   abund    [nsys*NEQ]       abundances + density (in/out: totals refreshed)
 *   av       [nsys]           visual extinction of each system
 *   phi      [nsys]           in: the CR-desorption yield the DESCR rates use
 *                             (the parameter, or what the previous evaluation
 *                             left); out: the grain-assisted recombination
 *                             parameter of the GAR rates, which the reference
 *                             stores in the same variable (rates.f90)
 *   rates    [nsys*nreac]     out */
int ucl_rates_batch(ucl_ctx* ctx, int nsys, const ucl_model_params* params,
                    double* abund, const double* av, double* phi,
                    double* rates);

/* Right-hand side F(t, y) for `nsys` systems.  Replaces F / GETYDOT
 * (src/fortran_src/chemistry.f90:294-352, odes.f90:6-5181).  The H2 and CO
 * photodissociation rates are re-evaluated from y as F does
 * (chemistry.f90:315-318); `rates` is not modified.
 *   y     [nsys*NEQ], rates [nsys*nreac], av [nsys], ydot [nsys*NEQ] out */
int ucl_rhs_batch(ucl_ctx* ctx, int nsys, const ucl_model_params* params,
                  const double* y, const double* rates, const double* av,
                  double* ydot);

/* Analytic Jacobian dF/dy for `nsys` systems, dense row-major NEQ x NEQ per
 * system: jac[s*NEQ*NEQ + i*NEQ + j] = dF_i/dy_j (the matrix DVODE's MITER=2
 * branch approximates by finite differences, dvode.f90:8331-8355). */
int ucl_jac_batch(ucl_ctx* ctx, int nsys, const ucl_model_params* params,
                  const double* y, const double* rates, const double* av,
                  double* jac);

/* Per-model results of a whole run. */
typedef struct ucl_model_stats {
  int64_t nst, nfe, nje, nlu, nni, ncfn, netf; /* DVODE counters, summed   */
  int32_t n_intervals, n_retries;              /* output rows, retry loops  */
  double solve_ms;                              /* device time of the model */
  double t_rates_ms, t_rhs_ms, t_jac_ms, t_lu_ms, t_solve_ms; /* phase split  */
  double queue_ms;   /* arrival (or launch) to start of integration          */
  double latency_ms; /* arrival (or launch) to completion                    */
} ucl_model_stats;

/* Integrate whole CLOUD models on the device, one output row per interval
 * of the reference schedule (cloud.f90:39-51), with the reference's retry
 * and failure logic (chemistry.f90:145-292) and output layout
 * (io.f90:74-82).  Replaces the time loop of solveAbundances
 * (src/fortran_src/wrap.f90:657-690) for `nmodels` independent models.
 *   params     [nmodels]
 *   start      [nmodels*NEQ] initial abundances + density, or NULL
 *              (elemental start of initializeChemistry)
 *   max_rows   rows available per model (TIMEPOINTS+1 in the reference)
 *   phys_out   [nmodels*max_rows*UCL_N_PHYS] out (row-major per model)
 *   abund_out  [nmodels*max_rows*nspec] out
 *   nrows_out  [nmodels] out: rows written
 *   flag_out   [nmodels] out: 0 or UCL_* per-model error code
 *   stats_out  [nmodels] out (may be NULL)
 *   precision  UCL_PREC_FP64 or UCL_PREC_MIXED
 *   rates_out  [nmodels*max_rows*nreac] out, or NULL: the rates array of
 *              returnRates (io.f90:89-93): per row the rate coefficients as
 *              the reference's rate() holds them at output time (the
 *              interval's calculateReactionRates values, with the H2 and CO
 *              photodissociation rates of the last F evaluation); row 0 is
 *              zero, as rate() is before the first interval.
 * Per-model options the reference rejects at start-up give that model
 * UCL_PHYSICS_INIT_ERROR and no rows: ionModel other than 'L'/'H',
 * improvedH2CRPDissociation without cosmicRayAttenuation
 * (physics-core.f90:55-64), a collapse mode other than 0-4
 * (collapse.f90:44-48), a hot-core temp_indx other than 0-6 or hot core
 * with collapse (hotcore.f90:38-44), and points != 1 (the reference's multi-parcel
 * column density reads coldens(0), outside its array, physics-core.f90:80).
 * With collapse 1-4 the model runs collapse.f90's physics module: its
 * initializePhysics (BE1.1 and BE4 set finalTime to 0.97 of their maxTime),
 * updateTargetTime and updatePhysics between intervals; with hotcore 1-6,
 * hotcore.f90's temperature ramp (to maxTemperature) and schedule. */
int ucl_solve_models(ucl_ctx* ctx, int nmodels, const ucl_model_params* params,
                     const double* start, int max_rows, double* phys_out,
                     double* abund_out, int* nrows_out, int* flag_out,
                     ucl_model_stats* stats_out, int precision, double* rates_out);

/* Same as ucl_solve_models with every array already in device memory of the
 * context's GPU (no host copies; the call only enqueues work).  `stream` is a
 * cudaStream_t (NULL = the context's stream); `max_ctas` caps the number of
 * concurrently integrated models (0 = as many as fit).  Completion is
 * observed by synchronising that stream. */
int ucl_solve_models_device(ucl_ctx* ctx, int nmodels, const ucl_model_params* params_dev,
                            const double* start_dev, int max_rows, double* phys_dev,
                            double* abund_dev, int* nrows_dev, int* flag_dev,
                            ucl_model_stats* stats_dev, int precision, int max_ctas,
                            void* stream, double* rates_dev);

/* ucl_solve_models_device for a context of several networks: model i is
 * integrated on network net_of_dev[i] (device array of indices into the
 * context's networks), all models in one launch.  Strides as for
 * ucl_ctx_create_multi.  A network without the UCLCHEM grain and photo
 * terms (no ices, no self-shielded photo reactions) needs start vectors. */
int ucl_solve_models_nets_device(ucl_ctx* ctx, int nmodels, const int* net_of_dev,
                                 const ucl_model_params* params_dev, const double* start_dev,
                                 int max_rows, double* phys_dev, double* abund_dev, int* nrows_dev,
                                 int* flag_dev, ucl_model_stats* stats_dev, double* rates_dev,
                                 int precision, int max_ctas, void* stream);

/* Serving form of ucl_solve_models_device: request i (params_dev[i], ...)
 * arrives arrival_s_dev[i] seconds after the launch starts (ascending), is
 * admitted by the first free slot (slots: as many as fit the context's HBM
 * budget and the GPU) no earlier than its arrival, and its queue and
 * latency times are measured from that arrival (stats queue_ms,
 * latency_ms).  The request queue and the admission live on the device; the
 * host makes one launch. */
int ucl_serve_models_device(ucl_ctx* ctx, int nmodels, const ucl_model_params* params_dev,
                            const double* arrival_s_dev, const double* start_dev, int max_rows,
                            double* phys_dev, double* abund_dev, int* nrows_dev, int* flag_dev,
                            ucl_model_stats* stats_dev, int precision, int max_ctas, void* stream);

/* Live serving session: one persistent solve launch on its own stream,
 * fed while it runs.  The host appends requests to a ring of `capacity`
 * records in pinned, device-mapped memory; an idle CTA claims the next
 * request, integrates it and flags it done.  Each record also holds the
 * request's outputs in device memory (max_rows rows), so `capacity` is the
 * number of requests that may be queued, running or finished-but-not-taken
 * at once: the HBM budget of the session (capacity 0 = as many records as
 * the context's hbm_budget holds).  A request is admitted only into a free
 * record: ucl_server_submit returns UCL_E_AGAIN while the record it needs
 * still holds an untaken result.  Every device wait is bounded: a CTA that
 * finds no request for idle_timeout_s seconds (0 = 1200 s) ends, and once
 * the solver has ended ucl_server_poll reports UCL_E_TIMEOUT.  While a session is open its context must not be
 * destroyed.  No counterpart in the reference, which runs one model per
 * call.  The server's calls may be made from different host threads. */
typedef struct ucl_server ucl_server;
int ucl_server_open(ucl_ctx* ctx, int capacity, int max_rows, int precision, int max_ctas,
                    double idle_timeout_s, ucl_server** out);
int ucl_server_capacity(const ucl_server* srv);
/* queue one model; *request receives its number (0, 1, ...) */
int ucl_server_submit(ucl_server* srv, const ucl_model_params* params, long long* request);
/* 1: the request's outputs are complete; 0: pending; < 0: error */
int ucl_server_poll(ucl_server* srv, long long request);
/* copy a finished request's outputs (layout of one model of
 * ucl_solve_models, max_rows rows) and free its record */
int ucl_server_take(ucl_server* srv, long long request, double* phys_out, double* abund_out,
                    int* nrows_out, int* flag_out, ucl_model_stats* stats_out);
/* end the session: requests already submitted are still served; then the
 * launch is waited for and everything is freed */
int ucl_server_close(ucl_server* srv);

/* Batched dense LU with partial pivoting of `nsys` row-major n x n matrices
 * in device memory (FP32 for UCL_PREC_MIXED, FP64 otherwise), in place: the
 * factorisation the solver applies to its Newton matrices (the reference's
 * DGEFA, dvode.f90:11982).  perm_dev[s*n + i] = original row of row i;
 * info_dev[s] = 0 or the first zero pivot (1-based).  n % 4 == 0 and
 * mats_dev 16-byte aligned.  `stream` is a cudaStream_t (NULL = context's). */
int ucl_lu_factor_device(ucl_ctx* ctx, int nsys, int n, int precision, void* mats_dev,
                         int* perm_dev, int* info_dev, void* stream);

/* Size of the fixed device scratch of ucl_lu_factor_device_static. */
#define UCL_LU_STATIC_SCRATCH_BYTES (16u << 20)

/* The batched LU of ucl_lu_factor_device without a context and without
 * allocating anything: no cudaMalloc/cudaFree and no allocating library
 * call, for callers whose device memory is all owned by another allocator
 * (a framework's caching allocator, or a serving loop that has handed its
 * whole HBM budget to resident model state) and callers that must not pay
 * the implicit device synchronisation of an allocation.  This entry point
 * has no counterpart in the reference (DGEFA works in the caller's arrays).
 * The row-interchange scratch is a fixed static device array of
 * UCL_LU_STATIC_SCRATCH_BYTES shared by every call; at most
 * UCL_LU_STATIC_SCRATCH_BYTES / (2 * NB * n * sizeof(element)) matrices, and
 * no more than fit on the GPU at once, are in flight (NB = 32 FP32, 16
 * FP64); the rest are taken in turn by the same CTAs.  Nothing in the scratch has to start at zero.  Calls that
 * overlap in time (different streams, or different host threads without
 * ordering) race on the scratch and must not be issued.  The first call on
 * each device performs the one-time set-up on that device (the scratch's
 * device address and the kernels' shared-memory limits), so make that first
 * call before any stream capture; a set-up that fails is tried again by the
 * next call.  Uses the current device; arguments as in ucl_lu_factor_device,
 * except that a NULL `stream` is the legacy default stream (there is no
 * context stream); n > 520 or n % 4 != 0 is rejected with UCL_E_ARG. */
int ucl_lu_factor_device_static(int nsys, int n, int precision, void* mats_dev, int* perm_dev,
                                int* info_dev, void* stream);

/* The FP32 Newton-matrix LU's trailing update the context's autotuner chose
 * for network `net`: 1 tensor cores, 0 CUDA cores (or < 0 on error).  At
 * context creation the autotuner times both on a wave of Newton-like test
 * matrices of the network's size and keeps the faster; the timings (us per
 * factorisation, 0 when not measured) are returned through the pointers
 * (either may be NULL).  UCL_AUTOTUNE=0 in the environment skips the timing
 * and keeps the tensor cores.  No counterpart in the reference. */
int ucl_ctx_lu_variant(const ucl_ctx* ctx, int net, float* us_tensor, float* us_cuda);

/* Models the context integrates concurrently at the given precision. */
int ucl_ctx_slots(const ucl_ctx* ctx, int precision);

#ifdef __cplusplus
}
#endif
#endif /* UCLCHEM_GB300_H */
