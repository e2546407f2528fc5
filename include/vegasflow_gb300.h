/*
 * vegasflow_gb300 -- C-ABI of the GB300 (sm_103a) VEGAS hot path.
 *
 * libvegasgb.so exports the entry points below.  Every buffer argument is a
 * caller-owned device pointer (plain pointers and sizes, no framework types);
 * `stream` is a cudaStream_t (NULL = the legacy default stream).  No entry point
 * allocates device memory or synchronises the stream, except vf_jit_integrand
 * (host-side compilation and module load).  Every call returns VF_OK (0) or a
 * VF_ERR_* code; vf_last_error_string() describes the last failure of the
 * calling thread.  Calls are thread-safe; work on one stream is ordered.
 *
 * Reference interfaces (N3PDF/vegasflow 1.4.0, paths inside that project) are
 * cited per entry point: each C function replaces the TensorFlow graph the
 * reference compiles for that step.
 */
#ifndef VEGASFLOW_GB300_H
#define VEGASFLOW_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define VF_OK 0
#define VF_ERR_ARG 1          /* invalid argument (pointer, size, mode)          */
#define VF_ERR_LAUNCH 2       /* a kernel launch failed                          */
#define VF_ERR_TIMEOUT 3      /* a bounded device-side wait gave up              */
#define VF_ERR_NONFINITE 4    /* a result was NaN/Inf                            */
#define VF_ERR_JIT 5          /* NVRTC compilation or module load failed         */
#define VF_ERR_CUDA 6         /* a CUDA runtime call failed                      */
#define VF_ERR_UNSUPPORTED 7  /* configuration not built (e.g. n_dim > 16)       */

/* ---- device error flags (bit set in the optional `flags` word) ------------ */
#define VF_FLAG_INDEX_RANGE 1     /* a uniform mapped outside the grid (clamped)  */
#define VF_FLAG_REFINE_OVERRUN 2  /* the rebinning walk ran past the last bin     */
#define VF_FLAG_NONFINITE 4       /* a partial sum was NaN or Inf                 */
#define VF_FLAG_TIMEOUT 8         /* a bounded device-side wait gave up (a copy that
                                     never completed); that launch's sums are partial */
#define VF_FLAG_HISTORY_FULL 16   /* vf_iteration_dev / vf_plus_iteration_dev found no
                                     history row left: that iteration's result was not
                                     recorded                                          */

/* ---- constants (configflow.py:13-24) -------------------------------------- */
#define VF_BINS_MAX 50
#define VF_MAX_DIM 16

/* ---- algorithms / precisions ---------------------------------------------- */
#define VF_ALG_VEGAS 0  /* importance sampling, vflow.py:215                     */
#define VF_ALG_PLAIN 1  /* plain MC, plain.py:11                                 */
#define VF_ALG_PLUS 2   /* VEGAS+ samplers (vf_jit_integrand only), vflowplus.py:83 */
#define VF_ALG_BATCH 3  /* batched sampler (vf_jit_integrand only): vf_batch_sample_jit */
#define VF_PREC_F64 0   /* the reference's float64 arithmetic                    */
#define VF_PREC_F32 1   /* fused fp32 form, compensated sums, float64 across blocks */

/* ---- built-in integrands (parameters are a float64 device array) --------- */
#define VF_INT_NONE 0          /* sample only (x, w, ind taps)                   */
#define VF_INT_SYMGAUSS 1      /* {a, (1/(a sqrt(pi)))^D}                        */
#define VF_INT_GAUSS 2         /* {mu[D], a[D]}                                  */
#define VF_INT_BREIT_WIGNER 3  /* {M, Gamma, c[D-1]}                             */
#define VF_INT_PROD 4          /* none                                           */
#define VF_INT_SUM 5           /* none                                           */
#define VF_INT_JIT_BASE 1000   /* ids returned by vf_jit_integrand               */

/* ---- tunables (vf_tune_set / vf_tune_get) ---------------------------------- */
#define VF_TUNE_F32_HIST_COPIES 1 /* fp32 VEGAS histogram layout: 0 = joint tables of
                                      dimension pairs (the only layout)                     */
#define VF_TUNE_F32_THREADS 2     /* fp32 VEGAS Philox sampler block size: 1024 (default) |
                                      512                                                   */
#define VF_TUNE_F32_BLOCKS_PER_SM 3 /* fp32 VEGAS persistent blocks per SM, 0 = all that fit
                                      (default); sets the events per thread                */

int vf_version(void);
const char* vf_last_error_string(void);
/* SM count and compute capability of the current device. */
int vf_device_info(int* sm_count, int* cc_major, int* cc_minor);

/*
 * Number of per-block partial rows (= blocks of the persistent grid) the
 * sampler uses for this configuration.  The caller sizes `partials` as
 * rows * (2 + 50 * n_dim) doubles.
 */
int vf_sample_rows(int alg, int precision, int n_dim, int integrand, int train, int* rows);

/*
 * One chunk of events through the fused sampler.  Replaces the compiled
 * `self.event` of MonteCarloFlow.compile (monte_carlo.py:593-600), i.e.
 * VegasFlow._run_event (vflow.py:389-430) = _generate_random_array
 * (monte_carlo.py:249-275, vflow.py:93-126, importance_sampling_digest
 * vflow.py:39-83) + integrand + reductions + _importance_sampling_array_filling
 * (vflow.py:370-387), and PlainFlow._run_event (plain.py:18-35).
 *
 *  grid      [n_dim][51] bin edges (VEGAS only)
 *  xjac      1 / events per iteration (monte_carlo.py:225-227)
 *  xmin, xdelta  nullable [n_dim] integration limits, xdeltajac = prod(xdelta)
 *  u_inj     nullable [n_events][n_dim] injected uniforms (post TECH_CUT affine);
 *            NULL = in-kernel Philox4x32-10 keyed by `seed`, counter (event
 *            ev_offset+i, call_ctr)
 *  integrand VF_INT_* or a JIT id; params its float64 parameters
 *  train     fill the per-bin histogram of (w f)^2
 *  partials  [rows][2 + 50 n_dim] block partials: stored (accumulate=0) or added
 *  ind_out, x_out, w_out, f_out  nullable per-event taps ([n][D] int32,
 *            [n][D] / [n] / [n] in the precision's type).  An fp32 VEGAS launch
 *            of VF_INT_SYMGAUSS or VF_INT_PROD with ind_out as its only tap runs
 *            the fused fp32 sampler itself (its parity instantiation), so the
 *            indices are those of the benchmarked kernel; other taps use the
 *            generic sampler.
 *  flags     nullable device int receiving VF_FLAG_* bits
 */
int vf_sample(int alg, int precision, const double* grid, int n_dim, long long n_events,
              long long ev_offset, double xjac, const double* xmin, const double* xdelta,
              double xdeltajac, const double* u_inj, unsigned long long seed,
              unsigned int call_ctr, int integrand, const double* params, int train,
              int accumulate, double* partials, int rows, int* ind_out, void* x_out,
              void* w_out, void* f_out, int* flags, void* stream);

/*
 * Partial rows from integrand values produced outside the sampler (a torch
 * callable evaluated on the sampler's x): tmp = w f, sums of tmp and tmp^2 per
 * output, histogram of the `main_dim` output.  Replaces vflow.py:414-428 /
 * plain.py:310-317 for integrands that are not device functions; `n_out` > 1 is
 * the vectorial case (vflow.py:245-252).
 */
int vf_reduce_events(int precision, const void* f, const void* w, const int* ind,
                     long long n_events, int n_dim, int n_out, int main_dim, int train,
                     int accumulate, double* partials, int rows, int* flags, void* stream);

/*
 * Iteration end: fixed-order sum of the partial rows, sigma
 * (vflow.py:437-438), history[iter] = (res, sigma), the running
 * 1/sigma^2-weighted mean, its sigma and chi^2/dof in avg[n_out][5] (iter = 0
 * starts a new average: avg's previous contents are not read)
 * (monte_carlo.py:712-732), and -- when train -- refine_grid (vflow.py:349-362,
 * refine_grid_per_dimension vflow.py:135-211) on `grid` in place: train = 1
 * refines in float64 (the reference's default arithmetic), train = 2 in float32
 * (the reference's float32 mode; what the fp32 sampler's grids use).
 */
int vf_iteration_end(const double* partials, int rows, int n_dim, int n_out, int train,
                     double n_events, double alpha, double* grid, double* hist_out,
                     double* sums_out, double* history, double* avg, int iter, int* flags,
                     void* stream);

/*
 * One whole iteration -- vf_sample over all n_events with a device integrand,
 * then vf_iteration_end -- whose per-iteration values live in device memory, so
 * that a CUDA graph captured around one call replays any number of iterations
 * with no host work: *call_dev is the Philox call counter the sampler reads,
 * *iter_dev the history row; the iteration end writes history[*iter_dev],
 * updates avg, refines `grid` when train (VEGAS only), then advances both
 * counters by one.  history has hist_cap rows of (res, sigma); an iteration that
 * finds none left records nothing and sets VF_FLAG_HISTORY_FULL.  The same
 * arithmetic as one _run_iteration of VegasFlow / PlainFlow
 * (vflow.py:432-442, plain.py:18-43, monte_carlo.py:645-741); the reference
 * has no device-side counterpart (TensorFlow traces its loop on the host).
 * Launch sizes and shared-memory limits are set by the first (uncaptured)
 * call for a configuration; a captured call makes no host-side CUDA call other
 * than the two launches.
 */
int vf_iteration_dev(int alg, int precision, double* grid, int n_dim, long long n_events, double xjac,
                     const double* xmin, const double* xdelta, double xdeltajac, unsigned long long seed,
                     unsigned int* call_dev, int* iter_dev, int integrand, const double* params, int train,
                     double alpha, double* partials, int rows, double* history, int hist_cap, double* avg,
                     int* flags, void* stream);

/*
 * VEGAS+ (VegasFlowPlus, vflowplus.py:83-247).  The events of an iteration are
 * laid out hypercube by hypercube: hypercube h (coordinates = digits of h in
 * base n_strat, last dimension fastest, vflowplus.py:126-128) owns the events
 * [ev_start[h], ev_start[h] + n_ev[h]); ev_start has n_hcubes + 1 entries, the
 * last one the iteration's event count.  Both arrays live on the device and are
 * rewritten by vf_plus_iteration_end when adaptive.
 */
/* Block count for the VEGAS+ kernels; partials hold rows * (2 + 50 n_dim) doubles. */
int vf_plus_rows(int precision, int n_dim, int n_hcubes, int* rows);

/*
 * One iteration's events: generate_samples_in_hypercubes (vflowplus.py:46-80:
 * xn = (p + u) 50 / n_strat, digest, w / n_ev[h]), the weight xjac = 1 /
 * n_hcubes, the integrand, the per-hypercube sums ress/ress2
 * (segment_sum, vflowplus.py:206-214) and the histogram rows.  Philox counter =
 * the event's index within the iteration.  VF_INT_NONE samples only (taps).
 * An fp32 launch of VF_INT_SYMGAUSS or VF_INT_BREIT_WIGNER with Philox uniforms,
 * ind_out and optionally x_out as its taps runs the fp32 sampler itself (its
 * parity instantiation); other taps use the float64-map sampler.
 */
int vf_plus_sample(int precision, const double* grid, int n_dim, int n_strat, int n_hcubes,
                   const int* n_ev, const long long* ev_start, double xjac, const double* xmin,
                   const double* xdelta, double xdeltajac, const double* u_inj,
                   unsigned long long seed, unsigned int call_ctr, int integrand, const double* params,
                   int train, double* ress, double* ress2, double* partials, int rows, int* ind_out,
                   void* x_out, void* w_out, int* flags, void* stream);

/* Per-hypercube sums and histogram rows from torch-evaluated f and the sampler's w, ind. */
int vf_plus_reduce_events(int precision, const void* f, const void* w, const int* ind, const int* n_ev,
                          const long long* ev_start, int n_dim, int n_hcubes, int train, double* ress,
                          double* ress2, double* partials, int rows, void* stream);

/*
 * VegasFlowPlus._iteration_content (vflowplus.py:222-241): res = sum ress,
 * sigma^2 = sum max(var, 0) / (n_ev - 1) with var = ress2 n_ev - ress^2,
 * history/average as vf_iteration_end; when adaptive, redistribute_samples
 * (vflowplus.py:153-163: n_ev = int(max(min_neval, var^(beta/2) N0 / 2 / sum)))
 * and the new ev_start; when train, the grid refinement (train = 1 in float64,
 * 2 in float32, as vf_iteration_end).  At most 16384 hypercubes.
 */
int vf_plus_iteration_end(const double* ress, const double* ress2, int* n_ev, long long* ev_start,
                          int n_hcubes, int adaptive, int min_neval, double init_calls,
                          const double* partials, int rows, int n_dim, int train, double alpha,
                          double beta, double* grid, double* hist_out, double* arr_var_out,
                          double* history, double* avg, int iter, int* flags, void* stream);

/*
 * One whole VEGAS+ iteration with device-side counters, for capture in a CUDA
 * graph (vflowplus.py:187-241 per replay): vf_plus_sample with Philox uniforms,
 * the call counter read from *call_dev, then vf_plus_iteration_end (train: the
 * refinement of `precision`) with the iteration index read from *iter_dev, after
 * which both advance by one.  history has hist_cap rows (VF_FLAG_HISTORY_FULL
 * when the index reaches it).  The adaptive reallocation stays on the device, so
 * replays need no host work between iterations.
 */
int vf_plus_iteration_dev(int precision, double* grid, int n_dim, int n_strat, int n_hcubes, int* n_ev,
                          long long* ev_start, double xjac, const double* xmin, const double* xdelta,
                          double xdeltajac, unsigned long long seed, unsigned int* call_dev, int* iter_dev,
                          int integrand, const double* params, int train, int adaptive, int min_neval,
                          double init_calls, double alpha, double beta, double* ress, double* ress2,
                          double* partials, int rows, double* history, int hist_cap, double* avg, int* flags,
                          void* stream);

/*
 * Batched VEGAS (no counterpart in the reference, which integrates one
 * integrand per VegasFlow instance): many independent integrals -- own
 * dimension count, event count, built-in integrand, grid -- sampled by one
 * persistent fp32 launch per iteration off a device work queue.  Each integral
 * is split into tiles of at most T events (fixed boundaries within the
 * integral); tile k's partial row [res, res2, hist[n_dim][50]] lives at
 * partials + tile_row[k].  The Philox stream of an integral is keyed by the
 * batch seed with its own stream_id and its own call counter, so its result
 * does not depend on the batch.  Per-integral state lives in slots:
 * iters[slot] (iterations in the running average), calls[slot] (Philox call
 * counter), history[slot][hist_cap][2], avg[slot][5]; integrals can join and
 * leave between iterations.  An iteration is vf_batch_sample followed by
 * vf_batch_iteration_end (which advances the counters and re-arms the queue),
 * so it can be captured in a CUDA graph.
 */
typedef struct vf_batch_item {
  long long n_events;
  long long grid_off;   /* doubles into grids: [n_dim][51] */
  long long param_off;  /* doubles into params */
  double xjac;          /* 1 / n_events */
  int n_dim;
  int integrand;        /* VF_INT_SYMGAUSS .. VF_INT_SUM (vf_batch_sample), or the id of vf_batch_sample_jit */
  int stream_id;
  int tile0;            /* first tile of this integral */
  int n_tiles;
  int train;
  int slot;             /* state slot */
  int pad;
} vf_batch_item;

/* Persistent grid size and dynamic shared memory for a batch whose largest n_dim is max_dim. */
int vf_batch_blocks(int max_dim, int* blocks, int* smem_bytes);
/* One iteration's events of every integral; *queue must be 0 (vf_batch_iteration_end re-arms it). */
int vf_batch_sample(const vf_batch_item* items, const int* tile_item, const long long* tile_start,
                    const int* tile_count, const long long* tile_row, int n_tiles, int max_dim, int* queue,
                    const unsigned int* calls, const double* grids, const double* params, double* partials,
                    unsigned long long seed, int* flags, int blocks, void* stream);
/* vf_batch_sample with a user integrand: every integral of the tiles given uses
 * integrand_id (vf_jit_integrand with VF_ALG_BATCH, VF_PREC_F32 and n_dim >= max_dim),
 * its parameters at params + param_off. */
int vf_batch_sample_jit(int integrand_id, const vf_batch_item* items, const int* tile_item,
                        const long long* tile_start, const int* tile_count, const long long* tile_row, int n_tiles,
                        int max_dim, int* queue, const unsigned int* calls, const double* grids, const double* params,
                        double* partials, unsigned long long seed, int* flags, int blocks, void* stream);
/* Per integral: sums of its tile rows in tile order, sigma, history[slot][iters[slot]],
 * the weighted average avg[slot][5], then iters[slot] += 1, calls[slot] += 1; per
 * (integral, dimension) block: refinement of that grid row; *queue = 0.  Block b serves
 * integral blk_item[b] in role blk_role[b] (a dimension, or -1 for the sums).
 * status: nullable [items][3] doubles receiving, for item i, the running mean,
 * its sigma and the iterations in the average after this one (avg[slot][2],
 * avg[slot][3], iters[slot]); device memory, or pinned host memory that the
 * device can address (read it after the stream synchronizes: no copy needed). */
int vf_batch_iteration_end(const vf_batch_item* items, const int* blk_item, const int* blk_role, int n_blocks,
                           const long long* tile_row, const double* partials, double* grids, double* history,
                           double* avg, int hist_cap, int* iters, unsigned int* calls, int* queue, int* flags,
                           double* status, void* stream);

/* VegasFlow.refine_grid(arr_res2) (vflow.py:349-362): hist [n_dim][50]. */
int vf_refine_grid(double* grid, const double* hist, int n_dim, double alpha, int* flags,
                   void* stream);

/* consume_array_into_indices (utils.py:17-44): out[size] = per-bin sums. */
int vf_consume_array_into_indices(const double* input, const int* indices, long long n,
                                  int result_size, double* out, int* flags, void* stream);

/*
 * The float64 uniforms that the fp32 samplers' integer maps stand for, for
 * precision statements on identical events (no counterpart in the reference):
 * u_out[e][d] = (word + 1/2) / 2^32 with `word` the Philox4x32-10 word d of
 * event ev_offset + e -- counter (ev, ev >> 32, call_ctr << 4 | d / 4, word3),
 * key `seed`.  word3 is call_ctr >> 28 for vf_sample (fp32 VEGAS) and
 * vf_plus_sample (fp32 VEGAS+, events in iteration order), and the integral's
 * stream id for vf_batch_sample.  Fed to the float64 samplers as injected
 * uniforms, they reproduce the fp32 kernels' events in the reference's float64
 * arithmetic.  u_out: device [n][n_dim].
 */
int vf_philox_uniforms(unsigned long long seed, unsigned int call_ctr, unsigned int word3, long long ev_offset,
                       long long n, int n_dim, double* u_out, void* stream);

/*
 * One VEGAS iteration (sample, reduce, sigma, and refinement of `grid` in place
 * when `train`) that allocates nothing.  No counterpart in the reference: it
 * serves callers that cannot call cudaMalloc -- plugins whose host framework
 * owns all device memory, code that must not allocate while a stream is being
 * captured, fixed-budget deployments.  The block-partial scratch lives in a
 * 4 MiB file-scope __device__ array inside the library (held by every GPU that
 * loads it until exit); the caller passes only inputs (grid [n_dim][51],
 * params) and outputs: res_sigma (device [2]: result, sigma) and, when not
 * NULL, flags_out (device int: this call's VF_FLAG_* bits, 0 when nothing went
 * wrong -- VF_FLAG_NONFINITE for a NaN/Inf sum, VF_FLAG_REFINE_OVERRUN from the
 * refinement).  train: 0 no histogram and no refinement, 1 float64 refinement,
 * 2 float32 refinement (as the fp32 integrators refine); other values are
 * rejected before anything is enqueued.
 *
 * Limits: n_dim 1..16 and a built-in integrand id; xjac = 1/n_events, no
 * integration limits, no per-event taps.  The first call on a device resolves
 * the scratch's device address (cudaGetSymbolAddress), and so does the first
 * call after a device reset (a new context): make that call before any stream
 * capture.  All calls share the scratch and it keeps the last call's contents
 * (the state that must start at zero is cleared per call); calls that overlap
 * on the GPU race on it and must be ordered by the caller.
 */
int vf_vegas_iteration_static(int precision, double* grid, int n_dim, long long n_events,
                              unsigned long long seed, unsigned int call_ctr, int integrand,
                              const double* params, int train, double* res_sigma, int* flags_out,
                              void* stream);

/*
 * User integrands as CUDA device functions (replaces the TF custom-op route of
 * examples/cuda/integrand.cpp:41-89 and the cffi route of
 * examples/simgauss_cffi.py:25-61).  `source` defines
 *     __device__ vf_real NAME(const vf_real* x, int n_dim, vf_real weight, const double* params)
 * where vf_real is double (VF_PREC_F64) or float (VF_PREC_F32), x the event's
 * point (integration limits applied), weight its full weight, params the
 * vf_sample `params` pointer.  NVRTC compiles it with the sampler into a kernel
 * for (alg, precision, n_dim) -- the fp32 VEGAS kernel specialised on n_dim, or
 * the generic sampler -- built for sm_103a and loaded into the current context;
 * *integrand_id (>= VF_INT_JIT_BASE) then selects it in vf_sample (VF_ALG_VEGAS,
 * VF_ALG_PLAIN), vf_plus_sample (VF_ALG_PLUS) or vf_batch_sample_jit
 * (VF_ALG_BATCH, fp32 only: the batched sampler for integrals of up to n_dim
 * dimensions, the function called with each integral's own n_dim).  This call
 * compiles on the host and loads a module: it is not for hot paths.
 */
int vf_jit_integrand(const char* source, const char* func_name, int alg, int precision, int n_dim,
                     int* integrand_id);
/* Compile only (no GPU needed): VF_OK, or VF_ERR_JIT with the NVRTC log in `log`. */
int vf_jit_check(const char* source, const char* func_name, int alg, int precision, int n_dim, char* log,
                 int log_size);

/*
 * Self-test of the device-side bounded wait (no counterpart in the reference):
 * one block waits, with the same bounded poll loop as the TMA-staged sampler,
 * on a barrier that nothing completes; after `polls` polls (1..2^20) every
 * thread gives up and VF_FLAG_TIMEOUT is or-ed into *flag (device memory).
 * Exercises the timeout path without any fault; the context stays usable.
 */
int vf_wait_selftest(int polls, int* flag, void* stream);

/*
 * Load every kernel of the library on the current device now (no counterpart
 * in the reference).  Kernels are otherwise loaded at their first launch; on
 * this platform a kernel loaded after a CUDA graph had been captured in the
 * process took ~2 s to load, so code that captures graphs calls this first.
 * Idempotent per device.
 */
int vf_preload(void);

/*
 * Process-wide tunables picked by the autotuner (no counterpart in the
 * reference, whose kernels are TensorFlow's).  Values apply to later launches.
 */
int vf_tune_set(int key, int value);
int vf_tune_get(int key, int* value);

/*
 * Calibration (no counterpart in the reference): `blocks` x 256 threads each
 * issue 128 * iters independent fp32 FMAs, so the kernel's duration gives the
 * achievable warp-instruction issue rate, the roofline of the compute-bound
 * fused sampler.  `out` is a device buffer of blocks * 256 floats (written only
 * on an impossible value); *fma_per_thread receives 128 * iters.
 */
int vf_issue_probe(float* out, int blocks, int iters, long long* fma_per_thread, void* stream);
/*
 * The same for the 64-bit integer multiplies of Philox4x32-10 and the integer
 * bin map (the FMA-heavy pipe): each thread runs 128 * iters steps of eight
 * independent chains shaped like a Philox round, one 32 x 32 -> 64-bit
 * multiply and one three-input XOR per step; *mul_per_thread receives
 * 128 * iters.  `out`: blocks * 256 unsigned ints (written only on an
 * impossible value).
 */
int vf_widemul_probe(unsigned* out, int blocks, int iters, long long* mul_per_thread, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* VEGASFLOW_GB300_H */
