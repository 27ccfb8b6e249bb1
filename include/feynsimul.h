/*
 * feynsimul.h -- C ABI of libfeynsimul_gb300.so, the GB300 (sm_103a) engine behind the
 * FeynSimul plugin API (physical_systems / KernelArgs / PIMCKernel / modN).
 *
 * Plain C types only.  Every call returns FS_OK (0) or a negative status; the handle's
 * last error string (fs_last_error) says what went wrong.  One handle per host thread;
 * calls on a handle are ordered on its CUDA stream.  The library owns all device memory
 * and copies host buffers in and out, so callers keep ownership of theirs.
 *
 * Reference interface each call replaces (file:line in the FeynSimul tree):
 *   fs_create ............ PIMCKernel.__init__          FeynSimul/kernel.py:53-457
 *   fs_compile_only ...... Program.build of __init__    FeynSimul/kernel.py:372-381
 *   fs_destroy ........... (PyOpenCL buffer release)    FeynSimul/kernel.py:386-457
 *   fs_run ............... PIMCKernel.run               FeynSimul/kernel.py:459-506
 *   fs_sync .............. PIMCKernel._queue.finish / kernelObj.wait   kernel.py:500, pimc_utils.py:187
 *   fs_ranlux_init ....... PIMCKernel.initRanlux        FeynSimul/kernel.py:508-530
 *   fs_ranlux_group_init . PIMCKernel.groupInitRanlux   FeynSimul/kernel.py:532-554
 *   fs_set_paths ......... PIMCKernel.setPaths          FeynSimul/kernel.py:567-574
 *   fs_get_paths ......... PIMCKernel.getPaths          FeynSimul/kernel.py:557-565
 *   fs_get_operators ..... PIMCKernel.getOperators (raw per-thread means)   kernel.py:576-606
 *   fs_get_correlator .... PIMCKernel.getCorrelator (raw sums)              kernel.py:608-617
 *   fs_get_bins .......... PIMCKernel.getBinCounts (raw counts)             kernel.py:619-637
 *   fs_get_accepts ....... PIMCKernel.getAcceptanceRate (raw counts)        kernel.py:648-658
 *   fs_get_run_time ...... PIMCKernel.getRunTime        FeynSimul/kernel.py:638-646
 *   fs_set_correlator / fs_set_bins / fs_set_histogram ... no reference counterpart: restore
 *                          running sums from a checkpoint (the reference checkpoints paths
 *                          only, pimc_utils.py:246-252)
 *   fs_build_log ......... PIMCKernel.getBuildLog       FeynSimul/kernel.py:778-785
 *   fs_source ............ the verbose cleaned.c dump   FeynSimul/kernel.py:351-364
 *   fs_query ............. PIMCKernel.getStats / exceedsLimits / getGlobalMemory  kernel.py:660-775
 *   fs_set_xorshift_seeds / fs_get_xorshift_seeds ... the seeds buffer  kernel.py:421-426
 *   fs_rng_ranlux_stream / fs_rng_xorshift_stream ... the stream kernels of
 *                                      examples/ranlux_test_kernel.c:90-161, :182-212
 */
#ifndef FEYNSIMUL_GB300_H
#define FEYNSIMUL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FS_OK 0
#define FS_ERR_CONFIG (-1)   /* invalid run parameters (kernel.py:93-211 checks) */
#define FS_ERR_COMPILE (-2)  /* NVRTC rejected the plugin code; see fs_build_log */
#define FS_ERR_OOM (-3)      /* device allocation failed (kernel.py:455-457) */
#define FS_ERR_LAUNCH (-4)   /* kernel launch or execution failed */
#define FS_ERR_TIMEOUT (-5)  /* fs_sync_timeout expired before the work finished */
#define FS_ERR_IO (-6)       /* host buffer size mismatch */
#define FS_ERR_CUDA (-7)     /* any other CUDA runtime error */
#define FS_ERR_STATE (-8)    /* call not valid for this handle's configuration */
#define FS_ERR_NUMERIC (-9)  /* a sweep left a non-finite path value (fs_sync / fs_sync_timeout) */

/* accumulation of operator / correlator running sums */
#define FS_ACCUM_REF_FP32 0  /* FP32 sums in the reference's order (kernel.c:622, :784) */
#define FS_ACCUM_FP64 1      /* FP64 sums (default) */
#define FS_ACCUM_KAHAN 2     /* compensated FP32 sums */
#define FS_ACCUM_STUDY 3     /* FP32, Kahan-FP32 and FP64 sums side by side */

typedef struct fs_handle fs_handle;

/* Run parameters: the fields of KernelArgs (FeynSimul/kernel_args.py:23-51) that reach
 * the device, plus this library's additions (marked "new"). */
typedef struct fs_config {
    int32_t dof;                          /* system.DOF */
    int32_t n_slices;                     /* N (power of two) */
    int32_t bisection_level;              /* S (2^S <= N) */
    double beta;                          /* beta; epsilon = beta / N */
    int32_t n_walkers;                    /* nbrOfWalkers */
    int32_t walkers_per_group;            /* nbrOfWalkersPerWorkGroup (thread-id layout) */
    int32_t operator_runs;                /* operatorRuns */
    int32_t metro_steps_per_operator_run; /* metroStepsPerOperatorRun */
    int32_t enable_parallelize_path;      /* enableParallelizePath */
    int32_t enable_ranlux;                /* enableRanlux */
    int32_t luxury_factor;                /* luxuaryFactor as the user gives it (kernel uses +1) */
    uint64_t ranlux_int_max;              /* ranluxIntMax as the user gives it (kernel uses +1) */
    int32_t enable_double;                /* enableDouble */
    int32_t enable_bins;                  /* enableBins */
    double x_min, x_max;                  /* xMin, xMax */
    int32_t bin_resolution_per_dof;       /* binResolutionPerDOF */
    /* new: histogram of plugin expressions (e.g. pair distances), shared bins */
    double hist_lo, hist_hi;
    int32_t hist_bins;
    /* new: 1 = reference-compatible random-number use (per-thread xorshift rows whose walker
     * stream is never written back, kernel.c:568-572; RANLUX tables all seeded from seeds[0],
     * kernel.c:155; RANLUX integers with zero low bits, kernel.c:206), 0 = fixed */
    int32_t compat;
    /* new: FS_ACCUM_* */
    int32_t accum;
    /* new: 1 = fast math intrinsics (the reference builds with -cl-fast-relaxed-math);
     * 0 = IEEE functions and no FMA contraction in plugin code (parity builds) */
    int32_t fast_math;
    /* new: walkers per CTA (0 = automatic) */
    int32_t walkers_per_block;
    /* new: CTAs per SM the sweep kernel is compiled to fit (its register budget); 0 = as
     * many as shared memory admits, at most 2048 threads and at least 64 registers each */
    int32_t min_blocks_per_sm;
    /* new: 1 = learned level-1 bisection proposal (Metropolis-Hastings corrected); needs
     * parallel-path mode, DOF <= 8 and whole warps of walkers; the model is set with
     * fs_set_learned_proposal (until then the network is zero, i.e. the free proposal) */
    int32_t learned;
    /* 1 = the walkers' paths stay in device memory and the sweep works on them in place
     * (enableGlobalPath: kernel.py:238-239, kernel.c:62-70, :582-588) instead of staging
     * each walker in shared memory; for paths larger than shared memory (e.g. 27 DOF x
     * 1024 slices in FP64).  Same arithmetic and results as the shared-memory sweep. */
    int32_t global_path;
    /* new: potential cache (V of every slice kept between moves, so a move evaluates the
     * potential only at its proposed nodes): 0 = automatic, 1 = in shared memory, 2 = off,
     * 3 = in device memory (N values per walker, L1/L2 resident).  Results are bit-identical
     * either way; in shared memory it trades occupancy for potential work, in device memory
     * cache traffic.  Automatic: shared memory where that costs no resident CTA per SM (or
     * for more than 8 DOF), else device memory for 3 or more DOF and launches of more than
     * one move, else none. */
    int32_t potential_cache;
    /* Move types per Metropolis step, walker mode (enable_parallelize_path = 0) for all but
     * the bisection: 0 = bisection only (the default); otherwise a mask of FS_MOVE_* --
     * enableBisection / enablePathShift / enableSingleNodeMove (kernel.py:68-73,
     * :192-198, kernel.c:640-705).  Per step the path shift comes first, then the
     * single-node move, then the bisection. */
    int32_t moves;
    double alpha;     /* single-node move width: node += alpha * (2u - 1) (kernel_args.py:124-126) */
    double ps_alpha;  /* path-shift width: offset = PSAlpha * (2u - 1) (kernel_args.py:128-131) */
    /* new: how one measurement's values are summed before their FP64 add to a running sum
     * (FP32 builds; FS_ACCUM_FP64 for the operators, FS_ACCUM_FP64 and FS_ACCUM_KAHAN for
     * the correlator).  FS_PARTIALS_FP32 (0, default): a thread's operator values of its
     * slices summed in FP32 in slice order, then one FP64 add; a lag's products in four FP32
     * fused multiply-add chains over the slices s mod 4, added pairwise, then one FP64 add.
     * FS_PARTIALS_EXACT (1): every operator value added in FP64; the rounded products of a
     * lag summed in float-float (about 48 significant bits).  FS_ACCUM_STUDY always uses
     * the exact partials (its FP64 column is the study's reference). */
    int32_t partials;
} fs_config;

#define FS_PARTIALS_FP32 0
#define FS_PARTIALS_EXACT 1

enum { FS_MOVE_BISECTION = 1, FS_MOVE_PATH_SHIFT = 2, FS_MOVE_SINGLE_NODE = 4 };

/* fs_query output */
typedef struct fs_info {
    int64_t n_threads;          /* reference work-items (walkers * N / 2^S, or walkers) */
    int64_t threads_per_walker;
    int64_t walkers_per_block;
    int64_t block_threads;
    int64_t grid_blocks;
    int64_t smem_bytes;         /* dynamic shared memory per CTA */
    int64_t registers;          /* registers per thread of the sweep kernel */
    int64_t device_bytes;       /* device memory held by the handle */
    int64_t uniforms_per_move;  /* 2 * DOF * (2^S - 1) + 1 */
    int64_t nodes_per_move;     /* 2^S - 1 */
    int64_t potential_cache;    /* the potential cache in use: 0 none, 1 shared memory, 3 device memory */
} fs_info;

/* Build the sweep for one configuration: validates, generates the CUDA source from the
 * plugin strings, compiles it with NVRTC for sm_103a and allocates the buffers (paths
 * zero-initialised, like kernel.py:387-389). */
int fs_create(const fs_config *cfg, const char *potential, const char *user_code,
              const char *const *operators, int32_t n_operators,
              const char *const *correlators, int32_t n_correlators,
              const char *const *histograms, int32_t n_histograms, fs_handle **out);
int fs_destroy(fs_handle *h);

/* Validate and compile only (no GPU needed): generates the CUDA source and compiles it
 * for sm_103a; the NVRTC log (with ptxas resource usage) or the error goes to log. */
int fs_compile_only(const fs_config *cfg, const char *potential, const char *user_code,
                    const char *const *operators, int32_t n_operators,
                    const char *const *correlators, int32_t n_correlators,
                    const char *const *histograms, int32_t n_histograms, char *log,
                    size_t log_capacity);

/* Last error of the handle, or of the calling thread's last failed fs_create when h is
 * NULL.  The pointer stays valid until the next call on the handle / thread. */
const char *fs_last_error(const fs_handle *h);
const char *fs_build_log(const fs_handle *h);
const char *fs_source(const fs_handle *h);
int fs_query(const fs_handle *h, fs_info *info);

/* Paths in the reference layout: [walkers][DOF][N], float (double when enable_double). */
int fs_set_paths(fs_handle *h, const void *host, size_t n_elems);
int fs_get_paths(fs_handle *h, void *host, size_t n_elems);

/* xorshift tables: per-thread rows [n_threads + 1][4]; per-walker rows [n_walkers][4]
 * (the walker integer streams of the fixed mode). */
int fs_set_xorshift_seeds(fs_handle *h, const uint32_t *rows, size_t n_rows);
int fs_get_xorshift_seeds(fs_handle *h, uint32_t *rows, size_t n_rows);
int fs_set_walker_seeds(fs_handle *h, const uint32_t *rows, size_t n_rows);
int fs_get_walker_seeds(fs_handle *h, uint32_t *rows, size_t n_rows);

/* RANLUX tables (28 words per row, the reference's ranluxcl_state_t layout): row i is
 * seeded by ranluxcl_init from xs[i].  Per-thread table: n_threads rows.  Group table:
 * n_threads rows in compat mode, n_walkers rows otherwise. */
int fs_ranlux_init(fs_handle *h, const uint64_t *xs, size_t n_rows);
int fs_ranlux_group_init(fs_handle *h, const uint64_t *xs, size_t n_rows);
int fs_get_ranlux_tables(fs_handle *h, uint32_t *tab, size_t n_tab_rows, uint32_t *group_tab,
                         size_t n_group_rows);
int fs_set_ranlux_tables(fs_handle *h, const uint32_t *tab, size_t n_tab_rows,
                         const uint32_t *group_tab, size_t n_group_rows);

/* One reference run() = operator_runs x metro_steps_per_operator_run sweeps, launched
 * n_launches times back to back.  Asynchronous. */
int fs_run(fs_handle *h, int32_t n_launches);
/* n_launches runs on host path buffers ([walkers][DOF][N] in the path precision; in and
 * out may be the same buffer), pipelined: the walkers are split into n_chunks chunks whose
 * copy-in, sweeps and copy-out overlap on three streams (n_chunks = 0: automatic, up to 4
 * chunks of at least half a wave of resident CTAs each).  Equivalent to fs_set_paths +
 * fs_run + fs_get_paths (kernel.py:567-574, :459-506, :557-565); asynchronous like fs_run
 * (the buffers must stay valid until fs_sync), and overlapping only for page-locked host
 * memory (fs_pin_host). */
int fs_run_host(fs_handle *h, const void *paths_in, void *paths_out, int32_t n_launches, int32_t n_chunks);
/* chunks the last fs_run_host call used (each chunk launches the sweep kernel n_launches times) */
int fs_get_last_chunks(const fs_handle *h, int32_t *chunks);
/* page-lock / release a host buffer (cudaHostRegister) for overlapped copies */
int fs_pin_host(void *ptr, size_t bytes);
int fs_unpin_host(void *ptr);
/* Wait for the handle's queued work (kernel.py:500).  Then read the sweeps' status word:
 * if a launch since the last check left a path value that is not finite (NaN or infinity:
 * a potential or operator that diverged), return FS_ERR_NUMERIC naming one such walker
 * (fs_last_error) and clear the word.  No counterpart in the reference, which does not
 * look at its paths. */
int fs_sync(fs_handle *h);
/* fs_sync that gives up after `seconds` with FS_ERR_TIMEOUT, polling the stream (the
 * reference's failure path is its wait on the kernel event, kernel.py:499-506) */
int fs_sync_timeout(fs_handle *h, double seconds);

/* Raw device results.  Operators: [n_threads][n_ops] per-thread means (FP32 values for
 * FS_ACCUM_REF_FP32 / FS_ACCUM_KAHAN in FP32 builds, else FP64; [..][3] FP64 for
 * FS_ACCUM_STUDY: plain FP32, Kahan FP32, FP64 sums of the same values), returned as
 * double.  Correlator: [walkers][n_corr][N/2] running sums since creation / the last
 * fs_zero_accumulators, as double; FS_ACCUM_STUDY: [..][4] = plain FP32 sum, Kahan sum,
 * Kahan compensation, FP64 sum.  In FP32 builds every mode but FS_ACCUM_REF_FP32 sums one
 * measurement's products of a lag in FP32 (fs_config.partials) before adding them to
 * the lag's FP64 running sum.  Bins: [res^DOF] counts.  Histogram: [hist_bins] counts. */
int fs_get_operators(fs_handle *h, double *out, size_t n);
int fs_get_correlator(fs_handle *h, double *out, size_t n);
/* Per-walker operator means [n_ops][walkers]: each walker's thread means averaged on the
 * device in FP64 (the fixed-mode reduction of PIMCKernel.getOperators, kernel.py:576-606).
 * Not for FS_ACCUM_STUDY. */
int fs_get_walker_operators(fs_handle *h, double *out, size_t n);
int fs_get_accepts(fs_handle *h, uint32_t *out, size_t n);
int fs_get_bins(fs_handle *h, uint32_t *out, size_t n);
int fs_get_histogram(fs_handle *h, uint64_t *out, size_t n);
int fs_zero_accumulators(fs_handle *h);
/* Restore running sums from a checkpoint (same shapes as the getters). */
int fs_set_correlator(fs_handle *h, const double *in, size_t n);
int fs_set_bins(fs_handle *h, const uint32_t *in, size_t n);
int fs_set_histogram(fs_handle *h, const uint64_t *in, size_t n);
/* Ensemble moments of the correlator over walkers [walker_begin, walker_end), reduced on
 * the device in FP64 (the host reduction of kernel.py:608-617 for walker counts whose
 * per-walker array is too large to copy): sum[l][col] and sumsq[l][col] for each lag
 * l = c * N/2 + tau, col = 0 (one column), or plain FP32, Kahan, FP64 (three columns,
 * FS_ACCUM_STUDY).  n = n_corr * N/2 * columns. */
int fs_reduce_correlator(fs_handle *h, int64_t walker_begin, int64_t walker_end, double *sum, double *sumsq,
                         size_t n);
/* Fill all walkers' paths from n_template walkers of host data ([n_template][DOF][N] in
 * the path precision): walker w gets template w % n_template, replicated on the device.
 * For walker counts whose full path array is impractical to stage in host memory. */
int fs_set_paths_tiled(fs_handle *h, const void *host, size_t n_template);
/* Metropolis steps of all launches so far (operator_runs * metro_steps_per_operator_run
 * per launch); the fixed mode's single-node and path-shift moves continue their node /
 * degree counter from it.  Set it when restoring a checkpoint. */
int fs_get_step_counter(fs_handle *h, uint64_t *steps);
int fs_set_step_counter(fs_handle *h, uint64_t steps);
/* device time of the last fs_run call (all its launches), seconds */
int fs_get_run_time(fs_handle *h, double *seconds);

/* Stand-alone generator streams (RNG parity tests): RANLUX: n_streams streams seeded from
 * xs[], n_calls 4-value calls each -> out[n_streams][4*n_calls] and the final 28-word
 * states.  lux_in_kernel is the luxury level the generator sees (luxuaryFactor + 1).
 * xorshift: n_draws integers and floats per 4-word state; states are advanced. */
int fs_rng_ranlux_stream(int32_t lux_in_kernel, const uint64_t *xs, int32_t n_streams,
                         int32_t n_calls, float *out, uint32_t *states);
int fs_rng_ranlux_stream64(int32_t lux_in_kernel, const uint64_t *xs, int32_t n_streams,
                           int32_t n_calls, double *out);
int fs_rng_xorshift_stream(uint32_t *states, int32_t n_streams, int32_t n_draws,
                           uint32_t *out, float *fout);

/* Seed a caller-owned RANLUX table without any device allocation: row i of table
 * (28 uint32 words per row, device memory) is seeded by ranluxcl_init from xs[i] (host or
 * device memory), exactly as fs_ranlux_init seeds a handle's table.  No counterpart in the
 * reference: it is for callers that cannot let a library call cudaMalloc (hosts whose
 * memory pool owns all device memory, bindings whose allocator must own every buffer).
 * The seed values are staged in a fixed 2 MiB scratch array inside the library (held on
 * every GPU that loads it until exit), so n_rows is limited to 262144 per call; larger
 * n_rows fail with FS_ERR_CONFIG.  Asynchronous on stream (a cudaStream_t; NULL for the
 * default stream): synchronise before reading the table.  xs may be reused when the call
 * returns only if it is pageable host memory.  Calls share the scratch array, so calls
 * that can overlap on the GPU race.  The first call on a device looks up the array's
 * device address and keeps it for the life of the process; make that first call before any
 * stream capture.  A device reset (cudaDeviceReset, or another library resetting the
 * primary context) invalidates the kept address: do not call this entry point again in a
 * process after such a reset. */
int fs_ranlux_init_noalloc(uint32_t *table, const uint64_t *xs, size_t n_rows, void *stream);

/* ---- learned bisection proposal (no counterpart in the reference) ----
 * A 16-128-128-128-16 ReLU network (BF16 weights, FP32 accumulation on the tensor cores)
 * predicts, from a segment's endpoints, a Gaussian for the segment's midpoint; the sweep
 * draws the midpoint from it and corrects the acceptance (Metropolis-Hastings), so the
 * sampled distribution is unchanged whatever the network.  Parameters are one FP32 array
 * of fs_mlp_sizes()->n_param floats: W1[128][16] b1 W2[128][128] b2 W3[128][128] b3
 * W4[16][128] b4.  Training entry points take device pointers and a cudaStream_t. */
int fs_mlp_sizes(int64_t *n_param, int64_t *n_bf16, int64_t *n_frag_u2, int64_t *n_bias);
/* One forward + backward pass over n_rows (features x[n][16], targets z[n][8]) adding the
 * gradient of the mean loss (inv_batch = 1/batch) to grad and the loss sum to *loss; on the
 * tcgen05 tensor cores (one CTA per SM, 222 KB of shared memory and all 512 tensor-memory
 * columns each).  wq, x and grad must be 16-byte aligned.  A CTA whose bounded wait on its
 * MMAs gives up adds NaN to *loss. */
int fs_mlp_train_step(const float *params, const uint16_t *wq, float *grad, const float *x,
                      const float *z, int32_t n_rows, int32_t dof, float inv_batch, float *loss,
                      void *stream);
/* Adam (beta 0.9 / 0.999) on params; refreshes the BF16 copy wq; clears grad. */
int fs_mlp_adam(float *params, float *m, float *v, float *grad, uint16_t *wq, int32_t step,
                float lr, void *stream);
/* params -> BF16 training copy, inference fragments (n_frag_u2 x 8 bytes), biases. */
int fs_mlp_pack(const float *params, uint16_t *wq, void *frag, float *bias, void *stream);
/* Inference of rows x[n][16] -> y[n][16] on the tcgen05 tensor cores (BF16 operands in
 * shared memory, FP32 accumulators in tensor memory), rounding to BF16 at the same points as
 * the sampler's device code (inputs, weights, post-ReLU activations).  A CTA whose bounded
 * wait for the tensor cores runs out writes NaN to its rows. */
int fs_mlp_infer(const void *frag, const float *bias, const float *x, float *y, int32_t n_rows,
                 void *stream);
/* Load a packed model (host buffers) into a handle created with cfg.learned = 1;
 * inv_scale multiplies the endpoint coordinates to form the features. */
int fs_set_learned_proposal(fs_handle *h, const void *frag, size_t frag_bytes, const float *bias,
                            size_t n_bias, double inv_scale);

/* ---- ragged batch (no counterpart in the reference) ----
 * Many independent systems in one persistent launch: each system has its own plugin
 * type (potential and operators compiled once per type), slice count, bisection level,
 * beta and walker count.  Work items are tiles of walkers; CTAs take them from a work
 * counter, largest first.  Sampling semantics are those of the fixed-mode xorshift sweep
 * (per-thread float streams, per-walker offset streams), FP32 paths, FP64 operator sums
 * per walker accumulated over launches. */
typedef struct fs_batch fs_batch;
typedef struct fs_batch_system {
    int32_t type;              /* index into the per-type plugin arrays */
    int32_t n_walkers;
    int32_t n_slices;          /* N, a power of two */
    int32_t bisection_level;   /* S, 1..10; N / 2^S threads per walker */
    double beta;
    int32_t walkers_per_tile;  /* 0 = as many as fit the block (output: the value used) */
} fs_batch_system;
/* ranlux_luxury: -1 = xorshift streams (rows set by fs_batch_set_seeds); otherwise RANLUX
 * tables for every system with luxuaryFactor ranlux_luxury (the kernel uses +1, as
 * fs_config.luxury_factor), seeded with distinct default values per system and row and
 * re-seeded by fs_batch_init_ranlux. */
int fs_batch_create(int32_t n_types, const int32_t *type_dof, const char *const *potentials,
                    const char *const *user_codes, const char *const *operators, int32_t n_ops,
                    int32_t n_systems, const fs_batch_system *systems, int32_t op_runs,
                    int32_t msteps, int32_t block_threads, int32_t ranlux_luxury, fs_batch **out);
int fs_batch_destroy(fs_batch *b);
/* n_launches persistent launches; use_graph = 1 replays a captured CUDA graph (counter
 * reset + launch) instead of launching directly.  Asynchronous. */
int fs_batch_run(fs_batch *b, int32_t n_launches, int32_t use_graph);
int fs_batch_sync(fs_batch *b);
int fs_batch_get_run_time(fs_batch *b, double *seconds);
int fs_batch_set_paths(fs_batch *b, int32_t system, const float *host, size_t n);
int fs_batch_get_paths(fs_batch *b, int32_t system, float *host, size_t n);
int fs_batch_set_seeds(fs_batch *b, int32_t system, const uint32_t *thread_rows, size_t n_threads,
                       const uint32_t *walker_rows, size_t n_walkers);
/* RANLUX batches: system's tables seeded by ranluxcl_init, row r of the thread table from
 * xs_threads[r] (thread = walker * threads per walker + t) and row w of the walker table
 * (segment offsets) from xs_walkers[w]; and both tables read back (28 words per row, the
 * reference's layout). */
int fs_batch_init_ranlux(fs_batch *b, int32_t system, const uint64_t *xs_threads, size_t n_threads,
                         const uint64_t *xs_walkers, size_t n_walkers);
int fs_batch_get_ranlux_tables(fs_batch *b, int32_t system, uint32_t *thread_rows, size_t n_threads,
                               uint32_t *walker_rows, size_t n_walkers);
int fs_batch_get_op_sums(fs_batch *b, int32_t system, double *out, size_t n);
int fs_batch_get_accepts(fs_batch *b, int32_t system, uint32_t *out, size_t n);
int fs_batch_query(const fs_batch *b, int64_t *node_updates_per_launch, int64_t *smem_bytes,
                   int64_t *registers, int64_t *n_items, int64_t *grid, int64_t *walkers_per_tile,
                   size_t n_systems);

/* Library version string. */
const char *fs_version(void);

#ifdef __cplusplus
}
#endif
#endif
