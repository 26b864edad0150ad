/* lenia_gb300.h -- C ABI of the GB300 Lenia engine (sm_103a).
 *
 * Drop-in device engine for leniax's Lenia hot path:
 *   leniax/core.py:13-49          core.update            -> lgx_update
 *   leniax/runner.py:119-164      runner.run_scan        -> lgx_run (trajectories on)
 *   leniax/runner.py:167-215      runner.run_scan_mem_optimized -> lgx_run
 *   leniax/statistics.py:11-128   compute_stats          -> lgx_run (stats output)
 *   leniax/statistics.py:134-205  check_heuristics / N   -> lgx_run (n_continue)
 *   leniax/growth_functions.py:256-264 growth register   -> LGX_GF_* ids
 *   leniax/core.py:322-326        get_state register     -> LGX_STATE_* ids
 *
 * Conventions
 *  - Plain C: raw device pointers, element counts, a cudaStream_t passed as
 *    void*.  No host synchronisation inside any call; all work is ordered on
 *    the given stream.  Calls on the same plan from several host threads are
 *    safe as long as each uses its own workspace.
 *  - All tensors are caller owned and C-contiguous float32.  Spectra are
 *    complex64 stored as interleaved (re, im) float pairs.
 *  - The kernel spectrum is leniax's full complex spectrum
 *    K[1, C, max_k, *world] (kernels.py:145-152) sliced to its Hermitian half
 *    K[..., :W/2+1]: shape [C, max_k, *world[:-1], W/2+1].
 *  - Return value 0 (LGX_OK) on success, otherwise an LGX_ERR_* code;
 *    lgx_last_error() returns the message of the calling thread's last error.
 *    The engine never falls back to a CPU path.
 */
#ifndef LENIA_GB300_H
#define LENIA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LGX_ABI_VERSION 2

#if defined(__GNUC__)
#define LGX_API __attribute__((visibility("default")))
#else
#define LGX_API
#endif

/* status codes */
#define LGX_OK 0
#define LGX_ERR_INVALID 1     /* bad shape / argument / null pointer        */
#define LGX_ERR_UNSUPPORTED 2 /* size, slug or combination not implemented   */
#define LGX_ERR_CUDA 3        /* CUDA runtime error                          */
#define LGX_ERR_WORKSPACE 4   /* workspace smaller than lgx_workspace_bytes  */
#define LGX_ERR_TIMEOUT 5     /* a bounded device-side wait expired          */
#define LGX_ERR_NONFINITE 6   /* reserved: non-finite input detected         */

/* growth functions, leniax/growth_functions.py:256-264 */
#define LGX_GF_POLY_QUAD4 0
#define LGX_GF_GAUSSIAN 1
#define LGX_GF_GAUSSIAN_TARGET 2
#define LGX_GF_STEP 3
#define LGX_GF_STAIRCASE 4
#define LGX_GF_TRIANGLE 5
#define LGX_GF_IDENTITY 6

/* state updates, leniax/core.py:322-326 */
#define LGX_STATE_V1 0     /* clip(s + dt*f, 0, 1)  */
#define LGX_STATE_V2 1     /* s*(1-dt) + dt*f       */
#define LGX_STATE_SIMPLE 2 /* s + dt*f              */

/* engine selection for lgx_run */
#define LGX_ENGINE_AUTO 0
#define LGX_ENGINE_RESIDENT 1 /* one world per CTA slice, state in registers across steps */
#define LGX_ENGINE_STREAMED 2 /* multi-pass, spectra through HBM/L2, any C/K             */
#define LGX_ENGINE_PLAIN 3    /* one world and one Euler step per launch (the reference
                                 one-world-per-launch step): the fused one-kernel step of
                                 the resident engine for its models, else the streamed
                                 engine's kernel sequence                               */
#define LGX_ENGINE_CTA 4      /* one world per CTA, persistent over a work queue: 3D
                                 worlds of side 32 / 64 (C = K = 1)                     */
#define LGX_ENGINE_PLAIN_STREAMED 5 /* one world and one step per launch through the streamed
                                 engine's kernel sequence (row, column, row-inverse and
                                 reduce kernels), for any model the streamed engine runs */
#define LGX_ENGINE_ND 6       /* general N-D engine: any 2D / 3D world whose sides are
                                 2..4096 with prime factors 2, 3, 5, 7 (mixed-radix lines)
                                 or any side 2..2048 (Bluestein chirp-z lines) -- odd,
                                 prime, non-square and 3D sides such as 48^3 included --
                                 with any C and K; line FFT passes over full complex
                                 spectra in HBM                                          */

/* number of scalar statistics besides the C channel masses */
#define LGX_NSTAT_SCALAR 11

/* Static description of a Lenia model: what leniax's build_update_fn
 * (helpers.py:401-427) and KernelMapping (kernels.py:10-63) close over. */
typedef struct lgx_model_desc {
  int nb_dims;          /* 2 or 3                                            */
  int world[3];         /* world axis sizes, outermost first (nb_dims used)  */
  int nb_channels;      /* C                                                 */
  int nb_kernels;       /* K: true kernels, in leniax's channel-sorted order */
  int max_k;            /* kernel slots per channel in the spectrum          */
  const int* kernel_cin;  /* [K] channel read by kernel k                    */
  const int* kernel_slot; /* [K] slot j of kernel k in spectrum[c_in, j]     */
  const int* growth_fn;   /* [K] LGX_GF_* id of kernel k                     */
  int state_fn;           /* LGX_STATE_*                                     */
  int weighted_average;   /* 1: weighted_mean, 0: weighted_sum (core.py:202-242) */
} lgx_model_desc;

typedef struct lgx_plan lgx_plan;

/* A batched rollout: leniax run_scan / run_scan_mem_optimized.
 * Worlds are indexed (sol, init); a solution owns its spectrum, growth
 * parameters, weights and T; inits of a solution share them. */
typedef struct lgx_rollout {
  int n_sols;            /* Ns (1 for run_scan)                                */
  int n_init;            /* Ni worlds per solution                             */
  int steps;             /* max_run_iter                                       */
  const float* cells0;   /* [Ns, Ni, C, *world]                                */
  const float* k_half;   /* [Ns, C, max_k, *world[:-1], W/2+1] complex64        */
  const float* gf_params;/* [Ns, K, 2]   (m, s) per kernel                      */
  const float* weights;  /* [Ns, C, K]   kernels_weight_per_channel             */
  const float* T;        /* [Ns]         dt = 1/T                               */
  float stats_R;         /* static R of compute_stats (statistics.py:22-24)     */
  float stats_T;         /* static T of compute_stats                           */
  float* final_cells;    /* [Ns, Ni, C, *world] or NULL                         */
  float* stats;          /* [Ns, steps, Ni, C + LGX_NSTAT_SCALAR] or NULL:
                            channel_mass[C], mass, mass_volume, mass_density,
                            growth, growth_volume, growth_density, mass_speed,
                            mass_angle_speed, mass_growth_dist, inertia,
                            potential_volume (statistics.py:102-115)            */
  float* n_continue;     /* [Ns, Ni] leniax N = sum_t check_heuristics, or NULL */
  float* n_box;          /* [Ns, Ni] box stop set N (mass < 1e-3, mass > 0.9*area,
                            live cell on the border), or NULL                   */
  float* traj_cells;     /* [steps, Ns*Ni, C, *world] pre-update states, or NULL */
  float* traj_field;     /* [steps, Ns*Ni, C, *world] or NULL                    */
  float* traj_potential; /* [steps, Ns*Ni, K, *world] or NULL                    */
  int engine;            /* LGX_ENGINE_*                                         */
  float* centroid;       /* [Ns, steps, Ni, nb_dims] per-step mass centroid as an
                            absolute torus position in [0, size) per axis (the
                            centred-frame centroid of statistics.py:83 plus the
                            carried shift), or NULL                              */
  void* main_events[2];  /* optional cudaEvent_t pair the engine records on the
                            stream right before and after its dominant kernel(s)
                            (the resident kernel, or the streamed step loop), so
                            callers can time them without a host sync; NULL to skip */
  const float* stats_R_sol; /* [Ns] per-solution static R of compute_stats, or NULL:
                               stats_R for every solution (uneven batches give every
                               world its own R)                                    */
  const float* stats_T_sol; /* [Ns] per-solution static T, or NULL: stats_T        */
} lgx_rollout;

/* ABI version (LGX_ABI_VERSION). */
LGX_API int lgx_version(void);

/* Message of the calling thread's last error ("" if none). */
LGX_API const char* lgx_last_error(void);

/* Validate a model and build a plan (host only, no device work).
 * Replaces helpers.build_update_fn (helpers.py:401-427). */
LGX_API int lgx_plan_create(const lgx_model_desc* desc, lgx_plan** out_plan);

/* Release a plan. */
LGX_API void lgx_plan_destroy(lgx_plan* plan);

/* Engine lgx_run would pick for this plan and batch (LGX_ENGINE_*), or -1. */
LGX_API int lgx_select_engine(const lgx_plan* plan, int n_sols, int n_init, int requested);

/* Workspace bytes lgx_run needs for this batch and engine. */
LGX_API size_t lgx_run_workspace_bytes(const lgx_plan* plan, int n_sols, int n_init, int steps, int engine);

/* Batched rollout, leniax runner.run_scan / run_scan_mem_optimized
 * (runner.py:119-215) including compute_stats and check_heuristics. */
LGX_API int lgx_run(const lgx_plan* plan, const lgx_rollout* job, void* workspace, size_t workspace_bytes,
            void* stream);

/* Device status of the last lgx_run / lgx_update / lgx_batch_run that used
 * `workspace`: 0 on success, 1 if a staged (TMA / bulk) copy did not land
 * within its bounded wait (the outputs are then incomplete).  Copies the word
 * to the host on `stream` and synchronises that stream. */
LGX_API int lgx_workspace_status(const void* workspace, void* stream, int* status);

/* Workspace bytes lgx_update needs for n worlds. */
LGX_API size_t lgx_update_workspace_bytes(const lgx_plan* plan, int n);

/* One Euler step of n worlds sharing one spectrum: leniax core.update
 * (core.py:13-49) with get_potential_fft / get_field / get_state.
 *   state [n, C, *world]; dt: 1 value, or n values when dt_per_world != 0;
 *   gf_params [K, 2]; weights [C, K]; outputs state_out [n, C, *world],
 *   field_out [n, C, *world] and potential_out [n, K, *world] (the latter two
 *   may be NULL). */
LGX_API int lgx_update(const lgx_plan* plan, int n, const float* state, const float* k_half, const float* gf_params,
               const float* weights, const float* dt, int dt_per_world, float* state_out, float* field_out,
               float* potential_out, void* workspace, size_t workspace_bytes, void* stream);

/* ---------------------------------------------------------------------------
 * Differentiation.  leniax differentiates its rollout with jax.grad through
 * the FFT (runner.py:363-448, make_pipeline_fn / make_gradient_fn); this
 * engine provides the adjoint by hand, for every model lgx_run runs with the
 * resident, streamed or N-D engines: 2D and 3D worlds, any number of channels
 * and kernels, weighted mean or sum (core.py:202-242).  2D C = K = 1 square
 * worlds of 32..256 take the specialised one-kernel adjoint, every other
 * model the general N-D adjoint.  The caller checkpoints states with
 * lgx_run, recomputes each segment's states s_t and potentials u_t (lgx_run
 * trajectories), and walks the segments backwards with lgx_adjoint. */
#define LGX_CLIP_GRAD_STE 0  /* clip gradient = 1 (leniax get_state v1, core.py:267-270) */
#define LGX_CLIP_GRAD_MASK 1 /* clip gradient = 1 where 0 < s + dt f < 1, else 0 */

typedef struct lgx_adjoint_job {
  int n_sols, n_init, steps;    /* batch as in lgx_rollout; steps of this segment     */
  const float* k_half;          /* [Ns, C, max_k, *world[:-1], W/2+1] complex64 spectra
                                   (the lgx_rollout layout)                           */
  const float* gf_params;       /* [Ns, K, 2]                                         */
  const float* weights;         /* [Ns, C, K]                                         */
  const float* T;               /* [Ns]   dt = 1/T                                    */
  const float* traj_cells;      /* [steps, Ns*Ni, C, *world] states entering each step */
  const float* traj_potential;  /* [steps, Ns*Ni, K, *world] potentials of each step  */
  const float* lambda_in;       /* [Ns*Ni, C, *world] dL/d(state after the segment)   */
  float* lambda_out;            /* [Ns*Ni, C, *world] dL/d(state before the segment);
                                   must not alias lambda_in                           */
  float* kernel_grad_acc;       /* kernel-gradient accumulator of
                                   lgx_adjoint_kernel_grad_acc_bytes bytes, zeroed by the
                                   caller before the first (last-in-time) segment     */
  float* grad_gf;               /* [Ns, K, 2] dL/d(m, s) per kernel, accumulated (+=)  */
  float* grad_weights;          /* [Ns, C, K] dL/d(kernels_weight_per_channel), every
                                   entry (zero weights included), accumulated (+=)     */
  int clip_grad;                /* LGX_CLIP_GRAD_*                                    */
  const float* cells_after;     /* [Ns*Ni, C, *world] state after the segment's last step
                                   (the next checkpoint, or the rollout's result), or NULL.
                                   With LGX_CLIP_GRAD_MASK the clip's mask is then read from
                                   the forward's own outputs -- 1 where the next state lies
                                   strictly inside (0, 1) -- so it is the exact derivative of
                                   the map the forward computed; without it the mask is
                                   re-derived from s + dt f                             */
} lgx_adjoint_job;

/* Adjoint engine of a plan: LGX_ENGINE_AUTO (default: the one-kernel adjoint
 * for 2D C = K = 1 square worlds of 32..256, the general N-D adjoint
 * otherwise) or LGX_ENGINE_ND (the general N-D adjoint for every model).  Set
 * before the plan's adjoint calls: the workspace and accumulator sizes, the
 * accumulator layout and lgx_adjoint_kernel_grad follow it. */
LGX_API int lgx_plan_set_adjoint_engine(lgx_plan* plan, int engine);

/* Workspace bytes of lgx_adjoint (and lgx_adjoint_kernel_grad) for a batch;
 * 0 when the model has no adjoint. */
LGX_API size_t lgx_adjoint_workspace_bytes(const lgx_plan* plan, int n_sols, int n_init);

/* Bytes of the kernel-gradient accumulator (lgx_adjoint_job.kernel_grad_acc)
 * for a batch; 0 when the model has no adjoint. */
LGX_API size_t lgx_adjoint_kernel_grad_acc_bytes(const lgx_plan* plan, int n_sols, int n_init);

/* Reverse one segment of a rollout (see above). */
LGX_API int lgx_adjoint(const lgx_plan* plan, const lgx_adjoint_job* job, void* workspace, size_t workspace_bytes,
                        void* stream);

/* dL/d(real kernel) [Ns, K, *world] from the accumulator after the last
 * segment: the gradient with respect to each kernel's world-sized, fftshifted
 * real kernel whose fftn is its spectrum (kernels.py:145-149), summed over the
 * inits of a solution; chain it to ring weights b etc. on the caller side.
 * Workspace: lgx_adjoint_workspace_bytes. */
LGX_API int lgx_adjoint_kernel_grad(const lgx_plan* plan, int n_sols, int n_init, const float* kernel_grad_acc,
                                    float* grad_kernel, void* workspace, size_t workspace_bytes, void* stream);

/* leniax's kernel spectrum on the device: fftn of `planes` real H x W planes
 * (world-sized, fftshifted kernels, kernels.py:145-149) written as Hermitian
 * halves [planes, H, W/2+1] complex64.  Square worlds of 32..256.  Workspace:
 * planes * H * W * 4 bytes. */
LGX_API int lgx_kernel_spectrum(int H, int W, int planes, const float* k_real, float* k_half, void* workspace,
                                size_t workspace_bytes, void* stream);

/* The same for any world of the N-D engine: fftn of `planes` real planes
 * [planes, *world] written as Hermitian halves [planes, *world[:-1], W/2+1]
 * complex64.  world[] holds nb_dims (2 or 3) sides, outermost first. */
LGX_API size_t lgx_kernel_spectrum_nd_workspace_bytes(int nb_dims, const int* world, int planes);
LGX_API int lgx_kernel_spectrum_nd(int nb_dims, const int* world, int planes, const float* k_real, float* k_half,
                                   void* workspace, size_t workspace_bytes, void* stream);

/* The step's pointwise stages on their own, for callers of leniax's building
 * blocks (every pointer a device pointer, stream-ordered, no workspace):
 *   lgx_growth   replaces the growth_functions.* calls of core.get_field
 *                (growth_functions.py:6-253): out[n, K, cells] = growth_k(potential)
 *                with gf_ids[k] (host array of K LGX_GF_* ids) and gf_params [K, 2];
 *   lgx_weighted replaces core.weighted_sum / weighted_mean (core.py:202-242):
 *                out[n, C, cells] = sum_k weights[c, k] fields[n, k] (divided by
 *                sum_k weights[c, k] when mean != 0);
 *   lgx_field    replaces core.get_field (core.py:163-199): growth and merge fused;
 *   lgx_state    replaces core.get_state / get_state_v2 / get_state_simple
 *                (core.py:245-319): out = f(state, field, dt) for LGX_STATE_* id,
 *                dt a scalar (dt_per_world 0) or [n].
 * Shapes: n worlds, K kernels <= 64, C channels <= 16, `cells` per plane. */
LGX_API int lgx_growth(int n, int K, long cells, const int* gf_ids, const float* potential, const float* gf_params,
                       float* out, void* stream);
LGX_API int lgx_weighted(int n, int K, int C, long cells, const float* fields, const float* weights, int mean,
                         float* out, void* stream);
LGX_API int lgx_field(int n, int K, int C, long cells, const int* gf_ids, const float* potential,
                      const float* gf_params, const float* weights, int mean, float* field, void* stream);
LGX_API int lgx_state(int n, int C, long cells, int state_fn, const float* state, const float* field,
                      const float* dt, int dt_per_world, float* out, void* stream);

/* Measurement helper (no counterpart in the reference): launch a pure-FMA
 * kernel of `blocks` x 256 threads and return the number of FP32 flops it
 * performs (or -1).  Timing it with events gives the FP32-pipe peak used as
 * the roofline of the resident engine.  `sink` is a device buffer of at
 * least `blocks` floats (written only if an impossible value appears). */
LGX_API long long lgx_fp32_probe(float* sink, int blocks, int iters, void* stream);

/* Failure-detection self test (no counterpart in the reference): one block
 * arms an mbarrier for two arrivals, makes one, and waits on it with the
 * engines' bounded wait, limited to `max_polls` polls.  The wait runs out,
 * the kernel writes the engines' timeout status (1) to `status` (a device int)
 * and returns; nothing faults and the context stays usable.  Returns
 * LGX_OK / LGX_ERR_INVALID / LGX_ERR_CUDA. */
LGX_API int lgx_selftest_wait_timeout(int max_polls, int* status, void* stream);

/* ---------------------------------------------------------------------------
 * Allocation-free rollout.  No counterpart in the reference: leniax runs on
 * JAX, which owns all device buffers.
 *
 * lgx_run_noalloc is lgx_run for resident models (2D, C=1, K=1, square worlds
 * of 32, 64 or 128) for callers that cannot allocate device memory when they
 * call the engine -- typically a host runtime that reserves nearly all GPU
 * memory for its own pool at start-up (a JAX/XLA process calling this engine
 * from a custom call, say), where a cudaMalloc fails or competes with that
 * pool, or a latency-sensitive caller that must not pay for the implicit
 * synchronisation of cudaMalloc/cudaFree.  The caller passes inputs and
 * outputs only (job->main_events and job->engine are ignored).
 *
 * The engine's scratch is a fixed device array of LGX_NOALLOC_SCRATCH_BYTES
 * that every GPU loading this library holds until the process exits.  The
 * first call on a device -- and the first call in any other CUDA context on
 * it, e.g. after a device reset or from a non-primary context -- resolves the
 * array's device address in that context; make that first call before any
 * stream capture.  The call itself performs no allocation.  steps = 0 behaves
 * as in lgx_run (initial cells copied to final_cells, stop counts 0) and uses
 * no scratch.  All calls on a device share the one array: calls
 * whose GPU work overlaps (other streams, other host threads) race on it and
 * must be serialised by the caller.  Batches needing more scratch than the
 * array holds (lgx_noalloc_scratch_bytes) are rejected with LGX_ERR_WORKSPACE;
 * messages are read with lgx_noalloc_last_error(). */
#define LGX_NOALLOC_SCRATCH_BYTES (16u * 1024u * 1024u)

/* Scratch bytes a batch needs (0 for an invalid request). */
LGX_API size_t lgx_noalloc_scratch_bytes(const lgx_plan* plan, int n_sols, int n_init, int steps);

/* lgx_run without a workspace: see above. */
LGX_API int lgx_run_noalloc(const lgx_plan* plan, const lgx_rollout* job, void* stream);

/* Message of the calling thread's last lgx_run_noalloc error ("" if none). */
LGX_API const char* lgx_noalloc_last_error(void);

/* ---------------------------------------------------------------------------
 * Ring kernels built on the device, a batch at a time: leniax's circle_2d
 * (kernels.py:176-212) with the kernel_functions registry, placed and
 * fftshifted as get_kernels_and_mapping does (kernels.py:66-158), each with its
 * own R, r, ring weights and kernel-function parameters; optionally their
 * Hermitian half spectra.  r R is formed in double precision and rounded to
 * float, as leniax forms it from Python floats.
 * ------------------------------------------------------------------------- */
#define LGX_KF_POLY_QUAD 0
#define LGX_KF_GAUSS_BUMP 1
#define LGX_KF_STEP 2
#define LGX_KF_GAUSS 3
#define LGX_KF_THRESHOLD 4
#define LGX_KF_STAIRCASE 5
#define LGX_KF_TRIANGLE 6

typedef struct lgx_ring_batch {
  int nb_dims;  /* 2 or 3 */
  int size;     /* world side: any square / cubic side the N-D engine takes (2..4096) */
  int n;        /* kernels */
  int kf_id;    /* LGX_KF_* */
  int nb_max;   /* row length of b */
  const float* R;         /* [n] world radius */
  const float* r;         /* [n] relative kernel radius (k_params[0]) */
  const float* b;         /* [n, nb_max] ring weights (k_params[1], zero-padded) */
  const int* nb;          /* [n] ring counts, 1..nb_max */
  const float* kf_params; /* [n, 2] kernel-function parameters (the second only for staircase / triangle) */
  float* kernel_out;      /* [n, size^nb_dims] normalised, fftshifted real kernels */
  float* k_half;          /* [n, size^(nb_dims-1), size/2+1] complex64 half spectra, or NULL */
  int* status;            /* device int, set to 1 if a kernel box (2 ceil(r R) cells) exceeds the
                             world or a ring count is out of range (that kernel is left zero) */
} lgx_ring_batch;

LGX_API int lgx_ring_kernels_workspace_bytes(const lgx_ring_batch* job, size_t* bytes);
LGX_API int lgx_ring_kernels(const lgx_ring_batch* job, void* workspace, size_t workspace_bytes, void* stream);

/* ---------------------------------------------------------------------------
 * Initial states generated on the device (leniax initializations.py:10-116 and
 * perlin.py:16-71; make_array_compressible, loader.py:16-30): nb_init states
 * per world from the world's 64-bit seed.  Random numbers: a counter-based
 * SplitMix64 hash of (seed, stream, index), not JAX's threefry stream.
 * ------------------------------------------------------------------------- */
#define LGX_INIT_RANDOM_UNIFORM 0 /* uniform [0, maxval_i), maxval = linspace(0.4, 1, nb_init) */
#define LGX_INIT_PERLIN 1         /* Perlin noise normalised per state, scaled from gf m */
#define LGX_INIT_CROPPED_PERLIN 2 /* the 2 ceil(R) square at [24, 24 + 2 ceil(R)) on a zero 128 x 128 world */

typedef struct lgx_init_job {
  int kind;          /* LGX_INIT_* */
  int n_worlds;
  int nb_init;       /* states per world */
  int H, W;          /* 2D world */
  float R;           /* kernel radius of the Perlin periods (world_params R) */
  int compressible;  /* 1: round to the NB_CHARS^2 - 1 grid of make_array_compressible */
  const uint64_t* seeds; /* [n_worlds] device */
  const float* gf_m;     /* [n_worlds] device: m of the first kernel (Perlin kinds) */
  float* out;            /* [n_worlds, nb_init, H, W] */
  const float* angles;   /* Perlin kinds: [n_worlds, nb_init, res0, res1] gradient angles in
                            radians, res0 = H // (3 ceil R), res1 = W // (2 ceil R) -- the
                            `angles` input of perlin.py:16-71 -- or NULL to draw them
                            uniformly in [0, 2 pi) from the seeds */
} lgx_init_job;

LGX_API int lgx_init_cells_workspace_bytes(const lgx_init_job* job, size_t* bytes);
LGX_API int lgx_init_cells(const lgx_init_job* job, void* workspace, size_t workspace_bytes, void* stream);

/* ---------------------------------------------------------------------------
 * Uneven batch: thousands of worlds of different sizes, dimensions, kernels,
 * growth parameters and time steps in ONE persistent launch.  Replaces
 * leniax's vmap over identically shaped worlds (leniax/runner.py:167-215,
 * run_scan_mem_optimized) when a search mixes world shapes.
 *
 * Worlds are grouped in classes of one shape.  Every world carries its own
 * kernel spectrum, growth parameters (m, s), kernel weight and T, and is
 * updated as core.update with one kernel on one channel (C = K = 1).
 * Supported shapes: 2D 32^2, 64^2, 128^2, 256^2; 3D 32^3, 64^3.
 *
 * lgx_batch_run only launches kernels and stream-ordered copies on `stream`
 * (no host synchronisation, no allocation), so it can be captured in a CUDA
 * graph; replays rebuild the work queue on the device.
 * ------------------------------------------------------------------------- */
#define LGX_BATCH_MAX_CLASSES 8

/* Queue order of the work items. */
#define LGX_ORDER_LARGEST_FIRST 0 /* classes by estimated item cost, largest first */
#define LGX_ORDER_AS_GIVEN 1      /* classes in the order of the classes array */
#define LGX_ORDER_EXPLICIT 2      /* classes in the order of job->class_order */

typedef struct lgx_batch_class {
  int nb_dims;   /* 2 or 3 */
  int size;      /* side of the (square / cubic) torus */
  int n_worlds;  /* >= 0 */
  int gf_id;     /* LGX_GF_* */
  int state_fn;  /* LGX_STATE_* */
  int mean;      /* 1: weighted_mean, 0: weighted_sum (core.py:202-242) */
  const float* cells0;    /* [n_worlds, size^nb_dims] */
  const float* k_half;    /* [n_worlds, size^(nb_dims-1), size/2+1] complex64: each world's
                             kernel spectrum (kernels.py:145-152) sliced to its Hermitian half */
  const float* gf_params; /* [n_worlds, 2]: m, s */
  const float* weights;   /* [n_worlds]: kernel weight */
  const float* T;         /* [n_worlds]: dt = 1 / T */
  const float* stats_R;   /* [n_worlds]: R of compute_stats; needed when any stats output is set */
  const float* stats_T;   /* [n_worlds]: T of compute_stats */
  float* final_cells;     /* [n_worlds, size^nb_dims] */
  float* stats;           /* [n_worlds, steps, 12] (compute_stats order, C = 1) or NULL */
  float* n_continue;      /* [n_worlds]: check_heuristics N, or NULL */
  float* n_box;           /* [n_worlds]: N with the bounding-box stop (runner.py:24-25), or NULL */
  float* centroid;        /* [n_worlds, steps, nb_dims]: absolute torus centroid, or NULL */
} lgx_batch_class;

typedef struct lgx_batch_job {
  int n_classes; /* 1 .. LGX_BATCH_MAX_CLASSES */
  int steps;
  const lgx_batch_class* classes;
  int order;      /* LGX_ORDER_* */
  int grid;       /* persistent CTAs; 0 = one per SM */
  int line_group; /* lanes per 3D line transform: 2 or 4; 0 = 4 */
  const int* class_order; /* host array [n_classes], a permutation of 0..n_classes-1
                             (LGX_ORDER_EXPLICIT only; read during the call) */
} lgx_batch_job;

/* Workspace for lgx_batch_run (depends on the classes, steps and grid):
 * *bytes on LGX_OK; LGX_ERR_INVALID / LGX_ERR_UNSUPPORTED for a bad job. */
LGX_API int lgx_batch_workspace_bytes(const lgx_batch_job* job, size_t* bytes);
/* Run every world of every class for `steps` steps.  Returns LGX_ERR_INVALID /
 * LGX_ERR_UNSUPPORTED for a bad job without launching anything. */
LGX_API int lgx_batch_run(const lgx_batch_job* job, void* workspace, size_t workspace_bytes, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* LENIA_GB300_H */
