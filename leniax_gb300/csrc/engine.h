// Internal interfaces between the C ABI layer and the CUDA kernels.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/lenia_gb300.h"

namespace lgx {

constexpr int kMaxKernels = 64;
constexpr int kMaxChannels = 16;

struct Model {
  int nb_dims;
  int world[3];
  int C, K, max_k;
  int cin[kMaxKernels];
  int slot[kMaxKernels];
  int gf[kMaxKernels];
  int state_fn;
  int mean;
  // derived
  int H, W, D;  // D = 1 for 2D
  long cells;   // D*H*W
};

// Record `msg` as the calling thread's lgx_last_error() and return `code`.
int api_error(int code, const char* msg);

// Unique id of the calling thread's current CUDA context (false if none).
bool current_context_id(unsigned long long* id);

// The model a plan was built from (capi.cu).
const Model* plan_model(const lgx_plan* plan);

// ---------------------------------------------------------------- resident
// Prepared spectrum pitch (float2) of the resident engine for an N x N world.
inline int resident_kpitch(int N) { return N / 2 + 2; }
bool resident_supported(const Model& m);
size_t resident_smem_bytes(int N);

struct ResidentArgs {
  int n_worlds, n_init, steps;
  int gf_id, state_fn, mean;
  const float* cells0;  // [n_worlds, N, N]
  const float2* kp;     // [Ns, N, kpitch]
  const float* gf;      // [Ns, K=1, 2]
  const float* w;       // [Ns, C=1, K=1]
  const float* T;       // [Ns]
  float* final_cells;   // [n_worlds, N, N] or null
  float* raw;           // [Ns, steps, Ni, raw_stride(1)]
  float* traj_cells;    // [steps, n_worlds, N, N] or null
  float* traj_field;
  float* traj_pot;
  int* status;          // device error word (0 = ok)
  // carried torus shift (statistics.py:117-124) across launches, [n_worlds, 2]
  // (y, x), or null: read before the first step, written after the last.  The
  // one-world-per-launch engine chains single-step launches through it.
  const int* shift_in;
  int* shift_out;
  // 1: no statistics are read from this rollout (no raw moments, no carried
  // shift): the 128 x 128 kernel then skips their per-cell work
  int no_stats;
};
cudaError_t launch_resident(int N, const ResidentArgs& a, int grid, cudaStream_t st);
int resident_max_grid(int N);

// Prepare the resident spectra: kp[s][ky][c] from the half spectrum.
cudaError_t launch_prepare_resident_spectrum(int N, int n_sols, const float2* k_half, float2* kp,
                                             cudaStream_t st);

// ---------------------------------------------------------------- uneven batch
// One world per CTA for sizes beyond the resident slices: 2D 256^2 and 3D
// 32^3 / 64^3.  World w belongs to solution w / n_init (spectrum and
// parameters per solution; n_init = 1 in uneven batches, where every world is
// its own solution); raw moments are [n_sols, steps, n_init, raw_stride(1)].
struct BigArgs {
  int n_worlds, n_init, steps;
  int gf_id, state_fn, mean;
  const float* cells0;   // [n_worlds, N^nd]
  const float2* kp;      // per solution; 2D: [N, N/2+2] (resident layout); 3D: [N, N, N/2+1] / N^3
  const float* gf;       // [n_sols, 2]
  const float* w;        // [n_sols]
  const float* T;        // [n_sols]
  float* state;          // [n_worlds, N^nd]: final cells (updated in place from step 1)
  float* raw;            // [n_worlds, steps, raw_stride(1)]
  float2* scratch;       // [grid, scratch_per_cta] spectrum scratch
  long scratch_per_cta;  // float2 elements
  int* status;           // device status word (set when a staged copy never lands), or null
  // 3D items: per-step outputs [steps, n_worlds, N^3] (pre-update cells, field, potential), or null
  float* traj_cells;
  float* traj_field;
  float* traj_pot;
  const float* dt;  // dt_mode 1: dt[0]; 2: dt[world]
  int dt_mode;      // 0: 1 / T[sol] (rollouts); 1: one dt; 2: one dt per world (single updates)
};
enum BatchKind : int { BK_R32 = 0, BK_R64 = 1, BK_R128 = 2, BK_B2D256 = 3, BK_B3D32 = 4, BK_B3D64 = 5 };
constexpr int kMaxBatchClasses = 8;
struct BatchClassArgs {
  int kind, gf_variant, line_group;  // line_group: 3D y/z line transform lanes (2 or 4)
  ResidentArgs r;                    // resident kinds (n_init = 1)
  BigArgs b;                         // big kinds
};
struct MixedArgs {
  int n_items, n_cls;
  const int2* items;           // [n_items] (class, item within class), processing order
  int* head;                   // queue head counter, zeroed before the launch
  const BatchClassArgs* cls;   // [n_cls] in device memory
};
// Spectrum scratch (float2 elements) one CTA needs for a big kind.
long batch_scratch_per_cta(int kind);
// Worlds processed per item of a kind.
int batch_worlds_per_item(int kind);
size_t mixed_smem_bytes();
int batch_kind_gf_variant(int gf_id);
cudaError_t launch_mixed(const MixedArgs& a, int grid, cudaStream_t st);
// Work queue and class table of one mixed launch, written on the device so a
// captured graph rebuilds them on every replay.
struct BatchSetup {
  BatchClassArgs cls[kMaxBatchClasses];
  int n_cls, n_items;
  int first_item[kMaxBatchClasses + 1];  // queue position of each rank's first item
  int cls_of_rank[kMaxBatchClasses];     // class processed at each rank
  BatchClassArgs* cls_out;
  int2* items;
  int* head;
};
cudaError_t launch_batch_setup(const BatchSetup& s, cudaStream_t st);
// lgx_run's one-world-per-CTA path: one class of big items (3D 32^3 / 64^3
// or 2D 256^2) through the mixed kernel.  setup_ws holds the class table and
// queue (big_rollout_setup_bytes), b.scratch grid * big_kind_scratch float2.
size_t big_rollout_setup_bytes(int n_worlds);
long big_kind_scratch(int nb_dims, int size);
cudaError_t launch_big_rollout(int nb_dims, int size, const BigArgs& b, int gf_id, int grid, void* setup_ws,
                               cudaStream_t st);
// 3D prepared spectrum: the [n, N, N, N/2+1] half spectrum scaled by 1/N^3.
cudaError_t launch_prepare_3d_spectrum(int N, long n, const float2* k_half, float2* kp, cudaStream_t st);

// ---------------------------------------------------------------- streamed
struct StreamedArgs;  // defined in streamed.cu
bool streamed_supported(const Model& m);
size_t streamed_workspace_bytes(const Model& m, int n_worlds, int n_sols);
int streamed_blocks_per_world(const Model& m);
// One step of n_worlds worlds (all solutions): see streamed.cu.
struct StreamedStep {
  const Model* m;
  int n_worlds, n_init;
  const float* state;      // [n_worlds, C, *world]
  float* state_out;        // [n_worlds, C, *world]
  const float2* kp;        // [Ns, C, max_k, W/2+2, H] prepared (scaled) spectra, column-major, per solution
  long kp_sol_stride;      // float2 elements between solutions (0: shared)
  const float* gf;         // [Ns, K, 2]
  long gf_sol_stride;
  const float* w;          // [Ns, C, K]
  long w_sol_stride;
  const float* dt;         // per world (dt_world=1) or per solution
  int dt_mode;             // 0: scalar dt[0]; 1: dt[world]; 2: 1/T[sol]
  float* field_out;        // [n_worlds, C, *world] or null
  float* pot_out;          // [n_worlds, K, *world] or null
  float* raw;              // raw moments [.., RAWS] for this step (indexed by world), or null
  long raw_world_stride;   // stride between worlds in floats (sol/init mapping below)
  long raw_sol_stride;
  int* shift;              // [n_worlds, 3] carried torus shift (read; updated by the stats reducer)
  float2* spec;            // workspace [n_worlds, C, H/2, W] packed row spectra
  float2* prod;            // workspace [n_worlds, K, H/2, W] packed product spectra
  float* partial;          // workspace per-block raw partials
  int* status;             // device status word (0 = ok; set when a staged copy times out), or null
  bool spec_ready;         // spec already holds the row spectra of `state` (written by the previous step)
  bool emit_spec;          // write the row spectra of `state_out` into spec for the next step
};
cudaError_t launch_streamed_step(const StreamedStep& s, cudaStream_t st);
// The step's moment reducer (bpw blocks of partials per world).
cudaError_t launch_streamed_reduce(const StreamedStep& s, int bpw, cudaStream_t st);
// Square 2D worlds of even side factoring into 2, 3, 5, 7 (not a power of
// two): the mixed-radix streamed step of generic.cu.
bool generic_size(int n);
int generic_blocks_per_world(int n);
cudaError_t launch_generic_step(const StreamedStep& s, cudaStream_t st);
cudaError_t launch_prepare_generic_spectrum(const Model& m, int n_sols, const float2* k_half, float2* kp,
                                            cudaStream_t st);
cudaError_t launch_prepare_streamed_spectrum(const Model& m, int n_sols, const float2* k_half, float2* kp,
                                             cudaStream_t st);

// ---------------------------------------------------------------- general N-D engine
// Any 2D / 3D torus whose sides factor into 2, 3, 5, 7 (2..512), any C and K:
// mixed-radix line passes over full complex spectra in HBM (nd.cu).
bool nd_side_ok(int n);
int nd_max_side();  // longest world axis of the N-D engine
bool nd_supported(const Model& m);
int nd_blocks_per_world(const Model& m, long n_worlds);
// Prepared spectra [Ns, C, max_k, cells] complex: the Hermitian half
// [Ns, C, max_k, D, H, W/2+1] extended to the full spectrum, scaled by 1/cells.
size_t nd_prepared_bytes(const Model& m, int n_sols);
cudaError_t launch_nd_prepare(const Model& m, int n_sols, const float2* k_half, float2* kf, cudaStream_t st);
struct NdStep {
  const Model* m;
  int n_worlds, n_init;
  const float* state;   // [n_worlds, C, cells]
  float* state_out;     // [n_worlds, C, cells]
  const float2* kf;     // prepared spectra per solution
  long kf_sol_stride;   // float2 elements between solutions (0: shared)
  const float* gf;      // [Ns, K, 2]
  long gf_sol_stride;
  const float* w;       // [Ns, C, K]
  long w_sol_stride;
  const float* dt;
  int dt_mode;          // 0: dt[0]; 1: dt[world]; 2: 1 / T[sol]
  float* field_out;     // [n_worlds, C, cells] or null
  float* pot_out;       // [n_worlds, K, cells] or null
  float* raw;           // raw moments of this step, or null
  long raw_world_stride, raw_sol_stride;
  int* shift;           // [n_worlds, 3] carried torus shift (read, then advanced)
  int* done;            // [n_worlds] per-world block counters, zero before the first step (kept zero)
  float* state_copy;    // [n_worlds, C, cells] copy of the entering state (trajectory), or null
  void* ws;             // nd_step_workspace_bytes
};
size_t nd_step_workspace_bytes(const Model& m, int n_worlds);
cudaError_t launch_nd_step(const NdStep& s, cudaStream_t st);
struct NdAdjoint {
  int n_sols, n_init, steps, clip_mask;
  const float2* k_half;         // [Ns, C, max_k, D, H, W/2+1]
  const float* gf_params;       // [Ns, K, 2]
  const float* weights;         // [Ns, C, K]
  const float* T;               // [Ns]
  const float* traj_cells;      // [steps, nw, C, cells]
  const float* traj_potential;  // [steps, nw, K, cells]
  const float* lambda_in;       // [nw, C, cells]
  float* lambda_out;            // [nw, C, cells]
  float2* gk;                   // [nw, K, cells] kernel-gradient spectra (+=)
  float* grad_gf;               // [Ns, K, 2] (+=)
  float* grad_weights;          // [Ns, C, K] (+=)
  const float* cells_after;     // [nw, C, cells] state after the last step, or null
};
size_t nd_adjoint_workspace_bytes(const Model& m, int n_sols, int n_init);
size_t nd_kernel_grad_acc_bytes(const Model& m, int n_sols, int n_init);
cudaError_t launch_nd_adjoint(const Model& m, const NdAdjoint& j, void* ws, cudaStream_t st);
size_t nd_kernel_grad_workspace_bytes(const Model& m, int n_sols);
// dL/d(world-sized real kernel) [Ns, K, cells] from the accumulated spectra.
cudaError_t launch_nd_kernel_grad(const Model& m, int n_sols, int n_init, const float2* gk, float* out, void* ws,
                                  cudaStream_t st);
size_t nd_spectrum_workspace_bytes(int nb_dims, const int* world, int planes);
cudaError_t launch_nd_spectrum(int nb_dims, const int* world, int planes, const float* k_real, float2* k_half,
                               void* ws, cudaStream_t st);

// ---------------------------------------------------------------- adjoint
struct AdjointSegment {
  int n_sols, n_init, steps;
  int gf_id, state_fn, mean, clip_mask;
  const float* gf_params;       // [Ns, 2]
  const float* weights;         // [Ns]
  const float* T;               // [Ns]
  const float2* kp;             // prepared spectra [Ns, N, N/2+2]
  const float* traj_cells;      // [steps, nw, N, N]
  const float* traj_potential;  // [steps, nw, N, N]
  const float* lambda_in;       // [nw, N, N]
  float* lambda_out;            // [nw, N, N]
  float *lam_a, *lam_b;         // [nw, N, N] ping-pong
  float2* spec;                 // [nw, 2, N/2, N]
  float2* prod;                 // [nw, N/2, N]
  float* partial;               // [nw, 64, 3] per-block parameter partials
  float2* gk;                   // [nw, N/2, N] kernel-gradient accumulator (column domain)
  float* grad_gf;               // [Ns, 2]   +=
  float* grad_w;                // [Ns]      +=
  const float* cells_after;     // [nw, N, N] state after the last step, or null
};
// Resident adjoint (adjoint_resident.cu): one launch per segment for the
// resident sizes, lambda in registers across the segment's steps.
struct AdjResArgs {
  int n_worlds, n_init, steps;
  int gf_id, state_fn, mean, clip_mask;
  const float* gf;              // [Ns, 2]
  const float* w;               // [Ns]
  const float* T;               // [Ns]
  const float2* kp;             // [Ns, N, N/2+2] prepared spectra
  const float* traj_cells;      // [steps, nw, N, N]
  const float* traj_pot;        // [steps, nw, N, N]
  const float* lambda_in;       // [nw, N, N]
  float* lambda_out;            // [nw, N, N]
  float2* gk;                   // [nw, N/2, N] kernel-gradient accumulator (+=)
  float* pacc;                  // [nw, 3] parameter partials (+=)
  const float* cells_after;     // [nw, N, N] state after the last step, or null
};
bool adjoint_resident_supported(const Model& m);
cudaError_t launch_adjoint_resident(int N, const AdjResArgs& a, cudaStream_t st);
// per solution: grad_gf += partial sums 0..1, grad_w += partial sum 2 over its inits and blocks
cudaError_t launch_param_reduce(int n_sols, int n_init, int blocks, const float* partial, float* grad_gf,
                                float* grad_w, cudaStream_t st);
bool adjoint_supported(const Model& m);
bool spectrum_supported(int H, int W);
cudaError_t launch_adjoint_segment(int N, const AdjointSegment& j, cudaStream_t st);
cudaError_t launch_gk_finish(int N, int n_sols, int n_init, const float2* gk, float2* prod, float* out,
                             cudaStream_t st);
cudaError_t launch_spectrum(int N, int planes, const float* k_real, float2* spec, float2* out, cudaStream_t st);

// ---------------------------------------------------------------- stats
// Turn raw moments [Ns, steps, Ni, RAWS] into leniax stats / N / N_box.
struct StatsArgs {
  int n_sols, n_init, steps, C, nb_dims;
  int world[3];
  float R, T;
  const float* R_arr;  // per-solution R overriding R, or null
  const float* T_arr;  // per-solution static T overriding T, or null
  const float* raw;
  float* stats;       // [Ns, steps, Ni, C + 11] or null
  float* n_continue;  // [Ns, Ni] or null
  float* n_box;       // [Ns, Ni] or null
  float* centroid;    // [Ns, steps, Ni, nb_dims] or null
};
cudaError_t launch_stats(const StatsArgs& a, cudaStream_t st);

}  // namespace lgx
