/*
 * cfd_gb300.h -- C ABI of the GB300-native jax-cfd time-stepping hot path.
 *
 * Plain C types only: device pointers are `float*` (complex64 arrays are
 * interleaved float pairs, the memory layout of the reference's complex64
 * rfftn output), streams are `void*` holding a cudaStream_t (NULL = legacy
 * default stream).  Every entry point returns a cfd_status; on failure
 * cfd_last_error() returns a message for the calling thread.  Calls only
 * enqueue work on the stream -- none of them synchronise -- except where a
 * comment says otherwise.
 *
 * Reference interfaces replaced (paths inside the jax-cfd 0.2.1 source tree):
 *   cfd_fvm_plan_create / cfd_fvm_step
 *       jax_cfd/base/equations.py:120-151   semi_implicit_navier_stokes(...)
 *         with forward_euler (time_stepping.py:109-119), the default
 *         convect = advect_van_leer_using_limiters (advection.py:387-395) or
 *         advection.convect_linear (advection.py:183-207), diffuse
 *         (diffusion.py:35-37), forcing built from forcings.py:63-178 and
 *         pressure_solve = pressure.solve_fast_diag (pressure.py:115-157);
 *       jax_cfd/base/funcutils.py:82-88     repeated(step_fn, steps)
 *   cfd_fvm_explicit_terms
 *       jax_cfd/base/equations.py:77-116    navier_stokes_explicit_terms
 *   cfd_fvm_projection
 *       jax_cfd/base/pressure.py:181-198    projection(v, solve_fast_diag)
 *   cfd_fvm_pressure_solve
 *       jax_cfd/base/pressure.py:115-157    solve_fast_diag(v)
 *   cfd_fvm_divergence, cfd_fvm_curl_2d
 *       jax_cfd/base/finite_differences.py:136-143, 186-193
 *   cfd_max_speed, cfd_scale_to_max_speed
 *       jax_cfd/base/initial_conditions.py:67-68, 112-121
 *   cfd_spec_plan_create / cfd_spec_step
 *       jax_cfd/spectral/time_stepping.py:117-197
 *         low_storage_runge_kutta_crank_nicolson / crank_nicolson_rk4 applied
 *         to spectral/equations.py:129-191 NavierStokes2D
 *   cfd_spec_set_forcing
 *       jax_cfd/spectral/equations.py:176-182 (rfft2 of a velocity-independent
 *         forcing + spectral_curl_2d, spectral/utils.py:199-203)
 *   cfd_rfft2, cfd_irfft2, cfd_spectral_filter
 *       jnp.fft.rfftn / irfftn as used by the two steps, and
 *       jax_cfd/base/filter_utils.py:32-42 filter(...)
 */
#ifndef CFD_GB300_H_
#define CFD_GB300_H_

#ifdef __cplusplus
extern "C" {
#endif

typedef enum cfd_status {
  CFD_OK = 0,
  CFD_ERR_INVALID_ARGUMENT = 1, /* bad shape / size / pointer: ValueError */
  CFD_ERR_UNSUPPORTED = 2,      /* option outside the hot path: NotImplementedError */
  CFD_ERR_CUDA = 3,             /* CUDA runtime error: RuntimeError */
  CFD_ERR_OUT_OF_MEMORY = 4,    /* device allocation failed: MemoryError */
  CFD_ERR_DEVICE_FAULT = 5      /* a kernel's bounded wait ran out: DeviceFaultError */
} cfd_status;

/* Advection schemes (the `convect` argument). */
enum { CFD_CONVECT_VAN_LEER = 0, CFD_CONVECT_LINEAR = 1 };

/* Velocity-independent forcing layouts. */
enum {
  CFD_FORCE_NONE = 0,
  CFD_FORCE_U_OF_Y = 1, /* u-forcing depends on j only: table of ny floats  */
  CFD_FORCE_V_OF_X = 2, /* v-forcing depends on i only: table of nx floats  */
  CFD_FORCE_FULL = 3    /* arbitrary fields: force_u, force_v of nx*ny each */
};

typedef struct cfd_fvm_config {
  int nx, ny;             /* grid shape; axis 1 contiguous; powers of 2 in [4, 4096] */
  double hx, hy;          /* grid step along each axis */
  double density;
  int has_viscosity;      /* 0 mirrors viscosity=None */
  double viscosity;
  double dt;
  int convect;            /* CFD_CONVECT_* */
  int has_linear_forcing; /* linear_forcing(grid, coefficient) term present */
  double linear_coefficient;
  int const_forcing;      /* CFD_FORCE_* */
  const float* force_u;   /* HOST pointers, copied at creation (may be NULL) */
  const float* force_v;
} cfd_fvm_config;

typedef struct cfd_fvm_plan cfd_fvm_plan;

const char* cfd_last_error(void);
/* Device-side fault word: non-zero after a kernel's bounded wait on an
 * asynchronous copy ran out (1 = bulk-copy wait); the kernel then skipped its
 * work instead of spinning.  Every compiled unit of the library keeps its own
 * word; this reports the first non-zero one, and clear != 0 resets them all.
 * Synchronous.  No counterpart in the reference (it has no device code). */
int cfd_device_fault(unsigned int* code, int clear);
/* Exercises the give-up path of the bounded waits (no counterpart in the
 * reference): launches one warp whose mbarrier wait can never complete (no
 * copy issued, no arrival) with a limit of `polls` polls, synchronises the
 * stream, and returns CFD_ERR_DEVICE_FAULT with the fault word set to 1 when
 * the wait gave up as designed.  Nothing is left running on the GPU.  Leaves
 * the fault word set: read and clear it with cfd_device_fault. */
int cfd_bounded_wait_selftest(void* stream, int polls);
int cfd_version(void);

int cfd_fvm_plan_create(const cfd_fvm_config* cfg, cfd_fvm_plan** plan);
int cfd_fvm_plan_destroy(cfd_fvm_plan* plan);
/* Device bytes held by the plan (workspace + tables). */
long long cfd_fvm_plan_bytes(const cfd_fvm_plan* plan);

/* `steps` forward-Euler steps; u/v are [nx, ny] float32 on the device at
 * offsets (1, .5) and (.5, 1).  u_out/v_out may alias u/v. */
int cfd_fvm_step(cfd_fvm_plan* plan, void* stream, const float* u,
                 const float* v, float* u_out, float* v_out, int steps);
/* diffusion.solve_fast_diag (jax_cfd/base/diffusion.py:166-212) for periodic
 * velocity components: u_out = u + irfftn(func(lambda) * rfftn(u)) with
 * func(x) = (dt nu) x / (1 - (dt nu) x) on the eigenvalues of the periodic
 * Laplacian (fast_diagonalization.py:199-225), same for v.  u_out/v_out may
 * alias u/v.  Uses the plan's grid, spectrum buffer and column scheme. */
int cfd_fvm_diffusion_solve(cfd_fvm_plan* plan, void* stream, const float* u,
                            const float* v, float* u_out, float* v_out,
                            double nu, double dt);
/* `steps` steps of implicit_diffusion_navier_stokes
 * (jax_cfd/base/equations.py:154-195, diffusion_solve = pressure_solve =
 * solve_fast_diag): convection + forcing / density explicitly, forward Euler
 * with the plan's dt, projection, then the implicit diffusion solve with
 * `viscosity`.  The plan must be created with has_viscosity = 0 (the
 * explicit terms of this step have no diffusion); CFD_ERR_UNSUPPORTED
 * otherwise.  u_out/v_out may alias u/v. */
int cfd_fvm_step_implicit(cfd_fvm_plan* plan, void* stream, const float* u,
                          const float* v, float* u_out, float* v_out, int steps,
                          double viscosity);
/* navier_stokes_rk (time_stepping.py:59-107) with an explicit Butcher
 * tableau of 1-4 stages: `a` holds rows 1 .. stages-1 of the lower triangle
 * concatenated (row i has i entries), `b` the `stages` weights; e.g.
 * midpoint_rk2 a = {0.5}, b = {0, 1}; classic_rk4 a = {0.5, 0, 0.5, 0, 0, 1},
 * b = {1/6, 1/3, 1/3, 1/6}.  Each stage's state is projected; the first call
 * allocates the plan's stage buffers (make it before any stream capture). */
int cfd_fvm_step_rk(cfd_fvm_plan* plan, void* stream, const float* u,
                    const float* v, float* u_out, float* v_out, int steps,
                    int stages, const double* a, const double* b);
/* cfd_fvm_step with a CUDA event pair around every launch; synchronises the
 * stream at the end and writes the mean duration in ms of each kernel kind to
 * ms_out[5] = {explicit stencil, divergence + row rFFT, column pinv,
 * row irFFT, final projection}.  For measurement (bench.py roofline). */
int cfd_fvm_profile(cfd_fvm_plan* plan, void* stream, const float* u,
                    const float* v, float* u_out, float* v_out, int steps,
                    float* ms_out);
/* Autotuner: times `steps` steps for each candidate launch configuration
 * (transform row-block shape x column-pass scheme x stencil scheme x row
 * feed x rows per stencil warp; u, v read-only, results go to the scratch
 * arrays), keeps the fastest
 * in the plan and writes its index (see cfd_fvm_plan_set_launch) to *chosen
 * (may be NULL).  Synchronises the stream. */
int cfd_fvm_plan_autotune(cfd_fvm_plan* plan, void* stream, const float* u,
                          const float* v, float* u_scratch, float* v_scratch,
                          int steps, int* chosen);
/* Pins the launch configuration (an index as cfd_fvm_plan_autotune reports:
 * row-transform shape (0 wide, 1 narrow) + 2 * column scheme (0 blocks,
 * 1/2 clusters of 4/8, 3/4 persistent pipelined groups of 4/2 columns, 5
 * groups of 4 staged by TMA tensor loads) + 12 * stencil scheme (0
 * shared-memory tiles, 1 warp streams) + 24 * row feed (0 registers, 1 bulk
 * copies) + 48 * rows per stencil warp (0: 16, 1: 8, 2: 32; 1 and 2 with warp
 * streams only, each warp re-reading 4 halo rows): 144 choices); results do
 * not depend on it.  cfd_fvm_plan_get_launch returns the current one. */
int cfd_fvm_plan_set_launch(cfd_fvm_plan* plan, int choice);
int cfd_fvm_plan_get_launch(const cfd_fvm_plan* plan);
/* du/dt from advection + diffusion + forcing (no projection). */
int cfd_fvm_explicit_terms(cfd_fvm_plan* plan, void* stream, const float* u,
                           const float* v, float* du, float* dv);
int cfd_fvm_projection(cfd_fvm_plan* plan, void* stream, const float* u,
                       const float* v, float* u_out, float* v_out);
/* Pressure correction q (offset (.5, .5)) with div(v - grad q) = 0. */
int cfd_fvm_pressure_solve(cfd_fvm_plan* plan, void* stream, const float* u,
                           const float* v, float* q);
int cfd_fvm_divergence(cfd_fvm_plan* plan, void* stream, const float* u,
                       const float* v, float* out);
int cfd_fvm_curl_2d(cfd_fvm_plan* plan, void* stream, const float* u,
                    const float* v, float* out);

/* funcutils.trajectory(repeated(step, inner), frames, post_process,
 * start_with_input) (funcutils.py:95-126) for the forward-Euler step, in one
 * call with the frames kept on the device: `frames` chunks of `inner` steps
 * run in place in (u_out, v_out) (which may alias u/v), and frame k -- the
 * state after chunk k, or before it with start_with_input -- is written to
 * frames_out + k * frame_size: CFD_FRAME_VELOCITY stores u then v (2 nx ny
 * floats; post_process = identity), CFD_FRAME_VORTICITY stores curl_2d of
 * the state (nx ny floats at offset (1, 1); post_process = curl_2d). */
enum { CFD_FRAME_VELOCITY = 0, CFD_FRAME_VORTICITY = 1 };
int cfd_fvm_trajectory(cfd_fvm_plan* plan, void* stream, const float* u, const float* v,
                       int inner, int frames, int frame_kind, int start_with_input,
                       float* frames_out, float* u_out, float* v_out);

/* Pressure projection that allocates nothing -- no counterpart in the
 * reference.  For callers that cannot call cudaMalloc (while capturing into a
 * graph memory pool they do not own, under allocators that forbid allocation
 * after start-up, or as a plugin handed only pre-allocated buffers): same
 * result as cfd_fvm_projection, without a plan.  Its scratch (row spectrum,
 * twiddles, Laplacian eigenvalues) is a fixed __device__ array that every GPU
 * loading the library keeps until exit.  Limit: nx * ny <= 262144 (512 x 512),
 * sides powers of two in [4, 4096]; larger grids return
 * CFD_ERR_INVALID_ARGUMENT.  Every call looks up the array's device address
 * in the current context (cudaGetSymbolAddress; the first lookup on a device
 * loads the module, so make the first call before any stream capture).  All
 * calls share the array and it keeps the last call's contents (each call
 * rewrites everything it reads): calls that overlap on the GPU race and must
 * be ordered by the caller.  u_out/v_out may alias u/v. */
int cfd_fvm_projection_noalloc(void* stream, int nx, int ny, double hx,
                               double hy, const float* u, const float* v,
                               float* u_out, float* v_out);

/* Adjoint of one step (no reference C counterpart: the reference gets it from
 * jax.grad through equations.py:120-151).  For the forward step v' = step(v)
 * at state (u, v) and a cotangent (gu, gv) of v', writes the cotangent of v
 * to (gu_out, gv_out) (which may alias gu, gv) and, if nu_dot is not NULL,
 * the per-cell products w . laplacian(v) with w the projected cotangent; the
 * derivative with respect to the viscosity is dt / density * sum(nu_dot).
 * Uses the plan's workspace like cfd_fvm_step. */
int cfd_fvm_adjoint_step(cfd_fvm_plan* plan, void* stream, const float* u,
                         const float* v, const float* gu, const float* gv,
                         float* gu_out, float* gv_out, float* nu_dot);

/* Adjoint of a segment of `steps` steps from the checkpoint (u0, v0), in one
 * call: recomputes the segment's states 1 .. steps-1 by single steps into
 * `states` (2 (steps - 1) nx ny floats, state k's u then v at
 * states + 2 (k - 1) nx ny; NULL when steps == 1), then runs the adjoint
 * steps newest first.  (gu, gv) hold the cotangent of the state after the
 * segment on entry and that of the checkpoint on return.  With nu_acc (a
 * device double) and nu_scratch (nx ny floats) both given, adds
 * sum over steps and cells of nu_dot (cfd_fvm_adjoint_step) to *nu_acc,
 * summed in double in a fixed order; both NULL skips it.  Each state and
 * cotangent is the bits that cfd_fvm_step (one step) and
 * cfd_fvm_adjoint_step give. */
int cfd_fvm_adjoint_segment(cfd_fvm_plan* plan, void* stream, const float* u0,
                            const float* v0, int steps, float* states, float* gu,
                            float* gv, float* nu_scratch, double* nu_acc);

/* ---- Batched FVM trajectories ----
 * Replaces the reference's one-trajectory-at-a-time use of
 * semi_implicit_navier_stokes + funcutils.repeated (equations.py:120-151,
 * funcutils.py:82-88) for many independent trajectories; the reference itself
 * has no batched entry point (callers vmap or loop in Python).
 *
 * A batch holds `count` slots of ONE grid shape, step and convection scheme
 * (taken from `shape`).  Each slot has its own viscosity, density, dt and
 * forcing (set with cfd_fvm_batch_set_slot; forcing tables over one axis
 * only), its own state (u, v) owned by the batch (cfd_fvm_batch_state returns
 * the device pointers) and its own step count for the next chunk
 * (cfd_fvm_batch_set_steps; 0 = idle).  cfd_fvm_batch_run advances every slot
 * by min(its steps, chunk) steps in place with one launch per kernel kind per
 * step for the whole batch; with use_graph != 0 the chunk is captured once per
 * chunk length as a CUDA graph and replayed.  Slot parameters and steps may
 * change between runs (they live in a device table uploaded on the run's
 * stream).  A slot's result does not depend on the other slots. */
typedef struct cfd_fvm_batch cfd_fvm_batch;
int cfd_fvm_batch_create(const cfd_fvm_config* shape, int count, cfd_fvm_batch** batch);
int cfd_fvm_batch_destroy(cfd_fvm_batch* batch);
int cfd_fvm_batch_size(const cfd_fvm_batch* batch);
long long cfd_fvm_batch_bytes(const cfd_fvm_batch* batch);
int cfd_fvm_batch_state(cfd_fvm_batch* batch, int slot, float** u, float** v);
/* Enqueues the forcing-table upload on `stream` (host tables may be reused
 * once the call returns). */
int cfd_fvm_batch_set_slot(cfd_fvm_batch* batch, void* stream, int slot,
                           const cfd_fvm_config* cfg);
int cfd_fvm_batch_set_steps(cfd_fvm_batch* batch, int slot, int steps);
int cfd_fvm_batch_run(cfd_fvm_batch* batch, void* stream, int chunk, int use_graph);
/* Times the launch configurations on a `steps`-step chunk of the current
 * slots, restores their states and keeps the fastest; *chosen = row-transform
 * shape (0 wide, 1 narrow) + 2 * column scheme (0 blocks, 1/2 clusters of
 * 4/8, 3 persistent pipelined groups of 4 columns over all slots staged by
 * cp.async, 4 the same staged by TMA tensor loads) + 10 * stencil (0
 * shared-memory tiles, 1 warp streams), or 20: each member's whole chunk
 * resident in shared memory, one block per member and one launch per chunk
 * (grids whose fields fit: 64x64, 64x128, 128x64), or 21 + (0 .. 19): the
 * same with the row transforms fed by bulk copies (rows of up to 1024
 * points): 41 choices.  Every configuration gives the same bits.
 * Synchronises. */
int cfd_fvm_batch_autotune(cfd_fvm_batch* batch, void* stream, int steps, int* chosen);
/* Pins the batch's launch configuration (index as cfd_fvm_batch_autotune
 * reports); CFD_ERR_UNSUPPORTED for a configuration the grid cannot take.
 * Results do not depend on it. */
int cfd_fvm_batch_set_launch(cfd_fvm_batch* batch, int choice);

/* Per-slot health after a chunk (no counterpart in the reference, whose only
 * failure checks are NaN checks on the state in its tests,
 * spectral/equations_test.py:137,166,233).  Every run ends with a reduction
 * over the state of each slot that ran: flags (CFD_HEALTH_NONFINITE: a NaN or
 * an infinity is present) and max_abs (largest magnitude among the finite
 * values: the largest velocity component for FVM slots, the largest
 * |vorticity spectrum| component for spectral slots).  Slots that did not run
 * keep their record.  The record is device memory owned by the batch, valid
 * once the run has completed on its stream. */
typedef struct cfd_health {
  unsigned int flags;
  float max_abs;
} cfd_health;
enum { CFD_HEALTH_NONFINITE = 1 };
/* Device pointer to the batch's `count` records. */
int cfd_fvm_batch_health(cfd_fvm_batch* batch, const cfd_health** records);
/* Also writes each run's records into `host_records` (`count` cfd_health in
 * pinned host memory, cudaHostAlloc or cudaHostRegister; NULL stops it) from
 * a kernel at the end of the chunk, so a host polling many batches reads
 * them once the run's stream has passed that point, without a
 * device-to-host copy (which would queue on the copy engine behind other
 * transfers).  The memory must outlive the batch's runs. */
int cfd_fvm_batch_set_health_mirror(cfd_fvm_batch* batch, void* host_records);

/* A ragged ensemble: members of any grid shapes, grouped into one batch per
 * (shape, step, convection).  cfd_fvm_ensemble_step advances every member by
 * `steps`; the batches run on forked streams (overlapping on the device), and
 * with use_graph != 0 the whole chunk is one CUDA graph launch. */
typedef struct cfd_fvm_ensemble cfd_fvm_ensemble;
int cfd_fvm_ensemble_create(const cfd_fvm_config* cfgs, int count,
                            cfd_fvm_ensemble** ens);
int cfd_fvm_ensemble_destroy(cfd_fvm_ensemble* ens);
int cfd_fvm_ensemble_size(const cfd_fvm_ensemble* ens);
int cfd_fvm_ensemble_batches(const cfd_fvm_ensemble* ens);
int cfd_fvm_ensemble_state(cfd_fvm_ensemble* ens, int index, float** u,
                           float** v);
/* Device pointer to member `index`'s health record (see cfd_health). */
int cfd_fvm_ensemble_health(cfd_fvm_ensemble* ens, int index, const cfd_health** record);
int cfd_fvm_ensemble_autotune(cfd_fvm_ensemble* ens, void* stream, int steps);
int cfd_fvm_ensemble_step(cfd_fvm_ensemble* ens, void* stream, int steps,
                          int use_graph);

/* max over cells of sqrt(u^2 + v^2) written as one float to device memory. */
int cfd_max_speed(void* stream, int n, const float* u, const float* v,
                  float* out);
/* u = (maximum_velocity * u) / vmax, same for v (vmax read from device). */
int cfd_scale_to_max_speed(void* stream, int n, float* u, float* v,
                           const float* vmax, double maximum_velocity);

typedef struct cfd_spec_config {
  int nx, ny;         /* powers of 2 in [4, 4096] */
  double hx, hy;
  double viscosity;
  double drag;
  double dt;
  int smooth;         /* 1: multiply by the 2/3 brick-wall filter (smooth is
                         not None, including smooth=False); 0: smooth=None */
  int num_stages;     /* low-storage RK/CN stages, 1..8 */
  const double* alphas; /* num_stages + 1 */
  const double* betas;  /* num_stages */
  const double* gammas; /* num_stages */
} cfd_spec_config;

typedef struct cfd_spec_plan cfd_spec_plan;

int cfd_spec_plan_create(const cfd_spec_config* cfg, cfd_spec_plan** plan);
int cfd_spec_plan_destroy(cfd_spec_plan* plan);
long long cfd_spec_plan_bytes(const cfd_spec_plan* plan);
/* Launch configuration of the column passes: 0 per-block columns, 1 clusters
 * of four one-column blocks exchanging rows through distributed shared memory
 * (256 <= nx <= 2048), 2/3 persistent blocks that stage the next group of
 * 4/2 columns with cp.async while transforming the current one in registers
 * (512 <= nx <= 4096), 4 as 2 with each stage's column update and the next
 * stage's column prep fused into one pass; plus 5 x the row scheme: 0 the
 * shared-memory row pass, 1 the register-pass row pass (512 <= ny <= 4096),
 * 2 the same with registers sized for three blocks per multiprocessor (four
 * at ny = 2048; 512 <= ny <= 2048): 15 choices.  Results are bit-for-bit the same for
 * every choice. */
int cfd_spec_plan_set_launch(cfd_spec_plan* plan, int choice);
int cfd_spec_plan_get_launch(const cfd_spec_plan* plan);
/* Velocity-independent forcing (fx, fy real [nx, ny] on the device, either may
 * be NULL): stores 2 pi i (kx rfft2(fy) - ky rfft2(fx)).  Synchronises the
 * stream once to decide whether the table lives only in row kx = 0. */
int cfd_spec_set_forcing(cfd_spec_plan* plan, void* stream, const float* fx,
                         const float* fy);
/* `steps` time steps of the vorticity rfft state [nx, ny/2+1] complex64.
 * w_out may alias w_in. */
int cfd_spec_step(cfd_spec_plan* plan, void* stream, const float* w_in,
                  float* w_out, int steps);
/* cfd_spec_step with event pairs; ms_out[4] = {row pass, column update,
 * column prep, fused column update + prep (column scheme 4)} mean durations
 * in ms (0 for a kind that did not run).  Synchronises the stream. */
int cfd_spec_profile(cfd_spec_plan* plan, void* stream, const float* w_in,
                     float* w_out, int steps, float* ms_out);
/* Explicit terms F(w) of NavierStokes2D (advection, filter, forcing). */
int cfd_spec_explicit_terms(cfd_spec_plan* plan, void* stream,
                            const float* w, float* out);
int cfd_rfft2(cfd_spec_plan* plan, void* stream, const float* x, float* xhat);
/* Destroys nothing: xhat is read-only (a workspace copy is transformed). */
int cfd_irfft2(cfd_spec_plan* plan, void* stream, const float* xhat, float* x);
/* out = irfft2(rfft2(x) * table), table real [nx, ny/2+1] on the device. */
int cfd_spectral_filter(cfd_spec_plan* plan, void* stream, const float* x,
                        const float* table, float* out);

/* Diagnostics (data/xarray_utils.py:155-167, 279-290, 370-401).
 * cfd_energy_spectrum_shells: the isotropic kinetic-energy spectrum, binsum
 * form, of the velocity (u, v) on the plan's grid: out[i] (nbins doubles on
 * the device) = sum over |k| in (ks (i + 0.5), ks (i + 1.5)] of
 * 0.5 (|fft2 u|^2 + |fft2 v|^2), with k = 2 pi fftfreq(n, d) per axis and
 * dnx = nx * hx, dny = ny * hy.  Uses the plan's column-field workspace.
 * cfd_enstrophy_sum: sum over cells of vorticity^2 / 2 (one double on the
 * device); divide by nx * ny for the mean. */
int cfd_energy_spectrum_shells(cfd_spec_plan* plan, void* stream, const float* u,
                               const float* v, double dnx, double dny, double ks,
                               int nbins, double* out);
int cfd_enstrophy_sum(void* stream, int nx, int ny, double hx, double hy,
                      const float* u, const float* v, double* out);

/* ---- Batched spectral trajectories ----
 * The cfd_fvm_batch model for NavierStokes2D + a low-storage RK/CN
 * integrator (spectral/equations.py:129-220, spectral/time_stepping.py:117-197):
 * `count` slots of one grid and stage count; per-slot viscosity, drag, dt and
 * smoothing from cfd_spec_batch_set_slot; the slot's forcing curl table is
 * borrowed from `forcing` (a plan on the same grid after cfd_spec_set_forcing,
 * or NULL for none), which must outlive its use.  cfd_spec_batch_state
 * returns the slot's state (rfft of the vorticity, complex64 nx x (ny/2+1)). */
typedef struct cfd_spec_batch cfd_spec_batch;
int cfd_spec_batch_create(const cfd_spec_config* shape, int count, cfd_spec_batch** batch);
int cfd_spec_batch_destroy(cfd_spec_batch* batch);
int cfd_spec_batch_size(const cfd_spec_batch* batch);
long long cfd_spec_batch_bytes(const cfd_spec_batch* batch);
int cfd_spec_batch_state(cfd_spec_batch* batch, int slot, float** w);
int cfd_spec_batch_set_slot(cfd_spec_batch* batch, int slot, const cfd_spec_config* cfg,
                            const cfd_spec_plan* forcing);
int cfd_spec_batch_set_steps(cfd_spec_batch* batch, int slot, int steps);
int cfd_spec_batch_run(cfd_spec_batch* batch, void* stream, int chunk, int use_graph);
/* Device pointer to the batch's `count` health records (see cfd_health). */
int cfd_spec_batch_health(cfd_spec_batch* batch, const cfd_health** records);
/* As cfd_fvm_batch_set_health_mirror. */
int cfd_spec_batch_set_health_mirror(cfd_spec_batch* batch, void* host_records);


#ifdef __cplusplus
}
#endif

#endif /* CFD_GB300_H_ */
