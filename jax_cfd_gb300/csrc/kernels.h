// Internal launch interface between the C ABI (capi.cu) and the kernels.
#pragma once

#include <cuda_runtime.h>

#include <string>

namespace cfd {

// Records the message cfd_last_error() returns on this thread.
void set_last_error(const std::string& msg);

// Reads (and optionally clears) the device fault word that bounded waits set.
cudaError_t read_device_fault(unsigned int* code, bool clear);

// Parameters of the staggered-grid (FVM) explicit step, already rounded to
// float32 the way the reference rounds its weakly typed Python scalars.
struct FvmParams {
  int nx, ny;          // grid shape; axis 1 (y, index j) is contiguous
  int log2nx, log2ny;
  float hx, hy;        // float32(step)
  float inv_hx, inv_hy;  // float32(1 / float32(step)): x / h is taken as x * (1/h)
  float cfl_x, cfl_y;  // float32(dt / step): Lax-Wendroff Courant factors
  float dt;            // float32(dt)
  float nu;            // float32(viscosity / density)
  float sx, sy, ssum;  // Laplacian scales (1/h)^2 formed in float32
  float lin;           // linear forcing coefficient
  float density;
  int rho_is_one;      // forcing / density is the identity
  int has_visc;        // viscosity is not None
  int has_forcing;     // any forcing term
  int has_lin;         // linear (drag) forcing present
  int convect;         // 0: Van Leer (TVD Lax-Wendroff), 1: linear
  const float* fu_y;   // Kolmogorov table for u over j (ny) or null
  const float* fv_x;   // swapped Kolmogorov table for v over i (nx) or null
  const float* fu_full;  // general constant forcing fields (nx*ny) or null
  const float* fv_full;
  // Pressure solve (fast diagonalisation through the real FFT).
  const float* lamx;   // eigenvalues of the 1-D Laplacian along x (nx)
  const float* lamy;   // eigenvalues along y, rfft half (ny/2 + 1)
  float cutoff;        // 10 * eps(float32)
  float pinv_scale;    // 1 / (nx * ny), folds irfftn's normalisation
  const float2* tw_y;  // exp(-2 pi i k / ny), 0 <= k < ny: real-FFT untangling
  const float2* twp_x;  // pass twiddle tables of the length-nx column FFT
  const float2* twp_y;  // pass twiddle tables of the length-ny/2 row FFT
  int fft_shape;       // transform block shape: 0 wide, 1 narrow (see fvm.cu)
  int col_mode;        // column pass: 0 per-block columns, 1/2 clusters of 4/8,
                       // 3/4 persistent register-pipelined groups of 4/2 columns,
                       // 5 as 3 with the groups staged by TMA tensor loads
  int stencil;         // explicit step: 0 shared-memory tiles, 1 warp streams,
                       // 2 (batches of small grids) whole chunks resident in shared memory
  int row_feed;        // row transforms: 0 loads through registers, 1 bulk copies
  int stream_rows;     // rows per warp of the warp-stream stencil: 0 16, 1 8, 2 32
  // Implicit diffusion (diffusion.solve_fast_diag) on the same transforms:
  int row_field;       // forward row transform of the field us itself, not div
  int col_diag;        // column-pass diagonal: 0 pinv(lambda), 1 x / (1 - x), x = dtnu lambda
  float dtnu;          // float32(dt * viscosity) for col_diag = 1
  int pdl;             // launch the step's kernels as programmatic dependents
  const void* col_tmap;  // HOST pointer to the CUtensorMap of the plan's spectrum (a batch's: 3-D, all slots)
  const void* col_tmap_spec;  // the spectrum buffer col_tmap describes (single plans)
                         // (col_mode 5), or null
};

// One slot of a same-shape batch of FVM trajectories (device-resident table
// read by the batch kernels; the member index is a grid axis).
struct FvmMember {
  FvmParams p;
  float* f[3][2];  // [0] state (u, v); [1], [2] ping-pong step buffers
  float2* spec;    // packed row spectrum / pressure q (nx * ny floats)
  int steps;       // steps of the current chunk; 0 = idle slot
  int pad_;
};

// Out-of-bounds / configuration errors are reported through return codes.
cudaError_t launch_fvm_explicit(const FvmParams& p, bool project, bool out_k0,
                                const float* ua, const float* va,
                                const float* q, float* uo, float* vo,
                                cudaStream_t s);
cudaError_t launch_fvm_div_rfft(const FvmParams& p, const float* us,
                                const float* vs, float2* spec, cudaStream_t s);
cudaError_t launch_fvm_col_pinv(const FvmParams& p, float2* spec,
                                cudaStream_t s);
// Whether the cluster column pass (col_mode 1/2) applies to this grid.
bool col_cluster_ok(const FvmParams& p, int cluster);
// Whether the persistent column pass (col_mode 3, or 4 with narrow != 0)
// applies to this grid.
bool col_pipe_ok(const FvmParams& p, int narrow);
// Whether the transform block shape (FvmParams::fft_shape) holds this grid's
// rows and, for the per-block column pass, its columns.
bool fft_shape_ok(const FvmParams& p);
// Whether the TMA-staged column pass (col_mode 5) can run on this grid (a
// tensor map of the spectrum is then needed in col_tmap).
bool col_tma_grid_ok(const FvmParams& p);
// Whether the warp-streaming stencil (stencil 1) applies to this grid.
bool stream_stencil_ok(const FvmParams& p);
// Whether the bulk-copy row transforms (row_feed 1) apply to this grid.
bool bulk_feed_ok(const FvmParams& p);
cudaError_t launch_fvm_irfft(const FvmParams& p, float2* spec, cudaStream_t s);
// Forward packed row rFFT of one field (row_field mode of the divergence
// transform, shared-memory engine).
cudaError_t launch_fvm_field_rfft(const FvmParams& p, const float* f, float2* spec,
                                  cudaStream_t s);
// u[i] += w[i] over n floats.
cudaError_t launch_fvm_add(size_t n, const float* w, float* u, cudaStream_t s);
cudaError_t launch_fvm_project_out(const FvmParams& p, const float* us,
                                   const float* vs, const float* q, float* uo,
                                   float* vo, cudaStream_t s);
// Batched launches over `count` same-shape members (`shape` carries nx, ny,
// convect and the chosen transform shapes).  Step k of a chunk reads buffer
// set 0 (k = 0) or the previous step's output and writes set 1 (k even) or 2
// (k odd); members with steps <= k skip.  project_out writes each member's
// final state back into set 0.
bool fvm_batch_shape_ok(const FvmParams& shape);
cudaError_t launch_fvm_batch_step(const FvmParams& shape, const FvmMember* members,
                                  int count, int k, cudaStream_t s);
cudaError_t launch_fvm_batch_project_out(const FvmParams& shape, const FvmMember* members,
                                         int count, cudaStream_t s);
// A whole chunk of every member (its steps, then the final projection into
// the state) in one launch, one block per member with the member's fields in
// shared memory; for grids whose fields fit (fvm_batch_resident_ok).  Same
// bits as the per-step launches.
bool fvm_batch_resident_ok(const FvmParams& shape);
cudaError_t launch_fvm_batch_resident(const FvmParams& shape, const FvmMember* members,
                                      int count, cudaStream_t s);
// Health record of one batch slot after a chunk (layout of the C ABI's
// cfd_health): flags (kHealthNonFinite: the state holds a NaN or an
// infinity) and the largest magnitude among the state's finite values.
struct Health {
  unsigned int flags;
  float max_abs;
};
constexpr unsigned int kHealthNonFinite = 1u;
// Health of every member that ran in the chunk (steps > 0), written to
// h[slot]; members that did not run keep their record.  With mirror (pinned
// host memory the device can address), the same records are stored there
// too by a kernel.
cudaError_t launch_fvm_batch_health(const FvmParams& shape, const FvmMember* members, int count,
                                    Health* h, Health* mirror, cudaStream_t s);
// Vector-Jacobian product of one FVM step at state (u, v) for the projected
// cotangent (wu, wv) = P g: (gu, gv) = w + dt (A^T w + nu lap w + lin w) and,
// if nu_dot is not null, nu_dot = w . lap(v) per cell.
// *acc += sum of x[0..n) in double, deterministically (partials: kSumBlocks
// doubles of scratch).
constexpr int kSumBlocks = 152;
cudaError_t launch_sum_to_double(const float* x, size_t n, double* partials, double* acc,
                                 cudaStream_t s);
cudaError_t launch_fvm_adjoint(const FvmParams& p, const float* u, const float* v,
                               const float* wu, const float* wv, float* gu, float* gv,
                               float* nu_dot, cudaStream_t s);
// Runge-Kutta stage combination (time_stepping.py:89-105):
// out = u0 + dt * (0 + c[0] k[0] + c[1] k[1] + ...), coefficients in float32,
// each product and sum rounded in that order, for the u and v fields.
struct RkCombine {
  const float* k[4][2];
  float c[4];
  int count;
};
cudaError_t launch_fvm_rk_combine(const FvmParams& p, const float* u0, const float* v0,
                                  const RkCombine& cb, float* uo, float* vo, cudaStream_t s);
// Diagnostics on staggered velocity fields.
cudaError_t launch_divergence(const FvmParams& p, const float* u,
                              const float* v, float* out, cudaStream_t s);
cudaError_t launch_curl2d(const FvmParams& p, const float* u, const float* v,
                          float* out, cudaStream_t s);
cudaError_t launch_max_speed(int n, const float* u, const float* v,
                             unsigned int* out_bits, cudaStream_t s);

// Pseudospectral vorticity step.
struct SpecParams {
  int nx, ny, L;        // L = ny / 2; rfft half spectrum has L + 1 columns
  int log2nx, log2ny, log2L;
  int col_mode;         // column passes: 0 per-block columns, 1 clusters of 4,
                        // 2/3 persistent register-pipelined groups of 4/2 columns
  float dn_x, dn_y;     // float32(step * n): fftfreq denominators
  float two_pi;         // float32(2 pi)
  float lap_coef;       // float32((2 pi i)^2) = -4 pi^2
  float nu, drag;       // float32 viscosity and drag
  float scale;          // 1 / (nx * ny)
  int filt_on;          // apply the 2/3 brick-wall filter
  int filt_lo, filt_hi, filt_cols;  // rows [0,lo) U [hi,nx), cols [0,cols)
  const float2* fc_full;  // forcing curl (nx x (L+1)) or null
  const float2* fc_row0;  // forcing curl only in row kx = 0 ((L+1)) or null
  const float2* tw_y;   // exp(-2 pi i k / ny): real-FFT untangling
  const float2* twp_x;  // pass twiddle tables of the length-nx column FFT
  const float2* twp_y;  // pass twiddle tables of the length-ny/2 row FFT
  const float* kx;      // fftfreq(nx, hx) in float32 (nx)
  const float* ky;      // rfftfreq(ny, hy) in float32 (L + 1)
  int pdl;              // launch the stage kernels as programmatic dependents
  int row_mode;         // row pass: 0 shared-memory engine, 1 register passes,
                        // 2 register passes with registers for 3 blocks per SM
                        //   (4 at ny = 2048)
  int pitch;            // row pitch (complex values) of the internal half spectra
                        // (the four column-transformed fields and the advection
                        // spectrum): L + 4, rows of a 32-byte multiple
  const void* stage_maps;  // HOST pointer to the plan's SpecStageMaps, or null
};

// Tensor maps (CUtensorMap: 128 bytes, 128-byte aligned) of a single
// spectral plan's advection spectrum and four column-transformed fields, as
// float32 [nx][2 pitch] with boxes of 8 floats x min(nx, 256) rows: the fused
// column stage stages its column groups by TMA loads and writes its fields by
// TMA stores where they encode.
struct alignas(128) SpecStageMaps {
  unsigned char ahat[128];
  unsigned char t[4][128];
};

// Whether the clustered spectral column passes (col_mode 1) apply to this grid.
bool spec_cluster_ok(const SpecParams& p);
// Whether the persistent spectral column passes (col_mode 2/3) apply to this grid.
bool spec_pipe_ok(const SpecParams& p);
// Whether the persistent column passes of this grid can keep the state and h
// in the column-group tiled layout (groups of 4 columns, each group's
// nx x 4 values contiguous) during a chunk; spec_tile_state converts.
bool spec_state_tiled_ok(const SpecParams& p);
size_t spec_tiled_elems(const SpecParams& p);
cudaError_t spec_tile_state(const SpecParams& p, const float2* src, float2* dst, bool to_tiled,
                            cudaStream_t s);
// Whether the fused column stage runs its TMA-staged form (the plan's maps
// encoded; groups of 4 columns of up to 2048 rows).
bool spec_stage_tma_ok(const SpecParams& p);
// Whether the register-pass row pass (row_mode 1 or 2) applies to this grid.
bool spec_row_pipe_ok(const SpecParams& p);

struct StageCoef {
  float beta;     // float32(beta_k), multiplies the previous h
  float gdt;      // float32(gamma_k * dt)
  float mu;       // float32(0.5 * dt * (alpha_{k+1} - alpha_k))
  int has_h_in;   // beta_k != 0 (the first stage adds a Python 0)
  int write_h;    // a later stage of this step reads h
  int prep_next;  // build the next stage's column-transformed fields
  int explicit_only;  // store F(u) into the state buffer instead of updating
  int tiled;      // state and h in the column-group tiled layout (spec_state_tiled_ok)
};

// One slot of a same-shape batch of spectral trajectories.
struct SpecMember {
  SpecParams p;
  StageCoef coef[8];
  int stages;      // low-storage RK/CN stages of this slot's integrator
  int steps;       // steps of the current chunk; 0 = idle slot
  float2* w;       // state: rfft of the vorticity, nx x (ny/2 + 1)
  float2* h;       // low-storage carry
  float2* t[4];    // column-transformed explicit-term inputs
  float2* ahat;    // advection row spectra
};

// Batched stage launches (slot index = last grid axis); slots with steps <= k
// skip.  A chunk is prep(k=-1) then, per step k and stage st: row(k),
// update(k, st), prep(k, st).
cudaError_t launch_spec_batch_prep(const SpecParams& shape, const SpecMember* mem, int count,
                                   int k, int stage, cudaStream_t s);
cudaError_t launch_spec_batch_row(const SpecParams& shape, const SpecMember* mem, int count,
                                  int k, cudaStream_t s);
cudaError_t launch_spec_batch_update(const SpecParams& shape, const SpecMember* mem, int count,
                                     int k, int stage, cudaStream_t s);

cudaError_t launch_spec_batch_health(const SpecParams& shape, const SpecMember* mem, int count,
                                     Health* h, Health* mirror, cudaStream_t s);

cudaError_t launch_spec_col_prep(const SpecParams& p, const float2* w,
                                 float2* const t4[4], cudaStream_t s);
cudaError_t launch_spec_row(const SpecParams& p, const float2* const t4[4],
                            float2* ahat, cudaStream_t s);
cudaError_t launch_spec_col_update(const SpecParams& p, const StageCoef& c,
                                   const float2* ahat, float2* w, float2* h,
                                   float2* const t4[4], cudaStream_t s);
// Generic 2-D real transforms on the (nx, ny) grid of a spectral plan.
cudaError_t launch_row_rfft(const SpecParams& p, const float* x, float2* X,
                            cudaStream_t s);
cudaError_t launch_row_irfft(const SpecParams& p, const float2* X, float* x,
                             float scale, cudaStream_t s);
// Column FFT over the (L+1) half-spectrum columns; sign -1 forward, +1
// inverse; an optional real table (nx x (L+1)) multiplies the result.
cudaError_t launch_col_fft(const SpecParams& p, float2* X, int sign,
                           const float* mult, cudaStream_t s);
// Diagnostics: shell sums of the kinetic-energy spectrum from the rfft half
// spectra of u and v (out: nbins doubles), and the sum of vorticity^2 / 2.
cudaError_t launch_shell_energy(const SpecParams& p, double dnx, double dny, double ks,
                                int nbins, const float2* uh, const float2* vh, double* out,
                                cudaStream_t s);
cudaError_t launch_enstrophy_sum(int nx, int ny, float hx, float hy, const float* u,
                                 const float* v, double* out, cudaStream_t s);
// curl table: 2 pi i (kx * fy_hat - ky * fx_hat)
cudaError_t launch_spec_curl_table(const SpecParams& p, const float2* fxh,
                                   const float2* fyh, float2* out,
                                   cudaStream_t s);

}  // namespace cfd
