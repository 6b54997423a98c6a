// C ABI: plans own the precomputed tables and the device workspace of one
// grid; entry points enqueue the kernels of kernels.h on the caller's stream.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "../../include/cfd_gb300.h"
#include "kernels.h"
#include "fft.cuh"
#include "wfft.cuh"

static_assert(sizeof(cfd_health) == sizeof(cfd::Health), "cfd_health layout");

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* where) {
  g_last_error = std::string(where) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? CFD_ERR_OUT_OF_MEMORY : CFD_ERR_CUDA;
}

#define CFD_CHECK(expr, where)                  \
  do {                                          \
    cudaError_t _e = (expr);                    \
    if (_e != cudaSuccess) return cuda_fail(_e, where); \
  } while (0)

bool valid_size(int n) { return n >= 4 && n <= 4096 && is_pow2(n); }

std::vector<float2> twiddles(int n) {
  std::vector<float2> t(n);
  for (int k = 0; k < n; ++k) {
    const double a = -2.0 * M_PI * (double)k / (double)n;
    t[k] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  return t;
}

// Concatenated pass twiddle tables of a length-2^log2L FFT (layout in
// fft.cuh): entry [r-1][k] of the pass with span Ns and radix R is
// exp(-2 pi i r k / (Ns R)), computed in double and rounded once.
std::vector<float2> pass_twiddles(int log2L) {
  const int stockham = cfd::fft_pass_table_size(log2L);
  std::vector<float2> t(std::max(1, stockham + cfd::wfft_table_size(log2L)));
  // The one-warp 1024-point transform's table follows the pass tables:
  // entry [k2 * 32 + n1] = exp(-2 pi i n1 k2 / 1024).
  if (cfd::wfft_table_size(log2L) > 0)
    for (int k2 = 0; k2 < 32; ++k2)
      for (int n1 = 0; n1 < 32; ++n1) {
        const double a = -2.0 * M_PI * (double)(n1 * k2) / 1024.0;
        t[cfd::wfft_table_offset(log2L) + k2 * 32 + n1] =
            make_float2((float)std::cos(a), (float)std::sin(a));
      }
  int off = 0, ns = 1;
  for (int q = 0; q < cfd::fft_num_passes(log2L); ++q) {
    const int R = cfd::fft_pass_radix(log2L, q);
    if (ns > 1) {
      for (int r = 1; r < R; ++r)
        for (int k = 0; k < ns; ++k) {
          const double a = -2.0 * M_PI * (double)r * (double)k / ((double)ns * R);
          t[off + (r - 1) * ns + k] = make_float2((float)std::cos(a), (float)std::sin(a));
        }
      off += (R - 1) * ns;
    }
    ns *= R;
  }
  return t;
}

// Eigenvalues of the periodic 1-D Laplacian circulant [-2, 1, 0..0, 1] / h^2
// (array_utils.py:168-173), i.e. fft of its first column, in double.
std::vector<float> laplacian_eigenvalues(int n, double h, int count) {
  std::vector<float> lam(count);
  for (int k = 0; k < count; ++k) {
    const double v = (k == 0) ? 0.0
                              : (2.0 * std::cos(2.0 * M_PI * (double)k / (double)n) - 2.0) /
                                    (h * h);
    lam[k] = (float)v;
  }
  return lam;
}

template <typename T>
cudaError_t upload(T** dev, const T* host, size_t count) {
  cudaError_t e = cudaMalloc((void**)dev, count * sizeof(T));
  if (e != cudaSuccess) return e;
  return cudaMemcpy(*dev, host, count * sizeof(T), cudaMemcpyHostToDevice);
}

cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Launch configurations of the FVM step (see cfd_fvm_plan_autotune).
// Index = row-transform shape + 2 * column scheme + 12 * stencil scheme
// + 24 * row feed + 48 * stream rows per warp (16, 8, 32; warp streams only).
constexpr int kLaunchChoices = 144;
bool launch_choice_ok(const cfd::FvmParams& p, int c) {
  const int col = (c >> 1) % 6, stencil = (c / 12) & 1, feed = (c / 24) & 1, rows = c / 48;
  if ((col == 1 || col == 2) && !cfd::col_cluster_ok(p, col == 1 ? 4 : 8)) return false;
  if ((col == 3 || col == 4) && !cfd::col_pipe_ok(p, col == 4)) return false;
  if (col == 5 && !(p.col_tmap && cfd::col_tma_grid_ok(p))) return false;
  if (rows != 0 && stencil != 1) return false;
  {
    cfd::FvmParams q = p;
    q.fft_shape = c & 1;
    q.col_mode = col;
    if (!cfd::fft_shape_ok(q)) return false;
  }
  if (stencil == 1) {
    cfd::FvmParams q = p;
    q.stream_rows = rows;
    if (!cfd::stream_stencil_ok(q)) return false;
  }
  if (feed == 1 && !cfd::bulk_feed_ok(p)) return false;
  return true;
}
void set_launch_choice(cfd::FvmParams* p, int c) {
  p->fft_shape = c & 1;
  p->col_mode = (c >> 1) % 6;
  p->stencil = (c / 12) & 1;
  p->row_feed = (c / 24) & 1;
  p->stream_rows = c / 48;
}

// Captures `enqueue` (run on a private capture stream) into an executable graph.
template <typename F>
int capture_graph(F enqueue, cudaGraph_t* graph, cudaGraphExec_t* exec) {
  cudaStream_t cap;
  CFD_CHECK(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking), "cudaStreamCreate");
  cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeRelaxed);
  int rc = e == cudaSuccess ? enqueue(cap) : CFD_OK;
  cudaGraph_t g = nullptr;
  cudaError_t e2 = e == cudaSuccess ? cudaStreamEndCapture(cap, &g) : cudaSuccess;
  cudaStreamDestroy(cap);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamBeginCapture");
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture");
  cudaGraphExec_t x = nullptr;
  e = cudaGraphInstantiate(&x, g, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    return cuda_fail(e, "cudaGraphInstantiate");
  }
  *graph = g;
  *exec = x;
  return CFD_OK;
}


}  // namespace

namespace cfd {
void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace cfd

struct cfd_fvm_plan {
  cfd::FvmParams p;
  float* au = nullptr;
  float* av = nullptr;
  float* bu = nullptr;
  float* bv = nullptr;
  float2* spec = nullptr;  // packed row spectrum / pressure q (nx * ny floats)
  float* lamx = nullptr;
  float* lamy = nullptr;
  float2* twy = nullptr;
  float2* twpx = nullptr;
  float2* twpy = nullptr;
  float* fu = nullptr;
  float* fv = nullptr;
  float* rk = nullptr;  // Runge-Kutta stage terms k_j (u, v), allocated on first use
  double* partials = nullptr;  // cfd::kSumBlocks doubles for the viscosity sums
  double dt = 0;        // the configuration's dt (double, as the reference's Python float)
  long long bytes = 0;
  // Tensor map of the packed spectrum for the TMA-staged column pass (the
  // type's own alignment; plans come from C++17 aligned new).
  CUtensorMap spec_map;
};

// A batch of same-shape FVM trajectories ("slots"): one device table of
// cfd::FvmMember entries read by the batched kernels, one slab of per-slot
// buffers, and the grid tables shared by every slot.
struct cfd_fvm_batch {
  cfd::FvmParams shape;  // grid, convection and launch choices of the batch
  double hx = 0, hy = 0;
  int count = 0;
  size_t n = 0;
  float* slab = nullptr;   // per slot: u, v, au, av, bu, bv, spec (7 n floats)
  float* force = nullptr;  // per slot: u-forcing over y (ny) then v-forcing over x (nx)
  float* lamx = nullptr;
  float* lamy = nullptr;
  float2* twy = nullptr;
  float2* twpx = nullptr;
  float2* twpy = nullptr;
  std::vector<cfd::FvmMember> host;
  std::vector<int> want;   // requested steps per slot
  cfd::FvmMember* dev = nullptr;
  int uploaded_chunk = -1;  // chunk length the device table was clamped to
  bool dirty = true;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int graph_chunk = -1;
  long long bytes = 0;
  // 3-D tensor map of every slot's spectrum for the TMA-staged column pass.
  CUtensorMap spec_map;
  cfd::Health* health = nullptr;  // per slot, written at the end of every chunk
  cfd::Health* mirror = nullptr;  // pinned host copy of `health`, or null
};

// Several batches (one per grid shape) stepped together: a chunk forks one
// stream per batch so the batches' kernels overlap, and can be captured as
// one CUDA graph.
struct cfd_fvm_ensemble {
  std::vector<cfd_fvm_batch*> batches;
  std::vector<std::pair<int, int>> where;  // member -> (batch, slot)
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> joins;
  cudaEvent_t fork = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int graph_steps = -1;
};

// A batch of same-shape spectral trajectories (slots), like cfd_fvm_batch:
// one device table of cfd::SpecMember entries, one slab of per-slot buffers
// (w, h, four column fields, advection spectra: 7 half spectra per slot) and
// the grid tables shared by every slot.
struct cfd_spec_batch {
  cfd::SpecParams shape;
  double hx = 0, hy = 0;
  int stages = 0;
  int count = 0;
  size_t ns = 0;  // complex entries of one half spectrum
  float2* slab = nullptr;
  float2* twy = nullptr;
  float2* twpx = nullptr;
  float2* twpy = nullptr;
  float* kx = nullptr;
  float* ky = nullptr;
  std::vector<cfd::SpecMember> host;
  std::vector<int> want;
  cfd::SpecMember* dev = nullptr;
  int uploaded_chunk = -1;
  bool dirty = true;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int graph_chunk = -1;
  long long bytes = 0;
  cfd::Health* health = nullptr;  // per slot, written at the end of every chunk
  cfd::Health* mirror = nullptr;  // pinned host copy of `health`, or null
};

static_assert(sizeof(CUtensorMap) == 128 && alignof(CUtensorMap) <= 128,
              "SpecStageMaps holds CUtensorMaps as 128-byte blocks");

struct cfd_spec_plan {
  cfd::SpecParams p;
  int stages = 0;
  cfd::StageCoef coef[8];
  float2* t4[4] = {nullptr, nullptr, nullptr, nullptr};
  float2* ahat = nullptr;
  float2* h = nullptr;
  float2* fc = nullptr;     // forcing curl table (full or row 0)
  float2* work = nullptr;   // scratch spectrum for rfft2 / irfft2 / filter
  float2* wt = nullptr;     // state and h in the column-group tiled layout during a
  float2* ht = nullptr;     // chunk of the fused column stage (cfd::spec_state_tiled_ok)
  cfd::SpecStageMaps maps;  // TMA maps of ahat and t4 (p.stage_maps when they encode)
  float2* twy = nullptr;
  float2* twpx = nullptr;
  float2* twpy = nullptr;
  float* kx = nullptr;
  float* ky = nullptr;
  long long bytes = 0;
};

extern "C" {

const char* cfd_last_error(void) { return g_last_error.c_str(); }

int cfd_device_fault(unsigned int* code, int clear) {
  if (!code) return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_device_fault: null pointer");
  CFD_CHECK(cfd::read_device_fault(code, clear != 0), "cfd_device_fault");
  return CFD_OK;
}

int cfd_version(void) { return 1; }

int cfd_fvm_plan_destroy(cfd_fvm_plan* plan) {
  if (!plan) return CFD_OK;
  void* ptrs[] = {plan->au, plan->av, plan->bu, plan->bv, plan->spec, plan->lamx,
                  plan->lamy, plan->twy, plan->twpx, plan->twpy, plan->fu, plan->fv,
                  plan->rk, plan->partials};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  delete plan;
  return CFD_OK;
}

// Scalar step parameters of one configuration (no device tables); shared by
// plans and batch slots.
static int fvm_params_from_config(const cfd_fvm_config* cfg, cfd::FvmParams* out) {
  if (!valid_size(cfg->nx) || !valid_size(cfg->ny))
    return fail(CFD_ERR_UNSUPPORTED,
                "grid shape must be powers of two in [4, 4096] (real-FFT pressure solve)");
  if (!(cfg->hx > 0) || !(cfg->hy > 0) || !(cfg->density != 0) || !std::isfinite(cfg->dt))
    return fail(CFD_ERR_INVALID_ARGUMENT, "invalid step, density or dt");
  if (cfg->convect != CFD_CONVECT_VAN_LEER && cfg->convect != CFD_CONVECT_LINEAR)
    return fail(CFD_ERR_UNSUPPORTED, "unsupported convection scheme");
  if (cfg->const_forcing < CFD_FORCE_NONE || cfg->const_forcing > CFD_FORCE_FULL)
    return fail(CFD_ERR_UNSUPPORTED, "unsupported forcing layout");
  if (cfg->const_forcing != CFD_FORCE_NONE && !cfg->force_u && !cfg->force_v)
    return fail(CFD_ERR_INVALID_ARGUMENT, "forcing layout given without tables");
  cfd::FvmParams& p = *out;
  std::memset(&p, 0, sizeof(p));
  const int nx = cfg->nx, ny = cfg->ny;
  p.nx = nx;
  p.ny = ny;
  p.log2nx = ilog2(nx);
  p.log2ny = ilog2(ny);
  // Python floats are rounded once to float32 where the reference's weakly
  // typed scalars meet float32 arrays.
  p.hx = (float)cfg->hx;
  p.hy = (float)cfg->hy;
  p.inv_hx = 1.f / p.hx;
  p.inv_hy = 1.f / p.hy;
  p.cfl_x = (float)(cfg->dt / cfg->hx);
  p.cfl_y = (float)(cfg->dt / cfg->hy);
  p.dt = (float)cfg->dt;
  p.has_visc = cfg->has_viscosity ? 1 : 0;
  p.nu = cfg->has_viscosity ? (float)(cfg->viscosity / cfg->density) : 0.f;
  // finite_differences.laplacian: scales = (1 / float32(step))^2 in float32.
  const float ihx = 1.f / p.hx, ihy = 1.f / p.hy;
  p.sx = ihx * ihx;
  p.sy = ihy * ihy;
  p.ssum = p.sx + p.sy;
  p.density = (float)cfg->density;
  p.rho_is_one = cfg->density == 1.0 ? 1 : 0;
  p.has_lin = cfg->has_linear_forcing ? 1 : 0;
  p.lin = (float)cfg->linear_coefficient;
  p.has_forcing = (p.has_lin || cfg->const_forcing != CFD_FORCE_NONE) ? 1 : 0;
  p.convect = cfg->convect;
  p.cutoff = 10.f * 1.1920928955078125e-07f;  // 10 * finfo(float32).eps
  p.pinv_scale = 1.f / ((float)nx * (float)ny);
  // Narrow transform blocks keep large grids resident in one wave; the
  // autotuner can revise the choice on the device.
  p.fft_shape = (nx >= 1024 && ny >= 1024) ? 1 : 0;
  // The warp-streaming stencil needs enough warps to fill the GPU.
  p.stencil = ((long long)nx * ny >= (1LL << 22) && cfd::stream_stencil_ok(p)) ? 1 : 0;
  // The persistent column pass measured fastest from 1024 rows up (GB300).
  p.col_mode = (nx >= 1024 && cfd::col_pipe_ok(p, 0)) ? 3 : 0;
  if (!cfd::fft_shape_ok(p)) p.fft_shape = 0;
  // The step's kernels start as programmatic dependents of their predecessor
  // (CFD_GB300_PDL=0 in the environment turns this off, for comparison).
  const char* pdl = std::getenv("CFD_GB300_PDL");
  p.pdl = (pdl && pdl[0] == '0') ? 0 : 1;
  return CFD_OK;
}

// Tensor map of `count` packed row spectra, each nx rows of ny float32 (2
// floats per complex value), spectrum z at spec + z * member_floats floats;
// boxes of 8 floats x min(nx, 256) rows x 1 spectrum.
// The CUDA driver's cuTensorMapEncodeTiled, looked up once (a function-local
// static: thread-safe initialisation); null where the lookup fails.
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static const PFN_cuTensorMapEncodeTiled_v12000 encode = []() {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      fn = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }();
  return encode;
}

// 2-D map of float32 rows [rows][width] (width * 4 bytes a multiple of 16)
// with boxes of 8 floats x min(rows, 256) rows.
static bool encode_rows_map(void* map, const void* base, int width, int rows) {
  const PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
  if (!encode || ((size_t)width * sizeof(float)) % 16 != 0) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)width, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)width * sizeof(float)};
  const cuuint32_t box[2] = {8, (cuuint32_t)(rows < 256 ? rows : 256)};
  const cuuint32_t estride[2] = {1, 1};
  return encode(static_cast<CUtensorMap*>(map), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                const_cast<void*>(base), dims, strides, box, estride,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
         CUDA_SUCCESS;
}

static bool encode_spec_map(CUtensorMap* map, float2* spec, int nx, int ny, int count = 1,
                            size_t member_floats = 0) {
  const PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
  if (!encode) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)ny, (cuuint64_t)nx, (cuuint64_t)count};
  const cuuint64_t strides[2] = {(cuuint64_t)ny * sizeof(float),
                                 (cuuint64_t)member_floats * sizeof(float)};
  const cuuint32_t box[3] = {8, (cuuint32_t)(nx < 256 ? nx : 256), 1};
  const cuuint32_t estride[3] = {1, 1, 1};
  if (count > 1 && (member_floats * sizeof(float)) % 16 != 0) return false;
  return encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, count > 1 ? 3 : 2, spec, dims, strides,
                box, estride,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
         CUDA_SUCCESS;
}

// Default launch of a single plan from 128^2 up, from a sweep of every
// configuration of the step at 128^2 .. 2048^2 on GB300 (the default is the
// fastest there or within 3 % of it; the autotuner can still revise it):
// narrow row blocks, rows fed by bulk copies where they fit, the persistent
// column pass from 256 rows (TMA-staged from 1024, where the map encodes),
// warp streams with 8 rows per warp up to 2^22 cells and 16 above.  Per
// step: 128^2 31.2 against 40.4 us for the earlier default (tiles, per-block
// columns, register feed), 256^2 23.0 against 39.4, 512^2 25.0 against
// 44.4, 1024^2 33.2 against 38.8; 2048^2 63.7 (8 rows per warp) against
// 64.6 (16).
static void plan_default_launch(cfd::FvmParams* p) {
  if ((long long)p->nx * p->ny < (1LL << 14)) return;
  p->fft_shape = 1;
  p->row_feed = cfd::bulk_feed_ok(*p) ? 1 : 0;
  if (p->nx >= 256 && cfd::col_pipe_ok(*p, 0)) p->col_mode = 3;
  if (!cfd::fft_shape_ok(*p)) p->fft_shape = 0;
  cfd::FvmParams q = *p;
  q.stream_rows = (long long)p->nx * p->ny <= (1LL << 22) ? 1 : 0;
  if (cfd::stream_stencil_ok(q)) {
    p->stencil = 1;
    p->stream_rows = q.stream_rows;
  }
}

int cfd_fvm_plan_create(const cfd_fvm_config* cfg, cfd_fvm_plan** out) {
  if (!cfg || !out) return fail(CFD_ERR_INVALID_ARGUMENT, "null config or output pointer");
  *out = nullptr;
  cfd::FvmParams params;
  int rc = fvm_params_from_config(cfg, &params);
  if (rc) return rc;
  plan_default_launch(&params);
  cfd_fvm_plan* plan = new cfd_fvm_plan();
  cfd::FvmParams& p = plan->p;
  p = params;
  plan->dt = cfg->dt;
  const int nx = cfg->nx, ny = cfg->ny;

  const size_t n = (size_t)nx * ny;
  cudaError_t e;
  long long bytes = 0;
#define CFD_ALLOC(ptr, count)                                              \
  do {                                                                     \
    e = cudaMalloc((void**)&(ptr), (count) * sizeof(*(ptr)));              \
    if (e != cudaSuccess) {                                                \
      cfd_fvm_plan_destroy(plan);                                          \
      return cuda_fail(e, "cfd_fvm_plan_create: cudaMalloc");              \
    }                                                                      \
    bytes += (long long)((count) * sizeof(*(ptr)));                        \
  } while (0)
  CFD_ALLOC(plan->au, n);
  CFD_ALLOC(plan->av, n);
  CFD_ALLOC(plan->bu, n);
  CFD_ALLOC(plan->bv, n);
  CFD_ALLOC(plan->spec, n / 2);
#undef CFD_ALLOC

  std::vector<float> lamx = laplacian_eigenvalues(nx, cfg->hx, nx);
  std::vector<float> lamy = laplacian_eigenvalues(ny, cfg->hy, ny / 2 + 1);
  std::vector<float2> twy = twiddles(ny);
  std::vector<float2> twpx = pass_twiddles(p.log2nx), twpy = pass_twiddles(p.log2ny - 1);
  if ((e = upload(&plan->lamx, lamx.data(), lamx.size())) != cudaSuccess ||
      (e = upload(&plan->lamy, lamy.data(), lamy.size())) != cudaSuccess ||
      (e = upload(&plan->twy, twy.data(), twy.size())) != cudaSuccess ||
      (e = upload(&plan->twpx, twpx.data(), twpx.size())) != cudaSuccess ||
      (e = upload(&plan->twpy, twpy.data(), twpy.size())) != cudaSuccess) {
    cfd_fvm_plan_destroy(plan);
    return cuda_fail(e, "cfd_fvm_plan_create: tables");
  }
  bytes += (long long)(lamx.size() + lamy.size()) * 4 +
           (long long)(twy.size() + twpx.size() + twpy.size()) * 8;
  p.lamx = plan->lamx;
  p.lamy = plan->lamy;
  p.tw_y = plan->twy;
  p.twp_x = plan->twpx;
  p.twp_y = plan->twpy;

  if (cfg->const_forcing != CFD_FORCE_NONE) {
    size_t cu = 0, cv = 0;
    if (cfg->const_forcing == CFD_FORCE_U_OF_Y) cu = ny;
    if (cfg->const_forcing == CFD_FORCE_V_OF_X) cv = nx;
    if (cfg->const_forcing == CFD_FORCE_FULL) cu = cv = n;
    if (cu && cfg->force_u) {
      if ((e = upload(&plan->fu, cfg->force_u, cu)) != cudaSuccess) {
        cfd_fvm_plan_destroy(plan);
        return cuda_fail(e, "cfd_fvm_plan_create: forcing");
      }
      bytes += (long long)cu * 4;
    }
    if (cv && cfg->force_v) {
      if ((e = upload(&plan->fv, cfg->force_v, cv)) != cudaSuccess) {
        cfd_fvm_plan_destroy(plan);
        return cuda_fail(e, "cfd_fvm_plan_create: forcing");
      }
      bytes += (long long)cv * 4;
    }
    if (cfg->const_forcing == CFD_FORCE_U_OF_Y) p.fu_y = plan->fu;
    if (cfg->const_forcing == CFD_FORCE_V_OF_X) p.fv_x = plan->fv;
    if (cfg->const_forcing == CFD_FORCE_FULL) {
      p.fu_full = plan->fu;
      p.fv_full = plan->fv;
    }
  }
  plan->bytes = bytes;
  // The TMA-staged column pass is a launch choice where the map encodes,
  // and replaces the cp.async-staged default from 1024 rows (3% faster on
  // 2048^2, even at 1024^2, 6% slower at 512^2).
  if (cfd::col_tma_grid_ok(p) && encode_spec_map(&plan->spec_map, plan->spec, nx, ny)) {
    p.col_tmap = &plan->spec_map;
    p.col_tmap_spec = plan->spec;
    if (p.col_mode == 3 && nx >= 1024) p.col_mode = 5;
  }
  *out = plan;
  return CFD_OK;
}

long long cfd_fvm_plan_bytes(const cfd_fvm_plan* plan) { return plan ? plan->bytes : 0; }

static int fvm_pressure(cfd_fvm_plan* plan, cudaStream_t s, const float* us,
                        const float* vs) {
  CFD_CHECK(cfd::launch_fvm_div_rfft(plan->p, us, vs, plan->spec, s), "div_rfft");
  CFD_CHECK(cfd::launch_fvm_col_pinv(plan->p, plan->spec, s), "col_pinv");
  CFD_CHECK(cfd::launch_fvm_irfft(plan->p, plan->spec, s), "irfft");
  return CFD_OK;
}

// One explicit step (u, v [projected with q]) -> (uo, vo) followed by the
// pressure solve of (uo, vo), leaving q in the plan's spectrum.  (Writing the
// divergence from the warp-stream stencil for the row transform to read
// measured slower at 2048^2: 68.7 against 66.2 us per step.)
static int fvm_step_once(cfd_fvm_plan* plan, cudaStream_t s, bool project, const float* u,
                         const float* v, const float* q, float* uo, float* vo) {
  CFD_CHECK(cfd::launch_fvm_explicit(plan->p, project, false, u, v, q, uo, vo, s), "explicit");
  return fvm_pressure(plan, s, uo, vo);
}

int cfd_fvm_step(cfd_fvm_plan* plan, void* stream, const float* u,
                 const float* v, float* u_out, float* v_out, int steps) {
  if (!plan || !u || !v || !u_out || !v_out)
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_step: null pointer");
  if (steps < 0) return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_step: steps < 0");
  cudaStream_t s = as_stream(stream);
  const cfd::FvmParams& p = plan->p;
  const size_t bytes = (size_t)p.nx * p.ny * sizeof(float);
  if (steps == 0) {
    if (u_out != u) CFD_CHECK(cudaMemcpyAsync(u_out, u, bytes, cudaMemcpyDeviceToDevice, s), "copy");
    if (v_out != v) CFD_CHECK(cudaMemcpyAsync(v_out, v, bytes, cudaMemcpyDeviceToDevice, s), "copy");
    return CFD_OK;
  }
  float *au = plan->au, *av = plan->av, *bu = plan->bu, *bv = plan->bv;
  const float* q = reinterpret_cast<const float*>(plan->spec);
  int rc = fvm_step_once(plan, s, false, u, v, nullptr, au, av);
  if (rc) return rc;
  for (int k = 1; k < steps; ++k) {
    rc = fvm_step_once(plan, s, true, au, av, q, bu, bv);
    if (rc) return rc;
    float* t = au; au = bu; bu = t;
    t = av; av = bv; bv = t;
  }
  CFD_CHECK(cfd::launch_fvm_project_out(p, au, av, q, u_out, v_out, s), "project_out");
  return CFD_OK;
}

// funcutils.trajectory(repeated(step, inner), frames, post_process)
// (funcutils.py:95-126) in one call: each chunk of `inner` steps runs in place
// in (u_out, v_out) and its frame is written into frames_out on the device.
int cfd_fvm_trajectory(cfd_fvm_plan* plan, void* stream, const float* u, const float* v,
                       int inner, int frames, int frame_kind, int start_with_input,
                       float* frames_out, float* u_out, float* v_out) {
  if (!plan || !u || !v || !u_out || !v_out || (frames > 0 && !frames_out))
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_trajectory: null pointer");
  if (inner < 0 || frames < 0)
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_trajectory: negative step or frame count");
  if (frame_kind != CFD_FRAME_VELOCITY && frame_kind != CFD_FRAME_VORTICITY)
    return fail(CFD_ERR_UNSUPPORTED, "cfd_fvm_trajectory: unknown frame kind");
  cudaStream_t s = as_stream(stream);
  const cfd::FvmParams& p = plan->p;
  const size_t n = (size_t)p.nx * p.ny;
  const size_t per_frame = frame_kind == CFD_FRAME_VELOCITY ? 2 * n : n;
  auto write_frame = [&](int k, const float* fu, const float* fv) -> int {
    float* dst = frames_out + (size_t)k * per_frame;
    if (frame_kind == CFD_FRAME_VELOCITY) {
      CFD_CHECK(cudaMemcpyAsync(dst, fu, n * sizeof(float), cudaMemcpyDeviceToDevice, s), "frame");
      CFD_CHECK(cudaMemcpyAsync(dst + n, fv, n * sizeof(float), cudaMemcpyDeviceToDevice, s),
                "frame");
    } else {
      CFD_CHECK(cfd::launch_curl2d(p, fu, fv, dst, s), "frame curl_2d");
    }
    return CFD_OK;
  };
  const float *cu = u, *cv = v;
  for (int k = 0; k < frames; ++k) {
    int rc;
    if (start_with_input && (rc = write_frame(k, cu, cv))) return rc;
    if ((rc = cfd_fvm_step(plan, stream, cu, cv, u_out, v_out, inner))) return rc;
    cu = u_out;
    cv = v_out;
    if (!start_with_input && (rc = write_frame(k, u_out, v_out))) return rc;
  }
  if (frames == 0) return cfd_fvm_step(plan, stream, u, v, u_out, v_out, 0);
  return CFD_OK;
}

// diffusion.solve_fast_diag (diffusion.py:166-212) on periodic fields, in
// place on (u, v): u + irfftn(func(lambda) rfftn(u)) per component, func(x) =
// (dt nu) x / (1 - (dt nu) x) on the summed eigenvalues of the periodic 1-D
// Laplacians (the same circulant for both staggered offsets).  Uses the
// plan's spectrum buffer and column-pass scheme.
static int fvm_diffuse_implicit(cfd_fvm_plan* plan, cudaStream_t s, float* u, float* v,
                                double nu, double dt) {
  cfd::FvmParams pd = plan->p;
  pd.col_diag = 1;
  pd.dtnu = (float)(dt * nu);
  const size_t n = (size_t)pd.nx * pd.ny;
  const float* w = reinterpret_cast<const float*>(plan->spec);
  for (float* c : {u, v}) {
    CFD_CHECK(cfd::launch_fvm_field_rfft(pd, c, plan->spec, s), "field_rfft");
    CFD_CHECK(cfd::launch_fvm_col_pinv(pd, plan->spec, s), "col_diffuse");
    CFD_CHECK(cfd::launch_fvm_irfft(pd, plan->spec, s), "irfft");
    CFD_CHECK(cfd::launch_fvm_add(n, w, c, s), "add");
  }
  return CFD_OK;
}

int cfd_fvm_diffusion_solve(cfd_fvm_plan* plan, void* stream, const float* u, const float* v,
                            float* u_out, float* v_out, double nu, double dt) {
  if (!plan || !u || !v || !u_out || !v_out)
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_diffusion_solve: null pointer");
  cudaStream_t s = as_stream(stream);
  const size_t bytes = (size_t)plan->p.nx * plan->p.ny * sizeof(float);
  if (u_out != u) CFD_CHECK(cudaMemcpyAsync(u_out, u, bytes, cudaMemcpyDeviceToDevice, s), "copy");
  if (v_out != v) CFD_CHECK(cudaMemcpyAsync(v_out, v, bytes, cudaMemcpyDeviceToDevice, s), "copy");
  return fvm_diffuse_implicit(plan, s, u_out, v_out, nu, dt);
}

// implicit_diffusion_navier_stokes (equations.py:154-195) with
// diffusion_solve = pressure_solve = solve_fast_diag: u* = u + dt (convection
// + forcing / density) (the stencil without its viscosity term), projection,
// then the implicit diffusion solve with the plan's dt.  The plan must be
// made without explicit viscosity.
int cfd_fvm_step_implicit(cfd_fvm_plan* plan, void* stream, const float* u, const float* v,
                          float* u_out, float* v_out, int steps, double viscosity) {
  if (!plan || !u || !v || !u_out || !v_out || steps < 0)
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_step_implicit: bad arguments");
  const cfd::FvmParams& p = plan->p;
  if (p.has_visc)
    return fail(CFD_ERR_UNSUPPORTED,
                "cfd_fvm_step_implicit: the plan's explicit terms must not include viscosity");
  cudaStream_t s = as_stream(stream);
  const size_t bytes = (size_t)p.nx * p.ny * sizeof(float);
  if (steps == 0) {
    if (u_out != u) CFD_CHECK(cudaMemcpyAsync(u_out, u, bytes, cudaMemcpyDeviceToDevice, s), "copy");
    if (v_out != v) CFD_CHECK(cudaMemcpyAsync(v_out, v, bytes, cudaMemcpyDeviceToDevice, s), "copy");
    return CFD_OK;
  }
  const float* q = reinterpret_cast<const float*>(plan->spec);
  const float *cu = u, *cv = v;
  for (int k = 0; k < steps; ++k) {
    CFD_CHECK(cfd::launch_fvm_explicit(p, false, false, cu, cv, nullptr, plan->au, plan->av, s),
              "explicit");
    int rc = fvm_pressure(plan, s, plan->au, plan->av);
    if (rc) return rc;
    CFD_CHECK(cfd::launch_fvm_project_out(p, plan->au, plan->av, q, u_out, v_out, s),
              "project_out");
    rc = fvm_diffuse_implicit(plan, s, u_out, v_out, viscosity, plan->dt);
    if (rc) return rc;
    cu = u_out;
    cv = v_out;
  }
  return CFD_OK;
}

// navier_stokes_rk (time_stepping.py:59-107) with an arbitrary explicit
// tableau of up to four stages: k_0 = F(u0); u_i = P(u0 + dt sum_j a_ij k_j),
// k_i = F(u_i); u' = P(u0 + dt sum_j b_j k_j).  F is the stencil in
// explicit-terms mode (with the projection of u_i folded into its load), P the
// fast-diagonalisation projection.
int cfd_fvm_step_rk(cfd_fvm_plan* plan, void* stream, const float* u, const float* v,
                    float* u_out, float* v_out, int steps, int stages, const double* a,
                    const double* b) {
  if (!plan || !u || !v || !u_out || !v_out || !b || steps < 0 || stages < 1 || stages > 4 ||
      (stages > 1 && !a))
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_step_rk: bad arguments");
  cudaStream_t s = as_stream(stream);
  const cfd::FvmParams& p = plan->p;
  const size_t n = (size_t)p.nx * p.ny;
  if (steps == 0) {
    if (u_out != u) CFD_CHECK(cudaMemcpyAsync(u_out, u, n * 4, cudaMemcpyDeviceToDevice, s), "copy");
    if (v_out != v) CFD_CHECK(cudaMemcpyAsync(v_out, v, n * 4, cudaMemcpyDeviceToDevice, s), "copy");
    return CFD_OK;
  }
  if (!plan->rk) {
    CFD_CHECK(cudaMalloc((void**)&plan->rk, 8 * n * sizeof(float)), "cfd_fvm_step_rk: cudaMalloc");
    plan->bytes += (long long)(8 * n * sizeof(float));
  }
  float* K[4][2];
  for (int j = 0; j < 4; ++j) {
    K[j][0] = plan->rk + (size_t)(2 * j) * n;
    K[j][1] = plan->rk + (size_t)(2 * j + 1) * n;
  }
  const float* q = reinterpret_cast<const float*>(plan->spec);
  // Python coefficient rows (skipping zeros as the reference's sum does).
  auto combo = [&](const double* coef, int count) {
    cfd::RkCombine cb{};
    for (int j = 0; j < count; ++j)
      if (coef[j] != 0.0) {
        cb.k[cb.count][0] = K[j][0];
        cb.k[cb.count][1] = K[j][1];
        cb.c[cb.count] = (float)coef[j];
        ++cb.count;
      }
    return cb;
  };
  const float *cu = u, *cv = v;
  for (int st = 0; st < steps; ++st) {
    float* ou = (st + 1 == steps) ? u_out : plan->bu;
    float* ov = (st + 1 == steps) ? v_out : plan->bv;
    CFD_CHECK(cfd::launch_fvm_explicit(p, false, true, cu, cv, nullptr, K[0][0], K[0][1], s),
              "explicit");
    const double* row = a;
    for (int i = 1; i < stages; ++i) {
      CFD_CHECK(cfd::launch_fvm_rk_combine(p, cu, cv, combo(row, i), plan->au, plan->av, s),
                "rk_combine");
      row += i;
      int rc = fvm_pressure(plan, s, plan->au, plan->av);
      if (rc) return rc;
      CFD_CHECK(cfd::launch_fvm_explicit(p, true, true, plan->au, plan->av, q, K[i][0], K[i][1], s),
                "explicit");
    }
    CFD_CHECK(cfd::launch_fvm_rk_combine(p, cu, cv, combo(b, stages), plan->au, plan->av, s),
              "rk_combine");
    int rc = fvm_pressure(plan, s, plan->au, plan->av);
    if (rc) return rc;
    CFD_CHECK(cfd::launch_fvm_project_out(p, plan->au, plan->av, q, ou, ov, s), "project_out");
    cu = ou;
    cv = ov;
  }
  return CFD_OK;
}

// Same launches as cfd_fvm_step, with an event pair recorded around every
// launch on `stream`; synchronises once at the end and writes the mean
// duration (ms) of each kernel kind to ms_out[CFD_FVM_PROFILE_KINDS].
int cfd_fvm_profile(cfd_fvm_plan* plan, void* stream, const float* u,
                    const float* v, float* u_out, float* v_out, int steps,
                    float* ms_out) {
  if (!plan || !u || !v || !u_out || !v_out || !ms_out || steps < 1)
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_profile: bad arguments");
  cudaStream_t s = as_stream(stream);
  const cfd::FvmParams& p = plan->p;
  const int launches = 4 * steps + 1;
  std::vector<cudaEvent_t> ev(2 * launches);
  std::vector<int> kind(launches);
  for (auto& e : ev) CFD_CHECK(cudaEventCreate(&e), "cudaEventCreate");
  int li = 0;
  auto timed = [&](int k, cudaError_t (*fn)(void*), void* ctx) -> cudaError_t {
    cudaError_t e = cudaEventRecord(ev[2 * li], s);
    if (e == cudaSuccess) e = fn(ctx);
    if (e == cudaSuccess) e = cudaEventRecord(ev[2 * li + 1], s);
    kind[li++] = k;
    return e;
  };
  struct Ctx {
    const cfd::FvmParams* p;
    const float *a, *b, *q;
    float *c, *d;
    float2* spec;
    bool project;
    cudaStream_t s;
  } ctx{&p, u, v, nullptr, plan->au, plan->av, plan->spec, false, s};
  auto explicit_fn = [](void* c) -> cudaError_t {
    Ctx* x = (Ctx*)c;
    return cfd::launch_fvm_explicit(*x->p, x->project, false, x->a, x->b, x->q, x->c, x->d, x->s);
  };
  auto div_fn = [](void* c) -> cudaError_t {
    Ctx* x = (Ctx*)c;
    return cfd::launch_fvm_div_rfft(*x->p, x->c, x->d, x->spec, x->s);
  };
  auto col_fn = [](void* c) -> cudaError_t {
    Ctx* x = (Ctx*)c;
    return cfd::launch_fvm_col_pinv(*x->p, x->spec, x->s);
  };
  auto irfft_fn = [](void* c) -> cudaError_t {
    Ctx* x = (Ctx*)c;
    return cfd::launch_fvm_irfft(*x->p, x->spec, x->s);
  };
  auto out_fn = [](void* c) -> cudaError_t {
    Ctx* x = (Ctx*)c;
    return cfd::launch_fvm_project_out(*x->p, x->a, x->b, x->q, x->c, x->d, x->s);
  };
  cudaError_t e = cudaSuccess;
  float *au = plan->au, *av = plan->av, *bu = plan->bu, *bv = plan->bv;
  const float* q = reinterpret_cast<const float*>(plan->spec);
  for (int k = 0; k < steps && e == cudaSuccess; ++k) {
    ctx.project = k > 0;
    ctx.a = k > 0 ? au : u;
    ctx.b = k > 0 ? av : v;
    ctx.q = q;
    ctx.c = k > 0 ? bu : au;
    ctx.d = k > 0 ? bv : av;
    e = timed(0, explicit_fn, &ctx);
    if (e == cudaSuccess) e = timed(1, div_fn, &ctx);
    if (e == cudaSuccess) e = timed(2, col_fn, &ctx);
    if (e == cudaSuccess) e = timed(3, irfft_fn, &ctx);
    if (k > 0) {
      float* t = au; au = bu; bu = t;
      t = av; av = bv; bv = t;
    }
  }
  if (e == cudaSuccess) {
    ctx.a = au; ctx.b = av; ctx.q = q; ctx.c = u_out; ctx.d = v_out;
    e = timed(4, out_fn, &ctx);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  double sum[5] = {0, 0, 0, 0, 0};
  int cnt[5] = {0, 0, 0, 0, 0};
  for (int i = 0; i < li && e == cudaSuccess; ++i) {
    float ms = 0.f;
    e = cudaEventElapsedTime(&ms, ev[2 * i], ev[2 * i + 1]);
    sum[kind[i]] += ms;
    cnt[kind[i]] += 1;
  }
  for (auto& x : ev) cudaEventDestroy(x);
  if (e != cudaSuccess) return cuda_fail(e, "cfd_fvm_profile");
  for (int k = 0; k < 5; ++k) ms_out[k] = cnt[k] ? (float)(sum[k] / cnt[k]) : 0.f;
  return CFD_OK;
}

// Autotuner over the transform block shapes (FvmParams::fft_shape): runs
// `steps` steps per candidate after one warm-up step, times them with CUDA
// events on `stream` (synchronising), and keeps the fastest in the plan.
int cfd_fvm_plan_autotune(cfd_fvm_plan* plan, void* stream, const float* u,
                          const float* v, float* u_scratch, float* v_scratch,
                          int steps, int* chosen) {
  if (!plan || !u || !v || !u_scratch || !v_scratch || steps < 1)
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_plan_autotune: bad arguments");
  cudaStream_t s = as_stream(stream);
  cudaEvent_t e0, e1;
  CFD_CHECK(cudaEventCreate(&e0), "cudaEventCreate");
  CFD_CHECK(cudaEventCreate(&e1), "cudaEventCreate");
  float best_ms = 0.f;
  int best = -1;
  int rc = CFD_OK;
  // Candidates: transform block shape (wide, narrow) x column pass (per-block
  // columns, clusters of 4, clusters of 8, persistent pipelined groups of 4
  // or 2 columns, TMA-staged groups of 4) x
  // stencil (shared-memory tiles, warp streams) x row feed; index as in
  // set_launch_choice.
  for (int cand = 0; cand < kLaunchChoices && rc == CFD_OK; ++cand) {
    if (!launch_choice_ok(plan->p, cand)) continue;
    set_launch_choice(&plan->p, cand);
    rc = cfd_fvm_step(plan, stream, u, v, u_scratch, v_scratch, 1);
    if (rc) break;
    cudaError_t e = cudaEventRecord(e0, s);
    if (e == cudaSuccess) rc = cfd_fvm_step(plan, stream, u, v, u_scratch, v_scratch, steps);
    if (rc) break;
    if (e == cudaSuccess) e = cudaEventRecord(e1, s);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e != cudaSuccess) {
      rc = cuda_fail(e, "cfd_fvm_plan_autotune");
      break;
    }
    if (best < 0 || ms < best_ms) {
      best_ms = ms;
      best = cand;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (best < 0) best = 0;
  set_launch_choice(&plan->p, best);
  if (chosen) *chosen = best;
  return rc;
}

int cfd_fvm_plan_set_launch(cfd_fvm_plan* plan, int choice) {
  if (!plan || choice < 0 || choice >= kLaunchChoices)
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_plan_set_launch: bad arguments");
  if (!launch_choice_ok(plan->p, choice))
    return fail(CFD_ERR_UNSUPPORTED, "cfd_fvm_plan_set_launch: choice not available on this grid");
  set_launch_choice(&plan->p, choice);
  return CFD_OK;
}

int cfd_fvm_plan_get_launch(const cfd_fvm_plan* plan) {
  if (!plan) return -1;
  return plan->p.fft_shape + 2 * plan->p.col_mode + 12 * plan->p.stencil +
         24 * plan->p.row_feed + 48 * plan->p.stream_rows;
}

// ---- Same-shape batches -------------------------------------------------

static void batch_drop_graph(cfd_fvm_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
  b->graph_chunk = -1;
}

int cfd_fvm_batch_destroy(cfd_fvm_batch* b) {
  if (!b) return CFD_OK;
  batch_drop_graph(b);
  void* ptrs[] = {b->slab, b->force, b->lamx, b->lamy, b->twy, b->twpx, b->twpy, b->dev,
                  b->health};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  delete b;
  return CFD_OK;
}

int cfd_fvm_batch_create(const cfd_fvm_config* shape, int count, cfd_fvm_batch** out) {
  if (!shape || !out || count < 1 || count > 65535)
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_batch_create: bad arguments");
  *out = nullptr;
  cfd::FvmParams p;
  int rc = fvm_params_from_config(shape, &p);
  if (rc) return rc;
  if (!cfd::fvm_batch_shape_ok(p))
    return fail(CFD_ERR_UNSUPPORTED, "batched steps need nx % 16 == 0 and ny % 64 == 0");
  // Batches launch their kernels plainly: several batches run concurrently in
  // an ensemble graph, and programmatic launch (blocks waiting early) measured
  // slower there (197k against 206k trajectory-steps/s, 96-member ensemble).
  p.pdl = 0;
  // Grids of up to 64 x 64 cells run each member's whole chunk resident in
  // shared memory by default: 2.1 against 3.1-3.3 ms per 100 steps for 16-64
  // members at 64^2 (the autotuner can still choose otherwise).  At 128 x 64
  // one block per multiprocessor fits and the per-step launches are faster.
  if ((long long)p.nx * p.ny <= 64 * 64 && cfd::fvm_batch_resident_ok(p)) {
    p.stencil = 2;
    p.fft_shape = 0;
    p.col_mode = 0;
  } else if ((long long)p.nx * p.ny >= (1LL << 14)) {
    // The fastest configuration of every square size measured from 128^2 to
    // 1024^2 (batches of 15-24 slots, 20-step chunks): narrow row blocks fed by
    // bulk copies, the persistent column pass from 256 rows (TMA-staged where
    // its map encodes), warp streams from 512^2.
    p.fft_shape = 1;
    p.row_feed = cfd::bulk_feed_ok(p) ? 1 : 0;
    if (p.nx >= 256 && cfd::col_pipe_ok(p, 0)) p.col_mode = 3;
    p.stencil = ((long long)p.nx * p.ny >= (1LL << 18) && cfd::stream_stencil_ok(p)) ? 1 : 0;
    if (!cfd::fft_shape_ok(p)) p.fft_shape = 0;
  }
  cfd_fvm_batch* b = new cfd_fvm_batch();
  b->shape = p;
  b->hx = shape->hx;
  b->hy = shape->hy;
  b->count = count;
  const int nx = p.nx, ny = p.ny;
  const size_t n = (size_t)nx * ny;
  b->n = n;
  cudaError_t e = cudaMalloc((void**)&b->slab, (size_t)count * 7 * n * sizeof(float));
  if (e == cudaSuccess) e = cudaMemset(b->slab, 0, (size_t)count * 7 * n * sizeof(float));
  if (e == cudaSuccess)
    e = cudaMalloc((void**)&b->force, (size_t)count * (nx + ny) * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc((void**)&b->dev, (size_t)count * sizeof(cfd::FvmMember));
  if (e == cudaSuccess) e = cudaMalloc((void**)&b->health, (size_t)count * sizeof(cfd::Health));
  if (e == cudaSuccess) e = cudaMemset(b->health, 0, (size_t)count * sizeof(cfd::Health));
  std::vector<float> lamx = laplacian_eigenvalues(nx, shape->hx, nx);
  std::vector<float> lamy = laplacian_eigenvalues(ny, shape->hy, ny / 2 + 1);
  std::vector<float2> twy = twiddles(ny);
  std::vector<float2> twpx = pass_twiddles(p.log2nx), twpy = pass_twiddles(p.log2ny - 1);
  if (e == cudaSuccess) e = upload(&b->lamx, lamx.data(), lamx.size());
  if (e == cudaSuccess) e = upload(&b->lamy, lamy.data(), lamy.size());
  if (e == cudaSuccess) e = upload(&b->twy, twy.data(), twy.size());
  if (e == cudaSuccess) e = upload(&b->twpx, twpx.data(), twpx.size());
  if (e == cudaSuccess) e = upload(&b->twpy, twpy.data(), twpy.size());
  if (e != cudaSuccess) {
    cfd_fvm_batch_destroy(b);
    return cuda_fail(e, "cfd_fvm_batch_create");
  }
  b->bytes = (long long)count * (7 * (long long)n + nx + ny) * 4 +
             (long long)count * sizeof(cfd::FvmMember);
  b->host.assign(count, cfd::FvmMember());
  b->want.assign(count, 0);
  for (int i = 0; i < count; ++i) {
    cfd::FvmMember& m = b->host[i];
    std::memset(&m, 0, sizeof(m));
    m.p = p;
    m.p.lamx = b->lamx;
    m.p.lamy = b->lamy;
    m.p.tw_y = b->twy;
    m.p.twp_x = b->twpx;
    m.p.twp_y = b->twpy;
    float* base = b->slab + (size_t)i * 7 * n;
    for (int set = 0; set < 3; ++set) {
      m.f[set][0] = base + (2 * set) * n;
      m.f[set][1] = base + (2 * set + 1) * n;
    }
    m.spec = reinterpret_cast<float2*>(base + 6 * n);
    m.steps = 0;
  }
  // Every slot's spectrum at one stride (7 n floats): one 3-D map covers
  // them for the TMA-staged column pass, the default where it encodes.
  if (cfd::col_tma_grid_ok(b->shape) &&
      encode_spec_map(&b->spec_map, b->host[0].spec, nx, ny, count, 7 * n)) {
    b->shape.col_tmap = &b->spec_map;
    if (b->shape.col_mode == 3) b->shape.col_mode = 5;
  }
  *out = b;
  return CFD_OK;
}

int cfd_fvm_batch_size(const cfd_fvm_batch* b) { return b ? b->count : 0; }

long long cfd_fvm_batch_bytes(const cfd_fvm_batch* b) { return b ? b->bytes : 0; }

int cfd_fvm_batch_state(cfd_fvm_batch* b, int slot, float** u, float** v) {
  if (!b || !u || !v || slot < 0 || slot >= b->count)
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_batch_state: bad arguments");
  *u = b->host[slot].f[0][0];
  *v = b->host[slot].f[0][1];
  return CFD_OK;
}

int cfd_fvm_batch_set_slot(cfd_fvm_batch* b, void* stream, int slot, const cfd_fvm_config* cfg) {
  if (!b || !cfg || slot < 0 || slot >= b->count)
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_batch_set_slot: bad arguments");
  if (cfg->nx != b->shape.nx || cfg->ny != b->shape.ny || cfg->hx != b->hx ||
      cfg->hy != b->hy || cfg->convect != b->shape.convect)
    return fail(CFD_ERR_INVALID_ARGUMENT,
                "cfd_fvm_batch_set_slot: grid, step and convection must match the batch");
  if (cfg->const_forcing == CFD_FORCE_FULL)
    return fail(CFD_ERR_UNSUPPORTED, "batched steps take forcing tables over one axis only");
  cfd::FvmParams p;
  int rc = fvm_params_from_config(cfg, &p);
  if (rc) return rc;
  cfd::FvmMember& m = b->host[slot];
  const int nx = b->shape.nx, ny = b->shape.ny;
  float* fu = b->force + (size_t)slot * (nx + ny);
  float* fv = fu + ny;
  cudaStream_t s = as_stream(stream);
  if (cfg->const_forcing == CFD_FORCE_U_OF_Y && cfg->force_u)
    CFD_CHECK(cudaMemcpyAsync(fu, cfg->force_u, ny * sizeof(float), cudaMemcpyHostToDevice, s),
              "cfd_fvm_batch_set_slot: forcing");
  if (cfg->const_forcing == CFD_FORCE_V_OF_X && cfg->force_v)
    CFD_CHECK(cudaMemcpyAsync(fv, cfg->force_v, nx * sizeof(float), cudaMemcpyHostToDevice, s),
              "cfd_fvm_batch_set_slot: forcing");
  p.lamx = b->lamx;
  p.lamy = b->lamy;
  p.tw_y = b->twy;
  p.twp_x = b->twpx;
  p.twp_y = b->twpy;
  p.fu_y = (cfg->const_forcing == CFD_FORCE_U_OF_Y && cfg->force_u) ? fu : nullptr;
  p.fv_x = (cfg->const_forcing == CFD_FORCE_V_OF_X && cfg->force_v) ? fv : nullptr;
  p.fft_shape = b->shape.fft_shape;
  p.col_mode = b->shape.col_mode;
  m.p = p;
  b->dirty = true;
  return CFD_OK;
}

int cfd_fvm_batch_set_steps(cfd_fvm_batch* b, int slot, int steps) {
  if (!b || slot < 0 || slot >= b->count || steps < 0)
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_batch_set_steps: bad arguments");
  if (b->want[slot] != steps) b->dirty = true;
  b->want[slot] = steps;
  return CFD_OK;
}

// Uploads the slot table with every slot's steps clamped to `chunk`.
static int batch_upload(cfd_fvm_batch* b, cudaStream_t s, int chunk) {
  if (!b->dirty && b->uploaded_chunk == chunk) return CFD_OK;
  for (int i = 0; i < b->count; ++i) {
    b->host[i].steps = std::min(b->want[i], chunk);
    b->host[i].p.fft_shape = b->shape.fft_shape;
    b->host[i].p.col_mode = b->shape.col_mode;
    b->host[i].p.row_feed = b->shape.row_feed;
  }
  CFD_CHECK(cudaMemcpyAsync(b->dev, b->host.data(), b->host.size() * sizeof(cfd::FvmMember),
                            cudaMemcpyHostToDevice, s),
            "cfd_fvm_batch: slot table");
  b->dirty = false;
  b->uploaded_chunk = chunk;
  return CFD_OK;
}

static int batch_enqueue(cfd_fvm_batch* b, cudaStream_t s, int chunk) {
  if (b->shape.stencil == 2) {
    CFD_CHECK(cfd::launch_fvm_batch_resident(b->shape, b->dev, b->count, s), "batch resident");
  } else {
    for (int k = 0; k < chunk; ++k)
      CFD_CHECK(cfd::launch_fvm_batch_step(b->shape, b->dev, b->count, k, s), "batch step");
    CFD_CHECK(cfd::launch_fvm_batch_project_out(b->shape, b->dev, b->count, s),
              "batch project_out");
  }
  CFD_CHECK(cfd::launch_fvm_batch_health(b->shape, b->dev, b->count, b->health, b->mirror, s),
            "batch health");
  return CFD_OK;
}

int cfd_fvm_batch_run(cfd_fvm_batch* b, void* stream, int chunk, int use_graph) {
  if (!b || chunk < 0) return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_batch_run: bad arguments");
  if (chunk == 0) return CFD_OK;
  cudaStream_t s = as_stream(stream);
  int rc = batch_upload(b, s, chunk);
  if (rc) return rc;
  if (!use_graph) return batch_enqueue(b, s, chunk);
  if (!b->exec || b->graph_chunk != chunk) {
    batch_drop_graph(b);
    rc = capture_graph([&](cudaStream_t c) { return batch_enqueue(b, c, chunk); }, &b->graph,
                       &b->exec);
    if (rc) return rc;
    b->graph_chunk = chunk;
  }
  CFD_CHECK(cudaGraphLaunch(b->exec, s), "cudaGraphLaunch");
  return CFD_OK;
}

// Times every transform launch configuration on a `steps`-step chunk of all
// slots (with their current parameters and steps = `steps`), restores the
// slot states afterwards and keeps the fastest configuration.  Synchronises.
// Whether batch launch configuration c (index as in cfd_fvm_batch_autotune)
// applies to the batch's grid; sets it in `shape` when it does.
// Index = row shape + 2 * column scheme (0 blocks, 1/2 clusters of 4/8, 3
// pipelined groups of 4 staged by cp.async, 4 the same staged by TMA, run as
// col_mode 5) + 10 * stencil (0 tiles, 1 warp streams, 2 whole chunks
// resident in shared memory: one configuration, index 20, small grids only).
constexpr int kBatchLaunchChoices = 41;
static bool batch_launch_choice(cfd::FvmParams* shape, int c) {
  if (c < 0 || c >= kBatchLaunchChoices) return false;
  cfd::FvmParams q = *shape;
  // 21 .. 40: choices 0 .. 19 with the rows fed by bulk copies.
  q.row_feed = c > 20 ? 1 : 0;
  if (c > 20) {
    c -= 21;
    if (!cfd::bulk_feed_ok(q)) return false;
  }
  const int col = (c >> 1) % 5;
  q.fft_shape = c & 1;
  q.col_mode = col == 4 ? 5 : col;
  q.stencil = c / 10;
  if (q.stencil == 2) {
    if (!cfd::fvm_batch_resident_ok(q)) return false;
    q.fft_shape = 0;
    q.col_mode = 0;
    *shape = q;
    return true;
  }
  if ((q.col_mode == 1 || q.col_mode == 2) && !cfd::col_cluster_ok(q, q.col_mode == 1 ? 4 : 8))
    return false;
  if (q.col_mode == 3 && !cfd::col_pipe_ok(q, 0)) return false;
  if (q.col_mode == 5 && !(q.col_tmap && cfd::col_tma_grid_ok(q))) return false;
  if (q.stencil == 1 && !cfd::stream_stencil_ok(q)) return false;
  if (!cfd::fft_shape_ok(q)) return false;
  *shape = q;
  return true;
}

int cfd_fvm_batch_set_launch(cfd_fvm_batch* b, int choice) {
  if (!b || choice < 0 || choice >= kBatchLaunchChoices)
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_batch_set_launch: bad arguments");
  if (!batch_launch_choice(&b->shape, choice))
    return fail(CFD_ERR_UNSUPPORTED, "cfd_fvm_batch_set_launch: choice not available on this grid");
  b->dirty = true;
  batch_drop_graph(b);
  return CFD_OK;
}

int cfd_fvm_batch_autotune(cfd_fvm_batch* b, void* stream, int steps, int* chosen) {
  if (!b || steps < 1) return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_batch_autotune: bad arguments");
  cudaStream_t s = as_stream(stream);
  const size_t n = b->n;
  float* backup = nullptr;
  CFD_CHECK(cudaMalloc((void**)&backup, (size_t)b->count * 2 * n * sizeof(float)),
            "cfd_fvm_batch_autotune");
  std::vector<int> want = b->want;
  auto save = [&](bool restore) -> cudaError_t {
    for (int i = 0; i < b->count; ++i) {
      float* st = b->host[i].f[0][0];  // u then v, contiguous in the slab
      float* bk = backup + (size_t)i * 2 * n;
      cudaError_t e = restore ? cudaMemcpyAsync(st, bk, 2 * n * sizeof(float),
                                                cudaMemcpyDeviceToDevice, s)
                              : cudaMemcpyAsync(bk, st, 2 * n * sizeof(float),
                                                cudaMemcpyDeviceToDevice, s);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  };
  cudaEvent_t e0, e1;
  cudaError_t e = save(false);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e != cudaSuccess) {
    cudaFree(backup);
    return cuda_fail(e, "cfd_fvm_batch_autotune");
  }
  for (int i = 0; i < b->count; ++i) b->want[i] = steps;
  b->dirty = true;
  int rc = CFD_OK, best = -1;
  float best_ms = 0.f;
  // Candidates: index = row-transform shape + 2 * column scheme (0 blocks, 1/2
  // clusters of 4/8, 3 persistent pipelined groups) + 8 * stencil (0 tiles,
  // 1 warp streams).
  for (int cand = 0; cand < kBatchLaunchChoices && rc == CFD_OK; ++cand) {
    if (!batch_launch_choice(&b->shape, cand)) continue;
    b->dirty = true;
    rc = cfd_fvm_batch_run(b, stream, 1, 0);  // warm-up (and per-kernel smem setup)
    if (rc) break;
    e = cudaEventRecord(e0, s);
    if (e == cudaSuccess) rc = cfd_fvm_batch_run(b, stream, steps, 0);
    if (rc) break;
    if (e == cudaSuccess) e = cudaEventRecord(e1, s);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess) e = save(true);
    if (e != cudaSuccess) {
      rc = cuda_fail(e, "cfd_fvm_batch_autotune");
      break;
    }
    if (best < 0 || ms < best_ms) {
      best_ms = ms;
      best = cand;
    }
  }
  if (rc == CFD_OK) {
    e = save(true);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = cuda_fail(e, "cfd_fvm_batch_autotune");
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(backup);
  if (best < 0 || !batch_launch_choice(&b->shape, best)) {
    best = 0;
    batch_launch_choice(&b->shape, 0);
  }
  b->want = want;
  b->dirty = true;
  batch_drop_graph(b);
  if (chosen) *chosen = best;
  return rc;
}

// ---- Ensembles of batches ------------------------------------------------

static void ensemble_drop_graph(cfd_fvm_ensemble* ens) {
  if (ens->exec) cudaGraphExecDestroy(ens->exec);
  if (ens->graph) cudaGraphDestroy(ens->graph);
  ens->exec = nullptr;
  ens->graph = nullptr;
  ens->graph_steps = -1;
}

int cfd_fvm_ensemble_destroy(cfd_fvm_ensemble* ens) {
  if (!ens) return CFD_OK;
  ensemble_drop_graph(ens);
  for (auto e : ens->joins) if (e) cudaEventDestroy(e);
  if (ens->fork) cudaEventDestroy(ens->fork);
  for (auto st : ens->streams) if (st) cudaStreamDestroy(st);
  for (auto b : ens->batches) cfd_fvm_batch_destroy(b);
  delete ens;
  return CFD_OK;
}

int cfd_fvm_ensemble_create(const cfd_fvm_config* cfgs, int count, cfd_fvm_ensemble** out) {
  if (!cfgs || !out || count < 1)
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_ensemble_create: bad arguments");
  *out = nullptr;
  // Members with the same grid, step and convection scheme share a batch.
  std::vector<int> bucket(count, -1);
  std::vector<int> reps, sizes;
  for (int i = 0; i < count; ++i) {
    const cfd_fvm_config& c = cfgs[i];
    for (size_t r = 0; r < reps.size(); ++r) {
      const cfd_fvm_config& d = cfgs[reps[r]];
      if (c.nx == d.nx && c.ny == d.ny && c.hx == d.hx && c.hy == d.hy &&
          c.convect == d.convect) {
        bucket[i] = (int)r;
        break;
      }
    }
    if (bucket[i] < 0) {
      bucket[i] = (int)reps.size();
      reps.push_back(i);
      sizes.push_back(0);
    }
    ++sizes[bucket[i]];
  }
  cfd_fvm_ensemble* ens = new cfd_fvm_ensemble();
  ens->where.assign(count, {0, 0});
  int rc = CFD_OK;
  for (size_t r = 0; r < reps.size() && rc == CFD_OK; ++r) {
    cfd_fvm_batch* b = nullptr;
    rc = cfd_fvm_batch_create(&cfgs[reps[r]], sizes[r], &b);
    if (rc == CFD_OK) ens->batches.push_back(b);
  }
  std::vector<int> fill(reps.size(), 0);
  for (int i = 0; i < count && rc == CFD_OK; ++i) {
    const int r = bucket[i];
    const int slot = fill[r]++;
    ens->where[i] = {r, slot};
    rc = cfd_fvm_batch_set_slot(ens->batches[r], nullptr, slot, &cfgs[i]);
  }
  cudaError_t e = cudaSuccess;
  if (rc == CFD_OK) e = cudaStreamSynchronize(nullptr);
  if (rc == CFD_OK && e == cudaSuccess) e = cudaEventCreateWithFlags(&ens->fork, cudaEventDisableTiming);
  for (size_t r = 0; r < ens->batches.size() && rc == CFD_OK && e == cudaSuccess; ++r) {
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    ens->streams.push_back(st);
    ens->joins.push_back(ev);
  }
  if (rc == CFD_OK && e != cudaSuccess) rc = cuda_fail(e, "cfd_fvm_ensemble_create");
  if (rc) {
    cfd_fvm_ensemble_destroy(ens);
    return rc;
  }
  *out = ens;
  return CFD_OK;
}

int cfd_fvm_ensemble_size(const cfd_fvm_ensemble* ens) {
  return ens ? (int)ens->where.size() : 0;
}

int cfd_fvm_ensemble_batches(const cfd_fvm_ensemble* ens) {
  return ens ? (int)ens->batches.size() : 0;
}

int cfd_fvm_ensemble_state(cfd_fvm_ensemble* ens, int index, float** u, float** v) {
  if (!ens || index < 0 || index >= (int)ens->where.size())
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_ensemble_state: bad arguments");
  const auto w = ens->where[index];
  return cfd_fvm_batch_state(ens->batches[w.first], w.second, u, v);
}

int cfd_fvm_batch_health(cfd_fvm_batch* b, const cfd_health** out) {
  if (!b || !out) return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_batch_health: null pointer");
  *out = reinterpret_cast<const cfd_health*>(b->health);
  return CFD_OK;
}

// A device-addressable host pointer for the health mirror: pinned memory
// (cudaHostAlloc / cudaHostRegister) maps into the device's address space.
static int health_mirror_ptr(void* host, int count, cfd::Health** out, const char* who) {
  *out = nullptr;
  if (!host) return CFD_OK;
  cudaPointerAttributes a;
  cudaError_t e = cudaPointerGetAttributes(&a, host);
  if (e != cudaSuccess) return cuda_fail(e, who);
  if (a.type != cudaMemoryTypeHost || !a.devicePointer)
    return fail(CFD_ERR_INVALID_ARGUMENT,
                std::string(who) + ": the mirror must be pinned host memory the device can address");
  (void)count;
  *out = static_cast<cfd::Health*>(a.devicePointer);
  return CFD_OK;
}

int cfd_fvm_batch_set_health_mirror(cfd_fvm_batch* b, void* host_records) {
  if (!b) return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_batch_set_health_mirror: null batch");
  cfd::Health* m = nullptr;
  int rc = health_mirror_ptr(host_records, b->count, &m, "cfd_fvm_batch_set_health_mirror");
  if (rc) return rc;
  if (m != b->mirror) {
    b->mirror = m;
    batch_drop_graph(b);  // the pointer is part of the captured chunk
  }
  return CFD_OK;
}

int cfd_fvm_ensemble_health(cfd_fvm_ensemble* ens, int index, const cfd_health** out) {
  if (!ens || !out || index < 0 || index >= (int)ens->where.size())
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_ensemble_health: bad arguments");
  const auto w = ens->where[index];
  *out = reinterpret_cast<const cfd_health*>(ens->batches[w.first]->health + w.second);
  return CFD_OK;
}

int cfd_fvm_ensemble_autotune(cfd_fvm_ensemble* ens, void* stream, int steps) {
  if (!ens) return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_ensemble_autotune: null");
  for (auto* b : ens->batches) {
    int rc = cfd_fvm_batch_autotune(b, stream, steps, nullptr);
    if (rc) return rc;
  }
  ensemble_drop_graph(ens);
  return CFD_OK;
}

static int ensemble_enqueue(cfd_fvm_ensemble* ens, cudaStream_t s, int steps) {
  CFD_CHECK(cudaEventRecord(ens->fork, s), "cudaEventRecord");
  for (size_t r = 0; r < ens->batches.size(); ++r) {
    CFD_CHECK(cudaStreamWaitEvent(ens->streams[r], ens->fork, 0), "cudaStreamWaitEvent");
    int rc = batch_enqueue(ens->batches[r], ens->streams[r], steps);
    if (rc) return rc;
    CFD_CHECK(cudaEventRecord(ens->joins[r], ens->streams[r]), "cudaEventRecord");
    CFD_CHECK(cudaStreamWaitEvent(s, ens->joins[r], 0), "cudaStreamWaitEvent");
  }
  return CFD_OK;
}

int cfd_fvm_ensemble_step(cfd_fvm_ensemble* ens, void* stream, int steps, int use_graph) {
  if (!ens || steps < 0) return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_ensemble_step: bad arguments");
  if (steps == 0) return CFD_OK;
  cudaStream_t s = as_stream(stream);
  for (auto* b : ens->batches) {
    for (int i = 0; i < b->count; ++i) cfd_fvm_batch_set_steps(b, i, steps);
    int rc = batch_upload(b, s, steps);
    if (rc) return rc;
  }
  if (!use_graph) return ensemble_enqueue(ens, s, steps);
  if (!ens->exec || ens->graph_steps != steps) {
    ensemble_drop_graph(ens);
    int rc = capture_graph([&](cudaStream_t c) { return ensemble_enqueue(ens, c, steps); },
                           &ens->graph, &ens->exec);
    if (rc) return rc;
    ens->graph_steps = steps;
  }
  CFD_CHECK(cudaGraphLaunch(ens->exec, s), "cudaGraphLaunch");
  return CFD_OK;
}

int cfd_fvm_adjoint_step(cfd_fvm_plan* plan, void* stream, const float* u, const float* v,
                         const float* gu, const float* gv, float* gu_out, float* gv_out,
                         float* nu_dot) {
  if (!plan || !u || !v || !gu || !gv || !gu_out || !gv_out)
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_adjoint_step: null pointer");
  cudaStream_t s = as_stream(stream);
  const cfd::FvmParams& p = plan->p;
  // w = P g into the plan's first step buffers.
  CFD_CHECK(cfd::launch_fvm_div_rfft(p, gu, gv, plan->spec, s), "div_rfft");
  CFD_CHECK(cfd::launch_fvm_col_pinv(p, plan->spec, s), "col_pinv");
  CFD_CHECK(cfd::launch_fvm_irfft(p, plan->spec, s), "irfft");
  CFD_CHECK(cfd::launch_fvm_project_out(p, gu, gv, reinterpret_cast<const float*>(plan->spec),
                                        plan->au, plan->av, s),
            "project_out");
  CFD_CHECK(cfd::launch_fvm_adjoint(p, u, v, plan->au, plan->av, gu_out, gv_out, nu_dot, s),
            "adjoint");
  return CFD_OK;
}

int cfd_fvm_adjoint_segment(cfd_fvm_plan* plan, void* stream, const float* u0,
                            const float* v0, int steps, float* states, float* gu, float* gv,
                            float* nu_scratch, double* nu_acc) {
  if (!plan || !u0 || !v0 || !gu || !gv || steps < 1 || (steps > 1 && !states) ||
      (!nu_scratch) != (!nu_acc))
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_adjoint_segment: bad arguments");
  cudaStream_t s = as_stream(stream);
  const size_t cells = (size_t)plan->p.nx * plan->p.ny;
  if (nu_acc && !plan->partials)
    CFD_CHECK(cudaMalloc((void**)&plan->partials, cfd::kSumBlocks * sizeof(double)),
              "cfd_fvm_adjoint_segment: cudaMalloc");
  // State k (k >= 1) of the segment at states + 2 (k - 1) cells (u, then v).
  auto su = [&](int k) { return k == 0 ? u0 : states + 2 * (size_t)(k - 1) * cells; };
  auto sv = [&](int k) { return k == 0 ? v0 : states + (2 * (size_t)(k - 1) + 1) * cells; };
  for (int k = 1; k < steps; ++k) {
    const int rc = cfd_fvm_step(plan, stream, su(k - 1), sv(k - 1), const_cast<float*>(su(k)),
                                const_cast<float*>(sv(k)), 1);
    if (rc) return rc;
  }
  for (int k = steps - 1; k >= 0; --k) {
    const int rc = cfd_fvm_adjoint_step(plan, stream, su(k), sv(k), gu, gv, gu, gv, nu_scratch);
    if (rc) return rc;
    if (nu_acc)
      CFD_CHECK(cfd::launch_sum_to_double(nu_scratch, cells, plan->partials, nu_acc, s),
                "viscosity sum");
  }
  return CFD_OK;
}

int cfd_fvm_explicit_terms(cfd_fvm_plan* plan, void* stream, const float* u,
                           const float* v, float* du, float* dv) {
  if (!plan || !u || !v || !du || !dv)
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_explicit_terms: null pointer");
  CFD_CHECK(cfd::launch_fvm_explicit(plan->p, false, true, u, v, nullptr, du, dv,
                                     as_stream(stream)),
            "explicit");
  return CFD_OK;
}

int cfd_fvm_projection(cfd_fvm_plan* plan, void* stream, const float* u,
                       const float* v, float* u_out, float* v_out) {
  if (!plan || !u || !v || !u_out || !v_out)
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_projection: null pointer");
  cudaStream_t s = as_stream(stream);
  int rc = fvm_pressure(plan, s, u, v);
  if (rc) return rc;
  CFD_CHECK(cfd::launch_fvm_project_out(plan->p, u, v,
                                        reinterpret_cast<const float*>(plan->spec),
                                        u_out, v_out, s),
            "project_out");
  return CFD_OK;
}

int cfd_fvm_pressure_solve(cfd_fvm_plan* plan, void* stream, const float* u,
                           const float* v, float* q) {
  if (!plan || !u || !v || !q)
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_pressure_solve: null pointer");
  cudaStream_t s = as_stream(stream);
  int rc = fvm_pressure(plan, s, u, v);
  if (rc) return rc;
  CFD_CHECK(cudaMemcpyAsync(q, plan->spec, (size_t)plan->p.nx * plan->p.ny * sizeof(float),
                            cudaMemcpyDeviceToDevice, s),
            "copy q");
  return CFD_OK;
}

int cfd_fvm_divergence(cfd_fvm_plan* plan, void* stream, const float* u,
                       const float* v, float* out) {
  if (!plan || !u || !v || !out)
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_divergence: null pointer");
  CFD_CHECK(cfd::launch_divergence(plan->p, u, v, out, as_stream(stream)), "divergence");
  return CFD_OK;
}

int cfd_fvm_curl_2d(cfd_fvm_plan* plan, void* stream, const float* u,
                    const float* v, float* out) {
  if (!plan || !u || !v || !out)
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_curl_2d: null pointer");
  CFD_CHECK(cfd::launch_curl2d(plan->p, u, v, out, as_stream(stream)), "curl_2d");
  return CFD_OK;
}

int cfd_max_speed(void* stream, int n, const float* u, const float* v, float* out) {
  if (n <= 0 || !u || !v || !out)
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_max_speed: bad arguments");
  CFD_CHECK(cfd::launch_max_speed(n, u, v, reinterpret_cast<unsigned int*>(out),
                                  as_stream(stream)),
            "max_speed");
  return CFD_OK;
}

}  // extern "C"

namespace {
__global__ void scale_to_max_kernel(int n, float* u, float* v, const float* vmax,
                                    float maxv) {
  const float m = *vmax;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    u[i] = (maxv * u[i]) / m;
    v[i] = (maxv * v[i]) / m;
  }
}
}  // namespace

extern "C" {

int cfd_scale_to_max_speed(void* stream, int n, float* u, float* v,
                           const float* vmax, double maximum_velocity) {
  if (n <= 0 || !u || !v || !vmax)
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_scale_to_max_speed: bad arguments");
  int blocks = (n + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  scale_to_max_kernel<<<blocks, 256, 0, as_stream(stream)>>>(n, u, v, vmax,
                                                             (float)maximum_velocity);
  CFD_CHECK(cudaGetLastError(), "scale_to_max_speed");
  return CFD_OK;
}

// ---------------------------------------------------------------------------
// Spectral plan
// ---------------------------------------------------------------------------
int cfd_spec_plan_destroy(cfd_spec_plan* plan) {
  if (!plan) return CFD_OK;
  void* ptrs[] = {plan->t4[0], plan->t4[1], plan->t4[2], plan->t4[3], plan->ahat,
                  plan->h, plan->fc, plan->work, plan->twy, plan->twpx, plan->twpy,
                  plan->kx, plan->ky, plan->wt, plan->ht};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  delete plan;
  return CFD_OK;
}

// Scalar parameters and stage coefficients of one spectral configuration (no
// device tables); shared by plans and batch slots.
static int spec_params_from_config(const cfd_spec_config* cfg, cfd::SpecParams* out,
                                   cfd::StageCoef* coef, int* stages) {
  if (!valid_size(cfg->nx) || !valid_size(cfg->ny))
    return fail(CFD_ERR_UNSUPPORTED, "grid shape must be powers of two in [4, 4096]");
  if (cfg->num_stages < 1 || cfg->num_stages > 8 || !cfg->alphas || !cfg->betas || !cfg->gammas)
    return fail(CFD_ERR_INVALID_ARGUMENT, "num_stages must be in [1, 8] with coefficient arrays");
  if (!(cfg->hx > 0) || !(cfg->hy > 0))
    return fail(CFD_ERR_INVALID_ARGUMENT, "invalid grid step");
  cfd::SpecParams& p = *out;
  std::memset(&p, 0, sizeof(p));
  const int nx = cfg->nx, ny = cfg->ny;
  p.nx = nx;
  p.ny = ny;
  // Programmatic dependent launch of the stage kernels: 0.713 against
  // 0.735 ms per 2048^2 CN-RK4 step (CFD_GB300_PDL=0 turns it off; batches
  // launch their kernels plainly whatever this says).
  const char* pdl = std::getenv("CFD_GB300_PDL");
  p.pdl = (pdl && pdl[0] == '0') ? 0 : 1;
  p.L = ny / 2;
  p.pitch = p.L + 4;
  p.log2nx = ilog2(nx);
  p.log2ny = ilog2(ny);
  p.log2L = p.log2ny - 1;
  p.dn_x = (float)(cfg->hx * nx);
  p.dn_y = (float)(cfg->hy * ny);
  p.two_pi = (float)(2.0 * M_PI);
  p.lap_coef = (float)(-4.0 * M_PI * M_PI);
  p.nu = (float)cfg->viscosity;
  p.drag = (float)cfg->drag;
  p.scale = 1.f / ((float)nx * (float)ny);
  p.filt_on = cfg->smooth ? 1 : 0;
  // brick_wall_filter_2d: rows [: int(2/3 n) // 2] and [-int(2/3 n) // 2 :]
  // (Python floor division of the negated int), cols [: int(2/3 (m//2+1))].
  {
    const int a = (int)(2.0 / 3.0 * nx);
    p.filt_lo = a / 2;
    const int neg = -a;
    const int start = (neg >= 0) ? neg / 2 : -((-neg + 1) / 2);  // floor(-a / 2)
    p.filt_hi = nx + start;
    p.filt_cols = (int)(2.0 / 3.0 * (ny / 2 + 1));
  }
  *stages = cfg->num_stages;
  for (int k = 0; k < cfg->num_stages; ++k) {
    cfd::StageCoef& c = coef[k];
    c.beta = (float)cfg->betas[k];
    c.gdt = (float)(cfg->gammas[k] * cfg->dt);
    c.mu = (float)(0.5 * cfg->dt * (cfg->alphas[k + 1] - cfg->alphas[k]));
    c.has_h_in = (k > 0 && cfg->betas[k] != 0.0) ? 1 : 0;
    c.write_h = (k + 1 < cfg->num_stages) ? 1 : 0;
    c.prep_next = 1;
    c.explicit_only = 0;
    c.tiled = 0;
  }
  return CFD_OK;
}

// Host tables of a spectral grid: real-FFT untangling twiddles, pass tables
// and the fftfreq / rfftfreq wavenumbers (float32 ordinals over
// float32(step * n), grids.py:618-658 via jnp.fft.fftfreq).
struct SpecTables {
  std::vector<float2> twy, twpx, twpy;
  std::vector<float> kx, ky;
};
static SpecTables spec_tables(const cfd::SpecParams& p) {
  SpecTables t;
  t.twy = twiddles(p.ny);
  t.twpx = pass_twiddles(p.log2nx);
  t.twpy = pass_twiddles(p.log2L);
  t.kx.resize(p.nx);
  t.ky.resize(p.L + 1);
  for (int k = 0; k < p.nx; ++k) t.kx[k] = (float)(k < p.nx / 2 ? k : k - p.nx) / p.dn_x;
  for (int k = 0; k <= p.L; ++k) t.ky[k] = (float)k / p.dn_y;
  return t;
}

int cfd_spec_plan_create(const cfd_spec_config* cfg, cfd_spec_plan** out) {
  if (!cfg || !out) return fail(CFD_ERR_INVALID_ARGUMENT, "null config or output pointer");
  *out = nullptr;
  cfd::SpecParams params;
  cfd::StageCoef coef[8];
  int stages = 0;
  int rc = spec_params_from_config(cfg, &params, coef, &stages);
  if (rc) return rc;
  cfd_spec_plan* plan = new cfd_spec_plan();
  cfd::SpecParams& p = plan->p;
  p = params;
  // Clustered column passes measured faster at 256^2 and 512^2, the
  // persistent pipelined ones with the fused update + prep at 2048^2 (GB300).
  p.col_mode = (cfg->nx >= 256 && cfg->nx <= 512) ? 1 : 0;
  if (cfg->nx >= 1024) {
    p.col_mode = 4;
    if (!cfd::spec_pipe_ok(p)) p.col_mode = 0;
  }
  // The register-pass row pass measured faster at 2048^2 (66.5 against 72.1 us),
  // and with registers for more blocks per multiprocessor faster still at
  // ny = 2048 (three blocks: 61.7 against 66.3 us; four, with one exchange
  // buffer per field: 42.1 against 43.6 us at three and 48.2 for the earlier
  // two-buffer layout) but not at ny = 1024 (24.6 against 20.8 us).
  p.row_mode = cfd::spec_row_pipe_ok(p) ? 1 : 0;
  if (p.row_mode == 1 && p.log2L == 10) p.row_mode = 2;
  plan->stages = stages;
  for (int k = 0; k < stages; ++k) plan->coef[k] = coef[k];
  const int nx = cfg->nx;
  const size_t ns = (size_t)nx * (p.L + 1);
  cudaError_t e;
  long long bytes = 0;
#define CFD_ALLOC(ptr, count)                                              \
  do {                                                                     \
    e = cudaMalloc((void**)&(ptr), (count) * sizeof(*(ptr)));              \
    if (e != cudaSuccess) {                                                \
      cfd_spec_plan_destroy(plan);                                         \
      return cuda_fail(e, "cfd_spec_plan_create: cudaMalloc");             \
    }                                                                      \
    bytes += (long long)((count) * sizeof(*(ptr)));                        \
  } while (0)
  // The four column-transformed fields and the advection spectrum: rows of
  // p.pitch values (32-byte multiples), of which the first L + 1 are columns.
  const size_t nsp = (size_t)nx * p.pitch;
  for (int f = 0; f < 4; ++f) CFD_ALLOC(plan->t4[f], nsp);
  CFD_ALLOC(plan->ahat, nsp);
  CFD_ALLOC(plan->h, ns);
  CFD_ALLOC(plan->work, ns);
  {
    // The tiled state for the fused column stage, on grids where that launch
    // choice exists (whatever the current one).
    cfd::SpecParams q = p;
    q.col_mode = 4;
    if (cfd::spec_state_tiled_ok(q)) {
      CFD_ALLOC(plan->wt, cfd::spec_tiled_elems(q));
      CFD_ALLOC(plan->ht, cfd::spec_tiled_elems(q));
    }
  }
#undef CFD_ALLOC
  {
    // TMA maps for the fused column stage (its groups of 4 columns, rows up
    // to 2048); without them the stage stages by cp.async (same results).
    bool ok = nx >= 256 && nx <= 2048;
    ok = ok && encode_rows_map(plan->maps.ahat, plan->ahat, 2 * p.pitch, nx);
    for (int f = 0; f < 4 && ok; ++f) ok = encode_rows_map(plan->maps.t[f], plan->t4[f], 2 * p.pitch, nx);
    p.stage_maps = ok ? &plan->maps : nullptr;
  }
  const SpecTables t = spec_tables(p);
  if ((e = upload(&plan->twy, t.twy.data(), t.twy.size())) != cudaSuccess ||
      (e = upload(&plan->twpx, t.twpx.data(), t.twpx.size())) != cudaSuccess ||
      (e = upload(&plan->twpy, t.twpy.data(), t.twpy.size())) != cudaSuccess ||
      (e = upload(&plan->kx, t.kx.data(), t.kx.size())) != cudaSuccess ||
      (e = upload(&plan->ky, t.ky.data(), t.ky.size())) != cudaSuccess) {
    cfd_spec_plan_destroy(plan);
    return cuda_fail(e, "cfd_spec_plan_create: tables");
  }
  bytes += (long long)(t.twy.size() + t.twpx.size() + t.twpy.size()) * 8 +
           (long long)(t.kx.size() + t.ky.size()) * 4;
  p.tw_y = plan->twy;
  p.twp_x = plan->twpx;
  p.twp_y = plan->twpy;
  p.kx = plan->kx;
  p.ky = plan->ky;
  plan->bytes = bytes;
  *out = plan;
  return CFD_OK;
}

long long cfd_spec_plan_bytes(const cfd_spec_plan* plan) { return plan ? plan->bytes : 0; }

// Spectral launch choice = column scheme (0..4) + 5 * row scheme (0..2).
int cfd_spec_plan_set_launch(cfd_spec_plan* plan, int choice) {
  if (!plan || choice < 0 || choice >= 15)
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_spec_plan_set_launch: bad arguments");
  cfd::SpecParams q = plan->p;
  q.col_mode = choice % 5;
  q.row_mode = choice / 5;
  if ((q.col_mode == 1 && !cfd::spec_cluster_ok(q)) || (q.col_mode >= 2 && !cfd::spec_pipe_ok(q)) ||
      (q.row_mode >= 1 && !cfd::spec_row_pipe_ok(q)))
    return fail(CFD_ERR_UNSUPPORTED, "cfd_spec_plan_set_launch: choice not available on this grid");
  plan->p.col_mode = q.col_mode;
  plan->p.row_mode = q.row_mode;
  return CFD_OK;
}

int cfd_spec_plan_get_launch(const cfd_spec_plan* plan) {
  return plan ? plan->p.col_mode + 5 * plan->p.row_mode : -1;
}

int cfd_rfft2(cfd_spec_plan* plan, void* stream, const float* x, float* xhat) {
  if (!plan || !x || !xhat) return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_rfft2: null pointer");
  cudaStream_t s = as_stream(stream);
  float2* X = reinterpret_cast<float2*>(xhat);
  CFD_CHECK(cfd::launch_row_rfft(plan->p, x, X, s), "row_rfft");
  CFD_CHECK(cfd::launch_col_fft(plan->p, X, -1, nullptr, s), "col_fft");
  return CFD_OK;
}

int cfd_irfft2(cfd_spec_plan* plan, void* stream, const float* xhat, float* x) {
  if (!plan || !x || !xhat) return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_irfft2: null pointer");
  cudaStream_t s = as_stream(stream);
  const size_t ns = (size_t)plan->p.nx * (plan->p.L + 1);
  CFD_CHECK(cudaMemcpyAsync(plan->work, xhat, ns * sizeof(float2), cudaMemcpyDeviceToDevice, s),
            "copy");
  CFD_CHECK(cfd::launch_col_fft(plan->p, plan->work, 1, nullptr, s), "col_ifft");
  CFD_CHECK(cfd::launch_row_irfft(plan->p, plan->work, x, plan->p.scale, s), "row_irfft");
  return CFD_OK;
}

int cfd_spectral_filter(cfd_spec_plan* plan, void* stream, const float* x,
                        const float* table, float* out) {
  if (!plan || !x || !table || !out)
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_spectral_filter: null pointer");
  cudaStream_t s = as_stream(stream);
  CFD_CHECK(cfd::launch_row_rfft(plan->p, x, plan->work, s), "row_rfft");
  CFD_CHECK(cfd::launch_col_fft(plan->p, plan->work, -1, table, s), "col_fft");
  CFD_CHECK(cfd::launch_col_fft(plan->p, plan->work, 1, nullptr, s), "col_ifft");
  CFD_CHECK(cfd::launch_row_irfft(plan->p, plan->work, out, plan->p.scale, s), "row_irfft");
  return CFD_OK;
}

int cfd_spec_set_forcing(cfd_spec_plan* plan, void* stream, const float* fx,
                         const float* fy) {
  if (!plan) return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_spec_set_forcing: null plan");
  cudaStream_t s = as_stream(stream);
  cfd::SpecParams& p = plan->p;
  p.fc_full = nullptr;
  p.fc_row0 = nullptr;
  if (plan->fc) {
    cudaFree(plan->fc);
    plan->fc = nullptr;
  }
  if (!fx && !fy) return CFD_OK;
  const size_t ns = (size_t)p.nx * (p.L + 1);
  float2 *fxh = plan->t4[0], *fyh = plan->t4[1];
  if (fx) {
    int rc = cfd_rfft2(plan, stream, fx, reinterpret_cast<float*>(fxh));
    if (rc) return rc;
  } else {
    CFD_CHECK(cudaMemsetAsync(fxh, 0, ns * sizeof(float2), s), "memset");
  }
  if (fy) {
    int rc = cfd_rfft2(plan, stream, fy, reinterpret_cast<float*>(fyh));
    if (rc) return rc;
  } else {
    CFD_CHECK(cudaMemsetAsync(fyh, 0, ns * sizeof(float2), s), "memset");
  }
  float2* table = nullptr;
  CFD_CHECK(cudaMalloc((void**)&table, ns * sizeof(float2)), "cfd_spec_set_forcing: cudaMalloc");
  int rc = CFD_OK;
  cudaError_t e = cfd::launch_spec_curl_table(p, fxh, fyh, table, s);
  std::vector<float2> host(ns);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(host.data(), table, ns * sizeof(float2), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    cudaFree(table);
    return cuda_fail(e, "cfd_spec_set_forcing");
  }
  bool row0_only = true;
  for (size_t g = (size_t)(p.L + 1); g < ns && row0_only; ++g)
    if (host[g].x != 0.f || host[g].y != 0.f) row0_only = false;
  if (row0_only) {
    // Keep only row kx = 0: the x-transform of an x-independent field.
    float2* row = nullptr;
    e = cudaMalloc((void**)&row, (p.L + 1) * sizeof(float2));
    if (e == cudaSuccess)
      e = cudaMemcpy(row, host.data(), (p.L + 1) * sizeof(float2), cudaMemcpyHostToDevice);
    cudaFree(table);
    if (e != cudaSuccess) return cuda_fail(e, "cfd_spec_set_forcing");
    plan->fc = row;
    p.fc_row0 = row;
  } else {
    plan->fc = table;
    p.fc_full = table;
  }
  return rc;
}

int cfd_spec_step(cfd_spec_plan* plan, void* stream, const float* w_in,
                  float* w_out, int steps) {
  if (!plan || !w_in || !w_out) return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_spec_step: null pointer");
  if (steps < 0) return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_spec_step: steps < 0");
  cudaStream_t s = as_stream(stream);
  const cfd::SpecParams& p = plan->p;
  const size_t ns = (size_t)p.nx * (p.L + 1);
  float2* w = reinterpret_cast<float2*>(w_out);
  if (w_out != w_in)
    CFD_CHECK(cudaMemcpyAsync(w_out, w_in, ns * sizeof(float2), cudaMemcpyDeviceToDevice, s),
              "copy");
  if (steps == 0) return CFD_OK;
  // The fused column stage keeps the state and h tiled by column groups for
  // the chunk (same values, contiguous per group); converted once each way.
  const bool tiled = plan->wt && cfd::spec_state_tiled_ok(p);
  float2* ws = tiled ? plan->wt : w;
  float2* hs = tiled ? plan->ht : plan->h;
  CFD_CHECK(cfd::launch_spec_col_prep(p, w, plan->t4, s), "col_prep");
  if (tiled) CFD_CHECK(cfd::spec_tile_state(p, w, ws, true, s), "tile state");
  for (int st = 0; st < steps; ++st) {
    for (int k = 0; k < plan->stages; ++k) {
      CFD_CHECK(cfd::launch_spec_row(p, plan->t4, plan->ahat, s), "row");
      cfd::StageCoef c = plan->coef[k];
      c.prep_next = (st + 1 == steps && k + 1 == plan->stages) ? 0 : 1;
      c.tiled = tiled ? 1 : 0;
      CFD_CHECK(cfd::launch_spec_col_update(p, c, plan->ahat, ws, hs, plan->t4, s),
                "col_update");
    }
  }
  if (tiled) CFD_CHECK(cfd::spec_tile_state(p, ws, w, false, s), "untile state");
  return CFD_OK;
}

// cfd_spec_step with an event pair around every launch; mean ms per kernel
// kind written to ms_out[3] = {row pass, column update, column prep}.
int cfd_spec_profile(cfd_spec_plan* plan, void* stream, const float* w_in,
                     float* w_out, int steps, float* ms_out) {
  if (!plan || !w_in || !w_out || !ms_out || steps < 1)
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_spec_profile: bad arguments");
  cudaStream_t s = as_stream(stream);
  const cfd::SpecParams& p = plan->p;
  const size_t ns = (size_t)p.nx * (p.L + 1);
  float2* w = reinterpret_cast<float2*>(w_out);
  if (w_out != w_in)
    CFD_CHECK(cudaMemcpyAsync(w_out, w_in, ns * sizeof(float2), cudaMemcpyDeviceToDevice, s),
              "copy");
  const int launches = 1 + steps * plan->stages * 3;
  const bool fused = p.col_mode == 4 && cfd::spec_pipe_ok(p);
  std::vector<cudaEvent_t> ev(2 * launches);
  std::vector<int> kind;
  for (auto& e : ev) CFD_CHECK(cudaEventCreate(&e), "cudaEventCreate");
  int li = 0;
  cudaError_t e = cudaSuccess;
  auto rec = [&](int k, bool start) {
    if (e == cudaSuccess) e = cudaEventRecord(ev[2 * li + (start ? 0 : 1)], s);
    if (!start) {
      kind.push_back(k);
      ++li;
    }
  };
  // The same tiled state as cfd_spec_step (conversions outside the timed launches).
  const bool tiled = fused && plan->wt && cfd::spec_state_tiled_ok(p);
  float2* ws = tiled ? plan->wt : w;
  float2* hs = tiled ? plan->ht : plan->h;
  rec(2, true);
  if (e == cudaSuccess) e = cfd::launch_spec_col_prep(p, w, plan->t4, s);
  rec(2, false);
  if (e == cudaSuccess && tiled) e = cfd::spec_tile_state(p, w, ws, true, s);
  for (int st = 0; st < steps && e == cudaSuccess; ++st) {
    for (int k = 0; k < plan->stages && e == cudaSuccess; ++k) {
      rec(0, true);
      if (e == cudaSuccess) e = cfd::launch_spec_row(p, plan->t4, plan->ahat, s);
      rec(0, false);
      cfd::StageCoef c = plan->coef[k];
      const bool prep = !(st + 1 == steps && k + 1 == plan->stages);
      if (prep && fused) {
        // Update and the next stage's prep in one launch.
        c.prep_next = 1;
        c.tiled = tiled ? 1 : 0;
        rec(3, true);
        if (e == cudaSuccess) e = cfd::launch_spec_col_update(p, c, plan->ahat, ws, hs, plan->t4, s);
        rec(3, false);
        continue;
      }
      c.prep_next = 0;
      c.tiled = tiled ? 1 : 0;
      rec(1, true);
      if (e == cudaSuccess) e = cfd::launch_spec_col_update(p, c, plan->ahat, ws, hs, plan->t4, s);
      rec(1, false);
      if (prep) {
        rec(2, true);
        if (e == cudaSuccess) e = cfd::launch_spec_col_prep(p, w, plan->t4, s);
        rec(2, false);
      }
    }
  }
  if (e == cudaSuccess && tiled) e = cfd::spec_tile_state(p, ws, w, false, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  double sum[4] = {0, 0, 0, 0};
  int cnt[4] = {0, 0, 0, 0};
  for (int i = 0; i < li && e == cudaSuccess; ++i) {
    float ms = 0.f;
    e = cudaEventElapsedTime(&ms, ev[2 * i], ev[2 * i + 1]);
    sum[kind[i]] += ms;
    cnt[kind[i]] += 1;
  }
  for (auto& x : ev) cudaEventDestroy(x);
  if (e != cudaSuccess) return cuda_fail(e, "cfd_spec_profile");
  for (int k = 0; k < 4; ++k) ms_out[k] = cnt[k] ? (float)(sum[k] / cnt[k]) : 0.f;
  return CFD_OK;
}

int cfd_spec_explicit_terms(cfd_spec_plan* plan, void* stream, const float* w,
                            float* out) {
  if (!plan || !w || !out) return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_spec_explicit_terms: null pointer");
  cudaStream_t s = as_stream(stream);
  const cfd::SpecParams& p = plan->p;
  CFD_CHECK(cfd::launch_spec_col_prep(p, reinterpret_cast<const float2*>(w), plan->t4, s),
            "col_prep");
  CFD_CHECK(cfd::launch_spec_row(p, plan->t4, plan->ahat, s), "row");
  cfd::StageCoef c{};
  c.explicit_only = 1;
  CFD_CHECK(cfd::launch_spec_col_update(p, c, plan->ahat, reinterpret_cast<float2*>(out),
                                        plan->h, plan->t4, s),
            "col_update");
  return CFD_OK;
}

// ---- Same-shape spectral batches ---------------------------------------

static void spec_batch_drop_graph(cfd_spec_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
  b->graph_chunk = -1;
}

int cfd_spec_batch_destroy(cfd_spec_batch* b) {
  if (!b) return CFD_OK;
  spec_batch_drop_graph(b);
  void* ptrs[] = {b->slab, b->twy, b->twpx, b->twpy, b->kx, b->ky, b->dev, b->health};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  delete b;
  return CFD_OK;
}

int cfd_spec_batch_create(const cfd_spec_config* shape, int count, cfd_spec_batch** out) {
  if (!shape || !out || count < 1 || count > 65535)
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_spec_batch_create: bad arguments");
  *out = nullptr;
  cfd::SpecParams p;
  cfd::StageCoef coef[8];
  int stages = 0;
  int rc = spec_params_from_config(shape, &p, coef, &stages);
  if (rc) return rc;
  if (p.log2L < 1) return fail(CFD_ERR_UNSUPPORTED, "batched spectral steps need ny >= 4");
  cfd_spec_batch* b = new cfd_spec_batch();
  b->shape = p;
  b->hx = shape->hx;
  b->hy = shape->hy;
  b->stages = stages;
  b->count = count;
  const size_t ns = (size_t)p.nx * (p.L + 1);
  // Each slot's seven buffers (state, h, four fields, advection spectrum) at
  // a stride of nx * pitch values: the fields and the spectrum use rows of
  // p.pitch values, the state and h their first ns values.
  const size_t nsp = (size_t)p.nx * p.pitch;
  b->ns = ns;
  cudaError_t e = cudaMalloc((void**)&b->slab, (size_t)count * 7 * nsp * sizeof(float2));
  if (e == cudaSuccess) e = cudaMemset(b->slab, 0, (size_t)count * 7 * nsp * sizeof(float2));
  if (e == cudaSuccess) e = cudaMalloc((void**)&b->dev, (size_t)count * sizeof(cfd::SpecMember));
  if (e == cudaSuccess) e = cudaMalloc((void**)&b->health, (size_t)count * sizeof(cfd::Health));
  if (e == cudaSuccess) e = cudaMemset(b->health, 0, (size_t)count * sizeof(cfd::Health));
  const SpecTables t = spec_tables(p);
  if (e == cudaSuccess) e = upload(&b->twy, t.twy.data(), t.twy.size());
  if (e == cudaSuccess) e = upload(&b->twpx, t.twpx.data(), t.twpx.size());
  if (e == cudaSuccess) e = upload(&b->twpy, t.twpy.data(), t.twpy.size());
  if (e == cudaSuccess) e = upload(&b->kx, t.kx.data(), t.kx.size());
  if (e == cudaSuccess) e = upload(&b->ky, t.ky.data(), t.ky.size());
  if (e != cudaSuccess) {
    cfd_spec_batch_destroy(b);
    return cuda_fail(e, "cfd_spec_batch_create");
  }
  b->bytes = (long long)count * 7 * (long long)nsp * 8 + (long long)count * sizeof(cfd::SpecMember);
  b->host.assign(count, cfd::SpecMember());
  b->want.assign(count, 0);
  for (int i = 0; i < count; ++i) {
    cfd::SpecMember& m = b->host[i];
    std::memset(&m, 0, sizeof(m));
    m.p = p;
    m.p.tw_y = b->twy;
    m.p.twp_x = b->twpx;
    m.p.twp_y = b->twpy;
    m.p.kx = b->kx;
    m.p.ky = b->ky;
    for (int k = 0; k < stages; ++k) m.coef[k] = coef[k];
    m.stages = stages;
    float2* base = b->slab + (size_t)i * 7 * nsp;
    m.w = base;
    m.h = base + nsp;
    for (int f = 0; f < 4; ++f) m.t[f] = base + (2 + f) * nsp;
    m.ahat = base + 6 * nsp;
    m.steps = 0;
  }
  *out = b;
  return CFD_OK;
}

int cfd_spec_batch_size(const cfd_spec_batch* b) { return b ? b->count : 0; }

long long cfd_spec_batch_bytes(const cfd_spec_batch* b) { return b ? b->bytes : 0; }

int cfd_spec_batch_state(cfd_spec_batch* b, int slot, float** w) {
  if (!b || !w || slot < 0 || slot >= b->count)
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_spec_batch_state: bad arguments");
  *w = reinterpret_cast<float*>(b->host[slot].w);
  return CFD_OK;
}

int cfd_spec_batch_health(cfd_spec_batch* b, const cfd_health** out) {
  if (!b || !out) return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_spec_batch_health: null pointer");
  *out = reinterpret_cast<const cfd_health*>(b->health);
  return CFD_OK;
}

int cfd_spec_batch_set_health_mirror(cfd_spec_batch* b, void* host_records) {
  if (!b) return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_spec_batch_set_health_mirror: null batch");
  cfd::Health* m = nullptr;
  int rc = health_mirror_ptr(host_records, b->count, &m, "cfd_spec_batch_set_health_mirror");
  if (rc) return rc;
  if (m != b->mirror) {
    b->mirror = m;
    spec_batch_drop_graph(b);  // the pointer is part of the captured chunk
  }
  return CFD_OK;
}

int cfd_spec_batch_set_slot(cfd_spec_batch* b, int slot, const cfd_spec_config* cfg,
                            const cfd_spec_plan* forcing) {
  if (!b || !cfg || slot < 0 || slot >= b->count)
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_spec_batch_set_slot: bad arguments");
  if (cfg->nx != b->shape.nx || cfg->ny != b->shape.ny || cfg->hx != b->hx || cfg->hy != b->hy ||
      cfg->num_stages != b->stages)
    return fail(CFD_ERR_INVALID_ARGUMENT,
                "cfd_spec_batch_set_slot: grid, step and stage count must match the batch");
  if (forcing && (forcing->p.nx != b->shape.nx || forcing->p.ny != b->shape.ny))
    return fail(CFD_ERR_INVALID_ARGUMENT,
                "cfd_spec_batch_set_slot: the forcing plan lives on another grid");
  cfd::SpecParams p;
  cfd::StageCoef coef[8];
  int stages = 0;
  int rc = spec_params_from_config(cfg, &p, coef, &stages);
  if (rc) return rc;
  cfd::SpecMember& m = b->host[slot];
  p.tw_y = b->twy;
  p.twp_x = b->twpx;
  p.twp_y = b->twpy;
  p.kx = b->kx;
  p.ky = b->ky;
  p.fc_full = forcing ? forcing->p.fc_full : nullptr;
  p.fc_row0 = forcing ? forcing->p.fc_row0 : nullptr;
  m.p = p;
  for (int k = 0; k < stages; ++k) m.coef[k] = coef[k];
  m.stages = stages;
  b->dirty = true;
  return CFD_OK;
}

int cfd_spec_batch_set_steps(cfd_spec_batch* b, int slot, int steps) {
  if (!b || slot < 0 || slot >= b->count || steps < 0)
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_spec_batch_set_steps: bad arguments");
  if (b->want[slot] != steps) b->dirty = true;
  b->want[slot] = steps;
  return CFD_OK;
}

static int spec_batch_upload(cfd_spec_batch* b, cudaStream_t s, int chunk) {
  if (!b->dirty && b->uploaded_chunk == chunk) return CFD_OK;
  for (int i = 0; i < b->count; ++i) b->host[i].steps = std::min(b->want[i], chunk);
  CFD_CHECK(cudaMemcpyAsync(b->dev, b->host.data(), b->host.size() * sizeof(cfd::SpecMember),
                            cudaMemcpyHostToDevice, s),
            "cfd_spec_batch: slot table");
  b->dirty = false;
  b->uploaded_chunk = chunk;
  return CFD_OK;
}

static int spec_batch_enqueue(cfd_spec_batch* b, cudaStream_t s, int chunk) {
  const cfd::SpecParams& p = b->shape;
  CFD_CHECK(cfd::launch_spec_batch_prep(p, b->dev, b->count, -1, -1, s), "batch prep");
  for (int k = 0; k < chunk; ++k)
    for (int st = 0; st < b->stages; ++st) {
      CFD_CHECK(cfd::launch_spec_batch_row(p, b->dev, b->count, k, s), "batch row");
      CFD_CHECK(cfd::launch_spec_batch_update(p, b->dev, b->count, k, st, s), "batch update");
      CFD_CHECK(cfd::launch_spec_batch_prep(p, b->dev, b->count, k, st, s), "batch prep");
    }
  CFD_CHECK(cfd::launch_spec_batch_health(p, b->dev, b->count, b->health, b->mirror, s),
            "batch health");
  return CFD_OK;
}

int cfd_spec_batch_run(cfd_spec_batch* b, void* stream, int chunk, int use_graph) {
  if (!b || chunk < 0) return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_spec_batch_run: bad arguments");
  if (chunk == 0) return CFD_OK;
  cudaStream_t s = as_stream(stream);
  int rc = spec_batch_upload(b, s, chunk);
  if (rc) return rc;
  if (!use_graph) return spec_batch_enqueue(b, s, chunk);
  if (!b->exec || b->graph_chunk != chunk) {
    spec_batch_drop_graph(b);
    rc = capture_graph([&](cudaStream_t c) { return spec_batch_enqueue(b, c, chunk); },
                       &b->graph, &b->exec);
    if (rc) return rc;
    b->graph_chunk = chunk;
  }
  CFD_CHECK(cudaGraphLaunch(b->exec, s), "cudaGraphLaunch");
  return CFD_OK;
}

// ---- Diagnostics -------------------------------------------------------

int cfd_energy_spectrum_shells(cfd_spec_plan* plan, void* stream, const float* u,
                               const float* v, double dnx, double dny, double ks, int nbins,
                               double* out) {
  if (!plan || !u || !v || !out || nbins < 1 || !(ks > 0))
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_energy_spectrum_shells: bad arguments");
  cudaStream_t s = as_stream(stream);
  float2* uh = plan->t4[0];
  float2* vh = plan->t4[1];
  CFD_CHECK(cfd::launch_row_rfft(plan->p, u, uh, s), "row_rfft");
  CFD_CHECK(cfd::launch_col_fft(plan->p, uh, -1, nullptr, s), "col_fft");
  CFD_CHECK(cfd::launch_row_rfft(plan->p, v, vh, s), "row_rfft");
  CFD_CHECK(cfd::launch_col_fft(plan->p, vh, -1, nullptr, s), "col_fft");
  CFD_CHECK(cfd::launch_shell_energy(plan->p, dnx, dny, ks, nbins, uh, vh, out, s),
            "shell_energy");
  return CFD_OK;
}

int cfd_enstrophy_sum(void* stream, int nx, int ny, double hx, double hy, const float* u,
                      const float* v, double* out) {
  if (!u || !v || !out || nx < 1 || ny < 1 || !(hx > 0) || !(hy > 0))
    return fail(CFD_ERR_INVALID_ARGUMENT, "cfd_enstrophy_sum: bad arguments");
  CFD_CHECK(cfd::launch_enstrophy_sum(nx, ny, (float)hx, (float)hy, u, v, out,
                                      as_stream(stream)),
            "enstrophy_sum");
  return CFD_OK;
}

}  // extern "C"
