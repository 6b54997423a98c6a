// Pressure projection that allocates nothing on the device.
//
// Some callers cannot call cudaMalloc: code that runs while a CUDA graph is
// being captured into a pool they do not own, allocators that forbid
// allocation after start-up (real-time or embedded hosts that reserve all
// device memory up front), and plugin hosts that hand the library only
// pre-allocated input and output buffers.  For them,
// cfd_fvm_projection_noalloc does the same work as cfd_fvm_projection (the
// real-FFT solve_fast_diag pressure projection) without a plan: its scratch
// -- the packed row spectrum / pressure field and the twiddle and Laplacian
// eigenvalue tables -- lives in one file-scope __device__ array of fixed size,
// which every GPU that loads this library holds until the process exits.
//
// Limit: nx * ny <= kNoallocMaxCells (512 * 512 cells), each side a power of
// two in [4, 4096].  The array is shared by every call on a device and keeps
// the previous call's contents; every byte a call reads is written earlier in
// the same call (tables first, then the spectrum), so nothing needs clearing.
// Calls whose work overlaps on the GPU (different streams, or different host
// threads on one device) race on the array; callers must order them.
#include <cmath>
#include <string>

#include "../../include/cfd_gb300.h"
#include "fft.cuh"
#include "wfft.cuh"
#include "kernels.h"

namespace {

constexpr int kNoallocMaxCells = 512 * 512;
constexpr int kNoallocMaxSide = 4096;
// Layout (in floats), each region rounded up to 64 floats: spectrum [nx*ny] |
// tw_y [2*ny] | concatenated pass tables of the column FFT (length nx) and of
// the row FFT (length ny/2), each followed by the one-warp 1024-point table
// when its length is 1024 | lam_x [nx] | lam_y [ny/2 + 1].  A pass table of
// length L holds fewer than L entries, so the bound below covers every shape
// the size check admits (noalloc_layout checks it again per call).
constexpr int kNoallocFloats =
    kNoallocMaxCells + 2 * kNoallocMaxSide + 2 * (kNoallocMaxSide + 1024) +
    2 * (kNoallocMaxSide / 2 + 1024) + kNoallocMaxSide + (kNoallocMaxSide / 2 + 1) + 6 * 64;

__device__ __align__(256) float g_noalloc_scratch[kNoallocFloats];

int round64(int n) { return (n + 63) & ~63; }

// Entries of the concatenated pass tables of a length-2^log2L FFT (layout in
// fft.cuh), followed, for length 1024, by the one-warp transform's table
// (wfft.cuh: entry [k2 * 32 + n1] = exp(-2 pi i n1 k2 / 1024)).
__host__ __device__ int table_entries(int log2L) {
  return cfd::fft_pass_table_size(log2L) + cfd::wfft_table_size(log2L);
}

// Angle numerator/denominator of entry `idx` of table_entries(log2L): the
// entry is exp(-2 pi i num / den).
__device__ void pass_entry(int log2L, int idx, int* num, int* den) {
  const int stockham = cfd::fft_pass_table_size(log2L);
  if (idx >= stockham) {
    const int w = idx - stockham;
    *num = (w & 31) * (w >> 5);
    *den = 1024;
    return;
  }
  int ns = 1;
  for (int q = 0; q < cfd::fft_num_passes(log2L); ++q) {
    const int R = cfd::fft_pass_radix(log2L, q);
    if (ns > 1) {
      const int size = (R - 1) * ns;
      if (idx < size) {
        *num = (idx / ns + 1) * (idx % ns);
        *den = ns * R;
        return;
      }
      idx -= size;
    }
    ns *= R;
  }
  *num = 0;
  *den = 1;
}

// Twiddles and Laplacian eigenvalues (2 cos(2 pi k / n) - 2) / h^2
// (array_utils.py:168-173, the fft of the circulant's first column), in double
// precision with sincospi/cospi, rounded once to float.
__global__ void noalloc_tables_kernel(int nx, int ny, double hx, double hy,
                                      float2* tw_y, float2* twp_x, float2* twp_y,
                                      float* lam_x, float* lam_y) {
  const int log2nx = ilog2(nx), log2L = ilog2(ny) - 1;
  const int sx = table_entries(log2nx), sy = table_entries(log2L);
  const int total = ny + sx + sy + nx + (ny / 2 + 1);
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += gridDim.x * blockDim.x) {
    double s, c;
    if (t < ny) {
      sincospi(-2.0 * t / ny, &s, &c);
      tw_y[t] = make_float2((float)c, (float)s);
    } else if (t < ny + sx) {
      int num, den;
      pass_entry(log2nx, t - ny, &num, &den);
      sincospi(-2.0 * num / den, &s, &c);
      twp_x[t - ny] = make_float2((float)c, (float)s);
    } else if (t < ny + sx + sy) {
      int num, den;
      pass_entry(log2L, t - ny - sx, &num, &den);
      sincospi(-2.0 * num / den, &s, &c);
      twp_y[t - ny - sx] = make_float2((float)c, (float)s);
    } else if (t < ny + sx + sy + nx) {
      const int k = t - ny - sx - sy;
      lam_x[k] = k == 0 ? 0.f : (float)((2.0 * cospi(2.0 * k / nx) - 2.0) / (hx * hx));
    } else {
      const int k = t - ny - sx - sy - nx;
      lam_y[k] = k == 0 ? 0.f : (float)((2.0 * cospi(2.0 * k / ny) - 2.0) / (hy * hy));
    }
  }
}

int noalloc_fail(int code, const std::string& msg) {
  cfd::set_last_error(msg);
  return code;
}

// Device address of the scratch array in the current device's context.  Host
// code may not use the array's name as a device pointer, so every call looks
// the address up with cudaGetSymbolAddress (cheap; an address cached across
// calls would go stale when the context is destroyed and re-created, e.g.
// after cudaDeviceReset, which reloads the module).
int noalloc_scratch(float** out) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p)
    return noalloc_fail(CFD_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  *out = static_cast<float*>(p);
  return CFD_OK;
}

// Float offsets of the scratch regions for an nx x ny grid; false if they do
// not fit the array.
struct NoallocLayout {
  int tw_y, twp_x, twp_y, lam_x, lam_y, end;
};
bool noalloc_layout(int nx, int ny, NoallocLayout* l) {
  l->tw_y = round64(nx * ny);
  l->twp_x = l->tw_y + round64(2 * ny);
  l->twp_y = l->twp_x + round64(2 * table_entries(ilog2(nx)));
  l->lam_x = l->twp_y + round64(2 * table_entries(ilog2(ny) - 1));
  l->lam_y = l->lam_x + round64(nx);
  l->end = l->lam_y + round64(ny / 2 + 1);
  return l->end <= kNoallocFloats;
}

}  // namespace

extern "C" int cfd_fvm_projection_noalloc(void* stream, int nx, int ny, double hx,
                                          double hy, const float* u, const float* v,
                                          float* u_out, float* v_out) {
  if (!u || !v || !u_out || !v_out)
    return noalloc_fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_projection_noalloc: null pointer");
  if (!is_pow2(nx) || !is_pow2(ny) || nx < 4 || ny < 4 || nx > kNoallocMaxSide ||
      ny > kNoallocMaxSide)
    return noalloc_fail(CFD_ERR_INVALID_ARGUMENT,
                        "cfd_fvm_projection_noalloc: nx and ny must be powers of two in [4, 4096]");
  if ((long long)nx * ny > kNoallocMaxCells)
    return noalloc_fail(CFD_ERR_INVALID_ARGUMENT,
                        "cfd_fvm_projection_noalloc: nx * ny exceeds the static scratch limit of "
                        "262144 cells (512 x 512); use cfd_fvm_projection with a plan");
  if (!(hx > 0) || !(hy > 0))
    return noalloc_fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_projection_noalloc: invalid grid step");
  float* base = nullptr;
  int rc = noalloc_scratch(&base);
  if (rc != CFD_OK) return rc;

  NoallocLayout lay;
  if (!noalloc_layout(nx, ny, &lay))
    return noalloc_fail(CFD_ERR_INVALID_ARGUMENT, "cfd_fvm_projection_noalloc: scratch layout exceeds the array");
  float* spec = base;
  float2* tw_y = reinterpret_cast<float2*>(base + lay.tw_y);
  float2* twp_x = reinterpret_cast<float2*>(base + lay.twp_x);
  float2* twp_y = reinterpret_cast<float2*>(base + lay.twp_y);
  float* lam_x = base + lay.lam_x;
  float* lam_y = base + lay.lam_y;

  cfd::FvmParams p{};
  p.nx = nx;
  p.ny = ny;
  p.log2nx = ilog2(nx);
  p.log2ny = ilog2(ny);
  p.hx = (float)hx;
  p.hy = (float)hy;
  p.inv_hx = 1.f / p.hx;
  p.inv_hy = 1.f / p.hy;
  p.cutoff = 10.f * 1.1920928955078125e-07f;
  p.pinv_scale = 1.f / ((float)nx * (float)ny);
  p.lamx = lam_x;
  p.lamy = lam_y;
  p.tw_y = tw_y;
  p.twp_x = twp_x;
  p.twp_y = twp_y;

  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int total = ny + table_entries(p.log2nx) + table_entries(p.log2ny - 1) + nx + ny / 2 + 1;
  noalloc_tables_kernel<<<(total + 255) / 256, 256, 0, s>>>(nx, ny, hx, hy, tw_y, twp_x,
                                                            twp_y, lam_x, lam_y);
  cudaError_t e = cudaGetLastError();
  float2* sp = reinterpret_cast<float2*>(spec);
  if (e == cudaSuccess) e = cfd::launch_fvm_div_rfft(p, u, v, sp, s);
  if (e == cudaSuccess) e = cfd::launch_fvm_col_pinv(p, sp, s);
  if (e == cudaSuccess) e = cfd::launch_fvm_irfft(p, sp, s);
  if (e == cudaSuccess) e = cfd::launch_fvm_project_out(p, u, v, spec, u_out, v_out, s);
  if (e != cudaSuccess)
    return noalloc_fail(CFD_ERR_CUDA, std::string("cfd_fvm_projection_noalloc: ") + cudaGetErrorString(e));
  return CFD_OK;
}
