// Staggered MAC-grid (FVM) kernels: the explicit Van Leer/diffusion/forcing
// stencil, and the real-FFT fast-diagonalisation pressure projection.
//
// One forward-Euler step of semi_implicit_navier_stokes
// (jax_cfd/base/equations.py:120-151, time_stepping.py:59-119) runs as
//   explicit   (u, v) [or (u*, v*, q) projected on the fly] -> (u*, v*)
//   div_rfft   (u*, v*) -> D^ rows            (backward-difference divergence
//                                              + real FFT along contiguous y)
//   col_pinv   D^ -> q^ (FFT along x, * pinv(lambda), inverse FFT along x)
//   irfft      q^ -> q  (inverse real FFT along y, in place)
// and the projection u = u* - forward_difference(q) is folded into the next
// step's stencil load, or into project_out at the end of a chunk.
//
// The half spectrum of a row of M reals is stored "packed" as M/2 complex
// numbers: element 0 holds (X[0], X[M/2]), both real.  The x-axis transforms
// of the DC and Nyquist columns run as two separate real sequences.
#include <cooperative_groups.h>
#include <cuda.h>

#include "bulk.cuh"
#include "colpipe.cuh"
#include "fft.cuh"
#include "kernels.h"
#include "wfft.cuh"

namespace cg = cooperative_groups;

namespace cfd {
namespace {

constexpr int kTI = 16;   // stencil tile rows (x)
constexpr int kTJ = 64;   // stencil tile columns (y, contiguous)
constexpr int kStencilThreads = 256;

// One face value of apply_tvd_limiter(lax_wendroff, van_leer_limiter) times
// the face velocity: interpolation.py:96-303 specialised to a forward
// half-cell interpolation with stencil c[-1], c[0], c[+1], c[+2] along the
// face normal and face velocity U.  The reference computes
//   upwind        c_low  = U > 0 ? c0 : c1
//   lax_wendroff  c_high = U > 0 ? c0 + 0.5(1-C)(c1-c0) : c1 - 0.5(1+C)(c1-c0)
//   ratio         r = safe_div(U > 0 ? c0-cm : c2-c1, c1-c0)
//   van Leer      phi = r > 0 ? 2r / (1+r) : 0
//   face value    c_low - (c_low - c_high) * phi
// In upwind-mirrored variables (a, b, c) = U > 0 ? (cm, c0, c1) : (c2, c1, c0)
// this is c_low = b, c_high = b + 0.5(1 - |C|)(c - b) and r = (b - a)/(c - b):
// both branches round exactly as above (the mirrored forms differ from them
// only by exact negations).  2r/(1+r) = 2 num / (den + num) with num = b - a,
// den = c - b, and r > 0 exactly when num * den > 0 (up to underflow of the
// product), so the limiter costs one approximate division.  Where c - b == 0
// the reference divides by 1 instead; there c_high - c_low is exactly 0, so
// phi does not change the face value.
CFD_D float tvd_flux(float cm, float c0, float c1, float c2, float U,
                     float cfl) {
  const bool pos = U > 0.f;
  const float a = pos ? cm : c2, b = pos ? c0 : c1, c = pos ? c1 : c0;
  const float C = cfl * U;
  const float diff = c - b;
  const float c_high = b + (0.5f * (1.f - fabsf(C))) * diff;
  const float num = b - a;
  const float phi = num * diff > 0.f ? __fdividef(num + num, diff + num) : 0.f;
  const float cf = b + (c_high - b) * phi;
  return cf * U;
}

template <bool PROJECT, bool OUT_K0, int CONVECT>
__global__ void __launch_bounds__(kStencilThreads)
    fvm_explicit_kernel(FvmParams p, const float* __restrict__ ua,
                        const float* __restrict__ va,
                        const float* __restrict__ q, float* __restrict__ uo,
                        float* __restrict__ vo) {
  __shared__ float su[kTI + 4][kTJ + 4];
  __shared__ float sv[kTI + 4][kTJ + 4];
  __shared__ float sq[PROJECT ? kTI + 5 : 1][PROJECT ? kTJ + 5 : 1];
  __shared__ float fx[kTI + 1][kTJ];  // x-face flux of u (offset 1.5, .5)
  __shared__ float gx[kTI + 1][kTJ];  // x-face flux of v (offset 1, 1)
  __shared__ float fy[kTI][kTJ + 1];  // y-face flux of u (offset 1, 1)
  __shared__ float gy[kTI][kTJ + 1];  // y-face flux of v (offset .5, 1.5)

  const int ti = min(kTI, p.nx), tj = min(kTJ, p.ny);
  const int i0 = blockIdx.y * ti, j0 = blockIdx.x * tj;
  const int mx = p.nx - 1, my = p.ny - 1;
  const int tid = threadIdx.x;
  const size_t ny = (size_t)p.ny;

  if (PROJECT) {
    // q on rows i0-2 .. i0+ti+2, columns j0-2 .. j0+tj+2.
    const int bi = ti + 5, bj = tj + 5;
    for (int idx = tid; idx < bi * bj; idx += kStencilThreads) {
      const int a = idx / bj, b = idx - a * bj;
      const int i = (i0 - 2 + a) & mx, j = (j0 - 2 + b) & my;
      sq[a][b] = __ldg(q + i * ny + j);
    }
    __syncthreads();
  }
  {
    // u, v on rows i0-2 .. i0+ti+1, columns j0-2 .. j0+tj+1.  With PROJECT,
    // u = u* - (q[i+1] - q[i]) / hx and v = v* - (q[j+1] - q[j]) / hy
    // (pressure.py:193-196, finite_differences.py:117-124).
    const int bi = ti + 4, bj = tj + 4;
    for (int idx = tid; idx < bi * bj; idx += kStencilThreads) {
      const int a = idx / bj, b = idx - a * bj;
      const int i = (i0 - 2 + a) & mx, j = (j0 - 2 + b) & my;
      float u = __ldg(ua + i * ny + j);
      float v = __ldg(va + i * ny + j);
      if (PROJECT) {
        u = u - (sq[a + 1][b] - sq[a][b]) * p.inv_hx;
        v = v - (sq[a][b + 1] - sq[a][b]) * p.inv_hy;
      }
      su[a][b] = u;
      sv[a][b] = v;
    }
  }
  __syncthreads();

  // Faces normal to x: face a sits after cell i = i0 - 1 + a (box row a + 1).
  for (int idx = tid; idx < (ti + 1) * tj; idx += kStencilThreads) {
    const int a = idx / tj, b = idx - a * tj;
    const int c = b + 2;
    // u's control volume: velocity 0.5 u[i] + 0.5 u[i+1] (interpolation.linear).
    const float U = 0.5f * su[a + 1][c] + 0.5f * su[a + 2][c];
    // v's control volume: u interpolated along y to (1, 1).
    const float Uv = 0.5f * su[a + 1][c] + 0.5f * su[a + 1][c + 1];
    if (CONVECT == 0) {
      fx[a][b] = tvd_flux(su[a][c], su[a + 1][c], su[a + 2][c], su[a + 3][c],
                          U, p.cfl_x);
      gx[a][b] = tvd_flux(sv[a][c], sv[a + 1][c], sv[a + 2][c], sv[a + 3][c],
                          Uv, p.cfl_x);
    } else {
      fx[a][b] = U * U;
      gx[a][b] = (0.5f * sv[a + 1][c] + 0.5f * sv[a + 2][c]) * Uv;
    }
  }
  // Faces normal to y: face b sits after cell j = j0 - 1 + b (box col b + 1).
  for (int idx = tid; idx < ti * (tj + 1); idx += kStencilThreads) {
    const int a = idx / (tj + 1), b = idx - a * (tj + 1);
    const int r = a + 2;
    // u's control volume: v interpolated along x to (1, 1).
    const float V = 0.5f * sv[r][b + 1] + 0.5f * sv[r + 1][b + 1];
    // v's control volume: 0.5 v[j] + 0.5 v[j+1].
    const float Vv = 0.5f * sv[r][b + 1] + 0.5f * sv[r][b + 2];
    if (CONVECT == 0) {
      fy[a][b] = tvd_flux(su[r][b], su[r][b + 1], su[r][b + 2], su[r][b + 3],
                          V, p.cfl_y);
      gy[a][b] = tvd_flux(sv[r][b], sv[r][b + 1], sv[r][b + 2], sv[r][b + 3],
                          Vv, p.cfl_y);
    } else {
      fy[a][b] = (0.5f * su[r][b + 1] + 0.5f * su[r][b + 2]) * V;
      gy[a][b] = Vv * Vv;
    }
  }
  __syncthreads();

  // Cell updates (equations.py:102-110, time_stepping.py:89-105).
  for (int idx = tid; idx < ti * tj; idx += kStencilThreads) {
    const int a = idx / tj, b = idx - a * tj;
    const int r = a + 2, c = b + 2;
    const int i = i0 + a, j = j0 + b;
    const float u = su[r][c], v = sv[r][c];
    // -divergence(flux): -((F[i] - F[i-1]) / hx + (F[j] - F[j-1]) / hy)
    float ku = -((fx[a + 1][b] - fx[a][b]) * p.inv_hx +
                 (fy[a][b + 1] - fy[a][b]) * p.inv_hy);
    float kv = -((gx[a + 1][b] - gx[a][b]) * p.inv_hx +
                 (gy[a][b + 1] - gy[a][b]) * p.inv_hy);
    if (p.has_visc) {
      // finite_differences.laplacian: -2c * sum(scales) + pairs * scale
      const float lu = ((-2.f * u) * p.ssum + (su[r - 1][c] + su[r + 1][c]) * p.sx) +
                       (su[r][c - 1] + su[r][c + 1]) * p.sy;
      const float lv = ((-2.f * v) * p.ssum + (sv[r - 1][c] + sv[r + 1][c]) * p.sx) +
                       (sv[r][c - 1] + sv[r][c + 1]) * p.sy;
      ku = ku + p.nu * lu;
      kv = kv + p.nu * lv;
    }
    if (p.has_forcing) {
      // sum_forcings(linear, constant): (0 + lin * u) + const
      float fu = 0.f, fv = 0.f;
      bool any_u = false, any_v = false;
      if (p.has_lin) {
        fu = p.lin * u;
        fv = p.lin * v;
        any_u = any_v = true;
      }
      if (p.fu_y) { fu = any_u ? fu + __ldg(p.fu_y + j) : __ldg(p.fu_y + j); any_u = true; }
      if (p.fv_x) { fv = any_v ? fv + __ldg(p.fv_x + i) : __ldg(p.fv_x + i); any_v = true; }
      if (p.fu_full) { const float f = __ldg(p.fu_full + i * ny + j); fu = any_u ? fu + f : f; any_u = true; }
      if (p.fv_full) { const float f = __ldg(p.fv_full + i * ny + j); fv = any_v ? fv + f : f; any_v = true; }
      if (!p.rho_is_one) {
        fu = fu / p.density;
        fv = fv / p.density;
      }
      if (any_u) ku = ku + fu;
      if (any_v) kv = kv + fv;
    }
    if (OUT_K0) {
      uo[i * ny + j] = ku;
      vo[i * ny + j] = kv;
    } else {
      uo[i * ny + j] = u + p.dt * ku;
      vo[i * ny + j] = v + p.dt * kv;
    }
  }
}

// Paired float32 arithmetic (sm_100+ f32x2 instructions): the u- and
// v-components of a face or cell run the same operation sequence, so they are
// packed as (u, v) pairs.  Each paired op rounds exactly like its scalar form.
CFD_D float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
CFD_D float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
CFD_D float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// a - b is a + (-b) exactly (IEEE subtraction is the addition of the
// negation), so the paired add of the negation rounds like two subtractions.
CFD_D float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
CFD_D float2 splat2(float a) { return make_float2(a, a); }
CFD_D float2 sel2(bool px, bool py, float2 a, float2 b) {
  return make_float2(px ? a.x : b.x, py ? a.y : b.y);
}

// Viscosity and forcing of one cell, added to the paired explicit terms kk:
// kk + nu lap(u) then + sum_forcings(linear, constant) / density, in the
// reference's order (equations.py:102-110, forcings.py:125-178).  FORCE = 1
// is the configuration of simple_turbulence_forcing (viscosity, linear drag
// and a u-forcing over y, density 1) with its flags resolved at compile time;
// FORCE = 0 reads them at run time.  Both evaluate the same expressions.
template <int FORCE>
CFD_D float2 add_diffusion_forcing(const FvmParams& p, float2 kk, float2 uv, float2 lx,
                                   float2 ly, int i, int j) {
  if (FORCE == 1 || p.has_visc) {
    // finite_differences.laplacian: -2c * sum(scales) + pairs * scale
    const float2 m2 = mul2(splat2(-2.f), uv);
    float2 lap = fma2(lx, splat2(p.sx), mul2(m2, splat2(p.ssum)));
    lap = fma2(ly, splat2(p.sy), lap);
    kk = fma2(splat2(p.nu), lap, kk);
  }
  if (FORCE == 1) {
    const float fu = p.lin * uv.x + __ldg(p.fu_y + j);
    const float fv = p.lin * uv.y;
    return make_float2(kk.x + fu, kk.y + fv);
  }
  if (p.has_forcing) {
    const size_t ny = (size_t)p.ny;
    float fu = 0.f, fv = 0.f;
    bool any_u = false, any_v = false;
    if (p.has_lin) {
      fu = p.lin * uv.x;
      fv = p.lin * uv.y;
      any_u = any_v = true;
    }
    if (p.fu_y) { fu = any_u ? fu + __ldg(p.fu_y + j) : __ldg(p.fu_y + j); any_u = true; }
    if (p.fv_x) { fv = any_v ? fv + __ldg(p.fv_x + i) : __ldg(p.fv_x + i); any_v = true; }
    if (p.fu_full) { const float f = __ldg(p.fu_full + i * ny + j); fu = any_u ? fu + f : f; any_u = true; }
    if (p.fv_full) { const float f = __ldg(p.fv_full + i * ny + j); fv = any_v ? fv + f : f; any_v = true; }
    if (!p.rho_is_one) {
      fu = fu / p.density;
      fv = fv / p.density;
    }
    if (any_u) kk.x = kk.x + fu;
    if (any_v) kk.y = kk.y + fv;
  }
  return kk;
}

// add_diffusion_forcing<1> with the Kolmogorov table value fu_y[j] passed in
// (loaded once per column by the streaming kernels): the same expressions.
template <int FORCE>
CFD_D float2 add_diffusion_forcing_fu(const FvmParams& p, float2 kk, float2 uv, float2 lx,
                                      float2 ly, float fuy) {
  static_assert(FORCE == 1, "simple_turbulence_forcing configuration only");
  const float2 m2 = mul2(splat2(-2.f), uv);
  float2 lap = fma2(lx, splat2(p.sx), mul2(m2, splat2(p.ssum)));
  lap = fma2(ly, splat2(p.sy), lap);
  kk = fma2(splat2(p.nu), lap, kk);
  const float fu = p.lin * uv.x + fuy;
  const float fv = p.lin * uv.y;
  return make_float2(kk.x + fu, kk.y + fv);
}

// Whether FORCE = 1 applies.
CFD_HD bool kolmogorov_config(const FvmParams& p) {
  return p.has_visc && p.has_forcing && p.has_lin && p.fu_y && !p.fv_x && !p.fu_full &&
         !p.fv_full && p.rho_is_one;
}

// Van Leer face values of two faces at once (tvd_flux in paired arithmetic).
CFD_D float2 tvd_flux2(float2 cm, float2 c0, float2 c1, float2 c2, float2 U,
                       float cfl) {
  const bool px = U.x > 0.f, py = U.y > 0.f;
  const float2 a = sel2(px, py, cm, c2), b = sel2(px, py, c0, c1),
               c = sel2(px, py, c1, c0);
  const float2 C = mul2(splat2(cfl), U);
  const float2 diff = sub2(c, b);
  const float2 t = mul2(splat2(0.5f), make_float2(1.f - fabsf(C.x), 1.f - fabsf(C.y)));
  const float2 c_high = fma2(t, diff, b);
  const float2 num = sub2(b, a);
  const float2 prod = mul2(num, diff);
  const float2 n2 = add2(num, num), dn = add2(diff, num);
  const float2 phi = make_float2(prod.x > 0.f ? __fdividef(n2.x, dn.x) : 0.f,
                                 prod.y > 0.f ? __fdividef(n2.y, dn.y) : 0.f);
  const float2 cf = fma2(sub2(c_high, b), phi, b);
  return mul2(cf, U);
}

// The step for grids whose shape is a multiple of the 16 x 64 tile, with
// compile-time tile geometry: the halo box (rows i0-2 .. i0+17, columns
// j0-4 .. j0+67) is loaded with aligned float4 reads (a 4-column group never
// straddles the periodic seam because ny is a multiple of 4) and stored
// interleaved as (u, v) pairs; face fluxes are computed once per face, for the
// u- and v-control volumes together, into paired shared arrays; each thread
// then updates 4 cells of one column.
constexpr int kBoxW = kTJ + 8;  // 72 columns: j0-4 .. j0+67
template <bool PROJECT, bool OUT_K0, int CONVECT, int FORCE = 0>
CFD_D void explicit_tile(const FvmParams& p, int bx, int by,
                         const float* __restrict__ ua, const float* __restrict__ va,
                         const float* __restrict__ q, float* __restrict__ uo,
                         float* __restrict__ vo) {
  __shared__ __align__(16) float2 sw[kTI + 4][kBoxW];  // (u, v)
  __shared__ __align__(16) float sq[PROJECT ? kTI + 5 : 1][PROJECT ? kBoxW : 4];
  __shared__ float2 fxg[kTI + 1][kTJ];  // x-normal faces: (F, G)
  __shared__ float2 fyg[kTI][kTJ + 1];  // y-normal faces: (F, G)

  const int i0 = by * kTI, j0 = bx * kTJ;
  const int mx = p.nx - 1, my = p.ny - 1;
  const int tid = threadIdx.x;
  const size_t ny = (size_t)p.ny;
  constexpr int kV4 = kBoxW / 4;  // float4 groups per box row

  if (PROJECT) {
    for (int idx = tid; idx < (kTI + 5) * kV4; idx += kStencilThreads) {
      const int a = idx / kV4, k = idx - a * kV4;
      const int i = (i0 - 2 + a) & mx, j = (j0 - 4 + 4 * k) & my;
      *reinterpret_cast<float4*>(&sq[a][4 * k]) =
          __ldg(reinterpret_cast<const float4*>(q + i * ny + j));
    }
    __syncthreads();
  }
  for (int idx = tid; idx < (kTI + 4) * kV4; idx += kStencilThreads) {
    const int a = idx / kV4, k = idx - a * kV4;
    const int i = (i0 - 2 + a) & mx, j = (j0 - 4 + 4 * k) & my;
    float4 u = __ldg(reinterpret_cast<const float4*>(ua + i * ny + j));
    float4 v = __ldg(reinterpret_cast<const float4*>(va + i * ny + j));
    if (PROJECT) {
      // u = u* - (q[i+1] - q[i]) / hx ; v = v* - (q[j+1] - q[j]) / hy
      const int c = 4 * k;
      const float q0 = sq[a][c], q1 = sq[a][c + 1], q2 = sq[a][c + 2], q3 = sq[a][c + 3];
      const float q4 = sq[a][c + 4 < kBoxW ? c + 4 : c + 3];
      u.x = u.x - (sq[a + 1][c] - q0) * p.inv_hx;
      u.y = u.y - (sq[a + 1][c + 1] - q1) * p.inv_hx;
      u.z = u.z - (sq[a + 1][c + 2] - q2) * p.inv_hx;
      u.w = u.w - (sq[a + 1][c + 3] - q3) * p.inv_hx;
      v.x = v.x - (q1 - q0) * p.inv_hy;
      v.y = v.y - (q2 - q1) * p.inv_hy;
      v.z = v.z - (q3 - q2) * p.inv_hy;
      v.w = v.w - (q4 - q3) * p.inv_hy;  // last group unused (box column 71)
    }
    float4* dst = reinterpret_cast<float4*>(&sw[a][4 * k]);
    dst[0] = make_float4(u.x, v.x, u.y, v.y);
    dst[1] = make_float4(u.z, v.z, u.w, v.w);
  }
  __syncthreads();

  const int b = tid & (kTJ - 1);
  const int w = tid >> 6;  // 0..3
  // x-normal faces: face a follows cell i0 - 1 + a (box row a + 1), a < 17.
  // u's control volume: face velocity 0.5 u[i] + 0.5 u[i+1];
  // v's control volume: u interpolated along y, 0.5 u[j] + 0.5 u[j+1].
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const int a = w + 4 * k;
    if (a <= kTI) {
      const int c = b + 4;
      const float2 cm = sw[a][c], c0 = sw[a + 1][c], c1 = sw[a + 2][c], c2 = sw[a + 3][c];
      const float uy1 = sw[a + 1][c + 1].x;
      const float2 U = mul2(splat2(0.5f), add2(splat2(c0.x), make_float2(c1.x, uy1)));
      if (CONVECT == 0) {
        fxg[a][b] = tvd_flux2(cm, c0, c1, c2, U, p.cfl_x);
      } else {
        // flux = c_face * U with c_face = linear interpolation of (u, v)
        const float2 cface = mul2(splat2(0.5f), add2(c0, c1));
        fxg[a][b] = mul2(make_float2(U.x, cface.y), make_float2(U.x, U.y));
      }
    }
  }
  // y-normal faces: face f follows cell j0 - 1 + f (box column f + 3), f < 65;
  // columns f = 0..63 by all threads, f = 64 by the first 16 threads.
  // u's control volume: v interpolated along x, 0.5 v[i] + 0.5 v[i+1];
  // v's control volume: 0.5 v[j] + 0.5 v[j+1].
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    int a, f;
    if (k < 4) {
      a = w + 4 * k;
      f = b;
    } else {
      if (tid >= kTI) break;
      a = tid;
      f = kTJ;
    }
    const int r = a + 2, c = f + 3;
    const float2 cm = sw[r][c - 1], c0 = sw[r][c], c1 = sw[r][c + 1], c2 = sw[r][c + 2];
    const float vx1 = sw[r + 1][c].y;
    const float2 V = mul2(splat2(0.5f), add2(splat2(c0.y), make_float2(vx1, c1.y)));
    if (CONVECT == 0) {
      fyg[a][f] = tvd_flux2(cm, c0, c1, c2, V, p.cfl_y);
    } else {
      const float2 cface = mul2(splat2(0.5f), add2(c0, c1));
      fyg[a][f] = mul2(make_float2(cface.x, V.y), make_float2(V.x, V.y));
    }
  }
  __syncthreads();

  const float2 ihx = splat2(p.inv_hx), ihy = splat2(p.inv_hy);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int a = w + 4 * k;
    const int r = a + 2, c = b + 4;
    const int i = i0 + a, j = j0 + b;
    const float2 uv = sw[r][c];
    // -divergence(flux): -((F[i] - F[i-1]) / hx + (F[j] - F[j-1]) / hy)
    const float2 dx = mul2(sub2(fxg[a + 1][b], fxg[a][b]), ihx);
    float2 kk = fma2(sub2(fyg[a][b + 1], fyg[a][b]), ihy, dx);
    kk = make_float2(-kk.x, -kk.y);
    kk = add_diffusion_forcing<FORCE>(p, kk, uv, add2(sw[r - 1][c], sw[r + 1][c]),
                                      add2(sw[r][c - 1], sw[r][c + 1]), i, j);
    if (OUT_K0) {
      uo[i * ny + j] = kk.x;
      vo[i * ny + j] = kk.y;
    } else {
      const float2 nxt = fma2(splat2(p.dt), kk, uv);
      uo[i * ny + j] = nxt.x;
      vo[i * ny + j] = nxt.y;
    }
  }
}

template <bool PROJECT, bool OUT_K0, int CONVECT, int FORCE>
__global__ void __launch_bounds__(kStencilThreads)
    fvm_explicit_tiled_kernel(FvmParams p, const float* __restrict__ ua,
                              const float* __restrict__ va,
                              const float* __restrict__ q,
                              float* __restrict__ uo, float* __restrict__ vo) {
  explicit_tile<PROJECT, OUT_K0, CONVECT, FORCE>(p, blockIdx.x, blockIdx.y, ua, va, q, uo,
                                                 vo);
}

// ---- Warp-streaming stencil ------------------------------------------------
// The same step as explicit_tile with no shared memory and no block barrier:
// a warp owns a strip of columns and walks down its rows with a window of
// projected (u, v) rows in registers, carrying the previous x-face flux;
// along y the neighbours' values and the left y-face flux come from warp
// shuffles.  Every expression is the one explicit_tile evaluates, in the same
// order, so the two kernels produce identical bits.
constexpr unsigned kFull = 0xffffffffu;

CFD_D float2 shfl_down2(float2 x, int d) {
  return make_float2(__shfl_down_sync(kFull, x.x, d), __shfl_down_sync(kFull, x.y, d));
}
CFD_D float2 shfl_up2(float2 x, int d) {
  return make_float2(__shfl_up_sync(kFull, x.x, d), __shfl_up_sync(kFull, x.y, d));
}

// x-face flux pair (F, G) after row a: window rows a-1, a, a+1, a+2 and u at
// (a, j + 1) for v's control volume.
template <int CONVECT>
CFD_D float2 stream_xface(const FvmParams& p, float2 cm, float2 c0, float2 c1, float2 c2,
                          float uy1) {
  const float2 U = mul2(splat2(0.5f), add2(splat2(c0.x), make_float2(c1.x, uy1)));
  if (CONVECT == 0) return tvd_flux2(cm, c0, c1, c2, U, p.cfl_x);
  const float2 cface = mul2(splat2(0.5f), add2(c0, c1));
  return mul2(make_float2(U.x, cface.y), make_float2(U.x, U.y));
}

// ---- Paired-column warp streams ---------------------------------------------
// Two adjacent columns per lane: lane L holds columns jl = j0 - 2 + 2L and
// jl + 1 (j0 = 60 s for strip s), so a warp covers 64 columns of which lanes
// 1..30 produce 60 (lane 0's first y-face lacks its left stencil column,
// lane 31's last its right one).  Rows are fetched as float2 pairs (jl is
// even, so the pairs are 8-byte aligned), results stored as float2 pairs,
// and a lane's second column takes its left neighbour, its x-face velocity
// and its left y-face flux from the lane's own first column: half the
// shuffles and a third of the loads per cell of one column per lane (which
// measured 33.1 against 30.7 us at 2048^2).  Each column evaluates exactly
// the expressions of explicit_tile.
constexpr int kStreamCols = 60;
// Rows per warp and prefetch depth.  A warp fetches SH + 4 rows for SH
// outputs, so the rows per warp trade halo re-reads against warps in flight;
// plans run 16, 8 and 32 (FvmParams::stream_rows, an autotuner dimension).
// The kernel is issue-bound, and registers set the warps in flight: with a
// prefetch of 2 rows the projecting Kolmogorov-forcing kernel (PROJECT,
// FORCE = 1: every step of a chunk but the first) fits 80 registers without
// spills, six 128-thread blocks (24 warps) per multiprocessor (the other
// variants would spill there and keep the compiler's choice).  2048^2 step (stencil): 63.7 us
// (29.4) at 8 rows per warp, 64.6 (30.9) at 16, against 65.0 (31.1) for the
// earlier 4-row prefetch at 94 registers (20 warps); the 4-row prefetch held
// to 80 registers spills (65.5), 72 registers (28 warps) spill too (65.4).
// Also measured slower: 24 rows per warp (one wave of warps at 2048^2, the
// last warp of a strip taking the remaining rows), 33.4 against 31.4 us; 64
// registers (32 warps), 32.5 against 30.7; one column per lane, 33.1.
constexpr int kStreamRows = 16, kStreamPrefetch = 2;
constexpr int kStreamBlocksPerSM = 6;
// The batched stream (run-time forcing flags, no register cap) keeps the
// 4-row prefetch it was measured with.
constexpr int kBatchStreamPrefetch = 4;
CFD_HD int stream_rows_of(int mode) { return mode == 1 ? 8 : mode == 2 ? 32 : kStreamRows; }

struct StreamRaw {
  float2 u, v, q;  // columns (jl, jl + 1)
  float qr;        // q at column jl + 2
};

template <bool PROJECT>
CFD_D StreamRaw stream_fetch(const FvmParams& p, const float* __restrict__ ua,
                               const float* __restrict__ va, const float* __restrict__ q,
                               int row, int j, int jr) {
  const unsigned base = (unsigned)(row & (p.nx - 1)) << p.log2ny;
  StreamRaw r;
  r.u = __ldg(reinterpret_cast<const float2*>(ua + base + j));
  r.v = __ldg(reinterpret_cast<const float2*>(va + base + j));
  r.q = PROJECT ? __ldg(reinterpret_cast<const float2*>(q + base + j)) : make_float2(0.f, 0.f);
  r.qr = PROJECT ? __ldg(q + base + jr) : 0.f;
  return r;
}

// Projected (u, v) of both columns; qn: q of the next row.
template <bool PROJECT>
CFD_D void stream_project(const FvmParams& p, const StreamRaw& r, float2 qn, float2& a,
                           float2& b) {
  if (!PROJECT) {
    a = make_float2(r.u.x, r.v.x);
    b = make_float2(r.u.y, r.v.y);
    return;
  }
  a = make_float2(r.u.x - (qn.x - r.q.x) * p.inv_hx, r.v.x - (r.q.y - r.q.x) * p.inv_hy);
  b = make_float2(r.u.y - (qn.y - r.q.y) * p.inv_hx, r.v.y - (r.qr - r.q.y) * p.inv_hy);
}

// Window of projected rows for both columns: w1 = row i - 1, w2 = row i,
// w3 = row i + 1 (A: column jl, B: column jl + 1).
struct StreamWindow {
  float2 a1, a2, a3, b1, b2, b3;
  float2 fxa, fxb;  // x-face fluxes after row i - 1
};

// Row i of the paired stream: u*, v* of both columns, stored when `out`.
template <bool PROJECT, int CONVECT, int FORCE>
CFD_D void stream_row(const FvmParams& p, int i, int jA, bool out, float2 fuy, StreamWindow& w,
                       const float2 a4, const float2 b4, float* __restrict__ uo,
                       float* __restrict__ vo) {
  const float2 ihx = splat2(p.inv_hx), ihy = splat2(p.inv_hy);
  // Row i of the neighbours: left lane's column B, right lane's columns A, B.
  const float2 lb = shfl_up2(w.b2, 1), ra = shfl_down2(w.a2, 1), rb = shfl_down2(w.b2, 1);
  // x-faces after row i.
  const float2 fxa = stream_xface<CONVECT>(p, w.a1, w.a2, w.a3, a4, w.b2.x);
  const float2 fxb = stream_xface<CONVECT>(p, w.b1, w.b2, w.b3, b4, ra.x);
  // y-faces after columns jl and jl + 1 (stencils jl-1 .. jl+2, jl .. jl+3).
  const float2 Va = mul2(splat2(0.5f), add2(splat2(w.a2.y), make_float2(w.a3.y, w.b2.y)));
  const float2 Vb = mul2(splat2(0.5f), add2(splat2(w.b2.y), make_float2(w.b3.y, ra.y)));
  float2 fya, fyb;
  if (CONVECT == 0) {
    fya = tvd_flux2(lb, w.a2, w.b2, ra, Va, p.cfl_y);
    fyb = tvd_flux2(w.a2, w.b2, ra, rb, Vb, p.cfl_y);
  } else {
    const float2 ca = mul2(splat2(0.5f), add2(w.a2, w.b2));
    const float2 cb = mul2(splat2(0.5f), add2(w.b2, ra));
    fya = mul2(make_float2(ca.x, Va.y), make_float2(Va.x, Va.y));
    fyb = mul2(make_float2(cb.x, Vb.y), make_float2(Vb.x, Vb.y));
  }
  const float2 fy_left = shfl_up2(fyb, 1);
  if (out) {
    const size_t at = ((size_t)i << p.log2ny) + jA;
    float2 ka = fma2(sub2(fya, fy_left), ihy, mul2(sub2(fxa, w.fxa), ihx));
    float2 kb = fma2(sub2(fyb, fya), ihy, mul2(sub2(fxb, w.fxb), ihx));
    ka = make_float2(-ka.x, -ka.y);
    kb = make_float2(-kb.x, -kb.y);
    if (FORCE == 1) {
      ka = add_diffusion_forcing_fu<1>(p, ka, w.a2, add2(w.a1, w.a3), add2(lb, w.b2), fuy.x);
      kb = add_diffusion_forcing_fu<1>(p, kb, w.b2, add2(w.b1, w.b3), add2(w.a2, ra), fuy.y);
    } else {
      ka = add_diffusion_forcing<FORCE>(p, ka, w.a2, add2(w.a1, w.a3), add2(lb, w.b2), i, jA);
      kb = add_diffusion_forcing<FORCE>(p, kb, w.b2, add2(w.b1, w.b3), add2(w.a2, ra), i,
                                        jA + 1);
    }
    const float2 na = fma2(splat2(p.dt), ka, w.a2), nb = fma2(splat2(p.dt), kb, w.b2);
    *reinterpret_cast<float2*>(uo + at) = make_float2(na.x, nb.x);
    *reinterpret_cast<float2*>(vo + at) = make_float2(na.y, nb.y);
  }
  w.fxa = fxa;
  w.fxb = fxb;
  w.a1 = w.a2;
  w.a2 = w.a3;
  w.a3 = a4;
  w.b1 = w.b2;
  w.b2 = w.b3;
  w.b3 = b4;
}

// bx: the block's index among the (ny / 60) x (nx / SH) / 4 blocks of a grid;
// each warp walks SH rows of its strip with rows fetched PF ahead (a ring of
// PF raw rows in registers).
template <bool PROJECT, int CONVECT, int FORCE, int SH, int PF>
CFD_D void explicit_stream_body(const FvmParams& p, int bx, const float* __restrict__ ua,
                                 const float* __restrict__ va, const float* __restrict__ q,
                                 float* __restrict__ uo, float* __restrict__ vo) {
  static_assert(SH % PF == 0, "rows per warp must be a multiple of the prefetch depth");
  const int lane = threadIdx.x & 31;
  const int warp = (int)((bx * blockDim.x + threadIdx.x) >> 5);
  const int strips = (p.ny + kStreamCols - 1) / kStreamCols;
  const int s = warp % strips, t = warp / strips;
  const int r0 = t * SH;
  if (r0 >= p.nx) return;  // uniform per warp
  const int my = p.ny - 1;
  const int jl = s * kStreamCols - 2 + 2 * lane;  // unwrapped first column of this lane
  const int j = jl & my, jr = (jl + 2) & my;
  const bool out = lane >= 1 && lane < 31 && jl < p.ny;
  const float2 fuy = FORCE == 1 ? __ldg(reinterpret_cast<const float2*>(p.fu_y + j))
                                : make_float2(0.f, 0.f);

  // Window rows r0-2 .. r0+1 (projected), ring of raw rows r0+2 .. r0+PF+1.
  const StreamRaw rm2 = stream_fetch<PROJECT>(p, ua, va, q, r0 - 2, j, jr);
  const StreamRaw rm1 = stream_fetch<PROJECT>(p, ua, va, q, r0 - 1, j, jr);
  const StreamRaw rz0 = stream_fetch<PROJECT>(p, ua, va, q, r0, j, jr);
  const StreamRaw rp1 = stream_fetch<PROJECT>(p, ua, va, q, r0 + 1, j, jr);
  StreamRaw ring[PF];
#pragma unroll
  for (int k = 0; k < PF; ++k) ring[k] = stream_fetch<PROJECT>(p, ua, va, q, r0 + 2 + k, j, jr);
  StreamWindow w;
  float2 a0, b0;
  stream_project<PROJECT>(p, rm2, rm1.q, a0, b0);
  stream_project<PROJECT>(p, rm1, rz0.q, w.a1, w.b1);
  stream_project<PROJECT>(p, rz0, rp1.q, w.a2, w.b2);
  stream_project<PROJECT>(p, rp1, ring[0].q, w.a3, w.b3);
  {
    // x-faces after row r0 - 1.
    const float2 ra1 = shfl_down2(w.a1, 1);
    w.fxa = stream_xface<CONVECT>(p, a0, w.a1, w.a2, w.a3, w.b1.x);
    w.fxb = stream_xface<CONVECT>(p, b0, w.b1, w.b2, w.b3, ra1.x);
  }
  // Row i projects row i + 2 (ring slot K, q of row i + 3 from slot K + 1, or
  // from slot 0 already refilled) and refills slot K with row i + 2 + PF.
#pragma unroll 1
  for (int a = 0; a < SH; a += PF) {
#pragma unroll
    for (int K = 0; K < PF; ++K) {
      const int i = r0 + a + K;
      float2 a4, b4;
      stream_project<PROJECT>(p, ring[K], ring[(K + 1) % PF].q, a4, b4);
      ring[K] = stream_fetch<PROJECT>(p, ua, va, q, i + 2 + PF, j, jr);
      stream_row<PROJECT, CONVECT, FORCE>(p, i, j, out, fuy, w, a4, b4, uo, vo);
    }
  }
}

template <bool PROJECT, int CONVECT, int FORCE, int SH>
__global__ void __launch_bounds__(128, PROJECT && FORCE == 1 ? kStreamBlocksPerSM : 1)
    fvm_explicit_stream_kernel(FvmParams p, const float* __restrict__ ua,
                                const float* __restrict__ va, const float* __restrict__ q,
                                float* __restrict__ uo, float* __restrict__ vo) {
  pdl_wait();
  pdl_trigger();
  explicit_stream_body<PROJECT, CONVECT, FORCE, SH, kStreamPrefetch>(p, blockIdx.x, ua, va, q,
                                                                     uo, vo);
}

// Every warp's SH rows lie inside the grid (nx a multiple of SH).
bool stream_ok(const FvmParams& p) {
  return p.ny >= 64 && p.nx % kStreamRows == 0 && p.nx % stream_rows_of(p.stream_rows) == 0;
}

// Backward-difference divergence of (u*, v*) (finite_differences.py:95-143)
// followed by the packed real FFT of each row along y.  Shared memory holds
// `rows` padded sequences of L = ny/2 complex values (pidx layout).
// MAXT/MINB: launch bounds of the block shape the launcher picked (wide
// 256-thread blocks, or narrow blocks capped at 72 registers so that a whole
// 2048^2 grid is resident in one wave).
CFD_D void div_rfft_rows(const FvmParams& p, int blk, int rows,
                         const float* __restrict__ us, const float* __restrict__ vs,
                         float2* __restrict__ spec) {
  extern __shared__ float2 sbuf[];
  const int L = p.ny >> 1, log2L = p.log2ny - 1, PL = padded_len(L);
  const int i0 = blk * rows;
  const int mx = p.nx - 1, my = p.ny - 1;
  const size_t ny = (size_t)p.ny;
  const int log2g = p.log2ny - 2;  // float4 groups per row
  const int groups = rows << log2g;
#pragma unroll 4
  for (int g = threadIdx.x; g < groups; g += blockDim.x) {
    const int r = g >> log2g, jj = (g & ((1 << log2g) - 1)) << 2;
    const int i = i0 + r, im = (i - 1) & mx;
    const float4 a = __ldg(reinterpret_cast<const float4*>(us + i * ny + jj));
    if (p.row_field) {
      // The field itself (implicit diffusion's rfftn(u)).
      float2* z = sbuf + r * PL;
      z[pidx(jj >> 1)] = make_float2(a.x, a.y);
      z[pidx((jj >> 1) + 1)] = make_float2(a.z, a.w);
      continue;
    }
    const float4 b = __ldg(reinterpret_cast<const float4*>(us + im * ny + jj));
    const float4 c = __ldg(reinterpret_cast<const float4*>(vs + i * ny + jj));
    const float cm = __ldg(vs + i * ny + ((jj - 1) & my));
    // D = (u - u[i-1]) / hx + (v - v[j-1]) / hy
    const float d0 = (a.x - b.x) * p.inv_hx + (c.x - cm) * p.inv_hy;
    const float d1 = (a.y - b.y) * p.inv_hx + (c.y - c.x) * p.inv_hy;
    const float d2 = (a.z - b.z) * p.inv_hx + (c.z - c.y) * p.inv_hy;
    const float d3 = (a.w - b.w) * p.inv_hx + (c.w - c.z) * p.inv_hy;
    const int n = jj >> 1;
    float2* z = sbuf + r * PL;
    z[pidx(n)] = make_float2(d0, d1);
    z[pidx(n + 1)] = make_float2(d2, d3);
  }
  __syncthreads();
  fft_inplace<-1>(sbuf, log2L, rows, PL, p.twp_y, threadIdx.x);
  // Untangle: pairs (k, L-k) for k in [1, L/2); the k = 0 slot also handles
  // the DC/Nyquist pair and the middle element k = L/2.
  const int half = L >> 1, log2h = log2L - 1;
  for (int idx = threadIdx.x; idx < (rows << log2h); idx += blockDim.x) {
    const int r = idx >> log2h, k = idx & (half - 1);
    float2* out = spec + (size_t)(i0 + r) * L;
    const float2* z = sbuf + r * PL;
    if (k == 0) {
      const float2 z0 = z[0];
      out[0] = make_float2(z0.x + z0.y, z0.x - z0.y);
      float2 xk, xm;
      const float2 zh = z[pidx(half)];
      rfft_post_pair(zh, zh, __ldg(p.tw_y + half), &xk, &xm);
      out[half] = xk;
    } else {
      float2 xk, xm;
      rfft_post_pair(z[pidx(k)], z[pidx(L - k)], __ldg(p.tw_y + k), &xk, &xm);
      out[k] = xk;
      out[L - k] = xm;
    }
  }
}

template <int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB)
    fvm_div_rfft_kernel(FvmParams p, int rows, const float* __restrict__ us,
                        const float* __restrict__ vs, float2* __restrict__ spec) {
  div_rfft_rows(p, blockIdx.x, rows, us, vs, spec);
}

// The same transform with the input rows staged by bulk copies: one thread
// requests u rows i0-1 .. i0+R-1 and v rows i0 .. i0+R-1 straight into shared
// memory (no registers hold data in flight), every thread waits on the
// mbarrier, and the divergence is formed from shared memory.  Shared memory:
// (2R + 1) rows of floats, then R padded FFT rows, then the barrier.
CFD_HD size_t div_rfft_bulk_smem(int ny, int rows) {
  return (size_t)(2 * rows + 1) * ny * 4 + (size_t)rows * padded_len(ny / 2) * 8 + 16;
}

CFD_D void div_rfft_rows_bulk(const FvmParams& p, int blk, int rows,
                              const float* __restrict__ us, const float* __restrict__ vs,
                              float2* __restrict__ spec) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ny = p.ny, L = ny >> 1, log2L = p.log2ny - 1, PL = padded_len(L);
  float* su = reinterpret_cast<float*>(smem_raw);
  float* sv = su + (size_t)(rows + 1) * ny;
  float2* sbuf = reinterpret_cast<float2*>(sv + (size_t)rows * ny);
  uint64_t* bar = reinterpret_cast<uint64_t*>(sbuf + (size_t)rows * PL);
  const int i0 = blk * rows, mx = p.nx - 1, my = ny - 1;
  const uint32_t rb = (uint32_t)ny * 4u;
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_arrive_expect_tx(bar, (uint32_t)(2 * rows + 1) * rb);
    bulk_load(su, us + (size_t)((i0 - 1) & mx) * ny, rb, bar);
    bulk_load(su + ny, us + (size_t)i0 * ny, (uint32_t)rows * rb, bar);
    bulk_load(sv, vs + (size_t)i0 * ny, (uint32_t)rows * rb, bar);
  }
  const bool ok = mbar_wait(bar, 0);
  if (__syncthreads_or(!ok)) return;
  const int log2g = p.log2ny - 2;  // float4 groups per row
  const int groups = rows << log2g;
  for (int g = threadIdx.x; g < groups; g += blockDim.x) {
    const int r = g >> log2g, jj = (g & ((1 << log2g) - 1)) << 2;
    const float4 a = *reinterpret_cast<const float4*>(su + (size_t)(r + 1) * ny + jj);
    const float4 b = *reinterpret_cast<const float4*>(su + (size_t)r * ny + jj);
    const float4 c = *reinterpret_cast<const float4*>(sv + (size_t)r * ny + jj);
    const float cm = sv[(size_t)r * ny + ((jj - 1) & my)];
    // D = (u - u[i-1]) / hx + (v - v[j-1]) / hy
    const float d0 = (a.x - b.x) * p.inv_hx + (c.x - cm) * p.inv_hy;
    const float d1 = (a.y - b.y) * p.inv_hx + (c.y - c.x) * p.inv_hy;
    const float d2 = (a.z - b.z) * p.inv_hx + (c.z - c.y) * p.inv_hy;
    const float d3 = (a.w - b.w) * p.inv_hx + (c.w - c.z) * p.inv_hy;
    const int n = jj >> 1;
    float2* z = sbuf + r * PL;
    z[pidx(n)] = make_float2(d0, d1);
    z[pidx(n + 1)] = make_float2(d2, d3);
  }
  __syncthreads();
  fft_inplace<-1>(sbuf, log2L, rows, PL, p.twp_y, threadIdx.x);
  const int half = L >> 1, log2h = log2L - 1;
  for (int idx = threadIdx.x; idx < (rows << log2h); idx += blockDim.x) {
    const int r = idx >> log2h, k = idx & (half - 1);
    float2* out = spec + (size_t)(i0 + r) * L;
    const float2* z = sbuf + r * PL;
    if (k == 0) {
      const float2 z0 = z[0];
      out[0] = make_float2(z0.x + z0.y, z0.x - z0.y);
      float2 xk, xm;
      const float2 zh = z[pidx(half)];
      rfft_post_pair(zh, zh, __ldg(p.tw_y + half), &xk, &xm);
      out[half] = xk;
    } else {
      float2 xk, xm;
      rfft_post_pair(z[pidx(k)], z[pidx(L - k)], __ldg(p.tw_y + k), &xk, &xm);
      out[k] = xk;
      out[L - k] = xm;
    }
  }
}

template <int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB)
    fvm_div_rfft_bulk_kernel(FvmParams p, int rows, const float* __restrict__ us,
                             const float* __restrict__ vs, float2* __restrict__ spec) {
  div_rfft_rows_bulk(p, blockIdx.x, rows, us, vs, spec);
}

// Diagonal of the column pass in the rfft basis, with irfftn's 1/(nx*ny)
// folded in (a power of two, so exact).  col_diag 0: the pseudoinverse of the
// periodic Laplacian (fast_diagonalization.py:199-266), 1/lambda where
// |lambda| > cutoff, else 0.  col_diag 1: implicit diffusion's
// func(lambda) = x / (1 - x), x = (dt nu) lambda (diffusion.py:176-182).
CFD_D float pinv_diag_at(const FvmParams& p, float lamx, int ky) {
  const float lam = lamx + __ldg(p.lamy + ky);
  if (p.col_diag == 1) {
    const float x = p.dtnu * lam;
    return p.pinv_scale * (x / (1.f - x));
  }
  return fabsf(lam) > p.cutoff ? p.pinv_scale / lam : 0.f;
}
CFD_D float pinv_diag(const FvmParams& p, int kx, int ky) {
  return pinv_diag_at(p, __ldg(p.lamx + kx), ky);
}

// Column pass of the packed row spectra.  Row element 0 holds the real DC and
// Nyquist values (X_0, X_L) of the row transform; their columns are
// transformed as two separate real sequences: the block of column 0 takes the
// DC column (imaginary parts zero) and one extra block past the last column
// group takes the Nyquist column.  (Transforming them together as one complex
// column A + iB would put the rounding error of the large DC column, whose
// low modes pinv amplifies, into the small Nyquist column: the projected
// field's divergence then grows tenfold at 2048 rows.)  Each writes back only
// its own float of element 0.
CFD_D void col_pinv_cols(const FvmParams& p, int blk, int W, int log2W, int bstride,
                          float2* __restrict__ spec) {
  extern __shared__ float2 sbuf[];
  const int L = p.ny >> 1, N = p.nx;
  const int c0 = blk * W;
  const bool nyq = c0 >= L;  // the extra block: Nyquist column in slot 0
  float* specf = reinterpret_cast<float*>(spec);
  const int tid = threadIdx.x;
#pragma unroll 4
  for (int idx = tid; idx < W * N; idx += blockDim.x) {
    const int w = idx & (W - 1), i = idx >> log2W, c = c0 + w;
    float2 x;
    if (nyq) x = make_float2(w == 0 ? specf[(size_t)i * L * 2 + 1] : 0.f, 0.f);
    else if (c == 0) x = make_float2(specf[(size_t)i * L * 2], 0.f);
    else x = spec[(size_t)i * L + c];
    sbuf[w * bstride + pidx(i)] = x;
  }
  __syncthreads();
  fft_inplace<-1>(sbuf, p.log2nx, W, bstride, p.twp_x, tid);
  for (int idx = tid; idx < W * N; idx += blockDim.x) {
    const int w = idx & (W - 1), kx = idx >> log2W;
    float2* e = sbuf + w * bstride + pidx(kx);
    *e = c_scale(*e, pinv_diag(p, kx, nyq ? L : c0 + w));
  }
  __syncthreads();
  fft_inplace<1>(sbuf, p.log2nx, W, bstride, p.twp_x, tid);
#pragma unroll 4
  for (int idx = tid; idx < W * N; idx += blockDim.x) {
    const int w = idx & (W - 1), i = idx >> log2W, c = c0 + w;
    const float2 x = sbuf[w * bstride + pidx(i)];
    if (nyq) {
      if (w == 0) specf[(size_t)i * L * 2 + 1] = x.x;
    } else if (c == 0) {
      specf[(size_t)i * L * 2] = x.x;
    } else {
      spec[(size_t)i * L + c] = x;
    }
  }
}

template <int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB)
    fvm_col_pinv_kernel(FvmParams p, int W, int log2W, int bstride,
                        float2* __restrict__ spec) {
  col_pinv_cols(p, blockIdx.x, W, log2W, bstride, spec);
}

// The column pass with one column per block and CL adjacent columns per
// thread-block cluster.  Global memory is read and written in CL-column row
// segments (32 or 64 bytes: whole sectors) through distributed shared memory:
// block `rank` of the cluster moves rows [rank*nx/CL, (rank+1)*nx/CL) of all
// CL columns between global memory and the owning blocks' shared memory, and
// each block transforms its own column.
// The column pass with one column per block and CL adjacent columns per
// thread-block cluster.  Global memory is read and written in CL-column row
// segments (32 or 64 bytes: whole sectors) through distributed shared memory:
// block `rank` of the cluster moves rows [rank*nx/CL, (rank+1)*nx/CL) of all
// CL columns between global memory and the owning blocks' shared memory, and
// each block transforms its own column.  As in col_pinv_cols, column 0 is the
// DC column alone and one extra cluster (first column L) carries the Nyquist
// column in its block 0 (its other blocks transform zeros and store nothing).
template <int CL>
CFD_D void col_pinv_cluster_cols(const FvmParams& p, float2* __restrict__ spec) {
  extern __shared__ float2 sbuf[];
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int L = p.ny >> 1, N = p.nx;
  const int c0 = blockIdx.x - rank;  // first column of this cluster
  const int c = c0 + rank;
  const bool nyq = c0 >= L;
  float* specf = reinterpret_cast<float*>(spec);
  const int tid = threadIdx.x;
  const int rows_per = N / CL, r0 = rank * rows_per;
  float2* dsm[CL];
#pragma unroll
  for (int r = 0; r < CL; ++r) dsm[r] = cluster.map_shared_rank(sbuf, r);
  // Every block of the cluster must be running before any block touches a
  // peer's shared memory.
  cluster.sync();
  if (nyq) {
    for (int row = r0 + tid; row < r0 + rows_per; row += blockDim.x) {
      dsm[0][pidx(row)] = make_float2(specf[(size_t)row * L * 2 + 1], 0.f);
#pragma unroll
      for (int r = 1; r < CL; ++r) dsm[r][pidx(row)] = make_float2(0.f, 0.f);
    }
  } else {
#pragma unroll 2
    for (int row = r0 + tid; row < r0 + rows_per; row += blockDim.x) {
      const float4* src = reinterpret_cast<const float4*>(spec + (size_t)row * L + c0);
      float4 v[CL / 2];
#pragma unroll
      for (int h = 1; h < CL / 2; ++h) v[h] = src[h];
      if (c0 == 0) {
        // DC value only: the Nyquist float belongs to the extra cluster.
        const float2 b = spec[(size_t)row * L + 1];
        v[0] = make_float4(specf[(size_t)row * L * 2], 0.f, b.x, b.y);
      } else {
        v[0] = src[0];
      }
#pragma unroll
      for (int h = 0; h < CL / 2; ++h) {
        dsm[2 * h][pidx(row)] = make_float2(v[h].x, v[h].y);
        dsm[2 * h + 1][pidx(row)] = make_float2(v[h].z, v[h].w);
      }
    }
  }
  cluster.sync();
  fft_inplace<-1>(sbuf, p.log2nx, 1, padded_len(N), p.twp_x, tid);
  const int cp = nyq ? L : c;  // pinv column index
  for (int kx = tid; kx < N; kx += blockDim.x)
    sbuf[pidx(kx)] = c_scale(sbuf[pidx(kx)], pinv_diag(p, kx, cp));
  __syncthreads();
  fft_inplace<1>(sbuf, p.log2nx, 1, padded_len(N), p.twp_x, tid);
  cluster.sync();
  if (nyq) {
    for (int row = r0 + tid; row < r0 + rows_per; row += blockDim.x)
      specf[(size_t)row * L * 2 + 1] = dsm[0][pidx(row)].x;
  } else {
#pragma unroll 2
    for (int row = r0 + tid; row < r0 + rows_per; row += blockDim.x) {
      float4* dst = reinterpret_cast<float4*>(spec + (size_t)row * L + c0);
#pragma unroll
      for (int h = 0; h < CL / 2; ++h) {
        const float2 a = dsm[2 * h][pidx(row)], b = dsm[2 * h + 1][pidx(row)];
        if (h == 0 && c0 == 0) {
          specf[(size_t)row * L * 2] = a.x;
          spec[(size_t)row * L + 1] = b;
        } else {
          dst[h] = make_float4(a.x, a.y, b.x, b.y);
        }
      }
    }
  }
  // No block may leave while a peer still reads its shared memory.
  cluster.sync();
}

template <int CL>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(128, 7)
    fvm_col_pinv_cluster_kernel(FvmParams p, float2* __restrict__ spec) {
  col_pinv_cluster_cols<CL>(p, spec);
}

// ---- Persistent FVM column pass (engine in colpipe.cuh) ----
// Requests worker t's pass-0 points of group g into its own staging slots
// stage[r * T + tid] (T threads per block).  Column c = g * CG + w; the
// Nyquist group's slot 0 reads row element 0 (its imaginary part is the
// Nyquist value), its other slots read nothing.
template <int LOG2N, int CG>
CFD_D void col_pipe_prefetch(const float2* __restrict__ spec, int L, int g, int w, int t,
                             float2* __restrict__ stage) {
  constexpr int NTHR = ColPipe<LOG2N>::NTHR, T = CG * NTHR;
  const bool nyq = g * CG >= L;
  if (nyq && w != 0) return;
  const int c = nyq ? 0 : g * CG + w;
  const int tid = t * CG + w;
#pragma unroll
  for (int r = 0; r < 16; ++r) cp_async8(stage + r * T + tid, spec + (size_t)(t + NTHR * r) * L + c);
}

// Worker t's pass-0 points from its staging slots: the DC column (c == 0)
// takes the real parts of row element 0, the Nyquist column their imaginary
// parts, both as real sequences; the Nyquist group's other slots are zeros.
template <int LOG2N, int CG>
CFD_D void col_pipe_take(const float2* __restrict__ stage, int L, int g, int w, int t,
                         float2 (&v)[16]) {
  constexpr int NTHR = ColPipe<LOG2N>::NTHR, T = CG * NTHR;
  const int c = g * CG + w;
  const bool nyq = g * CG >= L;
  const int tid = t * CG + w;
  if (!nyq && c != 0) {
#pragma unroll
    for (int r = 0; r < 16; ++r) v[r] = stage[r * T + tid];
  } else {
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      const float2 x = stage[r * T + tid];
      v[r] = make_float2(nyq ? (w == 0 ? x.y : 0.f) : x.x, 0.f);
    }
  }
}

template <int LOG2N, int CG>
CFD_D void col_pipe_store(float2* __restrict__ spec, int L, int g, int w, int t,
                          const float2 (&v)[16]) {
  constexpr int NTHR = ColPipe<LOG2N>::NTHR;
  const int c = g * CG + w;
  const bool nyq = g * CG >= L;
  if (!nyq && c != 0) {
#pragma unroll
    for (int r = 0; r < 16; ++r) spec[(size_t)(t + NTHR * r) * L + c] = v[r];
  } else if (!nyq || w == 0) {
    float* specf = reinterpret_cast<float*>(spec);
    const int off = nyq ? 1 : 0;
#pragma unroll
    for (int r = 0; r < 16; ++r) specf[(size_t)(t + NTHR * r) * L * 2 + off] = v[r].x;
  }
}

template <int LOG2N, int CG>
CFD_D void col_pinv_pipe_cols(const FvmParams& p, float2* __restrict__ spec, int g0,
                              int gstep) {
  using P = ColPipe<LOG2N>;
  extern __shared__ float2 sbuf[];
  const int L = p.ny >> 1;
  const int groups = L / CG + 1;
  const int w = threadIdx.x % CG, t = threadIdx.x / CG;
  const int bstride = col_pipe_bstride<LOG2N, CG>();
  float2* const buf[2] = {sbuf + w * bstride, sbuf + (CG + w) * bstride};
  float2* const stage = sbuf + 2 * CG * bstride;  // 16 * T slots
  constexpr int INV_FIRST = (P::PASSES - 1) & 1;
  if (g0 >= groups) return;  // uniform per block
  float2 v[16];
  // The constant tables first: under a programmatic launch this overlaps the
  // previous kernel's tail.
  const float2* tw;
  const float* lamx;
  col_pipe_tables<LOG2N, CG>(sbuf, p.twp_x, p.lamx, &tw, &lamx);
  pdl_wait();
  pdl_trigger();
  col_pipe_prefetch<LOG2N, CG>(spec, L, g0, w, t, stage);
  cp_async_commit();
#pragma unroll 1
  for (int g = g0; g < groups; g += gstep) {
    // Each thread reads back only the slots it requested itself, so its own
    // wait is the only ordering needed before it reuses them.
    cp_async_wait_all();
    col_pipe_take<LOG2N, CG>(stage, L, g, w, t, v);
    const int gn = g + gstep;
    if (gn < groups) col_pipe_prefetch<LOG2N, CG>(spec, L, gn, w, t, stage);
    cp_async_commit();
    col_pipe_fft<LOG2N, -1, 0>(v, buf, t, tw);
    const int cp = g * CG >= L ? L : g * CG + w;  // pinv column index
#pragma unroll
    for (int m = 0; m < 16; ++m)
      v[m] = c_scale(v[m], pinv_diag_at(p, lamx[t + P::NTHR * m], cp));
    col_pipe_fft<LOG2N, 1, INV_FIRST>(v, buf, t, tw);
    col_pipe_store<LOG2N, CG>(spec, L, g, w, t, v);
  }
  cp_async_wait_all();
}

template <int LOG2N, int CG>
__global__ void __launch_bounds__(CG * (1 << LOG2N) / 16,
                                  col_pipe_min_blocks(CG * (1 << LOG2N) / 16))
    fvm_col_pinv_pipe_kernel(FvmParams p, float2* __restrict__ spec) {
  col_pinv_pipe_cols<LOG2N, CG>(p, spec, blockIdx.x, gridDim.x);
}

// The persistent column pass with each group staged by TMA: one thread
// issues the group's tiled tensor loads (boxes of 4 columns x 256 rows) onto
// an mbarrier, and the box layout in shared memory, row-major over the 4
// columns, is exactly the per-thread staging layout of col_pinv_pipe_cols
// (worker t of column w reads rows t + (N/16) r at r * T + 4 t + w), so the
// transform code is shared and the bits are the same.  The next group's
// loads are issued after a block barrier (every thread has read the staged
// group) and an async-proxy fence.  Waits are bounded: a copy that never
// lands records g_cfd_device_fault and the whole block leaves together.
template <int LOG2N>
__global__ void __launch_bounds__(4 * (1 << LOG2N) / 16, col_pipe_min_blocks(4 * (1 << LOG2N) / 16))
    fvm_col_pinv_tma_kernel(FvmParams p, float2* __restrict__ spec,
                            const __grid_constant__ CUtensorMap tmap) {
  constexpr int CG = 4;
  using P = ColPipe<LOG2N>;
  constexpr int N = P::N, BOX = N < 256 ? N : 256, NBOX = N / BOX;
  constexpr uint32_t kGroupBytes = (uint32_t)N * CG * sizeof(float2);
  extern __shared__ float2 sbuf[];  // no static shared memory: 128-byte aligned
  const int L = p.ny >> 1, groups = L / CG + 1;
  const int w = threadIdx.x % CG, t = threadIdx.x / CG;
  const int bstride = col_pipe_bstride<LOG2N, CG>();
  float2* const buf[2] = {sbuf + w * bstride, sbuf + (CG + w) * bstride};
  float2* const stage = sbuf + 2 * CG * bstride;
  uint64_t* const bar =
      reinterpret_cast<uint64_t*>(reinterpret_cast<char*>(sbuf) + col_pipe_smem<LOG2N, CG>());
  constexpr int INV_FIRST = (P::PASSES - 1) & 1;
  int g = blockIdx.x;
  if (g >= groups) return;  // uniform per block
  const float2* tw;
  const float* lamx;
  col_pipe_tables<LOG2N, CG>(sbuf, p.twp_x, p.lamx, &tw, &lamx);
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  pdl_wait();
  pdl_trigger();
  // Group gg's columns start at float 8 gg of a row; the Nyquist group reads
  // row element 0 (its imaginary part), like the first group.
  auto issue = [&](int gg) {
    const int x = gg * CG >= L ? 0 : 2 * CG * gg;
    mbar_arrive_expect_tx(bar, kGroupBytes);
#pragma unroll
    for (int b = 0; b < NBOX; ++b) tma_load_2d(stage + b * BOX * CG, &tmap, x, b * BOX, bar);
  };
  if (threadIdx.x == 0) issue(g);
  uint32_t phase = 0;
  float2 v[16];
#pragma unroll 1
  for (; g < groups; g += gridDim.x) {
    const bool landed = mbar_wait(bar, phase);
    phase ^= 1u;
    if (landed) col_pipe_take<LOG2N, CG>(stage, L, g, w, t, v);
    // The staged group is read; a wait that gave up on any thread ends the
    // whole block here (no copy is then issued, none other is in flight).
    if (__syncthreads_or(!landed)) return;
    if (threadIdx.x == 0 && g + gridDim.x < groups) {
      fence_proxy_async_smem();
      issue(g + gridDim.x);
    }
    col_pipe_fft<LOG2N, -1, 0>(v, buf, t, tw);
    const int cp = g * CG >= L ? L : g * CG + w;  // pinv column index
#pragma unroll
    for (int m = 0; m < 16; ++m)
      v[m] = c_scale(v[m], pinv_diag_at(p, lamx[t + P::NTHR * m], cp));
    col_pipe_fft<LOG2N, 1, INV_FIRST>(v, buf, t, tw);
    col_pipe_store<LOG2N, CG>(spec, L, g, w, t, v);
  }
}

// The persistent column pass over a same-shape batch: the work items are the
// (member, group) pairs of the members that take this step, walked with the
// grid as stride, so many members keep every block's staging pipeline full.
// The grid tables are the batch's (member 0's pointers); the pinv scalars are
// each member's, equal across a batch.
template <int LOG2N, int CG>
__global__ void __launch_bounds__(CG * (1 << LOG2N) / 16,
                                  col_pipe_min_blocks(CG * (1 << LOG2N) / 16))
    fvm_batch_col_pinv_pipe_kernel(const FvmMember* __restrict__ mem, int count, int k) {
  using P = ColPipe<LOG2N>;
  extern __shared__ float2 sbuf[];
  const int L = mem[0].p.ny >> 1;
  const int groups = L / CG + 1, items = count * groups;
  const int w = threadIdx.x % CG, t = threadIdx.x / CG;
  const int bstride = col_pipe_bstride<LOG2N, CG>();
  float2* const buf[2] = {sbuf + w * bstride, sbuf + (CG + w) * bstride};
  float2* const stage = sbuf + 2 * CG * bstride;
  constexpr int INV_FIRST = (P::PASSES - 1) & 1;
  const float2* tw;
  const float* lamx;
  col_pipe_tables<LOG2N, CG>(sbuf, mem[0].p.twp_x, mem[0].p.lamx, &tw, &lamx);
  pdl_wait();
  pdl_trigger();
  // Next item at or after `it` (stride gridDim.x) whose member takes step k;
  // the same for every thread of the block.
  auto next_active = [&](int it) {
    while (it < items && k >= mem[it / groups].steps) it += gridDim.x;
    return it;
  };
  int it = next_active(blockIdx.x);
  if (it >= items) return;  // uniform per block
  col_pipe_prefetch<LOG2N, CG>(mem[it / groups].spec, L, it % groups, w, t, stage);
  cp_async_commit();
  float2 v[16];
#pragma unroll 1
  while (it < items) {
    const FvmMember& m = mem[it / groups];
    const int g = it % groups;
    cp_async_wait_all();
    col_pipe_take<LOG2N, CG>(stage, L, g, w, t, v);
    const int nit = next_active(it + gridDim.x);
    if (nit < items) col_pipe_prefetch<LOG2N, CG>(mem[nit / groups].spec, L, nit % groups, w, t, stage);
    cp_async_commit();
    col_pipe_fft<LOG2N, -1, 0>(v, buf, t, tw);
    const int cp = g * CG >= L ? L : g * CG + w;  // pinv column index
#pragma unroll
    for (int mm = 0; mm < 16; ++mm)
      v[mm] = c_scale(v[mm], pinv_diag_at(m.p, lamx[t + P::NTHR * mm], cp));
    col_pipe_fft<LOG2N, 1, INV_FIRST>(v, buf, t, tw);
    col_pipe_store<LOG2N, CG>(m.spec, L, g, w, t, v);
    it = nit;
  }
  cp_async_wait_all();
}

// The batched column pass with each (member, group) item staged by TMA: a
// 3-D tensor map covers the spectra of all members (they sit at one fixed
// stride in the batch's slab), so one thread loads an item's boxes at
// coordinates (float offset, row, member).  Staging layout, transforms and
// bits as fvm_batch_col_pinv_pipe_kernel; barriers and bounded waits as
// fvm_col_pinv_tma_kernel.
template <int LOG2N>
__global__ void __launch_bounds__(4 * (1 << LOG2N) / 16, col_pipe_min_blocks(4 * (1 << LOG2N) / 16))
    fvm_batch_col_pinv_tma_kernel(const FvmMember* __restrict__ mem, int count, int k,
                                  const __grid_constant__ CUtensorMap tmap) {
  constexpr int CG = 4;
  using P = ColPipe<LOG2N>;
  constexpr int N = P::N, BOX = N < 256 ? N : 256, NBOX = N / BOX;
  constexpr uint32_t kGroupBytes = (uint32_t)N * CG * sizeof(float2);
  extern __shared__ float2 sbuf[];  // no static shared memory: 128-byte aligned
  const int L = mem[0].p.ny >> 1;
  const int groups = L / CG + 1, items = count * groups;
  const int w = threadIdx.x % CG, t = threadIdx.x / CG;
  const int bstride = col_pipe_bstride<LOG2N, CG>();
  float2* const buf[2] = {sbuf + w * bstride, sbuf + (CG + w) * bstride};
  float2* const stage = sbuf + 2 * CG * bstride;
  uint64_t* const bar =
      reinterpret_cast<uint64_t*>(reinterpret_cast<char*>(sbuf) + col_pipe_smem<LOG2N, CG>());
  constexpr int INV_FIRST = (P::PASSES - 1) & 1;
  const float2* tw;
  const float* lamx;
  col_pipe_tables<LOG2N, CG>(sbuf, mem[0].p.twp_x, mem[0].p.lamx, &tw, &lamx);
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  pdl_wait();
  pdl_trigger();
  // Next item at or after `it` (stride gridDim.x) whose member takes step k;
  // the same for every thread of the block.
  auto next_active = [&](int it) {
    while (it < items && k >= mem[it / groups].steps) it += gridDim.x;
    return it;
  };
  auto issue = [&](int item) {
    const int gg = item % groups, z = item / groups;
    const int x = gg * CG >= L ? 0 : 2 * CG * gg;
    mbar_arrive_expect_tx(bar, kGroupBytes);
#pragma unroll
    for (int b = 0; b < NBOX; ++b)
      tma_load_3d(stage + b * BOX * CG, &tmap, x, b * BOX, z, bar);
  };
  int it = next_active(blockIdx.x);
  if (it >= items) return;  // uniform per block
  if (threadIdx.x == 0) issue(it);
  uint32_t phase = 0;
  float2 v[16];
#pragma unroll 1
  while (it < items) {
    const FvmMember& m = mem[it / groups];
    const int g = it % groups;
    const bool landed = mbar_wait(bar, phase);
    phase ^= 1u;
    if (landed) col_pipe_take<LOG2N, CG>(stage, L, g, w, t, v);
    // The staged item is read; a wait that gave up on any thread ends the
    // whole block here (no copy is then issued, none other is in flight).
    if (__syncthreads_or(!landed)) return;
    const int nit = next_active(it + gridDim.x);
    if (threadIdx.x == 0 && nit < items) {
      fence_proxy_async_smem();
      issue(nit);
    }
    col_pipe_fft<LOG2N, -1, 0>(v, buf, t, tw);
    const int cp = g * CG >= L ? L : g * CG + w;  // pinv column index
#pragma unroll
    for (int mm = 0; mm < 16; ++mm)
      v[mm] = c_scale(v[mm], pinv_diag_at(m.p, lamx[t + P::NTHR * mm], cp));
    col_pipe_fft<LOG2N, 1, INV_FIRST>(v, buf, t, tw);
    col_pipe_store<LOG2N, CG>(m.spec, L, g, w, t, v);
    it = nit;
  }
}

// Inverse packed real FFT of each row, in place: q^ rows -> q rows (floats).
CFD_D void irfft_rows(const FvmParams& p, int blk, int rows, float2* spec) {
  extern __shared__ float2 sbuf[];
  const int L = p.ny >> 1, log2L = p.log2ny - 1, PL = padded_len(L);
  const int i0 = blk * rows;
  const int half = L >> 1, log2h = log2L - 1;
  for (int idx = threadIdx.x; idx < (rows << log2h); idx += blockDim.x) {
    const int r = idx >> log2h, k = idx & (half - 1);
    const float2* in = spec + (size_t)(i0 + r) * L;
    float2* z = sbuf + r * PL;
    if (k == 0) {
      const float2 x0 = in[0];
      z[0] = make_float2(x0.x + x0.y, x0.x - x0.y);
      const float2 xh = in[half];
      float2 zk, zm;
      irfft_pre_pair(xh, xh, __ldg(p.tw_y + half), &zk, &zm);
      z[pidx(half)] = zk;
    } else {
      float2 zk, zm;
      irfft_pre_pair(in[k], in[L - k], __ldg(p.tw_y + k), &zk, &zm);
      z[pidx(k)] = zk;
      z[pidx(L - k)] = zm;
    }
  }
  __syncthreads();
  fft_inplace<1>(sbuf, log2L, rows, PL, p.twp_y, threadIdx.x);
  // q[2n], q[2n+1] = z[n]; two complex values per float4 store.
  const int log2p = log2L - 1;  // pairs per row
  for (int idx = threadIdx.x; idx < (rows << log2p); idx += blockDim.x) {
    const int r = idx >> log2p, n = (idx & ((1 << log2p) - 1)) << 1;
    const float2 a = sbuf[r * PL + pidx(n)], b = sbuf[r * PL + pidx(n + 1)];
    reinterpret_cast<float4*>(spec + (size_t)(i0 + r) * L)[n >> 1] = make_float4(a.x, a.y, b.x, b.y);
  }
}

template <int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB)
    fvm_irfft_kernel(FvmParams p, int rows, float2* spec) {
  irfft_rows(p, blockIdx.x, rows, spec);
}

// The inverse transform with its R spectrum rows staged by one bulk copy.
// Shared memory: R input rows (L complex each), R padded FFT rows, barrier.
CFD_HD size_t irfft_bulk_smem(int ny, int rows) {
  return (size_t)rows * (ny / 2) * 8 + (size_t)rows * padded_len(ny / 2) * 8 + 16;
}

CFD_D void irfft_rows_bulk(const FvmParams& p, int blk, int rows, float2* spec) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int L = p.ny >> 1, log2L = p.log2ny - 1, PL = padded_len(L);
  float2* sin = reinterpret_cast<float2*>(smem_raw);
  float2* sbuf = sin + (size_t)rows * L;
  uint64_t* bar = reinterpret_cast<uint64_t*>(sbuf + (size_t)rows * PL);
  const int i0 = blk * rows;
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t bytes = (uint32_t)rows * (uint32_t)L * 8u;
    mbar_arrive_expect_tx(bar, bytes);
    bulk_load(sin, spec + (size_t)i0 * L, bytes, bar);
  }
  const bool ok = mbar_wait(bar, 0);
  if (__syncthreads_or(!ok)) return;
  const int half = L >> 1, log2h = log2L - 1;
  for (int idx = threadIdx.x; idx < (rows << log2h); idx += blockDim.x) {
    const int r = idx >> log2h, k = idx & (half - 1);
    const float2* in = sin + (size_t)r * L;
    float2* z = sbuf + r * PL;
    if (k == 0) {
      const float2 x0 = in[0];
      z[0] = make_float2(x0.x + x0.y, x0.x - x0.y);
      const float2 xh = in[half];
      float2 zk, zm;
      irfft_pre_pair(xh, xh, __ldg(p.tw_y + half), &zk, &zm);
      z[pidx(half)] = zk;
    } else {
      float2 zk, zm;
      irfft_pre_pair(in[k], in[L - k], __ldg(p.tw_y + k), &zk, &zm);
      z[pidx(k)] = zk;
      z[pidx(L - k)] = zm;
    }
  }
  __syncthreads();
  fft_inplace<1>(sbuf, log2L, rows, PL, p.twp_y, threadIdx.x);
  const int log2p = log2L - 1;  // pairs per row
  for (int idx = threadIdx.x; idx < (rows << log2p); idx += blockDim.x) {
    const int r = idx >> log2p, n = (idx & ((1 << log2p) - 1)) << 1;
    const float2 a = sbuf[r * PL + pidx(n)], b = sbuf[r * PL + pidx(n + 1)];
    reinterpret_cast<float4*>(spec + (size_t)(i0 + r) * L)[n >> 1] = make_float4(a.x, a.y, b.x, b.y);
  }
}

template <int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB)
    fvm_irfft_bulk_kernel(FvmParams p, int rows, float2* spec) {
  irfft_rows_bulk(p, blockIdx.x, rows, spec);
}

// ---- One warp per row (ny = 2048: L = 1024 packed complex values) ----
// The row transforms of the pressure solve with the four-step warp FFT of
// wfft.cuh: lane l reads complex elements l + 32 m straight from global
// memory (coalesced), transforms in registers with one shared-memory
// transpose, and writes elements l + 32 k1 (coalesced).  The real-FFT
// untangling pairs X[k] with X[L - k] through a shuffle: for lane l >= 1 the
// partner lives in lane 32 - l, register 31 - k1; for lane 0 in lane 0,
// register 32 - k1.

CFD_HD bool warp_rows_ok(const FvmParams& p) { return p.log2ny - 1 == kWarpFftLog2; }
constexpr int kWarpRows = 4;  // rows (warps) per block

// The packed real FFT of row i from its samples (lane n1's x[n1 + 32 n2] in
// v[n2], as pairs of reals), written to the row's spectrum.
CFD_D void div_rfft_row_warp_tail(const FvmParams& p, int i, float2 (&v)[32],
                                  float2* __restrict__ spec, float2* tile) {
  const int lane = threadIdx.x & 31;
  const int L = p.ny >> 1;
  warp_fft1024<-1>(v, tile, p.twp_y + wfft_table_offset(kWarpFftLog2));
  float2* out = spec + (size_t)i * L;
#pragma unroll
  for (int k1 = 0; k1 < 32; ++k1) {
    const int k = lane + 32 * k1;
    const float2 z = v[wfft_slot(k1)], zp = wfft_mirror(v, k1, lane);
    float2 xk, xm;
    rfft_post_pair(z, zp, __ldg(p.tw_y + k), &xk, &xm);
    // element 0 packs the real DC and Nyquist values
    out[k] = k == 0 ? make_float2(z.x + z.y, z.x - z.y) : xk;
  }
}

CFD_D void div_rfft_row_warp(const FvmParams& p, int i, const float* __restrict__ us,
                             const float* __restrict__ vs, float2* __restrict__ spec,
                             float2* tile) {
  const int lane = threadIdx.x & 31;
  const int L = p.ny >> 1, mx = p.nx - 1;
  const size_t ny = (size_t)p.ny;
  const float2* ua = reinterpret_cast<const float2*>(us + i * ny);
  const float2* ub = reinterpret_cast<const float2*>(us + ((i - 1) & mx) * ny);
  const float2* vc = reinterpret_cast<const float2*>(vs + i * ny);
  float2 v[32], c[32];
  if (p.row_field) {
    // The field itself: a divergence the stencil already formed, or
    // implicit diffusion's rfftn(u).
#pragma unroll
    for (int m = 0; m < 32; ++m) v[m] = __ldg(ua + lane + 32 * m);
    div_rfft_row_warp_tail(p, i, v, spec, tile);
    return;
  }
#pragma unroll
  for (int m = 0; m < 32; ++m) c[m] = __ldg(vc + lane + 32 * m);
  // v[j - 1] for j = 2n is the odd half of element n - 1, held by lane - 1 in
  // the same slot; for lane 0 by lane 31 in the previous slot (cyclically).
  // Every lane passes its own slot-m value down one lane, and lane 0 keeps
  // what arrives for its next slot.
  float recv[32];
#pragma unroll
  for (int m = 0; m < 32; ++m) recv[m] = __shfl_sync(kFull, c[m].y, (lane - 1) & 31);
#pragma unroll
  for (int m = 0; m < 32; ++m) {
    const int n = lane + 32 * m;
    const float2 a = __ldg(ua + n), b = __ldg(ub + n);
    const float cm = lane == 0 ? recv[(m - 1) & 31] : recv[m];
    // D = (u - u[i-1]) / hx + (v - v[j-1]) / hy, as in div_rfft_rows
    v[m] = make_float2((a.x - b.x) * p.inv_hx + (c[m].x - cm) * p.inv_hy,
                       (a.y - b.y) * p.inv_hx + (c[m].y - c[m].x) * p.inv_hy);
  }
  div_rfft_row_warp_tail(p, i, v, spec, tile);
}

CFD_D void irfft_row_warp(const FvmParams& p, int i, float2* spec, float2* tile) {
  const int lane = threadIdx.x & 31;
  const int L = p.ny >> 1;
  float2* row = spec + (size_t)i * L;
  // Each element once (32 loads per lane, all in flight together); the
  // mirror X[L - k] of k = lane + 32 m is lane (32 - lane)'s slot 31 - m, or
  // lane 0's own slot 32 - m.
  float2 x[32], v[32];
#pragma unroll
  for (int m = 0; m < 32; ++m) x[m] = row[lane + 32 * m];
#pragma unroll
  for (int m = 0; m < 32; ++m) {
    const int k = lane + 32 * m;
    float2 xm = wfft_shfl_idx2(x[31 - m], (32 - lane) & 31);
    if (lane == 0) xm = x[(32 - m) & 31];
    float2 zk, zm;
    irfft_pre_pair(x[m], xm, __ldg(p.tw_y + k), &zk, &zm);
    v[m] = k == 0 ? make_float2(x[m].x + x[m].y, x[m].x - x[m].y) : zk;
  }
  warp_fft1024<1>(v, tile, p.twp_y + wfft_table_offset(kWarpFftLog2));
  // q[2n], q[2n+1] = z[n] over the same row (every load above has completed:
  // the transform depends on all of them).
#pragma unroll
  for (int k1 = 0; k1 < 32; ++k1) row[lane + 32 * k1] = v[wfft_slot(k1)];
}

__global__ void __launch_bounds__(32 * kWarpRows)
    fvm_div_rfft_warp_kernel(FvmParams p, const float* __restrict__ us,
                             const float* __restrict__ vs, float2* __restrict__ spec) {
  pdl_wait();
  pdl_trigger();
  __shared__ float2 tiles[kWarpRows][kWarpFftTile];
  const int w = threadIdx.x >> 5;
  div_rfft_row_warp(p, blockIdx.x * kWarpRows + w, us, vs, spec, tiles[w]);
}

__global__ void __launch_bounds__(32 * kWarpRows)
    fvm_irfft_warp_kernel(FvmParams p, float2* spec) {
  pdl_wait();
  pdl_trigger();
  __shared__ float2 tiles[kWarpRows][kWarpFftTile];
  const int w = threadIdx.x >> 5;
  irfft_row_warp(p, blockIdx.x * kWarpRows + w, spec, tiles[w]);
}

// u = u* - (q[i+1] - q[i]) / hx ; v = v* - (q[j+1] - q[j]) / hy.
CFD_D void project_out_cells(const FvmParams& p, int blk, int nblk,
                              const float* __restrict__ us, const float* __restrict__ vs,
                              const float* __restrict__ q, float* __restrict__ uo,
                              float* __restrict__ vo) {
  const size_t n = (size_t)p.nx * p.ny;
  const int mx = p.nx - 1, my = p.ny - 1;
  for (size_t idx = blk * (size_t)blockDim.x + threadIdx.x; idx < n;
       idx += (size_t)nblk * blockDim.x) {
    const int i = (int)(idx >> p.log2ny), j = (int)(idx & my);
    const float q0 = __ldg(q + idx);
    const float qx = __ldg(q + (size_t)((i + 1) & mx) * p.ny + j);
    const float qy = __ldg(q + (size_t)i * p.ny + ((j + 1) & my));
    uo[idx] = __ldg(us + idx) - (qx - q0) * p.inv_hx;
    vo[idx] = __ldg(vs + idx) - (qy - q0) * p.inv_hy;
  }
}

// u += w: the last sum of diffusion.solve_fast_diag, u_interior +
// u_dt_diffused (diffusion.py:203-210).
__global__ void fvm_add_kernel(size_t n, const float* __restrict__ w, float* __restrict__ u) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    u[i] = u[i] + w[i];
}

__global__ void fvm_project_out_kernel(FvmParams p, const float* __restrict__ us,
                                       const float* __restrict__ vs,
                                       const float* __restrict__ q,
                                       float* __restrict__ uo,
                                       float* __restrict__ vo) {
  pdl_wait();
  pdl_trigger();
  project_out_cells(p, blockIdx.x, gridDim.x, us, vs, q, uo, vo);
}

// u0 + dt * sum_j c_j k_j, summed from 0 in the reference's order.
__global__ void fvm_rk_combine_kernel(FvmParams p, const float* __restrict__ u0,
                                      const float* __restrict__ v0, RkCombine cb,
                                      float* __restrict__ uo, float* __restrict__ vo) {
  const size_t n = (size_t)p.nx * p.ny;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n;
       idx += (size_t)gridDim.x * blockDim.x) {
    float au = 0.f, av = 0.f;
    for (int j = 0; j < cb.count; ++j) {
      au = au + cb.c[j] * __ldg(cb.k[j][0] + idx);
      av = av + cb.c[j] * __ldg(cb.k[j][1] + idx);
    }
    uo[idx] = __ldg(u0 + idx) + p.dt * au;
    vo[idx] = __ldg(v0 + idx) + p.dt * av;
  }
}

__global__ void divergence_kernel(FvmParams p, const float* __restrict__ u,
                                  const float* __restrict__ v,
                                  float* __restrict__ out) {
  const size_t n = (size_t)p.nx * p.ny;
  const int mx = p.nx - 1, my = p.ny - 1;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(idx >> p.log2ny), j = (int)(idx & my);
    const float dx = (__ldg(u + idx) - __ldg(u + (size_t)((i - 1) & mx) * p.ny + j)) / p.hx;
    const float dy = (__ldg(v + idx) - __ldg(v + (size_t)i * p.ny + ((j - 1) & my))) / p.hy;
    out[idx] = dx + dy;
  }
}

// curl_2d (finite_differences.py:186-193): forward_difference(v, x) -
// forward_difference(u, y), located at offset (1, 1).
__global__ void curl2d_kernel(FvmParams p, const float* __restrict__ u,
                              const float* __restrict__ v,
                              float* __restrict__ out) {
  const size_t n = (size_t)p.nx * p.ny;
  const int mx = p.nx - 1, my = p.ny - 1;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(idx >> p.log2ny), j = (int)(idx & my);
    const float dvx = (__ldg(v + (size_t)((i + 1) & mx) * p.ny + j) - __ldg(v + idx)) / p.hx;
    const float duy = (__ldg(u + (size_t)i * p.ny + ((j + 1) & my)) - __ldg(u + idx)) / p.hy;
    out[idx] = dvx - duy;
  }
}

// max over cells of sqrt(u^2 + v^2); non-negative floats order like their
// bit patterns, so an unsigned atomicMax on the bits is exact.
__global__ void max_speed_kernel(int n, const float* __restrict__ u,
                                 const float* __restrict__ v,
                                 unsigned int* __restrict__ out) {
  float m = 0.f;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n;
       idx += gridDim.x * blockDim.x) {
    const float a = __ldg(u + idx), b = __ldg(v + idx);
    m = fmaxf(m, sqrtf(a * a + b * b));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

// ---- Batched variants: the member index is the last grid axis ----
// Buffer sets of step k: input 0 (k = 0) / 1 (k odd) / 2 (k even > 0),
// output 1 (k even) / 2 (k odd).
CFD_D int batch_src(int k) { return k == 0 ? 0 : ((k & 1) ? 1 : 2); }
CFD_D int batch_dst(int k) { return (k & 1) ? 2 : 1; }

template <bool PROJECT, int CONVECT>
__global__ void __launch_bounds__(kStencilThreads)
    fvm_batch_explicit_kernel(const FvmMember* __restrict__ mem, int k) {
  pdl_wait();
  pdl_trigger();
  const FvmMember& m = mem[blockIdx.z];
  if (k >= m.steps) return;
  const FvmParams p = m.p;
  const int src = batch_src(k), dst = batch_dst(k);
  explicit_tile<PROJECT, false, CONVECT>(p, blockIdx.x, blockIdx.y, m.f[src][0], m.f[src][1],
                                         reinterpret_cast<const float*>(m.spec),
                                         m.f[dst][0], m.f[dst][1]);
}

// The warp-streaming stencil over a batch (member on grid axis y); the
// forcing flags are read at run time (members may differ in them), which
// evaluates the same expressions as the tiles.
template <bool PROJECT, int CONVECT>
__global__ void __launch_bounds__(128)
    fvm_batch_explicit_stream_kernel(const FvmMember* __restrict__ mem, int k) {
  pdl_wait();
  pdl_trigger();
  const FvmMember& m = mem[blockIdx.y];
  if (k >= m.steps) return;
  const FvmParams p = m.p;
  const int src = batch_src(k), dst = batch_dst(k);
  explicit_stream_body<PROJECT, CONVECT, 0, kStreamRows, kBatchStreamPrefetch>(
      p, blockIdx.x, m.f[src][0], m.f[src][1], reinterpret_cast<const float*>(m.spec),
      m.f[dst][0], m.f[dst][1]);
}

template <int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB)
    fvm_batch_div_rfft_kernel(const FvmMember* __restrict__ mem, int k, int rows) {
  pdl_wait();
  pdl_trigger();
  const FvmMember& m = mem[blockIdx.y];
  if (k >= m.steps) return;
  const FvmParams p = m.p;
  const int dst = batch_dst(k);
  div_rfft_rows(p, blockIdx.x, rows, m.f[dst][0], m.f[dst][1], m.spec);
}

// The bulk-copy row feed over a batch (the single kernels' bodies; slot on
// grid axis y).  The slots' fields sit at 16-byte multiples in the batch slab.
template <int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB)
    fvm_batch_div_rfft_bulk_kernel(const FvmMember* __restrict__ mem, int k, int rows) {
  pdl_wait();
  pdl_trigger();
  const FvmMember& m = mem[blockIdx.y];
  if (k >= m.steps) return;
  const FvmParams p = m.p;
  const int dst = batch_dst(k);
  div_rfft_rows_bulk(p, blockIdx.x, rows, m.f[dst][0], m.f[dst][1], m.spec);
}

template <int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB)
    fvm_batch_irfft_bulk_kernel(const FvmMember* __restrict__ mem, int k, int rows) {
  pdl_wait();
  pdl_trigger();
  const FvmMember& m = mem[blockIdx.y];
  if (k >= m.steps) return;
  const FvmParams p = m.p;
  irfft_rows_bulk(p, blockIdx.x, rows, m.spec);
}

template <int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB)
    fvm_batch_col_pinv_kernel(const FvmMember* __restrict__ mem, int k, int W, int log2W,
                              int bstride) {
  pdl_wait();
  pdl_trigger();
  const FvmMember& m = mem[blockIdx.y];
  if (k >= m.steps) return;
  const FvmParams p = m.p;
  col_pinv_cols(p, blockIdx.x, W, log2W, bstride, m.spec);
}

// Every block of a cluster belongs to one member (clusters span x only), so
// an idle member's cluster leaves as a whole.
template <int CL>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(128, 7)
    fvm_batch_col_pinv_cluster_kernel(const FvmMember* __restrict__ mem, int k) {
  pdl_wait();
  pdl_trigger();
  const FvmMember& m = mem[blockIdx.y];
  if (k >= m.steps) return;
  const FvmParams p = m.p;
  col_pinv_cluster_cols<CL>(p, m.spec);
}

template <int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB)
    fvm_batch_irfft_kernel(const FvmMember* __restrict__ mem, int k, int rows) {
  pdl_wait();
  pdl_trigger();
  const FvmMember& m = mem[blockIdx.y];
  if (k >= m.steps) return;
  const FvmParams p = m.p;
  irfft_rows(p, blockIdx.x, rows, m.spec);
}

__global__ void __launch_bounds__(32 * kWarpRows)
    fvm_batch_div_rfft_warp_kernel(const FvmMember* __restrict__ mem, int k) {
  pdl_wait();
  pdl_trigger();
  __shared__ float2 tiles[kWarpRows][kWarpFftTile];
  const FvmMember& m = mem[blockIdx.y];
  if (k >= m.steps) return;
  const FvmParams p = m.p;
  const int dst = batch_dst(k), w = threadIdx.x >> 5;
  div_rfft_row_warp(p, blockIdx.x * kWarpRows + w, m.f[dst][0], m.f[dst][1], m.spec, tiles[w]);
}

__global__ void __launch_bounds__(32 * kWarpRows)
    fvm_batch_irfft_warp_kernel(const FvmMember* __restrict__ mem, int k) {
  pdl_wait();
  pdl_trigger();
  __shared__ float2 tiles[kWarpRows][kWarpFftTile];
  const FvmMember& m = mem[blockIdx.y];
  if (k >= m.steps) return;
  const FvmParams p = m.p;
  const int w = threadIdx.x >> 5;
  irfft_row_warp(p, blockIdx.x * kWarpRows + w, m.spec, tiles[w]);
}

__global__ void fvm_batch_project_out_kernel(const FvmMember* __restrict__ mem) {
  pdl_wait();
  pdl_trigger();
  const FvmMember& m = mem[blockIdx.y];
  if (m.steps <= 0) return;
  const FvmParams p = m.p;
  const int cur = batch_dst(m.steps - 1);
  project_out_cells(p, blockIdx.x, gridDim.x, m.f[cur][0], m.f[cur][1],
                    reinterpret_cast<const float*>(m.spec), m.f[0][0], m.f[0][1]);
}

// ---- Shared-memory-resident chunk for small grids ----
// One block per member runs the member's whole chunk with everything in
// shared memory: the state (u*, v* after each stencil), its projected copy,
// the packed row spectrum / pressure q, and the transform buffer.  Each phase
// evaluates the expressions of the per-step kernels -- the tiles' face fluxes
// and cell update (explicit_tile), div_rfft_rows, col_pinv_cols and
// irfft_rows on the same Stockham engine, project_out_cells -- so a member's
// bits equal those of the launch-per-step path; only the launches, the
// global round trips and the grid-wide step boundaries go away.
constexpr int kResidentThreads = 512;

CFD_HD size_t resident_smem(int nx, int ny) {
  const int L = ny / 2;
  const size_t n = (size_t)nx * ny;
  const size_t rows_w = (size_t)nx * padded_len(L);
  const size_t cols_w = (size_t)(L + 1) * padded_len(nx);
  return 5 * n * sizeof(float) + (rows_w > cols_w ? rows_w : cols_w) * sizeof(float2);
}

// x-face flux pair after row r at column j of the smem fields (u, v), as
// explicit_tile computes it: rows r-1 .. r+2 and u at (r, j+1).
template <int CONVECT>
CFD_D float2 resident_xface(const FvmParams& p, const float* __restrict__ su,
                            const float* __restrict__ sv, int r, int j) {
  const int mx = p.nx - 1, my = p.ny - 1, lg = p.log2ny;
  auto at = [&](int i, int jj) {
    const int k = ((i & mx) << lg) + (jj & my);
    return make_float2(su[k], sv[k]);
  };
  const float2 cm = at(r - 1, j), c0 = at(r, j), c1 = at(r + 1, j), c2 = at(r + 2, j);
  const float uy1 = su[((r & mx) << lg) + ((j + 1) & my)];
  const float2 U = mul2(splat2(0.5f), add2(splat2(c0.x), make_float2(c1.x, uy1)));
  if (CONVECT == 0) return tvd_flux2(cm, c0, c1, c2, U, p.cfl_x);
  const float2 cface = mul2(splat2(0.5f), add2(c0, c1));
  return mul2(make_float2(U.x, cface.y), make_float2(U.x, U.y));
}

// y-face flux pair after column j at row i: columns j-1 .. j+2 and v at
// (i+1, j).
template <int CONVECT>
CFD_D float2 resident_yface(const FvmParams& p, const float* __restrict__ su,
                            const float* __restrict__ sv, int i, int j) {
  const int mx = p.nx - 1, my = p.ny - 1, lg = p.log2ny;
  const int row = (i & mx) << lg;
  auto at = [&](int jj) {
    const int k = row + (jj & my);
    return make_float2(su[k], sv[k]);
  };
  const float2 cm = at(j - 1), c0 = at(j), c1 = at(j + 1), c2 = at(j + 2);
  const float vx1 = sv[(((i + 1) & mx) << lg) + (j & my)];
  const float2 V = mul2(splat2(0.5f), add2(splat2(c0.y), make_float2(vx1, c1.y)));
  if (CONVECT == 0) return tvd_flux2(cm, c0, c1, c2, V, p.cfl_y);
  const float2 cface = mul2(splat2(0.5f), add2(c0, c1));
  return mul2(make_float2(cface.x, V.y), make_float2(V.x, V.y));
}

// fft_inplace as a call: the resident kernel makes four transforms, and four
// inlined copies of the engine exhaust its registers (3 KB of stack and
// spills); as calls each keeps the engine's own allocation.
template <int SIGN>
__device__ __noinline__ void resident_fft(float2* buf, int log2L, int batch, int bstride,
                                          const float2* __restrict__ twp, int t) {
  fft_inplace<SIGN>(buf, log2L, batch, bstride, twp, t);
}

template <int CONVECT>
__global__ void __launch_bounds__(kResidentThreads, 1)
    fvm_batch_resident_kernel(const FvmMember* __restrict__ mem) {
  const FvmMember& m = mem[blockIdx.x];
  const int steps = m.steps;
  if (steps <= 0) return;  // uniform per block
  const FvmParams p = m.p;
  extern __shared__ float4 smem_resident[];
  const int nx = p.nx, ny = p.ny, L = ny >> 1, lg = p.log2ny, log2L = lg - 1;
  const int n = nx * ny, mx = nx - 1, my = ny - 1;
  float* const Au = reinterpret_cast<float*>(smem_resident);  // projected input
  float* const Av = Au + n;
  float* const Bu = Av + n;  // u*, v* after the stencil
  float* const Bv = Bu + n;
  float* const Q = Bv + n;  // packed row spectrum, then q
  float2* const Qc = reinterpret_cast<float2*>(Q);
  float2* const W = reinterpret_cast<float2*>(Q + n);
  const int tid = threadIdx.x, T = blockDim.x;
  const int PL = padded_len(L), CS = padded_len(nx);
  const float2 ihx = splat2(p.inv_hx), ihy = splat2(p.inv_hy);

  for (int idx = tid; idx < n; idx += T) {
    Au[idx] = m.f[0][0][idx];
    Av[idx] = m.f[0][1][idx];
  }
  __syncthreads();
#pragma unroll 1
  for (int k = 0; k < steps; ++k) {
    if (k > 0) {
      // u = u* - (q[i+1] - q[i]) / hx, v = v* - (q[j+1] - q[j]) / hy
      for (int idx = tid; idx < n; idx += T) {
        const int i = idx >> lg, j = idx & my;
        const float q0 = Q[idx];
        const float qx = Q[(((i + 1) & mx) << lg) + j], qy = Q[(i << lg) + ((j + 1) & my)];
        Au[idx] = Bu[idx] - (qx - q0) * p.inv_hx;
        Av[idx] = Bv[idx] - (qy - q0) * p.inv_hy;
      }
      __syncthreads();
    }
    // Explicit terms and forward Euler (equations.py:102-110): (A) -> (B).
    for (int idx = tid; idx < n; idx += T) {
      const int i = idx >> lg, j = idx & my;
      const float2 uv = make_float2(Au[idx], Av[idx]);
      const float2 fx_hi = resident_xface<CONVECT>(p, Au, Av, i, j);
      const float2 fx_lo = resident_xface<CONVECT>(p, Au, Av, i - 1, j);
      const float2 fy_hi = resident_yface<CONVECT>(p, Au, Av, i, j);
      const float2 fy_lo = resident_yface<CONVECT>(p, Au, Av, i, j - 1);
      const float2 dx = mul2(sub2(fx_hi, fx_lo), ihx);
      float2 kk = fma2(sub2(fy_hi, fy_lo), ihy, dx);
      kk = make_float2(-kk.x, -kk.y);
      const int up = (((i - 1) & mx) << lg) + j, dn = (((i + 1) & mx) << lg) + j;
      const int lf = (i << lg) + ((j - 1) & my), rt = (i << lg) + ((j + 1) & my);
      kk = add_diffusion_forcing<0>(p, kk, uv,
                                    add2(make_float2(Au[up], Av[up]), make_float2(Au[dn], Av[dn])),
                                    add2(make_float2(Au[lf], Av[lf]), make_float2(Au[rt], Av[rt])),
                                    i, j);
      const float2 nxt = fma2(splat2(p.dt), kk, uv);
      Bu[idx] = nxt.x;
      Bv[idx] = nxt.y;
    }
    __syncthreads();
    // Backward-difference divergence and packed row rFFT (div_rfft_rows).
    {
      const int log2g = lg - 2;
      for (int g = tid; g < (nx << log2g); g += T) {
        const int i = g >> log2g, jj = (g & ((1 << log2g) - 1)) << 2;
        const int a0 = (i << lg) + jj, b0 = (((i - 1) & mx) << lg) + jj;
        const float cm = Bv[(i << lg) + ((jj - 1) & my)];
        const float d0 = (Bu[a0] - Bu[b0]) * p.inv_hx + (Bv[a0] - cm) * p.inv_hy;
        const float d1 = (Bu[a0 + 1] - Bu[b0 + 1]) * p.inv_hx + (Bv[a0 + 1] - Bv[a0]) * p.inv_hy;
        const float d2 = (Bu[a0 + 2] - Bu[b0 + 2]) * p.inv_hx + (Bv[a0 + 2] - Bv[a0 + 1]) * p.inv_hy;
        const float d3 = (Bu[a0 + 3] - Bu[b0 + 3]) * p.inv_hx + (Bv[a0 + 3] - Bv[a0 + 2]) * p.inv_hy;
        float2* z = W + i * PL;
        z[pidx(jj >> 1)] = make_float2(d0, d1);
        z[pidx((jj >> 1) + 1)] = make_float2(d2, d3);
      }
      __syncthreads();
      resident_fft<-1>(W, log2L, nx, PL, p.twp_y, tid);
      const int half = L >> 1, log2h = log2L - 1;
      for (int idx = tid; idx < (nx << log2h); idx += T) {
        const int r = idx >> log2h, kq = idx & (half - 1);
        float2* out = Qc + r * L;
        const float2* z = W + r * PL;
        if (kq == 0) {
          const float2 z0 = z[0];
          out[0] = make_float2(z0.x + z0.y, z0.x - z0.y);
          float2 xk, xm;
          const float2 zh = z[pidx(half)];
          rfft_post_pair(zh, zh, __ldg(p.tw_y + half), &xk, &xm);
          out[half] = xk;
        } else {
          float2 xk, xm;
          rfft_post_pair(z[pidx(kq)], z[pidx(L - kq)], __ldg(p.tw_y + kq), &xk, &xm);
          out[kq] = xk;
          out[L - kq] = xm;
        }
      }
      __syncthreads();
    }
    // Column pass (col_pinv_cols): the L complex columns, the DC column
    // (column 0's real parts) and the Nyquist column (its imaginary parts) as
    // L + 1 sequences.
    {
      for (int idx = tid; idx < (L + 1) * nx; idx += T) {
        const int i = idx / (L + 1), w = idx - i * (L + 1);
        float2 x;
        if (w == L) x = make_float2(Q[i * L * 2 + 1], 0.f);
        else if (w == 0) x = make_float2(Q[i * L * 2], 0.f);
        else x = Qc[i * L + w];
        W[w * CS + pidx(i)] = x;
      }
      __syncthreads();
      resident_fft<-1>(W, p.log2nx, L + 1, CS, p.twp_x, tid);
      for (int idx = tid; idx < (L + 1) * nx; idx += T) {
        const int kx = idx / (L + 1), w = idx - kx * (L + 1);
        float2* e = W + w * CS + pidx(kx);
        *e = c_scale(*e, pinv_diag(p, kx, w));
      }
      __syncthreads();
      resident_fft<1>(W, p.log2nx, L + 1, CS, p.twp_x, tid);
      for (int idx = tid; idx < (L + 1) * nx; idx += T) {
        const int i = idx / (L + 1), w = idx - i * (L + 1);
        const float2 x = W[w * CS + pidx(i)];
        if (w == L) Q[i * L * 2 + 1] = x.x;
        else if (w == 0) Q[i * L * 2] = x.x;
        else Qc[i * L + w] = x;
      }
      __syncthreads();
    }
    // Packed row irFFT -> q (irfft_rows).
    {
      const int half = L >> 1, log2h = log2L - 1;
      for (int idx = tid; idx < (nx << log2h); idx += T) {
        const int r = idx >> log2h, kq = idx & (half - 1);
        const float2* in = Qc + r * L;
        float2* z = W + r * PL;
        if (kq == 0) {
          const float2 x0 = in[0];
          z[0] = make_float2(x0.x + x0.y, x0.x - x0.y);
          const float2 xh = in[half];
          float2 zk, zm;
          irfft_pre_pair(xh, xh, __ldg(p.tw_y + half), &zk, &zm);
          z[pidx(half)] = zk;
        } else {
          float2 zk, zm;
          irfft_pre_pair(in[kq], in[L - kq], __ldg(p.tw_y + kq), &zk, &zm);
          z[pidx(kq)] = zk;
          z[pidx(L - kq)] = zm;
        }
      }
      __syncthreads();
      resident_fft<1>(W, log2L, nx, PL, p.twp_y, tid);
      for (int idx = tid; idx < nx * L; idx += T) {
        const int r = idx / L, nn = idx - r * L;
        const float2 a = W[r * PL + pidx(nn)];
        Q[r * ny + 2 * nn] = a.x;
        Q[r * ny + 2 * nn + 1] = a.y;
      }
      __syncthreads();
    }
  }
  // The chunk's final projection (project_out_cells) into the state.
  for (int idx = tid; idx < n; idx += T) {
    const int i = idx >> lg, j = idx & my;
    const float q0 = Q[idx];
    const float qx = Q[(((i + 1) & mx) << lg) + j], qy = Q[(i << lg) + ((j + 1) & my)];
    m.f[0][0][idx] = Bu[idx] - (qx - q0) * p.inv_hx;
    m.f[0][1][idx] = Bv[idx] - (qy - q0) * p.inv_hy;
  }
}

int fft_rows_per_block(int log2L, int nrows, int target_threads = 256) {
  const int P = log2L >= 4 ? 16 : (1 << log2L);
  int rows = (target_threads * P) >> log2L;
  if (rows < 1) rows = 1;
  if (rows > nrows) rows = nrows;
  return rows;
}

int block_threads(int workers) {
  int t = ((workers + 31) / 32) * 32;
  return t < 64 ? 64 : t;
}

template <typename K>
cudaError_t set_smem(K kernel, size_t bytes) {
  if (bytes > 48 * 1024)
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)bytes);
  return cudaSuccess;
}

}  // namespace

template <bool PR, bool K0, int CV, int FO>
static void launch_explicit_variant(const FvmParams& p, bool stream, bool tiled, dim3 grid,
                                    const float* ua, const float* va, const float* q,
                                    float* uo, float* vo, cudaStream_t s) {
  if (stream) {
    const int sh = stream_rows_of(p.stream_rows);
    const long long warps = (long long)((p.ny + kStreamCols - 1) / kStreamCols) * (p.nx / sh);
    const dim3 grid_s((int)((warps + 3) / 4));
    if (sh == 8)
      launch_maybe_pdl(p.pdl, fvm_explicit_stream_kernel<PR, CV, FO, 8>, grid_s, dim3(128), 0, s,
                       p, ua, va, q, uo, vo);
    else if (sh == 32)
      launch_maybe_pdl(p.pdl, fvm_explicit_stream_kernel<PR, CV, FO, 32>, grid_s, dim3(128), 0, s,
                       p, ua, va, q, uo, vo);
    else
      launch_maybe_pdl(p.pdl, fvm_explicit_stream_kernel<PR, CV, FO, kStreamRows>, grid_s,
                       dim3(128), 0, s, p, ua, va, q, uo, vo);
  } else if (tiled) {
    fvm_explicit_tiled_kernel<PR, K0, CV, FO><<<grid, kStencilThreads, 0, s>>>(p, ua, va, q, uo,
                                                                               vo);
  } else {
    fvm_explicit_kernel<PR, K0, CV><<<grid, kStencilThreads, 0, s>>>(p, ua, va, q, uo, vo);
  }
}

cudaError_t launch_fvm_explicit(const FvmParams& p, bool project, bool out_k0,
                                const float* ua, const float* va,
                                const float* q, float* uo, float* vo,
                                cudaStream_t s) {
  const bool stream = p.stencil == 1 && !out_k0 && stream_ok(p);
  const bool tiled = p.nx % kTI == 0 && p.ny % kTJ == 0;
  const int ti = tiled ? kTI : (p.nx < kTI ? p.nx : kTI);
  const int tj = tiled ? kTJ : (p.ny < kTJ ? p.ny : kTJ);
  const dim3 grid(p.ny / tj, p.nx / ti);
  const bool ko = kolmogorov_config(p) && !out_k0;
#define CFD_EXPLICIT(PR, K0, CV)                                                          \
  do {                                                                                    \
    if (ko) launch_explicit_variant<PR, K0, CV, 1>(p, stream, tiled, grid, ua, va, q, uo, vo, s); \
    else launch_explicit_variant<PR, K0, CV, 0>(p, stream, tiled, grid, ua, va, q, uo, vo, s);    \
  } while (0)
  if (p.convect == 0) {
    if (project) {
      if (out_k0) CFD_EXPLICIT(true, true, 0); else CFD_EXPLICIT(true, false, 0);
    } else {
      if (out_k0) CFD_EXPLICIT(false, true, 0); else CFD_EXPLICIT(false, false, 0);
    }
  } else {
    if (project) {
      if (out_k0) CFD_EXPLICIT(true, true, 1); else CFD_EXPLICIT(true, false, 1);
    } else {
      if (out_k0) CFD_EXPLICIT(false, true, 1); else CFD_EXPLICIT(false, false, 1);
    }
  }
#undef CFD_EXPLICIT
  return cudaGetLastError();
}

// Block shapes of the transform kernels (FvmParams::fft_shape): 0 = wide
// (256-thread blocks, up to 85 registers), 1 = narrow (64-thread row blocks
// and 128-thread column blocks capped at 72 registers).
template <int MAXT, int MINB>
static cudaError_t div_rfft_impl(const FvmParams& p, int target, const float* us,
                                 const float* vs, float2* spec, cudaStream_t s) {
  const int log2L = p.log2ny - 1;
  if (warp_rows_ok(p)) {
    return launch_maybe_pdl(p.pdl, fvm_div_rfft_warp_kernel, dim3(p.nx / kWarpRows),
                            dim3(32 * kWarpRows), 0, s, p, us, vs, spec);
  }
  const int rows = fft_rows_per_block(log2L, p.nx, target);
  const bool aligned = (((uintptr_t)us | (uintptr_t)vs | (uintptr_t)spec) & 15) == 0;
  if (p.row_feed == 1 && aligned && !p.row_field) {
    const size_t smem = div_rfft_bulk_smem(p.ny, rows);
    cudaError_t e = set_smem(fvm_div_rfft_bulk_kernel<MAXT, MINB>, smem);
    if (e != cudaSuccess) return e;
    fvm_div_rfft_bulk_kernel<MAXT, MINB><<<p.nx / rows, block_threads(fft_workers(log2L, rows)),
                                           smem, s>>>(p, rows, us, vs, spec);
    return cudaGetLastError();
  }
  const size_t smem = (size_t)rows * padded_len(p.ny / 2) * sizeof(float2);
  cudaError_t e = set_smem(fvm_div_rfft_kernel<MAXT, MINB>, smem);
  if (e != cudaSuccess) return e;
  fvm_div_rfft_kernel<MAXT, MINB><<<p.nx / rows, block_threads(fft_workers(log2L, rows)),
                                    smem, s>>>(p, rows, us, vs, spec);
  return cudaGetLastError();
}

cudaError_t launch_fvm_field_rfft(const FvmParams& p, const float* f, float2* spec,
                                  cudaStream_t s) {
  FvmParams q = p;
  q.row_field = 1;
  const int log2L = q.log2ny - 1;
  const int rows = fft_rows_per_block(log2L, q.nx, 256);
  const size_t smem = (size_t)rows * padded_len(q.ny / 2) * sizeof(float2);
  cudaError_t e = set_smem(fvm_div_rfft_kernel<256, 3>, smem);
  if (e != cudaSuccess) return e;
  fvm_div_rfft_kernel<256, 3><<<q.nx / rows, block_threads(fft_workers(log2L, rows)), smem, s>>>(
      q, rows, f, f, spec);
  return cudaGetLastError();
}

cudaError_t launch_fvm_div_rfft(const FvmParams& p, const float* us,
                                const float* vs, float2* spec, cudaStream_t s) {
  return p.fft_shape == 1 ? div_rfft_impl<64, 14>(p, 64, us, vs, spec, s)
                          : div_rfft_impl<256, 3>(p, 256, us, vs, spec, s);
}

template <int MAXT, int MINB>
static cudaError_t col_pinv_impl(const FvmParams& p, int target, float2* spec,
                                 cudaStream_t s) {
  const int L = p.ny / 2;
  // W columns per block so that the block has `target` threads (W * nx =
  // 16 * target points); one column at least.
  int W = (16 * target) >> p.log2nx;
  if (W < 1) W = 1;
  if (W > L) W = L;
  // +8 slots: consecutive columns start 16 banks apart.
  const int bstride = padded_len(p.nx) + 8;
  const size_t smem = (size_t)W * bstride * sizeof(float2);
  cudaError_t e = set_smem(fvm_col_pinv_kernel<MAXT, MINB>, smem);
  if (e != cudaSuccess) return e;
  // L / W column groups plus the Nyquist block
  fvm_col_pinv_kernel<MAXT, MINB><<<L / W + 1, block_threads(fft_workers(p.log2nx, W)), smem,
                                    s>>>(p, W, ilog2(W), bstride, spec);
  return cudaGetLastError();
}

template <int CL>
static cudaError_t col_pinv_cluster_impl(const FvmParams& p, float2* spec, cudaStream_t s) {
  const int L = p.ny / 2;
  const size_t smem = (size_t)padded_len(p.nx) * sizeof(float2);
  cudaError_t e = set_smem(fvm_col_pinv_cluster_kernel<CL>, smem);
  if (e != cudaSuccess) return e;
  // L columns plus the Nyquist cluster
  fvm_col_pinv_cluster_kernel<CL><<<L + CL, block_threads(fft_workers(p.log2nx, 1)), smem, s>>>(
      p, spec);
  return cudaGetLastError();
}

bool col_cluster_ok(const FvmParams& p, int cl) {
  // One column per block with nx/16 <= 128 workers; nx/CL rows per block.
  return p.nx >= 256 && p.nx <= 2048 && (p.ny / 2) % cl == 0;
}

// Persistent column pass: as many blocks as fit on the device at once (one
// per multiprocessor at 2048 rows), never more than there are groups.
template <int LOG2N, int CG>
static cudaError_t col_pinv_pipe_impl(const FvmParams& p, float2* spec, cudaStream_t s) {
  const size_t smem = col_pipe_smem<LOG2N, CG>();
  const int threads = CG * (1 << LOG2N) / 16;
  auto kern = fvm_col_pinv_pipe_kernel<LOG2N, CG>;
  cudaError_t e = set_smem(kern, smem);
  if (e != cudaSuccess) return e;
  static std::atomic<int> per_sm_cache{0};  // per instantiation
  int per_sm = 1;
  e = cached_blocks_per_sm(kern, threads, smem, per_sm_cache, &per_sm);
  if (e != cudaSuccess) return e;
  const int groups = p.ny / 2 / CG + 1;
  const int slots = col_pipe_device_sms() * per_sm;
  return launch_maybe_pdl(p.pdl, kern, dim3(groups < slots ? groups : slots), dim3(threads), smem,
                          s, p, spec);
}

// Column groups of the persistent pass: 4 columns per block (wide, col_mode
// 3; 2 at 4096 rows) or 2 (narrow, col_mode 4: two independent blocks per
// multiprocessor at 2048 rows, so their barriers do not stall one another).
bool col_pipe_ok(const FvmParams& p, int narrow) {
  const int cg = (narrow || p.log2nx == 12) ? 2 : 4;
  return p.log2nx >= 8 && p.log2nx <= 12 && (p.ny / 2) % cg == 0;
}

bool col_tma_grid_ok(const FvmParams& p) {
  return p.log2nx >= 8 && p.log2nx <= 11 && (p.ny / 2) % 4 == 0;
}

// The narrow transform blocks hold one row's ny/32 workers in 64 threads and
// one column's nx/16 workers in 128 threads: rows up to 2048 (at 2048 the
// one-warp row kernels run whatever the shape) and, for the per-block column
// pass, columns up to 2048.  The wide blocks (256 threads) hold either at
// 4096.
bool fft_shape_ok(const FvmParams& p) {
  if (p.fft_shape != 1) return true;
  const bool rows = warp_rows_ok(p) || p.ny <= 2048;
  const bool cols = p.col_mode != 0 || p.nx <= 2048;
  return rows && cols;
}

template <int LOG2N>
static cudaError_t col_pinv_tma_impl(const FvmParams& p, float2* spec, cudaStream_t s) {
  const size_t smem = col_pipe_smem<LOG2N, 4>() + 16;  // + the mbarrier
  const int threads = 4 * (1 << LOG2N) / 16;
  auto kern = fvm_col_pinv_tma_kernel<LOG2N>;
  cudaError_t e = set_smem(kern, smem);
  if (e != cudaSuccess) return e;
  static std::atomic<int> per_sm_cache{0};  // per instantiation
  int per_sm = 1;
  e = cached_blocks_per_sm(kern, threads, smem, per_sm_cache, &per_sm);
  if (e != cudaSuccess) return e;
  const int groups = p.ny / 2 / 4 + 1;
  const int slots = col_pipe_device_sms() * per_sm;
  const CUtensorMap map = *static_cast<const CUtensorMap*>(p.col_tmap);
  return launch_maybe_pdl(p.pdl, kern, dim3(groups < slots ? groups : slots), dim3(threads), smem,
                          s, p, spec, map);
}

static cudaError_t col_pinv_tma_launch(const FvmParams& p, float2* spec, cudaStream_t s) {
  switch (p.log2nx) {
    case 8: return col_pinv_tma_impl<8>(p, spec, s);
    case 9: return col_pinv_tma_impl<9>(p, spec, s);
    case 10: return col_pinv_tma_impl<10>(p, spec, s);
    default: return col_pinv_tma_impl<11>(p, spec, s);
  }
}

static cudaError_t col_pinv_pipe_launch(const FvmParams& p, float2* spec, cudaStream_t s) {
  if (p.col_mode == 4) {
    switch (p.log2nx) {
      case 8: return col_pinv_pipe_impl<8, 2>(p, spec, s);
      case 9: return col_pinv_pipe_impl<9, 2>(p, spec, s);
      case 10: return col_pinv_pipe_impl<10, 2>(p, spec, s);
      case 11: return col_pinv_pipe_impl<11, 2>(p, spec, s);
      default: return col_pinv_pipe_impl<12, 2>(p, spec, s);
    }
  }
  switch (p.log2nx) {
    case 8: return col_pinv_pipe_impl<8, 4>(p, spec, s);
    case 9: return col_pinv_pipe_impl<9, 4>(p, spec, s);
    case 10: return col_pinv_pipe_impl<10, 4>(p, spec, s);
    case 11: return col_pinv_pipe_impl<11, 4>(p, spec, s);
    default: return col_pinv_pipe_impl<12, 2>(p, spec, s);
  }
}

// col_mode 1/2: clusters of 4/8 single-column blocks; 3/4: the persistent
// register-pipelined pass with 4 / 2 columns per block.
cudaError_t launch_fvm_col_pinv(const FvmParams& p, float2* spec,
                                cudaStream_t s) {
  if (p.col_mode == 5 && p.col_tmap && p.col_tmap_spec == spec && col_tma_grid_ok(p))
    return col_pinv_tma_launch(p, spec, s);
  if ((p.col_mode == 3 || p.col_mode == 4) && col_pipe_ok(p, p.col_mode == 4))
    return col_pinv_pipe_launch(p, spec, s);
  if (p.col_mode == 2 && col_cluster_ok(p, 8)) return col_pinv_cluster_impl<8>(p, spec, s);
  if ((p.col_mode == 1 || p.col_mode == 2) && col_cluster_ok(p, 4))
    return col_pinv_cluster_impl<4>(p, spec, s);
  return p.fft_shape == 1 ? col_pinv_impl<128, 7>(p, 128, spec, s)
                          : col_pinv_impl<256, 3>(p, 256, spec, s);
}

template <int MAXT, int MINB>
static cudaError_t irfft_impl(const FvmParams& p, int target, float2* spec,
                              cudaStream_t s) {
  const int log2L = p.log2ny - 1;
  if (warp_rows_ok(p)) {
    return launch_maybe_pdl(p.pdl, fvm_irfft_warp_kernel, dim3(p.nx / kWarpRows),
                            dim3(32 * kWarpRows), 0, s, p, spec);
  }
  const int rows = fft_rows_per_block(log2L, p.nx, target);
  if (p.row_feed == 1 && (((uintptr_t)spec) & 15) == 0) {
    const size_t smem = irfft_bulk_smem(p.ny, rows);
    cudaError_t e = set_smem(fvm_irfft_bulk_kernel<MAXT, MINB>, smem);
    if (e != cudaSuccess) return e;
    fvm_irfft_bulk_kernel<MAXT, MINB><<<p.nx / rows, block_threads(fft_workers(log2L, rows)),
                                        smem, s>>>(p, rows, spec);
    return cudaGetLastError();
  }
  const size_t smem = (size_t)rows * padded_len(p.ny / 2) * sizeof(float2);
  cudaError_t e = set_smem(fvm_irfft_kernel<MAXT, MINB>, smem);
  if (e != cudaSuccess) return e;
  fvm_irfft_kernel<MAXT, MINB><<<p.nx / rows, block_threads(fft_workers(log2L, rows)),
                                 smem, s>>>(p, rows, spec);
  return cudaGetLastError();
}

cudaError_t launch_fvm_irfft(const FvmParams& p, float2* spec, cudaStream_t s) {
  return p.fft_shape == 1 ? irfft_impl<64, 14>(p, 64, spec, s)
                          : irfft_impl<256, 3>(p, 256, spec, s);
}

static int elementwise_blocks(size_t n) {
  size_t b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return (int)b;
}

cudaError_t launch_fvm_project_out(const FvmParams& p, const float* us,
                                   const float* vs, const float* q, float* uo,
                                   float* vo, cudaStream_t s) {
  const size_t n = (size_t)p.nx * p.ny;
  return launch_maybe_pdl(p.pdl, fvm_project_out_kernel, dim3(elementwise_blocks(n)), dim3(256),
                          0, s, p, us, vs, q, uo, vo);
}

cudaError_t launch_fvm_add(size_t n, const float* w, float* u, cudaStream_t s) {
  fvm_add_kernel<<<elementwise_blocks(n), 256, 0, s>>>(n, w, u);
  return cudaGetLastError();
}

cudaError_t launch_fvm_rk_combine(const FvmParams& p, const float* u0, const float* v0,
                                  const RkCombine& cb, float* uo, float* vo, cudaStream_t s) {
  if (cb.count < 0 || cb.count > 4) return cudaErrorInvalidValue;
  const size_t n = (size_t)p.nx * p.ny;
  fvm_rk_combine_kernel<<<elementwise_blocks(n), 256, 0, s>>>(p, u0, v0, cb, uo, vo);
  return cudaGetLastError();
}

cudaError_t launch_divergence(const FvmParams& p, const float* u,
                              const float* v, float* out, cudaStream_t s) {
  const size_t n = (size_t)p.nx * p.ny;
  divergence_kernel<<<elementwise_blocks(n), 256, 0, s>>>(p, u, v, out);
  return cudaGetLastError();
}

cudaError_t launch_curl2d(const FvmParams& p, const float* u, const float* v,
                          float* out, cudaStream_t s) {
  const size_t n = (size_t)p.nx * p.ny;
  curl2d_kernel<<<elementwise_blocks(n), 256, 0, s>>>(p, u, v, out);
  return cudaGetLastError();
}

cudaError_t launch_max_speed(int n, const float* u, const float* v,
                             unsigned int* out_bits, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(out_bits, 0, sizeof(unsigned int), s);
  if (e != cudaSuccess) return e;
  max_speed_kernel<<<elementwise_blocks((size_t)n), 256, 0, s>>>(n, u, v, out_bits);
  return cudaGetLastError();
}

bool stream_stencil_ok(const FvmParams& p) { return stream_ok(p); }

bool bulk_feed_ok(const FvmParams& p) {
  // Whole rows move by bulk copies: 16-byte multiples, and the staged rows of
  // the widest block shape must fit in shared memory.
  const int log2L = p.log2ny - 1;
  if (p.ny < 8 || warp_rows_ok(p)) return false;
  const int rows = fft_rows_per_block(log2L, p.nx, 256);
  // mbarrier transaction counts stay below 2^20 bytes.
  const size_t tx = (size_t)(2 * rows + 1) * p.ny * 4;
  return div_rfft_bulk_smem(p.ny, rows) <= 200 * 1024 && tx < (1u << 20);
}

bool fvm_batch_shape_ok(const FvmParams& p) {
  return p.nx % kTI == 0 && p.ny % kTJ == 0;
}

template <int MAXT, int MINB>
static cudaError_t batch_rows_impl(const FvmParams& p, int target, const FvmMember* mem,
                                   int count, int k, bool inverse, cudaStream_t s) {
  const int log2L = p.log2ny - 1;
  if (warp_rows_ok(p)) {
    const dim3 wgrid(p.nx / kWarpRows, count);
    if (inverse)
      launch_maybe_pdl(p.pdl, fvm_batch_irfft_warp_kernel, wgrid, dim3(32 * kWarpRows), 0, s, mem, k);
    else
      launch_maybe_pdl(p.pdl, fvm_batch_div_rfft_warp_kernel, wgrid, dim3(32 * kWarpRows), 0, s, mem,
                       k);
    return cudaGetLastError();
  }
  const int rows = fft_rows_per_block(log2L, p.nx, target);
  const size_t smem = (size_t)rows * padded_len(p.ny / 2) * sizeof(float2);
  const dim3 grid(p.nx / rows, count);
  const int threads = block_threads(fft_workers(log2L, rows));
  cudaError_t e;
  if (p.row_feed == 1 && bulk_feed_ok(p)) {
    if (inverse) {
      const size_t bs = irfft_bulk_smem(p.ny, rows);
      if ((e = set_smem(fvm_batch_irfft_bulk_kernel<MAXT, MINB>, bs)) != cudaSuccess) return e;
      launch_maybe_pdl(p.pdl, fvm_batch_irfft_bulk_kernel<MAXT, MINB>, grid, dim3(threads), bs, s,
                       mem, k, rows);
    } else {
      const size_t bs = div_rfft_bulk_smem(p.ny, rows);
      if ((e = set_smem(fvm_batch_div_rfft_bulk_kernel<MAXT, MINB>, bs)) != cudaSuccess) return e;
      launch_maybe_pdl(p.pdl, fvm_batch_div_rfft_bulk_kernel<MAXT, MINB>, grid, dim3(threads), bs,
                       s, mem, k, rows);
    }
    return cudaGetLastError();
  }
  if (inverse) {
    if ((e = set_smem(fvm_batch_irfft_kernel<MAXT, MINB>, smem)) != cudaSuccess) return e;
    launch_maybe_pdl(p.pdl, fvm_batch_irfft_kernel<MAXT, MINB>, grid, dim3(threads), smem, s, mem, k,
                     rows);
  } else {
    if ((e = set_smem(fvm_batch_div_rfft_kernel<MAXT, MINB>, smem)) != cudaSuccess) return e;
    launch_maybe_pdl(p.pdl, fvm_batch_div_rfft_kernel<MAXT, MINB>, grid, dim3(threads), smem, s, mem,
                     k, rows);
  }
  return cudaGetLastError();
}

template <int MAXT, int MINB>
static cudaError_t batch_col_impl(const FvmParams& p, int target, const FvmMember* mem,
                                  int count, int k, cudaStream_t s) {
  const int L = p.ny / 2;
  int W = (16 * target) >> p.log2nx;
  if (W < 1) W = 1;
  if (W > L) W = L;
  const int bstride = padded_len(p.nx) + 8;
  const size_t smem = (size_t)W * bstride * sizeof(float2);
  cudaError_t e = set_smem(fvm_batch_col_pinv_kernel<MAXT, MINB>, smem);
  if (e != cudaSuccess) return e;
  launch_maybe_pdl(p.pdl, fvm_batch_col_pinv_kernel<MAXT, MINB>, dim3(L / W + 1, count),
                   dim3(block_threads(fft_workers(p.log2nx, W))), smem, s, mem, k, W, ilog2(W),
                   bstride);
  return cudaGetLastError();
}

template <int CL>
static cudaError_t batch_col_cluster_impl(const FvmParams& p, const FvmMember* mem, int count,
                                          int k, cudaStream_t s) {
  const size_t smem = (size_t)padded_len(p.nx) * sizeof(float2);
  cudaError_t e = set_smem(fvm_batch_col_pinv_cluster_kernel<CL>, smem);
  if (e != cudaSuccess) return e;
  launch_maybe_pdl(p.pdl, fvm_batch_col_pinv_cluster_kernel<CL>, dim3(p.ny / 2 + CL, count),
                   dim3(block_threads(fft_workers(p.log2nx, 1))), smem, s, mem, k);
  return cudaGetLastError();
}

template <int LOG2N, int CG>
static cudaError_t batch_col_pipe_impl(const FvmParams& p, const FvmMember* mem, int count,
                                       int k, cudaStream_t s) {
  const size_t smem = col_pipe_smem<LOG2N, CG>();
  const int threads = CG * (1 << LOG2N) / 16;
  auto kern = fvm_batch_col_pinv_pipe_kernel<LOG2N, CG>;
  cudaError_t e = set_smem(kern, smem);
  if (e != cudaSuccess) return e;
  static std::atomic<int> per_sm_cache{0};  // per instantiation
  int per_sm = 1;
  e = cached_blocks_per_sm(kern, threads, smem, per_sm_cache, &per_sm);
  if (e != cudaSuccess) return e;
  const long long items = (long long)count * (p.ny / 2 / CG + 1);
  const long long slots = (long long)col_pipe_device_sms() * per_sm;
  return launch_maybe_pdl(p.pdl, kern, dim3((int)(items < slots ? items : slots)), dim3(threads),
                          smem, s, mem, count, k);
}

static cudaError_t batch_col_pipe_launch(const FvmParams& p, const FvmMember* mem, int count,
                                         int k, cudaStream_t s) {
  switch (p.log2nx) {
    case 8: return batch_col_pipe_impl<8, 4>(p, mem, count, k, s);
    case 9: return batch_col_pipe_impl<9, 4>(p, mem, count, k, s);
    case 10: return batch_col_pipe_impl<10, 4>(p, mem, count, k, s);
    case 11: return batch_col_pipe_impl<11, 4>(p, mem, count, k, s);
    default: return batch_col_pipe_impl<12, 2>(p, mem, count, k, s);
  }
}

template <int LOG2N>
static cudaError_t batch_col_tma_impl(const FvmParams& p, const FvmMember* mem, int count, int k,
                                      cudaStream_t s) {
  const size_t smem = col_pipe_smem<LOG2N, 4>() + 16;  // + the mbarrier
  const int threads = 4 * (1 << LOG2N) / 16;
  auto kern = fvm_batch_col_pinv_tma_kernel<LOG2N>;
  cudaError_t e = set_smem(kern, smem);
  if (e != cudaSuccess) return e;
  static std::atomic<int> per_sm_cache{0};  // per instantiation
  int per_sm = 1;
  e = cached_blocks_per_sm(kern, threads, smem, per_sm_cache, &per_sm);
  if (e != cudaSuccess) return e;
  const long long items = (long long)count * (p.ny / 2 / 4 + 1);
  const long long slots = (long long)col_pipe_device_sms() * per_sm;
  const CUtensorMap map = *static_cast<const CUtensorMap*>(p.col_tmap);
  return launch_maybe_pdl(p.pdl, kern, dim3((int)(items < slots ? items : slots)), dim3(threads),
                          smem, s, mem, count, k, map);
}

static cudaError_t batch_col_tma_launch(const FvmParams& p, const FvmMember* mem, int count,
                                        int k, cudaStream_t s) {
  switch (p.log2nx) {
    case 8: return batch_col_tma_impl<8>(p, mem, count, k, s);
    case 9: return batch_col_tma_impl<9>(p, mem, count, k, s);
    case 10: return batch_col_tma_impl<10>(p, mem, count, k, s);
    default: return batch_col_tma_impl<11>(p, mem, count, k, s);
  }
}

bool fvm_batch_resident_ok(const FvmParams& p) {
  return fvm_batch_shape_ok(p) && resident_smem(p.nx, p.ny) <= 227 * 1024;
}

cudaError_t launch_fvm_batch_resident(const FvmParams& p, const FvmMember* mem, int count,
                                      cudaStream_t s) {
  if (!fvm_batch_resident_ok(p) || count < 1) return cudaErrorInvalidValue;
  const size_t smem = resident_smem(p.nx, p.ny);
  if (p.convect == 0) {
    cudaError_t e = set_smem(fvm_batch_resident_kernel<0>, smem);
    if (e != cudaSuccess) return e;
    fvm_batch_resident_kernel<0><<<count, kResidentThreads, smem, s>>>(mem);
  } else {
    cudaError_t e = set_smem(fvm_batch_resident_kernel<1>, smem);
    if (e != cudaSuccess) return e;
    fvm_batch_resident_kernel<1><<<count, kResidentThreads, smem, s>>>(mem);
  }
  return cudaGetLastError();
}

cudaError_t launch_fvm_batch_step(const FvmParams& p, const FvmMember* mem, int count, int k,
                                  cudaStream_t s) {
  if (!fvm_batch_shape_ok(p) || count < 1 || count > 65535) return cudaErrorInvalidValue;
  if (p.stencil == 1 && stream_ok(p)) {
    const long long warps =
        (long long)((p.ny + kStreamCols - 1) / kStreamCols) * ((p.nx + kStreamRows - 1) / kStreamRows);
    const dim3 sg((unsigned)((warps + 3) / 4), count);
    if (p.convect == 0) {
      if (k > 0) launch_maybe_pdl(p.pdl, fvm_batch_explicit_stream_kernel<true, 0>, sg, dim3(128), 0, s, mem, k);
      else launch_maybe_pdl(p.pdl, fvm_batch_explicit_stream_kernel<false, 0>, sg, dim3(128), 0, s, mem, k);
    } else {
      if (k > 0) launch_maybe_pdl(p.pdl, fvm_batch_explicit_stream_kernel<true, 1>, sg, dim3(128), 0, s, mem, k);
      else launch_maybe_pdl(p.pdl, fvm_batch_explicit_stream_kernel<false, 1>, sg, dim3(128), 0, s, mem, k);
    }
  } else {
    const dim3 grid(p.ny / kTJ, p.nx / kTI, count);
    if (p.convect == 0) {
      if (k > 0) launch_maybe_pdl(p.pdl, fvm_batch_explicit_kernel<true, 0>, grid, dim3(kStencilThreads), 0, s,
                         mem, k);
      else launch_maybe_pdl(p.pdl, fvm_batch_explicit_kernel<false, 0>, grid, dim3(kStencilThreads), 0, s,
                         mem, k);
    } else {
      if (k > 0) launch_maybe_pdl(p.pdl, fvm_batch_explicit_kernel<true, 1>, grid, dim3(kStencilThreads), 0, s,
                         mem, k);
      else launch_maybe_pdl(p.pdl, fvm_batch_explicit_kernel<false, 1>, grid, dim3(kStencilThreads), 0, s,
                         mem, k);
    }
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = p.fft_shape == 1 ? batch_rows_impl<64, 14>(p, 64, mem, count, k, false, s)
                       : batch_rows_impl<256, 3>(p, 256, mem, count, k, false, s);
  if (e != cudaSuccess) return e;
  if (p.col_mode == 5 && p.col_tmap && col_tma_grid_ok(p))
    e = batch_col_tma_launch(p, mem, count, k, s);
  else if (p.col_mode == 3 && col_pipe_ok(p, 0)) e = batch_col_pipe_launch(p, mem, count, k, s);
  else if (p.col_mode == 2 && col_cluster_ok(p, 8)) e = batch_col_cluster_impl<8>(p, mem, count, k, s);
  else if ((p.col_mode == 1 || p.col_mode == 2) && col_cluster_ok(p, 4))
    e = batch_col_cluster_impl<4>(p, mem, count, k, s);
  else e = p.fft_shape == 1 ? batch_col_impl<128, 7>(p, 128, mem, count, k, s)
                            : batch_col_impl<256, 3>(p, 256, mem, count, k, s);
  if (e != cudaSuccess) return e;
  return p.fft_shape == 1 ? batch_rows_impl<64, 14>(p, 64, mem, count, k, true, s)
                          : batch_rows_impl<256, 3>(p, 256, mem, count, k, true, s);
}

cudaError_t launch_fvm_batch_project_out(const FvmParams& p, const FvmMember* mem, int count,
                                         cudaStream_t s) {
  if (count < 1 || count > 65535) return cudaErrorInvalidValue;
  const size_t n = (size_t)p.nx * p.ny;
  int per = (int)((n + 255) / 256);
  const int cap = (152 * 16 + count - 1) / count;
  if (per > cap) per = cap;
  if (per < 1) per = 1;
  return launch_maybe_pdl(p.pdl, fvm_batch_project_out_kernel, dim3(per, count), dim3(256), 0, s,
                          mem);
}

}  // namespace cfd
