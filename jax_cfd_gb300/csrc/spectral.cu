// Pseudospectral NavierStokes2D kernels (jax_cfd/spectral/equations.py:129-220,
// spectral/utils.py:128-203, spectral/time_stepping.py:117-197).
//
// The state is the rfftn of the vorticity, complex64 [nx, ny/2 + 1]
// (axis 0 = kx, full FFT; axis 1 = ky, half spectrum).  One low-storage
// Runge-Kutta / Crank-Nicolson stage is two launches:
//
//   col pass  (per ky column)  FFT_x of the advection row spectra,
//             * 2/3 filter, + forcing curl, h = F + beta h,
//             u = (u + gamma dt h + mu L u) / (1 - mu L);
//             then, for the next stage, the four x-inverse transforms of
//             A = psi^, B = kx psi^, C = kx w^, D = w^ (psi^ = -w^/lap).
//   row pass  (per x row)      apply the ky factors (vx = i ky A, vy = -i B,
//             gx = i C, gy = i ky D, all times 2 pi), four inverse real
//             FFTs, advection = -(gx vx + gy vy), forward real FFT.
//
// Multiplying by a function of ky commutes with the x transforms, so the ky
// factors are applied on the row side.  All transforms are unnormalised; the
// irfftn 1/(nx*ny) is a power of two applied once to the product.
#include <cooperative_groups.h>
#include <cstring>
#include <type_traits>
#include <cuda.h>

#include "bulk.cuh"
#include "colpipe.cuh"
#include "fft.cuh"
#include "kernels.h"

namespace cg = cooperative_groups;

namespace cfd {
namespace {

// fftfreq / rfftfreq ordinals over float32(step * n) (grids.py:618-658),
// tabulated on the host in float32 exactly as jnp computes them.
CFD_D float kx_of(const SpecParams& p, int k) { return __ldg(p.kx + k); }
CFD_D float ky_of(const SpecParams& p, int k) { return __ldg(p.ky + k); }

// Brick-wall 2/3 filter (spectral/utils.py:128-134).
CFD_D float filt(const SpecParams& p, int kx, int c) {
  const bool row = kx < p.filt_lo || kx >= p.filt_hi;
  return (row && c < p.filt_cols) ? 1.f : 0.f;
}

// The four column-transformed inputs of the explicit terms for element
// (kx, c) of the state u.
// kxf: the kx wavenumber of row kx (from the table, wherever it is read).
CFD_D float2 prep_factor_k(const SpecParams& p, int f, int kx, float kxf, int c, float2 u) {
  const float kyf = ky_of(p, c);
  if (f == 3) return u;
  const float ax = p.two_pi * kxf;
  if (f == 2) return make_float2(ax * u.x, ax * u.y);
  // vorticity_to_velocity: laplace = (2 pi i)^2 (|kx|^2 + |ky|^2), [0,0] = 1;
  // psi = (-1 / laplace) * w.
  float lap = p.lap_coef * (kxf * kxf + kyf * kyf);
  if (kx == 0 && c == 0) lap = 1.f;
  const float pm = -__frcp_rn(lap);  // -1 / lap, correctly rounded
  const float2 psi = make_float2(pm * u.x, pm * u.y);
  if (f == 0) return psi;
  return make_float2(ax * psi.x, ax * psi.y);
}

CFD_D float2 prep_factor(const SpecParams& p, int f, int kx, int c, float2 u) {
  return prep_factor_k(p, f, kx, kx_of(p, kx), c, u);
}

// Field f's 16 prep values of a column-pipe worker (rows t + NTHR r) from the
// state u[r], with f resolved at compile time: inside the stage kernels'
// field loop a run-time f left every element with the code of all four
// fields (the gy field is the state itself, gx one product, vx/vy a
// reciprocal); 2048^2 fused stage: 1.5 us of each field's 3.6 us per group
// before.  Same expressions, same bits.
template <int NTHR>
CFD_D void prep_fields(const SpecParams& p, int f, const float* kxt, int c, bool live, int t,
                       const float2 (&u)[16], float2 (&v)[16]) {
  auto fill = [&](auto fc) {
    constexpr int F = decltype(fc)::value;
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      const int kx = t + NTHR * r;
      v[r] = live ? prep_factor_k(p, F, kx, kxt[kx], c, u[r]) : make_float2(0.f, 0.f);
    }
  };
  switch (f) {
    case 0: fill(std::integral_constant<int, 0>{}); break;
    case 1: fill(std::integral_constant<int, 1>{}); break;
    case 2: fill(std::integral_constant<int, 2>{}); break;
    default: fill(std::integral_constant<int, 3>{}); break;
  }
}

// ky-side factors: vx = i ay A, vy = -i B, gx = i C, gy = i ay D.
// kyf: the ky wavenumber of column k (from the table, wherever it is read).
CFD_D float2 row_factor_k(const SpecParams& p, int f, float kyf, float2 x) {
  if (f == 1) return make_float2(x.y, -x.x);
  if (f == 2) return make_float2(-x.y, x.x);
  const float ay = p.two_pi * kyf;
  return make_float2(-(ay * x.y), ay * x.x);
}

CFD_D float2 row_factor(const SpecParams& p, int f, int k, float2 x) {
  if (f == 1) return make_float2(x.y, -x.x);
  if (f == 2) return make_float2(-x.y, x.x);
  const float ay = p.two_pi * ky_of(p, k);
  return make_float2(-(ay * x.y), ay * x.x);
}

struct T4 {
  float2* t[4];
};

// Column-transformed inputs of the explicit terms: block (x, f) builds field
// f of columns [x*W, x*W + W) from the state and writes its inverse
// x-transform.  One transform per block keeps register use at that of a single
// FFT.
CFD_D void col_prep_cols(const SpecParams& p, int blk, int f, int W, int log2W, int bstride,
                          const float2* __restrict__ w, float2* __restrict__ dst) {
  extern __shared__ float2 sbuf[];
  const int N = p.nx, ncols = p.L + 1;
  const int c0 = blk * W;
  const int tid = threadIdx.x;
#pragma unroll 4
  for (int e = tid; e < W * N; e += blockDim.x) {
    const int ww = e & (W - 1), kx = e >> log2W, c = c0 + ww;
    sbuf[ww * bstride + pidx(kx)] =
        c < ncols ? prep_factor(p, f, kx, c, w[(size_t)kx * ncols + c])
                  : make_float2(0.f, 0.f);
  }
  __syncthreads();
  fft_inplace<1>(sbuf, p.log2nx, W, bstride, p.twp_x, tid);
#pragma unroll 4
  for (int e = tid; e < W * N; e += blockDim.x) {
    const int ww = e & (W - 1), i = e >> log2W, c = c0 + ww;
    if (c < ncols) dst[(size_t)i * p.pitch + c] = sbuf[ww * bstride + pidx(i)];
  }
}

__global__ void __launch_bounds__(256, 3)
    spec_col_prep_kernel(SpecParams p, int W, int log2W, int bstride,
                         const float2* __restrict__ w, T4 t4) {
  col_prep_cols(p, blockIdx.x, blockIdx.y, W, log2W, bstride, w, t4.t[blockIdx.y]);
}

// x-transform of the advection row spectra, then one low-storage RK/CN stage
// (or, with explicit_only, just F(u)).
// Element (kx, c) of one low-storage RK/CN stage given the x-transformed
// advection spectrum a (spectral/equations.py:160-190,
// spectral/time_stepping.py:163-169), or just F(u) with explicit_only.
// The stage arithmetic of one element from its loaded state u and register h
// (ho, read only when sc.has_h_in): returns the new state, sets *h_new.
CFD_D float2 stage_update_core_k(const SpecParams& p, const StageCoef& sc, int kx, float kxf,
                                 int c, float2 a, float2 u, float2 ho, float2* h_new) {
  const int ncols = p.L + 1;
  const size_t g = (size_t)kx * ncols + c;
  // explicit_terms: rfftn(advection) * filter (+ forcing curl)
  float2 F = a;
  if (p.filt_on) {
    const float fl = filt(p, kx, c);
    F = make_float2(a.x * fl, a.y * fl);
  }
  if (p.fc_full) F = c_add(F, __ldg(p.fc_full + g));
  else if (p.fc_row0 && kx == 0) F = c_add(F, __ldg(p.fc_row0 + c));
  if (sc.explicit_only) {
    *h_new = F;
    return F;
  }
  // h = F(u) + beta_k h
  float2 h = F;
  if (sc.has_h_in) h = c_add(F, make_float2(sc.beta * ho.x, sc.beta * ho.y));
  // linear_term = nu * laplace - drag; laplace = (2 pi i)^2 |k|^2
  const float kyf = ky_of(p, c);
  const float lin = p.nu * (p.lap_coef * (kxf * kxf + kyf * kyf)) - p.drag;
  // u + gamma dt h + mu G(u), G(u) = linear_term * u
  const float2 x = make_float2((u.x + sc.gdt * h.x) + sc.mu * (lin * u.x),
                               (u.y + sc.gdt * h.y) + sc.mu * (lin * u.y));
  // implicit_solve: 1 / (1 - mu * linear_term) * x
  const float inv = __frcp_rn(1.f - sc.mu * lin);
  *h_new = h;
  return make_float2(inv * x.x, inv * x.y);
}

CFD_D float2 stage_update_core(const SpecParams& p, const StageCoef& sc, int kx, int c,
                               float2 a, float2 u, float2 ho, float2* h_new) {
  return stage_update_core_k(p, sc, kx, kx_of(p, kx), c, a, u, ho, h_new);
}

CFD_D void stage_update_at(const SpecParams& p, const StageCoef& sc, int kx, int c, float2 a,
                           float2* __restrict__ wst, float2* __restrict__ hst) {
  const size_t g = (size_t)kx * (p.L + 1) + c;
  float2 h;
  if (sc.explicit_only) {
    wst[g] = stage_update_core(p, sc, kx, c, a, a, a, &h);
    return;
  }
  const float2 ho = sc.has_h_in ? hst[g] : make_float2(0.f, 0.f);
  wst[g] = stage_update_core(p, sc, kx, c, a, wst[g], ho, &h);
  if (sc.write_h) hst[g] = h;
}

CFD_D void col_update_cols(const SpecParams& p, const StageCoef& sc, int blk, int W,
                            int log2W, int bstride, const float2* __restrict__ ahat,
                            float2* __restrict__ wst, float2* __restrict__ hst) {
  extern __shared__ float2 sbuf[];
  const int N = p.nx, ncols = p.L + 1;
  const int c0 = blk * W;
  const int tid = threadIdx.x;
#pragma unroll 4
  for (int e = tid; e < W * N; e += blockDim.x) {
    const int w = e & (W - 1), i = e >> log2W, c = c0 + w;
    sbuf[w * bstride + pidx(i)] =
        c < ncols ? ahat[(size_t)i * p.pitch + c] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  fft_inplace<-1>(sbuf, p.log2nx, W, bstride, p.twp_x, tid);
  for (int e = tid; e < W * N; e += blockDim.x) {
    const int w = e & (W - 1), kx = e >> log2W, c = c0 + w;
    if (c >= ncols) continue;
    stage_update_at(p, sc, kx, c, sbuf[w * bstride + pidx(kx)], wst, hst);
  }
}

__global__ void __launch_bounds__(256, 3)
    spec_col_update_kernel(SpecParams p, StageCoef sc, int W, int log2W,
                           int bstride, const float2* __restrict__ ahat,
                           float2* __restrict__ wst, float2* __restrict__ hst) {
  col_update_cols(p, sc, blockIdx.x, W, log2W, bstride, ahat, wst, hst);
}

CFD_D void row_advect_rows(const SpecParams& p, int blk, int rows,
                            const float2* __restrict__ t0, const float2* __restrict__ t1,
                            const float2* __restrict__ t2, const float2* __restrict__ t3,
                            float2* __restrict__ ahat) {
  extern __shared__ float2 sbuf[];
  const int L = p.L, log2L = p.log2L, ncols = L + 1, PL = padded_len(L);
  const int half = L >> 1, log2h = log2L - 1;
  const int i0 = blk * rows;
  const float2* tf[4] = {t0, t1, t2, t3};
  // Inverse real transforms along y: build the half-length complex inputs.
  // Pairs (k, L-k) for k in [1, L/2); the k = 0 slot also does DC/Nyquist and
  // the middle element.
  for (int idx = threadIdx.x; idx < ((rows * 4) << log2h); idx += blockDim.x) {
    const int rf = idx >> log2h, k = idx & (half - 1);
    const int r = rf >> 2, f = rf & 3;
    const float2* in = tf[f] + (size_t)(i0 + r) * p.pitch;
    float2* z = sbuf + rf * PL;
    if (k == 0) {
      const float2 x0 = row_factor(p, f, 0, in[0]);
      const float2 xl = row_factor(p, f, L, in[L]);
      z[0] = make_float2(x0.x + xl.x, x0.x - xl.x);
      const float2 xh = row_factor(p, f, half, in[half]);
      float2 zk, zm;
      irfft_pre_pair(xh, xh, __ldg(p.tw_y + half), &zk, &zm);
      z[pidx(half)] = zk;
    } else {
      const float2 xk = row_factor(p, f, k, in[k]);
      const float2 xm = row_factor(p, f, L - k, in[L - k]);
      float2 zk, zm;
      irfft_pre_pair(xk, xm, __ldg(p.tw_y + k), &zk, &zm);
      z[pidx(k)] = zk;
      z[pidx(L - k)] = zm;
    }
  }
  __syncthreads();
  fft_inplace<1>(sbuf, log2L, rows * 4, PL, p.twp_y, threadIdx.x);
  // advection = -(gx * vx + gy * vy), each field scaled by 1/(nx*ny).
  const float s2 = p.scale * p.scale;
  for (int idx = threadIdx.x; idx < (rows << log2L); idx += blockDim.x) {
    const int r = idx >> log2L, n = idx & (L - 1);
    float2* z = sbuf + (r * 4) * PL + pidx(n);
    const float2 vx = z[0], vy = z[PL], gx = z[2 * PL], gy = z[3 * PL];
    z[0] = make_float2(-(gx.x * vx.x + gy.x * vy.x) * s2,
                       -(gx.y * vx.y + gy.y * vy.y) * s2);
  }
  __syncthreads();
  fft_inplace<-1>(sbuf, log2L, rows, 4 * PL, p.twp_y, threadIdx.x);
  for (int idx = threadIdx.x; idx < (rows << log2h); idx += blockDim.x) {
    const int r = idx >> log2h, k = idx & (half - 1);
    const float2* z = sbuf + (r * 4) * PL;
    float2* out = ahat + (size_t)(i0 + r) * p.pitch;
    if (k == 0) {
      const float2 z0 = z[0];
      out[0] = make_float2(z0.x + z0.y, 0.f);
      out[L] = make_float2(z0.x - z0.y, 0.f);
      const float2 zh = z[pidx(half)];
      float2 xk, xm;
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

__global__ void __launch_bounds__(256, 3)
    spec_row_kernel(SpecParams p, int rows, const float2* __restrict__ t0,
                    const float2* __restrict__ t1, const float2* __restrict__ t2,
                    const float2* __restrict__ t3, float2* __restrict__ ahat) {
  pdl_wait();
  pdl_trigger();
  row_advect_rows(p, blockIdx.x, rows, t0, t1, t2, t3, ahat);
}

// Isotropic kinetic-energy spectrum, binsum form (data/xarray_utils.py:
// 279-290, 370-401): 0.5 (|u^|^2 + |v^|^2) of the unnormalised 2-D FFTs summed
// over shells bounds[i] < |k| <= bounds[i+1], bounds = ks (i + 0.5), with
// |k| = 2 pi |fftfreq| formed in double.  The rfft half spectrum stands for
// the full one: columns 1 .. L-1 have a mirror image at -ky with the same
// energy and |k| (weight 2); columns 0 and L appear once.  Per-block shared
// histograms in double, added to `out` (nbins doubles, zeroed by the caller).
__global__ void shell_energy_kernel(int nx, int ny, double dnx, double dny, double ks,
                                    int nbins, const float2* __restrict__ uh,
                                    const float2* __restrict__ vh, double* __restrict__ out) {
  extern __shared__ double hist[];
  for (int b = threadIdx.x; b < nbins; b += blockDim.x) hist[b] = 0.0;
  __syncthreads();
  const int L = ny / 2, ncols = L + 1;
  const size_t n = (size_t)nx * ncols;
  const double two_pi = 6.283185307179586476925286766559;
  for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < n;
       g += (size_t)gridDim.x * blockDim.x) {
    const int kx = (int)(g / ncols), c = (int)(g - (size_t)kx * ncols);
    const double fx = (double)(kx < nx / 2 ? kx : kx - nx) / dnx;
    const double fy = (double)(c < ny / 2 ? c : c - ny) / dny;
    const double k = two_pi * sqrt(fx * fx + fy * fy);
    const int bin = (int)ceil(k / ks - 1.5);
    if (bin < 0 || bin >= nbins) continue;
    const float2 a = uh[g], b = vh[g];
    const double e = 0.5 * ((double)a.x * a.x + (double)a.y * a.y + (double)b.x * b.x +
                            (double)b.y * b.y);
    atomicAdd(&hist[bin], (c == 0 || c == L) ? e : 2.0 * e);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < nbins; b += blockDim.x)
    if (hist[b] != 0.0) atomicAdd(&out[b], hist[b]);
}

// Sum over cells of vorticity^2 / 2 (xarray_utils.py:155-167) in double,
// vorticity = (v[i+1] - v) / hx - (u[j+1] - u) / hy at offset (1, 1).
__global__ void enstrophy_sum_kernel(int nx, int ny, float hx, float hy,
                                     const float* __restrict__ u, const float* __restrict__ v,
                                     double* __restrict__ out) {
  const size_t n = (size_t)nx * ny;
  double acc = 0.0;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(idx / ny), j = (int)(idx - (size_t)i * ny);
    const float dv = (__ldg(v + (size_t)((i + 1) % nx) * ny + j) - __ldg(v + idx)) / hx;
    const float du = (__ldg(u + (size_t)i * ny + (j + 1) % ny) - __ldg(u + idx)) / hy;
    const double w = (double)(dv - du);
    acc += 0.5 * w * w;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, acc);
}

// Clustered column passes, the scheme of the FVM column pass: clusters of CL
// one-column blocks; block `rank` moves rows [rank N/CL, (rank+1) N/CL) of the
// cluster's CL columns (CL consecutive complex values per row) between global
// memory and the owning blocks' shared memory, and each block transforms its
// own column.  Columns past the last one (ncols = L + 1 is odd) transform
// zeros and store nothing.  Each block's arithmetic is that of the per-block
// kernels, so both give the same bits.
template <int CL>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(128, 7)
    spec_col_prep_cluster_kernel(SpecParams p, const float2* __restrict__ w, T4 t4) {
  extern __shared__ float2 sbuf[];
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int N = p.nx, ncols = p.L + 1, f = blockIdx.y;
  const int c0 = blockIdx.x - rank;
  const int tid = threadIdx.x;
  const int rows_per = N / CL, r0 = rank * rows_per;
  // Every block of the cluster runs before any block touches a peer.
  cluster.sync();
  for (int row = r0 + tid; row < r0 + rows_per; row += blockDim.x) {
#pragma unroll
    for (int q = 0; q < CL; ++q) {
      const int col = c0 + q;
      cluster.map_shared_rank(sbuf, q)[pidx(row)] =
          col < ncols ? prep_factor(p, f, row, col, w[(size_t)row * ncols + col])
                      : make_float2(0.f, 0.f);
    }
  }
  cluster.sync();
  fft_inplace<1>(sbuf, p.log2nx, 1, padded_len(N), p.twp_x, tid);
  cluster.sync();
  float2* dst = t4.t[f];
  for (int row = r0 + tid; row < r0 + rows_per; row += blockDim.x) {
#pragma unroll
    for (int q = 0; q < CL; ++q) {
      const int col = c0 + q;
      if (col < ncols) dst[(size_t)row * p.pitch + col] = cluster.map_shared_rank(sbuf, q)[pidx(row)];
    }
  }
  // No block may leave while a peer still reads its shared memory.
  cluster.sync();
}

template <int CL>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(128, 7)
    spec_col_update_cluster_kernel(SpecParams p, StageCoef sc, const float2* __restrict__ ahat,
                                   float2* __restrict__ wst, float2* __restrict__ hst) {
  extern __shared__ float2 sbuf[];
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int N = p.nx, ncols = p.L + 1;
  const int c0 = blockIdx.x - rank;
  const int tid = threadIdx.x;
  const int rows_per = N / CL, r0 = rank * rows_per;
  cluster.sync();
  for (int row = r0 + tid; row < r0 + rows_per; row += blockDim.x) {
#pragma unroll
    for (int q = 0; q < CL; ++q) {
      const int col = c0 + q;
      cluster.map_shared_rank(sbuf, q)[pidx(row)] =
          col < ncols ? ahat[(size_t)row * p.pitch + col] : make_float2(0.f, 0.f);
    }
  }
  cluster.sync();
  fft_inplace<-1>(sbuf, p.log2nx, 1, padded_len(N), p.twp_x, tid);
  cluster.sync();
  // The stage update on this block's row range, in row order (coalesced).
  for (int row = r0 + tid; row < r0 + rows_per; row += blockDim.x) {
#pragma unroll
    for (int q = 0; q < CL; ++q) {
      const int col = c0 + q;
      if (col < ncols)
        stage_update_at(p, sc, row, col, cluster.map_shared_rank(sbuf, q)[pidx(row)], wst, hst);
    }
  }
  cluster.sync();
}

// ---- Persistent column passes (engine in colpipe.cuh) ----
// Work items of the update pass are groups of CG of the ncols = L + 1
// half-spectrum columns (the last group padded with zero columns that store
// nothing); items of the prep pass are (group, field) pairs, one inverse
// transform each.  Every item reads its column inputs through the staging
// slots while the previous item is transformed.  Each element is computed by
// the expressions col_update_cols / col_prep_cols evaluate, after the same
// butterflies, so all column schemes give the same bits.  One transform makes
// two exchanges at 512 to 4096 rows, so every item starts on buffer 0.
// src: rows of `pitch` values, of which the first ncols are columns.
template <int LOG2N, int CG>
CFD_D void spec_pipe_prefetch(const float2* __restrict__ src, int pitch, int ncols, int c, int t,
                              float2* __restrict__ stage) {
  constexpr int NTHR = ColPipe<LOG2N>::NTHR, T = CG * NTHR;
  if (c >= ncols) return;
  const int tid = t * CG + (c % CG);
#pragma unroll
  for (int r = 0; r < 16; ++r)
    cp_async8(stage + r * T + tid, src + (size_t)(t + NTHR * r) * pitch + c);
}

// Element (kx, c) of the state or h: row-major [nx, L + 1], or tiled by
// column groups of CG ([group][kx][c % CG], each group's values contiguous) so
// that a warp of the persistent column passes (8 workers x CG columns) reads
// and writes 256 contiguous bytes instead of 8 separate 32-byte row segments.
template <int CG, bool TILED>
CFD_D size_t state_at(int nx, int ncols, int kx, int c) {
  return TILED ? ((size_t)(c / CG) * nx + kx) * CG + (c % CG) : (size_t)kx * ncols + c;
}

template <int LOG2N, int CG, bool TILED = false>
__global__ void __launch_bounds__(CG * (1 << LOG2N) / 16,
                                  col_pipe_min_blocks(CG * (1 << LOG2N) / 16))
    spec_col_update_pipe_kernel(SpecParams p, StageCoef sc, const float2* __restrict__ ahat,
                                float2* __restrict__ wst, float2* __restrict__ hst) {
  using P = ColPipe<LOG2N>;
  constexpr int T = CG * P::NTHR;
  extern __shared__ float2 sbuf[];
  const int ncols = p.L + 1, groups = (ncols + CG - 1) / CG;
  const int w = threadIdx.x % CG, t = threadIdx.x / CG, tid = threadIdx.x;
  const int bstride = col_pipe_bstride<LOG2N, CG>();
  float2* const buf[2] = {sbuf + w * bstride, sbuf + (CG + w) * bstride};
  float2* const stage = sbuf + 2 * CG * bstride;
  int g = blockIdx.x;
  if (g >= groups) return;  // uniform per block
  // The constant tables first: under a programmatic launch this overlaps the
  // previous kernel's tail.
  const float2* tw;
  const float* kxt;
  col_pipe_tables<LOG2N, CG>(sbuf, p.twp_x, p.kx, &tw, &kxt);
  pdl_wait();
  pdl_trigger();
  spec_pipe_prefetch<LOG2N, CG>(ahat, p.pitch, ncols, g * CG + w, t, stage);
  cp_async_commit();
  float2 v[16], us[16], hs[16];
#pragma unroll 1
  for (; g < groups; g += gridDim.x) {
    const int c = g * CG + w;
    cp_async_wait_all();
#pragma unroll
    for (int r = 0; r < 16; ++r) v[r] = c < ncols ? stage[r * T + tid] : make_float2(0.f, 0.f);
    const int gn = g + gridDim.x;
    if (gn < groups) spec_pipe_prefetch<LOG2N, CG>(ahat, p.pitch, ncols, gn * CG + w, t, stage);
    cp_async_commit();
    if (c < ncols && !sc.explicit_only) {
      // All of this column's state and h values are requested before any is
      // used (each element is read and written by this thread only).
#pragma unroll
      for (int m = 0; m < 16; ++m) {
        const size_t gi = state_at<CG, TILED>(p.nx, ncols, t + P::NTHR * m, c);
        us[m] = wst[gi];
        hs[m] = sc.has_h_in ? hst[gi] : make_float2(0.f, 0.f);
      }
    }
    col_pipe_fft<LOG2N, -1, 0>(v, buf, t, tw);
    if (c < ncols) {
#pragma unroll
      for (int m = 0; m < 16; ++m) {
        const int kx = t + P::NTHR * m;
        const size_t gi = state_at<CG, TILED>(p.nx, ncols, kx, c);
        if (sc.explicit_only) {
          stage_update_at(p, sc, kx, c, v[m], wst, hst);
        } else {
          float2 h;
          wst[gi] = stage_update_core_k(p, sc, kx, kxt[kx], c, v[m], us[m], hs[m], &h);
          if (sc.write_h) hst[gi] = h;
        }
      }
    }
  }
  cp_async_wait_all();
}

// Column update fused with the next stage's column prep: after the forward
// transform and the stage update, the thread holds the new state of its
// column at kx = t + (N/16) m, which are exactly the first inverse pass's
// input positions, so the four prep fields are formed in registers and
// transformed without re-reading the state.  Every value is the one the
// separate update and prep passes compute, so the bits are the same.  One
// item makes ten exchanges (five transforms), so items start on buffer 0.
template <int LOG2N, int CG, bool TILED = false>
__global__ void __launch_bounds__(CG * (1 << LOG2N) / 16,
                                  col_pipe_min_blocks(CG * (1 << LOG2N) / 16))
    spec_col_stage_pipe_kernel(SpecParams p, StageCoef sc, const float2* __restrict__ ahat,
                               float2* __restrict__ wst, float2* __restrict__ hst, T4 t4) {
  using P = ColPipe<LOG2N>;
  constexpr int T = CG * P::NTHR;
  extern __shared__ float2 sbuf[];
  const int ncols = p.L + 1, groups = (ncols + CG - 1) / CG;
  const int w = threadIdx.x % CG, t = threadIdx.x / CG, tid = threadIdx.x;
  const int bstride = col_pipe_bstride<LOG2N, CG>();
  float2* const buf[2] = {sbuf + w * bstride, sbuf + (CG + w) * bstride};
  float2* const stage = sbuf + 2 * CG * bstride;
  int g = blockIdx.x;
  if (g >= groups) return;  // uniform per block
  // The constant tables first: under a programmatic launch this overlaps the
  // previous kernel's tail.
  const float2* tw;
  const float* kxt;
  col_pipe_tables<LOG2N, CG>(sbuf, p.twp_x, p.kx, &tw, &kxt);
  pdl_wait();
  pdl_trigger();
  spec_pipe_prefetch<LOG2N, CG>(ahat, p.pitch, ncols, g * CG + w, t, stage);
  cp_async_commit();
  float2 v[16], u[16], hs[16];
#pragma unroll 1
  for (; g < groups; g += gridDim.x) {
    const int c = g * CG + w;
    const bool live = c < ncols;
    cp_async_wait_all();
#pragma unroll
    for (int r = 0; r < 16; ++r) v[r] = live ? stage[r * T + tid] : make_float2(0.f, 0.f);
    const int gn = g + gridDim.x;
    if (gn < groups) spec_pipe_prefetch<LOG2N, CG>(ahat, p.pitch, ncols, gn * CG + w, t, stage);
    cp_async_commit();
    // The column's state and h values are requested before the transform
    // (each element is read and written by this thread only).
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      const size_t gi = state_at<CG, TILED>(p.nx, ncols, t + P::NTHR * m, c);
      u[m] = live ? wst[gi] : make_float2(0.f, 0.f);
      hs[m] = (live && sc.has_h_in) ? hst[gi] : make_float2(0.f, 0.f);
    }
    col_pipe_fft<LOG2N, -1, 0>(v, buf, t, tw);
    if (live) {
#pragma unroll
      for (int m = 0; m < 16; ++m) {
        const int kx = t + P::NTHR * m;
        const size_t gi = state_at<CG, TILED>(p.nx, ncols, kx, c);
        float2 h;
        u[m] = stage_update_core_k(p, sc, kx, kxt[kx], c, v[m], u[m], hs[m], &h);
        wst[gi] = u[m];
        if (sc.write_h) hst[gi] = h;
      }
    }
#pragma unroll 1
    for (int f = 0; f < 4; ++f) {
      prep_fields<P::NTHR>(p, f, kxt, c, live, t, u, v);
      col_pipe_fft<LOG2N, 1, 0>(v, buf, t, tw);
      if (live) {
        float2* dst = f == 0 ? t4.t[0] : f == 1 ? t4.t[1] : f == 2 ? t4.t[2] : t4.t[3];
#pragma unroll
        for (int m = 0; m < 16; ++m) dst[(size_t)(t + P::NTHR * m) * p.pitch + c] = v[m];
      }
    }
  }
  cp_async_wait_all();
}

// The fused stage with TMA: each group's advection-spectrum columns arrive
// by TMA tensor loads (boxes of 4 columns x BOX rows, one thread issuing onto
// an mbarrier, the next group's while this one is transformed), and each of
// the four fields leaves by TMA tensor stores from the transform's second
// exchange buffers, which the field's values are copied into in the boxes'
// row-major layout once the inverse transform has read them; the thread that
// issued the stores waits for them to have read shared memory before its
// next transform's first barrier, so no thread rewrites those buffers
// earlier.  Same values as spec_col_stage_pipe_kernel; groups of 4 columns.
struct SpecT4Maps {
  CUtensorMap t[4];
};

template <int LOG2N, bool TILED>
__global__ void __launch_bounds__(4 * (1 << LOG2N) / 16,
                                  col_pipe_min_blocks(4 * (1 << LOG2N) / 16))
    spec_col_stage_tma_kernel(SpecParams p, StageCoef sc, const __grid_constant__ CUtensorMap amap,
                              const __grid_constant__ SpecT4Maps tmaps, float2* __restrict__ wst,
                              float2* __restrict__ hst) {
  constexpr int CG = 4;
  using P = ColPipe<LOG2N>;
  constexpr int N = P::N, BOX = N < 256 ? N : 256, NBOX = N / BOX;
  constexpr uint32_t kGroupBytes = (uint32_t)N * CG * sizeof(float2);
  extern __shared__ float2 sbuf[];  // no static shared memory: 128-byte aligned
  const int ncols = p.L + 1, groups = (ncols + CG - 1) / CG;
  const int w = threadIdx.x % CG, t = threadIdx.x / CG, tid = threadIdx.x;
  const int bstride = col_pipe_bstride<LOG2N, CG>();
  float2* const buf[2] = {sbuf + w * bstride, sbuf + (CG + w) * bstride};
  float2* const stage = sbuf + 2 * CG * bstride;
  // The four columns' second exchange buffers, contiguous: the store boxes.
  float2* const out = sbuf + CG * bstride;
  uint64_t* const bar =
      reinterpret_cast<uint64_t*>(reinterpret_cast<char*>(sbuf) + col_pipe_smem<LOG2N, CG>());
  int g = blockIdx.x;
  if (g >= groups) return;  // uniform per block
  const float2* tw;
  const float* kxt;
  col_pipe_tables<LOG2N, CG>(sbuf, p.twp_x, p.kx, &tw, &kxt);
  if (tid == 0) {
    mbar_init(bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  pdl_wait();
  pdl_trigger();
  auto issue = [&](int gg) {
    mbar_arrive_expect_tx(bar, kGroupBytes);
#pragma unroll
    for (int b = 0; b < NBOX; ++b) tma_load_2d(stage + b * BOX * CG, &amap, 8 * gg, b * BOX, bar);
  };
  if (tid == 0) issue(g);
  uint32_t phase = 0;
  float2 v[16], u[16], hs[16];
  // The state of a group is loaded while the previous group's last field is
  // transformed (u is free once that field's prep has read it), so the loads
  // are in flight during that transform; the first group's here.
  auto load_state = [&](int gg) {
    const int cc = gg * CG + w;
    const bool ll = gg < groups && cc < ncols;
#pragma unroll
    for (int m = 0; m < 16; ++m)
      u[m] = ll ? wst[state_at<CG, TILED>(p.nx, ncols, t + P::NTHR * m, cc)] : make_float2(0.f, 0.f);
  };
  load_state(g);
#pragma unroll 1
  for (; g < groups; g += gridDim.x) {
    const int c = g * CG + w;
    const bool live = c < ncols;
    const bool landed = mbar_wait(bar, phase);
    phase ^= 1u;
#pragma unroll
    for (int r = 0; r < 16; ++r) v[r] = live ? stage[(t + P::NTHR * r) * CG + w] : make_float2(0.f, 0.f);
    // The staged group is read; a wait that gave up on any thread ends the
    // block (after its own stores have left shared memory).
    if (__syncthreads_or(!landed)) {
      if (tid == 0) bulk_wait_all();
      return;
    }
    if (tid == 0 && g + gridDim.x < groups) {
      fence_proxy_async_smem();
      issue(g + gridDim.x);
    }
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      const size_t gi = state_at<CG, TILED>(p.nx, ncols, t + P::NTHR * m, c);
      hs[m] = (live && sc.has_h_in) ? hst[gi] : make_float2(0.f, 0.f);
    }
    if (tid == 0) bulk_wait_read_all();
    col_pipe_fft<LOG2N, -1, 0>(v, buf, t, tw);
    if (live) {
#pragma unroll
      for (int m = 0; m < 16; ++m) {
        const int kx = t + P::NTHR * m;
        const size_t gi = state_at<CG, TILED>(p.nx, ncols, kx, c);
        float2 h;
        u[m] = stage_update_core_k(p, sc, kx, kxt[kx], c, v[m], u[m], hs[m], &h);
        wst[gi] = u[m];
        if (sc.write_h) hst[gi] = h;
      }
    }
#pragma unroll 1
    for (int f = 0; f < 4; ++f) {
      prep_fields<P::NTHR>(p, f, kxt, c, live, t, u, v);
      if (f == 3) load_state(g + gridDim.x);
      if (tid == 0) bulk_wait_read_all();
      col_pipe_fft<LOG2N, 1, 0>(v, buf, t, tw);
      // Every thread is past the transform's reads of the second buffers.
      __syncthreads();
#pragma unroll
      for (int m = 0; m < 16; ++m) out[(t + P::NTHR * m) * CG + w] = v[m];
      fence_proxy_async_smem();
      __syncthreads();
      if (tid == 0) {
#pragma unroll
        for (int b = 0; b < NBOX; ++b)
          tma_store_2d(&tmaps.t[f], 8 * g, b * BOX, out + b * BOX * CG);
        bulk_commit_group();
      }
    }
  }
  if (tid == 0) bulk_wait_all();
}

template <int LOG2N, int CG>
__global__ void __launch_bounds__(CG * (1 << LOG2N) / 16,
                                  col_pipe_min_blocks(CG * (1 << LOG2N) / 16))
    spec_col_prep_pipe_kernel(SpecParams p, const float2* __restrict__ wst, T4 t4) {
  using P = ColPipe<LOG2N>;
  constexpr int T = CG * P::NTHR;
  extern __shared__ float2 sbuf[];
  const int ncols = p.L + 1, items = 4 * ((ncols + CG - 1) / CG);
  const int w = threadIdx.x % CG, t = threadIdx.x / CG, tid = threadIdx.x;
  const int bstride = col_pipe_bstride<LOG2N, CG>();
  float2* const buf[2] = {sbuf + w * bstride, sbuf + (CG + w) * bstride};
  float2* const stage = sbuf + 2 * CG * bstride;
  int it = blockIdx.x;
  if (it >= items) return;  // uniform per block
  const float2* tw;
  const float* kxt;
  col_pipe_tables<LOG2N, CG>(sbuf, p.twp_x, p.kx, &tw, &kxt);
  pdl_wait();
  pdl_trigger();
  spec_pipe_prefetch<LOG2N, CG>(wst, ncols, ncols, (it >> 2) * CG + w, t, stage);
  cp_async_commit();
  float2 v[16];
#pragma unroll 1
  for (; it < items; it += gridDim.x) {
    const int f = it & 3, c = (it >> 2) * CG + w;
    cp_async_wait_all();
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      const int kx = t + P::NTHR * r;
      v[r] = c < ncols ? prep_factor_k(p, f, kx, kxt[kx], c, stage[r * T + tid])
                       : make_float2(0.f, 0.f);
    }
    const int in = it + gridDim.x;
    if (in < items) spec_pipe_prefetch<LOG2N, CG>(wst, ncols, ncols, (in >> 2) * CG + w, t, stage);
    cp_async_commit();
    col_pipe_fft<LOG2N, 1, 0>(v, buf, t, tw);
    if (c < ncols) {
      float2* dst = f == 0 ? t4.t[0] : f == 1 ? t4.t[1] : f == 2 ? t4.t[2] : t4.t[3];
#pragma unroll
      for (int m = 0; m < 16; ++m) dst[(size_t)(t + P::NTHR * m) * p.pitch + c] = v[m];
    }
  }
  cp_async_wait_all();
}

// ---- Row pass with register-resident Stockham passes ----
// One row per block.  Thread (f, t) -- field f = threadIdx.x / (L/16), worker
// t -- builds the 16 inputs of field f's inverse real transform that the first
// Stockham pass gives worker t straight from global memory, with the
// pre-untangling of row_advect_rows (for k > L/2 as the second output of the
// pair (L - k, k), so each element rounds as there), and runs the passes of
// colpipe.cuh.  The four fields' samples meet in shared memory for the
// advection product, which the field-0 threads form at exactly the forward
// transform's first-pass positions; the post-untangling partners again come
// from shared memory.  Same butterflies, twiddles and element formulas as
// row_advect_rows, so the same bits, with no shared-memory round trip around
// the transforms' global loads and stores.
//
// Shared memory: one exchange buffer per field (each exchange waits for the
// previous one's reads before it writes) and a table region that nothing
// overwrites, holding the ky table and the untangling twiddles for the pre-
// and post-untangling.  At ny = 2048 that is 47 KB per block, so that four
// blocks (64 registers) fit on a multiprocessor; with two buffers per field
// and the tables in them it was 68 KB and three blocks.
template <int LOG2L>
CFD_HD size_t spec_row_pipe_smem() {
  constexpr int L = 1 << LOG2L;
  return ((size_t)4 * padded_len(L) + (L + 2) / 2 + L) * sizeof(float2);
}

template <int LOG2L>
CFD_D void spec_row_pipe_body(const SpecParams& p, int row, const float2* __restrict__ t0,
                              const float2* __restrict__ t1, const float2* __restrict__ t2,
                              const float2* __restrict__ t3, float2* __restrict__ ahat) {
  using P = ColPipe<LOG2L>;
  constexpr int NTHR = P::NTHR, L = P::N, half = L / 2;
  // From 32 workers per field on, a field's transforms synchronise only its
  // own warps (named barrier 1 + f): its buffer is its own until the samples
  // meet for the product.
  constexpr int BARN = NTHR >= 32 ? NTHR : 0;
  extern __shared__ float2 sbuf[];
  const int f = threadIdx.x / NTHR, t = threadIdx.x % NTHR;
  const int bstride = padded_len(L);
  float2* const fb = sbuf + f * bstride;
  float2* const buf[2] = {fb, fb};
  float* const kys = reinterpret_cast<float*>(sbuf + 4 * bstride);  // L + 1 values
  float2* const tws = sbuf + 4 * bstride + (L + 2) / 2;             // L values
  const float2* gin = (f == 0 ? t0 : f == 1 ? t1 : f == 2 ? t2 : t3) + (size_t)row * p.pitch;
  // The field's row (L + 1 values), the ky table and the twiddles are first
  // copied into shared memory, all of a thread's loads issued before any
  // store, and the pre-untangling reads them there: read from global memory
  // inside the branchy loop below, the loads of each element, its mirror, ky
  // and the twiddle were taken one round trip at a time.  2048^2 row pass:
  // 61.9 us reading global memory in the loop, 57.1 with the rows staged,
  // 48.2 with the tables staged as well.
  float2* const in = fb;
  {
    float2 x[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) x[r] = gin[t + NTHR * r];
    const float2 xl = t == 0 ? gin[L] : make_float2(0.f, 0.f);
    constexpr int T = 4 * NTHR;
    float kv[(L + T) / T];
    float2 tv[(L + T - 1) / T];
#pragma unroll
    for (int r = 0; r < (L + T) / T; ++r) {
      const int e = (int)threadIdx.x + T * r;
      kv[r] = e <= L ? __ldg(p.ky + e) : 0.f;
    }
#pragma unroll
    for (int r = 0; r < (L + T - 1) / T; ++r) {
      const int e = (int)threadIdx.x + T * r;
      tv[r] = e < L ? __ldg(p.tw_y + e) : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int r = 0; r < 16; ++r) in[t + NTHR * r] = x[r];
    if (t == 0) in[L] = xl;
#pragma unroll
    for (int r = 0; r < (L + T) / T; ++r) {
      const int e = (int)threadIdx.x + T * r;
      if (e <= L) kys[e] = kv[r];
    }
#pragma unroll
    for (int r = 0; r < (L + T - 1) / T; ++r) {
      const int e = (int)threadIdx.x + T * r;
      if (e < L) tws[e] = tv[r];
    }
  }
  __syncthreads();
  float2 v[16];
#pragma unroll
  for (int r = 0; r < 16; ++r) {
    const int k = t + NTHR * r;
    float2 zk, zm;
    if (k == 0) {
      const float2 x0 = row_factor_k(p, f, kys[0], in[0]);
      const float2 xl = row_factor_k(p, f, kys[L], in[L]);
      v[r] = make_float2(x0.x + xl.x, x0.x - xl.x);
    } else if (k == half) {
      const float2 xh = row_factor_k(p, f, kys[half], in[half]);
      irfft_pre_pair(xh, xh, tws[half], &zk, &zm);
      v[r] = zk;
    } else if (k < half) {
      const float2 xk = row_factor_k(p, f, kys[k], in[k]);
      const float2 xm = row_factor_k(p, f, kys[L - k], in[L - k]);
      irfft_pre_pair(xk, xm, tws[k], &zk, &zm);
      v[r] = zk;
    } else {
      const int kp = L - k;
      const float2 xk = row_factor_k(p, f, kys[kp], in[kp]);
      const float2 xm = row_factor_k(p, f, kys[k], in[k]);
      irfft_pre_pair(xk, xm, tws[kp], &zk, &zm);
      v[r] = zm;
    }
  }
  // The transform's first exchange rewrites the copy of the row.
  col_pipe_sync<BARN>(1 + f);
  col_pipe_fft<LOG2L, 1, 0, true, BARN, true>(v, buf, t, p.twp_y, true, 1 + f);
  // Samples n = t + NTHR m of every field into its buffer, once the
  // transform's last reads of it are done.
  col_pipe_sync<BARN>(1 + f);
#pragma unroll
  for (int m = 0; m < 16; ++m) fb[pidx(t + NTHR * m)] = v[m];
  __syncthreads();
  const bool lead = f == 0;
  if constexpr (BARN != 0) {
    if (!lead) return;  // fields 1-3 are done; the field-0 warps go on alone
  }
  if (lead) {
    // advection = -(gx * vx + gy * vy), each field scaled by 1/(nx*ny).
    const float s2 = p.scale * p.scale;
    const float2* vyb = sbuf + 1 * bstride;
    const float2* gxb = sbuf + 2 * bstride;
    const float2* gyb = sbuf + 3 * bstride;
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      const int n = pidx(t + NTHR * m);
      const float2 vx = v[m], vy = vyb[n], gx = gxb[n], gy = gyb[n];
      v[m] = make_float2(-(gx.x * vx.x + gy.x * vy.x) * s2, -(gx.y * vx.y + gy.y * vy.y) * s2);
    }
  }
  // Forward transform of the advection (field-0 threads) in field 0's buffer,
  // whose samples nobody reads.
  col_pipe_fft<LOG2L, -1, 1, true, BARN, true>(v, buf, t, p.twp_y, lead, 1);
  // Z[k] into field 0's buffer once the transform's last reads of it are
  // done, then each output from the pair (k, L - k).
  col_pipe_sync<BARN>(1);
  if (lead) {
#pragma unroll
    for (int m = 0; m < 16; ++m) fb[pidx(t + NTHR * m)] = v[m];
  }
  col_pipe_sync<BARN>(1);
  if (!lead) return;
  float2* out = ahat + (size_t)row * p.pitch;
#pragma unroll
  for (int m = 0; m < 16; ++m) {
    const int k = t + NTHR * m;
    const float2 z = v[m];
    float2 xk, xm;
    if (k == 0) {
      out[0] = make_float2(z.x + z.y, 0.f);
      out[L] = make_float2(z.x - z.y, 0.f);
    } else if (k == half) {
      rfft_post_pair(z, z, tws[half], &xk, &xm);
      out[half] = xk;
    } else if (k < half) {
      rfft_post_pair(z, fb[pidx(L - k)], tws[k], &xk, &xm);
      out[k] = xk;
    } else {
      rfft_post_pair(fb[pidx(L - k)], z, tws[L - k], &xk, &xm);
      out[k] = xm;
    }
  }
}

// OCC: resident threads per multiprocessor the register budget is sized for
// (512: 128 registers; 768: 80, three blocks; 1024: 64, four 256-thread blocks
// at ny = 2048, which the row pass's 47 KB of shared memory also allows).
template <int LOG2L, int OCC>
__global__ void __launch_bounds__(4 * (1 << LOG2L) / 16, OCC / (4 * (1 << LOG2L) / 16))
    spec_row_pipe_kernel(SpecParams p, const float2* __restrict__ t0,
                         const float2* __restrict__ t1, const float2* __restrict__ t2,
                         const float2* __restrict__ t3, float2* __restrict__ ahat) {
  pdl_wait();
  pdl_trigger();
  spec_row_pipe_body<LOG2L>(p, blockIdx.x, t0, t1, t2, t3, ahat);
}

// The register-pass row pass over a batch (slot on grid axis y).
template <int LOG2L>
__global__ void __launch_bounds__(4 * (1 << LOG2L) / 16, 512 / (4 * (1 << LOG2L) / 16))
    spec_batch_row_pipe_kernel(const SpecMember* __restrict__ mem, int k) {
  const SpecMember& m = mem[blockIdx.y];
  if (k >= m.steps) return;
  const SpecParams p = m.p;
  spec_row_pipe_body<LOG2L>(p, blockIdx.x, m.t[0], m.t[1], m.t[2], m.t[3], m.ahat);
}

// Batched persistent column passes: the work items are (slot, group) pairs
// -- (slot, group, field) for the prep before a chunk's first step -- of the
// slots that take step k, walked with the grid as stride.  The grid tables
// are the batch's (slot 0's pointers); coefficients and pointers are each
// slot's.  The update item also builds the slot's next-stage fields unless
// this is the slot's last stage of its last step, as the per-block update
// and prep passes do, so the bits are theirs.
template <int LOG2N, int CG>
__global__ void __launch_bounds__(CG * (1 << LOG2N) / 16,
                                  col_pipe_min_blocks(CG * (1 << LOG2N) / 16))
    spec_batch_col_stage_pipe_kernel(const SpecMember* __restrict__ mem, int count, int k,
                                     int stage) {
  using P = ColPipe<LOG2N>;
  constexpr int T = CG * P::NTHR;
  extern __shared__ float2 sbuf[];
  const int ncols = mem[0].p.L + 1, groups = (ncols + CG - 1) / CG, items = count * groups;
  const int w = threadIdx.x % CG, t = threadIdx.x / CG, tid = threadIdx.x;
  const int bstride = col_pipe_bstride<LOG2N, CG>();
  float2* const buf[2] = {sbuf + w * bstride, sbuf + (CG + w) * bstride};
  float2* const stg = sbuf + 2 * CG * bstride;
  const float2* tw;
  const float* kxt;
  col_pipe_tables<LOG2N, CG>(sbuf, mem[0].p.twp_x, mem[0].p.kx, &tw, &kxt);
  auto next_active = [&](int it) {
    while (it < items && k >= mem[it / groups].steps) it += gridDim.x;
    return it;
  };
  int it = next_active(blockIdx.x);
  if (it >= items) return;  // uniform per block
  spec_pipe_prefetch<LOG2N, CG>(mem[it / groups].ahat, mem[0].p.pitch, ncols, (it % groups) * CG + w, t, stg);
  cp_async_commit();
  float2 v[16], u[16], hs[16];
#pragma unroll 1
  while (it < items) {
    const SpecMember& m = mem[it / groups];
    const SpecParams& p = m.p;
    const StageCoef sc = m.coef[stage];
    const int c = (it % groups) * CG + w;
    const bool live = c < ncols;
    const bool prep = !(k == m.steps - 1 && stage == m.stages - 1);
    cp_async_wait_all();
#pragma unroll
    for (int r = 0; r < 16; ++r) v[r] = live ? stg[r * T + tid] : make_float2(0.f, 0.f);
    const int nit = next_active(it + gridDim.x);
    if (nit < items)
      spec_pipe_prefetch<LOG2N, CG>(mem[nit / groups].ahat, mem[0].p.pitch, ncols, (nit % groups) * CG + w, t, stg);
    cp_async_commit();
#pragma unroll
    for (int mm = 0; mm < 16; ++mm) {
      const size_t gi = (size_t)(t + P::NTHR * mm) * ncols + c;
      u[mm] = live ? m.w[gi] : make_float2(0.f, 0.f);
      hs[mm] = (live && sc.has_h_in) ? m.h[gi] : make_float2(0.f, 0.f);
    }
    col_pipe_fft<LOG2N, -1, 0>(v, buf, t, tw);
    if (live) {
#pragma unroll
      for (int mm = 0; mm < 16; ++mm) {
        const int kx = t + P::NTHR * mm;
        const size_t gi = (size_t)kx * ncols + c;
        float2 h;
        u[mm] = stage_update_core_k(p, sc, kx, kxt[kx], c, v[mm], u[mm], hs[mm], &h);
        m.w[gi] = u[mm];
        if (sc.write_h) m.h[gi] = h;
      }
    }
    if (prep) {
#pragma unroll 1
      for (int f = 0; f < 4; ++f) {
        prep_fields<P::NTHR>(p, f, kxt, c, live, t, u, v);
        col_pipe_fft<LOG2N, 1, 0>(v, buf, t, tw);
        if (live) {
          float2* dst = m.t[f];
#pragma unroll
          for (int mm = 0; mm < 16; ++mm) dst[(size_t)(t + P::NTHR * mm) * mem[0].p.pitch + c] = v[mm];
        }
      }
    }
    it = nit;
  }
  cp_async_wait_all();
}

template <int LOG2N, int CG>
__global__ void __launch_bounds__(CG * (1 << LOG2N) / 16,
                                  col_pipe_min_blocks(CG * (1 << LOG2N) / 16))
    spec_batch_col_prep_pipe_kernel(const SpecMember* __restrict__ mem, int count) {
  using P = ColPipe<LOG2N>;
  constexpr int T = CG * P::NTHR;
  extern __shared__ float2 sbuf[];
  const int ncols = mem[0].p.L + 1, per = 4 * ((ncols + CG - 1) / CG), items = count * per;
  const int w = threadIdx.x % CG, t = threadIdx.x / CG, tid = threadIdx.x;
  const int bstride = col_pipe_bstride<LOG2N, CG>();
  float2* const buf[2] = {sbuf + w * bstride, sbuf + (CG + w) * bstride};
  float2* const stg = sbuf + 2 * CG * bstride;
  const float2* tw;
  const float* kxt;
  col_pipe_tables<LOG2N, CG>(sbuf, mem[0].p.twp_x, mem[0].p.kx, &tw, &kxt);
  auto next_active = [&](int it) {
    while (it < items && mem[it / per].steps <= 0) it += gridDim.x;
    return it;
  };
  int it = next_active(blockIdx.x);
  if (it >= items) return;  // uniform per block
  spec_pipe_prefetch<LOG2N, CG>(mem[it / per].w, ncols, ncols, ((it % per) >> 2) * CG + w, t, stg);
  cp_async_commit();
  float2 v[16];
#pragma unroll 1
  while (it < items) {
    const SpecMember& m = mem[it / per];
    const int f = (it % per) & 3, c = ((it % per) >> 2) * CG + w;
    cp_async_wait_all();
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      const int kx = t + P::NTHR * r;
      v[r] = c < ncols ? prep_factor_k(m.p, f, kx, kxt[kx], c, stg[r * T + tid])
                       : make_float2(0.f, 0.f);
    }
    const int nit = next_active(it + gridDim.x);
    if (nit < items)
      spec_pipe_prefetch<LOG2N, CG>(mem[nit / per].w, ncols, ncols, ((nit % per) >> 2) * CG + w, t, stg);
    cp_async_commit();
    col_pipe_fft<LOG2N, 1, 0>(v, buf, t, tw);
    if (c < ncols) {
      float2* dst = m.t[f];
#pragma unroll
      for (int mm = 0; mm < 16; ++mm) dst[(size_t)(t + P::NTHR * mm) * mem[0].p.pitch + c] = v[mm];
    }
    it = nit;
  }
  cp_async_wait_all();
}

// ---- Batched variants: the slot index is the last grid axis ----
// Column prep after stage `stage` of step k builds the inputs of the next
// stage (k = -1: before the first step of the chunk).
__global__ void __launch_bounds__(256, 3)
    spec_batch_col_prep_kernel(const SpecMember* __restrict__ mem, int k, int stage, int W,
                               int log2W, int bstride) {
  const SpecMember& m = mem[blockIdx.z];
  if (m.steps <= 0 || k >= m.steps) return;
  if (k == m.steps - 1 && stage == m.stages - 1) return;
  const SpecParams p = m.p;
  col_prep_cols(p, blockIdx.x, blockIdx.y, W, log2W, bstride, m.w, m.t[blockIdx.y]);
}

__global__ void __launch_bounds__(256, 3)
    spec_batch_row_kernel(const SpecMember* __restrict__ mem, int k, int rows) {
  const SpecMember& m = mem[blockIdx.y];
  if (k >= m.steps) return;
  const SpecParams p = m.p;
  row_advect_rows(p, blockIdx.x, rows, m.t[0], m.t[1], m.t[2], m.t[3], m.ahat);
}

__global__ void __launch_bounds__(256, 3)
    spec_batch_col_update_kernel(const SpecMember* __restrict__ mem, int k, int stage, int W,
                                 int log2W, int bstride) {
  const SpecMember& m = mem[blockIdx.y];
  if (k >= m.steps) return;
  const SpecParams p = m.p;
  const StageCoef sc = m.coef[stage];
  col_update_cols(p, sc, blockIdx.x, W, log2W, bstride, m.ahat, m.w, m.h);
}

// Real rows -> unpacked half spectra (rfft along y).
__global__ void __launch_bounds__(256, 3)
    row_rfft_kernel(SpecParams p, int rows, const float* __restrict__ x,
                    float2* __restrict__ X) {
  extern __shared__ float2 sbuf[];
  const int L = p.L, log2L = p.log2L, ncols = L + 1, PL = padded_len(L);
  const int half = L >> 1, log2h = log2L - 1;
  const int i0 = blockIdx.x * rows;
  for (int idx = threadIdx.x; idx < (rows << log2L); idx += blockDim.x) {
    const int r = idx >> log2L, n = idx & (L - 1);
    sbuf[r * PL + pidx(n)] =
        __ldg(reinterpret_cast<const float2*>(x + (size_t)(i0 + r) * p.ny) + n);
  }
  __syncthreads();
  fft_inplace<-1>(sbuf, log2L, rows, PL, p.twp_y, threadIdx.x);
  for (int idx = threadIdx.x; idx < (rows << log2h); idx += blockDim.x) {
    const int r = idx >> log2h, k = idx & (half - 1);
    const float2* z = sbuf + r * PL;
    float2* out = X + (size_t)(i0 + r) * ncols;
    if (k == 0) {
      const float2 z0 = z[0];
      out[0] = make_float2(z0.x + z0.y, 0.f);
      out[L] = make_float2(z0.x - z0.y, 0.f);
      const float2 zh = z[pidx(half)];
      float2 xk, xm;
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

// Unpacked half spectra -> real rows (irfft along y), times `scale`.
__global__ void __launch_bounds__(256, 3)
    row_irfft_kernel(SpecParams p, int rows, const float2* __restrict__ X,
                     float* __restrict__ x, float scale) {
  extern __shared__ float2 sbuf[];
  const int L = p.L, log2L = p.log2L, ncols = L + 1, PL = padded_len(L);
  const int half = L >> 1, log2h = log2L - 1;
  const int i0 = blockIdx.x * rows;
  for (int idx = threadIdx.x; idx < (rows << log2h); idx += blockDim.x) {
    const int r = idx >> log2h, k = idx & (half - 1);
    const float2* in = X + (size_t)(i0 + r) * ncols;
    float2* z = sbuf + r * PL;
    if (k == 0) {
      const float2 x0 = in[0], xl = in[L];
      z[0] = make_float2(x0.x + xl.x, x0.x - xl.x);
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
  for (int idx = threadIdx.x; idx < (rows << log2L); idx += blockDim.x) {
    const int r = idx >> log2L, n = idx & (L - 1);
    const float2 z = sbuf[r * PL + pidx(n)];
    reinterpret_cast<float2*>(x + (size_t)(i0 + r) * p.ny)[n] =
        make_float2(z.x * scale, z.y * scale);
  }
}

template <int SIGN>
__global__ void __launch_bounds__(256, 3) col_fft_kernel(SpecParams p, int W, int log2W, int bstride,
                               float2* __restrict__ X,
                               const float* __restrict__ mult) {
  extern __shared__ float2 sbuf[];
  const int N = p.nx, ncols = p.L + 1;
  const int c0 = blockIdx.x * W;
  for (int e = threadIdx.x; e < W * N; e += blockDim.x) {
    const int w = e & (W - 1), i = e >> log2W, c = c0 + w;
    sbuf[w * bstride + pidx(i)] = c < ncols ? X[(size_t)i * ncols + c] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  fft_inplace<SIGN>(sbuf, p.log2nx, W, bstride, p.twp_x, threadIdx.x);
  for (int e = threadIdx.x; e < W * N; e += blockDim.x) {
    const int w = e & (W - 1), i = e >> log2W, c = c0 + w;
    if (c < ncols) {
      float2 v = sbuf[w * bstride + pidx(i)];
      if (mult) v = c_scale(v, __ldg(mult + (size_t)i * ncols + c));
      X[(size_t)i * ncols + c] = v;
    }
  }
}

// spectral_curl_2d (spectral/utils.py:199-203): 2 pi i (vhat kx - uhat ky).
__global__ void curl_table_kernel(SpecParams p, const float2* __restrict__ fxh,
                                  const float2* __restrict__ fyh,
                                  float2* __restrict__ out) {
  const int ncols = p.L + 1;
  const size_t n = (size_t)p.nx * ncols;
  for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < n;
       g += (size_t)gridDim.x * blockDim.x) {
    const int kx = (int)(g / ncols), c = (int)(g - (size_t)kx * ncols);
    const float kxf = kx_of(p, kx), kyf = ky_of(p, c);
    const float2 a = fyh[g], b = fxh[g];
    const float2 d = make_float2(a.x * kxf - b.x * kyf, a.y * kxf - b.y * kyf);
    out[g] = make_float2(-(p.two_pi * d.y), p.two_pi * d.x);
  }
}

struct ColCfg {
  int W, log2W, bstride, blocks, threads;
  size_t smem;
};

ColCfg col_cfg(const SpecParams& p) {
  ColCfg c;
  int W = 4096 >> p.log2nx;  // 256-thread blocks
  if (W < 1) W = 1;
  const int ncols = p.L + 1;
  // W never needs to exceed the next power of two above ncols.
  int cap = 1;
  while (cap < ncols) cap <<= 1;
  if (W > cap) W = cap;
  c.W = W;
  c.log2W = ilog2(W);
  c.bstride = padded_len(p.nx) + 8;  // consecutive columns 16 banks apart
  c.blocks = (ncols + W - 1) / W;
  const int workers = fft_workers(p.log2nx, W);
  int t = ((workers + 31) / 32) * 32;
  c.threads = t < 64 ? 64 : t;
  c.smem = (size_t)W * c.bstride * sizeof(float2);
  return c;
}

int rows_per_block(int log2L, int batch_per_row, int nrows) {
  const int P = log2L >= 4 ? 16 : (1 << log2L);
  int rows = (256 * P) / (batch_per_row << log2L);
  if (rows < 1) rows = 1;
  if (rows > nrows) rows = nrows;
  return rows;
}

int threads_for(int workers) {
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

constexpr int kSpecCluster = 4;

bool spec_cluster_ok(const SpecParams& p) {
  return p.col_mode == 1 && p.nx >= 256 && p.nx <= 2048;
}

// col_mode 2: groups of 4 columns per block (2 at 4096 rows); 3: groups of 2;
// 4: groups of 4 with the update and the next stage's prep fused.
bool spec_pipe_ok(const SpecParams& p) {
  return p.col_mode >= 2 && p.col_mode <= 4 && p.log2nx >= 9 && p.log2nx <= 12;
}

// Persistent column passes: as many blocks as fit on the device at once,
// never more than there are work items.
template <int LOG2N, int CG, typename K>
static cudaError_t spec_pipe_grid(K kern, int items, int* grid, size_t* smem, int* threads) {
  *smem = col_pipe_smem<LOG2N, CG>();
  *threads = CG * (1 << LOG2N) / 16;
  cudaError_t e = set_smem(kern, *smem);
  if (e != cudaSuccess) return e;
  static std::atomic<int> per_sm_cache{0};  // per instantiation
  int per_sm = 1;
  e = cached_blocks_per_sm(kern, *threads, *smem, per_sm_cache, &per_sm);
  if (e != cudaSuccess) return e;
  const int slots = col_pipe_device_sms() * per_sm;
  *grid = items < slots ? items : slots;
  return cudaSuccess;
}

template <int LOG2N, int CG>
static cudaError_t spec_prep_pipe_impl(const SpecParams& p, const float2* w, const T4& tt,
                                       cudaStream_t s) {
  int grid, threads;
  size_t smem;
  auto kern = spec_col_prep_pipe_kernel<LOG2N, CG>;
  cudaError_t e = spec_pipe_grid<LOG2N, CG>(kern, 4 * ((p.L + 1 + CG - 1) / CG), &grid, &smem,
                                            &threads);
  if (e != cudaSuccess) return e;
  return launch_maybe_pdl(p.pdl, kern, dim3(grid), dim3(threads), smem, s, p, w, tt);
}

template <int LOG2N, int CG>
static cudaError_t spec_stage_pipe_impl(const SpecParams& p, const StageCoef& sc,
                                        const float2* ahat, float2* w, float2* h, const T4& tt,
                                        cudaStream_t s) {
  int grid, threads;
  size_t smem;
  auto kern = sc.tiled ? spec_col_stage_pipe_kernel<LOG2N, CG, true>
                       : spec_col_stage_pipe_kernel<LOG2N, CG, false>;
  cudaError_t e = spec_pipe_grid<LOG2N, CG>(kern, (p.L + 1 + CG - 1) / CG, &grid, &smem,
                                            &threads);
  if (e != cudaSuccess) return e;
  return launch_maybe_pdl(p.pdl, kern, dim3(grid), dim3(threads), smem, s, p, sc, ahat, w, h,
                          tt);
}

template <int LOG2N>
static cudaError_t spec_stage_tma_impl(const SpecParams& p, const StageCoef& sc, float2* w,
                                       float2* h, cudaStream_t s) {
  const SpecStageMaps* maps = static_cast<const SpecStageMaps*>(p.stage_maps);
  CUtensorMap amap;
  SpecT4Maps tm;
  std::memcpy(&amap, maps->ahat, sizeof(amap));
  for (int f = 0; f < 4; ++f) std::memcpy(&tm.t[f], maps->t[f], sizeof(CUtensorMap));
  auto kern = sc.tiled ? spec_col_stage_tma_kernel<LOG2N, true>
                       : spec_col_stage_tma_kernel<LOG2N, false>;
  const size_t smem = col_pipe_smem<LOG2N, 4>() + 16;  // + the mbarrier
  const int threads = 4 * (1 << LOG2N) / 16;
  cudaError_t e = set_smem(kern, smem);
  if (e != cudaSuccess) return e;
  static std::atomic<int> per_sm_cache{0};
  int per_sm = 1;
  e = cached_blocks_per_sm(kern, threads, smem, per_sm_cache, &per_sm);
  if (e != cudaSuccess) return e;
  const int items = (p.L + 1 + 3) / 4, slots = col_pipe_device_sms() * per_sm;
  return launch_maybe_pdl(p.pdl, kern, dim3(items < slots ? items : slots), dim3(threads), smem,
                          s, p, sc, amap, tm, w, h);
}

// The TMA-staged fused stage: groups of 4 columns of up to 2048 rows, where
// the plan's maps encoded.
bool spec_stage_tma_ok(const SpecParams& p) {
  return p.stage_maps && p.col_mode == 4 && spec_pipe_ok(p) && p.log2nx <= 11;
}

template <int LOG2N, int CG>
static cudaError_t spec_update_pipe_impl(const SpecParams& p, const StageCoef& sc,
                                         const float2* ahat, float2* w, float2* h,
                                         cudaStream_t s) {
  int grid, threads;
  size_t smem;
  auto kern = sc.tiled ? spec_col_update_pipe_kernel<LOG2N, CG, true>
                       : spec_col_update_pipe_kernel<LOG2N, CG, false>;
  cudaError_t e = spec_pipe_grid<LOG2N, CG>(kern, (p.L + 1 + CG - 1) / CG, &grid, &smem,
                                            &threads);
  if (e != cudaSuccess) return e;
  return launch_maybe_pdl(p.pdl, kern, dim3(grid), dim3(threads), smem, s, p, sc, ahat, w, h);
}

cudaError_t launch_spec_col_prep(const SpecParams& p, const float2* w,
                                 float2* const t4[4], cudaStream_t s) {
  T4 tt{{t4[0], t4[1], t4[2], t4[3]}};
  if (spec_pipe_ok(p) && p.col_mode == 3) {
    switch (p.log2nx) {
      case 9: return spec_prep_pipe_impl<9, 2>(p, w, tt, s);
      case 10: return spec_prep_pipe_impl<10, 2>(p, w, tt, s);
      case 11: return spec_prep_pipe_impl<11, 2>(p, w, tt, s);
      default: return spec_prep_pipe_impl<12, 2>(p, w, tt, s);
    }
  }
  if (spec_pipe_ok(p)) {
    switch (p.log2nx) {
      case 9: return spec_prep_pipe_impl<9, 4>(p, w, tt, s);
      case 10: return spec_prep_pipe_impl<10, 4>(p, w, tt, s);
      case 11: return spec_prep_pipe_impl<11, 4>(p, w, tt, s);
      default: return spec_prep_pipe_impl<12, 2>(p, w, tt, s);
    }
  }
  if (spec_cluster_ok(p)) {
    const int ncols = p.L + 1;
    const int gx = (ncols + kSpecCluster - 1) / kSpecCluster * kSpecCluster;
    const size_t smem = (size_t)padded_len(p.nx) * sizeof(float2);
    cudaError_t e = set_smem(spec_col_prep_cluster_kernel<kSpecCluster>, smem);
    if (e != cudaSuccess) return e;
    spec_col_prep_cluster_kernel<kSpecCluster><<<dim3(gx, 4), threads_for(fft_workers(p.log2nx, 1)),
                                                 smem, s>>>(p, w, tt);
    return cudaGetLastError();
  }
  const ColCfg c = col_cfg(p);
  cudaError_t e = set_smem(spec_col_prep_kernel, c.smem);
  if (e != cudaSuccess) return e;
  T4 t{{t4[0], t4[1], t4[2], t4[3]}};
  spec_col_prep_kernel<<<dim3(c.blocks, 4), c.threads, c.smem, s>>>(
      p, c.W, c.log2W, c.bstride, w, t);
  return cudaGetLastError();
}

cudaError_t launch_spec_col_update(const SpecParams& p, const StageCoef& sc,
                                   const float2* ahat, float2* w, float2* h,
                                   float2* const t4[4], cudaStream_t s) {
  cudaError_t e;
  if (spec_pipe_ok(p) && p.col_mode == 4 && sc.prep_next && !sc.explicit_only) {
    // Update and the next stage's prep in one pass.
    if (spec_stage_tma_ok(p)) {
      switch (p.log2nx) {
        case 9: return spec_stage_tma_impl<9>(p, sc, w, h, s);
        case 10: return spec_stage_tma_impl<10>(p, sc, w, h, s);
        default: return spec_stage_tma_impl<11>(p, sc, w, h, s);
      }
    }
    T4 tt{{t4[0], t4[1], t4[2], t4[3]}};
    switch (p.log2nx) {
      case 9: return spec_stage_pipe_impl<9, 4>(p, sc, ahat, w, h, tt, s);
      case 10: return spec_stage_pipe_impl<10, 4>(p, sc, ahat, w, h, tt, s);
      case 11: return spec_stage_pipe_impl<11, 4>(p, sc, ahat, w, h, tt, s);
      default: return spec_stage_pipe_impl<12, 2>(p, sc, ahat, w, h, tt, s);
    }
  }
  if (spec_pipe_ok(p) && p.col_mode == 3) {
    switch (p.log2nx) {
      case 9: e = spec_update_pipe_impl<9, 2>(p, sc, ahat, w, h, s); break;
      case 10: e = spec_update_pipe_impl<10, 2>(p, sc, ahat, w, h, s); break;
      case 11: e = spec_update_pipe_impl<11, 2>(p, sc, ahat, w, h, s); break;
      default: e = spec_update_pipe_impl<12, 2>(p, sc, ahat, w, h, s); break;
    }
    if (e != cudaSuccess) return e;
  } else if (spec_pipe_ok(p)) {
    switch (p.log2nx) {
      case 9: e = spec_update_pipe_impl<9, 4>(p, sc, ahat, w, h, s); break;
      case 10: e = spec_update_pipe_impl<10, 4>(p, sc, ahat, w, h, s); break;
      case 11: e = spec_update_pipe_impl<11, 4>(p, sc, ahat, w, h, s); break;
      default: e = spec_update_pipe_impl<12, 2>(p, sc, ahat, w, h, s); break;
    }
    if (e != cudaSuccess) return e;
  } else if (spec_cluster_ok(p)) {
    const int ncols = p.L + 1;
    const int gx = (ncols + kSpecCluster - 1) / kSpecCluster * kSpecCluster;
    const size_t smem = (size_t)padded_len(p.nx) * sizeof(float2);
    e = set_smem(spec_col_update_cluster_kernel<kSpecCluster>, smem);
    if (e != cudaSuccess) return e;
    spec_col_update_cluster_kernel<kSpecCluster><<<gx, threads_for(fft_workers(p.log2nx, 1)),
                                                   smem, s>>>(p, sc, ahat, w, h);
  } else {
    const ColCfg c = col_cfg(p);
    e = set_smem(spec_col_update_kernel, c.smem);
    if (e != cudaSuccess) return e;
    spec_col_update_kernel<<<c.blocks, c.threads, c.smem, s>>>(
        p, sc, c.W, c.log2W, c.bstride, ahat, w, h);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess || !sc.prep_next || sc.explicit_only) return e;
  return launch_spec_col_prep(p, w, t4, s);
}

template <int LOG2L, int OCC>
static cudaError_t spec_row_pipe_impl(const SpecParams& p, const float2* const t4[4],
                                      float2* ahat, cudaStream_t s) {
  const size_t smem = spec_row_pipe_smem<LOG2L>();
  auto kern = spec_row_pipe_kernel<LOG2L, OCC>;
  cudaError_t e = set_smem(kern, smem);
  if (e != cudaSuccess) return e;
  return launch_maybe_pdl(p.pdl, kern, dim3(p.nx), dim3(4 * (1 << LOG2L) / 16), smem, s, p,
                          t4[0], t4[1], t4[2], t4[3], ahat);
}

// The tiled layout serves the groups of 4 columns of the fused column stage
// (rows up to 2048; 4096 rows take groups of 2).
bool spec_state_tiled_ok(const SpecParams& p) {
  return p.col_mode == 4 && spec_pipe_ok(p) && p.log2nx <= 11;
}

size_t spec_tiled_elems(const SpecParams& p) {
  return (size_t)((p.L + 1 + 3) / 4) * p.nx * 4;
}

// Row-major [nx, L + 1] <-> tiled by groups of 4 columns (state_at); the
// tiled side is walked in order, so its accesses are contiguous.  Padding
// columns of the last group read as zeros and are not written back.
__global__ void spec_tile_state_kernel(int nx, int ncols, const float2* __restrict__ src,
                                       float2* __restrict__ dst, int to_tiled) {
  const size_t total = (size_t)((ncols + 3) / 4) * nx * 4;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int w = (int)(i & 3);
    const size_t r = i >> 2;
    const int kx = (int)(r % (size_t)nx), c = (int)(r / (size_t)nx) * 4 + w;
    const size_t j = (size_t)kx * ncols + c;
    if (to_tiled)
      dst[i] = c < ncols ? src[j] : make_float2(0.f, 0.f);
    else if (c < ncols)
      dst[j] = src[i];
  }
}

cudaError_t spec_tile_state(const SpecParams& p, const float2* src, float2* dst, bool to_tiled,
                            cudaStream_t s) {
  const size_t total = spec_tiled_elems(p);
  size_t blocks = (total + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  spec_tile_state_kernel<<<(int)blocks, 256, 0, s>>>(p.nx, p.L + 1, src, dst, to_tiled ? 1 : 0);
  return cudaGetLastError();
}

bool spec_row_pipe_ok(const SpecParams& p) {
  // row_mode 2 sizes registers for 768 resident threads (1024 at ny = 2048):
  // blocks of <= 256.
  return p.log2L >= 8 && p.log2L <= (p.row_mode == 2 ? 10 : 11);
}

cudaError_t launch_spec_row(const SpecParams& p, const float2* const t4[4],
                            float2* ahat, cudaStream_t s) {
  if (p.row_mode == 2 && spec_row_pipe_ok(p)) {
    switch (p.log2L) {
      case 8: return spec_row_pipe_impl<8, 768>(p, t4, ahat, s);
      case 9: return spec_row_pipe_impl<9, 768>(p, t4, ahat, s);
      default: return spec_row_pipe_impl<10, 1024>(p, t4, ahat, s);
    }
  }
  if (p.row_mode >= 1 && spec_row_pipe_ok(p)) {
    switch (p.log2L) {
      case 8: return spec_row_pipe_impl<8, 512>(p, t4, ahat, s);
      case 9: return spec_row_pipe_impl<9, 512>(p, t4, ahat, s);
      case 10: return spec_row_pipe_impl<10, 512>(p, t4, ahat, s);
      default: return spec_row_pipe_impl<11, 512>(p, t4, ahat, s);
    }
  }
  const int rows = rows_per_block(p.log2L, 4, p.nx);
  const size_t smem = (size_t)rows * 4 * padded_len(p.L) * sizeof(float2);
  cudaError_t e = set_smem(spec_row_kernel, smem);
  if (e != cudaSuccess) return e;
  return launch_maybe_pdl(p.pdl, spec_row_kernel, dim3(p.nx / rows),
                          dim3(threads_for(fft_workers(p.log2L, rows * 4))), smem, s, p, rows,
                          t4[0], t4[1], t4[2], t4[3], ahat);
}

cudaError_t launch_row_rfft(const SpecParams& p, const float* x, float2* X,
                            cudaStream_t s) {
  const int rows = rows_per_block(p.log2L, 1, p.nx);
  const size_t smem = (size_t)rows * padded_len(p.L) * sizeof(float2);
  cudaError_t e = set_smem(row_rfft_kernel, smem);
  if (e != cudaSuccess) return e;
  row_rfft_kernel<<<p.nx / rows, threads_for(fft_workers(p.log2L, rows)), smem,
                    s>>>(p, rows, x, X);
  return cudaGetLastError();
}

cudaError_t launch_row_irfft(const SpecParams& p, const float2* X, float* x,
                             float scale, cudaStream_t s) {
  const int rows = rows_per_block(p.log2L, 1, p.nx);
  const size_t smem = (size_t)rows * padded_len(p.L) * sizeof(float2);
  cudaError_t e = set_smem(row_irfft_kernel, smem);
  if (e != cudaSuccess) return e;
  row_irfft_kernel<<<p.nx / rows, threads_for(fft_workers(p.log2L, rows)), smem,
                     s>>>(p, rows, X, x, scale);
  return cudaGetLastError();
}

cudaError_t launch_col_fft(const SpecParams& p, float2* X, int sign,
                           const float* mult, cudaStream_t s) {
  const ColCfg c = col_cfg(p);
  cudaError_t e;
  if (sign < 0) {
    e = set_smem(col_fft_kernel<-1>, c.smem);
    if (e != cudaSuccess) return e;
    col_fft_kernel<-1><<<c.blocks, c.threads, c.smem, s>>>(p, c.W, c.log2W,
                                                           c.bstride, X, mult);
  } else {
    e = set_smem(col_fft_kernel<1>, c.smem);
    if (e != cudaSuccess) return e;
    col_fft_kernel<1><<<c.blocks, c.threads, c.smem, s>>>(p, c.W, c.log2W,
                                                          c.bstride, X, mult);
  }
  return cudaGetLastError();
}

cudaError_t launch_spec_curl_table(const SpecParams& p, const float2* fxh,
                                   const float2* fyh, float2* out,
                                   cudaStream_t s) {
  const size_t n = (size_t)p.nx * (p.L + 1);
  size_t b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  curl_table_kernel<<<(int)b, 256, 0, s>>>(p, fxh, fyh, out);
  return cudaGetLastError();
}

// Batched pipelined passes (column scheme 4 and the register row pass).
template <int LOG2N, int CG>
static cudaError_t spec_batch_stage_pipe_impl(const SpecParams& p, const SpecMember* mem,
                                              int count, int k, int stage, cudaStream_t s) {
  int grid, threads;
  size_t smem;
  auto kern = spec_batch_col_stage_pipe_kernel<LOG2N, CG>;
  const long long items = (long long)count * ((p.L + 1 + CG - 1) / CG);
  cudaError_t e = spec_pipe_grid<LOG2N, CG>(kern, (int)(items < (1 << 30) ? items : (1 << 30)),
                                            &grid, &smem, &threads);
  if (e != cudaSuccess) return e;
  kern<<<grid, threads, smem, s>>>(mem, count, k, stage);
  return cudaGetLastError();
}

template <int LOG2N, int CG>
static cudaError_t spec_batch_prep_pipe_impl(const SpecParams& p, const SpecMember* mem,
                                             int count, cudaStream_t s) {
  int grid, threads;
  size_t smem;
  auto kern = spec_batch_col_prep_pipe_kernel<LOG2N, CG>;
  const long long items = (long long)count * 4 * ((p.L + 1 + CG - 1) / CG);
  cudaError_t e = spec_pipe_grid<LOG2N, CG>(kern, (int)(items < (1 << 30) ? items : (1 << 30)),
                                            &grid, &smem, &threads);
  if (e != cudaSuccess) return e;
  kern<<<grid, threads, smem, s>>>(mem, count);
  return cudaGetLastError();
}

static bool spec_batch_fused(const SpecParams& p) { return p.col_mode == 4 && spec_pipe_ok(p); }

cudaError_t launch_spec_batch_prep(const SpecParams& p, const SpecMember* mem, int count,
                                   int k, int stage, cudaStream_t s) {
  if (count < 1 || count > 65535) return cudaErrorInvalidValue;
  if (spec_batch_fused(p)) {
    if (k >= 0) return cudaSuccess;  // built by the fused update pass
    switch (p.log2nx) {
      case 9: return spec_batch_prep_pipe_impl<9, 4>(p, mem, count, s);
      case 10: return spec_batch_prep_pipe_impl<10, 4>(p, mem, count, s);
      case 11: return spec_batch_prep_pipe_impl<11, 4>(p, mem, count, s);
      default: return spec_batch_prep_pipe_impl<12, 2>(p, mem, count, s);
    }
  }
  const ColCfg c = col_cfg(p);
  cudaError_t e = set_smem(spec_batch_col_prep_kernel, c.smem);
  if (e != cudaSuccess) return e;
  spec_batch_col_prep_kernel<<<dim3(c.blocks, 4, count), c.threads, c.smem, s>>>(
      mem, k, stage, c.W, c.log2W, c.bstride);
  return cudaGetLastError();
}

template <int LOG2L>
static cudaError_t spec_batch_row_pipe_impl(const SpecParams& p, const SpecMember* mem, int count,
                                            int k, cudaStream_t s) {
  const size_t smem = spec_row_pipe_smem<LOG2L>();
  auto kern = spec_batch_row_pipe_kernel<LOG2L>;
  cudaError_t e = set_smem(kern, smem);
  if (e != cudaSuccess) return e;
  kern<<<dim3(p.nx, count), 4 * (1 << LOG2L) / 16, smem, s>>>(mem, k);
  return cudaGetLastError();
}

cudaError_t launch_spec_batch_row(const SpecParams& p, const SpecMember* mem, int count, int k,
                                  cudaStream_t s) {
  if (count < 1 || count > 65535) return cudaErrorInvalidValue;
  if (p.row_mode == 1 && spec_row_pipe_ok(p)) {
    switch (p.log2L) {
      case 8: return spec_batch_row_pipe_impl<8>(p, mem, count, k, s);
      case 9: return spec_batch_row_pipe_impl<9>(p, mem, count, k, s);
      case 10: return spec_batch_row_pipe_impl<10>(p, mem, count, k, s);
      default: return spec_batch_row_pipe_impl<11>(p, mem, count, k, s);
    }
  }
  const int rows = rows_per_block(p.log2L, 4, p.nx);
  const size_t smem = (size_t)rows * 4 * padded_len(p.L) * sizeof(float2);
  cudaError_t e = set_smem(spec_batch_row_kernel, smem);
  if (e != cudaSuccess) return e;
  spec_batch_row_kernel<<<dim3(p.nx / rows, count), threads_for(fft_workers(p.log2L, rows * 4)),
                          smem, s>>>(mem, k, rows);
  return cudaGetLastError();
}

cudaError_t launch_spec_batch_update(const SpecParams& p, const SpecMember* mem, int count,
                                     int k, int stage, cudaStream_t s) {
  if (count < 1 || count > 65535) return cudaErrorInvalidValue;
  if (spec_batch_fused(p)) {
    switch (p.log2nx) {
      case 9: return spec_batch_stage_pipe_impl<9, 4>(p, mem, count, k, stage, s);
      case 10: return spec_batch_stage_pipe_impl<10, 4>(p, mem, count, k, stage, s);
      case 11: return spec_batch_stage_pipe_impl<11, 4>(p, mem, count, k, stage, s);
      default: return spec_batch_stage_pipe_impl<12, 2>(p, mem, count, k, stage, s);
    }
  }
  const ColCfg c = col_cfg(p);
  cudaError_t e = set_smem(spec_batch_col_update_kernel, c.smem);
  if (e != cudaSuccess) return e;
  spec_batch_col_update_kernel<<<dim3(c.blocks, count), c.threads, c.smem, s>>>(
      mem, k, stage, c.W, c.log2W, c.bstride);
  return cudaGetLastError();
}

cudaError_t launch_shell_energy(const SpecParams& p, double dnx, double dny, double ks,
                                int nbins, const float2* uh, const float2* vh, double* out,
                                cudaStream_t s) {
  if (nbins < 1 || nbins > 8192) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(out, 0, (size_t)nbins * sizeof(double), s);
  if (e != cudaSuccess) return e;
  const size_t n = (size_t)p.nx * (p.L + 1);
  size_t blocks = (n + 255) / 256;
  if (blocks > 152 * 4) blocks = 152 * 4;
  shell_energy_kernel<<<(int)blocks, 256, (size_t)nbins * sizeof(double), s>>>(
      p.nx, p.ny, dnx, dny, ks, nbins, uh, vh, out);
  return cudaGetLastError();
}

cudaError_t launch_enstrophy_sum(int nx, int ny, float hx, float hy, const float* u,
                                 const float* v, double* out, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double), s);
  if (e != cudaSuccess) return e;
  const size_t n = (size_t)nx * ny;
  size_t blocks = (n + 255) / 256;
  if (blocks > 152 * 4) blocks = 152 * 4;
  enstrophy_sum_kernel<<<(int)blocks, 256, 0, s>>>(nx, ny, hx, hy, u, v, out);
  return cudaGetLastError();
}

}  // namespace cfd
