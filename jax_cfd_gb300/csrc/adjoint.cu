// Hand-written adjoint (vector-Jacobian product) of one forward-Euler FVM
// step of semi_implicit_navier_stokes (equations.py:120-151,
// time_stepping.py:59-119):
//
//   v' = P(v + dt F(v)),  F = advection (advection.py:81-116,387-395)
//                           + (nu / rho) laplacian (diffusion.py:35-37)
//                           + forcing / rho (forcings.py:107-178),
//
// so for a cotangent g of v':  w = P^T g = P g (the projection
// I - grad L^+ div is self-adjoint: backward difference = -forward^T), and
//
//   g_v  = w + dt (A(v)^T w + (nu/rho) laplacian(w) + (lin/rho) w)
//   g_nu = dt / rho * <w, laplacian(v)>     (summed by the caller)
//
// A(v)^T is the transpose of the Jacobian of the limited Van Leer (or
// linear) advection: each face flux F = c_face(c[-1..2], U) * U, with the
// derivative of apply_tvd_limiter(lax_wendroff, van_leer_limiter)
// (interpolation.py:158-303) taken branch by branch the way jax.grad
// differentiates jnp.where and safe_div (the unselected branch and the
// replaced denominator get no gradient).  A block owns a 16 x 32 tile of
// cells: it first evaluates the vector-Jacobian product of every face of the
// four flux families (u and v, x- and y-normal faces) that the tile's cells
// read, once per face, into shared memory, then each cell gathers the
// contributions of the faces that read it: as advected quantity (4 faces per
// direction) and as face velocity (2 faces).
#include "common.cuh"
#include "kernels.h"

namespace cfd {
namespace {

struct FaceVjp {
  float g[4];  // dF/dc[-1], dF/dc[0], dF/dc[+1], dF/dc[+2], times Fbar
  float gU;    // dF/dU times Fbar
};

template <int CONVECT>
CFD_D FaceVjp face_vjp(float cm, float c0, float c1, float c2, float U, float cfl,
                       float Fbar) {
  FaceVjp o;
  if (CONVECT == 1) {
    // interpolation.linear: c_face = 0.5 c0 + 0.5 c1; F = c_face * U.
    const float h = 0.5f * U * Fbar;
    o.g[0] = 0.f;
    o.g[1] = h;
    o.g[2] = h;
    o.g[3] = 0.f;
    o.gU = (0.5f * c0 + 0.5f * c1) * Fbar;
    return o;
  }
  // Upwind-mirrored stencil (a, b, c) = U > 0 ? (cm, c0, c1) : (c2, c1, c0):
  // c_face = b + kappa d phi(r), kappa = (1 - |C|) / 2, d = c - b,
  // r = (b - a) / d (the reference's ratio in both branches).
  const bool pos = U > 0.f;
  const float a = pos ? cm : c2, b = pos ? c0 : c1, c = pos ? c1 : c0;
  const float C = cfl * U;
  const float kap = 0.5f * (1.f - fabsf(C));
  const float d = c - b, n = b - a;
  // safe_div: where d == 0 the reference divides its own numerator by 1,
  // which is (b - a) for U > 0 and (a - b) otherwise.
  // (Approximate reciprocals: the derivative is compared with float64
  // autograd within float32 tolerances, not bit for bit.)
  const float r = d != 0.f ? __fdividef(n, d) : (pos ? n : -n);
  const bool lim = r > 0.f;
  const float inv = lim ? __fdividef(1.f, 1.f + r) : 0.f;
  const float phi = 2.f * r * inv;
  const float dphi = 2.f * inv * inv;
  const float cf = b + kap * d * phi;
  float da, db, dc;
  if (d != 0.f) {
    da = -kap * dphi;
    dc = kap * (phi - r * dphi);
    db = 1.f - kap * phi + kap * dphi * (1.f + r);
  } else {
    da = 0.f;
    dc = kap * phi;
    db = 1.f - kap * phi;
  }
  // d kappa / dU = -cfl sign(U) / 2, with U <= 0 taking the negative branch.
  const float dcf_dU = -0.5f * (pos ? cfl : -cfl) * d * phi;
  const float FU = Fbar * U;
  if (pos) {
    o.g[0] = FU * da;
    o.g[1] = FU * db;
    o.g[2] = FU * dc;
    o.g[3] = 0.f;
  } else {
    o.g[0] = 0.f;
    o.g[1] = FU * dc;
    o.g[2] = FU * db;
    o.g[3] = FU * da;
  }
  o.gU = Fbar * (cf + U * dcf_dU);
  return o;
}

struct Field {
  const float* __restrict__ a;
  int mx, my, log2ny;
  CFD_D float operator()(int i, int j) const {
    return __ldg(a + ((size_t)(i & mx) << log2ny) + (j & my));
  }
};

CFD_D float lap_at(const FvmParams& p, const Field& f, int i, int j) {
  // finite_differences.laplacian: -2c * sum(scales) + pairs * scale.
  return ((-2.f * f(i, j)) * p.ssum + (f(i - 1, j) + f(i + 1, j)) * p.sx) +
         (f(i, j - 1) + f(i, j + 1)) * p.sy;
}

constexpr int kAdjTI = 16, kAdjTJ = 32;                  // cells per tile
constexpr int kAdjFI = kAdjTI + 3, kAdjFJ = kAdjTJ + 3;  // faces: rows/cols from i0-2 / j0-2
constexpr int kAdjFaces = kAdjFI * kAdjFJ;
constexpr int kAdjThreads = 256;
// Shared memory: 4 families x 5 values (g[0..3], gU) per face.
constexpr size_t kAdjSmem = (size_t)4 * 5 * kAdjFaces * sizeof(float);

template <int CONVECT>
__global__ void __launch_bounds__(kAdjThreads)
    fvm_adjoint_kernel(FvmParams p, const float* __restrict__ u, const float* __restrict__ v,
                       const float* __restrict__ wu_, const float* __restrict__ wv_,
                       float* __restrict__ gu, float* __restrict__ gv,
                       float* __restrict__ nu_dot) {
  extern __shared__ float adj_smem[];
  const int mx = p.nx - 1, my = p.ny - 1;
  const Field U{u, mx, my, p.log2ny}, V{v, mx, my, p.log2ny};
  const Field WU{wu_, mx, my, p.log2ny}, WV{wv_, mx, my, p.log2ny};
  const int i0 = blockIdx.y * kAdjTI, j0 = blockIdx.x * kAdjTJ;
  const int tid = threadIdx.x;
  // Family f, value k of face slot s at adj_smem[(f * 5 + k) * kAdjFaces + s];
  // slot s = (fi - i0 + 2) * kAdjFJ + (fj - j0 + 2).
  auto rec = [&](int fam, int k, int fi, int fj) -> float& {
    return adj_smem[(fam * 5 + k) * kAdjFaces + (fi - i0 + 2) * kAdjFJ + (fj - j0 + 2)];
  };
  for (int e = tid; e < 4 * kAdjFaces; e += kAdjThreads) {
    const int fam = e / kAdjFaces, sl = e - fam * kAdjFaces;
    const int fi = i0 - 2 + sl / kAdjFJ, fj = j0 - 2 + sl % kAdjFJ;
    FaceVjp o;
    if (fam == 0) {
      // u's x-face after row fi: c = u along x, U = 0.5 u[fi] + 0.5 u[fi+1].
      o = face_vjp<CONVECT>(U(fi - 1, fj), U(fi, fj), U(fi + 1, fj), U(fi + 2, fj),
                            0.5f * U(fi, fj) + 0.5f * U(fi + 1, fj), p.cfl_x,
                            (WU(fi + 1, fj) - WU(fi, fj)) * p.inv_hx);
    } else if (fam == 1) {
      // u's y-face after column fj: c = u along y, V = 0.5 v[fi] + 0.5 v[fi+1].
      o = face_vjp<CONVECT>(U(fi, fj - 1), U(fi, fj), U(fi, fj + 1), U(fi, fj + 2),
                            0.5f * V(fi, fj) + 0.5f * V(fi + 1, fj), p.cfl_y,
                            (WU(fi, fj + 1) - WU(fi, fj)) * p.inv_hy);
    } else if (fam == 2) {
      // v's y-face after column fj: c = v along y, V = 0.5 v[fj] + 0.5 v[fj+1].
      o = face_vjp<CONVECT>(V(fi, fj - 1), V(fi, fj), V(fi, fj + 1), V(fi, fj + 2),
                            0.5f * V(fi, fj) + 0.5f * V(fi, fj + 1), p.cfl_y,
                            (WV(fi, fj + 1) - WV(fi, fj)) * p.inv_hy);
    } else {
      // v's x-face after row fi: c = v along x, U = 0.5 u[fj] + 0.5 u[fj+1].
      o = face_vjp<CONVECT>(V(fi - 1, fj), V(fi, fj), V(fi + 1, fj), V(fi + 2, fj),
                            0.5f * U(fi, fj) + 0.5f * U(fi, fj + 1), p.cfl_x,
                            (WV(fi + 1, fj) - WV(fi, fj)) * p.inv_hx);
    }
    float* base = adj_smem + fam * 5 * kAdjFaces + sl;
    base[0] = o.g[0];
    base[kAdjFaces] = o.g[1];
    base[2 * kAdjFaces] = o.g[2];
    base[3 * kAdjFaces] = o.g[3];
    base[4 * kAdjFaces] = o.gU;
  }
  __syncthreads();
  for (int c = tid; c < kAdjTI * kAdjTJ; c += kAdjThreads) {
    const int i = i0 + c / kAdjTJ, j = j0 + c % kAdjTJ;
    if (i > mx || j > my) continue;
    float au = 0.f, av = 0.f;
#pragma unroll
    for (int q = -1; q <= 2; ++q) {
      // u's x-faces f = i - q and v's x-faces f = i - q at column j.
      au += rec(0, q + 1, i - q, j);
      av += rec(3, q + 1, i - q, j);
      // u's and v's y-faces g = j - q at row i.
      au += rec(1, q + 1, i, j - q);
      av += rec(2, q + 1, i, j - q);
      if (q == 0 || q == 1) {
        au += 0.5f * rec(0, 4, i - q, j);
        av += 0.5f * rec(2, 4, i, j - q);
      }
      if (q == 0) {
        av += 0.5f * rec(1, 4, i, j);
        au += 0.5f * rec(3, 4, i, j);
      }
    }
    // The two velocity-only faces: u's y-face (i-1, j) reads v[i, j] and v's
    // x-face (i, j-1) reads u[i, j].
    av += 0.5f * rec(1, 4, i - 1, j);
    au += 0.5f * rec(3, 4, i, j - 1);
    const float wu = WU(i, j), wv = WV(i, j);
    float ku = au, kv = av;
    if (p.has_visc) {
      ku += p.nu * lap_at(p, WU, i, j);
      kv += p.nu * lap_at(p, WV, i, j);
    }
    if (p.has_lin) {
      const float lin = p.rho_is_one ? p.lin : p.lin / p.density;
      ku += lin * wu;
      kv += lin * wv;
    }
    const size_t idx = ((size_t)i << p.log2ny) + j;
    gu[idx] = wu + p.dt * ku;
    gv[idx] = wv + p.dt * kv;
    if (nu_dot) nu_dot[idx] = wu * lap_at(p, U, i, j) + wv * lap_at(p, V, i, j);
  }
}

// Deterministic float -> double sum: kSumBlocks fixed blocks each reduce a
// grid-stride share in a fixed tree, then one thread adds the block partials
// in order to *acc.  The same inputs give the same bits whatever else runs.
constexpr int kSumThreads = 256;
__global__ void __launch_bounds__(kSumThreads)
    sum_partials_kernel(const float* __restrict__ x, size_t n, double* __restrict__ partials) {
  __shared__ double sh[kSumThreads];
  double acc = 0.0;
  for (size_t i = (size_t)blockIdx.x * kSumThreads + threadIdx.x; i < n;
       i += (size_t)gridDim.x * kSumThreads)
    acc += (double)x[i];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int w = kSumThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partials[blockIdx.x] = sh[0];
}

__global__ void sum_finish_kernel(const double* __restrict__ partials, int count,
                                  double* __restrict__ acc) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double t = 0.0;
  for (int b = 0; b < count; ++b) t += partials[b];
  *acc += t;
}

}  // namespace

cudaError_t launch_sum_to_double(const float* x, size_t n, double* partials, double* acc,
                                 cudaStream_t s) {
  sum_partials_kernel<<<kSumBlocks, kSumThreads, 0, s>>>(x, n, partials);
  sum_finish_kernel<<<1, 32, 0, s>>>(partials, kSumBlocks, acc);
  return cudaGetLastError();
}

cudaError_t launch_fvm_adjoint(const FvmParams& p, const float* u, const float* v,
                               const float* wu, const float* wv, float* gu, float* gv,
                               float* nu_dot, cudaStream_t s) {
  const dim3 grid((p.ny + kAdjTJ - 1) / kAdjTJ, (p.nx + kAdjTI - 1) / kAdjTI);
  if (p.convect == 0) {
    cudaError_t e = cudaFuncSetAttribute(fvm_adjoint_kernel<0>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kAdjSmem);
    if (e != cudaSuccess) return e;
    fvm_adjoint_kernel<0><<<grid, kAdjThreads, kAdjSmem, s>>>(p, u, v, wu, wv, gu, gv, nu_dot);
  } else {
    cudaError_t e = cudaFuncSetAttribute(fvm_adjoint_kernel<1>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kAdjSmem);
    if (e != cudaSuccess) return e;
    fvm_adjoint_kernel<1><<<grid, kAdjThreads, kAdjSmem, s>>>(p, u, v, wu, wv, gu, gv, nu_dot);
  }
  return cudaGetLastError();
}

}  // namespace cfd
