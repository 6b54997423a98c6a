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
// replaced denominator get no gradient).  A thread owns one cell and gathers
// the contributions of every face flux that reads the cell: as advected
// quantity (4 faces per direction) and as face velocity (2 faces).
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
  const float r = d != 0.f ? n / d : (pos ? n : -n);
  const bool lim = r > 0.f;
  const float phi = lim ? 2.f * r / (1.f + r) : 0.f;
  const float dphi = lim ? 2.f / ((1.f + r) * (1.f + r)) : 0.f;
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

template <int CONVECT>
__global__ void __launch_bounds__(256)
    fvm_adjoint_kernel(FvmParams p, const float* __restrict__ u, const float* __restrict__ v,
                       const float* __restrict__ wu_, const float* __restrict__ wv_,
                       float* __restrict__ gu, float* __restrict__ gv,
                       float* __restrict__ nu_dot) {
  const int mx = p.nx - 1, my = p.ny - 1;
  const Field U{u, mx, my, p.log2ny}, V{v, mx, my, p.log2ny};
  const Field WU{wu_, mx, my, p.log2ny}, WV{wv_, mx, my, p.log2ny};
  const size_t n = (size_t)p.nx * p.ny;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(idx >> p.log2ny), j = (int)(idx & my);
    float au = 0.f, av = 0.f;
#pragma unroll
    for (int q = -1; q <= 2; ++q) {
      // u's x-faces f = i - q: c = u along x, U = 0.5 u[f] + 0.5 u[f+1].
      {
        const int f = i - q;
        const FaceVjp o = face_vjp<CONVECT>(
            U(f - 1, j), U(f, j), U(f + 1, j), U(f + 2, j), 0.5f * U(f, j) + 0.5f * U(f + 1, j),
            p.cfl_x, (WU(f + 1, j) - WU(f, j)) * p.inv_hx);
        au += o.g[q + 1];
        if (q == 0 || q == 1) au += 0.5f * o.gU;
      }
      // u's y-faces g = j - q: c = u along y, V = 0.5 v[i, g] + 0.5 v[i+1, g].
      {
        const int g = j - q;
        const FaceVjp o = face_vjp<CONVECT>(
            U(i, g - 1), U(i, g), U(i, g + 1), U(i, g + 2), 0.5f * V(i, g) + 0.5f * V(i + 1, g),
            p.cfl_y, (WU(i, g + 1) - WU(i, g)) * p.inv_hy);
        au += o.g[q + 1];
        if (q == 0) av += 0.5f * o.gU;
      }
      // v's y-faces g = j - q: c = v along y, V = 0.5 v[g] + 0.5 v[g+1].
      {
        const int g = j - q;
        const FaceVjp o = face_vjp<CONVECT>(
            V(i, g - 1), V(i, g), V(i, g + 1), V(i, g + 2), 0.5f * V(i, g) + 0.5f * V(i, g + 1),
            p.cfl_y, (WV(i, g + 1) - WV(i, g)) * p.inv_hy);
        av += o.g[q + 1];
        if (q == 0 || q == 1) av += 0.5f * o.gU;
      }
      // v's x-faces f = i - q: c = v along x, U = 0.5 u[f, j] + 0.5 u[f, j+1].
      {
        const int f = i - q;
        const FaceVjp o = face_vjp<CONVECT>(
            V(f - 1, j), V(f, j), V(f + 1, j), V(f + 2, j), 0.5f * U(f, j) + 0.5f * U(f, j + 1),
            p.cfl_x, (WV(f + 1, j) - WV(f, j)) * p.inv_hx);
        av += o.g[q + 1];
        if (q == 0) au += 0.5f * o.gU;
      }
    }
    // The two velocity-only faces: u's y-face (i-1, j) reads v[i, j] and v's
    // x-face (i, j-1) reads u[i, j].
    {
      const FaceVjp o = face_vjp<CONVECT>(
          U(i - 1, j - 1), U(i - 1, j), U(i - 1, j + 1), U(i - 1, j + 2),
          0.5f * V(i - 1, j) + 0.5f * V(i, j), p.cfl_y, (WU(i - 1, j + 1) - WU(i - 1, j)) * p.inv_hy);
      av += 0.5f * o.gU;
    }
    {
      const FaceVjp o = face_vjp<CONVECT>(
          V(i - 1, j - 1), V(i, j - 1), V(i + 1, j - 1), V(i + 2, j - 1),
          0.5f * U(i, j - 1) + 0.5f * U(i, j), p.cfl_x, (WV(i + 1, j - 1) - WV(i, j - 1)) * p.inv_hx);
      au += 0.5f * o.gU;
    }
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
    gu[idx] = wu + p.dt * ku;
    gv[idx] = wv + p.dt * kv;
    if (nu_dot) nu_dot[idx] = wu * lap_at(p, U, i, j) + wv * lap_at(p, V, i, j);
  }
}

}  // namespace

cudaError_t launch_fvm_adjoint(const FvmParams& p, const float* u, const float* v,
                               const float* wu, const float* wv, float* gu, float* gv,
                               float* nu_dot, cudaStream_t s) {
  const size_t n = (size_t)p.nx * p.ny;
  size_t blocks = (n + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;
  if (p.convect == 0)
    fvm_adjoint_kernel<0><<<(int)blocks, 256, 0, s>>>(p, u, v, wu, wv, gu, gv, nu_dot);
  else
    fvm_adjoint_kernel<1><<<(int)blocks, 256, 0, s>>>(p, u, v, wu, wv, gu, gv, nu_dot);
  return cudaGetLastError();
}

}  // namespace cfd
