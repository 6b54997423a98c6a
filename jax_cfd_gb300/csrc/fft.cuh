// Shared-memory Stockham FFT engine used by every transform on the hot path.
//
// A thread block holds `batch` complex sequences of length L = 2^log2L in
// shared memory (sequence b starts at buf + b * bstride) and transforms them
// in place.  Every pass is mixed-radix Stockham autosort (no bit reversal):
// pass p with radix R and running span Ns reads x[j + r*L/R], applies the
// twiddles w^(r * (j mod Ns) * L/(Ns*R)), does an R-point DFT in registers and
// writes y[(j/Ns)*Ns*R + (j mod Ns) + r*Ns].  Each thread owns P = min(16, L)
// points per pass (P/R butterflies), so the whole block issues exactly
// batch*L/P threads of work; all reads of a pass land in registers before a
// barrier and all writes happen after it, which is what makes in-place legal.
//
// Twiddles come from per-pass tables (fft_pass_table_offset) computed on the
// host in double precision and rounded once to float.  The inverse transform
// (SIGN = +1) conjugates them and is unnormalised, like the backward pass of
// numpy/jnp before their 1/n factor.
#pragma once

#include "common.cuh"

namespace cfd {

// w = cos(2*pi*k/16) + SIGN*i*sin(2*pi*k/16); a * w.
template <int SIGN>
CFD_D float2 twmul(float2 a, float c, float s) {
  const float ss = SIGN < 0 ? -s : s;
  return make_float2(__fmaf_rn(a.x, c, -(a.y * ss)), __fmaf_rn(a.x, ss, a.y * c));
}

constexpr float kC1_16 = 0.92387953251128675613f;  // cos(pi/8)
constexpr float kS1_16 = 0.38268343236508977173f;  // sin(pi/8)
constexpr float kSqrtHalf = 0.70710678118654752440f;

template <int R, int SIGN>
struct Dft;

template <int SIGN>
struct Dft<2, SIGN> {
  static CFD_D void run(float2* v) {
    const float2 a = v[0], b = v[1];
    v[0] = c_add(a, b);
    v[1] = c_sub(a, b);
  }
};

template <int SIGN>
struct Dft<4, SIGN> {
  static CFD_D void run(float2* v) {
    const float2 t0 = c_add(v[0], v[2]), t1 = c_sub(v[0], v[2]);
    const float2 t2 = c_add(v[1], v[3]), t3 = c_mul_i<SIGN>(c_sub(v[1], v[3]));
    v[0] = c_add(t0, t2);
    v[2] = c_sub(t0, t2);
    v[1] = c_add(t1, t3);
    v[3] = c_sub(t1, t3);
  }
};

template <int SIGN>
struct Dft<8, SIGN> {
  static CFD_D void run(float2* v) {
    float2 e[4] = {v[0], v[2], v[4], v[6]};
    float2 o[4] = {v[1], v[3], v[5], v[7]};
    Dft<4, SIGN>::run(e);
    Dft<4, SIGN>::run(o);
    const float2 t0 = o[0];
    const float2 t1 = twmul<SIGN>(o[1], kSqrtHalf, kSqrtHalf);
    const float2 t2 = c_mul_i<SIGN>(o[2]);
    const float2 t3 = twmul<SIGN>(o[3], -kSqrtHalf, kSqrtHalf);
    v[0] = c_add(e[0], t0); v[4] = c_sub(e[0], t0);
    v[1] = c_add(e[1], t1); v[5] = c_sub(e[1], t1);
    v[2] = c_add(e[2], t2); v[6] = c_sub(e[2], t2);
    v[3] = c_add(e[3], t3); v[7] = c_sub(e[3], t3);
  }
};

template <int SIGN>
struct Dft<16, SIGN> {
  static CFD_D void run(float2* v) {
    float2 e[8], o[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      e[k] = v[2 * k];
      o[k] = v[2 * k + 1];
    }
    Dft<8, SIGN>::run(e);
    Dft<8, SIGN>::run(o);
    float2 t[8];
    t[0] = o[0];
    t[1] = twmul<SIGN>(o[1], kC1_16, kS1_16);
    t[2] = twmul<SIGN>(o[2], kSqrtHalf, kSqrtHalf);
    t[3] = twmul<SIGN>(o[3], kS1_16, kC1_16);
    t[4] = c_mul_i<SIGN>(o[4]);
    t[5] = twmul<SIGN>(o[5], -kS1_16, kC1_16);
    t[6] = twmul<SIGN>(o[6], -kSqrtHalf, kSqrtHalf);
    t[7] = twmul<SIGN>(o[7], -kC1_16, kS1_16);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      v[k] = c_add(e[k], t[k]);
      v[k + 8] = c_sub(e[k], t[k]);
    }
  }
};

template <int R>
struct Log2c;
template <> struct Log2c<2> { static constexpr int v = 1; };
template <> struct Log2c<4> { static constexpr int v = 2; };
template <> struct Log2c<8> { static constexpr int v = 3; };
template <> struct Log2c<16> { static constexpr int v = 4; };

// Shared-memory index of complex element n: one padding slot after every 16
// elements, which spreads the stride-16 writes of the first radix-16 pass over
// all banks.  Every FFT buffer access goes through pidx(); a sequence of L
// elements occupies padded_len(L) slots.
CFD_HD int pidx(int n) { return n + (n >> 4); }
CFD_HD int padded_len(int L) { return L + (L >> 4); }

// Pass twiddle tables.  An FFT of length 2^log2L runs radix-16 passes at spans
// Ns = 1, 16, 256, ... and then one pass of the remaining radix R (2, 4 or 8);
// a pass with Ns > 1 reads w^(r*k), w = exp(-2 pi i / (Ns*R)), for r = 1..R-1
// and k = 0..Ns-1 from a table laid out [r-1][k] (k contiguous, so the lanes
// of a warp, which hold consecutive k, read consecutive addresses).  The
// tables of all passes are concatenated in pass order.
CFD_HD int fft_pass_radix(int log2L, int pass) {
  const int n16 = log2L >> 2;
  if (log2L < 4) return 1 << log2L;
  return pass < n16 ? 16 : (1 << (log2L & 3));
}
CFD_HD int fft_num_passes(int log2L) {
  if (log2L < 4) return 1;
  return (log2L >> 2) + ((log2L & 3) ? 1 : 0);
}
// Offset (in complex entries) of pass `pass`'s table.
CFD_HD int fft_pass_table_offset(int log2L, int pass) {
  int off = 0, ns = 1;
  for (int q = 0; q < pass; ++q) {
    const int R = fft_pass_radix(log2L, q);
    if (ns > 1) off += (R - 1) * ns;
    ns *= R;
  }
  return off;
}
CFD_HD int fft_pass_table_size(int log2L) {
  return fft_pass_table_offset(log2L, fft_num_passes(log2L));
}

// Multiplies v[r] by w^(r k) (conjugated for the inverse), r = 1..R-1.  The
// powers r = 1, 2, 3 and 4, 8, 12 come straight from the pass table (each
// rounded once from double); the others are one product of two table values,
// r = 4b + a -> w^(4b k) * w^(a k), so no twiddle is more than one complex
// rounding away from the correctly rounded value.
// LDG: the table is in global memory (read through the read-only path);
// otherwise it is read with plain loads (a copy in shared memory).
template <int R, int SIGN, bool LDG = true>
CFD_D float2 load_tw(const float2* __restrict__ twp, int Ns, int r, int k) {
  float2 w = LDG ? __ldg(twp + (r - 1) * Ns + k) : twp[(r - 1) * Ns + k];
  if (SIGN > 0) w.y = -w.y;
  return w;
}

template <int R, int SIGN, bool LDG = true>
CFD_D void apply_twiddles(float2* v, const float2* __restrict__ twp, int Ns,
                          int k) {
  const float2 w1 = load_tw<R, SIGN, LDG>(twp, Ns, 1, k);
  if (R == 2) {
    v[1] = c_mul(v[1], w1);
    return;
  }
  const float2 w2 = load_tw<R, SIGN, LDG>(twp, Ns, 2, k);
  const float2 w3 = load_tw<R, SIGN, LDG>(twp, Ns, 3, k);
  v[1] = c_mul(v[1], w1);
  v[2] = c_mul(v[2], w2);
  v[3] = c_mul(v[3], w3);
  if (R == 4) return;
  float2 wb[4];
  wb[0] = make_float2(1.f, 0.f);
  wb[1] = load_tw<R, SIGN, LDG>(twp, Ns, 4, k);
  if (R == 16) {
    wb[2] = load_tw<R, SIGN, LDG>(twp, Ns, 8, k);
    wb[3] = load_tw<R, SIGN, LDG>(twp, Ns, 12, k);
  }
  const float2 wa[4] = {make_float2(1.f, 0.f), w1, w2, w3};
#pragma unroll
  for (int b = 1; b < R / 4; ++b) {
    v[4 * b] = c_mul(v[4 * b], wb[b]);
#pragma unroll
    for (int a = 1; a < 4; ++a) v[4 * b + a] = c_mul(v[4 * b + a], c_mul(wa[a], wb[b]));
  }
}

// One in-place Stockham pass.  `t` is the worker index in [0, nthr); threads of
// the block with t >= nthr only take part in the barriers.  `twp` is this
// pass's twiddle table (unused when Ns == 1).
template <int R, int NB, int SIGN>
CFD_D void stockham_pass(float2* buf, int log2L, int log2Ns, int bstride,
                         const float2* __restrict__ twp, int t, int nthr) {
  constexpr int lr = Log2c<R>::v;
  const int log2LR = log2L - lr;
  const int LR = 1 << log2LR;
  const int Ns = 1 << log2Ns;
  float2 v[NB][R];
  int kk[NB], out[NB], bb[NB];
  const bool active = t < nthr;
  if (active) {
#pragma unroll
    for (int q = 0; q < NB; ++q) {
      const int it = t + q * nthr;
      const int b = it >> log2LR;
      const int j = it & (LR - 1);
      const float2* s = buf + b * bstride;
#pragma unroll
      for (int r = 0; r < R; ++r) v[q][r] = s[pidx(j + (r << log2LR))];
      const int k = j & (Ns - 1);
      kk[q] = k;
      bb[q] = b * bstride;
      out[q] = ((j - k) << lr) + k;
    }
  }
  __syncthreads();
  if (active) {
#pragma unroll
    for (int q = 0; q < NB; ++q) {
      if (Ns > 1) apply_twiddles<R, SIGN>(v[q], twp, Ns, kk[q]);
      Dft<R, SIGN>::run(v[q]);
      float2* d = buf + bb[q];
#pragma unroll
      for (int r = 0; r < R; ++r) d[pidx(out[q] + (r << log2Ns))] = v[q][r];
    }
  }
  __syncthreads();
}

// Number of worker threads fft_inplace needs for `batch` sequences of 2^log2L.
CFD_HD int fft_workers(int log2L, int batch) {
  const int P = log2L >= 4 ? 16 : (1 << log2L);
  return (batch << log2L) / P;
}

// In-place batched FFT of `batch` sequences (sequence b at buf + b*bstride,
// element n at pidx(n)); must be called by every thread of the block (it
// contains barriers).  t = worker index (usually threadIdx.x); `twp` is the
// concatenated pass twiddle table for this length.  Radix-16 passes first,
// then one pass of the remaining radix; sequences shorter than 16 take a
// single pass.  (Keeping the pass sequence in this shape, with the radix-16
// loop not unrolled, holds register use near that of a single pass.)
template <int SIGN>
CFD_D void fft_inplace(float2* buf, int log2L, int batch, int bstride,
                       const float2* __restrict__ twp, int t) {
  const int nthr = fft_workers(log2L, batch);
  if (log2L < 4) {
    if (log2L == 3)
      stockham_pass<8, 1, SIGN>(buf, log2L, 0, bstride, twp, t, nthr);
    else if (log2L == 2)
      stockham_pass<4, 1, SIGN>(buf, log2L, 0, bstride, twp, t, nthr);
    else if (log2L == 1)
      stockham_pass<2, 1, SIGN>(buf, log2L, 0, bstride, twp, t, nthr);
    return;
  }
  const int n16 = log2L >> 2, rem = log2L & 3;
  const float2* tp = twp;
#pragma unroll 1
  for (int q = 0; q < n16; ++q) {
    stockham_pass<16, 1, SIGN>(buf, log2L, 4 * q, bstride, tp, t, nthr);
    if (q > 0) tp += 15 << (4 * q);
  }
  const int ns = 4 * n16;
  if (rem == 3)
    stockham_pass<8, 2, SIGN>(buf, log2L, ns, bstride, tp, t, nthr);
  else if (rem == 2)
    stockham_pass<4, 4, SIGN>(buf, log2L, ns, bstride, tp, t, nthr);
  else if (rem == 1)
    stockham_pass<2, 8, SIGN>(buf, log2L, ns, bstride, tp, t, nthr);
}

// --- Real <-> half-complex helpers (length M = 2L real, via an L-point FFT) ---
//
// Forward: z[n] = x[2n] + i x[2n+1], Z = FFT_L(z).  For 0 < k < L,
//   E = (Z[k] + conj Z[L-k]) / 2,  T = -i w^k (Z[k] - conj Z[L-k]) / 2,
//   X[k] = E + T,  X[L-k] = conj(E - T),   w = exp(-2 pi i / M);
// X[0] = Re Z0 + Im Z0 and X[L] = Re Z0 - Im Z0 are real.
CFD_D void rfft_post_pair(float2 zk, float2 zm, float2 w, float2* xk,
                          float2* xm) {
  const float2 b = c_conj(zm);
  const float2 e = c_scale(c_add(zk, b), 0.5f);
  const float2 o = c_scale(c_sub(zk, b), 0.5f);
  const float2 t = c_mul_i<-1>(c_mul(w, o));
  *xk = c_add(e, t);
  *xm = c_conj(c_sub(e, t));
}

// Inverse: from X[0..L] (Hermitian half spectrum) build Z with
//   E = X[k] + conj X[L-k],  T = i conj(w^k) (X[k] - conj X[L-k]),
//   Z[k] = E + T,  Z[L-k] = conj(E - T);  Z[0] = (X0 + XL) + i (X0 - XL)
// (real parts of X0, XL only, as irfft does).  Then IFFT_L(Z)[n] =
// M * (x[2n] + i x[2n+1]) -- the 1/M (and any other) scale is applied by the
// caller.
CFD_D void irfft_pre_pair(float2 xk, float2 xm, float2 w, float2* zk,
                          float2* zm) {
  const float2 b = c_conj(xm);
  const float2 e = c_add(xk, b);
  const float2 o = c_sub(xk, b);
  const float2 t = c_mul_i<1>(c_mul(c_conj(w), o));
  *zk = c_add(e, t);
  *zm = c_conj(c_sub(e, t));
}

}  // namespace cfd
