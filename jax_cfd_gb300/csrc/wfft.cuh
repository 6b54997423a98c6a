// One-warp FFTs of 1024 points held in registers (four-step: 32 x 32).
//
// Lane n1 holds x[n1 + 32 n2] in v[n2] (so a warp-wide access of register n2
// touches 32 consecutive elements: coalesced loads and stores).  Step 1 is a
// 32-point DFT over n2 in each lane's registers, step 2 multiplies by
// w_1024^(n1 k2) (a 32 x 32 table, read with lanes on consecutive entries),
// step 3 transposes through a 33-float2-stride shared-memory tile (one
// store and one load per element, conflict-free per half warp), step 4 is a
// 32-point DFT over n1.  On return lane k2 holds X[k2 + 32 k1] in
// v[wfft_slot(k1)].  Compared with the shared-memory Stockham passes of
// fft.cuh this keeps the data in registers between one global load and one
// global store, with a single shared-memory exchange.
#pragma once

#include "common.cuh"
#include "fft.cuh"

namespace cfd {

constexpr int kWarpFftLog2 = 10;            // the length this file implements
constexpr int kWarpFftTile = 32 * 33;       // float2 slots of one warp's transpose tile

// cos and sin of 2 pi j / 32 for j in [0, 16), rounded once from the exact
// values (folded into immediates after unrolling).
CFD_D float w32_cos(int j) {
  switch (j) {
    case 0: return 1.0f;
    case 1: return 0.98078525f;
    case 2: return 0.9238795f;
    case 3: return 0.8314696f;
    case 4: return 0.70710677f;
    case 5: return 0.55557024f;
    case 6: return 0.38268343f;
    case 7: return 0.19509032f;
    case 8: return 0.0f;
    case 9: return -0.19509032f;
    case 10: return -0.38268343f;
    case 11: return -0.55557024f;
    case 12: return -0.70710677f;
    case 13: return -0.8314696f;
    case 14: return -0.9238795f;
    default: return -0.98078525f;
  }
}

// sin(2 pi j / 32) = cos(2 pi (8 - j) / 32), cos being even.
CFD_D float w32_sin(int j) { return w32_cos(j <= 8 ? 8 - j : j - 8); }

// d * exp(SIGN 2 pi i e / 32), e in [0, 16).
template <int SIGN>
CFD_D float2 w32_rotate(float2 d, int e) {
  if (e == 0) return d;
  if (e == 8) return c_mul_i<SIGN>(d);
  return c_mul(d, make_float2(w32_cos(e), SIGN * w32_sin(e)));
}

// Bit reversal of a 5-bit index.
CFD_HD int bitrev5(int k) {
  return ((k & 1) << 4) | ((k & 2) << 2) | (k & 4) | ((k & 8) >> 2) | ((k & 16) >> 4);
}

// In-place radix-2 decimation-in-frequency 32-point DFT with sign SIGN
// (-1 forward): natural-order input, X[k] in v[bitrev5(k)] on return.
template <int SIGN>
CFD_D void dft32(float2 (&v)[32]) {
#pragma unroll
  for (int span = 16; span >= 1; span >>= 1) {
#pragma unroll
    for (int start = 0; start < 32; start += 2 * span) {
#pragma unroll
      for (int j = 0; j < span; ++j) {
        const float2 a = v[start + j], b = v[start + j + span];
        v[start + j] = c_add(a, b);
        v[start + j + span] = w32_rotate<SIGN>(c_sub(a, b), j * (16 / span));
      }
    }
  }
}

// Register slot of X[lane + 32 k1] after warp_fft1024.
CFD_HD int wfft_slot(int k1) { return bitrev5(k1); }

// Offset (float2 entries) of the warp-FFT table in the concatenated pass
// table of a length-1024 transform: after the Stockham pass tables.
CFD_HD int wfft_table_offset(int log2L) { return fft_pass_table_size(log2L); }
// Entries the warp-FFT table adds to the pass table of length 2^log2L:
// [k2 * 32 + n1] = exp(-2 pi i n1 k2 / 1024).
CFD_HD int wfft_table_size(int log2L) { return log2L == kWarpFftLog2 ? 1024 : 0; }

// 1024-point DFT of sign SIGN by the calling warp (all 32 lanes).  v: lane
// n1's x[n1 + 32 n2] in v[n2]; on return lane k2's X[k2 + 32 k1] in
// v[wfft_slot(k1)].  tile: this warp's kWarpFftTile float2 of shared memory.
// tw: the warp-FFT table, entry [k2 * 32 + n1] = exp(-2 pi i n1 k2 / 1024).
template <int SIGN>
CFD_D void warp_fft1024(float2 (&v)[32], float2* __restrict__ tile,
                        const float2* __restrict__ tw) {
  const int lane = threadIdx.x & 31;
  dft32<SIGN>(v);
  // Y[n1][k2] is in v[bitrev5(k2)]; rotate and store transposed.
#pragma unroll
  for (int k2 = 0; k2 < 32; ++k2) {
    float2 y = v[bitrev5(k2)];
    if (k2 != 0) {
      const float2 w = __ldg(tw + k2 * 32 + lane);
      y = c_mul(y, SIGN < 0 ? w : c_conj(w));
    }
    tile[k2 * 33 + lane] = y;
  }
  __syncwarp();
#pragma unroll
  for (int n1 = 0; n1 < 32; ++n1) v[n1] = tile[lane * 33 + n1];
  // The tile is reused by the caller's next transform.
  __syncwarp();
  dft32<SIGN>(v);
}

CFD_D float2 wfft_shfl_idx2(float2 x, int src) {
  return make_float2(__shfl_sync(0xffffffffu, x.x, src), __shfl_sync(0xffffffffu, x.y, src));
}

// Z[L - k] for k = lane + 32 k1 (L = 1024), from warp_fft1024's output
// registers: for lane l >= 1 the partner lives in lane 32 - l, register
// 31 - k1; for lane 0 in lane 0, register 32 - k1.
CFD_D float2 wfft_mirror(const float2 (&v)[32], int k1, int lane) {
  float2 zp = wfft_shfl_idx2(v[wfft_slot(31 - k1)], (32 - lane) & 31);
  if (lane == 0) zp = v[wfft_slot((32 - k1) & 31)];
  return zp;
}

}  // namespace cfd
