#pragma once

#include <atomic>

#include "common.cuh"
#include "fft.cuh"

namespace cfd {

// Persistent column passes with register-resident Stockham passes, shared by
// the FVM pressure solve and the spectral stage kernels.
//
// A block owns CG adjacent columns at a time (a group), walks its work items
// with the grid as its stride, and copies the next item's input into shared
// memory (cp.async, each thread its own points) while it transforms the
// current one, so the global traffic of one item overlaps the arithmetic of
// the other.  Worker t of a column holds the 16 points x[t + (N/16) r] that
// the first Stockham pass of fft_inplace gives it; every pass runs the same
// butterflies on the same twiddles as fft_inplace (so results are bit for bit
// those of the shared-memory engine), with shared memory used only to
// exchange data between passes: two buffers written alternately, one barrier
// per exchange.  The last pass leaves X[t + (N/16) m] in the worker's
// registers, which are exactly the first inverse pass's inputs, so a scaling
// between a forward and an inverse transform needs no exchange at all.
template <int LOG2N>
struct ColPipe {
  static constexpr int N = 1 << LOG2N;
  static constexpr int NTHR = N / 16;     // workers per column
  static constexpr int N16 = LOG2N >> 2;  // radix-16 passes
  static constexpr int REM = LOG2N & 3;   // radix 2^REM of the last pass (0: none)
  static constexpr int PASSES = N16 + (REM ? 1 : 0);
};

// Float2 slots per column buffer: the padded sequence plus 16/CG slots, so
// the CG columns a half warp touches start in different banks.
template <int LOG2N, int CG>
CFD_HD int col_pipe_bstride() {
  return padded_len(1 << LOG2N) + 16 / CG;
}

// Up to 2048 rows the block also keeps the pass twiddle table and one
// length-N float table (eigenvalues or wavenumbers) in shared memory: with
// the exchange buffers and staging slots taking most of the 227 KB, the L1
// left over cannot hold them next to the staged traffic.
template <int LOG2N>
constexpr bool col_pipe_smem_tables() { return LOG2N <= 11; }

// Two exchange buffers per column, then 16 staging slots per thread, then
// (col_pipe_smem_tables) the twiddle table and the float table.
template <int LOG2N, int CG>
CFD_HD size_t col_pipe_smem() {
  size_t b = ((size_t)2 * CG * col_pipe_bstride<LOG2N, CG>() + (size_t)CG * (1 << LOG2N)) *
             sizeof(float2);
  if (col_pipe_smem_tables<LOG2N>())
    b += (size_t)fft_pass_table_size(LOG2N) * sizeof(float2) + (size_t)(1 << LOG2N) * sizeof(float);
  return b;
}

// The tables' place in shared memory, after the staging slots.
template <int LOG2N, int CG>
CFD_D float2* col_pipe_tw_smem(float2* sbuf) {
  return sbuf + 2 * CG * col_pipe_bstride<LOG2N, CG>() + CG * (1 << LOG2N);
}
template <int LOG2N, int CG>
CFD_D float* col_pipe_tab_smem(float2* sbuf) {
  return reinterpret_cast<float*>(col_pipe_tw_smem<LOG2N, CG>(sbuf) +
                                  fft_pass_table_size(LOG2N));
}

// Copies the twiddle table and the float table `tab` (N entries) into shared
// memory when col_pipe_smem_tables; returns the pointers the block reads
// them through (shared copies or the global tables).  Ends with a barrier.
template <int LOG2N, int CG>
CFD_D void col_pipe_tables(float2* sbuf, const float2* __restrict__ twp,
                           const float* __restrict__ tab, const float2** tw_out,
                           const float** tab_out) {
  if (col_pipe_smem_tables<LOG2N>()) {
    float2* tw = col_pipe_tw_smem<LOG2N, CG>(sbuf);
    float* tb = col_pipe_tab_smem<LOG2N, CG>(sbuf);
    const int ntw = fft_pass_table_size(LOG2N);
    for (int i = threadIdx.x; i < ntw; i += blockDim.x) tw[i] = __ldg(twp + i);
    for (int i = threadIdx.x; i < (1 << LOG2N); i += blockDim.x) tb[i] = __ldg(tab + i);
    *tw_out = tw;
    *tab_out = tb;
  } else {
    *tw_out = twp;
    *tab_out = tab;
  }
  __syncthreads();
}

// The barrier of a transform's exchanges: the whole block (BARN == 0), or the
// BARN threads (whole warps) that own one column, on named barrier bar_id.
template <int BARN>
CFD_D void col_pipe_sync(int bar_id) {
  if constexpr (BARN == 0) {
    __syncthreads();
  } else {
    static_assert(BARN % 32 == 0, "a named barrier counts whole warps");
    asm volatile("bar.sync %0, %1;\n" ::"r"(bar_id), "n"(BARN) : "memory");
  }
}

// One transform of sign SIGN of the calling worker's column; twp is the pass
// table as col_pipe_tables returned it.  v: the pass-0
// inputs x[t + NTHR r] on entry, X[t + NTHR m] in v[m] on return.  buf[0],
// buf[1]: this column's two exchange buffers; the k-th exchange of the
// transform writes buf[(FIRST + k) & 1].  Called by every thread of the block
// (it contains barriers).
// LDG: twp is the global table (else a shared copy).  A thread with
// active == false computes nothing but takes part in every barrier.
// BARN != 0: the exchanges synchronise only the BARN threads of this column
// (named barrier bar_id), for columns whose buffers no other thread touches.
// SINGLE: buf[0] and buf[1] are one buffer, so each exchange after the first
// also waits for every read of the previous one before it writes (half the
// shared memory, one more barrier per exchange).
template <int LOG2N, int SIGN, int FIRST, bool LDG = !col_pipe_smem_tables<LOG2N>(),
          int BARN = 0, bool SINGLE = false>
CFD_D void col_pipe_fft(float2 (&v)[16], float2* const (&buf)[2], int t,
                        const float2* __restrict__ twp, bool active = true, int bar_id = 0) {
  using P = ColPipe<LOG2N>;
  int wsel = FIRST;
  int tw_off = 0;
#pragma unroll
  for (int q = 0; q < P::N16; ++q) {
    const int Ns = 1 << (4 * q);
    const int k = t & (Ns - 1);
    if (active) {
      if (q > 0) {
        const float2* in = buf[wsel ^ 1];
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = in[pidx(t + P::NTHR * r)];
      }
      if (Ns > 1) apply_twiddles<16, SIGN, LDG>(v, twp + tw_off, Ns, k);
      Dft<16, SIGN>::run(v);
    }
    if (q > 0) tw_off += 15 << (4 * q);
    const bool last = q == P::N16 - 1 && P::REM == 0;
    if (!last) {
      if constexpr (SINGLE) {
        if (q > 0) col_pipe_sync<BARN>(bar_id);
      }
      if (active) {
        float2* out = buf[wsel];
        const int o = ((t - k) << 4) + k;
#pragma unroll
        for (int r = 0; r < 16; ++r) out[pidx(o + r * Ns)] = v[r];
      }
      wsel ^= 1;
      col_pipe_sync<BARN>(bar_id);
    }
  }
  if constexpr (P::REM > 0) {
    if (!active) return;
    constexpr int R = 1 << P::REM, NB = 16 / R;
    constexpr int Ns = P::N / R;  // = N / R: the final span
    const float2* in = buf[wsel ^ 1];
    float2 vv[NB][R];
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      const int j = t + P::NTHR * b;
#pragma unroll
      for (int r = 0; r < R; ++r) vv[b][r] = in[pidx(j + Ns * r)];
    }
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      const int j = t + P::NTHR * b;
      apply_twiddles<R, SIGN, LDG>(vv[b], twp + tw_off, Ns, j);
      Dft<R, SIGN>::run(vv[b]);
      // X[j + Ns r] = X[t + NTHR (b + NB r)]
#pragma unroll
      for (int r = 0; r < R; ++r) v[b + NB * r] = vv[b][r];
    }
  }
}

// Asynchronous 8-byte global -> shared copy (cp.async, L1-allocating).
CFD_D void cp_async8(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
CFD_D void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
CFD_D void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Multiprocessors of the current device (host side; 1 if the query fails).
static inline int col_pipe_device_sms() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1)
    return 1;
  return n;
}

// Resident blocks per multiprocessor of `kern` at this block size and shared
// memory (at least 1), queried once per call site and cached in `cache`; the
// cache is atomic because any host thread may launch.
template <typename K>
inline cudaError_t cached_blocks_per_sm(K kern, int threads, size_t smem, std::atomic<int>& cache,
                                        int* out) {
  int v = cache.load(std::memory_order_relaxed);
  if (v == 0) {
    int nb = 0;
    const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, threads, smem);
    if (e != cudaSuccess) return e;
    v = nb > 0 ? nb : 1;
    cache.store(v, std::memory_order_relaxed);
  }
  *out = v;
  return cudaSuccess;
}

// Register cap of 128 at every block size (512 threads per multiprocessor or
// more), for __launch_bounds__(T, col_pipe_min_blocks(T)).
constexpr int col_pipe_min_blocks(int threads) { return threads >= 512 ? 1 : 512 / threads; }

}  // namespace cfd
