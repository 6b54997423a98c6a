// Per-slot health of batched trajectories, recorded at the end of every chunk.
//
// The reference's own failure checks are NaN checks on the state
// (spectral/equations_test.py:137,166,233).  A batch of trajectories needs the
// same check per slot without a host round trip per step: after each chunk's
// last kernel, a reset kernel and a grid-stride reduction write, for every
// slot that ran in the chunk, whether its state holds a non-finite value and
// the largest magnitude among its finite values (cfd_health).  Slots that did
// not run keep their previous record.  Both kernels are captured in the
// chunk's CUDA graph.
#include "kernels.h"

namespace cfd {
namespace {

constexpr int kHealthThreads = 256;
// Blocks over all slots of one launch: enough loads in flight to cover the
// memory latency (with 64 blocks per slot a 1024^2 batch of four slots took
// 12 us at 35 % of DRAM bandwidth, stalled on long scoreboard).
constexpr int kHealthBlocksTotal = 152 * 8;

__global__ void health_reset_fvm_kernel(const FvmMember* __restrict__ mem, int count,
                                        Health* __restrict__ h) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < count && mem[s].steps > 0) h[s] = Health{0u, 0.f};
}

__global__ void health_reset_spec_kernel(const SpecMember* __restrict__ mem, int count,
                                         Health* __restrict__ h) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < count && mem[s].steps > 0) h[s] = Health{0u, 0.f};
}

// Accumulates n4 float4 groups of `a` into (bad, mx).
__device__ __forceinline__ void health_scan(const float4* __restrict__ a, size_t n4,
                                            unsigned& bad, float& mx) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4;
       i += (size_t)gridDim.x * blockDim.x) {
    const float4 x = __ldg(a + i);
    const float e[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (isfinite(e[k])) mx = fmaxf(mx, fabsf(e[k]));
      else bad = 1u;
    }
  }
}

// Block-wide OR of bad and max of mx, then one atomic pair per block.  Finite
// magnitudes are non-negative, so their bit patterns order like the values.
__device__ __forceinline__ void health_commit(unsigned bad, float mx, Health* h) {
  __shared__ unsigned sbad[kHealthThreads / 32];
  __shared__ float smx[kHealthThreads / 32];
  for (int d = 16; d > 0; d >>= 1) {
    bad |= __shfl_xor_sync(0xffffffffu, bad, d);
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, d));
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    sbad[warp] = bad;
    smx[warp] = mx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < kHealthThreads / 32; ++w) {
      bad |= sbad[w];
      mx = fmaxf(mx, smx[w]);
    }
    if (bad) atomicOr(&h->flags, kHealthNonFinite);
    atomicMax(reinterpret_cast<unsigned int*>(&h->max_abs), __float_as_uint(mx));
  }
}

// FVM slot state (u, v) after a chunk: m.f[0] (project_out's destination).
__global__ void __launch_bounds__(kHealthThreads)
    health_fvm_kernel(const FvmMember* __restrict__ mem, Health* __restrict__ h) {
  const FvmMember& m = mem[blockIdx.y];
  if (m.steps <= 0) return;
  const size_t n4 = ((size_t)m.p.nx * m.p.ny) >> 2;
  unsigned bad = 0u;
  float mx = 0.f;
  health_scan(reinterpret_cast<const float4*>(m.f[0][0]), n4, bad, mx);
  health_scan(reinterpret_cast<const float4*>(m.f[0][1]), n4, bad, mx);
  health_commit(bad, mx, h + blockIdx.y);
}

// Spectral slot state: the vorticity spectrum, nx x (ny/2 + 1) complex values
// (an even number of floats per row times nx rows: a whole number of float4
// groups for nx >= 2; the slot's buffers are 16-byte aligned).
__global__ void __launch_bounds__(kHealthThreads)
    health_spec_kernel(const SpecMember* __restrict__ mem, Health* __restrict__ h) {
  const SpecMember& m = mem[blockIdx.y];
  if (m.steps <= 0) return;
  const size_t floats = (size_t)m.p.nx * (m.p.ny / 2 + 1) * 2;
  unsigned bad = 0u;
  float mx = 0.f;
  health_scan(reinterpret_cast<const float4*>(m.w), floats >> 2, bad, mx);
  if ((floats & 3) && blockIdx.x == 0 && threadIdx.x == 0) {
    const float* tail = reinterpret_cast<const float*>(m.w) + (floats & ~(size_t)3);
    for (size_t k = 0; k < (floats & 3); ++k) {
      if (isfinite(tail[k])) mx = fmaxf(mx, fabsf(tail[k]));
      else bad = 1u;
    }
  }
  health_commit(bad, mx, h + blockIdx.y);
}

// Copies the records of the slots that ran to `mirror` (pinned host memory
// the device can address): the host reads them after the chunk without a
// device-to-host copy, which would queue on the copy engine behind other
// streams' transfers.
template <typename M>
__global__ void health_publish_kernel(const M* __restrict__ mem, int count,
                                      const Health* __restrict__ h, Health* mirror) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < count && mem[s].steps > 0) mirror[s] = h[s];
}

int health_blocks(size_t n4, int count) {
  size_t b = (n4 + kHealthThreads - 1) / kHealthThreads;
  const size_t cap = (size_t)(kHealthBlocksTotal / (count > 0 ? count : 1));
  if (b > cap) b = cap;
  return b < 1 ? 1 : (int)b;
}

}  // namespace

cudaError_t launch_fvm_batch_health(const FvmParams& shape, const FvmMember* mem, int count,
                                    Health* h, Health* mirror, cudaStream_t s) {
  health_reset_fvm_kernel<<<(count + 127) / 128, 128, 0, s>>>(mem, count, h);
  const size_t n4 = ((size_t)shape.nx * shape.ny) >> 2;
  health_fvm_kernel<<<dim3(health_blocks(n4, count), count), kHealthThreads, 0, s>>>(mem, h);
  if (mirror) health_publish_kernel<<<(count + 127) / 128, 128, 0, s>>>(mem, count, h, mirror);
  return cudaGetLastError();
}

cudaError_t launch_spec_batch_health(const SpecParams& shape, const SpecMember* mem, int count,
                                     Health* h, Health* mirror, cudaStream_t s) {
  health_reset_spec_kernel<<<(count + 127) / 128, 128, 0, s>>>(mem, count, h);
  const size_t n4 = ((size_t)shape.nx * (shape.ny / 2 + 1) * 2) >> 2;
  health_spec_kernel<<<dim3(health_blocks(n4, count), count), kHealthThreads, 0, s>>>(mem, h);
  if (mirror) health_publish_kernel<<<(count + 127) / 128, 128, 0, s>>>(mem, count, h, mirror);
  return cudaGetLastError();
}

}  // namespace cfd
