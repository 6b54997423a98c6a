// Shared helpers for the jax-cfd GB300 kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define CFD_HD __host__ __device__ __forceinline__
#define CFD_D __device__ __forceinline__

// Complex numbers are interleaved float2 (the complex64 layout of the
// reference's rfftn output).
CFD_D float2 c_add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
CFD_D float2 c_sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
CFD_D float2 c_conj(float2 a) { return make_float2(a.x, -a.y); }
CFD_D float2 c_scale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// The library is compiled with -fmad=false, so every multiply-add that should
// fuse is written as an explicit fma: the rounding of each expression is then
// fixed by the source, not by the inlining context it is compiled in (the
// batched and single-trajectory kernels share their bodies and must agree bit
// for bit).
CFD_D float2 c_mul(float2 a, float2 b) {
  return make_float2(__fmaf_rn(a.x, b.x, -(a.y * b.y)), __fmaf_rn(a.x, b.y, a.y * b.x));
}
// Multiply by SIGN * i (SIGN = -1 gives -i, the forward-transform rotation).
template <int SIGN>
CFD_D float2 c_mul_i(float2 a) {
  return SIGN < 0 ? make_float2(a.y, -a.x) : make_float2(-a.y, a.x);
}

CFD_HD int ilog2(int x) {
  int r = 0;
  while ((1 << r) < x) ++r;
  return r;
}

CFD_HD bool is_pow2(int x) { return x > 0 && (x & (x - 1)) == 0; }

// Programmatic dependent launch (sm_90+).  A kernel launched with
// cudaLaunchAttributeProgrammaticStreamSerialization may start while the
// previous kernel in the stream is still running; pdl_wait() blocks until
// that kernel has completed and its writes are visible, so it must precede
// every read of the previous kernel's output.  pdl_trigger() lets the next
// kernel be launched once every block of this one is running.  Without the
// attribute both are no-ops.
CFD_D void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
CFD_D void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;\n" :::); }

// Launches `kern` on stream s, as a programmatic dependent of the previous
// kernel when pdl != 0.
template <typename... KArgs, typename... Args>
cudaError_t launch_maybe_pdl(bool pdl, void (*kern)(KArgs...), dim3 grid, dim3 block,
                             size_t smem, cudaStream_t s, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}
