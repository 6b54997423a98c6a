// Bulk asynchronous copies (the TMA's untiled cp.async.bulk) into shared
// memory with mbarrier completion, and bounded waits.
//
// Every wait on an mbarrier gives up after a bounded number of polls
// (kBulkWaitLimit unless the caller passes a smaller limit) or kBulkWaitNs of
// wall-clock time, whichever comes first: the kernel then records the failure
// in its unit's fault word (read by cfd_device_fault()), waits once more,
// with the same limits, for the copies it issued, and leaves without using
// the data.  Nothing spins without bound, and a copy that can never complete
// costs a launch tens of milliseconds, not seconds.
#pragma once

#include <stdint.h>

#include "common.cuh"

namespace cfd {

// Non-zero after a bounded wait ran out (the code of the first failure).
// Without relocatable device code every translation unit that includes this
// header has its own word; each unit registers a reader of its word when the
// library loads, and read_device_fault() (kernels.h) consults all of them.
static __device__ unsigned int g_cfd_device_fault = 0;
constexpr unsigned int kFaultBulkWait = 1;
constexpr int kBulkWaitLimit = 1 << 22;
constexpr unsigned long long kBulkWaitNs = 20000000ull;  // 20 ms

// Reads (and optionally clears) one translation unit's fault word.
using FaultWordReader = cudaError_t (*)(unsigned int* code, bool clear);
// Adds a reader to the library's list (faults.cu); returns true.
bool register_fault_word(FaultWordReader reader);

namespace {
cudaError_t unit_device_fault(unsigned int* code, bool clear) {
  cudaError_t e = cudaMemcpyFromSymbol(code, g_cfd_device_fault, sizeof(unsigned int));
  if (e == cudaSuccess && clear) {
    const unsigned int zero = 0;
    e = cudaMemcpyToSymbol(g_cfd_device_fault, &zero, sizeof(unsigned int));
  }
  return e;
}
const bool g_unit_fault_registered = register_fault_word(&unit_device_fault);
}  // namespace

CFD_D uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

CFD_D void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

// Makes the initialised barrier visible to the async (TMA) proxy.
CFD_D void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// One arrival that also announces `bytes` of expected transactions.
CFD_D void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

// Global -> shared bulk copy; `bytes` and both addresses are multiples of 16.
CFD_D void bulk_load(void* dst_smem, const void* src_global, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_addr(dst_smem)),
      "l"(src_global), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// Tiled 2-D TMA load of one box of the tensor map `tmap` (the generic
// address of a __grid_constant__ CUtensorMap) at element coordinates (x, y)
// into shared memory; x times the element size must be a multiple of 16 B.
CFD_D void tma_load_2d(void* dst_smem, const void* tmap, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%2, %3}], [%4];" ::"r"(smem_addr(dst_smem)),
      "l"(tmap), "r"(x), "r"(y), "r"(smem_addr(bar))
      : "memory");
}

// The same for a 3-D tensor map at element coordinates (x, y, z).
CFD_D void tma_load_3d(void* dst_smem, const void* tmap, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(dst_smem)),
      "l"(tmap), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}

// Tiled 2-D TMA store of one box from shared memory (16-byte aligned) to the
// tensor map's global memory at element coordinates (x, y): x times the
// element size a multiple of 16 B, both coordinates non-negative.  Joins the
// calling thread's current bulk group.
CFD_D void tma_store_2d(const void* tmap, int x, int y, const void* src_smem) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::
                   "l"(tmap), "r"(x), "r"(y), "r"(smem_addr(src_smem))
               : "memory");
}

// Closes the calling thread's current bulk group.
CFD_D void bulk_commit_group() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

// Waits until every committed bulk group of the calling thread has read its
// shared-memory source (the buffer may then be rewritten).
CFD_D void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }

// Waits until every committed bulk group of the calling thread has completed.
CFD_D void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// Orders this thread's earlier generic-proxy accesses to shared memory before
// its later async-proxy (TMA) accesses.
CFD_D void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

CFD_D bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

CFD_D unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Polls phase `parity` until it completes (true) or `limit` polls or
// kBulkWaitNs have passed (false).
CFD_D bool mbar_poll(uint64_t* bar, uint32_t parity, int limit) {
  const unsigned long long t0 = global_ns();
  for (int k = 0; k < limit; ++k) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((k & 255) == 255 && global_ns() - t0 > kBulkWaitNs) return false;
  }
  return false;
}

// Bounded wait for phase `parity`; false if it gave up (recorded).
CFD_D bool mbar_wait(uint64_t* bar, uint32_t parity, int limit = kBulkWaitLimit) {
  if (mbar_poll(bar, parity, limit)) return true;
  atomicCAS(&g_cfd_device_fault, 0u, kFaultBulkWait);
  // Give the copies in flight one more bounded chance to land before the
  // block leaves (their destination is this block's shared memory).
  mbar_poll(bar, parity, limit);
  return false;
}

}  // namespace cfd
