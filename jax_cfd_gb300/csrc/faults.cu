// Device fault words and the bounded-wait self-test.
//
// Kernels never trap or spin without bound: a wait on an asynchronous copy
// that runs out records a code in its translation unit's fault word
// (bulk.cuh) and the block leaves.  This file keeps the list of every unit's
// word, reads them for cfd_device_fault(), and provides a self-test whose
// kernel waits on an mbarrier that nothing ever arrives on, so that the
// give-up path can be exercised without a fault, a hang or a copy in flight.
#include <mutex>
#include <string>
#include <vector>

#include "../../include/cfd_gb300.h"
#include "bulk.cuh"
#include "kernels.h"

namespace cfd {

namespace {
std::mutex& fault_mu() {
  static std::mutex mu;
  return mu;
}
std::vector<FaultWordReader>& fault_readers() {
  static std::vector<FaultWordReader> readers;
  return readers;
}
}  // namespace

bool register_fault_word(FaultWordReader reader) {
  std::lock_guard<std::mutex> lock(fault_mu());
  fault_readers().push_back(reader);
  return true;
}

// The first non-zero word in registration order (0 if none); with clear,
// every word is reset.
cudaError_t read_device_fault(unsigned int* code, bool clear) {
  std::vector<FaultWordReader> readers;
  {
    std::lock_guard<std::mutex> lock(fault_mu());
    readers = fault_readers();
  }
  *code = 0;
  for (FaultWordReader r : readers) {
    unsigned int c = 0;
    cudaError_t e = r(&c, clear);
    if (e != cudaSuccess) return e;
    if (*code == 0) *code = c;
  }
  return cudaSuccess;
}

namespace {

// One warp; thread 0 initialises an mbarrier that expects one arrival and no
// transaction bytes, issues no copy and never arrives, then waits for phase 0
// with the given poll limit.  The phase cannot complete, so the wait gives up,
// records kFaultBulkWait in this unit's fault word, and the kernel returns.
__global__ void bounded_wait_probe_kernel(int polls) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) mbar_init(&bar, 1);
  __syncthreads();
  if (threadIdx.x == 0) mbar_wait(&bar, 0, polls);
}

}  // namespace
}  // namespace cfd

extern "C" int cfd_bounded_wait_selftest(void* stream, int polls) {
  if (polls < 1 || polls > cfd::kBulkWaitLimit) {
    cfd::set_last_error("cfd_bounded_wait_selftest: polls must be in [1, 2^22]");
    return CFD_ERR_INVALID_ARGUMENT;
  }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  cfd::bounded_wait_probe_kernel<<<1, 32, 0, s>>>(polls);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  unsigned int code = 0;
  if (e == cudaSuccess) e = cfd::read_device_fault(&code, false);
  if (e != cudaSuccess) {
    cfd::set_last_error(std::string("cfd_bounded_wait_selftest: ") + cudaGetErrorString(e));
    return CFD_ERR_CUDA;
  }
  if (code != 0) {
    cfd::set_last_error("cfd_bounded_wait_selftest: a bounded wait ran out (device fault word " +
                        std::to_string(code) + ")");
    return CFD_ERR_DEVICE_FAULT;
  }
  return CFD_OK;
}
