// mg_common.cuh — status handling and owning buffers for the engine's host code.
//
// The reference reports every CUDA failure through HANDLE_ERROR, which prints and calls exit()
// (include/mppi/utils/gpu_err_chk.cuh:32-40).  The engine instead returns an mppi_status and records a message that
// mppi_last_error_string() hands back.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>

#include "../../include/mppi_gb.h"

namespace mg
{
void set_error(const char* fmt, ...);
void clear_error();

#define MG_CUDA(call)                                                                                                 \
  do                                                                                                                  \
  {                                                                                                                   \
    cudaError_t mg_e_ = (call);                                                                                       \
    if (mg_e_ != cudaSuccess)                                                                                         \
    {                                                                                                                 \
      ::mg::set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(mg_e_), __FILE__, __LINE__);                 \
      return MPPI_ECUDA;                                                                                              \
    }                                                                                                                 \
  } while (0)

#define MG_TRY(call)                                                                                                  \
  do                                                                                                                  \
  {                                                                                                                   \
    mppi_status mg_s_ = (call);                                                                                       \
    if (mg_s_ != MPPI_OK) return mg_s_;                                                                               \
  } while (0)

#define MG_CHECK(cond, ...)                                                                                           \
  do                                                                                                                  \
  {                                                                                                                   \
    if (!(cond))                                                                                                      \
    {                                                                                                                 \
      ::mg::set_error(__VA_ARGS__);                                                                                   \
      return MPPI_EINVAL;                                                                                             \
    }                                                                                                                 \
  } while (0)

// Device allocation owned by the engine.
template <class T>
struct DevBuf
{
  T* p = nullptr;
  size_t n = 0;
  bool owned = true;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { reset(); }
  void reset()
  {
    if (p && owned) cudaFree(p);
    p = nullptr;
    n = 0;
    owned = true;
  }
  // Point at count elements inside a block another buffer owns.
  void view(T* ptr, size_t count)
  {
    reset();
    p = ptr;
    n = count;
    owned = false;
  }
  mppi_status alloc(size_t count)
  {
    reset();
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void**)&p, count * sizeof(T));
    if (e != cudaSuccess)
    {
      p = nullptr;
      set_error("cudaMalloc(%zu bytes) failed: %s", count * sizeof(T), cudaGetErrorString(e));
      return e == cudaErrorMemoryAllocation ? MPPI_ENOMEM : MPPI_ECUDA;
    }
    n = count;
    return MPPI_OK;
  }
};

// Page-locked host staging owned by the engine (H2D / D2H copies inside captured graphs read and write these).
template <class T>
struct PinnedBuf
{
  T* p = nullptr;
  size_t n = 0;
  bool owned = true;
  PinnedBuf() = default;
  PinnedBuf(const PinnedBuf&) = delete;
  PinnedBuf& operator=(const PinnedBuf&) = delete;
  ~PinnedBuf() { reset(); }
  void reset()
  {
    if (p && owned) cudaFreeHost(p);
    p = nullptr;
    n = 0;
    owned = true;
  }
  // Point at count elements inside a block another buffer owns.
  void view(T* ptr, size_t count)
  {
    reset();
    p = ptr;
    n = count;
    owned = false;
  }
  mppi_status alloc(size_t count)
  {
    reset();
    if (count == 0) count = 1;
    cudaError_t e = cudaMallocHost((void**)&p, count * sizeof(T));
    if (e != cudaSuccess)
    {
      p = nullptr;
      set_error("cudaMallocHost(%zu bytes) failed: %s", count * sizeof(T), cudaGetErrorString(e));
      return MPPI_ENOMEM;
    }
    memset(p, 0, count * sizeof(T));
    n = count;
    return MPPI_OK;
  }
};

// CTAs of `kern` that can be resident on one SM with `threads` threads and `dyn_smem` bytes of dynamic shared memory.
// The kernel's shared-memory carveout preference is set to the maximum first, so the L1 / shared split leaves room
// for that many; the count is the smaller of the register, shared-memory, thread and CTA-slot limits (the larger of
// that and the runtime's occupancy answer).
// Raises a kernel's dynamic shared-memory cap to at least `bytes`, never lowering it: the cap belongs to the function
// and is shared by every engine of the process, so an engine with a smaller need must not undercut a larger one's.
template <class Kernel>
inline cudaError_t raise_smem_cap(Kernel kern, size_t bytes)
{
  if (bytes <= 48 * 1024) return cudaSuccess;
  static std::mutex mu;
  static std::map<const void*, size_t> caps;
  std::lock_guard<std::mutex> lock(mu);
  size_t& cur = caps[reinterpret_cast<const void*>(kern)];
  if (bytes <= cur) return cudaSuccess;
  const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) cur = bytes;
  return e;
}

template <class Kernel>
inline cudaError_t resident_ctas_per_sm(Kernel kern, int threads, size_t dyn_smem, int* out)
{
  *out = 1;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                       (int)cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return e;
  cudaFuncAttributes fa;
  if ((e = cudaFuncGetAttributes(&fa, kern)) != cudaSuccess) return e;
  int dev = 0, smem_sm = 0, resv = 0, regs_sm = 0, thr_sm = 0, blk_sm = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&resv, cudaDevAttrReservedSharedMemoryPerBlock, dev);
  cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&thr_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev);
  cudaDeviceGetAttribute(&blk_sm, cudaDevAttrMaxBlocksPerMultiprocessor, dev);
  const int warps = (threads + 31) / 32;
  const int regs_warp = ((fa.numRegs * 32 + 255) / 256) * 256;  // allocation granule: 256 registers per warp
  int n = blk_sm > 0 ? blk_sm : 32;
  if (regs_warp > 0) n = std::min(n, regs_sm / (regs_warp * warps));
  n = std::min(n, thr_sm / (warps * 32));
  const size_t smem_blk = fa.sharedSizeBytes + dyn_smem + (size_t)resv;
  if (smem_blk > 0) n = std::min(n, (int)((size_t)smem_sm / smem_blk));
  int api = 0;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&api, kern, threads, dyn_smem)) != cudaSuccess) return e;
  *out = std::max(1, std::max(n, api));
  return cudaSuccess;
}

}  // namespace mg
