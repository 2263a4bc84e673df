// mg_common.cuh — status handling and owning buffers for the engine's host code.
//
// The reference reports every CUDA failure through HANDLE_ERROR, which prints and calls exit()
// (include/mppi/utils/gpu_err_chk.cuh:32-40).  The engine instead returns an mppi_status and records a message that
// mppi_last_error_string() hands back.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <cstring>
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
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { reset(); }
  void reset()
  {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
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
  PinnedBuf() = default;
  PinnedBuf(const PinnedBuf&) = delete;
  PinnedBuf& operator=(const PinnedBuf&) = delete;
  ~PinnedBuf() { reset(); }
  void reset()
  {
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
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

}  // namespace mg
