// mg_noalloc.cu — the weighted-reduction (control update) entry point for callers that must not allocate memory.
//
// Who needs this: code that runs where cudaMalloc is off limits — a real-time control loop that has frozen its
// memory map after start-up, a host process whose GPU memory is owned by another framework's pool, or a safety-
// certified build that bans allocation after initialisation.  mppi_kernel_weighted_reduction allocates its scratch
// (chunk table, partial sums, arrival counters) on the stream for every call; this variant uses one fixed scratch
// array that lives in the library's device image instead, so a call performs no allocation or free of any kind.
//
// The array is `g_reduction_scratch` below: kNoAllocScratchBytes (4 MiB) of device memory that every GPU loading the
// library keeps until the process exits.  Host code reaches it through its device address, looked up with
// cudaGetSymbolAddress by every call made outside stream capture; a call under capture reuses the address the last
// uncaptured call on that device found (so make the first call on a device before any stream capture).  All calls
// share the array: calls that overlap on the GPU (on different streams, or from different host threads) race on it
// and must be serialised by the caller.  Each call clears the counters that must start at zero.
#include <mutex>

#include "mg_common.cuh"
#include "mg_kernels.cuh"

namespace mg
{
namespace
{
constexpr size_t kNoAllocScratchBytes = 4u << 20;
constexpr int kNoAllocMaxRollouts = 65536;
constexpr int kNoAllocMaxTC = 1024;  // num_timesteps * control_dim
constexpr int kNoAllocChunk = 128;   // samples per CTA, as the allocating entry point uses

static __device__ __align__(256) unsigned char g_reduction_scratch[kNoAllocScratchBytes];

// Layout of the scratch (byte offsets, each 256-byte aligned).
struct ScratchLayout
{
  size_t inst, chunks, part_off, chunk0, part_w, stats, counters, bn, partials, total;
};

ScratchLayout layout_for(int nch, int tc)
{
  ScratchLayout L{};
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off += (bytes + 255) / 256 * 256;
    return o;
  };
  L.inst = take(sizeof(InstDesc));
  L.chunks = take(sizeof(int4) * nch);
  L.part_off = take(sizeof(long long) * nch);
  L.chunk0 = take(sizeof(int));
  L.part_w = take(sizeof(double) * 2 * nch);
  L.stats = take(sizeof(double) * 3);
  L.counters = take(sizeof(unsigned int) * 4);
  L.bn = take(sizeof(float) * 2);
  L.partials = take(sizeof(float) * (size_t)nch * tc);
  L.total = off;
  return L;
}

// Writes the descriptor tables into the scratch and clears the arrival counters (device code names the array
// directly; host code never dereferences it).
__global__ void noalloc_setup_kernel(ScratchLayout L, int K, int T, int nch, int tc)
{
  unsigned char* base = g_reduction_scratch;
  if (blockIdx.x == 0 && threadIdx.x == 0)
  {
    InstDesc d;
    memset(&d, 0, sizeof(d));
    d.K = K;
    d.T = T;
    d.num_chunks = nch;
    *reinterpret_cast<InstDesc*>(base + L.inst) = d;
    *reinterpret_cast<int*>(base + L.chunk0) = 0;
    unsigned int* cnt = reinterpret_cast<unsigned int*>(base + L.counters);
    cnt[0] = cnt[1] = cnt[2] = cnt[3] = 0u;
  }
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nch; c += gridDim.x * blockDim.x)
  {
    reinterpret_cast<int4*>(base + L.chunks)[c] =
        make_int4(0, c * kNoAllocChunk, min(K, (c + 1) * kNoAllocChunk), c);
    reinterpret_cast<long long*>(base + L.part_off)[c] = (long long)c * tc;
  }
}

struct DeviceScratch
{
  std::mutex mu;
  void* addr[256] = {};
};
DeviceScratch g_scratch;

// The array's device address on the current device.  Outside stream capture it is looked up on every call (a host-
// side table lookup, no allocation), so a context that was torn down and created again (cudaDeviceReset) hands out
// the array's new address; during capture, where the lookup could load the module, the address recorded by the
// last call outside capture on this device is used.
mppi_status scratch_address(cudaStream_t s, void** out)
{
  int dev = 0;
  MG_CUDA(cudaGetDevice(&dev));
  MG_CHECK(dev >= 0 && dev < 256, "device ordinal %d out of range", dev);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  MG_CUDA(cudaStreamIsCapturing(s, &cap));
  std::lock_guard<std::mutex> lock(g_scratch.mu);
  if (cap == cudaStreamCaptureStatusNone)
  {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_reduction_scratch);
    if (e != cudaSuccess || !p)
    {
      set_error("cudaGetSymbolAddress(g_reduction_scratch) failed on device %d: %s", dev, cudaGetErrorString(e));
      return MPPI_ECUDA;
    }
    g_scratch.addr[dev] = p;
  }
  MG_CHECK(g_scratch.addr[dev] != nullptr,
           "the first allocation-free call on device %d must come before any stream capture", dev);
  *out = g_scratch.addr[dev];
  return MPPI_OK;
}
}  // namespace
}  // namespace mg

using namespace mg;

extern "C" {

mppi_status mppi_kernel_weighted_reduction_noalloc(const float* weights_d, const float* controls_d, float* new_u_d,
                                                   const float* baseline_norm_d, int index, int num_timesteps,
                                                   int num_rollouts, int control_dim, void* stream)
{
  clear_error();
  MG_CHECK(weights_d && controls_d && new_u_d && baseline_norm_d, "device pointers must not be NULL");
  MG_CHECK(num_rollouts >= 1 && num_timesteps >= 1, "num_rollouts and num_timesteps must be >= 1");
  MG_CHECK(control_dim >= 1 && control_dim <= MPPI_MAX_CONTROL_DIM, "control_dim must be in [1, %d]",
           MPPI_MAX_CONTROL_DIM);
  MG_CHECK(index >= 0, "index must be >= 0");
  MG_CHECK(num_rollouts <= kNoAllocMaxRollouts,
           "num_rollouts %d exceeds the allocation-free limit of %d (use mppi_kernel_weighted_reduction)",
           num_rollouts, kNoAllocMaxRollouts);
  const long long tc = (long long)num_timesteps * control_dim;
  MG_CHECK(tc <= kNoAllocMaxTC,
           "num_timesteps * control_dim = %lld exceeds the allocation-free limit of %d "
           "(use mppi_kernel_weighted_reduction)",
           tc, kNoAllocMaxTC);
  const int nch = (num_rollouts + kNoAllocChunk - 1) / kNoAllocChunk;
  const ScratchLayout L = layout_for(nch, (int)tc);
  MG_CHECK(L.total <= kNoAllocScratchBytes, "problem needs %zu scratch bytes, more than the %zu available", L.total,
           kNoAllocScratchBytes);
  cudaStream_t s = (cudaStream_t)stream;
  void* scratch = nullptr;
  MG_TRY(scratch_address(s, &scratch));
  noalloc_setup_kernel<<<(nch + 255) / 256, 256, 0, s>>>(L, num_rollouts, num_timesteps, nch, (int)tc);
  MG_CUDA(cudaGetLastError());
  char* base = (char*)scratch;
  WeightsArgs a{};
  a.inst = (const InstDesc*)(base + L.inst);
  a.chunks = (const int4*)(base + L.chunks);
  a.part_off = (const long long*)(base + L.part_off);
  a.inst_chunk0 = (const int*)(base + L.chunk0);
  a.num_chunks = nch;
  a.num_instances = 1;
  a.costs = nullptr;
  a.weights = const_cast<float*>(weights_d);
  a.samples = controls_d;
  a.partials = (float*)(base + L.partials);
  a.part_w = (double*)(base + L.part_w);
  a.baseline_bits = (unsigned int*)(base + L.counters) + 3;
  a.arrive = (unsigned int*)(base + L.counters);
  a.inst_done = (unsigned int*)(base + L.counters) + 1;
  a.noise_counter = nullptr;
  a.mean_out = new_u_d;
  a.baseline_norm = (float*)(base + L.bn);
  a.stats = (double*)(base + L.stats);
  a.lambda_inv = 1.0f;
  a.weights_given = 1;
  a.given_norm = baseline_norm_d + 2 * (size_t)index + 1;
  switch (control_dim)
  {
    case 1: weights_update_kernel<1><<<nch, 256, 0, s>>>(a); break;
    case 2: weights_update_kernel<2><<<nch, 256, 0, s>>>(a); break;
    case 3: weights_update_kernel<3><<<nch, 256, 0, s>>>(a); break;
    default: weights_update_kernel<4><<<nch, 256, 0, s>>>(a); break;
  }
  MG_CUDA(cudaGetLastError());
  return MPPI_OK;
}

}  // extern "C"
