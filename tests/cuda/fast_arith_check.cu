// Exactness of the rollouts' branch-free arithmetic (FastArith in mg_math.cuh) against its IEEE definition.
//
//   fast_arith_check [a_stride]
//
// 1. Division: for every significand of b in [1, 2) and every a_stride-th significand of a in [1, 2) (a_stride = 1:
//    all 2^46 pairs), FastArith::div(a, b) must be the correctly rounded quotient, checked from the definition: the
//    remainder r = a - b q (exact under FMA for a faithful q) must satisfy |r| < b ulp(q) / 2 (no ties exist for
//    binary division).  The hardware reciprocal must also commute with negation and with scaling by 2^k, |k| <= 60,
//    which carries the result to every |a|, |b| in [2^-60, 2^60] where the division reports itself valid.
// 2. Angle wrap: FastArith::wrap(a) must equal normalize_angle(a) bit for bit for every one of the 2^32 floats where
//    it reports itself valid.
// Prints the counts and exits non-zero on any mismatch.
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include <cuda_runtime.h>

#include "../../mppi_generic_vendor_gb300/csrc/mg_math.cuh"

using mg::FastArith;

__global__ void div_pairs(uint32_t a_first, uint32_t a_stride, uint32_t a_count, unsigned long long* bad,
                          unsigned long long* invalid)
{
  const uint32_t bm = blockIdx.x * blockDim.x + threadIdx.x;
  if (bm >= (1u << 23)) return;
  const float b = __uint_as_float(0x3f800000u | bm);
  const float h_hi = b * 0x1p-24f, h_lo = b * 0x1p-25f;
  unsigned int nbad = 0, ninv = 0;
  for (uint32_t i = 0; i < a_count; ++i)
  {
    const uint32_t am = a_first + i * a_stride;
    if (am >= (1u << 23)) break;
    const float a = __uint_as_float(0x3f800000u | am);
    FastArith fa;
    const float q = fa.div(a, b);
    if (!fa.ok) ++ninv;
    const float r = fmaf(-b, q, a);
    float h = q >= 1.0f ? h_hi : h_lo;
    if (q == 1.0f && r < 0.0f) h = h_lo;  // below 1 the float spacing halves
    if (!(fabsf(r) < h)) ++nbad;
  }
  if (nbad) atomicAdd(bad, (unsigned long long)nbad);
  if (ninv) atomicAdd(invalid, (unsigned long long)ninv);
}

__global__ void rcp_scaling(int k, unsigned long long* bad)
{
  const uint32_t bm = blockIdx.x * blockDim.x + threadIdx.x;
  if (bm >= (1u << 23)) return;
  const float b = __uint_as_float(0x3f800000u | bm);
  const float s = ldexpf(1.0f, k), si = ldexpf(1.0f, -k);
  float y, ys, yn;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(b));
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(ys) : "f"(b * s));
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(yn) : "f"(-(b * s)));
  if (__float_as_uint(ys) != __float_as_uint(y * si) || __float_as_uint(yn) != __float_as_uint(-(y * si)))
    atomicAdd(bad, 1ull);
}

__global__ void wrap_all(uint32_t base, unsigned long long* bad, unsigned long long* valid)
{
  const uint32_t bits = base + blockIdx.x * blockDim.x + threadIdx.x;
  const float a = __uint_as_float(bits);
  FastArith fa;
  const float f = fa.wrap(a);
  const float g = mg::normalize_angle(a);
  const bool mismatch = fa.ok && __float_as_uint(f) != __float_as_uint(g);
  const unsigned int nval = __popc(__ballot_sync(0xffffffffu, fa.ok));
  const unsigned int nbad = __popc(__ballot_sync(0xffffffffu, mismatch));
  if ((threadIdx.x & 31) == 0)
  {
    atomicAdd(valid, (unsigned long long)nval);
    if (nbad) atomicAdd(bad, (unsigned long long)nbad);
  }
}

static int check(cudaError_t e, const char* what)
{
  if (e != cudaSuccess)
  {
    std::fprintf(stderr, "%s: %s\n", what, cudaGetErrorString(e));
    std::exit(2);
  }
  return 0;
}

int main(int argc, char** argv)
{
  const uint32_t a_stride = argc > 1 ? (uint32_t)std::strtoul(argv[1], nullptr, 10) : 1u;
  unsigned long long* d = nullptr;
  check(cudaMalloc(&d, 4 * sizeof(unsigned long long)), "cudaMalloc");
  check(cudaMemset(d, 0, 4 * sizeof(unsigned long long)), "cudaMemset");
  // 1. division: launches of 2^23 threads, each walking a_count significands of a
  const uint32_t n_a = ((1u << 23) + a_stride - 1) / a_stride;
  const uint32_t per_launch = 1u << 12;
  for (uint32_t i0 = 0; i0 < n_a; i0 += per_launch)
    div_pairs<<<(1 << 23) / 256, 256>>>(i0 * a_stride, a_stride, per_launch, d, d + 1);
  check(cudaGetLastError(), "div_pairs");
  for (int k = -60; k <= 60; ++k) rcp_scaling<<<(1 << 23) / 256, 256>>>(k, d + 2);
  check(cudaGetLastError(), "rcp_scaling");
  unsigned long long h[4];
  check(cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost), "copy");
  std::printf("division: %llu pairs, %llu not correctly rounded, %llu reported invalid\n",
              (unsigned long long)n_a << 23, h[0], h[1]);
  std::printf("reciprocal scaling and negation, |k| <= 60: %llu mismatches\n", h[2]);
  const bool div_ok = h[0] == 0 && h[1] == 0 && h[2] == 0;
  // 2. angle wrap over every float
  check(cudaMemset(d, 0, 4 * sizeof(unsigned long long)), "cudaMemset");
  for (uint64_t base = 0; base < (1ull << 32); base += (1ull << 28))
    wrap_all<<<(1 << 28) / 256, 256>>>((uint32_t)base, d, d + 1);
  check(cudaGetLastError(), "wrap_all");
  check(cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost), "copy");
  std::printf("angle wrap: %llu of 2^32 floats valid, %llu mismatches\n", h[1], h[0]);
  const bool wrap_ok = h[0] == 0 && h[1] > 0;
  cudaFree(d);
  return div_ok && wrap_ok ? 0 : 1;
}
