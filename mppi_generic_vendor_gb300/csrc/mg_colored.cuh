// mg_colored.cuh — colored (power-law) noise sampler: one kernel from Philox spectrum to constrained control samples.
//
// Restates ColoredNoiseDistributionImpl::generateSamples (colored_noise.cu:285-392): per (sample, control) row, a
// complex standard-normal spectrum of F = T + 1 frequencies (curandGenerateNormal, :343) is scaled by
// s_f = f^(-beta/2) with the DC imaginary part (and the Nyquist one when F is odd) zeroed (configureFrequencyNoise,
// :12-37); an unnormalised inverse real FFT of length N = 2T (cufftExecC2R, :358) gives x[n]; the noise is
// eps[t] = (x[t] - x[offset] * decay^t) / (sigma_c * 2T) (rearrangeNoise, :39-56); then the Gaussian rewrite
// (setGaussianControls, gaussian.cu:17-277) and the control constraints (dynamics.cu:107-126) are applied.
//
// The kernel lives in its own translation unit (mg_colored.cu), compiled with FMA contraction: unlike the rollout,
// its parity with the FP64 reference transform is a tolerance, not bit equality.
#pragma once

#include "mg_kernels.cuh"

namespace mg
{
constexpr int kColoredMaxT = 256;

struct ColoredArgs
{
  const InstDesc* inst;
  const int2* work;  // (instance, first sample)
  int num_work;
  const float* tables;    // per-T blocks, see Engine::build_colored_tables
  const int* tab_off;     // per instance: offset of its block
  const int4* tab_parts;  // per instance: (scale_off, sigma_off, decay_off, 0) relative to the block
  float* samples;
  const float* mean;
  const float* injected_spec;  // [K][C][F][2] per instance at spec_off, or nullptr for Philox
  const unsigned int* noise_counter;
  uint32_t seed_lo, seed_hi;
  int stride;
  float decay_pow;  // std_dev_decay ^ iteration
  SampleShared sh;
};

// Samples per CTA for control dimension C (one warp per (sample, control) row, 8 warps per CTA).
template <int C>
struct ColoredShape
{
  static constexpr int SPB = (8 / C) > 0 ? 8 / C : 1;
  static constexpr int THREADS = 32 * SPB * C;
};

// CTA shape of the four-threads-per-row transform for T = 4L (L = 8, 16, 32): 256 threads (64 rows), the output
// tile, then the exchange buffer of the rows' L-point transforms ([64 rows][4][L + 1] float2, 16-byte aligned).
template <int C, int L>
struct ColoredQuadShape
{
  static constexpr int SPB = 64 / C;
  static constexpr int MIN_CTAS = L >= 32 ? 2 : 3;
  static constexpr int TILE_FLOATS = SPB * (4 * L * C + L / 2 + 1);
  static constexpr int XBUF_OFFSET = (TILE_FLOATS + 3) / 4 * 4;  // floats
  static constexpr size_t SMEM_BYTES = sizeof(float) * (size_t)XBUF_OFFSET + 8u * 64 * 4 * (L + 1);
};

// Horizon class of an instance: 0 = direct transform, 1..3 = four threads per row with T = 32, 64, 128, 4 = one warp
// per row with T = 256.
inline int colored_class(int T)
{
  switch (T)
  {
    case 32: return 1;
    case 64: return 2;
    case 128: return 3;
    case 256: return 4;
    default: return 0;
  }
}

// Launch the colored sampler over every instance of `a`: the work list is grouped by horizon class, class k owning
// items [class_begin[k], class_begin[k + 1]); one launch per non-empty class (defined in mg_colored.cu, C = 1..4).
template <int C>
mppi_status launch_colored_sampler(const ColoredArgs& a, const int* class_begin, int max_t, int num_sms,
                                   cudaStream_t s);

// Samples per work item of horizon class cls.
template <int C>
constexpr int colored_class_spb(int cls)
{
  return (cls >= 1 && cls <= 3) ? ColoredQuadShape<C, 8>::SPB : ColoredShape<C>::SPB;
}

// Uploads the sampler's constant twiddle table (once per engine creation, outside any graph capture).
mppi_status colored_init_constants();

}  // namespace mg
