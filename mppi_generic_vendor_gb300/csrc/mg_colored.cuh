// mg_colored.cuh — colored (power-law) noise sampler: one kernel from Philox spectrum to constrained control samples.
//
// Restates ColoredNoiseDistributionImpl::generateSamples (colored_noise.cu:285-392): per (sample, control) row, a
// complex standard-normal spectrum of F = T + 1 frequencies (curandGenerateNormal, :343) is scaled by
// s_f = f^(-beta/2) with the DC imaginary part (and the Nyquist one when F is odd) zeroed (configureFrequencyNoise,
// :12-37); an unnormalised inverse real FFT of length N = 2T (cufftExecC2R, :358) gives x[n]; the noise is
// eps[t] = (x[t] - x[offset] * decay^t) / (sigma_c * 2T) (rearrangeNoise, :39-56); then the Gaussian rewrite
// (setGaussianControls, gaussian.cu:17-277) and the control constraints (dynamics.cu:107-126) are applied.
//
// GB300 design: one warp per row.  The length-2T real inverse transform is computed as a T-point complex inverse FFT
// of the even/odd-packed spectrum Z[k] = (X[k] + conj X[T-k]) + i (X[k] - conj X[T-k]) e^{2 pi i k / 2T}, whose
// output z[m] = x[2m] + i x[2m+1]; the radix-2 stages run in warp-private shared memory (T a power of two up to 256;
// other T use a direct transform over a twiddle table).  The CTA owns SPB whole samples (all their controls), so the
// finished tile is written to the [K][T][C] sample buffer with coalesced 16-byte stores.  Host-side per-T tables hold
// the twiddles e^{2 pi i j / N} (computed in double), the frequency scales and sigma (computed in float exactly as the
// reference's host code), and decay^t (host powf).
#pragma once

#include "mg_kernels.cuh"

namespace mg
{
constexpr int kColoredMaxT = 256;

// Layout of one per-T table block (floats, each part 4-float aligned):
//   [0, 2N)                 twiddles (cos, sin) of 2 pi j / N, j < N
//   [tw_end, +F*C)          frequency scales s[f][c]
//   [.., +C)                sigma[c]
//   [.., +T)                decay^t
struct ColoredTable
{
  int scale_off, sigma_off, decay_off;
};

struct ColoredArgs
{
  const InstDesc* inst;
  const int2* work;  // (instance, first sample)
  int num_work;
  int samples_per_item;
  const float* tables;        // per-instance block at tab_off[inst]
  const int* tab_off;         // per instance
  const int4* tab_parts;      // per instance: (scale_off, sigma_off, decay_off, 0) relative to the block
  float* samples;
  const float* mean;
  const float* injected_spec;  // [K][C][F][2] per instance at spec_off, or nullptr for Philox
  const unsigned int* noise_counter;
  uint32_t seed_lo, seed_hi;
  int stride;
  float decay_pow;  // std_dev_decay ^ iteration
  SampleShared sh;
};

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

template <int C, int SPB>
__global__ void __launch_bounds__(32 * SPB * C) colored_sample_kernel(const __grid_constant__ ColoredArgs a)
{
  constexpr int WARPS = SPB * C;
  extern __shared__ __align__(16) float smem[];
  // per warp: X[F] (spectrum, up to kColoredMaxT + 1 complex) and Z[T] (FFT buffer); then the output tile
  float2* Xall = reinterpret_cast<float2*>(smem);
  float2* Zall = Xall + WARPS * (kColoredMaxT + 2);
  float* tile = reinterpret_cast<float*>(Zall + WARPS * kColoredMaxT);  // [SPB][T][C]

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float2* X = Xall + warp * (kColoredMaxT + 2);
  float2* Z = Zall + warp * kColoredMaxT;
  const uint32_t counter = a.noise_counter ? *a.noise_counter : 0u;

  for (int item = blockIdx.x; item < a.num_work; item += gridDim.x)
  {
    const int2 w = a.work[item];
    const InstDesc d = a.inst[w.x];
    const int T = d.T, N = 2 * T, F = T + 1, M = T;
    const float* tab = a.tables + a.tab_off[w.x];
    const int4 parts = a.tab_parts[w.x];
    const float2* tw = reinterpret_cast<const float2*>(tab);
    const float* scale = tab + parts.x;
    const float* sigma = tab + parts.y;
    const float* decay_t = tab + parts.z;
    const int s_local = warp / C, c = warp - s_local * C;
    const int k = w.y + s_local;
    const int nsamp = min(SPB, d.K - w.y);
    const bool active = s_local < nsamp;

    if (active)
    {
      // ---- 1. scaled spectrum X[f]
      const long long row = (long long)k * C + c;
      const int npairs = (F + 1) / 2;
      for (int p = lane; p < npairs; p += 32)
      {
        float4 z;
        if (a.injected_spec)
        {
          const float* src = a.injected_spec + d.spec_off + row * F * 2 + 4 * p;
          z.x = src[0];
          z.y = src[1];
          if (2 * p + 1 < F)
          {
            z.z = src[2];
            z.w = src[3];
          }
          else
          {
            z.z = z.w = 0.0f;
          }
        }
        else
        {
          z = philox_normal4((uint64_t)(row * npairs + p), (uint32_t)w.x | 0x80000000u, counter, a.seed_lo,
                             a.seed_hi);
        }
        const int f0 = 2 * p, f1 = 2 * p + 1;
        const float s0 = scale[f0 * C + c];
        X[f0] = make_float2(z.x * s0, (f0 == 0 || (f0 == F - 1 && (F & 1))) ? 0.0f : z.y * s0);
        if (f1 < F)
        {
          const float s1 = scale[f1 * C + c];
          X[f1] = make_float2(z.z * s1, (f1 == F - 1 && (F & 1)) ? 0.0f : z.w * s1);
        }
      }
      __syncwarp();

      const bool pow2 = (M & (M - 1)) == 0;
      const int logM = 31 - __clz(M);
      float x_off;
      if (pow2)
      {
        // ---- 2. even/odd packing into Z (bit-reversed order)
        for (int kk = lane; kk < M; kk += 32)
        {
          float2 zk;
          if (kk == 0)
          {
            const float e = X[0].x + X[M].x;
            const float o = X[0].x - X[M].x;
            zk = make_float2(e, o);
          }
          else
          {
            const float2 xa = X[kk];
            const float2 xb = make_float2(X[M - kk].x, -X[M - kk].y);
            const float2 e = make_float2(xa.x + xb.x, xa.y + xb.y);
            const float2 o = cmul(make_float2(xa.x - xb.x, xa.y - xb.y), tw[kk]);
            zk = make_float2(e.x - o.y, e.y + o.x);
          }
          const int r = logM ? (int)(__brev((unsigned)kk) >> (32 - logM)) : 0;
          Z[r] = zk;
        }
        __syncwarp();
        // ---- 3. radix-2 inverse FFT (positive exponent, unnormalised)
        for (int len = 2; len <= M; len <<= 1)
        {
          const int half = len >> 1;
          const int tstep = N / len;  // e^{2 pi i j / len} = tw[j * N / len]
          for (int b = lane; b < M / 2; b += 32)
          {
            const int g = b / half, j = b - g * half;
            const int i0 = g * len + j, i1 = i0 + half;
            const float2 t = cmul(tw[j * tstep], Z[i1]);
            const float2 u = Z[i0];
            Z[i0] = make_float2(u.x + t.x, u.y + t.y);
            Z[i1] = make_float2(u.x - t.x, u.y - t.y);
          }
          __syncwarp();
        }
        const int off = a.stride;
        x_off = (off & 1) ? Z[off >> 1].y : Z[off >> 1].x;
      }
      else
      {
        // direct inverse real transform of the Hermitian half spectrum (T not a power of two)
        for (int n = lane; n < T; n += 32)
        {
          float acc = X[0].x + ((n & 1) ? -X[T].x : X[T].x);
          for (int f = 1; f < T; ++f)
          {
            const float2 e = tw[(int)(((long long)f * n) % N)];
            acc += 2.0f * (X[f].x * e.x - X[f].y * e.y);
          }
          reinterpret_cast<float*>(Z)[n] = acc;
        }
        if (lane == 0)
        {
          const int n = a.stride;
          float acc = X[0].x + ((n & 1) ? -X[T].x : X[T].x);
          for (int f = 1; f < T; ++f)
          {
            const float2 e = tw[(int)(((long long)f * n) % N)];
            acc += 2.0f * (X[f].x * e.x - X[f].y * e.y);
          }
          reinterpret_cast<float*>(Z)[T] = acc;
        }
        __syncwarp();
        x_off = reinterpret_cast<float*>(Z)[T];
      }
      // ---- 4. offset / decay / normalisation into the output tile
      const float div = sigma[c] * 2.0f * (float)T;
      for (int t = lane; t < T; t += 32)
      {
        float xt;
        if (pow2)
          xt = (t & 1) ? Z[t >> 1].y : Z[t >> 1].x;
        else
          xt = reinterpret_cast<float*>(Z)[t];
        tile[(s_local * T + t) * C + c] = (xt - x_off * decay_t[t]) / div;
      }
    }
    __syncthreads();
    // ---- 5. Gaussian rewrite + constraints, coalesced store of nsamp whole samples
    const int TC = T * C;
    const int n = nsamp * TC;
    const float pure_threshold = (1.0f - a.sh.pure_pct) * (float)d.K;
    float* dst = a.samples + d.u_off + (long long)w.y * TC;
    for (int e = threadIdx.x; e < n; e += blockDim.x)
    {
      const int sl = e / TC;
      const int rem = e - sl * TC;
      const int t = rem / C, cc = rem - t * C;
      const int kk = w.y + sl;
      const float m = a.mean[d.t_off + rem];
      const float sd = a.decay_pow * a.sh.std_dev[cc];
      const float eps = tile[e];
      float u;
      if (kk == 0 || t < a.stride)
        u = m;
      else if ((float)kk >= pure_threshold)
        u = sd * eps;
      else
        u = fmaf(sd, eps, m);
      dst[e] = enforce_constraint(u, a.sh.lower[cc], a.sh.upper[cc], a.sh.deadband[cc], a.sh.zero[cc]);
    }
    __syncthreads();
  }
}

template <int C, int SPB>
constexpr size_t colored_smem_bytes(int max_t)
{
  return sizeof(float2) * (size_t)SPB * C * (kColoredMaxT + 2) + sizeof(float2) * (size_t)SPB * C * kColoredMaxT +
         sizeof(float) * (size_t)SPB * max_t * C;
}

}  // namespace mg
