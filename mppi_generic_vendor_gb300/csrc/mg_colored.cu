// mg_colored.cu — the colored-noise sampler kernel (see mg_colored.cuh for what it restates).
//
// GB300 design: one warp per (sample, control) row and the whole transform in registers.  The length-2T real inverse
// FFT is computed as a T-point complex inverse FFT of the even/odd-packed spectrum
//     Z[k] = (X[k] + conj X[T-k]) + i (X[k] - conj X[T-k]) e^{2 pi i k / 2T},   z = IFFT_T(Z),   z[m] = x[2m] + i x[2m+1]
// For T = 32 R (R = 1, 2, 4, 8) every lane holds R complex values, element index lane + 32 r.  The decimation-in-
// frequency stages whose butterfly distance is a multiple of 32 combine registers of the same lane; the five shorter
// stages exchange values with __shfl_xor_sync.  The output comes out in bit-reversed order and is scattered once into
// the CTA's output tile.  Per-stage twiddles come from a host-built table laid out [stage][register][lane], so every
// twiddle read is a contiguous 256-byte warp access.  Horizons that are not 32 x a power of two use a direct
// transform over a shared-memory copy of the spectrum.  The CTA owns whole samples, so the finished [samples][T][C]
// tile is written with coalesced stores after the Gaussian rewrite and the control constraints.
#include "mg_colored.cuh"
#include "mg_common.cuh"

namespace mg
{
namespace
{
__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Four standard normals of the row-private Philox stream: counter (lane/block id, row, instance tag, iteration).
__device__ __forceinline__ float4 row_normals(uint32_t lane_block, long long row, int inst, uint32_t counter,
                                              uint32_t k0, uint32_t k1)
{
  const u32x4 r = philox4x32_10(u32x4{ lane_block, (uint32_t)row, (uint32_t)inst | 0x80000000u, counter }, k0, k1);
  float4 z;
  box_muller_fast(r.x, r.y, &z.x, &z.y);
  box_muller_fast(r.z, r.w, &z.z, &z.w);
  return z;
}

// Output tile layout: sample row s at s * tile_row_floats(T), element (t, c) at t * C + c + (t >> 3).  The pad of one
// float per 8 steps spreads the bit-reversed stores of the register transform (lanes 8 or 4 steps apart) over the
// shared-memory banks.
__host__ __device__ __forceinline__ int tile_pos(int t, int c, int C) { return t * C + c + (t >> 3); }
__host__ __device__ __forceinline__ int tile_row_floats(int T, int C) { return T * C + (T >> 3) + 1; }

// Register-resident row transform for T = 32 R.  Writes eps[t] (t < T) to tile_row[tile_pos(t, 0, C)].
template <int C, int R>
__device__ __forceinline__ void row_transform_pow2(const ColoredArgs& a, const InstDesc& d, int inst, long long row,
                                                   int c, int lane, const float* tab, const int4 parts,
                                                   float* tile_row, uint32_t counter)
{
  constexpr int M = 32 * R;
  constexpr int LOGM = (R == 1) ? 5 : (R == 2) ? 6 : (R == 4) ? 7 : 8;
  constexpr int LOGR = LOGM - 5;
  const unsigned FULL = 0xffffffffu;
  const float2* tw_pack = reinterpret_cast<const float2*>(tab);
  const float2* tw_reg = tw_pack + M;  // [LOGR][R][32]
  const float2* tw_lane = reinterpret_cast<const float2*>(tab + parts.w);  // [5][32]
  const float* scale = tab + parts.x;
  const float* decay_t = tab + parts.z;
  const float inv_div = 1.0f / (tab[parts.y + c] * 2.0f * (float)M);

  float2 z[R];
  float nyq = 0.0f;
  // ---- 1. scaled spectrum, element f = lane + 32 r, Nyquist (f = M) on lane 0
  if (a.injected_spec)
  {
    const float* src = a.injected_spec + d.spec_off + row * (long long)(M + 1) * 2;
#pragma unroll
    for (int r = 0; r < R; ++r)
    {
      const int f = lane + 32 * r;
      z[r] = make_float2(src[2 * f], src[2 * f + 1]);
    }
    nyq = src[2 * M];
  }
  else
  {
#pragma unroll
    for (int q = 0; q < (R + 1) / 2; ++q)
    {
      const float4 n = row_normals((uint32_t)(lane << 4) | (uint32_t)q, row, inst, counter, a.seed_lo, a.seed_hi);
      z[2 * q] = make_float2(n.x, n.y);
      if (2 * q + 1 < R)
        z[2 * q + 1] = make_float2(n.z, n.w);
      else
        nyq = n.z;
    }
    if ((R % 2) == 0 && lane == 0)
    {
      const float4 n = row_normals((uint32_t)(R / 2), row, inst, counter, a.seed_lo, a.seed_hi);
      nyq = n.x;
    }
  }
#pragma unroll
  for (int r = 0; r < R; ++r)
  {
    const int f = lane + 32 * r;
    const float s = __ldg(scale + f * C + c);
    z[r].x *= s;
    z[r].y = (f == 0) ? 0.0f : z[r].y * s;
  }
  nyq *= __ldg(scale + M * C + c);

  // ---- 2. even/odd packing: partner X[M-k] lives on lane (32 - lane) & 31, register R-1-r (lane 0: R-r / Nyquist)
  {
    float2 p[R];
    const int src = (32 - lane) & 31;
#pragma unroll
    for (int r = 0; r < R; ++r)
    {
      p[r].x = __shfl_sync(FULL, z[R - 1 - r].x, src);
      p[r].y = __shfl_sync(FULL, z[R - 1 - r].y, src);
    }
    if (lane == 0)
    {
#pragma unroll
      for (int r = 0; r < R; ++r)
      {
        if (r == 0)
          p[r] = make_float2(nyq, 0.0f);
        else
          p[r] = z[(R - r) & (R - 1)];
      }
    }
#pragma unroll
    for (int r = 0; r < R; ++r)
    {
      const float2 x = z[r];
      const float2 b = make_float2(p[r].x, -p[r].y);  // conj X[M-k]
      const float2 e = make_float2(x.x + b.x, x.y + b.y);
      const float2 o = cmul(make_float2(x.x - b.x, x.y - b.y), __ldg(tw_pack + lane + 32 * r));
      z[r] = make_float2(e.x - o.y, e.y + o.x);
    }
  }

  // ---- 3. decimation-in-frequency inverse FFT, natural order in, bit-reversed order out
  {
    int s = 0;
#pragma unroll
    for (int hr = R / 2; hr >= 1; hr >>= 1, ++s)
    {
#pragma unroll
      for (int r = 0; r < R; ++r)
      {
        if ((r & hr) == 0)
        {
          const float2 x = z[r], y = z[r + hr];
          z[r] = make_float2(x.x + y.x, x.y + y.y);
          z[r + hr] = cmul(make_float2(x.x - y.x, x.y - y.y), __ldg(tw_reg + (s * R + r) * 32 + lane));
        }
      }
    }
  }
  // Branch-free butterflies: the lower lane of a pair forms z + p, the upper p - z (a sign flip inside one fma), and
  // both multiply by their table twiddle, which is exactly 1 for lower lanes.  The output positions kept below all
  // sit on even lanes unless the offset sample lies in the second half (stride >= T), so the last stage is a plain
  // sum there.
  const bool need_odd = a.stride >= M;
#pragma unroll
  for (int st = 0; st < 5; ++st)
  {
    const int half = 16 >> st;
    const float sgn = (lane & half) ? -1.0f : 1.0f;
    if (st < 4 || need_odd)
    {
      const float2 w = __ldg(tw_lane + st * 32 + lane);
#pragma unroll
      for (int r = 0; r < R; ++r)
      {
        const float px = __shfl_xor_sync(FULL, z[r].x, half);
        const float py = __shfl_xor_sync(FULL, z[r].y, half);
        z[r] = cmul(make_float2(fmaf(z[r].x, sgn, px), fmaf(z[r].y, sgn, py)), w);
      }
    }
    else
    {
#pragma unroll
      for (int r = 0; r < R; ++r)
      {
        const float px = __shfl_xor_sync(FULL, z[r].x, half);
        const float py = __shfl_xor_sync(FULL, z[r].y, half);
        z[r] = make_float2(z[r].x + px, z[r].y + py);
      }
    }
  }

  // ---- 4. x[2m] = Re z[m], x[2m+1] = Im z[m]; position j holds m = bitrev(j)
  const int off = a.stride;
  const int jo = (int)(__brev((unsigned)(off >> 1)) >> (32 - LOGM));
  float sel = 0.0f;
#pragma unroll
  for (int r = 0; r < R; ++r)
    if (r == (jo >> 5)) sel = (off & 1) ? z[r].y : z[r].x;
  const float x_off = __shfl_sync(FULL, sel, jo & 31);
#pragma unroll
  for (int r = 0; r < R; ++r)
  {
    const int m = (int)(__brev((unsigned)(lane + 32 * r)) >> (32 - LOGM));
    if (m < M / 2)
    {
      const int t0 = 2 * m;
      tile_row[tile_pos(t0, 0, C)] = (z[r].x - x_off * __ldg(decay_t + t0)) * inv_div;
      tile_row[tile_pos(t0 + 1, 0, C)] = (z[r].y - x_off * __ldg(decay_t + t0 + 1)) * inv_div;
    }
  }
}

// Direct inverse real transform for horizons that are not 32 x a power of two (X staged in shared memory).
template <int C>
__device__ __forceinline__ void row_transform_direct(const ColoredArgs& a, const InstDesc& d, int inst, long long row,
                                                     int c, int lane, const float* tab, const int4 parts,
                                                     float* tile_row, float2* X, uint32_t counter)
{
  const int T = d.T, N = 2 * T, F = T + 1;
  const float2* tw = reinterpret_cast<const float2*>(tab);  // e^{2 pi i j / N}, j < N
  const float* scale = tab + parts.x;
  const float* decay_t = tab + parts.z;
  const float div = tab[parts.y + c] * 2.0f * (float)T;
  for (int f0 = 2 * lane; f0 < F; f0 += 64)
  {
    float4 n;
    if (a.injected_spec)
    {
      const float* src = a.injected_spec + d.spec_off + row * (long long)F * 2 + 2 * f0;
      n.x = src[0];
      n.y = src[1];
      n.z = (f0 + 1 < F) ? src[2] : 0.0f;
      n.w = (f0 + 1 < F) ? src[3] : 0.0f;
    }
    else
    {
      n = row_normals((uint32_t)(f0 >> 1), row, inst, counter, a.seed_lo, a.seed_hi);
    }
    const float s0 = __ldg(scale + f0 * C + c);
    X[f0] = make_float2(n.x * s0, (f0 == 0 || (f0 == F - 1 && (F & 1))) ? 0.0f : n.y * s0);
    if (f0 + 1 < F)
    {
      const float s1 = __ldg(scale + (f0 + 1) * C + c);
      X[f0 + 1] = make_float2(n.z * s1, (f0 + 1 == F - 1 && (F & 1)) ? 0.0f : n.w * s1);
    }
  }
  __syncwarp();
  auto eval = [&](int n) {
    float acc = X[0].x + ((n & 1) ? -X[T].x : X[T].x);
    int idx = 0;
    for (int f = 1; f < T; ++f)
    {
      idx += n;
      if (idx >= N) idx -= N;
      const float2 e = __ldg(tw + idx);
      acc += 2.0f * (X[f].x * e.x - X[f].y * e.y);
    }
    return acc;
  };
  const float x_off = eval(a.stride);
  for (int t = lane; t < T; t += 32) tile_row[tile_pos(t, 0, C)] = (eval(t) - x_off * __ldg(decay_t + t)) / div;
  __syncwarp();
}

// One launch per horizon class: R = T / 32 for T = 32, 64, 128, 256, R = 0 for the direct transform.  Specialising
// the kernel on R keeps the register footprint of a single transform size.
template <int C, int SPB, int R>
__global__ void __launch_bounds__(32 * SPB * C, (R >= 8 || R == 0) ? 2 : 3)
    colored_sample_kernel(const __grid_constant__ ColoredArgs a)
{
  extern __shared__ __align__(16) float smem[];
  // direct transform only: per-warp spectrum buffers [warps][kColoredMaxT + 2]; then the output tile [SPB][T][C]
  float2* Xall = reinterpret_cast<float2*>(smem);
  float* tile = reinterpret_cast<float*>(Xall + (R == 0 ? SPB * C * (kColoredMaxT + 2) : 0));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t counter = a.noise_counter ? *a.noise_counter : 0u;

  for (int item = blockIdx.x; item < a.num_work; item += gridDim.x)
  {
    const int2 w = a.work[item];
    const InstDesc d = a.inst[w.x];
    const int T = d.T;
    const float* tab = a.tables + a.tab_off[w.x];
    const int4 parts = a.tab_parts[w.x];
    const int s_local = warp / C, c = warp - s_local * C;
    const int nsamp = min(SPB, d.K - w.y);
    if (s_local < nsamp)
    {
      const long long row = (long long)(w.y + s_local) * C + c;
      float* tile_row = tile + s_local * tile_row_floats(T, C) + c;
      if constexpr (R > 0)
        row_transform_pow2<C, R>(a, d, w.x, row, c, lane, tab, parts, tile_row, counter);
      else
        row_transform_direct<C>(a, d, w.x, row, c, lane, tab, parts, tile_row, Xall + warp * (kColoredMaxT + 2),
                                counter);
    }
    __syncthreads();
    // ---- Gaussian rewrite + constraints, coalesced store of nsamp whole samples ([K][T][C] rows are contiguous)
    const int TC = T * C;
    const float pure_threshold = (1.0f - a.sh.pure_pct) * (float)d.K;
    float* dst = a.samples + d.u_off + (long long)w.y * TC;
    if (TC <= (int)blockDim.x && (blockDim.x % TC) == 0)
    {
      const int per_pass = blockDim.x / TC;
      const int rem = threadIdx.x % TC;
      const int t = rem / C, cc = rem - t * C;
      const float m = a.mean[d.t_off + rem];
      const float sd = a.decay_pow * a.sh.std_dev[cc];
      const float lo = a.sh.lower[cc], hi = a.sh.upper[cc], db = a.sh.deadband[cc], zc = a.sh.zero[cc];
      for (int sl = threadIdx.x / TC; sl < nsamp; sl += per_pass)
      {
        const int kk = w.y + sl;
        const float eps = tile[sl * tile_row_floats(T, C) + rem + (t >> 3)];
        float u;
        if (kk == 0 || t < a.stride)
          u = m;
        else if ((float)kk >= pure_threshold)
          u = sd * eps;
        else
          u = fmaf(sd, eps, m);
        dst[sl * TC + rem] = enforce_constraint(u, lo, hi, db, zc);
      }
    }
    else
    {
      const int n = nsamp * TC;
      for (int e = threadIdx.x; e < n; e += blockDim.x)
      {
        const int sl = e / TC;
        const int rem = e - sl * TC;
        const int t = rem / C, cc = rem - t * C;
        const int kk = w.y + sl;
        const float m = a.mean[d.t_off + rem];
        const float sd = a.decay_pow * a.sh.std_dev[cc];
        const float eps = tile[sl * tile_row_floats(T, C) + rem + (t >> 3)];
        float u;
        if (kk == 0 || t < a.stride)
          u = m;
        else if ((float)kk >= pure_threshold)
          u = sd * eps;
        else
          u = fmaf(sd, eps, m);
        dst[e] = enforce_constraint(u, a.sh.lower[cc], a.sh.upper[cc], a.sh.deadband[cc], a.sh.zero[cc]);
      }
    }
    __syncthreads();
  }
}
}  // namespace

template <int C, int R>
static mppi_status launch_class(const ColoredArgs& a, int max_t, int num_sms, cudaStream_t s)
{
  constexpr int SPB = ColoredShape<C>::SPB;
  constexpr int THREADS = ColoredShape<C>::THREADS;
  const size_t xbuf = (R == 0) ? sizeof(float2) * (size_t)SPB * C * (kColoredMaxT + 2) : 0;
  const int tmax = (R == 0) ? max_t : 32 * R;
  const size_t smem = xbuf + sizeof(float) * (size_t)SPB * tile_row_floats(tmax, C);
  auto kern = colored_sample_kernel<C, SPB, R>;
  if (smem > 48 * 1024) MG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 1;
  MG_CUDA(resident_ctas_per_sm(kern, THREADS, smem, &per_sm));
  const int grid = std::max(1, std::min(a.num_work, std::max(per_sm, 1) * num_sms));
  kern<<<grid, THREADS, smem, s>>>(a);
  MG_CUDA(cudaGetLastError());
  return MPPI_OK;
}

template <int C>
mppi_status launch_colored_sampler(const ColoredArgs& a, const int* class_begin, int max_t, int num_sms,
                                   cudaStream_t s)
{
  // class k (R = 0, 1, 2, 4, 8) owns work items [class_begin[k], class_begin[k + 1])
  for (int k = 0; k < 5; ++k)
  {
    const int n = class_begin[k + 1] - class_begin[k];
    if (n <= 0) continue;
    ColoredArgs b = a;
    b.work = a.work + class_begin[k];
    b.num_work = n;
    switch (k)
    {
      case 0: MG_TRY((launch_class<C, 0>(b, max_t, num_sms, s))); break;
      case 1: MG_TRY((launch_class<C, 1>(b, max_t, num_sms, s))); break;
      case 2: MG_TRY((launch_class<C, 2>(b, max_t, num_sms, s))); break;
      case 3: MG_TRY((launch_class<C, 4>(b, max_t, num_sms, s))); break;
      default: MG_TRY((launch_class<C, 8>(b, max_t, num_sms, s))); break;
    }
  }
  return MPPI_OK;
}

template mppi_status launch_colored_sampler<1>(const ColoredArgs&, const int*, int, int, cudaStream_t);
template mppi_status launch_colored_sampler<2>(const ColoredArgs&, const int*, int, int, cudaStream_t);
template mppi_status launch_colored_sampler<3>(const ColoredArgs&, const int*, int, int, cudaStream_t);
template mppi_status launch_colored_sampler<4>(const ColoredArgs&, const int*, int, int, cudaStream_t);

}  // namespace mg
