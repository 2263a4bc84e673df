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

// e^{2 pi i j / 256}, j < 128 (FP64 cos / sin rounded to float): the packing twiddles e^{2 pi i k / 2T}, the
// half-length transforms' twiddles and the final combine's e^{2 pi i m / T}, for every T <= 128.  Indexed with
// compile-time constants in the unrolled transforms, so each twiddle is a constant-bank operand.
__constant__ float2 c_w256[128];

// a * e^{2 pi i idx / 256}, idx a compile-time constant; the trivial rotations cost nothing.
__device__ __forceinline__ float2 rot256(float2 a, int idx)
{
  if (idx == 0) return a;
  if (idx == 64) return make_float2(-a.y, a.x);
  return cmul(a, c_w256[idx]);
}

__host__ __device__ constexpr int bitrev(int x, int bits)
{
  int r = 0;
  for (int b = 0; b < bits; ++b) r |= ((x >> b) & 1) << (bits - 1 - b);
  return r;
}

__host__ __device__ constexpr int ilog2(int x) { return x <= 1 ? 0 : 1 + ilog2(x >> 1); }

// Unnormalised inverse DFT of H points in registers (decimation in frequency, radix 2): v[i] ends up holding output
// bitrev(i).
template <int H>
__device__ __forceinline__ void ifft_dif_regs(float2 (&v)[H + 1])
{
#pragma unroll
  for (int len = H; len >= 2; len >>= 1)
  {
    const int half = len >> 1;
#pragma unroll
    for (int blk = 0; blk < H; blk += len)
#pragma unroll
      for (int j = 0; j < half; ++j)
      {
        const float2 x = v[blk + j], y = v[blk + j + half];
        v[blk + j] = make_float2(x.x + y.x, x.y + y.y);
        v[blk + j + half] = rot256(make_float2(x.x - y.x, x.y - y.y), j * (256 / len));
      }
  }
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

// Four standard normals for block b of parity class p of a row (the two-threads-per-row transform's stream).
__device__ __forceinline__ float4 pair_normals(int b, int p, long long row, int inst, uint32_t counter, uint32_t k0,
                                               uint32_t k1)
{
  const u32x4 r = philox4x32_10(
      u32x4{ (uint32_t)(2 * b + p) | 0x40000000u, (uint32_t)row, (uint32_t)inst | 0x80000000u, counter }, k0, k1);
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

// Gaussian rewrite + constraints of a CTA's finished tile and its coalesced store (nsamp whole samples; [K][T][C]
// rows are contiguous).
template <int C>
__device__ __forceinline__ void colored_store_tile(const ColoredArgs& a, const InstDesc& d, int first, int nsamp,
                                                   const float* tile)
{
  const int T = d.T;
  const int TC = T * C;
  const float pure_threshold = (1.0f - a.sh.pure_pct) * (float)d.K;
  float* dst = a.samples + d.u_off + (long long)first * TC;
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
      const int kk = first + sl;
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
      const int kk = first + sl;
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
}

// Two threads per (sample, control) row for T = 2H in {32, 64, 128}.  With M = T the length-2T real inverse FFT is
// the M-point complex inverse FFT z = IFFT_M(Z) of the packed spectrum (as in row_transform_pow2), and
// z[m] = E[m] + e^{2 pi i m / M} O[m], E and O the H-point inverse FFTs of Z at even and odd k.  Thread p (the lane's
// parity) owns the frequencies k = p (mod 2): it draws and scales X[k] (thread 0 also the Nyquist X[M]), packs
// Z[k] (the partner X[M - k] has the same parity), transforms its half in registers with compile-time twiddles, and
// after one exchange of half its results with the partner lane forms z[m] for m in [p H/2, (p+1) H/2), i.e. the
// outputs t in [p H, (p+1) H).  Register r of thread 0 holds k = 2r (r = H: the Nyquist bin); thread 1 holds
// k = 2r + 1 for r < H/2 and k = 2r - 1 for r > H/2 (register H/2 unused), so that for both threads registers r and
// H - r hold a conjugate pair (k, M - k).  No shuffles inside the transform, one 16-entry-per-output exchange.
template <int C, int H>
__global__ void __launch_bounds__(ColoredPairShape<C, H>::THREADS, ColoredPairShape<C, H>::MIN_CTAS)
    colored_pair_kernel(const __grid_constant__ ColoredArgs a)
{
  constexpr int M = 2 * H;
  constexpr int SPB = ColoredPairShape<C, H>::SPB;
  constexpr int LOGH = ilog2(H);
  constexpr int TW = 256 / M;  // c_w256 index step of e^{2 pi i / M}; e^{2 pi i k / 2M} steps by TW / 2
  extern __shared__ __align__(16) float tile[];
  const int tid = threadIdx.x, lane = tid & 31, p = tid & 1;
  const int row_local = tid >> 1;
  const int s_local = row_local / C, c = row_local - s_local * C;
  const unsigned pair = 3u << (lane & ~1);
  const uint32_t counter = a.noise_counter ? *a.noise_counter : 0u;
  for (int item = blockIdx.x; item < a.num_work; item += gridDim.x)
  {
    const int2 w = a.work[item];
    const InstDesc d = a.inst[w.x];
    const float* tab = a.tables + a.tab_off[w.x];
    const int4 parts = a.tab_parts[w.x];
    const int nsamp = min(SPB, d.K - w.y);
    if (s_local < nsamp)  // both threads of a row take the same branch
    {
      const long long row = (long long)(w.y + s_local) * C + c;
      const float* scale = tab + parts.x;
      const float* decay_t = tab + parts.z;
      const float inv_div = 1.0f / (tab[parts.y + c] * 2.0f * (float)M);
      auto freq = [&](int r) { return p == 0 ? 2 * r : (r < H / 2 ? 2 * r + 1 : 2 * r - 1); };
      float2 v[H + 1];
      // ---- 1. the scaled spectrum of this thread's frequencies
      if (a.injected_spec)
      {
        const float* src = a.injected_spec + d.spec_off + row * (long long)(M + 1) * 2;
#pragma unroll
        for (int r = 0; r <= H; ++r)
        {
          const int f = freq(r);
          v[r] = make_float2(src[2 * f], src[2 * f + 1]);
        }
      }
      else
      {
#pragma unroll
        for (int b = 0; b < H / 2; ++b)
        {
          const float4 n = pair_normals(b, p, row, w.x, counter, a.seed_lo, a.seed_hi);
          v[2 * b] = make_float2(n.x, n.y);
          v[2 * b + 1] = make_float2(n.z, n.w);
        }
        // thread 0: the Nyquist bin takes the DC bin's imaginary draw (which the DC bin discards); thread 1:
        // register H takes register H/2's draw
        v[H] = p == 0 ? make_float2(v[0].y, 0.0f) : v[H / 2];
      }
#pragma unroll
      for (int r = 0; r <= H; ++r)
      {
        const float sc = __ldg(scale + freq(r) * C + c);
        v[r].x *= sc;
        v[r].y *= sc;
      }
      v[0].y = p ? v[0].y : 0.0f;  // DC and Nyquist bins are real
      v[H].y = p ? v[H].y : 0.0f;
      // ---- 2. packing Z[k] = (X[k] + conj X[M-k]) + i (X[k] - conj X[M-k]) e^{2 pi i k / 2M}, pairwise in place
#pragma unroll
      for (int r = 0; r <= H / 2; ++r)
      {
        const int rr = H - r;
        const float2 x = v[r], y = v[rr];
        auto pack = [&](float2 xa, float2 xb, int r_of) {
          const int k0 = 2 * r_of, k1 = r_of < H / 2 ? 2 * r_of + 1 : 2 * r_of - 1;
          // e^{2 pi i k / 2M} for this thread's k (k = M, thread 0's Nyquist register, has no Z of its own)
          const float2 w0 = k0 < M ? c_w256[k0 * TW / 2] : make_float2(1.0f, 0.0f);
          const float2 w1 = c_w256[k1 * TW / 2];
          const float2 tw = p ? w1 : w0;
          const float2 e = make_float2(xa.x + xb.x, xa.y - xb.y);
          const float2 o = cmul(make_float2(xa.x - xb.x, xa.y + xb.y), tw);
          return make_float2(e.x - o.y, e.y + o.x);
        };
        v[r] = pack(x, y, r);
        if (rr != r) v[rr] = pack(y, x, rr);
      }
      // ---- 3. this thread's half: u[j] = Z[2j + p]; thread 1's upper half sits one register up
#pragma unroll
      for (int j = H / 2; j < H; ++j) v[j] = p ? v[j + 1] : v[j];
      ifft_dif_regs<H>(v);
      // ---- 4. exchange and combine: thread 0 holds E, thread 1 holds O, at register bitrev(m)
      const int m_off = a.stride >> 1;
      const bool wrap = m_off >= H;  // x[stride] in the second half of z: E[m'] - W^m' O[m']
      const int mm = wrap ? m_off - H : m_off;
      const int p_o = mm >= H / 2 ? 1 : 0, i_o = mm - p_o * (H / 2);
      float2 zz[H / 2];
      float xo = 0.0f;
#pragma unroll
      for (int i = 0; i < H / 2; ++i)
      {
        const float2 lo = v[bitrev(i, LOGH)], hi = v[bitrev(H / 2 + i, LOGH)];
        const float2 send = p ? lo : hi;  // thread 0 sends E[H/2 + i], thread 1 sends O[i]
        float2 recv;
        recv.x = __shfl_xor_sync(pair, send.x, 1);
        recv.y = __shfl_xor_sync(pair, send.y, 1);
        // m = p H/2 + i: z[m] = E[m] + W^m O[m] with W^m = W^i (thread 0) or i W^i (thread 1)
        const float2 e = p ? recv : lo;
        float2 o = p ? hi : recv;
        o = p ? make_float2(-o.y, o.x) : o;
        const float2 t = rot256(o, i * TW);
        zz[i] = make_float2(e.x + t.x, e.y + t.y);
        if (i == i_o)
        {
          const float2 zo = wrap ? make_float2(e.x - t.x, e.y - t.y) : zz[i];
          xo = (a.stride & 1) ? zo.y : zo.x;
        }
      }
      const float x_off = __shfl_sync(pair, xo, (lane & ~1) | p_o);
      // ---- 5. eps[t] = (x[t] - x[offset] decay^t) / (sigma_c 2T) into the CTA's tile
      float* tile_row = tile + s_local * tile_row_floats(M, C) + c;
#pragma unroll
      for (int i = 0; i < H / 2; ++i)
      {
        const int t0 = p * H + 2 * i;
        tile_row[tile_pos(t0, 0, C)] = (zz[i].x - x_off * __ldg(decay_t + t0)) * inv_div;
        tile_row[tile_pos(t0 + 1, 0, C)] = (zz[i].y - x_off * __ldg(decay_t + t0 + 1)) * inv_div;
      }
    }
    __syncthreads();
    colored_store_tile<C>(a, d, w.y, nsamp, tile);
    __syncthreads();
  }
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
    colored_store_tile<C>(a, d, w.y, nsamp, tile);
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

template <int C, int H>
static mppi_status launch_pair(const ColoredArgs& a, int num_sms, cudaStream_t s)
{
  using Shape = ColoredPairShape<C, H>;
  const size_t smem = sizeof(float) * (size_t)Shape::SPB * tile_row_floats(2 * H, C);
  auto kern = colored_pair_kernel<C, H>;
  if (smem > 48 * 1024) MG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 1;
  MG_CUDA(resident_ctas_per_sm(kern, Shape::THREADS, smem, &per_sm));
  const int grid = std::max(1, std::min(a.num_work, std::max(per_sm, 1) * num_sms));
  kern<<<grid, Shape::THREADS, smem, s>>>(a);
  MG_CUDA(cudaGetLastError());
  return MPPI_OK;
}

mppi_status colored_init_constants()
{
  float2 w[128];
  for (int j = 0; j < 128; ++j)
    w[j] = make_float2((float)std::cos(2.0 * M_PI * j / 256.0), (float)std::sin(2.0 * M_PI * j / 256.0));
  MG_CUDA(cudaMemcpyToSymbol(c_w256, w, sizeof(w)));
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
      case 1: MG_TRY((launch_pair<C, 16>(b, num_sms, s))); break;
      case 2: MG_TRY((launch_pair<C, 32>(b, num_sms, s))); break;
      case 3: MG_TRY((launch_pair<C, 64>(b, num_sms, s))); break;
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
