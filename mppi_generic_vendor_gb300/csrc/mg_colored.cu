// mg_colored.cu — the colored-noise sampler kernels (see mg_colored.cuh for what they restate).
//
// GB300 design.  The length-2T real inverse FFT of a (sample, control) row is computed as a T-point complex inverse
// FFT of the even/odd-packed spectrum
//     Z[k] = (X[k] + conj X[T-k]) + i (X[k] - conj X[T-k]) e^{2 pi i k / 2T},   z = IFFT_T(Z),   z[m] = x[2m] + i x[2m+1]
// of which only z[m < T/2] (x[t < T]) and x[offset] are needed.
//  * T = 32, 64, 128 (colored_quad_kernel): four lanes per row, lane q owning the frequencies k = q (mod 4); each
//    draws, scales and packs its quarter, runs a T/4-point transform in registers with constant-bank twiddles, and
//    one exchange through shared memory and a radix-4 combine give the row's T outputs.  Most arithmetic is plain
//    FMA on registers; per output about one shared-memory word moves.
//  * T = 256 (colored_sample_kernel, R = 8): one warp per row, every lane holding R complex values (element index
//    lane + 32 r); the decimation-in-frequency stages of butterfly distance >= 32 stay in a lane's registers, the
//    five shorter ones exchange values with __shfl_xor_sync, twiddles from a host-built [stage][register][lane] table.
//  * other T (R = 0): a direct transform over a shared-memory copy of the spectrum.
// Every form scatters its noise into the CTA's output tile, and the finished [samples][T][C] tile is written with
// coalesced stores after the Gaussian rewrite and the control constraints.
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

// complex sum and difference as one paired FP32 instruction each (add / sub .rn.f32x2)
__device__ __forceinline__ float2 cadd(float2 a, float2 b)
{
  const f32x2 r = add2({ a.x, a.y }, { b.x, b.y });
  return make_float2(r.x, r.y);
}
__device__ __forceinline__ float2 csub(float2 a, float2 b)
{
  const f32x2 r = sub2({ a.x, a.y }, { b.x, b.y });
  return make_float2(r.x, r.y);
}

// e^{2 pi i j / 256}, j < 128 (FP64 cos / sin rounded to float): the packing twiddles e^{2 pi i k / 2T}, the
// half-length transforms' twiddles and the final combine's e^{2 pi i m / T}, for every T <= 128.  Indexed with
// compile-time constants in the unrolled transforms, so each twiddle is a constant-bank operand.
__constant__ float2 c_w256[128];

// a * e^{2 pi i idx / 256}, idx a compile-time constant in [0, 256); the trivial rotations cost nothing.
__device__ __forceinline__ float2 rot256(float2 a, int idx)
{
  if (idx >= 128) a = make_float2(-a.x, -a.y), idx -= 128;
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
        v[blk + j] = cadd(x, y);
        v[blk + j + half] = rot256(csub(x, y), j * (256 / len));
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
    const float* src = a.injected_spec + d.noise_spec_off + row * (long long)(M + 1) * 2;
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
      const float* src = a.injected_spec + d.noise_spec_off + row * (long long)F * 2 + 2 * f0;
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

// Four threads per (sample, control) row for T = M = 4 L (L = 8, 16, 32: T = 32, 64, 128): with k = 4j + q and
// m = m1 + L m2 (m1 < L),
//   z[m1 + L m2] = sum_q i^{q m2} W^{q m1} A_q[m1],   A_q = IFFT_L(Z[4j + q]),   W = e^{2 pi i / M}.
// Thread q (lane & 3) owns the frequencies k = q (mod 4): it draws and scales X[k], packs Z[k] (the partner
// X[M - k] is its own for q = 0, 2 and lane q ^ 2's for q = 1, 3, exchanged a register pair at a time), runs its
// L-point transform in registers and writes A_q to shared memory; after a warp barrier it reads A_q'[m1] for
// m1 = 4 i + q (i < L / 4) of the row's four threads and forms z[m1] and z[m1 + L], i.e. x[t] for the outputs
// t = 8 i + 2 q (+1) (+2L).  Register r holds j = r (r < L) for q != 0; for q = 0 it holds j = r (r < L/2),
// j = r + 1 (L/2 <= r < L; r = L - 1: the Nyquist bin) and j = L/2 (r = L), so that registers r and L - 1 - r hold
// a conjugate pair (k, M - k) for every q.
template <int C, int L>
__global__ void __launch_bounds__(256, ColoredQuadShape<C, L>::MIN_CTAS)
    colored_quad_kernel(const __grid_constant__ ColoredArgs a)
{
  constexpr int M = 4 * L;
  constexpr int LOGL = ilog2(L);
  constexpr int TW = 256 / M;  // c_w256 index step of e^{2 pi i / M}; e^{2 pi i k / 2M} steps by TW / 2
  constexpr int SPB = ColoredQuadShape<C, L>::SPB;
  constexpr int SEG = L + 1;  // float2 per (row, q) segment of the exchange buffer (one float2 of padding)
  extern __shared__ __align__(16) float smem[];
  float* tile = smem;
  float2* xbuf = reinterpret_cast<float2*>(smem + ColoredQuadShape<C, L>::XBUF_OFFSET);
  const int tid = threadIdx.x, lane = tid & 31, q = tid & 3;
  const int row_local = tid >> 2;
  const int s_local = row_local / C, c = row_local - s_local * C;
  const unsigned quad = 0xFu << (lane & ~3);
  const uint32_t counter = a.noise_counter ? *a.noise_counter : 0u;
  float2* my_seg = xbuf + (row_local * 4 + q) * SEG;
  const float2* row_seg = xbuf + row_local * 4 * SEG;
  for (int item = blockIdx.x; item < a.num_work; item += gridDim.x)
  {
    const int2 w = a.work[item];
    const InstDesc d = a.inst[w.x];
    const float* tab = a.tables + a.tab_off[w.x];
    const int4 parts = a.tab_parts[w.x];
    const int nsamp = min(SPB, d.K - w.y);
    if (s_local < nsamp)  // the four threads of a row take the same branch
    {
      const long long row = (long long)(w.y + s_local) * C + c;
      const float* scale = tab + parts.x;
      const float* decay_t = tab + parts.z;
      const float inv_div = 1.0f / (tab[parts.y + c] * 2.0f * (float)M);
      // frequency of register r (0 for thread q != 0's unused register L)
      auto freq = [&](int r) {
        if (q == 0) return 4 * (r < L / 2 ? r : (r < L ? r + 1 : L / 2));
        return r < L ? 4 * r + q : 0;
      };
      float2 v[L + 1];
      // ---- 1. the scaled spectrum of this thread's frequencies
      if (a.injected_spec)
      {
        const float* src = a.injected_spec + d.noise_spec_off + row * (long long)(M + 1) * 2;
#pragma unroll
        for (int r = 0; r <= L; ++r)
        {
          const int f = freq(r);
          v[r] = make_float2(src[2 * f], src[2 * f + 1]);
        }
      }
      else
      {
#pragma unroll
        for (int b = 0; b < L / 2; ++b)
        {
          const u32x4 u = philox4x32_10(u32x4{ (uint32_t)(4 * b + q) | 0x20000000u, (uint32_t)row,
                                               (uint32_t)d.noise_inst | 0x80000000u, counter },
                                        a.seed_lo, a.seed_hi);
          box_muller_fast(u.x, u.y, &v[2 * b].x, &v[2 * b].y);
          box_muller_fast(u.z, u.w, &v[2 * b + 1].x, &v[2 * b + 1].y);
        }
        // thread 0: j = L/2 takes the imaginary draws the DC and Nyquist bins discard
        v[L] = make_float2(v[0].y, v[L - 1].y);
      }
#pragma unroll
      for (int r = 0; r <= L; ++r)
      {
        const float sc = __ldg(scale + freq(r) * C + c);
        const f32x2 w = mul2({ v[r].x, v[r].y }, { sc, sc });
        v[r] = make_float2(w.x, w.y);
      }
      v[0].y = q ? v[0].y : 0.0f;  // thread 0: the DC and Nyquist bins are real
      v[L - 1].y = q ? v[L - 1].y : 0.0f;
      // ---- 2. packing Z[k] = (X[k] + conj X[M-k]) + i (X[k] - conj X[M-k]) e^{2 pi i k / 2M}
      // e^{2 pi i k / 2M} = e^{2 pi i 4 r / 2M} * phi, phi per thread (and per register half for thread 0)
      const float2 phi_lo = q ? c_w256[q * TW / 2] : make_float2(1.0f, 0.0f);
      const float2 phi_hi = q ? c_w256[q * TW / 2] : c_w256[4 * TW / 2];
      auto pack = [&](float2 x, float2 y, int r) {
        const float2 e = make_float2(x.x + y.x, x.y - y.y);
        const float2 o =
            rot256(cmul(make_float2(x.x - y.x, x.y + y.y), r < L / 2 ? phi_lo : phi_hi), 4 * r * TW / 2);
        return make_float2(e.x - o.y, e.y + o.x);
      };
#pragma unroll
      for (int r = 0; r < L / 2; ++r)
      {
        const int rr = L - 1 - r;
        const float2 x = v[r], y = v[rr];
        float2 rx, ry;  // lane q ^ 2's registers r and L - 1 - r
        rx.x = __shfl_xor_sync(quad, x.x, 2);
        rx.y = __shfl_xor_sync(quad, x.y, 2);
        ry.x = __shfl_xor_sync(quad, y.x, 2);
        ry.y = __shfl_xor_sync(quad, y.y, 2);
        const bool remote = (q & 1) != 0;
        v[r] = pack(x, remote ? ry : y, r);
        v[rr] = pack(y, remote ? rx : x, rr);
      }
      {
        // thread 0's self-conjugate bin k = M/2 (register L): e^{2 pi i (M/2) / 2M} = i
        const float2 x = v[L];
        const float2 e = make_float2(2.0f * x.x, 0.0f);
        const float2 o = make_float2(-2.0f * x.y, 0.0f);  // (x - conj x) * i = (2i Im x) * i
        v[L] = make_float2(e.x - o.y, e.y + o.x);
      }
      // ---- 3. natural order u[j] = Z[4j + q] for thread 0, then the L-point transform
#pragma unroll
      for (int j = L - 1; j >= L / 2 + 1; --j) v[j] = q ? v[j] : v[j - 1];
      v[L / 2] = q ? v[L / 2] : v[L];
      ifft_dif_regs<L>(v);
#pragma unroll
      for (int m1 = 0; m1 < L; ++m1) my_seg[m1] = v[bitrev(m1, LOGL)];
      __syncwarp(quad);
      // ---- 4. z[m1 + L m2] = sum_q' i^{q' m2} W^{q' m1} A_q'[m1] for this thread's m1 = 4 i + q
      const float2 w1 = c_w256[q * TW], w2 = c_w256[2 * q * TW], w3 = c_w256[3 * q * TW];  // W^{q' q}
      const int m_off = a.stride >> 1;
      const int m1_o = m_off & (L - 1), m2_o = m_off >> LOGL, q_o = m1_o & 3, i_o = m1_o >> 2;
      float2 z0[L / 4], z1[L / 4];
      float xo = 0.0f;
#pragma unroll
      for (int i = 0; i < L / 4; ++i)
      {
        const int m1 = 4 * i + q;
        const float2 b0 = row_seg[m1];
        const float2 b1 = rot256(cmul(row_seg[SEG + m1], w1), 4 * i * TW);
        const float2 b2 = rot256(cmul(row_seg[2 * SEG + m1], w2), 8 * i * TW);
        const float2 b3 = rot256(cmul(row_seg[3 * SEG + m1], w3), 12 * i * TW);
        const float2 s02 = cadd(b0, b2), d02 = csub(b0, b2);
        const float2 s13 = cadd(b1, b3), d13 = csub(b1, b3);
        z0[i] = cadd(s02, s13);  // m2 = 0
        z1[i] = make_float2(d02.x - d13.y, d02.y + d13.x);  // m2 = 1: b0 + i b1 - b2 - i b3
        if (i == i_o)
        {
          const float2 z2 = make_float2(s02.x - s13.x, s02.y - s13.y);  // m2 = 2
          const float2 z3 = make_float2(d02.x + d13.y, d02.y - d13.x);  // m2 = 3
          const float2 zo = m2_o == 0 ? z0[i] : m2_o == 1 ? z1[i] : m2_o == 2 ? z2 : z3;
          xo = (a.stride & 1) ? zo.y : zo.x;
        }
      }
      const float x_off = __shfl_sync(quad, xo, (lane & ~3) | q_o);
      // ---- 5. eps[t] = (x[t] - x[offset] decay^t) / (sigma_c 2T) into the CTA's tile
      float* tile_row = tile + s_local * tile_row_floats(M, C) + c;
#pragma unroll
      for (int i = 0; i < L / 4; ++i)
      {
#pragma unroll
        for (int m2 = 0; m2 < 2; ++m2)
        {
          const float2 z = m2 ? z1[i] : z0[i];
          const int t0 = 8 * i + 2 * q + 2 * L * m2;
          // (x[t] - x[offset] decay^t) / (sigma_c 2T) for the output pair (t0, t0 + 1)
          const f32x2 e = mul2(fma2({ -x_off, -x_off }, { __ldg(decay_t + t0), __ldg(decay_t + t0 + 1) }, { z.x, z.y }),
                               { inv_div, inv_div });
          tile_row[tile_pos(t0, 0, C)] = e.x;
          tile_row[tile_pos(t0 + 1, 0, C)] = e.y;
        }
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
        row_transform_pow2<C, R>(a, d, d.noise_inst, row, c, lane, tab, parts, tile_row, counter);
      else
        row_transform_direct<C>(a, d, d.noise_inst, row, c, lane, tab, parts, tile_row,
                                Xall + warp * (kColoredMaxT + 2), counter);
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
  MG_CUDA(raise_smem_cap(kern, smem));
  int per_sm = 1;
  MG_CUDA(resident_ctas_per_sm(kern, THREADS, smem, &per_sm));
  const int grid = std::max(1, std::min(a.num_work, std::max(per_sm, 1) * num_sms));
  kern<<<grid, THREADS, smem, s>>>(a);
  MG_CUDA(cudaGetLastError());
  return MPPI_OK;
}

template <int C, int L>
static mppi_status launch_quad(const ColoredArgs& a, int num_sms, cudaStream_t s)
{
  using Shape = ColoredQuadShape<C, L>;
  const size_t smem = Shape::SMEM_BYTES;
  auto kern = colored_quad_kernel<C, L>;
  MG_CUDA(raise_smem_cap(kern, smem));
  int per_sm = 1;
  MG_CUDA(resident_ctas_per_sm(kern, 256, smem, &per_sm));
  const int grid = std::max(1, std::min(a.num_work, std::max(per_sm, 1) * num_sms));
  kern<<<grid, 256, smem, s>>>(a);
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
      case 1: MG_TRY((launch_quad<C, 8>(b, num_sms, s))); break;
      case 2: MG_TRY((launch_quad<C, 16>(b, num_sms, s))); break;
      case 3: MG_TRY((launch_quad<C, 32>(b, num_sms, s))); break;
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
