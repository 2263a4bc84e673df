// mg_surrogate.cu — the learned dynamics surrogate: training data from the analytic model, forward / backward kernels,
// Adam, validation.  The reference only evaluates pre-trained networks (FNNHelper, fnn_helper.cu:418-495, loaded from
// .npz files); training on the GPU is new.
//
// Network: 9 -> 64 -> 64 -> 5, tanh hidden layers, linear output (FNNHelper::forward, fnn_helper.cu:353-382).  Inputs are
// the full state (x, y, yaw, vx, vy, yaw_rate, steer) and the controls (throttle, steer_cmd); outputs are the time
// derivatives of (yaw, vx, vy, yaw_rate, steer); x and y derivatives stay analytic (NeuralNetModel::computeKinematics,
// ar_nn_model.cu:119-124).
//
// Training step: one CTA per 64 samples computes the forward pass, the loss and the back-propagated gradient of its
// samples in shared memory and writes its partial gradient row; a second kernel adds the rows in CTA order (a fixed
// order, so training is deterministic for a given seed) and applies Adam.
//
// Quantisation-aware training (weight format BF16 or FP8): the forward and backward passes use the weights as the
// tensor-core rollout will hold them (rounded to BF16, or E4M3 with the per-layer power-of-two scale of the current
// weights) and Adam updates the FP32 master weights with that gradient (straight-through: the rounding is treated as
// the identity when differentiating), so the network learns to work through its own quantisation.
#include <cuda_bf16.h>
#include <cuda_fp8.h>

#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

#include "mg_common.cuh"
#include "mg_kernels.cuh"

struct mppi_surrogate;

namespace mg
{
namespace
{
constexpr int kIn = 9, kHid = 64, kOut = 5;
constexpr int oW1 = 0, oB1 = oW1 + kHid * kIn, oW2 = oB1 + kHid, oB2 = oW2 + kHid * kHid, oW3 = oB2 + kHid,
              oB3 = oW3 + kOut * kHid, kNW = oB3 + kOut;
constexpr int oInMean = kNW, oInStd = oInMean + kIn, oOutMean = oInStd + kIn, oOutStd = oOutMean + kOut,
              kNP = oOutStd + kOut;
static_assert(kNW == MPPI_MLP_WEIGHTS && kNP == MPPI_MLP_PARAMS, "parameter layout");
constexpr int kSB = 64;         // samples per CTA in the training kernels
constexpr int kPad = 65;        // padded activation row (bank-conflict free column access)
constexpr int kRow = kNW + 1;   // partial row: gradient + loss
constexpr uint32_t kDataTag = 0x51u, kValTag = 0x52u, kBatchTag = 0x53u;

struct Norm
{
  float in_mean[kIn], in_std[kIn], out_mean[kOut], out_std[kOut];
};

struct Box
{
  float lo[7], hi[7];
};

// Transition i of a Philox stream: state uniform in the box, controls uniform in [-1, 1], analytic derivatives.
__device__ __forceinline__ void draw_transition(const mppi_bicycle_slip_params& p, const Box& box, uint32_t k0,
                                                uint32_t k1, uint32_t tag, uint32_t i, float* x, float* y)
{
  float u[12];
#pragma unroll
  for (int q = 0; q < 3; ++q)
  {
    const u32x4 r = philox4x32_10(u32x4{ i, (uint32_t)q, tag, 0u }, k0, k1);
    u[4 * q] = uniform_open01(r.x);
    u[4 * q + 1] = uniform_open01(r.y);
    u[4 * q + 2] = uniform_open01(r.z);
    u[4 * q + 3] = uniform_open01(r.w);
  }
  float s[7], c[2], xd[7];
#pragma unroll
  for (int j = 0; j < 7; ++j) s[j] = box.lo[j] + (box.hi[j] - box.lo[j]) * u[j];
  c[0] = 2.0f * u[7] - 1.0f;
  c[1] = 2.0f * u[8] - 1.0f;
  BicycleSlipModel::computeDynamics(p, s, c, xd);
#pragma unroll
  for (int j = 0; j < 7; ++j) x[j] = s[j];
  x[7] = c[0];
  x[8] = c[1];
#pragma unroll
  for (int j = 0; j < kOut; ++j) y[j] = xd[2 + j];
}

__global__ void data_kernel(mppi_bicycle_slip_params p, Box box, uint32_t k0, uint32_t k1, int n, float* X, float* Y,
                            double* stats /* [gridDim][2 * kOut] */)
{
  double s1[kOut] = {}, s2[kOut] = {};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
  {
    float x[kIn], y[kOut];
    draw_transition(p, box, k0, k1, kDataTag, (uint32_t)i, x, y);
    for (int j = 0; j < kIn; ++j) X[(size_t)i * kIn + j] = x[j];
    for (int j = 0; j < kOut; ++j)
    {
      Y[(size_t)i * kOut + j] = y[j];
      s1[j] += y[j];
      s2[j] += (double)y[j] * y[j];
    }
  }
  __shared__ double red[2 * kOut][32];
  for (int j = 0; j < kOut; ++j)
  {
    double a = s1[j], b = s2[j];
    for (int off = 16; off > 0; off >>= 1)
    {
      a += __shfl_xor_sync(0xffffffffu, a, off);
      b += __shfl_xor_sync(0xffffffffu, b, off);
    }
    if ((threadIdx.x & 31) == 0)
    {
      red[j][threadIdx.x >> 5] = a;
      red[kOut + j][threadIdx.x >> 5] = b;
    }
  }
  __syncthreads();
  if (threadIdx.x < 2 * kOut)
  {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[threadIdx.x][w];
    stats[blockIdx.x * 2 * kOut + threadIdx.x] = t;
  }
}

// Per-layer power-of-two scale of the FP8 weight format (the smallest with max |W| / scale <= 448, 1 for an all-zero
// layer), the same choice the rollout's weight preparation makes; one CTA per layer.
__global__ void __launch_bounds__(256) weight_scale_kernel(const float* params, float* scales)
{
  __shared__ float s_max[8];
  const int off[3] = { oW1, oW2, oW3 }, len[3] = { kHid * kIn, kHid * kHid, kOut * kHid };
  const int l = blockIdx.x;
  float m = 0.0f;
  for (int e = threadIdx.x; e < len[l]; e += blockDim.x) m = fmaxf(m, fabsf(params[off[l] + e]));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0)
  {
    float a = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) a = fmaxf(a, s_max[w]);
    float scale = 1.0f;
    if (a > 0.0f)
    {
      int ex = 0;
      const float fr = frexpf(a / 448.0f, &ex);
      scale = ldexpf(1.0f, fr == 0.5f ? ex - 1 : ex);
    }
    scales[l] = scale;
  }
}

// A weight as the tensor cores see it in weight format `fmt` (0 BF16, 1 E4M3 times the layer scale, 2 FP32).
__device__ __forceinline__ float quantize_weight(float w, int fmt, float scale)
{
  if (fmt == 0) return __bfloat162float(__float2bfloat16_rn(w));
  if (fmt == 1) return (float)__nv_fp8_e4m3(w / scale) * scale;
  return w;
}

struct GradArgs
{
  const float* params;
  int wfmt;             // weight format of the forward / backward passes (2: FP32 master weights as they are)
  const float* wscale;  // per-layer FP8 scales (wfmt 1)
  const float* X;
  const float* Y;
  int n;               // rows in X / Y
  int batch;           // samples in this step
  int pre_normalized;  // 1: X / Y hold normalised rows used in order (gradient check)
  uint32_t k0, k1, step;
  Norm norm;
  float* partials;  // [gridDim][kRow]
};

__global__ void __launch_bounds__(256) grad_kernel(const __grid_constant__ GradArgs a)
{
  extern __shared__ __align__(16) float sm[];
  float* W = sm;                // natural parameter layout
  float* xs = W + 5128;         // [kSB][9]
  float* h1 = xs + kSB * kIn;   // [kSB][kPad]
  float* h2 = h1 + kSB * kPad;  // [kSB][kPad], later dL/dh1
  float* d2 = h2 + kSB * kPad;  // [kSB][kPad] dL/dh2
  float* dy = d2 + kSB * kPad;  // [kSB][5]  targets, then dL/dy
  __shared__ float s_loss[8];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int b0 = blockIdx.x * kSB;
  const int nb = min(kSB, a.batch - b0);
  const float scale = 2.0f / ((float)a.batch * kOut);

  for (int i = tid; i < kNW; i += nt)
  {
    const int l = i < oB1 ? 0 : (i >= oW2 && i < oB2) ? 1 : (i >= oW3 && i < oB3) ? 2 : -1;
    W[i] = (l >= 0 && a.wfmt != 2) ? quantize_weight(a.params[i], a.wfmt, a.wfmt == 1 ? a.wscale[l] : 1.0f)
                                   : a.params[i];
  }
  for (int b = tid; b < kSB; b += nt)
  {
    int row = 0;
    if (b < nb)
    {
      if (a.pre_normalized)
        row = b0 + b;
      else
        row = (int)(philox4x32_10(u32x4{ (uint32_t)(b0 + b), a.step, kBatchTag, 0u }, a.k0, a.k1).x % (uint32_t)a.n);
    }
    for (int i = 0; i < kIn; ++i)
    {
      float v = (b < nb) ? a.X[(size_t)row * kIn + i] : 0.0f;
      if (!a.pre_normalized) v = (v - a.norm.in_mean[i]) / a.norm.in_std[i];
      xs[b * kIn + i] = v;
    }
    for (int j = 0; j < kOut; ++j)
    {
      float v = (b < nb) ? a.Y[(size_t)row * kOut + j] : 0.0f;
      if (!a.pre_normalized) v = (v - a.norm.out_mean[j]) / a.norm.out_std[j];
      dy[b * kOut + j] = v;
    }
  }
  __syncthreads();
  // ---- forward
  for (int e = tid; e < kHid * kSB; e += nt)
  {
    const int j = e / kSB, b = e - j * kSB;
    float acc = W[oB1 + j];
    for (int i = 0; i < kIn; ++i) acc = fmaf(W[oW1 + j * kIn + i], xs[b * kIn + i], acc);
    h1[b * kPad + j] = tanhf(acc);
  }
  __syncthreads();
  for (int e = tid; e < kHid * kSB; e += nt)
  {
    const int j = e / kSB, b = e - j * kSB;
    float acc = W[oB2 + j];
    for (int i = 0; i < kHid; ++i) acc = fmaf(W[oW2 + j * kHid + i], h1[b * kPad + i], acc);
    h2[b * kPad + j] = tanhf(acc);
  }
  __syncthreads();
  float loss = 0.0f;
  for (int e = tid; e < kOut * kSB; e += nt)
  {
    const int j = e / kSB, b = e - j * kSB;
    float acc = W[oB3 + j];
    for (int i = 0; i < kHid; ++i) acc = fmaf(W[oW3 + j * kHid + i], h2[b * kPad + i], acc);
    const float err = acc - dy[b * kOut + j];
    const bool live = b < nb;
    if (live) loss = fmaf(err, err, loss);
    dy[b * kOut + j] = live ? scale * err : 0.0f;
  }
  __syncthreads();
  // ---- backward: dL/dh2 (pre-activation), output-layer gradient
  for (int e = tid; e < kHid * kSB; e += nt)
  {
    const int i = e / kSB, b = e - i * kSB;
    float s = 0.0f;
    for (int j = 0; j < kOut; ++j) s = fmaf(dy[b * kOut + j], W[oW3 + j * kHid + i], s);
    const float h = h2[b * kPad + i];
    d2[b * kPad + i] = s * (1.0f - h * h);
  }
  float* P = a.partials + (size_t)blockIdx.x * kRow;
  for (int e = tid; e < kOut * kHid; e += nt)
  {
    const int j = e / kHid, i = e - j * kHid;
    float s = 0.0f;
    for (int b = 0; b < kSB; ++b) s = fmaf(dy[b * kOut + j], h2[b * kPad + i], s);
    P[oW3 + e] = s;
  }
  if (tid < kOut)
  {
    float s = 0.0f;
    for (int b = 0; b < kSB; ++b) s += dy[b * kOut + tid];
    P[oB3 + tid] = s;
  }
  __syncthreads();
  // dL/dh1 (pre-activation) into the h2 buffer
  for (int e = tid; e < kHid * kSB; e += nt)
  {
    const int i = e / kSB, b = e - i * kSB;
    float s = 0.0f;
    for (int j = 0; j < kHid; ++j) s = fmaf(d2[b * kPad + j], W[oW2 + j * kHid + i], s);
    const float h = h1[b * kPad + i];
    h2[b * kPad + i] = s * (1.0f - h * h);
  }
  for (int e = tid; e < kHid * kHid; e += nt)
  {
    const int j = e / kHid, i = e - j * kHid;
    float s = 0.0f;
    for (int b = 0; b < kSB; ++b) s = fmaf(d2[b * kPad + j], h1[b * kPad + i], s);
    P[oW2 + e] = s;
  }
  if (tid < kHid)
  {
    float s = 0.0f;
    for (int b = 0; b < kSB; ++b) s += d2[b * kPad + tid];
    P[oB2 + tid] = s;
  }
  __syncthreads();
  for (int e = tid; e < kHid * kIn; e += nt)
  {
    const int j = e / kIn, i = e - j * kIn;
    float s = 0.0f;
    for (int b = 0; b < kSB; ++b) s = fmaf(h2[b * kPad + j], xs[b * kIn + i], s);
    P[oW1 + e] = s;
  }
  if (tid < kHid)
  {
    float s = 0.0f;
    for (int b = 0; b < kSB; ++b) s += h2[b * kPad + tid];
    P[oB1 + tid] = s;
  }
  for (int off = 16; off > 0; off >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, off);
  if ((tid & 31) == 0) s_loss[tid >> 5] = loss;
  __syncthreads();
  if (tid == 0)
  {
    float s = 0.0f;
    for (int w = 0; w < (nt >> 5); ++w) s += s_loss[w];
    P[kNW] = s;
  }
}

constexpr size_t kGradSmem = sizeof(float) * (5128 + kSB * kIn + 3 * kSB * kPad + kSB * kOut);

// Sum the partial rows in CTA order; with adam != 0 apply one Adam step, else write the summed gradient.
__global__ void reduce_adam_kernel(float* params, float* m, float* v, const float* partials, int nparts, int batch,
                                   float lr, float beta1, float beta2, float eps, float c1, float c2, int adam,
                                   float* grad_out, float* loss_out)
{
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < kNW)
  {
    float g = 0.0f;
    for (int c = 0; c < nparts; ++c) g += partials[(size_t)c * kRow + p];
    if (adam)
    {
      const float mm = beta1 * m[p] + (1.0f - beta1) * g;
      const float vv = beta2 * v[p] + (1.0f - beta2) * g * g;
      m[p] = mm;
      v[p] = vv;
      params[p] -= lr * (mm * c1) / (sqrtf(vv * c2) + eps);
    }
    else
    {
      grad_out[p] = g;
    }
  }
  if (p == 0 && loss_out)
  {
    float s = 0.0f;
    for (int c = 0; c < nparts; ++c) s += partials[(size_t)c * kRow + kNW];
    *loss_out = s / ((float)batch * kOut);
  }
}

// Squared error per output (physical units) on fresh transitions.
__global__ void validate_kernel(mppi_bicycle_slip_params p, Box box, uint32_t k0, uint32_t k1, int n,
                                const float* params, Norm norm, double* out /* [gridDim][kOut] */)
{
  __shared__ float W[kNW];
  for (int i = threadIdx.x; i < kNW; i += blockDim.x) W[i] = params[i];
  __syncthreads();
  double se[kOut] = {};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
  {
    float x[kIn], y[kOut], h1[kHid], h2[kHid];
    draw_transition(p, box, k0, k1, kValTag, (uint32_t)i, x, y);
    for (int j = 0; j < kIn; ++j) x[j] = (x[j] - norm.in_mean[j]) / norm.in_std[j];
    for (int j = 0; j < kHid; ++j)
    {
      float acc = W[oB1 + j];
      for (int q = 0; q < kIn; ++q) acc = fmaf(W[oW1 + j * kIn + q], x[q], acc);
      h1[j] = tanhf(acc);
    }
    for (int j = 0; j < kHid; ++j)
    {
      float acc = W[oB2 + j];
      for (int q = 0; q < kHid; ++q) acc = fmaf(W[oW2 + j * kHid + q], h1[q], acc);
      h2[j] = tanhf(acc);
    }
    for (int j = 0; j < kOut; ++j)
    {
      float acc = W[oB3 + j];
      for (int q = 0; q < kHid; ++q) acc = fmaf(W[oW3 + j * kHid + q], h2[q], acc);
      const float e = acc * norm.out_std[j] + norm.out_mean[j] - y[j];
      se[j] += (double)e * e;
    }
  }
  __shared__ double red[kOut][32];
  for (int j = 0; j < kOut; ++j)
  {
    double a = se[j];
    for (int off = 16; off > 0; off >>= 1) a += __shfl_xor_sync(0xffffffffu, a, off);
    if ((threadIdx.x & 31) == 0) red[j][threadIdx.x >> 5] = a;
  }
  __syncthreads();
  if (threadIdx.x < kOut)
  {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[threadIdx.x][w];
    out[blockIdx.x * kOut + threadIdx.x] = t;
  }
}

// splitmix64 for the host-side weight initialisation (S. Vigna's published mixer).
uint64_t splitmix64(uint64_t& s)
{
  uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
}  // namespace

class Surrogate
{
public:
  mppi_bicycle_slip_params dyn{};
  mppi_surrogate_config cfg{};
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int num_sms = 1;
  DevBuf<float> X, Y, params, m, v, partials, loss, wscale;
  DevBuf<double> stats;
  std::vector<float> host_params = std::vector<float>(kNP, 0.0f);
  Norm norm{};
  bool generated = false;
  int adam_t = 0;
  int wfmt = 2;  // weight format the training passes see (2: FP32)

  ~Surrogate()
  {
    if (stream) cudaStreamSynchronize(stream);
    if (own_stream && stream) cudaStreamDestroy(stream);
  }

  Box box() const
  {
    Box b;
    for (int j = 0; j < 7; ++j)
    {
      b.lo[j] = cfg.state_lower[j];
      b.hi[j] = cfg.state_upper[j];
    }
    return b;
  }

  mppi_status init()
  {
    MG_CHECK(cfg.num_transitions >= kSB, "num_transitions must be >= %d", kSB);
    for (int j = 0; j < 7; ++j)
      MG_CHECK(std::isfinite(cfg.state_lower[j]) && std::isfinite(cfg.state_upper[j]) &&
                   cfg.state_upper[j] >= cfg.state_lower[j],
               "state bound %d is invalid", j);
    if (!stream)
    {
      MG_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
      own_stream = true;
    }
    int dev = 0;
    MG_CUDA(cudaGetDevice(&dev));
    MG_CUDA(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev));
    MG_CUDA(cudaFuncSetAttribute(grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGradSmem));
    // Xavier-uniform weights, zero biases, identity normalisation until generate() fixes it
    uint64_t s = cfg.seed ^ 0x6a09e667f3bcc909ULL;
    auto fill = [&](int off, int rows, int cols) {
      const double lim = std::sqrt(6.0 / (rows + cols));
      for (int i = 0; i < rows * cols; ++i)
      {
        const double u = (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0);
        host_params[off + i] = (float)((2.0 * u - 1.0) * lim);
      }
    };
    fill(oW1, kHid, kIn);
    fill(oW2, kHid, kHid);
    fill(oW3, kOut, kHid);
    for (int j = 0; j < kIn; ++j)
    {
      host_params[oInMean + j] = 0.0f;
      host_params[oInStd + j] = 1.0f;
    }
    for (int j = 0; j < kOut; ++j)
    {
      host_params[oOutMean + j] = 0.0f;
      host_params[oOutStd + j] = 1.0f;
    }
    MG_TRY(params.alloc(kNP));
    MG_TRY(wscale.alloc(3));
    MG_TRY(m.alloc(kNW));
    MG_TRY(v.alloc(kNW));
    MG_CUDA(cudaMemset(m.p, 0, sizeof(float) * kNW));
    MG_CUDA(cudaMemset(v.p, 0, sizeof(float) * kNW));
    return upload_params();
  }

  mppi_status upload_params()
  {
    for (int j = 0; j < kIn; ++j)
    {
      norm.in_mean[j] = host_params[oInMean + j];
      norm.in_std[j] = host_params[oInStd + j];
    }
    for (int j = 0; j < kOut; ++j)
    {
      norm.out_mean[j] = host_params[oOutMean + j];
      norm.out_std[j] = host_params[oOutStd + j];
    }
    MG_CUDA(cudaMemcpy(params.p, host_params.data(), sizeof(float) * kNP, cudaMemcpyHostToDevice));
    return MPPI_OK;
  }

  mppi_status download_params()
  {
    MG_CUDA(cudaStreamSynchronize(stream));
    MG_CUDA(cudaMemcpy(host_params.data(), params.p, sizeof(float) * kNW, cudaMemcpyDeviceToHost));
    return MPPI_OK;
  }

  mppi_status generate()
  {
    const int n = cfg.num_transitions;
    MG_TRY(X.alloc((size_t)n * kIn));
    MG_TRY(Y.alloc((size_t)n * kOut));
    const int grid = std::min((n + 255) / 256, 4 * num_sms);
    MG_TRY(stats.alloc((size_t)grid * 2 * kOut));
    data_kernel<<<grid, 256, 0, stream>>>(dyn, box(), (uint32_t)cfg.seed, (uint32_t)(cfg.seed >> 32), n, X.p, Y.p,
                                          stats.p);
    MG_CUDA(cudaGetLastError());
    std::vector<double> st((size_t)grid * 2 * kOut);
    MG_CUDA(cudaStreamSynchronize(stream));
    MG_CUDA(cudaMemcpy(st.data(), stats.p, sizeof(double) * st.size(), cudaMemcpyDeviceToHost));
    for (int j = 0; j < kOut; ++j)
    {
      double s1 = 0.0, s2 = 0.0;
      for (int g = 0; g < grid; ++g)
      {
        s1 += st[(size_t)g * 2 * kOut + j];
        s2 += st[(size_t)g * 2 * kOut + kOut + j];
      }
      const double mu = s1 / n;
      const double var = std::max(s2 / n - mu * mu, 1e-12);
      host_params[oOutMean + j] = (float)mu;
      host_params[oOutStd + j] = (float)std::sqrt(var);
    }
    // uniform inputs: mean (lo + hi) / 2, standard deviation (hi - lo) / sqrt(12); controls uniform in [-1, 1]
    for (int j = 0; j < 7; ++j)
    {
      const double lo = cfg.state_lower[j], hi = cfg.state_upper[j];
      host_params[oInMean + j] = (float)(0.5 * (lo + hi));
      host_params[oInStd + j] = hi > lo ? (float)((hi - lo) / std::sqrt(12.0)) : 1.0f;
    }
    // The body-frame derivatives do not depend on position or heading: those inputs get mean 0 and scale 1e30, so
    // they reach the network as (numerically) zero and a rollout that leaves the training box in x / y / yaw never
    // makes the network extrapolate.
    for (int j = 0; j < 3; ++j)
    {
      host_params[oInMean + j] = 0.0f;
      host_params[oInStd + j] = 1e30f;
    }
    for (int j = 7; j < kIn; ++j)
    {
      host_params[oInMean + j] = 0.0f;
      host_params[oInStd + j] = (float)(2.0 / std::sqrt(12.0));
    }
    MG_TRY(download_params());
    MG_TRY(upload_params());
    generated = true;
    return MPPI_OK;
  }

  mppi_status ensure_partials(int batch)
  {
    const int nparts = (batch + kSB - 1) / kSB;
    if (partials.n < (size_t)nparts * kRow) MG_TRY(partials.alloc((size_t)nparts * kRow));
    return MPPI_OK;
  }

  mppi_status train(int steps, int batch, float lr, float lr_final, float* loss_out)
  {
    MG_CHECK(generated, "call mppi_surrogate_generate first");
    MG_CHECK(steps >= 1 && batch >= kSB && batch <= (1 << 20), "steps >= 1 and batch in [%d, 2^20] required", kSB);
    MG_CHECK(lr > 0.0f && lr_final > 0.0f, "learning rates must be positive");
    MG_TRY(ensure_partials(batch));
    MG_TRY(loss.alloc(steps));
    const int nparts = (batch + kSB - 1) / kSB;
    const float decay = std::pow(lr_final / lr, 1.0f / std::max(1, steps - 1));
    const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
    float cur = lr;
    GradArgs a;
    a.params = params.p;
    a.X = X.p;
    a.Y = Y.p;
    a.n = cfg.num_transitions;
    a.batch = batch;
    a.pre_normalized = 0;
    a.k0 = (uint32_t)cfg.seed;
    a.k1 = (uint32_t)(cfg.seed >> 32);
    a.norm = norm;
    a.partials = partials.p;
    a.wfmt = wfmt;
    a.wscale = wscale.p;
    for (int s = 0; s < steps; ++s)
    {
      a.step = (uint32_t)(adam_t + 1);
      if (wfmt == 1) weight_scale_kernel<<<3, 256, 0, stream>>>(params.p, wscale.p);
      grad_kernel<<<nparts, 256, kGradSmem, stream>>>(a);
      ++adam_t;
      const float c1 = 1.0f / (1.0f - std::pow(beta1, (float)adam_t));
      const float c2 = 1.0f / (1.0f - std::pow(beta2, (float)adam_t));
      reduce_adam_kernel<<<(kNW + 255) / 256, 256, 0, stream>>>(params.p, m.p, v.p, partials.p, nparts, batch, cur,
                                                                 beta1, beta2, eps, c1, c2, 1, nullptr, loss.p + s);
      cur *= decay;
    }
    MG_CUDA(cudaGetLastError());
    MG_CUDA(cudaStreamSynchronize(stream));
    if (loss_out) MG_CUDA(cudaMemcpy(loss_out, loss.p, sizeof(float) * steps, cudaMemcpyDeviceToHost));
    return download_params();
  }

  mppi_status gradient(const float* Xh, const float* Yh, int batch, float* grad_out, float* loss_out)
  {
    MG_CHECK(Xh && Yh && grad_out && batch >= 1 && batch <= (1 << 16), "bad gradient-check arguments");
    DevBuf<float> xd, yd, g, l;
    MG_TRY(xd.alloc((size_t)batch * kIn));
    MG_TRY(yd.alloc((size_t)batch * kOut));
    MG_TRY(g.alloc(kNW));
    MG_TRY(l.alloc(1));
    MG_TRY(ensure_partials(batch));
    MG_CUDA(cudaMemcpy(xd.p, Xh, sizeof(float) * batch * kIn, cudaMemcpyHostToDevice));
    MG_CUDA(cudaMemcpy(yd.p, Yh, sizeof(float) * batch * kOut, cudaMemcpyHostToDevice));
    GradArgs a;
    a.params = params.p;
    a.X = xd.p;
    a.Y = yd.p;
    a.n = batch;
    a.batch = batch;
    a.pre_normalized = 1;
    a.k0 = a.k1 = a.step = 0;
    a.norm = norm;
    a.partials = partials.p;
    a.wfmt = wfmt;
    a.wscale = wscale.p;
    const int nparts = (batch + kSB - 1) / kSB;
    if (wfmt == 1) weight_scale_kernel<<<3, 256, 0, stream>>>(params.p, wscale.p);
    grad_kernel<<<nparts, 256, kGradSmem, stream>>>(a);
    reduce_adam_kernel<<<(kNW + 255) / 256, 256, 0, stream>>>(params.p, m.p, v.p, partials.p, nparts, batch, 0.0f,
                                                               0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0, g.p, l.p);
    MG_CUDA(cudaGetLastError());
    MG_CUDA(cudaStreamSynchronize(stream));
    MG_CUDA(cudaMemcpy(grad_out, g.p, sizeof(float) * kNW, cudaMemcpyDeviceToHost));
    if (loss_out) MG_CUDA(cudaMemcpy(loss_out, l.p, sizeof(float), cudaMemcpyDeviceToHost));
    return MPPI_OK;
  }

  mppi_status validate(int n, float* rmse)
  {
    MG_CHECK(n >= 1 && rmse, "n >= 1 and an output array are required");
    const int grid = std::min((n + 255) / 256, 4 * num_sms);
    DevBuf<double> out;
    MG_TRY(out.alloc((size_t)grid * kOut));
    validate_kernel<<<grid, 256, 0, stream>>>(dyn, box(), (uint32_t)cfg.seed, (uint32_t)(cfg.seed >> 32), n,
                                              params.p, norm, out.p);
    MG_CUDA(cudaGetLastError());
    std::vector<double> h((size_t)grid * kOut);
    MG_CUDA(cudaStreamSynchronize(stream));
    MG_CUDA(cudaMemcpy(h.data(), out.p, sizeof(double) * h.size(), cudaMemcpyDeviceToHost));
    for (int j = 0; j < kOut; ++j)
    {
      double s = 0.0;
      for (int g = 0; g < grid; ++g) s += h[(size_t)g * kOut + j];
      rmse[j] = (float)std::sqrt(s / n);
    }
    return MPPI_OK;
  }
};

}  // namespace mg

struct mppi_surrogate
{
  mg::Surrogate* impl;
};

using namespace mg;

extern "C" {

void mppi_default_surrogate_config(mppi_surrogate_config* c)
{
  if (!c) return;
  memset(c, 0, sizeof(*c));
  c->num_transitions = 1 << 20;
  const float lo[7] = { 0.0f, 0.0f, -3.14159265f, 1.0f, -2.0f, -1.5f, -0.5f };
  const float hi[7] = { 51.2f, 51.2f, 3.14159265f, 15.0f, 2.0f, 1.5f, 0.5f };
  for (int j = 0; j < 7; ++j)
  {
    c->state_lower[j] = lo[j];
    c->state_upper[j] = hi[j];
  }
  c->seed = 7;
}

mppi_status mppi_surrogate_create(const mppi_bicycle_slip_params* dyn, const mppi_surrogate_config* cfg, void* stream,
                                  mppi_surrogate** out)
{
  clear_error();
  MG_CHECK(dyn && cfg && out, "arguments must not be NULL");
  *out = nullptr;
  Surrogate* s = new Surrogate();
  s->dyn = *dyn;
  s->cfg = *cfg;
  s->stream = (cudaStream_t)stream;
  mppi_status st = s->init();
  if (st != MPPI_OK)
  {
    delete s;
    return st;
  }
  *out = new mppi_surrogate{ s };
  return MPPI_OK;
}

mppi_status mppi_surrogate_destroy(mppi_surrogate* s)
{
  if (!s) return MPPI_OK;
  delete s->impl;
  delete s;
  return MPPI_OK;
}

#define SUR_OK(s)                                                                                                     \
  do                                                                                                                  \
  {                                                                                                                   \
    if (!(s) || !(s)->impl)                                                                                           \
    {                                                                                                                 \
      set_error("invalid surrogate handle");                                                                          \
      return MPPI_EINVAL;                                                                                             \
    }                                                                                                                 \
  } while (0)

mppi_status mppi_surrogate_generate(mppi_surrogate* s)
{
  SUR_OK(s);
  return s->impl->generate();
}

mppi_status mppi_surrogate_train(mppi_surrogate* s, int steps, int batch, float lr, float lr_final, float* loss_out)
{
  SUR_OK(s);
  return s->impl->train(steps, batch, lr, lr_final, loss_out);
}

mppi_status mppi_surrogate_set_weight_format(mppi_surrogate* s, int precision)
{
  SUR_OK(s);
  MG_CHECK(precision >= 0 && precision <= 2, "weight format must be 0 (bf16), 1 (fp8 e4m3) or 2 (fp32)");
  s->impl->wfmt = precision;
  return MPPI_OK;
}

mppi_status mppi_surrogate_gradient(mppi_surrogate* s, const float* X, const float* Y, int batch, float* grad_out,
                                    float* loss_out)
{
  SUR_OK(s);
  return s->impl->gradient(X, Y, batch, grad_out, loss_out);
}

mppi_status mppi_surrogate_validate(mppi_surrogate* s, int n, float* rmse5)
{
  SUR_OK(s);
  return s->impl->validate(n, rmse5);
}

mppi_status mppi_surrogate_get_params(mppi_surrogate* s, float* out)
{
  SUR_OK(s);
  MG_CHECK(out, "out must not be NULL");
  memcpy(out, s->impl->host_params.data(), sizeof(float) * MPPI_MLP_PARAMS);
  return MPPI_OK;
}

mppi_status mppi_surrogate_set_params(mppi_surrogate* s, const float* in)
{
  SUR_OK(s);
  MG_CHECK(in, "in must not be NULL");
  for (int i = 0; i < MPPI_MLP_PARAMS; ++i) MG_CHECK(std::isfinite(in[i]), "parameter %d is not finite", i);
  memcpy(s->impl->host_params.data(), in, sizeof(float) * MPPI_MLP_PARAMS);
  return s->impl->upload_params();
}

}  // extern "C"
