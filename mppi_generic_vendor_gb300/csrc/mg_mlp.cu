// mg_mlp.cu — tensor-core evaluation of the surrogate MLP: a standalone forward entry point and the rollout kernel of
// the MLP bicycle model (the per-timestep inference over all samples is one BF16 tcgen05 GEMM chain per 128-sample
// tile, FP32 accumulation in TMEM; see mg_mlp.cuh).
#include <algorithm>
#include <cmath>

#include "mg_common.cuh"
#include "mg_mlp.cuh"

namespace mg
{
namespace
{
// Every CTA of the MLP kernels allocates MlpSmem::TMEM_COLS = 256 TMEM columns; requesting at least this much
// shared memory keeps two CTAs per SM at most, so allocation never waits on another CTA's columns.
constexpr size_t kMlpMinSmem = 100 * 1024;

__global__ void __launch_bounds__(128) mlp_forward_kernel(const float* params, const float* X, float* Y, int B,
                                                          unsigned int* status)
{
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t s_tmem;
  const int tid = threadIdx.x, warp = tid >> 5;
  if (warp == 0)
  {
    tmem_alloc(&s_tmem, MlpSmem::TMEM_COLS);
    tmem_relinquish();
  }
  if (tid == 0)
  {
    mbar_init(&mbar, 1);
    fence_mbarrier_init();
  }
  mlp_load_weights(sm, params);
  tc_fence_before_sync();
  __syncthreads();
  tc_fence_after_sync();
  const uint32_t taddr = s_tmem;
  uint32_t phase = 0;
  const float* nrm = reinterpret_cast<const float*>(sm + MlpSmem::NORM);
  for (int tile = blockIdx.x; tile * 128 < B; tile += gridDim.x)
  {
    const int row = tile * 128 + tid;
    float x[kMlpIn], y[kMlpOut];
#pragma unroll
    for (int i = 0; i < kMlpIn; ++i) x[i] = row < B ? (X[(size_t)row * kMlpIn + i] - nrm[i]) / nrm[9 + i] : 0.0f;
    if (!mlp_tile_forward(sm, taddr, &mbar, phase, x, y))
    {
      if (tid == 0) atomicOr(status, 1u);
      break;
    }
    if (row < B)
#pragma unroll
      for (int j = 0; j < kMlpOut; ++j) Y[(size_t)row * kMlpOut + j] = y[j] * nrm[23 + j] + nrm[18 + j];
  }
  tc_fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(taddr, MlpSmem::TMEM_COLS);
}

// Surrogate rollout: BicycleSlipModel with the (yaw, vx, vy, yaw_rate, steer) derivatives from the MLP and the
// x / y rows analytic (NeuralNetModel::computeKinematics, ar_nn_model.cu:119-124).  One persistent CTA per SM slot
// walks 128-sample tiles; the Euler step, the costmap cost and the likelihood term follow rolloutKernel
// (mppi_common.cu:105-152) exactly as the analytic rollout does.
__global__ void __launch_bounds__(128) rollout_mlp_kernel(const __grid_constant__ RolloutArgs<BicycleSlipMLPModel> a,
                                                          const float* mlp)
{
  using Model = BicycleSlipMLPModel;
  constexpr int S = Model::STATE_DIM, C = Model::CONTROL_DIM;
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t s_tmem;
  __shared__ int s_tile;
  __shared__ unsigned int s_min;
  const int tid = threadIdx.x, warp = tid >> 5;
  if (warp == 0)
  {
    tmem_alloc(&s_tmem, MlpSmem::TMEM_COLS);
    tmem_relinquish();
  }
  if (tid == 0)
  {
    mbar_init(&mbar, 1);
    fence_mbarrier_init();
  }
  mlp_load_weights(sm, mlp);
  tc_fence_before_sync();
  __syncthreads();
  tc_fence_after_sync();
  const uint32_t taddr = s_tmem;
  uint32_t phase = 0;
  const float* nrm = reinterpret_cast<const float*>(sm + MlpSmem::NORM);
  bool ok = true;
  for (;;)
  {
    if (tid == 0)
    {
      s_tile = (int)atomicAdd(&a.tile_counter[0], 1u);
      s_min = kOrderedPosInf;
    }
    __syncthreads();
    const int tile = s_tile;
    if (tile >= a.num_tiles) break;
    const int2 w = a.tiles[tile];
    const InstDesc d = a.inst[w.x];
    const int k = w.y + tid;
    const bool active = k < d.K;
    const typename Model::CostParams& cp = a.cost[w.x];
    const float* urow = a.samples + d.u_off + (long long)(active ? k : w.y) * d.T * C;
    float x[S];
#pragma unroll
    for (int i = 0; i < S; ++i) x[i] = a.x0[d.x_off + i];
    float running = 0.0f;
    float2 u_next = active ? __ldg(reinterpret_cast<const float2*>(urow)) : make_float2(0.0f, 0.0f);
    for (int t = 0; t < d.T && ok; ++t)
    {
      const float u[2] = { u_next.x, u_next.y };
      if (active && t + 1 < d.T) u_next = __ldg(reinterpret_cast<const float2*>(urow + (t + 1) * C));
      float xin[kMlpIn], y[kMlpOut];
#pragma unroll
      for (int i = 0; i < S; ++i) xin[i] = (x[i] - nrm[i]) / nrm[9 + i];
      xin[7] = (u[0] - nrm[7]) / nrm[16];
      xin[8] = (u[1] - nrm[8]) / nrm[17];
      ok = mlp_tile_forward(sm, taddr, &mbar, phase, xin, y);
      if (!ok) break;
      float xd[S];
      float sy, cy;
      sincos_f(x[2], &sy, &cy);
      xd[0] = x[3] * cy - x[4] * sy;
      xd[1] = x[3] * sy + x[4] * cy;
#pragma unroll
      for (int j = 0; j < kMlpOut; ++j) xd[2 + j] = y[j] * nrm[23 + j] + nrm[18 + j];
      float xn[S];
#pragma unroll
      for (int i = 0; i < S; ++i) xn[i] = fmaf(xd[i], a.dt, x[i]);
      if (active)
      {
        float step_cost = Model::computeStateCost(cp, a.aux, xn, t) + Model::computeControlCost(cp, u, t);
        if (a.use_likelihood)
        {
          const bool zero_mean = (float)k >= (1.0f - a.sh.pure_pct) * (float)d.K;
          float lc = 0.0f;
#pragma unroll
          for (int c = 0; c < C; ++c)
          {
            const float m = zero_mean ? 0.0f : a.mean[d.t_off + t * C + c];
            const float sd = a.sh.std_dev[c];
            lc += a.sh.control_cost_coeff[c] * m * (m - 2.0f * u[c]) / (sd * sd);
          }
          step_cost += 0.5f * a.lambda * (1.0f - a.alpha) * lc;
        }
        running += step_cost;
      }
#pragma unroll
      for (int i = 0; i < S; ++i) x[i] = xn[i];
    }
    if (!ok)
    {
      if (tid == 0) atomicOr(a.status, 1u);
      break;
    }
    unsigned int o = kOrderedPosInf;
    if (active)
    {
      const float tf = (float)d.T;
      const float cost = running / tf + Model::terminalCost(cp, a.aux, x) / tf;
      a.costs[d.k_off + k] = cost;
      o = float_to_ordered(cost);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) o = min(o, __shfl_xor_sync(0xffffffffu, o, off));
    if ((tid & 31) == 0) atomicMin(&s_min, o);
    __syncthreads();
    if (tid == 0) atomicMin(&a.baseline_bits[w.x], s_min);
  }
  tc_fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(taddr, MlpSmem::TMEM_COLS);
  if (tid == 0)
  {
    __threadfence();
    const unsigned int done = atomicAdd(&a.tile_counter[1], 1u);
    if (done == gridDim.x - 1)
    {
      a.tile_counter[0] = 0u;
      a.tile_counter[1] = 0u;
      __threadfence();
    }
  }
}
}  // namespace

mppi_status launch_mlp_rollout(const RolloutArgs<BicycleSlipMLPModel>& a, const float* mlp_d, int num_sms,
                               cudaStream_t s)
{
  const size_t smem = kMlpMinSmem;
  MG_CUDA(cudaFuncSetAttribute(rollout_mlp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int grid = std::max(1, std::min(a.num_tiles, 2 * num_sms));
  rollout_mlp_kernel<<<grid, 128, smem, s>>>(a, mlp_d);
  MG_CUDA(cudaGetLastError());
  return MPPI_OK;
}

}  // namespace mg

using namespace mg;

extern "C" {

mppi_status mppi_kernel_mlp_forward(const float* params, const float* X_d, float* Y_d, int batch, void* stream)
{
  clear_error();
  MG_CHECK(params && X_d && Y_d, "pointers must not be NULL");
  MG_CHECK(batch >= 1, "batch must be >= 1");
  for (int i = 0; i < MPPI_MLP_PARAMS; ++i) MG_CHECK(std::isfinite(params[i]), "parameter %d is not finite", i);
  for (int i = 0; i < kMlpIn; ++i) MG_CHECK(params[kMlpInStd + i] > 0.0f, "input scale %d must be positive", i);
  cudaStream_t s = (cudaStream_t)stream;
  void* buf = nullptr;
  const size_t bytes = sizeof(float) * MPPI_MLP_PARAMS + 256;
  cudaError_t e = cudaMallocAsync(&buf, bytes, s);
  if (e != cudaSuccess)
  {
    set_error("cudaMallocAsync failed: %s", cudaGetErrorString(e));
    return MPPI_ENOMEM;
  }
  float* p_d = (float*)buf;
  unsigned int* status = (unsigned int*)((char*)buf + sizeof(float) * MPPI_MLP_PARAMS + 128);
  mppi_status st = MPPI_OK;
  do
  {
    if ((e = cudaMemcpyAsync(p_d, params, sizeof(float) * MPPI_MLP_PARAMS, cudaMemcpyHostToDevice, s)) != cudaSuccess)
      break;
    if ((e = cudaMemsetAsync(status, 0, sizeof(unsigned int), s)) != cudaSuccess) break;
    if ((e = cudaFuncSetAttribute(mlp_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kMlpMinSmem)) != cudaSuccess)
      break;
    const int tiles = (batch + 127) / 128;
    mlp_forward_kernel<<<std::min(tiles, 1024), 128, kMlpMinSmem, s>>>(p_d, X_d, Y_d, batch, status);
    if ((e = cudaGetLastError()) != cudaSuccess) break;
    unsigned int h = 0;
    if ((e = cudaMemcpyAsync(&h, status, sizeof(h), cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) break;
    if (h)
    {
      set_error("a bounded wait for the tensor cores gave up");
      st = MPPI_ETIMEOUT;
    }
  } while (0);
  cudaFreeAsync(buf, s);
  if (e != cudaSuccess)
  {
    set_error("CUDA failure in mppi_kernel_mlp_forward: %s", cudaGetErrorString(e));
    return MPPI_ECUDA;
  }
  return st;
}

}  // extern "C"
