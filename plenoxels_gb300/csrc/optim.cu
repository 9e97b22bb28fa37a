// The optimiser side of the reference's training step (scripts/train.py): the TV loss
// (:44-65, :163-168), Adam (:89, :182) and the |grad| accumulator (:184), as streaming
// passes over the dense [X,Y,Z,4] grid.
//
//  pgb_tv_sumsq  Q = sum over axis-neighbour pairs of (v_i - v_j)^2 (one deterministic
//                reduction: fp32 per thread over a fixed cell range, fp64 per block, the
//                last block sums the blocks in order)
//  pgb_tv_grad   grad += w / sqrt(Q) * sum_{j in N(i)} (v_i - v_j), the gradient of w*sqrt(Q)
//  pgb_adam_step torch.optim.Adam's update (lerp of the first moment, bias corrections),
//                accum += |grad|, grad = 0, in one pass
//  pgb_adam_tv_step  the two passes above fused: Adam on grad + the TV gradient, written
//                to a second parameter buffer
#include <algorithm>
#include <cmath>

#include "pgb_host.h"
#include "pgb_device.cuh"

namespace pgb {
namespace {

constexpr int kTvThreads = 256;
constexpr int kTvMaxBlocks = 1 << 18;

__device__ __forceinline__ float sq4(float4 a, float4 b) {
  const float x = a.x - b.x, y = a.y - b.y, z = a.z - b.z, w = a.w - b.w;
  return x * x + y * y + z * z + w * w;
}

// Block (bz, y, xc) covers z in [bz*T, bz*T + T) of row y and the run of consecutive x
// values xc*XL .. xc*XL + XL - 1, so the x-neighbours come from the previous and next
// iteration's registers; no integer division per cell, coalesced along z.
constexpr int kTvXChunks = 8;  // x-runs per (z-block, y) row: measured best against 3, 16, 32

__global__ void __launch_bounds__(kTvThreads) tv_sumsq_kernel(const float4* __restrict__ v, int X, int Y,
                                                              int Z, double* __restrict__ partials,
                                                              unsigned* __restrict__ counter,
                                                              double* __restrict__ out) {
  const int z = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  const int64_t YZ = (int64_t)Y * Z;
  const int XL = (X + gridDim.z - 1) / gridDim.z;
  const int x0 = blockIdx.z * XL, x1 = min(X, x0 + XL);
  // fp32 runs of at most 32 cells folded into a TwoSum pair; the block and the grid then
  // sum pairs (GB300's fp64 rate is low: fp64 sums made this pass fp64-bound)
  LossSum<float> acc_s;
  if (z < Z && x0 < x1) {
    float acc = 0.f;
    int64_t i = (int64_t)x0 * YZ + (int64_t)y * Z + z;
    float4 c = __ldg(v + i);
    for (int x = x0; x < x1; ++x, i += YZ) {
      if (z + 1 < Z) acc += sq4(c, __ldg(v + i + 1));
      if (y + 1 < Y) acc += sq4(c, __ldg(v + i + Z));
      float4 nx = c;
      if (x + 1 < X) {
        nx = __ldg(v + i + YZ);
        acc += sq4(c, nx);
      }
      c = nx;
      if (((x - x0) & 31) == 31) {  // bound the fp32 run
        acc_s.add(acc);
        acc = 0.f;
      }
    }
    acc_s.add(acc);
  }
  // block: warps in warp order (kTvThreads / 32 warp partials), one pair per block
  __shared__ double red[kTvThreads / 32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  acc_s = warp_sum(acc_s);
  if (lane == 0) acc_s.store(&red[wid]);
  __syncthreads();
  const unsigned nblocks = gridDim.x * gridDim.y * gridDim.z;
  const unsigned bid = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
  if (threadIdx.x == 0) {
    LossSum<float> b;
    for (int w = 0; w < kTvThreads / 32; ++w) b.add(LossSum<float>::load_volatile(&red[w]));
    b.store(partials + bid);
    __threadfence();
    last = atomicAdd(counter, 1u) == nblocks - 1u;
  }
  __syncthreads();
  if (last) {
    // the block pairs, thread-strided, then the warps in order
    __threadfence();
    LossSum<float> t;
    for (unsigned b = threadIdx.x; b < nblocks; b += blockDim.x) t.add(LossSum<float>::load_cg(partials + b));
    t = warp_sum(t);
    __syncthreads();
    if (lane == 0) t.store(&red[wid]);
    __syncthreads();
    if (threadIdx.x == 0) {
      LossSum<float> total;
      for (int w = 0; w < kTvThreads / 32; ++w) total.add(LossSum<float>::load_volatile(&red[w]));
      out[0] = total.value();
      *counter = 0u;
    }
  }
}

// weight / sqrt(q) for the TV gradient, in fp32 arithmetic as the reference takes the TV
// norm (torch.sqrt of an fp32 sum; scripts/train.py:62); 0 when q is not positive (a
// constant grid: sqrt is not differentiable at 0). One conversion from the double sum and
// no other fp64 work per thread.
__device__ __forceinline__ float tv_scale(double q, float weight) {
  const float qf = (float)q;
  return qf > 0.f ? __fdiv_rn(weight, __fsqrt_rn(qf)) : 0.f;
}

__global__ void __launch_bounds__(kTvThreads) tv_grad_kernel(const float4* __restrict__ v, int X, int Y,
                                                             int Z, const double* __restrict__ sumsq,
                                                             float weight, float4* __restrict__ grad) {
  const float c = tv_scale(sumsq[0], weight);
  if (c == 0.f) return;  // no TV weight, or a constant grid
  const int z = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  const int XL = (X + gridDim.z - 1) / gridDim.z;
  const int x0 = blockIdx.z * XL, x1 = min(X, x0 + XL);
  if (z >= Z || x0 >= x1) return;
  const int64_t YZ = (int64_t)Y * Z;
  int64_t i = (int64_t)x0 * YZ + (int64_t)y * Z + z;
  float4 prev = x0 > 0 ? __ldg(v + i - YZ) : make_float4(0.f, 0.f, 0.f, 0.f);
  float4 m = __ldg(v + i);
  for (int x = x0; x < x1; ++x, i += YZ) {
    const float4 next = x + 1 < X ? __ldg(v + i + YZ) : m;
    float4 d = make_float4(0.f, 0.f, 0.f, 0.f);
    auto add = [&](float4 nb) {
      d.x += m.x - nb.x; d.y += m.y - nb.y; d.z += m.z - nb.z; d.w += m.w - nb.w;
    };
    if (z > 0) add(__ldg(v + i - 1));
    if (z + 1 < Z) add(__ldg(v + i + 1));
    if (y > 0) add(__ldg(v + i - Z));
    if (y + 1 < Y) add(__ldg(v + i + Z));
    if (x > 0) add(prev);
    if (x + 1 < X) add(next);
    float4 g = grad[i];
    g.x += c * d.x; g.y += c * d.y; g.z += c * d.z; g.w += c * d.w;
    grad[i] = g;
    prev = m;
    m = next;
  }
}

struct AdamConst {
  float one_minus_b1, b2, one_minus_b2, step_size, inv_bc2_sqrt, eps;
};

__device__ __forceinline__ float adam_one(float& p, float g, float& m, float& s, const AdamConst& k) {
  m = m + k.one_minus_b1 * (g - m);        // exp_avg.lerp_(grad, 1 - beta1)
  s = s * k.b2 + k.one_minus_b2 * g * g;   // exp_avg_sq.mul_(beta2).addcmul_(grad, grad, 1 - beta2)
  const float denom = sqrtf(s) * k.inv_bc2_sqrt + k.eps;
  p = p - k.step_size * (m / denom);
  return fabsf(g);
}

__global__ void adam_kernel(float4* __restrict__ p, float4* __restrict__ g, float4* __restrict__ m,
                            float4* __restrict__ s, float4* __restrict__ acc, int64_t n4,
                            AdamConst k, int zero_grad) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4;
       i += (int64_t)gridDim.x * blockDim.x) {
    float4 P = p[i], Gr = g[i], M = m[i], S = s[i];
    float4 A = make_float4(0.f, 0.f, 0.f, 0.f);
    A.x = adam_one(P.x, Gr.x, M.x, S.x, k);
    A.y = adam_one(P.y, Gr.y, M.y, S.y, k);
    A.z = adam_one(P.z, Gr.z, M.z, S.z, k);
    A.w = adam_one(P.w, Gr.w, M.w, S.w, k);
    p[i] = P;
    m[i] = M;
    s[i] = S;
    if (acc) {
      float4 a = acc[i];
      a.x += A.x; a.y += A.y; a.z += A.z; a.w += A.w;
      acc[i] = a;
    }
    if (zero_grad) g[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

// Adam with the TV gradient added on the fly: the tv_grad_kernel stencil (same neighbour
// order, same fp32 expression) feeding adam_one, over the (z-blocks, Y, x-chunks) grid of
// the TV kernels. Neighbours are read from pin while cells are updated, so the update goes
// to pout (a different buffer): one pass instead of the TV gradient's read-modify-write of
// grad followed by Adam.
__global__ void __launch_bounds__(kTvThreads) adam_tv_kernel(
    const float4* __restrict__ pin, float4* __restrict__ pout, float4* __restrict__ g,
    float4* __restrict__ mo, float4* __restrict__ so, float4* __restrict__ acc, int X, int Y,
    int Z, const double* __restrict__ sumsq, float weight, AdamConst k, int zero_grad) {
  const float c = tv_scale(sumsq[0], weight);
  const bool tv = c != 0.f;  // no TV weight, or a constant grid (as tv_grad_kernel)
  const int z = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y;
  const int XL = (X + gridDim.z - 1) / gridDim.z;
  const int x0 = blockIdx.z * XL, x1 = min(X, x0 + XL);
  if (z >= Z || x0 >= x1) return;
  const int64_t YZ = (int64_t)Y * Z;
  int64_t i = (int64_t)x0 * YZ + (int64_t)y * Z + z;
  float4 prev = x0 > 0 ? __ldg(pin + i - YZ) : make_float4(0.f, 0.f, 0.f, 0.f);
  float4 m = __ldg(pin + i);
  for (int x = x0; x < x1; ++x, i += YZ) {
    const float4 next = x + 1 < X ? __ldg(pin + i + YZ) : m;
    float4 Gr = g[i];
    if (tv) {
      float4 d = make_float4(0.f, 0.f, 0.f, 0.f);
      auto add = [&](float4 nb) {
        d.x += m.x - nb.x; d.y += m.y - nb.y; d.z += m.z - nb.z; d.w += m.w - nb.w;
      };
      if (z > 0) add(__ldg(pin + i - 1));
      if (z + 1 < Z) add(__ldg(pin + i + 1));
      if (y > 0) add(__ldg(pin + i - Z));
      if (y + 1 < Y) add(__ldg(pin + i + Z));
      if (x > 0) add(prev);
      if (x + 1 < X) add(next);
      Gr.x += c * d.x; Gr.y += c * d.y; Gr.z += c * d.z; Gr.w += c * d.w;
    }
    float4 P = m, M = mo[i], S = so[i];
    float4 A;
    A.x = adam_one(P.x, Gr.x, M.x, S.x, k);
    A.y = adam_one(P.y, Gr.y, M.y, S.y, k);
    A.z = adam_one(P.z, Gr.z, M.z, S.z, k);
    A.w = adam_one(P.w, Gr.w, M.w, S.w, k);
    pout[i] = P;
    mo[i] = M;
    so[i] = S;
    if (acc) {
      float4 a = acc[i];
      a.x += A.x; a.y += A.y; a.z += A.z; a.w += A.w;
      acc[i] = a;
    }
    if (zero_grad) g[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    prev = m;
    m = next;
  }
}

AdamConst adam_const(double lr, double beta1, double beta2, double eps, int64_t step) {
  // torch.optim.Adam (non-capturable path): bias corrections in double on the host
  const double bc1 = 1.0 - std::pow(beta1, (double)step);
  const double bc2 = 1.0 - std::pow(beta2, (double)step);
  AdamConst k;
  k.one_minus_b1 = (float)(1.0 - beta1);
  k.b2 = (float)beta2;
  k.one_minus_b2 = (float)(1.0 - beta2);
  k.step_size = (float)(lr / bc1);
  k.inv_bc2_sqrt = (float)(1.0 / std::sqrt(bc2));
  k.eps = (float)eps;
  return k;
}

inline unsigned stream_blocks(int64_t n) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16));
}

inline bool al16(const void* p) { return ((uintptr_t)p % 16) == 0; }

}  // namespace
}  // namespace pgb

using namespace pgb;

extern "C" {

// partial sums: one per block of the (z-blocks, Y, kTvXChunks) grid
int64_t pgb_tv_workspace_bytes(void) { return (int64_t)sizeof(double) * kTvMaxBlocks + 256; }

int pgb_tv_sumsq(const float* cells, const int32_t dims[3], double* sumsq_out, void* workspace,
                 pgb_stream_t stream) {
  if (!cells || !dims || !sumsq_out || !workspace) return PGB_ERR_ARG;
  if (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return PGB_ERR_ARG;
  if (!al16(cells) || !al16(workspace)) return PGB_ERR_ALIGN;
  if (dims[1] > 65535) return PGB_ERR_UNSUPPORTED;
  const dim3 grid((dims[2] + kTvThreads - 1) / kTvThreads, dims[1], std::min(dims[0], kTvXChunks));
  if ((int64_t)grid.x * grid.y * grid.z > kTvMaxBlocks) return PGB_ERR_UNSUPPORTED;
  tv_sumsq_kernel<<<grid, kTvThreads, 0, stream>>>(
      reinterpret_cast<const float4*>(cells), dims[0], dims[1], dims[2], (double*)workspace,
      (unsigned*)((char*)workspace + sizeof(double) * kTvMaxBlocks), sumsq_out);
  return after_launch();
}

int pgb_tv_grad(const float* cells, const int32_t dims[3], const double* sumsq, float weight,
                float* grad_cells, pgb_stream_t stream) {
  if (!cells || !dims || !sumsq || !grad_cells) return PGB_ERR_ARG;
  if (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return PGB_ERR_ARG;
  if (!al16(cells) || !al16(grad_cells)) return PGB_ERR_ALIGN;
  if (dims[1] > 65535) return PGB_ERR_UNSUPPORTED;
  const dim3 grid((dims[2] + kTvThreads - 1) / kTvThreads, dims[1], std::min(dims[0], kTvXChunks));
  tv_grad_kernel<<<grid, kTvThreads, 0, stream>>>(reinterpret_cast<const float4*>(cells), dims[0], dims[1],
                                                  dims[2], sumsq, weight, reinterpret_cast<float4*>(grad_cells));
  return after_launch();
}

int pgb_adam_step(float* param, float* grad, float* exp_avg, float* exp_avg_sq, float* abs_grad_accum,
                  int64_t count, double lr, double beta1, double beta2, double eps, int64_t step,
                  int32_t zero_grad, pgb_stream_t stream) {
  if (count < 0 || step < 1) return PGB_ERR_ARG;
  if (count == 0) return PGB_OK;
  if (!param || !grad || !exp_avg || !exp_avg_sq) return PGB_ERR_ARG;
  if (count % 4 != 0) return PGB_ERR_UNSUPPORTED;
  if (!al16(param) || !al16(grad) || !al16(exp_avg) || !al16(exp_avg_sq) ||
      (abs_grad_accum && !al16(abs_grad_accum)))
    return PGB_ERR_ALIGN;
  const AdamConst k = adam_const(lr, beta1, beta2, eps, step);
  const int64_t n4 = count / 4;
  adam_kernel<<<stream_blocks(n4), 256, 0, stream>>>(
      reinterpret_cast<float4*>(param), reinterpret_cast<float4*>(grad),
      reinterpret_cast<float4*>(exp_avg), reinterpret_cast<float4*>(exp_avg_sq),
      reinterpret_cast<float4*>(abs_grad_accum), n4, k, zero_grad ? 1 : 0);
  return after_launch();
}

int pgb_adam_tv_step(const float* param_in, float* param_out, float* grad, float* exp_avg,
                     float* exp_avg_sq, float* abs_grad_accum, const int32_t dims[3],
                     const double* tv_sumsq, float tv_weight, double lr, double beta1, double beta2,
                     double eps, int64_t step, int32_t zero_grad, pgb_stream_t stream) {
  if (!dims || step < 1) return PGB_ERR_ARG;
  if (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return PGB_ERR_ARG;
  if (!param_in || !param_out || !grad || !exp_avg || !exp_avg_sq || !tv_sumsq) return PGB_ERR_ARG;
  if (param_in == param_out) return PGB_ERR_ARG;  // neighbours are read while cells are updated
  if (!al16(param_in) || !al16(param_out) || !al16(grad) || !al16(exp_avg) || !al16(exp_avg_sq) ||
      (abs_grad_accum && !al16(abs_grad_accum)))
    return PGB_ERR_ALIGN;
  if (dims[1] > 65535) return PGB_ERR_UNSUPPORTED;
  const AdamConst k = adam_const(lr, beta1, beta2, eps, step);
  const dim3 grid((dims[2] + kTvThreads - 1) / kTvThreads, dims[1], std::min(dims[0], kTvXChunks));
  adam_tv_kernel<<<grid, kTvThreads, 0, stream>>>(
      reinterpret_cast<const float4*>(param_in), reinterpret_cast<float4*>(param_out),
      reinterpret_cast<float4*>(grad), reinterpret_cast<float4*>(exp_avg),
      reinterpret_cast<float4*>(exp_avg_sq), reinterpret_cast<float4*>(abs_grad_accum), dims[0],
      dims[1], dims[2], tv_sumsq, tv_weight, k, zero_grad ? 1 : 0);
  return after_launch();
}

}  // extern "C"
