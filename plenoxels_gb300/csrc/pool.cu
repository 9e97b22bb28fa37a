// Average pooling of the grid for coarse-to-fine training (src/grid_functions.py:173-181,
// average_pool3d_grid: avg_pool3d of the channels-last grid with a cubic window of r
// cells and stride s, no padding), and its adjoint.
//
// The window sum is separable, so both directions run as three 1-D passes over the
// channels-last layout (z, then y, then x forward; x, then y, then z backward), each
// thread producing one float4 cell. The last backward pass writes every cell of the full
// gradient (cells under no window get 0), so it also clears it.
#include <algorithm>

#include "pgb_host.h"
#include "pgb_device.cuh"

namespace pgb {
namespace {

inline unsigned blocks_of(int64_t n) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 1 << 20));
}

// out[a, o, b] = scale * sum_{k<r} in[a, o*s + k, b] for a [A, N, B] float4 view
__global__ void pool_axis_kernel(const float4* __restrict__ in, float4* __restrict__ out, int64_t A,
                                 int N, int64_t B, int No, int r, int s, float scale) {
  const int64_t total = A * No * B;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i % B;
    const int64_t ao = i / B;
    const int o = (int)(ao % No);
    const int64_t a = ao / No;
    const float4* p = in + (a * N + (int64_t)o * s) * B + b;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int k = 0; k < r; ++k) {
      const float4 v = __ldg(p + (int64_t)k * B);
      acc.x += v.x; acc.y += v.y; acc.z += v.z; acc.w += v.w;
    }
    acc.x *= scale; acc.y *= scale; acc.z *= scale; acc.w *= scale;
    out[i] = acc;
  }
}

// adjoint of pool_axis: din[a, n, b] = scale * sum over windows o containing n of dout[a, o, b]
__global__ void unpool_axis_kernel(const float4* __restrict__ dout, float4* __restrict__ din, int64_t A,
                                   int N, int64_t B, int No, int r, int s, float scale) {
  const int64_t total = A * N * B;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i % B;
    const int64_t an = i / B;
    const int n = (int)(an % N);
    const int64_t a = an / N;
    // windows o with o*s <= n < o*s + r
    const int hi = min(No - 1, n / s);
    const int lo = n - r + 1 <= 0 ? 0 : (n - r + 1 + s - 1) / s;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int o = lo; o <= hi; ++o) {
      const float4 v = __ldg(dout + (a * No + o) * B + b);
      acc.x += v.x; acc.y += v.y; acc.z += v.z; acc.w += v.w;
    }
    acc.x *= scale; acc.y *= scale; acc.z *= scale; acc.w *= scale;
    din[i] = acc;
  }
}

int out_size(int n, int r, int s) { return n < r ? 0 : (n - r) / s + 1; }

}  // namespace
}  // namespace pgb

using namespace pgb;

extern "C" {

int pgb_avg_pool3d_shape(const int32_t dims[3], int32_t window, int32_t stride, int32_t out_dims[3],
                         int64_t* scratch_bytes) {
  if (!dims || !out_dims || window < 1 || stride < 1) return PGB_ERR_ARG;
  for (int a = 0; a < 3; ++a) {
    if (dims[a] <= 0) return PGB_ERR_ARG;
    out_dims[a] = out_size(dims[a], window, stride);
    if (out_dims[a] <= 0) return PGB_ERR_UNSUPPORTED;  // window larger than the grid
  }
  if (scratch_bytes) {
    // two intermediates: [X,Y,Zo,4] and [X,Yo,Zo,4] floats
    const int64_t t1 = (int64_t)dims[0] * dims[1] * out_dims[2] * 16;
    const int64_t t2 = (int64_t)dims[0] * out_dims[1] * out_dims[2] * 16;
    *scratch_bytes = ((t1 + 255) / 256) * 256 + t2;
  }
  return PGB_OK;
}

int pgb_avg_pool3d_fwd(const float* cells, const int32_t dims[3], int32_t window, int32_t stride,
                       void* scratch, float* out, pgb_stream_t s) {
  int32_t od[3];
  int64_t bytes = 0;
  int st = pgb_avg_pool3d_shape(dims, window, stride, od, &bytes);
  if (st) return st;
  if (!cells || !scratch || !out) return PGB_ERR_ARG;
  if (((uintptr_t)cells | (uintptr_t)scratch | (uintptr_t)out) % 16) return PGB_ERR_ALIGN;
  const int X = dims[0], Y = dims[1], Z = dims[2];
  float4* t1 = reinterpret_cast<float4*>(scratch);
  float4* t2 = reinterpret_cast<float4*>((char*)scratch +
                                         (((int64_t)X * Y * od[2] * 16 + 255) / 256) * 256);
  const float inv = 1.0f / ((float)window * (float)window * (float)window);
  pool_axis_kernel<<<blocks_of((int64_t)X * Y * od[2]), 256, 0, s>>>(
      reinterpret_cast<const float4*>(cells), t1, (int64_t)X * Y, Z, 1, od[2], window, stride, 1.f);
  if ((st = after_launch())) return st;
  pool_axis_kernel<<<blocks_of((int64_t)X * od[1] * od[2]), 256, 0, s>>>(
      t1, t2, X, Y, od[2], od[1], window, stride, 1.f);
  if ((st = after_launch())) return st;
  pool_axis_kernel<<<blocks_of((int64_t)od[0] * od[1] * od[2]), 256, 0, s>>>(
      t2, reinterpret_cast<float4*>(out), 1, X, (int64_t)od[1] * od[2], od[0], window, stride, inv);
  return after_launch();
}

int pgb_avg_pool3d_bwd(const float* d_out, const int32_t dims[3], int32_t window, int32_t stride,
                       void* scratch, float* d_cells, pgb_stream_t s) {
  int32_t od[3];
  int64_t bytes = 0;
  int st = pgb_avg_pool3d_shape(dims, window, stride, od, &bytes);
  if (st) return st;
  if (!d_out || !scratch || !d_cells) return PGB_ERR_ARG;
  if (((uintptr_t)d_out | (uintptr_t)scratch | (uintptr_t)d_cells) % 16) return PGB_ERR_ALIGN;
  const int X = dims[0], Y = dims[1], Z = dims[2];
  float4* t1 = reinterpret_cast<float4*>(scratch);  // [X,Y,Zo]
  float4* t2 = reinterpret_cast<float4*>((char*)scratch +
                                         (((int64_t)X * Y * od[2] * 16 + 255) / 256) * 256);  // [X,Yo,Zo]
  const float inv = 1.0f / ((float)window * (float)window * (float)window);
  unpool_axis_kernel<<<blocks_of((int64_t)X * od[1] * od[2]), 256, 0, s>>>(
      reinterpret_cast<const float4*>(d_out), t2, 1, X, (int64_t)od[1] * od[2], od[0], window, stride, inv);
  if ((st = after_launch())) return st;
  unpool_axis_kernel<<<blocks_of((int64_t)X * Y * od[2]), 256, 0, s>>>(
      t2, t1, X, Y, od[2], od[1], window, stride, 1.f);
  if ((st = after_launch())) return st;
  unpool_axis_kernel<<<blocks_of((int64_t)X * Y * Z), 256, 0, s>>>(
      t1, reinterpret_cast<float4*>(d_cells), (int64_t)X * Y, Z, 1, od[2], window, stride, 1.f);
  return after_launch();
}

}  // extern "C"
