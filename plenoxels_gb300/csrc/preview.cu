// Grid previews and clean-up outside the render path:
//  - the point-splat preview of src/visualization.py:157-232 (visulize_3d_in_2d_fast):
//    every cell with alpha above a floor projects to a pixel; the nearest one paints it
//    (the reference sorts far to near and lets the last write win), white elsewhere;
//  - the stray-voxel clean-up of src/grid_functions.py:260-280
//    (convolve_grid_to_remove_noise): repeatedly, the alpha of each cell's neighbours
//    within `radius` (a filled-ball kernel without its centre, zero padding) is summed and
//    cells whose sum is below the threshold are cleared (all four channels).
#include <algorithm>
#include <cmath>

#include "pgb_host.h"
#include "pgb_device.cuh"

namespace pgb {
namespace {

struct SplatCam {
  float T[12];  // rows 0..2 of the camera-to-world matrix
  float fov, aspect, pd;
  int xs, ys;
  float hx, hy, hz;  // ceil(shape / 2)
  float alpha_min;
};

__device__ __forceinline__ float dot3_ref(float a0, float a1, float a2, float b0, float b1, float b2) {
  return radd(radd(rmul(a0, b0), rmul(a1, b1)), rmul(a2, b2));
}

__global__ void splat_kernel(const float4* __restrict__ cells, int X, int Y, int Z, SplatCam k,
                             unsigned long long* __restrict__ keys) {
  const int64_t G = (int64_t)X * Y * Z;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < G;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float4 c = __ldg(cells + i);
    if (!(c.w > k.alpha_min)) continue;
    const int iz = (int)(i % Z);
    const int64_t ij = i / Z;
    const int iy = (int)(ij % Y), ix = (int)(ij / Y);
    // world position ((index - ceil(shape/2)) + 1) * pd, then relative to the camera
    const float px = rmul(radd(rsub((float)ix, k.hx), 1.f), k.pd);
    const float py = rmul(radd(rsub((float)iy, k.hy), 1.f), k.pd);
    const float pz = rmul(radd(rsub((float)iz, k.hz), 1.f), k.pd);
    const float cx = rsub(px, k.T[3]), cy = rsub(py, k.T[7]), cz = rsub(pz, k.T[11]);
    // camera axes: x axis = column 0 (the "yz plane normal"), y axis = column 1
    const float dyz = dot3_ref(cx, cy, cz, k.T[0], k.T[4], k.T[8]);
    const float dxz = dot3_ref(cx, cy, cz, k.T[1], k.T[5], k.T[9]);
    const float dist = rsqrt_exact(rfma(cz, cz, rfma(cy, cy, rmul(cx, cx))));
    const float nyz = rsqrt_exact(radd(radd(rmul(k.T[0], k.T[0]), rmul(k.T[4], k.T[4])), rmul(k.T[8], k.T[8])));
    const float norms = rmul(dist, nyz);
    const float ax = rdiv(dyz, norms), ay = rdiv(dxz, norms);
    const float xn = radd(0.5f, rdiv(ay, -k.fov));
    const float yn = radd(0.5f, rdiv(ax, rdiv(k.fov, k.aspect)));
    if (!(xn < 1.f && xn >= 0.f && yn < 1.f && yn >= 0.f)) continue;
    const int xx = (int)fminf(fmaxf(rintf(rmul((float)k.xs, xn)), 0.f), (float)(k.xs - 1));
    const int yy = (int)fminf(fmaxf(rintf(rmul((float)k.ys, yn)), 0.f), (float)(k.ys - 1));
    // nearest point wins; among equal distances the later cell in row-major order
    const unsigned long long key = ((unsigned long long)__float_as_uint(dist) << 32) |
                                   (unsigned long long)(0xffffffffu - (uint32_t)i);
    atomicMin(keys + (int64_t)xx * k.ys + yy, key);
  }
}

__global__ void splat_resolve_kernel(const float4* __restrict__ cells,
                                     const unsigned long long* __restrict__ keys, int64_t npix,
                                     float* __restrict__ img) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < npix;
       p += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long key = keys[p];
    float r = 1.f, g = 1.f, b = 1.f;  // white background
    if (key != ~0ull) {
      const uint32_t i = 0xffffffffu - (uint32_t)(key & 0xffffffffull);
      const float4 c = __ldg(cells + i);
      r = c.x; g = c.y; b = c.z;
    }
    img[3 * p + 0] = r;
    img[3 * p + 1] = g;
    img[3 * p + 2] = b;
  }
}

__global__ void fill_u64_kernel(unsigned long long* p, int64_t n, unsigned long long v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] = v;
}

// Offsets of the filled-ball kernel (src/grid_functions.py:260-267), decided on the host
// in double precision as the reference decides them: bit ((dx+h)*k + (dy+h))*k + (dz+h).
struct BallMask {
  uint32_t w[11];  // kernel_size <= 7: at most 343 offsets
};

// neighbour sum of alpha over the ball offsets, zero padding
__global__ void ball_sum_kernel(const float4* __restrict__ cells, int X, int Y, int Z, int h, BallMask m,
                                float* __restrict__ out) {
  const int z = blockIdx.x * blockDim.x + threadIdx.x;
  if (z >= Z) return;
  const int y = blockIdx.y, x = blockIdx.z;
  float s = 0.f;
  for (int dx = -h; dx <= h; ++dx) {
    const int xx = x + dx;
    if (xx < 0 || xx >= X) continue;
    for (int dy = -h; dy <= h; ++dy) {
      const int yy = y + dy;
      if (yy < 0 || yy >= Y) continue;
      for (int dz = -h; dz <= h; ++dz) {
        const int zz = z + dz;
        if (zz < 0 || zz >= Z) continue;
        const int k = 2 * h + 1;
        const int bit = ((dx + h) * k + (dy + h)) * k + (dz + h);
        if (!((m.w[bit >> 5] >> (bit & 31)) & 1u)) continue;
        s += __ldg(cells + ((int64_t)xx * Y + yy) * Z + zz).w;
      }
    }
  }
  out[((int64_t)x * Y + y) * Z + z] = s;
}

__global__ void clear_below_kernel(float4* __restrict__ cells, const float* __restrict__ sums, int64_t G,
                                   float threshold) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < G;
       i += (int64_t)gridDim.x * blockDim.x)
    if (sums[i] < threshold) cells[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

inline unsigned nblocks(int64_t n) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 32));
}

// Host fp32 arithmetic, rounded op by op (this file is compiled without FMA contraction).
inline float norm3_plain(float x, float y, float z) {
  const float xx = x * x, yy = y * y, zz = z * z;
  const float s = xx + yy;
  return std::sqrt(s + zz);
}

}  // namespace
}  // namespace pgb

using namespace pgb;

extern "C" {

int pgb_splat_size(const float* transform, int32_t size_y, int32_t* width_out) {
  if (!transform || !width_out || size_y <= 0) return PGB_ERR_ARG;
  const float aspect = norm3_plain(transform[0], transform[4], transform[8]) /
                       norm3_plain(transform[1], transform[5], transform[9]);
  const float w = (float)size_y * aspect;
  if (!(w >= 1.f) || w > 1.0e6f) return PGB_ERR_ARG;
  *width_out = (int32_t)w;
  return PGB_OK;
}

int pgb_splat_preview(const float* cells, const int32_t dims[3], float points_distance,
                      const float* transform, float camera_angle_x, int32_t size_y, float alpha_min,
                      unsigned long long* keys_scratch, float* image_out, pgb_stream_t stream) {
  if (!cells || !dims || !transform || !keys_scratch || !image_out) return PGB_ERR_ARG;
  if (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return PGB_ERR_ARG;
  const int64_t G = (int64_t)dims[0] * dims[1] * dims[2];
  if (G > 0xffffffffll) return PGB_ERR_UNSUPPORTED;
  if (((uintptr_t)cells % 16) || ((uintptr_t)keys_scratch % 8)) return PGB_ERR_ALIGN;
  int32_t xs = 0;
  int st = pgb_splat_size(transform, size_y, &xs);
  if (st) return st;
  SplatCam k;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 4; ++c) k.T[4 * r + c] = transform[4 * r + c];
  k.fov = camera_angle_x;
  k.aspect = norm3_plain(transform[0], transform[4], transform[8]) /
             norm3_plain(transform[1], transform[5], transform[9]);
  k.pd = points_distance;
  k.xs = xs;
  k.ys = size_y;
  k.hx = std::ceil((float)dims[0] / 2.f);
  k.hy = std::ceil((float)dims[1] / 2.f);
  k.hz = std::ceil((float)dims[2] / 2.f);
  k.alpha_min = alpha_min;
  const int64_t npix = (int64_t)xs * size_y;
  fill_u64_kernel<<<nblocks(npix), 256, 0, stream>>>(keys_scratch, npix, ~0ull);
  if ((st = after_launch())) return st;
  splat_kernel<<<nblocks(G), 256, 0, stream>>>(reinterpret_cast<const float4*>(cells), dims[0], dims[1],
                                               dims[2], k, keys_scratch);
  if ((st = after_launch())) return st;
  splat_resolve_kernel<<<nblocks(npix), 256, 0, stream>>>(reinterpret_cast<const float4*>(cells),
                                                          keys_scratch, npix, image_out);
  return after_launch();
}

int pgb_remove_noise(float* cells, const int32_t dims[3], int32_t kernel_size, double radius,
                     float threshold, int32_t repeats, float* sums_scratch, pgb_stream_t stream) {
  if (!cells || !dims || !sums_scratch || repeats < 0) return PGB_ERR_ARG;
  if (kernel_size < 1 || kernel_size % 2 == 0 || kernel_size > 7) return PGB_ERR_ARG;
  if (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return PGB_ERR_ARG;
  if (dims[0] > 65535 || dims[1] > 65535) return PGB_ERR_UNSUPPORTED;
  if ((uintptr_t)cells % 16) return PGB_ERR_ALIGN;
  const int h = kernel_size / 2;
  BallMask m = {};
  bool any = false;
  for (int dx = -h; dx <= h; ++dx)
    for (int dy = -h; dy <= h; ++dy)
      for (int dz = -h; dz <= h; ++dz) {
        const int d2 = dx * dx + dy * dy + dz * dz;
        if (d2 != 0 && std::sqrt((double)d2) <= radius) {
          const int bit = ((dx + h) * kernel_size + (dy + h)) * kernel_size + (dz + h);
          m.w[bit >> 5] |= 1u << (bit & 31);
          any = true;
        }
      }
  // a ball with no cell besides the centre: the reference's normalised kernel is 0/0
  // (NaN) and no sum compares below the threshold, so nothing is cleared
  if (!any) return PGB_OK;
  const int64_t G = (int64_t)dims[0] * dims[1] * dims[2];
  const dim3 grid((dims[2] + 127) / 128, dims[1], dims[0]);
  for (int it = 0; it < repeats; ++it) {
    ball_sum_kernel<<<grid, 128, 0, stream>>>(reinterpret_cast<const float4*>(cells), dims[0], dims[1],
                                              dims[2], h, m, sums_scratch);
    int st = after_launch();
    if (st) return st;
    clear_below_kernel<<<nblocks(G), 256, 0, stream>>>(reinterpret_cast<float4*>(cells), sums_scratch, G,
                                                       threshold);
    if ((st = after_launch())) return st;
  }
  return PGB_OK;
}

}  // extern "C"
