// Fused render kernels: ray sampling -> voxel lookup -> front-to-back compositing, and the
// hand-written adjoint, one warp per ray.
//
// What one launch replaces (paths relative to the reference repository):
//   src/ray_sampling.py:195-264  generate_rays_batched       (in-kernel when cameras are given)
//   src/ray_sampling.py:161-167  sample positions o + d * (delta * k)
//   src/ray_sampling.py:12-13    normalisation (p - min) / points_distance
//   src/grid_functions.py:103-114 nearest lookup / :7-44, :220-246 trilinear lookup
//   scripts/train.py:146-147     grid.clip(0, 1) and the in-bounds mask
//   src/ray_sampling.py:172-192  compute_alpha_weighted_pixels
//   scripts/train.py:156, 181    mse_loss and its backward through all of the above
//
// Work layout: a warp owns one ray at a time. Samples are dealt to lanes in "slots":
// slot k of lane l is sample 32*k + l, so each load instruction of a warp touches 32
// consecutive samples of one ray (a compact run of cells). A chunk is K slots (32*K
// samples). The transmittance is an exclusive prefix product, computed per slot with a
// warp scan and carried across slots and chunks. The adjoint needs, per sample,
//     d alpha_s = T_s * (G_s - S_{s+1}),   G_s = <g_rgb, c_s> + g_A,
//     S_s = G_s * alpha_s + (1 - alpha_s) * S_{s+1},  S_{end} = 0,
// a suffix recurrence of affine maps evaluated with a second warp scan. It contains no
// division, so alpha == 1 (transmittance exactly 0 after the clip) is exact. Per-sample
// values of the current chunk stay in registers; in the reverse pass the chunks before the
// last come back from the warp's shared-memory stage (the last few chunks) or are gathered
// again from the grid (the transmittance at each chunk start is kept in lane c).
#pragma once

#include "pgb_device.cuh"

namespace pgb {

enum Phase { kForward = 0, kBackward = 1, kTrain = 2 };

template <typename Real>
struct GridP {
  const void* cells;
  int X, Y, Z;
  Real fX, fY, fZ;
  Real ox, oy, oz;
  Real pd;
  int clip;
  float alpha_floor;  // >0: clamped alpha below it reads as 0 (inference threshold)
};

template <typename Real>
struct RenderArgs {
  GridP<Real> g;
  // explicit rays
  const Real* origins;
  const Real* dirs;
  // in-kernel camera rays
  int use_cameras;
  const float* transforms;
  const float* images;
  int C, H, W;
  float fov, near_dist;
  uint64_t cam_seed;
  // sampling
  int64_t R;
  int S;
  Real delta;
  int stratified;
  uint64_t strat_seed;
  int64_t first_ray;  // index of ray 0 in the stratification stream
  float term_thr;
  int chunk_samples;  // host-side chunk request (pick_slots)
  int use_bg;      // rgb += (1 - A) * bg after compositing
  float bg[3];
  // outputs / adjoint inputs
  Real* rgba_out;
  const Real* d_rgba;
  const Real* target;
  Real* grad;
  uint32_t* grad_marks;  // optional: units of written gradient cells are marked here
  Real* loss_out;
  double* partials;
  unsigned* counter;
  double loss_w;
  double inv_count;
  // beta loss of scripts/train.py:170-177: beta_w * mean over all R*S samples of
  // log(alpha + eps) - log(1 - alpha + eps) (0: off)
  double beta_w;
  float beta_eps;
  double inv_samples;
  double* partials_beta;
  // derived on the host (finish_args): GB300's fp64 rate is low, and every warp would
  // otherwise evaluate these double expressions at its start
  int use_beta;       // beta_w != 0
  Real grad_scale;    // 2 * loss_w * inv_count: d(weighted MSE)/d pixel
  Real beta_scale;    // beta_w * inv_samples * (1 + 2 eps)
};

template <typename Real>
struct Ray {
  Real ox, oy, oz, dx, dy, dz;
  Real tgt[4];
  uint64_t h;  // stratification stream of this ray
};

// Euclidean norm of a 3-vector as the reference's CPU torch.norm evaluates it. Over a
// contiguous last dimension (the direction tensor) it accumulates with FMAs:
// sqrt(fma(z, z, fma(y, y, x * x))); over a strided view (the camera axes T[:, :3, i])
// it rounds every product and sum: sqrt((x*x + y*y) + z*z).
__device__ __forceinline__ float norm3_ref(float x, float y, float z) {
  return rsqrt_exact(rfma(z, z, rfma(y, y, rmul(x, x))));
}
__device__ __forceinline__ float norm3_strided_ref(float x, float y, float z) {
  return rsqrt_exact(radd(radd(rmul(x, x), rmul(y, y)), rmul(z, z)));
}

// Direction of a camera ray from uniforms (u, v), src/ray_sampling.py:215-262, rounded
// op by op as the reference's fp32 tensor program.
__device__ __forceinline__ void camera_direction(const float* T, float fov, float u, float v,
                                                 float d[3]) {
  // T is row-major 4x4: column 0 = x axis, column 1 = y axis, column 2 = back axis.
  const float xa0 = T[0], xa1 = T[4], xa2 = T[8];
  const float ya0 = T[1], ya1 = T[5], ya2 = T[9];
  const float za0 = -T[2], za1 = -T[6], za2 = -T[10];
  const float aspect = rdiv(norm3_strided_ref(xa0, xa1, xa2), norm3_strided_ref(ya0, ya1, ya2));
  const float ru = rmul(fov, rsub(u, 0.5f));
  const float rv = -rmul(rmul(fov, rdiv(1.0f, aspect)), rsub(v, 0.5f));
  const float e0 = radd(radd(rmul(ru, xa0), rmul(rv, ya0)), za0);
  const float e1 = radd(radd(rmul(ru, xa1), rmul(rv, ya1)), za1);
  const float e2 = radd(radd(rmul(ru, xa2), rmul(rv, ya2)), za2);
  const float n = norm3_ref(e0, e1, e2);
  d[0] = rdiv(e0, n);
  d[1] = rdiv(e1, n);
  d[2] = rdiv(e2, n);
}

// Pixel of a ray (src/ray_sampling.py:238-248): column from u scaled by H, row from v
// scaled by W, round half to even, clamp to the last index.
__device__ __forceinline__ void camera_pixel(int H, int W, float u, float v, int& row, int& col) {
  col = (int)fminf(rintf(rmul((float)H, u)), (float)(H - 1));
  row = (int)fminf(rintf(rmul((float)W, v)), (float)(W - 1));
}

template <typename Real>
__device__ __forceinline__ void load_ray(const RenderArgs<Real>& a, int64_t r, Ray<Real>& ray,
                                         bool need_target) {
  if (a.use_cameras) {
    // cameras get contiguous runs of rays (camera-major, src/ray_sampling.py:243)
    // floor(r * C / R), in 32-bit arithmetic when r * C fits (the 64-bit divide is a long
    // instruction sequence)
    const uint64_t rc = (uint64_t)r * (uint64_t)a.C;
    const int c = (rc >> 32) == 0 && ((uint64_t)a.R >> 32) == 0
                      ? (int)((uint32_t)rc / (uint32_t)a.R)
                      : (int)(rc / (uint64_t)a.R);
    const float* T = a.transforms + 16 * (int64_t)c;
    const uint64_t h = hash_stream(a.cam_seed, (uint64_t)r);
    const float u = hash_to_unit(h, 0u), v = hash_to_unit(h, 1u);
    float d[3];
    camera_direction(T, a.fov, u, v, d);
    ray.dx = d[0]; ray.dy = d[1]; ray.dz = d[2];
    ray.ox = radd(T[3], rmul(a.near_dist, d[0]));
    ray.oy = radd(T[7], rmul(a.near_dist, d[1]));
    ray.oz = radd(T[11], rmul(a.near_dist, d[2]));
    if (need_target) {
      int row, col;
      camera_pixel(a.H, a.W, u, v, row, col);
      const float4 px = __ldg(reinterpret_cast<const float4*>(a.images) +
                              (((int64_t)c * a.H + row) * a.W + col));
      ray.tgt[0] = px.x; ray.tgt[1] = px.y; ray.tgt[2] = px.z; ray.tgt[3] = px.w;
    }
  } else {
    ray.ox = a.origins[3 * r + 0]; ray.oy = a.origins[3 * r + 1]; ray.oz = a.origins[3 * r + 2];
    ray.dx = a.dirs[3 * r + 0];    ray.dy = a.dirs[3 * r + 1];    ray.dz = a.dirs[3 * r + 2];
    if (need_target) {
#pragma unroll
      for (int c = 0; c < 4; ++c) ray.tgt[c] = a.target[4 * r + c];
    }
  }
  ray.h = a.stratified ? hash_stream(a.strat_seed, (uint64_t)(r + a.first_ray)) : 0ull;
}

// Normalised grid coordinates of sample s (0-based) of a ray:
//   t = delta * (s + 1) [- jitter],  p = o + d * t,  n = (p - origin) / pd
// each op rounded separately (src/ray_sampling.py:161-167, :13).
template <typename Real>
__device__ __forceinline__ void sample_coords(const RenderArgs<Real>& a, const Ray<Real>& ray,
                                              int s, Real& nx, Real& ny, Real& nz) {
  Real k = (Real)(s + 1);
  if (a.stratified) k = rsub(k, (Real)hash_to_unit(ray.h, (uint32_t)s));
  const Real t = rmul(a.delta, k);
  const Real px = radd(ray.ox, rmul(ray.dx, t));
  const Real py = radd(ray.oy, rmul(ray.dy, t));
  const Real pz = radd(ray.oz, rmul(ray.dz, t));
  nx = rdiv(rsub(px, a.g.ox), a.g.pd);
  ny = rdiv(rsub(py, a.g.oy), a.g.pd);
  nz = rdiv(rsub(pz, a.g.oz), a.g.pd);
}

template <typename Real>
__device__ __forceinline__ uint64_t cell_index(const GridP<Real>& g, int i, int j, int k) {
  return ((uint64_t)i * (uint64_t)g.Y + (uint64_t)j) * (uint64_t)g.Z + (uint64_t)k;
}

// Trilinear corner geometry of an in-bounds sample: wrapped ceil/floor indices per axis
// and the fractional weights (src/grid_functions.py:29, :230-244, :75-77). For an
// in-bounds coordinate 0 <= n < dim, only ceil can leave the grid (n in (dim-1, dim)),
// and it wraps to 0.
template <typename Real>
struct Corners {
  int c[3], f[3];
  Real w[3];  // frac(n) per axis
};

template <typename Real>
__device__ __forceinline__ bool trilinear_corners(const GridP<Real>& g, Real nx, Real ny, Real nz,
                                                  Corners<Real>& q) {
  if (!(nx >= Real(0) && nx < g.fX && ny >= Real(0) && ny < g.fY && nz >= Real(0) && nz < g.fZ))
    return false;
  const Real n[3] = {nx, ny, nz};
  const int dim[3] = {g.X, g.Y, g.Z};
#pragma unroll
  for (int ax = 0; ax < 3; ++ax) {
    const Real fl = rfloor(n[ax]);
    q.f[ax] = (int)fl;
    const int ce = (int)rceil(n[ax]);
    q.c[ax] = ce >= dim[ax] ? ce - dim[ax] : ce;
    q.w[ax] = rsub(n[ax], fl);  // == n - trunc(n) for n >= 0
  }
  return true;
}

// Value of one sample, masked to zero outside the grid. bits: gradient-pass flags of
// the clamp, bit 4*corner + channel (trilinear; corner order of
// src/grid_functions.py:16-24) or bit channel (nearest). Zero when out of bounds.
template <typename Real, typename Store, int MODE>
__device__ __forceinline__ void sample_value(const GridP<Real>& g, Real nx, Real ny, Real nz,
                                             Real v[4], uint32_t& bits) {
  bits = 0u;
  v[0] = v[1] = v[2] = v[3] = Real(0);
  if (MODE == PGB_NEAREST) {
    const Real rx = rround(nx), ry = rround(ny), rz = rround(nz);
    if (!(rx >= Real(0) && rx < g.fX && ry >= Real(0) && ry < g.fY && rz >= Real(0) && rz < g.fZ))
      return;
    Real cv[4];
    CellIO<Store>::load(g.cells, cell_index(g, (int)rx, (int)ry, (int)rz), cv);
#pragma unroll
    for (int ch = 0; ch < 4; ++ch) {
      if (g.clip) {
        bits |= (in01(cv[ch]) ? 1u : 0u) << ch;
        v[ch] = clamp01(cv[ch]);
      } else {
        bits |= 1u << ch;
        v[ch] = cv[ch];
      }
    }
    if (g.alpha_floor > 0.0f && v[3] < (Real)g.alpha_floor) {
      v[3] = Real(0);
      bits &= ~8u;
    }
  } else {
    Corners<Real> q;
    if (!trilinear_corners(g, nx, ny, nz, q)) return;
    Real cv[8][4];
#pragma unroll
    for (int corner = 0; corner < 8; ++corner) {
      const int ix = (corner & 4) ? q.f[0] : q.c[0];
      const int iy = (corner & 2) ? q.f[1] : q.c[1];
      const int iz = (corner & 1) ? q.f[2] : q.c[2];
      CellIO<Store>::load(g.cells, cell_index(g, ix, iy, iz), cv[corner]);
    }
#pragma unroll
    for (int corner = 0; corner < 8; ++corner) {
#pragma unroll
      for (int ch = 0; ch < 4; ++ch) {
        if (g.clip) {
          bits |= (in01(cv[corner][ch]) ? 1u : 0u) << (4 * corner + ch);
          cv[corner][ch] = clamp01(cv[corner][ch]);
        } else {
          bits |= 1u << (4 * corner + ch);
        }
      }
      if (g.alpha_floor > 0.0f && cv[corner][3] < (Real)g.alpha_floor) {
        cv[corner][3] = Real(0);
        bits &= ~(8u << (4 * corner));
      }
    }
    // blend x, then y, then z, as src/grid_functions.py:34-42
    const Real wx = q.w[0], wy = q.w[1], wz = q.w[2];
    const Real ux = rsub(Real(1), wx), uy = rsub(Real(1), wy), uz = rsub(Real(1), wz);
#pragma unroll
    for (int ch = 0; ch < 4; ++ch) {
      Real a4[4];
#pragma unroll
      for (int yz = 0; yz < 4; ++yz)
        a4[yz] = radd(rmul(cv[yz][ch], wx), rmul(cv[4 + yz][ch], ux));
      const Real b0 = radd(rmul(a4[0], wy), rmul(a4[2], uy));
      const Real b1 = radd(rmul(a4[1], wy), rmul(a4[3], uy));
      v[ch] = radd(rmul(b0, wz), rmul(b1, uz));
    }
  }
}

#ifndef PGB_SCATTER_INLINE
#define PGB_SCATTER_INLINE 1
#endif
#if PGB_SCATTER_INLINE
#define PGB_SCATTER_ATTR __device__ __forceinline__
#else
#define PGB_SCATTER_ATTR __device__ __noinline__
#endif

// Marks the gradient unit of cell c in the bitmap of units (mark_unit_of).
__device__ __forceinline__ void mark_unit(uint32_t* marks, uint64_t c) {
  const uint64_t u = mark_unit_of(c);
  atomicOr(marks + (u >> 5), 1u << ((uint32_t)u & 31u));
}

// Scatter dL/dvalue of one sample into the dense gradient (the autograd replay of the
// blend, the clamp mask and index_put accumulate). marks (optional): the unit of every
// written cell is marked.
template <typename Real, int MODE>
PGB_SCATTER_ATTR void sample_scatter(const GridP<Real>& g, Real* grad, Real nx, Real ny,
                                     Real nz, const Real dv[4], uint32_t bits,
                                     uint32_t* marks = nullptr) {
  if (bits == 0u) return;
  if (MODE == PGB_NEAREST) {
    Real gv[4];
#pragma unroll
    for (int ch = 0; ch < 4; ++ch) gv[ch] = ((bits >> ch) & 1u) ? dv[ch] : Real(0);
    const uint64_t c = cell_index(g, (int)rround(nx), (int)rround(ny), (int)rround(nz));
    grad_add(grad, c, gv);
    if (marks != nullptr) mark_unit(marks, c);
  } else {
    Corners<Real> q;
    trilinear_corners(g, nx, ny, nz, q);
    const Real wx = q.w[0], wy = q.w[1], wz = q.w[2];
    const Real ux = rsub(Real(1), wx), uy = rsub(Real(1), wy), uz = rsub(Real(1), wz);
    // corner weights, corner order of src/grid_functions.py:16-24
    const Real wyz[4] = {wy * wz, wy * uz, uy * wz, uy * uz};
    const uint64_t rowc = (uint64_t)q.c[0] * (uint64_t)g.Y, rowf = (uint64_t)q.f[0] * (uint64_t)g.Y;
    // marks of the two z-neighbour corners (same x, y) mostly fall in one word: OR them
    // together and flush once per pair
    uint64_t mark_word = 0;
    uint32_t mark_bits = 0u;
#pragma unroll
    for (int corner = 0; corner < 8; ++corner) {
      if (marks != nullptr && (corner & 1) == 0 && mark_bits != 0u) {
        atomicOr(marks + mark_word, mark_bits);
        mark_bits = 0u;
      }
      const Real wc = ((corner & 4) ? ux : wx) * wyz[corner & 3];
      const uint32_t cb = bits >> (4 * corner);
      if ((cb & 0xfu) == 0u) continue;
      Real gv[4];
      bool any = false;
#pragma unroll
      for (int ch = 0; ch < 4; ++ch) {
        gv[ch] = ((cb >> ch) & 1u) ? dv[ch] * wc : Real(0);
        any |= gv[ch] != Real(0);
      }
      if (any) {
        const uint64_t row = (corner & 4) ? rowf : rowc;
        const int iy = (corner & 2) ? q.f[1] : q.c[1];
        const int iz = (corner & 1) ? q.f[2] : q.c[2];
        const uint64_t cell = (row + (uint64_t)iy) * (uint64_t)g.Z + (uint64_t)iz;
        grad_add(grad, cell, gv);
        if (marks != nullptr) {
          const uint64_t unit = mark_unit_of(cell);
          const uint64_t word = unit >> 5;
          const uint32_t bit = 1u << ((uint32_t)unit & 31u);
          if (mark_bits != 0u && word != mark_word) {
            atomicOr(marks + mark_word, mark_bits);
            mark_bits = 0u;
          }
          mark_word = word;
          mark_bits |= bit;
        }
      }
    }
    if (marks != nullptr && mark_bits != 0u) atomicOr(marks + mark_word, mark_bits);
  }
}

// sample_scatter for trilinear lookup with the updates of a warp merged per cell. For each
// corner, lanes whose update goes to the same cell as their lower neighbour's form a run
// (consecutive samples of a ray inside one cell, which is where a cell repeats: samples
// move monotonically along the ray); the run's partials are summed into its first lane
// by a segmented shuffle reduction and that lane issues the one atomic. A cell split
// over two runs gets two atomics, so the result is the same sum in another order. Every
// lane of the warp must call it; has = false marks a lane with nothing to add.
template <typename Real>
__device__ __forceinline__ void warp_merged_scatter(const GridP<Real>& g, Real* grad, bool has,
                                                    Real nx, Real ny, Real nz, const Real dv[4],
                                                    uint32_t bits, int lane) {
  Corners<Real> q = {};
  if (has) has = trilinear_corners(g, nx, ny, nz, q);
  const Real wx = q.w[0], wy = q.w[1], wz = q.w[2];
  const Real ux = Real(1) - wx, uy = Real(1) - wy, uz = Real(1) - wz;
  const Real wyz[4] = {wy * wz, wy * uz, uy * wz, uy * uz};
#pragma unroll 1
  for (int corner = 0; corner < 8; ++corner) {
    const uint32_t cb = has ? (bits >> (4 * corner)) & 0xfu : 0u;
    const Real wc = ((corner & 4) ? ux : wx) * wyz[corner & 3];
    Real gv[4];
    bool any = false;
#pragma unroll
    for (int ch = 0; ch < 4; ++ch) {
      gv[ch] = ((cb >> ch) & 1u) ? dv[ch] * wc : Real(0);
      any |= gv[ch] != Real(0);
    }
    if (!__any_sync(kFull, any)) continue;
    // a lane with nothing to add gets a key no other lane and no cell has
    const int ix = (corner & 4) ? q.f[0] : q.c[0];
    const int iy = (corner & 2) ? q.f[1] : q.c[1];
    const int iz = (corner & 1) ? q.f[2] : q.c[2];
    const uint64_t key = any ? cell_index(g, ix, iy, iz) : ~0ull - (uint64_t)lane;
    const uint64_t prev = __shfl_up_sync(kFull, key, 1);
    const bool head = lane == 0 || prev != key;
    const uint32_t heads = __ballot_sync(kFull, head);
    const uint32_t later = lane == kWarp - 1 ? 0u : heads & ~((2u << lane) - 1u);
    const int seg_end = later ? __ffs(later) - 2 : kWarp - 1;
#pragma unroll
    for (int d = 1; d < kWarp; d <<= 1) {
#pragma unroll
      for (int ch = 0; ch < 4; ++ch) {
        const Real y = __shfl_down_sync(kFull, gv[ch], d);
        if (lane + d <= seg_end) gv[ch] += y;
      }
    }
    if (head && any) grad_add(grad, key, gv);
  }
}

// Tuning knobs (compile-time; the shipped values are the measured best on GB300).
#ifndef PGB_RENDER_THREADS
#define PGB_RENDER_THREADS 256
#endif
#ifndef PGB_RENDER_MIN_BLOCKS
#define PGB_RENDER_MIN_BLOCKS 0
#endif
// Nearest lookup (one load per sample) gains from more resident warps even at 64
// registers with spills: 4 blocks per SM measured 0.0697 ms against 0.0765 ms at 2.
#ifndef PGB_RENDER_MIN_BLOCKS_NEAREST
#define PGB_RENDER_MIN_BLOCKS_NEAREST 4
#endif
// Trilinear lookup with 32-sample chunks: 24 resident warps per SM (80 registers, a
// 32-byte spill) measured 0.127 ms per step against 0.133 ms at 16 (256^3, 8192 rays x
// 256). Its blocks are 128 threads: a block holds its SM slot until its slowest ray ends,
// and rays end at very different depths once they stop behind opaque cells, so smaller
// blocks free slots sooner (kernel 0.094 ms against 0.098 ms at 256 threads; 64 threads
// took 0.102 ms). Nearest lookup measured best at 256 threads.
#ifndef PGB_RENDER_THREADS_K1
#define PGB_RENDER_THREADS_K1 128
#endif
#ifndef PGB_RENDER_MIN_BLOCKS_K1
#define PGB_RENDER_MIN_BLOCKS_K1 (3 * 256 / PGB_RENDER_THREADS_K1)
#endif

constexpr int kRenderThreads = PGB_RENDER_THREADS;
constexpr int kRenderThreadsK1 = PGB_RENDER_THREADS_K1;
// the smallest block of any render launch (it bounds the number of blocks per ray count)
constexpr int kRenderMinThreads = kRenderThreads < kRenderThreadsK1 ? kRenderThreads
                                                                     : kRenderThreadsK1;


// The per-warp shared-memory stage of the render and batched kernels: per chunk slot,
// for the last M chunks,
//   - the normalised coordinates (COORDS; otherwise the reverse pass recomputes them from
//     the ray: the stratification hash and the exact divisions),
//   - with M > 1, the clamped values and clamp-pass bits, so the reverse pass reads the
//     M - 1 chunks before the last from here instead of gathering them from the grid
//     again,
//   - with TS, the forward pass's transmittances, so the reverse pass skips their scan.
// Layout [slot][field][K][32]: each lane reads back only what it wrote, without bank
// conflicts.
template <typename Real, int K, int MSLOTS, bool COORDS = true, bool TS = false>
struct ChunkStage {
  static constexpr int M = MSLOTS;
  static constexpr bool kHasCoords = COORDS;
  static constexpr bool kHasTs = TS;  // the transmittance of every sample too
  static_assert((M & (M - 1)) == 0, "stage slots must be a power of two");
  static_assert(COORDS || M > 1, "a stage without coordinates holds values");
  static_assert(!TS || M > 1, "transmittances are held with the values");
  static constexpr int kCoordBytes = COORDS ? 3 * K * kWarp * (int)sizeof(Real) : 0;
  static constexpr int kVBytes = 4 * K * kWarp * (int)sizeof(Real);
  static constexpr int kBitsBytes = K * kWarp * 4;
  static constexpr int kTsBytes = TS ? K * kWarp * (int)sizeof(Real) : 0;
  static constexpr int kValBytes = M > 1 ? kVBytes + kBitsBytes + kTsBytes : 0;
  static constexpr int kSlotBytes = kCoordBytes + kValBytes;
  static constexpr int kBytesPerWarp = M * kSlotBytes;
  unsigned char* base;
  __device__ __forceinline__ ChunkStage(unsigned char* all, int warp)
      : base(all + (size_t)warp * kBytesPerWarp) {}
  __device__ __forceinline__ unsigned char* slot(int c) const { return base + (c & (M - 1)) * kSlotBytes; }
  // chunk c is still in the stage when the reverse pass reaches it (last = last chunk)
  __device__ __forceinline__ static bool holds(int c, int last) { return M > 1 && c > last - M; }
  __device__ __forceinline__ void put(int c, int k, int lane, Real x, Real y, Real z) {
    if constexpr (!COORDS) return;
    Real* n = reinterpret_cast<Real*>(slot(c));
    n[(0 * K + k) * kWarp + lane] = x;
    n[(1 * K + k) * kWarp + lane] = y;
    n[(2 * K + k) * kWarp + lane] = z;
  }
  __device__ __forceinline__ void get(int c, int k, int lane, Real& x, Real& y, Real& z) const {
    const Real* n = reinterpret_cast<const Real*>(slot(c));
    x = n[(0 * K + k) * kWarp + lane];
    y = n[(1 * K + k) * kWarp + lane];
    z = n[(2 * K + k) * kWarp + lane];
  }
  __device__ __forceinline__ void put_vals(int c, int k, int lane, const Real v[4], uint32_t bits) {
    if constexpr (M > 1) {
      Real* w = reinterpret_cast<Real*>(slot(c) + kCoordBytes);
#pragma unroll
      for (int ch = 0; ch < 4; ++ch) w[(ch * K + k) * kWarp + lane] = v[ch];
      reinterpret_cast<uint32_t*>(slot(c) + kCoordBytes + kVBytes)[k * kWarp + lane] = bits;
    }
  }
  __device__ __forceinline__ void get_vals(int c, int k, int lane, Real v[4], uint32_t& bits) const {
    if constexpr (M > 1) {
      const Real* w = reinterpret_cast<const Real*>(slot(c) + kCoordBytes);
#pragma unroll
      for (int ch = 0; ch < 4; ++ch) v[ch] = w[(ch * K + k) * kWarp + lane];
      bits = reinterpret_cast<const uint32_t*>(slot(c) + kCoordBytes + kVBytes)[k * kWarp + lane];
    }
  }
  __device__ __forceinline__ void put_t(int c, int k, int lane, Real t) {
    if constexpr (TS) reinterpret_cast<Real*>(slot(c) + kCoordBytes + kVBytes + kBitsBytes)[k * kWarp + lane] = t;
  }
  __device__ __forceinline__ Real get_t(int c, int k, int lane) const {
    if constexpr (TS)
      return reinterpret_cast<const Real*>(slot(c) + kCoordBytes + kVBytes + kBitsBytes)[k * kWarp + lane];
    return Real(0);
  }
};

#ifndef PGB_RENDER_GATHER_INLINE
#define PGB_RENDER_GATHER_INLINE 1
#endif
#if PGB_RENDER_GATHER_INLINE
#define PGB_RENDER_GATHER_ATTR __device__ __forceinline__
#else
#define PGB_RENDER_GATHER_ATTR __device__ __noinline__
#endif

// One sample of a ray: coordinates and value (zero outside the grid).
template <typename Real, typename Store, int MODE>
PGB_RENDER_GATHER_ATTR void render_sample(const RenderArgs<Real>& a, const Ray<Real>& ray, int s,
                                          Real v[4], uint32_t& bits, Real& nx, Real& ny, Real& nz) {
  sample_coords(a, ray, s, nx, ny, nz);
  sample_value<Real, Store, MODE>(a.g, nx, ny, nz, v, bits);
}

// Gathers chunk `c` (K slots) of a ray into registers (and its coordinates into the
// stage when the adjoint follows and the stage keeps coordinates).
template <typename Real, typename Store, int MODE, int K, bool ADJ, typename Stage>
__device__ __forceinline__ void gather_chunk(const RenderArgs<Real>& a, const Ray<Real>& ray, int c,
                                             int lane, Real v[K][4], uint32_t bits[K], Stage& cs) {
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const int s = (c * K + k) * kWarp + lane;
    v[k][0] = v[k][1] = v[k][2] = v[k][3] = Real(0);
    bits[k] = 0u;
    if (s < a.S) {
      Real nx, ny, nz;
      render_sample<Real, Store, MODE>(a, ray, s, v[k], bits[k], nx, ny, nz);
      if (ADJ) cs.put(c, k, lane, nx, ny, nz);
    }
  }
}

// Exclusive transmittance of every sample of a chunk from the chunk's starting T;
// returns T after the chunk.
#ifndef PGB_SLOT_SKIP
#define PGB_SLOT_SKIP 0  // 1: skip the scans of slots whose 32 samples all have alpha 0
#endif                   //    (exact; a vote per slot costs more than it saves here)
#ifndef PGB_REVERSE_LOOP
#define PGB_REVERSE_LOOP 1  // 1: one copy of the trilinear reverse-pass body in a slot loop
#endif                      // (the gather stays unrolled for its load parallelism):
                            // 0.158 -> 0.147 ms; 2: also for nearest; 0: unrolled
#ifndef PGB_SKIP_ZERO_DV
#define PGB_SKIP_ZERO_DV 1  // skip the scatter of samples whose four partials are all 0
#endif

template <typename Real, int K>
__device__ __forceinline__ Real scan_chunk(const Real v[K][4], Real T, int lane, Real Ts[K]) {
#pragma unroll
  for (int k = 0; k < K; ++k) {
    if (PGB_SLOT_SKIP && !__any_sync(kFull, v[k][3] != Real(0))) {
      Ts[k] = T;  // every factor (1 - alpha) is 1: the exact result of the scan
      continue;
    }
    const Real incl = warp_incl_prod(Real(1) - v[k][3], lane);
    Real excl = __shfl_up_sync(kFull, incl, 1);
    if (lane == 0) excl = Real(1);
    Ts[k] = T * excl;
    T *= __shfl_sync(kFull, incl, kWarp - 1);
  }
  return T;
}

// Error-free sum a + b = s + e (Knuth's TwoSum, six additions, no FMA). An infinite sum
// (an opaque sample: log(1 - 1) = -inf) carries no error term.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  if (isinf(s)) {
    e = 0.0f;
    return;
  }
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Compensated log-sum form of scan_chunk: T_s = exp(sum_{j<s} log(1 - alpha_j)), the sum
// carried as an unevaluated pair (L + C) across slots and chunks, each warp-scan step an
// error-free TwoSum whose error joins the compensation term (Kahan-Babuska style). Alpha
// must lie in [0, 1] (clipped cells): log1p(-alpha) is -inf at alpha = 1 and T is then 0.
template <int K>
__device__ __forceinline__ void scan_chunk_log(const float v[K][4], float& L, float& C, int lane,
                                               float Ts[K]) {
#pragma unroll
  for (int k = 0; k < K; ++k) {
    float a = log1pf(-v[k][3]);
    float c = 0.0f;
#pragma unroll
    for (int d = 1; d < kWarp; d <<= 1) {
      const float ya = __shfl_up_sync(kFull, a, d), yc = __shfl_up_sync(kFull, c, d);
      if (lane >= d) {
        float sum, err;
        two_sum(ya, a, sum, err);
        a = sum;
        c = __fadd_rn(__fadd_rn(c, yc), err);
      }
    }
    float ea = __shfl_up_sync(kFull, a, 1), ec = __shfl_up_sync(kFull, c, 1);
    if (lane == 0) ea = ec = 0.0f;
    float sum, err;
    two_sum(L, ea, sum, err);
    Ts[k] = isinf(sum) ? 0.0f : expf(__fadd_rn(sum, __fadd_rn(__fadd_rn(C, ec), err)));
    const float ta = __shfl_sync(kFull, a, kWarp - 1), tc = __shfl_sync(kFull, c, kWarp - 1);
    two_sum(L, ta, sum, err);
    L = sum;
    C = isinf(sum) ? 0.0f : __fadd_rn(__fadd_rn(C, tc), err);
  }
}

// v[i] for a runtime i in [0,4) without indexing a register array dynamically.
template <typename Real>
__device__ __forceinline__ Real pick4(const Real v[4], int i) {
  return i == 0 ? v[0] : (i == 1 ? v[1] : (i == 2 ? v[2] : v[3]));
}

// The render kernel's stage at 32-sample chunks: the values and clamp bits of the last
// PGB_RENDER_STAGE_CHUNKS chunks, without their coordinates (the reverse pass recomputes
// a sample's coordinates from its ray: cheaper than gathering a chunk from the grid
// again). 256^3, 8192 rays x 256 samples: 8 chunks without coordinates (5 KB per warp)
// 0.0928 ms per step; 4 chunks with them (4 KB) 0.1000 ms, without 0.0976 ms; 8 chunks
// with them (8 KB, 192 KB of shared memory per SM, leaving little L1) 0.175 ms.
#ifndef PGB_RENDER_STAGE_CHUNKS
#define PGB_RENDER_STAGE_CHUNKS 8
#endif
#ifndef PGB_RENDER_STAGE_COORDS
#define PGB_RENDER_STAGE_COORDS 0
#endif
// The staged chunks' transmittances as well (0: never, 1: always, 2: for the log-sum
// transmittance only). Recomputing them in the reverse pass is a warp scan; for the
// compensated log-sum it is a costly one. 512^3 log-sum, 65,536 rays x 512: 0.4567 ms
// staged against 0.4865 ms; 256^3 product: 0.0965 against 0.0934 ms.
#ifndef PGB_RENDER_STAGE_TS
#define PGB_RENDER_STAGE_TS 2
#endif
template <typename Real, int K, bool LOGT = false>
using RenderStage =
    ChunkStage<Real, K, (K == 1 ? PGB_RENDER_STAGE_CHUNKS : 1),
               (K != 1 || PGB_RENDER_STAGE_COORDS != 0),
               (K == 1 && (PGB_RENDER_STAGE_TS == 1 || (PGB_RENDER_STAGE_TS == 2 && LOGT)))>;

template <typename Real, int K, bool LOGT = false>
constexpr int render_smem_bytes(int warps_per_block) {
  return RenderStage<Real, K, LOGT>::kBytesPerWarp * warps_per_block;
}

template <int MODE, int K>
constexpr int render_threads() {
  return MODE != PGB_NEAREST && K == 1 ? kRenderThreadsK1 : kRenderThreads;
}

template <int MODE, int K>
constexpr int render_min_blocks() {
  return MODE == PGB_NEAREST ? PGB_RENDER_MIN_BLOCKS_NEAREST
                             : (K == 1 ? PGB_RENDER_MIN_BLOCKS_K1 : PGB_RENDER_MIN_BLOCKS);
}

// LOGT: transmittance as the compensated log-sum (scan_chunk_log, fp32 only) instead of
// the reference's product scan.
template <typename Real, typename Store, int MODE, int K, int PHASE, bool LOGT = false>
__global__ void __launch_bounds__((render_threads<MODE, K>()), (render_min_blocks<MODE, K>()))
render_kernel(const RenderArgs<Real> a) {
  static_assert(!LOGT || sizeof(Real) == 4, "log-sum transmittance is an fp32 form");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr bool ADJ = PHASE != kForward;
  const int lane = threadIdx.x & (kWarp - 1);
  const int warps_per_block = blockDim.x >> 5;
  const int64_t gw = (int64_t)blockIdx.x * warps_per_block + (threadIdx.x >> 5);
  const int64_t nw = (int64_t)gridDim.x * warps_per_block;
  const int nchunks = (a.S + kWarp * K - 1) / (kWarp * K);
  RenderStage<Real, K, LOGT> cs(smem_raw, threadIdx.x >> 5);
  LossSum<Real> loss_lane;  // lane 0: squared errors of the warp's rays
  LossSum<Real> beta_lane;  // per lane: beta terms of its samples
  const bool with_beta = PHASE == kTrain && a.use_beta;
  // Exact early stop. With alpha clamped to [0,1], T is exactly 0 only behind an opaque
  // sample z (alpha_z = 1) or after an underflow, and every later sample then has weight
  // 0 and colour and alpha gradients 0. One term still reads them: z's own alpha gradient
  // T_z (G_z - S_{z+1}), whose suffix S_{z+1} runs over the samples behind z up to the next
  // opaque one. So a ray stops after the chunk in which T reached 0 once z's alpha
  // gradient is masked by the clamp (stored alpha above 1) or a second opaque sample has
  // been gathered; an underflowed T drops terms below T's own magnitude (< 1e-38). The
  // beta term reads every sample's alpha, so it keeps them all.
  const bool stop_at_zero = a.g.clip && !with_beta;
  constexpr uint32_t kAlphaBits = MODE == PGB_NEAREST ? 0x8u : 0x88888888u;
  // beta_w / (R*S) * (1 + 2 eps): the numerator of 1/(alpha+eps) + 1/(1-alpha+eps)
  const Real beta_scale = a.beta_scale;
  const Real grad_scale = a.grad_scale;
  __shared__ double s_part[32];  // per-warp loss partials (training phase)
  __shared__ double s_part_beta[32];
  __shared__ unsigned s_done;    // warps of this block that finished (training phase)
  if (PHASE == kTrain) {
    if (threadIdx.x == 0) s_done = 0u;
    __syncthreads();
  }

  for (int64_t r = gw; r < a.R; r += nw) {
    Ray<Real> ray;
    load_ray(a, r, ray, PHASE == kTrain);

    Real v[K][4];
    uint32_t bits[K];
    Real Ts[K];
    Real acc[4] = {Real(0), Real(0), Real(0), Real(0)};
    Real T = Real(1);
    Real Tstart = Real(1);  // lane c: transmittance at the start of chunk c
    float LT = 0.0f, LC = 0.0f, LTstart = 0.0f, LCstart = 0.0f;  // LOGT: log T = LT + LC
    int last = -1;          // last composited chunk (-1: none, e.g. zero samples)
    int n_opaque = 0;       // opaque samples gathered so far (warp-uniform)
    bool first_needs = false;  // the first opaque sample's alpha gradient passes the clamp
    for (int c = 0; c < nchunks; ++c) {
      if (lane == c) {
        Tstart = T;
        LTstart = LT;
        LCstart = LC;
      }
      __syncwarp();
      gather_chunk<Real, Store, MODE, K, ADJ>(a, ray, c, lane, v, bits, cs);
      if (ADJ) {
#pragma unroll
        for (int k = 0; k < K; ++k) cs.put_vals(c, k, lane, v[k], bits[k]);
      }
      if constexpr (LOGT) {
        scan_chunk_log<K>(v, LT, LC, lane, Ts);
        T = isinf(LT) ? Real(0) : (Real)expf(LT + LC);
      } else {
        T = scan_chunk<Real, K>(v, T, lane, Ts);
      }
      if (ADJ) {
#pragma unroll
        for (int k = 0; k < K; ++k) cs.put_t(c, k, lane, Ts[k]);
      }
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const Real w = v[k][3] * Ts[k];
        acc[0] += w * v[k][0];
        acc[1] += w * v[k][1];
        acc[2] += w * v[k][2];
        acc[3] += w;
      }
      if (with_beta) {  // per-chunk partial in Real, one fp64 add per chunk
        Real bsum = Real(0);
#pragma unroll
        for (int k = 0; k < K; ++k) {
          if ((c * K + k) * kWarp + lane < a.S) {
            const Real al = v[k][3], e = (Real)a.beta_eps;
            bsum += log(al + e) - log(Real(1) - al + e);
          }
        }
        beta_lane.add(bsum);
      }
      last = c;
      if (stop_at_zero) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
          const unsigned opq = __ballot_sync(kFull, Real(1) - v[k][3] == Real(0));
          if (opq != 0u) {
            const unsigned need =
                __ballot_sync(kFull, (bits[k] & kAlphaBits) != 0u && Ts[k] > Real(0));
            if (n_opaque == 0) first_needs = ((need >> (__ffs(opq) - 1)) & 1u) != 0u;
            n_opaque += __popc(opq);
          }
        }
        if (T == Real(0) && (!first_needs || n_opaque >= 2)) break;
      }
      if (a.term_thr > 0.0f && T < (Real)a.term_thr) break;
    }
    Real px[4];
#pragma unroll
    for (int ch = 0; ch < 4; ++ch) px[ch] = warp_sum(acc[ch]);
    if (a.use_bg) {
#pragma unroll
      for (int ch = 0; ch < 3; ++ch) px[ch] += (Real(1) - px[3]) * (Real)a.bg[ch];
    }

    if (PHASE == kForward) {
      if (lane < 4) a.rgba_out[4 * r + lane] = pick4(px, lane);
      continue;
    }

    Real gpx[4];
    if (PHASE == kBackward) {
#pragma unroll
      for (int ch = 0; ch < 4; ++ch) gpx[ch] = a.d_rgba[4 * r + ch];
    } else {
      // the ray's squared error in Real (4 terms), accumulated over rays in double
      Real sq = Real(0);
#pragma unroll
      for (int ch = 0; ch < 4; ++ch) {
        const Real diff = px[ch] - ray.tgt[ch];
        sq += diff * diff;
        gpx[ch] = grad_scale * diff;
      }
      if (lane == 0) loss_lane.add(sq);
      if (a.rgba_out != nullptr && lane < 4) a.rgba_out[4 * r + lane] = pick4(px, lane);
    }
    if (a.use_bg)  // d(rgb + (1 - A) bg)/dA = -bg
      gpx[3] -= gpx[0] * (Real)a.bg[0] + gpx[1] * (Real)a.bg[1] + gpx[2] * (Real)a.bg[2];

    // reverse pass over the chunks that were composited
    Real Snext_carry = Real(0);  // S at the first sample after the current slot
    for (int c = last; c >= 0; --c) {
      if (c != last) {
        __syncwarp();
        const bool staged = RenderStage<Real, K, LOGT>::holds(c, last);
        if (staged) {  // the chunk's values are still staged
#pragma unroll
          for (int k = 0; k < K; ++k) cs.get_vals(c, k, lane, v[k], bits[k]);
        } else {
          gather_chunk<Real, Store, MODE, K, true>(a, ray, c, lane, v, bits, cs);
        }
        if (RenderStage<Real, K, LOGT>::kHasTs && staged) {  // the forward pass's transmittances
#pragma unroll
          for (int k = 0; k < K; ++k) Ts[k] = cs.get_t(c, k, lane);
        } else if constexpr (LOGT) {
          float l = __shfl_sync(kFull, LTstart, c), lc = __shfl_sync(kFull, LCstart, c);
          scan_chunk_log<K>(v, l, lc, lane, Ts);
        } else {
          scan_chunk<Real, K>(v, __shfl_sync(kFull, Tstart, c), lane, Ts);
        }
      }
      __syncwarp();
      // trilinear: a loop (the 8-corner scatter body is large); nearest: unrolled
      constexpr int kRevUnroll =
          (PGB_REVERSE_LOOP == 2 || (PGB_REVERSE_LOOP == 1 && MODE == PGB_TRILINEAR)) ? 1 : K;
#pragma unroll kRevUnroll
      for (int k = K - 1; k >= 0; --k) {
        Real vk[4], tk;
        uint32_t bk;
#pragma unroll
        for (int kk = 0; kk < K; ++kk) {
          if (kk == k) {
            vk[0] = v[kk][0]; vk[1] = v[kk][1]; vk[2] = v[kk][2]; vk[3] = v[kk][3];
            bk = bits[kk];
            tk = Ts[kk];
          }
        }
        // a slot with alpha 0 and nothing to scatter leaves S unchanged (identity maps)
        if (PGB_SLOT_SKIP && !__any_sync(kFull, bk != 0u || vk[3] != Real(0))) continue;
        const Real al = vk[3];
        const Real G = gpx[0] * vk[0] + gpx[1] * vk[1] + gpx[2] * vk[2] + gpx[3];
        Real fa = G * al, fb = Real(1) - al;
        warp_suffix_affine(fa, fb, lane);
        const Real S_here = fa + fb * Snext_carry;          // S_s for this lane's sample
        Real S_after = __shfl_down_sync(kFull, S_here, 1);  // S_{s+1}
        if (lane == kWarp - 1) S_after = Snext_carry;
        Snext_carry = __shfl_sync(kFull, S_here, 0);
        if (bk != 0u) {
          const Real w = al * tk;
          Real dv[4];
          dv[0] = gpx[0] * w;
          dv[1] = gpx[1] * w;
          dv[2] = gpx[2] * w;
          dv[3] = tk * (G - S_after);
          if (with_beta) {  // d/dalpha of log(alpha + e) - log(1 - alpha + e), one division
            const Real e = (Real)a.beta_eps;
            dv[3] += beta_scale / ((al + e) * (Real(1) - al + e));
          }
          // behind an opaque sample (T = 0) every partial is 0 and no corner would be written
          if (PGB_SKIP_ZERO_DV &&
              !(dv[0] != Real(0) || dv[1] != Real(0) || dv[2] != Real(0) || dv[3] != Real(0)))
            continue;
          Real nx, ny, nz;
          if constexpr (RenderStage<Real, K, LOGT>::kHasCoords)
            cs.get(c, k, lane, nx, ny, nz);
          else
            sample_coords(a, ray, (c * K + k) * kWarp + lane, nx, ny, nz);
          sample_scatter<Real, MODE>(a.g, a.grad, nx, ny, nz, dv, bk, a.grad_marks);
        }
      }
    }
  }

  if (PHASE == kTrain) {
    // deterministic loss without a barrier: warps count themselves out in shared memory,
    // the block's last warp sums the block in warp order and takes one global ticket, and
    // the last block sums the blocks in block order
    const int wib = threadIdx.x >> 5;
    unsigned last_warp = 0;
    if (with_beta) beta_lane = warp_sum(beta_lane);
    if (lane == 0) {
      loss_lane.store_volatile(&s_part[wib]);
      beta_lane.store_volatile(&s_part_beta[wib]);
      __threadfence_block();
      last_warp = atomicAdd(&s_done, 1u) == (unsigned)warps_per_block - 1u;
    }
    last_warp = __shfl_sync(kFull, last_warp, 0);
    if (last_warp) {
      unsigned last_block = 0;
      if (lane == 0) {
        __threadfence_block();
        LossSum<Real> sum, bsum;
        for (int i = 0; i < warps_per_block; ++i) {
          sum.add(LossSum<Real>::load_volatile(&s_part[i]));
          bsum.add(LossSum<Real>::load_volatile(&s_part_beta[i]));
        }
        sum.store(a.partials + blockIdx.x);
        if (with_beta) bsum.store(a.partials_beta + blockIdx.x);
        __threadfence();
        last_block = atomicAdd(a.counter, 1u) == gridDim.x - 1u;
      }
      last_block = __shfl_sync(kFull, last_block, 0);
      if (last_block) {
        __threadfence();
        // block partials in block order, eight loads in flight per lane (L2 reads: the
        // partials were written by other blocks before their ticket)
        LossSum<Real> sum, bsum;
        for (unsigned i0 = lane; i0 < gridDim.x; i0 += 8 * kWarp) {
          LossSum<Real> p[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const unsigned i = i0 + u * kWarp;
            if (i < gridDim.x) p[u] = LossSum<Real>::load_cg(a.partials + i);
          }
#pragma unroll
          for (int u = 0; u < 8; ++u) sum.add(p[u]);
          if (with_beta) {
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              const unsigned i = i0 + u * kWarp;
              if (i < gridDim.x) p[u] = LossSum<Real>::load_cg(a.partials_beta + i);
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) bsum.add(p[u]);
          }
        }
        sum = warp_sum(sum);
        if (with_beta) bsum = warp_sum(bsum);
        if (lane == 0) {
          a.loss_out[0] = (Real)(a.loss_w * sum.value() * a.inv_count);
          if (with_beta) a.loss_out[1] = (Real)(a.beta_w * bsum.value() * a.inv_samples);
          *a.counter = 0u;
        }
      }
    }
  }
}

}  // namespace pgb
