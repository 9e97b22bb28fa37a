// Batched form of the fused training step: many scenes of different sizes, rays of
// uneven cost (empty-space skipping, early termination), one persistent launch.
//
// Work distribution: a persistent grid whose warps pull rays from a global queue (one
// atomic per ray), so rays that terminate early or cross empty space free their warp for
// the next ray. Per ray the work is the fused training step of render.cuh (sampling,
// lookup, compositing, MSE gradient, division-free adjoint), on the ray's own scene.
//
// Empty-space skipping: a sample is skipped (value 0, no gradient) when the brick of its
// floor corner is clear in the scene's dilated brick mask, i.e. all eight trilinear
// corners (and the nearest cell) are unoccupied. Unoccupied cells are zero and are not
// parameters, so skipping changes neither the rendered value nor the gradient of any
// occupied cell. Samples whose floor corner sits on an upper face (where the ceil corner
// wraps to index 0) are never skipped.
#include <algorithm>

// Warps of the persistent kernel sit in different phases (gather, scan, scatter) of
// different rays, so the whole kernel body competes for the instruction cache: the
// per-sample gather and scatter must exist once, not once per unrolled slot (unrolled
// inline copies measured 1.66x slower). PGB_BATCH_LOOP=1 keeps one inline copy of each in
// a slot loop that is not unrolled, moving each slot's values in and out of the register
// arrays by compile-time selects; PGB_BATCH_LOOP=0 calls out-of-line functions instead,
// whose reference arguments and saved registers go through the stack.
#ifndef PGB_BATCH_LOOP
#define PGB_BATCH_LOOP 1
#endif
#ifndef PGB_SCATTER_INLINE
#define PGB_SCATTER_INLINE PGB_BATCH_LOOP
#endif
#ifndef PGB_BATCH_GATHER_INLINE
#define PGB_BATCH_GATHER_INLINE PGB_BATCH_LOOP
#endif
// Resident 256-thread blocks per SM the register allocation must allow. With 32-sample
// chunks (K = 1) a cap of 80 registers for a third block spills a little and measured
// faster (64-scene step 7.32 -> 6.78 ms); longer chunks keep two blocks (their spills
// at 80 registers cost more than the extra warps give).
#ifndef PGB_BATCH_MIN_BLOCKS_K1
#define PGB_BATCH_MIN_BLOCKS_K1 3
#endif
#ifndef PGB_BATCH_MIN_BLOCKS
#define PGB_BATCH_MIN_BLOCKS 2
#endif
// Skip the transmittance and adjoint scans of slots with nothing in them (exact).
#ifndef PGB_SLOT_SKIP
#define PGB_SLOT_SKIP 1
#endif

#include "pgb_host.h"
#include "render.cuh"

namespace pgb {
namespace {

constexpr int kMaxScenes = 256;
constexpr int kBatchMaxThreads = 256;

struct BatchArgs {
  const pgb_scene* scenes;
  int num_scenes;
  int clip;
  const float* origins;
  const float* dirs;
  const float* target;
  const int32_t* ray_scene;
  int64_t R;
  float term_thr;
  int stratified;
  uint64_t seed;
  double loss_w;
  double inv_count;
  float grad_scale;          // 2 * loss_w * inv_count, rounded on the host
  float* rgba_out;
  float* loss_out;
  unsigned long long* work;  // ray queue head
  unsigned* ticket;          // finished blocks
  float* ray_loss;           // [R] squared error per ray
};

// Workspace: the queue head (8 B), the finished-block ticket (4 B) and the loss sum's
// ticket (4 B) in the first 64 B, then the loss sum's block partials, then one float per
// ray.
constexpr int kLossBlocks = 1024;
constexpr int64_t kLossPartialsOffset = 64;
constexpr int64_t kRayLossOffset = kLossPartialsOffset + 8 * kLossBlocks;

__device__ __forceinline__ bool brick_clear(const pgb_scene& sc, float nx, float ny, float nz) {
  if (sc.bricks == nullptr) return false;
  if (!(nx >= 0.f && ny >= 0.f && nz >= 0.f)) return false;
  const int fx = (int)floorf(nx), fy = (int)floorf(ny), fz = (int)floorf(nz);
  if (fx >= sc.dims[0] - 1 || fy >= sc.dims[1] - 1 || fz >= sc.dims[2] - 1) return false;
  const int L = sc.brick_log2;
  const uint32_t b = ((uint32_t)(fx >> L) * (uint32_t)sc.brick_dims[1] + (uint32_t)(fy >> L)) *
                         (uint32_t)sc.brick_dims[2] + (uint32_t)(fz >> L);
  return ((__ldg(sc.bricks + (b >> 5)) >> (b & 31u)) & 1u) == 0u;
}

__device__ __forceinline__ uint32_t cell_occupied(const pgb_scene& sc, uint64_t c) {
  return (__ldg(sc.occupancy + (c >> 5)) >> (uint32_t)(c & 31u)) & 1u;
}

// Clears the gradient-pass bits of a sample's corners that are not occupied (unoccupied
// cells are not parameters), in the bit layout of sample_value.
template <int MODE>
__device__ __forceinline__ uint32_t occupied_bits(const pgb_scene& sc, const GridP<float>& g,
                                                  float nx, float ny, float nz, uint32_t bits) {
  if (sc.occupancy == nullptr || bits == 0u) return bits;
  if (MODE == PGB_NEAREST) {
    const uint64_t c = cell_index(g, (int)rintf(nx), (int)rintf(ny), (int)rintf(nz));
    return cell_occupied(sc, c) ? bits : 0u;
  }
  Corners<float> q;
  trilinear_corners(g, nx, ny, nz, q);
#pragma unroll
  for (int corner = 0; corner < 8; ++corner) {
    const int ix = (corner & 4) ? q.f[0] : q.c[0];
    const int iy = (corner & 2) ? q.f[1] : q.c[1];
    const int iz = (corner & 1) ? q.f[2] : q.c[2];
    if (!cell_occupied(sc, cell_index(g, ix, iy, iz))) bits &= ~(0xfu << (4 * corner));
  }
  return bits;
}

#if PGB_BATCH_GATHER_INLINE
#define PGB_BATCH_GATHER_ATTR __device__ __forceinline__
#else
#define PGB_BATCH_GATHER_ATTR __device__ __noinline__
#endif

// One sample of a batched ray: coordinates, the brick test and, unless skipped, the value
// and its gradient-pass bits (occupancy folded in). Returns whether it was looked up.
template <typename Store, int MODE>
PGB_BATCH_GATHER_ATTR bool batch_sample(const RenderArgs<float>& ra, const Ray<float>& ray,
                                        const pgb_scene& sc, int s, float v[4], uint32_t& bits,
                                        float& nx, float& ny, float& nz) {
  v[0] = v[1] = v[2] = v[3] = 0.f;
  bits = 0u;
  if (s >= ra.S) return false;
  sample_coords(ra, ray, s, nx, ny, nz);
  if (brick_clear(sc, nx, ny, nz)) return false;
  sample_value<float, Store, MODE>(ra.g, nx, ny, nz, v, bits);
  bits = occupied_bits<MODE>(sc, ra.g, nx, ny, nz, bits);
  return true;
}

// The batched kernel's stage at 32-sample chunks: the values and clamp bits of the last
// PGB_BATCH_STAGE_CHUNKS chunks, with the coordinates recomputed from the ray in the
// reverse pass when PGB_BATCH_STAGE_COORDS is 0 (as the single-scene kernel does).
#ifndef PGB_BATCH_STAGE_CHUNKS
#define PGB_BATCH_STAGE_CHUNKS 8
#endif
#ifndef PGB_BATCH_STAGE_COORDS
#define PGB_BATCH_STAGE_COORDS 0
#endif
template <int K>
using BatchStage = ChunkStage<float, K, (K == 1 ? PGB_BATCH_STAGE_CHUNKS : 1),
                              (K != 1 || PGB_BATCH_STAGE_COORDS != 0)>;

// MERGE: the trilinear scatter merges the warp's updates of the same cell
// (warp_merged_scatter) before its atomics.
template <typename Store, int MODE, int K, bool MERGE>
__global__ void __launch_bounds__(kBatchMaxThreads, K == 1 ? PGB_BATCH_MIN_BLOCKS_K1 : PGB_BATCH_MIN_BLOCKS)
    batch_train_kernel(const BatchArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  pgb_scene* sc_tab = reinterpret_cast<pgb_scene*>(smem_raw);
  const size_t tab_bytes = ((size_t)a.num_scenes * sizeof(pgb_scene) + 15) & ~(size_t)15;
  {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(a.scenes);
    uint32_t* dst = reinterpret_cast<uint32_t*>(smem_raw);
    const int words = (int)((size_t)a.num_scenes * sizeof(pgb_scene) / 4);
    for (int i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
  const int lane = threadIdx.x & (kWarp - 1);
  const int wib = threadIdx.x >> 5;
  BatchStage<K> cs(smem_raw + tab_bytes, wib);
  const float grad_scale = a.grad_scale;  // d(weighted MSE)/d pixel

  for (;;) {
    unsigned long long rr = 0;
    if (lane == 0) rr = atomicAdd(a.work, 1ull);
    rr = __shfl_sync(kFull, rr, 0);
    if ((int64_t)rr >= a.R) break;
    const int64_t r = (int64_t)rr;
    const int sid = a.ray_scene[r];
    if ((unsigned)sid >= (unsigned)a.num_scenes) {  // not a scene of this batch: no work
      if (lane == 0) a.ray_loss[r] = 0.f;
      if (a.rgba_out != nullptr && lane < 4) a.rgba_out[4 * r + lane] = 0.f;
      continue;
    }
    const pgb_scene& sc = sc_tab[sid];

    // the ray's scene as the single-scene kernels see it
    RenderArgs<float> ra = {};
    ra.g.cells = sc.cells;
    ra.g.X = sc.dims[0]; ra.g.Y = sc.dims[1]; ra.g.Z = sc.dims[2];
    ra.g.fX = (float)ra.g.X; ra.g.fY = (float)ra.g.Y; ra.g.fZ = (float)ra.g.Z;
    ra.g.ox = sc.origin[0]; ra.g.oy = sc.origin[1]; ra.g.oz = sc.origin[2];
    ra.g.pd = sc.points_distance;
    ra.g.clip = a.clip;
    ra.S = sc.num_samples;
    ra.delta = sc.delta_step;
    ra.stratified = a.stratified;
    ra.strat_seed = a.seed;
    float* grad = reinterpret_cast<float*>(sc.grad_cells);

    Ray<float> ray;
    ray.ox = a.origins[3 * r + 0]; ray.oy = a.origins[3 * r + 1]; ray.oz = a.origins[3 * r + 2];
    ray.dx = a.dirs[3 * r + 0];    ray.dy = a.dirs[3 * r + 1];    ray.dz = a.dirs[3 * r + 2];
#pragma unroll
    for (int c = 0; c < 4; ++c) ray.tgt[c] = a.target[4 * r + c];
    ray.h = a.stratified ? hash_stream(a.seed, (uint64_t)r) : 0ull;

    const int nchunks = (ra.S + kWarp * K - 1) / (kWarp * K);
    if (nchunks > kWarp) {  // a chunk start per lane: more chunks are not supported
      if (lane == 0) a.ray_loss[r] = __int_as_float(0x7fc00000);  // NaN loss
      if (a.rgba_out != nullptr && lane < 4) a.rgba_out[4 * r + lane] = __int_as_float(0x7fc00000);
      continue;
    }
    float v[K][4];
    uint32_t bits[K];
    float Ts[K];
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    float T = 1.f, Tstart = 1.f;
    int last = -1;

    auto gather = [&](int c) {
#if PGB_BATCH_LOOP
#pragma unroll 1
      for (int k = 0; k < K; ++k) {
        float t[4], nx, ny, nz;
        uint32_t b;
        if (batch_sample<Store, MODE>(ra, ray, sc, (c * K + k) * kWarp + lane, t, b, nx, ny, nz))
          cs.put(c, k, lane, nx, ny, nz);
#pragma unroll
        for (int kk = 0; kk < K; ++kk) {
          if (kk == k) {
            v[kk][0] = t[0]; v[kk][1] = t[1]; v[kk][2] = t[2]; v[kk][3] = t[3];
            bits[kk] = b;
          }
        }
      }
#else
#pragma unroll
      for (int k = 0; k < K; ++k) {
        float nx, ny, nz;
        if (batch_sample<Store, MODE>(ra, ray, sc, (c * K + k) * kWarp + lane, v[k], bits[k], nx, ny, nz))
          cs.put(c, k, lane, nx, ny, nz);
      }
#endif
    };

    for (int c = 0; c < nchunks; ++c) {
      if (lane == c) Tstart = T;
      __syncwarp();
      gather(c);
#pragma unroll
      for (int k = 0; k < K; ++k) cs.put_vals(c, k, lane, v[k], bits[k]);
      T = scan_chunk<float, K>(v, T, lane, Ts);
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const float w = v[k][3] * Ts[k];
        acc[0] += w * v[k][0];
        acc[1] += w * v[k][1];
        acc[2] += w * v[k][2];
        acc[3] += w;
      }
      last = c;
      if (a.term_thr > 0.0f && T < a.term_thr) break;
    }
    float px[4];
#pragma unroll
    for (int ch = 0; ch < 4; ++ch) px[ch] = warp_sum(acc[ch]);
    float gpx[4];
    float sq = 0.f;
#pragma unroll
    for (int ch = 0; ch < 4; ++ch) {
      const float diff = px[ch] - ray.tgt[ch];
      sq += diff * diff;
      gpx[ch] = grad_scale * diff;
    }
    if (lane == 0) a.ray_loss[r] = sq;
    if (a.rgba_out != nullptr && lane < 4) a.rgba_out[4 * r + lane] = pick4(px, lane);

    float Snext_carry = 0.f;
    for (int c = last; c >= 0; --c) {
      if (c != last) {
        __syncwarp();
        if (BatchStage<K>::holds(c, last)) {  // the chunk's values are still staged
#pragma unroll
          for (int k = 0; k < K; ++k) cs.get_vals(c, k, lane, v[k], bits[k]);
        } else {
          gather(c);
        }
        scan_chunk<float, K>(v, __shfl_sync(kFull, Tstart, c), lane, Ts);
      }
      __syncwarp();
#if PGB_BATCH_LOOP
#pragma unroll 1
#else
#pragma unroll
#endif
      for (int k = K - 1; k >= 0; --k) {
        float vk[4], tk;
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
        if (PGB_SLOT_SKIP && !__any_sync(kFull, bk != 0u || vk[3] != 0.f)) continue;
        const float al = vk[3];
        const float G = gpx[0] * vk[0] + gpx[1] * vk[1] + gpx[2] * vk[2] + gpx[3];
        float fa = G * al, fb = 1.f - al;
        warp_suffix_affine(fa, fb, lane);
        const float S_here = fa + fb * Snext_carry;
        float S_after = __shfl_down_sync(kFull, S_here, 1);
        if (lane == kWarp - 1) S_after = Snext_carry;
        Snext_carry = __shfl_sync(kFull, S_here, 0);
        if (MERGE && MODE == PGB_TRILINEAR) {
          float dv[4] = {0.f, 0.f, 0.f, 0.f};
          float nx = 0.f, ny = 0.f, nz = 0.f;
          bool has = false;
          if (bk != 0u) {
            const float w = al * tk;
            dv[0] = gpx[0] * w; dv[1] = gpx[1] * w; dv[2] = gpx[2] * w;
            dv[3] = tk * (G - S_after);
            has = dv[0] != 0.f || dv[1] != 0.f || dv[2] != 0.f || dv[3] != 0.f;
            if (has) {
              if constexpr (BatchStage<K>::kHasCoords)
                cs.get(c, k, lane, nx, ny, nz);
              else
                sample_coords(ra, ray, (c * K + k) * kWarp + lane, nx, ny, nz);
            }
          }
          warp_merged_scatter<float>(ra.g, grad, has, nx, ny, nz, dv, bk, lane);
        } else if (bk != 0u) {
          const float w = al * tk;
          float dv[4] = {gpx[0] * w, gpx[1] * w, gpx[2] * w, tk * (G - S_after)};
          if (!(dv[0] != 0.f || dv[1] != 0.f || dv[2] != 0.f || dv[3] != 0.f)) continue;
          float nx, ny, nz;
          if constexpr (BatchStage<K>::kHasCoords)
            cs.get(c, k, lane, nx, ny, nz);
          else
            sample_coords(ra, ray, (c * K + k) * kWarp + lane, nx, ny, nz);
          sample_scatter<float, MODE>(ra.g, grad, nx, ny, nz, dv, bk);
        }
      }
    }
  }

  // the last block to finish resets the queue (ray_loss_sum_kernel, launched next, sums
  // the per-ray losses)
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(a.ticket, 1u) == gridDim.x - 1u) {
      *a.work = 0ull;
      *a.ticket = 0u;
    }
  }
}

// The weighted MSE from the per-ray squared errors, in a fixed order: block b adds rays
// [b * seg, (b + 1) * seg) (thread-strided, then a tree), and the last block to finish
// adds the block sums in block order. Every SM takes a share of the fp64 adds (GB300's
// fp64 rate is low), instead of one block adding all rays.
__global__ void __launch_bounds__(256) ray_loss_sum_kernel(const float* __restrict__ ray_loss,
                                                           int64_t R, int64_t seg,
                                                           double* __restrict__ partials,
                                                           unsigned* ticket, float* loss_out,
                                                           double loss_w, double inv_count) {
  __shared__ double red[256];
  __shared__ unsigned s_last;
  const int64_t lo = (int64_t)blockIdx.x * seg;
  const int64_t hi = lo + seg < R ? lo + seg : R;
  double sum = 0.0;
  for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) sum += (double)ray_loss[i];
  red[threadIdx.x] = sum;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = red[0];
    __threadfence();
    s_last = atomicAdd(ticket, 1u) == gridDim.x - 1u;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  double t = 0.0;
  for (unsigned i = threadIdx.x; i < gridDim.x; i += blockDim.x) t += __ldcg(partials + i);
  red[threadIdx.x] = t;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    loss_out[0] = (float)(loss_w * red[0] * inv_count);
    *ticket = 0u;
  }
}

// --------------------------------------------------------------- brick masks
__global__ void pack_mask_kernel(const uint8_t* __restrict__ m, int64_t count, uint32_t* __restrict__ out) {
  const int64_t words = (count + 31) / 32;
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < words;
       w += (int64_t)gridDim.x * blockDim.x) {
    uint32_t b = 0u;
    for (int i = 0; i < 32; ++i) {
      const int64_t c = w * 32 + i;
      if (c < count && m[c]) b |= 1u << i;
    }
    out[w] = b;
  }
}

// Dilated brick mask straight from the cell bits: thread b scans the cells of bricks
// b + {0,1}^3 (2^(L+1) cells per axis, clamped to the grid); a warp ballot assembles 32
// bricks into one mask word.
__global__ void build_bricks_kernel(const uint32_t* __restrict__ cell_bits, int X, int Y, int Z,
                                    int L, int BX, int BY, int BZ, uint32_t* __restrict__ out) {
  const int64_t NB = (int64_t)BX * BY * BZ;
  const int64_t words = (NB + 31) / 32;
  const int lane = threadIdx.x & 31;
  for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < words;
       w += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int64_t b = w * 32 + lane;
    bool any = false;
    if (b < NB) {
      const int bz = (int)(b % BZ);
      const int64_t bxy = b / BZ;
      const int by = (int)(bxy % BY), bx = (int)(bxy / BY);
      const int x0 = bx << L, x1 = min(X, (bx + 2) << L);
      const int y0 = by << L, y1 = min(Y, (by + 2) << L);
      const int z0 = bz << L, z1 = min(Z, (bz + 2) << L);  // cells [z0, z1) of each row
      for (int x = x0; x < x1 && !any; ++x) {
        for (int y = y0; y < y1 && !any; ++y) {
          const int64_t c0 = ((int64_t)x * Y + y) * Z + z0, c1 = c0 + (z1 - z0);  // [c0, c1)
          for (int64_t wd = c0 >> 5; wd <= (c1 - 1) >> 5 && !any; ++wd) {
            uint32_t m = 0xffffffffu;
            if (wd == (c0 >> 5)) m &= 0xffffffffu << (c0 & 31);
            if (wd == ((c1 - 1) >> 5)) m &= 0xffffffffu >> (31 - ((c1 - 1) & 31));
            any = (__ldg(cell_bits + wd) & m) != 0u;
          }
        }
      }
    }
    const uint32_t word = __ballot_sync(0xffffffffu, any);
    if (lane == 0) out[w] = word;
  }
}

__global__ void batch_zero_kernel(const pgb_scene* __restrict__ scenes) {
  const pgb_scene sc = scenes[blockIdx.y];
  const int64_t cells = (int64_t)sc.dims[0] * sc.dims[1] * sc.dims[2];  // one float4 per cell
  uint4* p = reinterpret_cast<uint4*>(sc.grad_cells);
  if (sc.occupancy == nullptr) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cells;
         i += (int64_t)gridDim.x * blockDim.x)
      p[i] = make_uint4(0u, 0u, 0u, 0u);
    return;
  }
  // only occupied cells ever receive gradient: clear those
  const int64_t words = (cells + 31) / 32;
  for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < words;
       w += (int64_t)gridDim.x * blockDim.x) {
    uint32_t bits = __ldg(sc.occupancy + w);
    while (bits) {
      const int i = __ffs(bits) - 1;
      bits &= bits - 1;
      const int64_t c = w * 32 + i;
      if (c < cells) p[c] = make_uint4(0u, 0u, 0u, 0u);
    }
  }
}

inline unsigned grid_for(int64_t n, int threads = 256) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + threads - 1) / threads, 1 << 20));
}

template <typename Store, int MODE, int K, bool MERGE>
int launch_batch_k(const BatchArgs& a, int threads, cudaStream_t s) {
  const int warps = threads / kWarp;
  const size_t tab = (((size_t)a.num_scenes * sizeof(pgb_scene)) + 15) & ~(size_t)15;
  const size_t smem = tab + (size_t)BatchStage<K>::kBytesPerWarp * warps;
  auto kern = batch_train_kernel<Store, MODE, K, MERGE>;
  int dev = 0;
  cudaGetDevice(&dev);
  static int configured[64] = {0};
  if (dev >= 0 && dev < 64 && !configured[dev]) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024) != cudaSuccess)
      return PGB_ERR_LAUNCH;
    configured[dev] = 1;
  }
  int sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem) != cudaSuccess ||
      per_sm < 1)
    return PGB_ERR_LAUNCH;
  int64_t blocks = (int64_t)sms * per_sm;
  blocks = std::min<int64_t>(blocks, (a.R + warps - 1) / warps);
  blocks = std::max<int64_t>(blocks, 1);
  kern<<<(unsigned)blocks, threads, smem, s>>>(a);
  return after_launch();
}

template <typename Store, int MODE, bool MERGE>
int launch_batch_km(const BatchArgs& a, int K, int threads, cudaStream_t s) {
  switch (K) {
    case 1: return launch_batch_k<Store, MODE, 1, MERGE>(a, threads, s);
    case 2: return launch_batch_k<Store, MODE, 2, MERGE>(a, threads, s);
    case 4: return launch_batch_k<Store, MODE, 4, MERGE>(a, threads, s);
    case 8: return launch_batch_k<Store, MODE, 8, MERGE>(a, threads, s);
    default: return PGB_ERR_ARG;
  }
}

template <typename Store, int MODE>
int launch_batch_m(const BatchArgs& a, int K, int threads, int merge, cudaStream_t s) {
  // nearest lookup scatters one cell per sample: no merged form
  if (merge && MODE == PGB_TRILINEAR) return launch_batch_km<Store, MODE, true>(a, K, threads, s);
  return launch_batch_km<Store, MODE, false>(a, K, threads, s);
}

}  // namespace
}  // namespace pgb

using namespace pgb;

extern "C" {

int64_t pgb_batch_workspace_bytes(int64_t num_rays) {
  return kRayLossOffset + 4 * std::max<int64_t>(num_rays, 1);
}

int pgb_batch_train(const pgb_scene* scenes, int32_t num_scenes, int32_t dtype, int32_t mode,
                    int32_t clip, const float* origins, const float* dirs, const float* target,
                    const int32_t* ray_scene, int64_t num_rays, float term_threshold,
                    int32_t stratified, uint64_t seed, double loss_weight, float* rgba_out,
                    float* loss_out, void* workspace, int32_t slots_per_lane,
                    int32_t threads_per_block, int32_t merge_updates, pgb_stream_t stream) {
  if (!scenes || num_scenes <= 0 || num_scenes > kMaxScenes || num_rays < 0) return PGB_ERR_ARG;
  if (dtype != PGB_F32 && dtype != PGB_BF16) return PGB_ERR_UNSUPPORTED;
  if (mode != PGB_NEAREST && mode != PGB_TRILINEAR) return PGB_ERR_ARG;
  if (!loss_out || !workspace) return PGB_ERR_ARG;
  if (num_rays > 0 && (!origins || !dirs || !target || !ray_scene)) return PGB_ERR_ARG;
  if (((uintptr_t)workspace % 16) != 0) return PGB_ERR_ALIGN;
  const int K = slots_per_lane == 0 ? 2 : slots_per_lane;
  const int threads = threads_per_block == 0 ? 256 : threads_per_block;
  if (K != 1 && K != 2 && K != 4 && K != 8) return PGB_ERR_ARG;
  if (threads != 128 && threads != 256) return PGB_ERR_ARG;
  BatchArgs a = {};
  a.scenes = scenes;
  a.num_scenes = num_scenes;
  a.clip = clip ? 1 : 0;
  a.origins = origins;
  a.dirs = dirs;
  a.target = target;
  a.ray_scene = ray_scene;
  a.R = num_rays;
  a.term_thr = term_threshold;
  a.stratified = stratified ? 1 : 0;
  a.seed = seed;
  a.loss_w = loss_weight;
  a.inv_count = num_rays > 0 ? 1.0 / (4.0 * (double)num_rays) : 0.0;
  a.grad_scale = (float)(2.0 * a.loss_w * a.inv_count);
  a.rgba_out = rgba_out;
  a.loss_out = loss_out;
  a.work = reinterpret_cast<unsigned long long*>(workspace);
  a.ticket = reinterpret_cast<unsigned*>((char*)workspace + 8);
  a.ray_loss = reinterpret_cast<float*>((char*)workspace + kRayLossOffset);
  const int merge = merge_updates ? 1 : 0;
  int st;
  if (dtype == PGB_BF16)
    st = mode == PGB_NEAREST
             ? launch_batch_m<__nv_bfloat16, PGB_NEAREST>(a, K, threads, merge, stream)
             : launch_batch_m<__nv_bfloat16, PGB_TRILINEAR>(a, K, threads, merge, stream);
  else
    st = mode == PGB_NEAREST ? launch_batch_m<float, PGB_NEAREST>(a, K, threads, merge, stream)
                             : launch_batch_m<float, PGB_TRILINEAR>(a, K, threads, merge, stream);
  if (st != PGB_OK) return st;
  // about 1024 rays per block, at most kLossBlocks blocks
  const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(kLossBlocks, (num_rays + 1023) / 1024));
  const int64_t seg = (num_rays + blocks - 1) / blocks;
  ray_loss_sum_kernel<<<(unsigned)blocks, 256, 0, stream>>>(
      a.ray_loss, num_rays, seg, reinterpret_cast<double*>((char*)workspace + kLossPartialsOffset),
      reinterpret_cast<unsigned*>((char*)workspace + 12), loss_out, a.loss_w, a.inv_count);
  return after_launch();
}

int pgb_pack_mask(const uint8_t* mask, int64_t count, uint32_t* bits_out, pgb_stream_t stream) {
  if (count < 0) return PGB_ERR_ARG;
  if (count == 0) return PGB_OK;
  if (!mask || !bits_out) return PGB_ERR_ARG;
  pack_mask_kernel<<<grid_for((count + 31) / 32), 256, 0, stream>>>(mask, count, bits_out);
  return after_launch();
}

int pgb_build_bricks(const uint32_t* cell_bits, const int32_t dims[3], int32_t brick_log2,
                     uint32_t* bricks_out, pgb_stream_t stream) {
  if (!cell_bits || !dims || !bricks_out || brick_log2 < 0 || brick_log2 > 8) return PGB_ERR_ARG;
  if (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return PGB_ERR_ARG;
  const int L = brick_log2;
  const int BX = (dims[0] + (1 << L) - 1) >> L, BY = (dims[1] + (1 << L) - 1) >> L,
            BZ = (dims[2] + (1 << L) - 1) >> L;
  const int64_t words = ((int64_t)BX * BY * BZ + 31) / 32;
  // whole warps per mask word: the grid-stride loop runs over warps
  const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>((words * 32 + 255) / 256, 1 << 16));
  build_bricks_kernel<<<blocks, 256, 0, stream>>>(cell_bits, dims[0], dims[1], dims[2], L, BX, BY,
                                                  BZ, bricks_out);
  return after_launch();
}

int pgb_batch_zero_grads(const pgb_scene* scenes, int32_t num_scenes, int64_t max_cells,
                         pgb_stream_t stream) {
  if (!scenes || num_scenes <= 0 || num_scenes > 65535 || max_cells < 0) return PGB_ERR_ARG;
  const dim3 grid(std::max(1u, std::min(grid_for(max_cells), 4096u)), (unsigned)num_scenes);
  batch_zero_kernel<<<grid, 256, 0, stream>>>(scenes);
  return after_launch();
}

}  // extern "C"
