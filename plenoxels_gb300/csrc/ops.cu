// Drop-in operator kernels: one kernel (or a short chain) per reference function, with
// the reference's tensor semantics (shapes, index order, wrap and mask rules). The fused
// kernels in render.cuh compose the same arithmetic without materialising anything.
#include <algorithm>

#include "pgb_host.h"
#include "render.cuh"

namespace pgb {

namespace {

constexpr int kThreads = 256;

inline unsigned blocks_for(int64_t n, int per_thread = 1) {
  int64_t b = (n + (int64_t)kThreads * per_thread - 1) / ((int64_t)kThreads * per_thread);
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)1 << 22));
}

// grid-stride loop helper
#define PGB_FOR(i, n)                                                            \
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (n);     \
       i += (int64_t)gridDim.x * blockDim.x)

// --------------------------------------------------------------- ray generation
// src/ray_sampling.py:195-264. One thread per ray (camera-major).
__global__ void generate_rays_kernel(const float* __restrict__ T, int C, int64_t Rc, float fov,
                                     const float* __restrict__ images, int H, int W,
                                     const float* __restrict__ uv, int even_side,
                                     float* __restrict__ dirs, float* __restrict__ pixels,
                                     int* __restrict__ status) {
  const int64_t total = (int64_t)C * Rc;
  PGB_FOR(r, total) {
    const int c = (int)(r / Rc);
    const int64_t i = r - (int64_t)c * Rc;
    float u, v;
    if (uv != nullptr) {
      u = uv[2 * r];
      v = uv[2 * r + 1];
    } else {
      // torch.linspace(0, 1, n) (fp32 step, upper half counted back from the end) and
      // torch.cartesian_prod(l, l): ray i = (l[i / n], l[i % n]).
      const int n = even_side;
      const int64_t iu = i / n, iv = i - iu * n;
      if (n == 1) {
        u = 0.0f;
        v = 0.0f;
      } else {
        const float step = rdiv(1.0f, (float)(n - 1));
        const int half = n / 2;
        u = iu < half ? rmul(step, (float)iu) : rfma(-step, (float)(n - 1 - iu), 1.0f);
        v = iv < half ? rmul(step, (float)iv) : rfma(-step, (float)(n - 1 - iv), 1.0f);
      }
    }
    float d[3];
    camera_direction(T + 16 * (int64_t)c, fov, u, v, d);
    dirs[3 * r + 0] = d[0];
    dirs[3 * r + 1] = d[1];
    dirs[3 * r + 2] = d[2];
    int row, col;
    camera_pixel(H, W, u, v, row, col);
    // torch indexing: a negative index counts from the end; anything else outside the
    // image is an IndexError, reported through the status word (the access is skipped)
    if (row < 0) row += H;
    if (col < 0) col += W;
    if (row < 0 || row >= H || col < 0 || col >= W) {
      if (status) atomicOr(status, 1);
      reinterpret_cast<float4*>(pixels)[r] = make_float4(0.f, 0.f, 0.f, 0.f);
      continue;
    }
    const float4 px = __ldg(reinterpret_cast<const float4*>(images) + (((int64_t)c * H + row) * W + col));
    reinterpret_cast<float4*>(pixels)[r] = px;
  }
}

// src/ray_sampling.py:159-167: sample (r, k) = position(camera of r) + dirs[r] * (delta * k).
__global__ void sample_points_kernel(const float* __restrict__ T, int64_t Rc, int S,
                                     const float* __restrict__ dirs, float delta, int64_t total,
                                     float* __restrict__ out) {
  PGB_FOR(i, total) {
    const int64_t r = i / S;
    const int k = (int)(i - r * S) + 1;
    const int c = (int)(r / Rc);
    const float t = rmul(delta, (float)k);
    const float* P = T + 16 * (int64_t)c;
    out[3 * i + 0] = radd(P[3], rmul(dirs[3 * r + 0], t));
    out[3 * i + 1] = radd(P[7], rmul(dirs[3 * r + 1], t));
    out[3 * i + 2] = radd(P[11], rmul(dirs[3 * r + 2], t));
  }
}

// --------------------------------------------------------------- min reduction
// Order-preserving map of float bits to signed int (so integer min == float min).
__device__ __forceinline__ int float_to_ordered(float f) {
  const int i = __float_as_int(f);
  return i >= 0 ? i : (i ^ 0x7fffffff);
}
__device__ __forceinline__ float ordered_to_float(int i) {
  return __int_as_float(i >= 0 ? i : (i ^ 0x7fffffff));
}

__global__ void min_init_kernel(int* out) {
  if (threadIdx.x < 3) out[threadIdx.x] = float_to_ordered(__int_as_float(0x7f800000));  // +inf
}

// Per-axis minimum: a grid-stride pass (a few waves of blocks), warp and block
// reductions, then one ordered-int atomicMin per block and axis (same-address atomics
// from every warp serialised the reduction at ~0.2 ms for a 256^3 grid).
__global__ void __launch_bounds__(kThreads) coords_min_kernel(const float* __restrict__ coords,
                                                              int64_t count, int* out) {
  float m[3] = {__int_as_float(0x7f800000), __int_as_float(0x7f800000), __int_as_float(0x7f800000)};
  PGB_FOR(i, count) {
#pragma unroll
    for (int a = 0; a < 3; ++a) m[a] = fminf(m[a], __ldg(coords + 3 * i + a));
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) m[a] = fminf(m[a], __shfl_xor_sync(kFull, m[a], d));
  }
  __shared__ float part[kThreads / 32][3];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
#pragma unroll
    for (int a = 0; a < 3; ++a) part[warp][a] = m[a];
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      float x = lane < (int)(blockDim.x >> 5) ? part[lane][a] : __int_as_float(0x7f800000);
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) x = fminf(x, __shfl_xor_sync(kFull, x, d));
      if (lane == 0) atomicMin(out + a, float_to_ordered(x));
    }
  }
}

__global__ void min_finish_kernel(int* out) {
  if (threadIdx.x < 3) {
    const float f = ordered_to_float(out[threadIdx.x]);
    reinterpret_cast<float*>(out)[threadIdx.x] = f;
  }
}

// src/ray_sampling.py:13
__global__ void normalize_kernel(const float* __restrict__ samples, int64_t count,
                                 const float* __restrict__ gmin, float pd, float* __restrict__ out) {
  const float m0 = gmin[0], m1 = gmin[1], m2 = gmin[2];
  PGB_FOR(i, count) {
    out[3 * i + 0] = rdiv(rsub(samples[3 * i + 0], m0), pd);
    out[3 * i + 1] = rdiv(rsub(samples[3 * i + 1], m1), pd);
    out[3 * i + 2] = rdiv(rsub(samples[3 * i + 2], m2), pd);
  }
}

// --------------------------------------------------------------- index helpers
// Real -> int64 as torch's .to(torch.long) on an integral-valued float.
template <typename Real>
__device__ __forceinline__ long long to_i64(Real x) { return (long long)x; }

template <typename Real>
__device__ __forceinline__ void nearest_index(Real nx, Real ny, Real nz, const int dims[3],
                                              long long idx[3], bool& inb) {
  const Real n[3] = {nx, ny, nz};
  inb = true;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const long long i = to_i64(rround(n[a]));
    inb = inb && (i >= 0) && (i < dims[a]);
    idx[a] = floor_mod(i, dims[a]);
  }
}

template <typename Real>
__device__ __forceinline__ bool float_in_bounds(Real nx, Real ny, Real nz, const int dims[3]) {
  return nx < (Real)dims[0] && nx >= Real(0) && ny < (Real)dims[1] && ny >= Real(0) &&
         nz < (Real)dims[2] && nz >= Real(0);
}

// src/grid_functions.py:103-114
template <typename Real, typename Store>
__global__ void nearest_gather_kernel(GridP<Real> g, const Real* __restrict__ n, int64_t count,
                                      Real* __restrict__ vals, uint8_t* __restrict__ inb_out,
                                      int64_t* __restrict__ idx_out) {
  const int dims[3] = {g.X, g.Y, g.Z};
  PGB_FOR(i, count) {
    long long idx[3];
    bool inb;
    nearest_index(n[3 * i], n[3 * i + 1], n[3 * i + 2], dims, idx, inb);
    Real cv[4];
    CellIO<Store>::load(g.cells, cell_index(g, (int)idx[0], (int)idx[1], (int)idx[2]), cv);
#pragma unroll
    for (int ch = 0; ch < 4; ++ch) vals[4 * i + ch] = g.clip ? clamp01(cv[ch]) : cv[ch];
    if (inb_out) inb_out[i] = inb ? 1 : 0;
    if (idx_out) {
      idx_out[3 * i + 0] = idx[0];
      idx_out[3 * i + 1] = idx[1];
      idx_out[3 * i + 2] = idx[2];
    }
  }
}

template <typename Real, typename Store>
__global__ void nearest_scatter_kernel(GridP<Real> g, const Real* __restrict__ n, int64_t count,
                                       const Real* __restrict__ dv, Real* __restrict__ grad) {
  const int dims[3] = {g.X, g.Y, g.Z};
  PGB_FOR(i, count) {
    long long idx[3];
    bool inb;
    nearest_index(n[3 * i], n[3 * i + 1], n[3 * i + 2], dims, idx, inb);
    const uint64_t c = cell_index(g, (int)idx[0], (int)idx[1], (int)idx[2]);
    Real gv[4];
    bool any = false;
    if (g.clip) {
      Real cv[4];
      CellIO<Store>::load(g.cells, c, cv);
#pragma unroll
      for (int ch = 0; ch < 4; ++ch) gv[ch] = in01(cv[ch]) ? dv[4 * i + ch] : Real(0);
    } else {
#pragma unroll
      for (int ch = 0; ch < 4; ++ch) gv[ch] = dv[4 * i + ch];
    }
#pragma unroll
    for (int ch = 0; ch < 4; ++ch) any |= gv[ch] != Real(0);
    if (any) grad_add(grad, c, gv);
  }
}

// src/grid_functions.py:220-246: corners in the order x in {ceil, floor}, y in {ceil,
// floor}, z in {ceil, floor}; not wrapped.
template <typename Real>
__global__ void corner_indices_kernel(const Real* __restrict__ n, int64_t count,
                                      int64_t* __restrict__ out) {
  PGB_FOR(i, count) {
    long long c[3], f[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      c[a] = to_i64(rceil(n[3 * i + a]));
      f[a] = to_i64(rfloor(n[3 * i + a]));
    }
#pragma unroll
    for (int corner = 0; corner < 8; ++corner) {
      int64_t* o = out + 24 * i + 3 * corner;
      o[0] = (corner & 4) ? f[0] : c[0];
      o[1] = (corner & 2) ? f[1] : c[1];
      o[2] = (corner & 1) ? f[2] : c[2];
    }
  }
}

// src/grid_functions.py:47-63
template <typename T>
__global__ void in_bounds_kernel(const T* __restrict__ idx, int64_t count, int X, int Y, int Z,
                                 uint8_t* __restrict__ out) {
  PGB_FOR(i, count) {
    const T a = idx[3 * i], b = idx[3 * i + 1], c = idx[3 * i + 2];
    out[i] = (a < (T)X && a >= (T)0 && b < (T)Y && b >= (T)0 && c < (T)Z && c >= (T)0) ? 1 : 0;
  }
}

// src/grid_functions.py:66-79
__global__ void wrap_kernel(int64_t* __restrict__ idx, int64_t count, int X, int Y, int Z) {
  PGB_FOR(i, count) {
    idx[3 * i + 0] = floor_mod(idx[3 * i + 0], X);
    idx[3 * i + 1] = floor_mod(idx[3 * i + 1], Y);
    idx[3 * i + 2] = floor_mod(idx[3 * i + 2], Z);
  }
}

// src/grid_functions.py:7-44. Corners are used as given (the reference indexes the grid
// with whatever the caller passes, normally already wrapped).
// Cell of a caller-supplied corner; false (and the status bit) when it lies outside the
// grid, where the reference's advanced indexing raises IndexError. Negative indices
// count from the end, as in torch indexing.
template <typename Real>
__device__ __forceinline__ bool corner_cell(const GridP<Real>& g, const int64_t* o, uint64_t& cell,
                                            int* status) {
  long long i = o[0], j = o[1], k = o[2];
  if (i < 0) i += g.X;
  if (j < 0) j += g.Y;
  if (k < 0) k += g.Z;
  if (i < 0 || i >= g.X || j < 0 || j >= g.Y || k < 0 || k >= g.Z) {
    if (status) atomicOr(status, 1);
    return false;
  }
  cell = ((uint64_t)i * (uint64_t)g.Y + (uint64_t)j) * (uint64_t)g.Z + (uint64_t)k;
  return true;
}

template <typename Real>
__device__ __forceinline__ Real frac_ref(Real x) { return rsub(x, rtrunc(x)); }

template <typename Real, typename Store>
__global__ void trilinear_gather_kernel(GridP<Real> g, const Real* __restrict__ n,
                                        const int64_t* __restrict__ corners, int64_t count,
                                        Real* __restrict__ out, int* __restrict__ status) {
  PGB_FOR(i, count) {
    const Real wx = frac_ref(n[3 * i]), wy = frac_ref(n[3 * i + 1]), wz = frac_ref(n[3 * i + 2]);
    const Real ux = rsub(Real(1), wx), uy = rsub(Real(1), wy), uz = rsub(Real(1), wz);
    Real cv[8][4];
#pragma unroll
    for (int corner = 0; corner < 8; ++corner) {
      uint64_t cell;
      if (corner_cell(g, corners + 24 * i + 3 * corner, cell, status)) {
        CellIO<Store>::load(g.cells, cell, cv[corner]);
      } else {
        cv[corner][0] = cv[corner][1] = cv[corner][2] = cv[corner][3] = Real(0);
      }
      if (g.clip) {
#pragma unroll
        for (int ch = 0; ch < 4; ++ch) cv[corner][ch] = clamp01(cv[corner][ch]);
      }
    }
#pragma unroll
    for (int ch = 0; ch < 4; ++ch) {
      Real a4[4];
#pragma unroll
      for (int yz = 0; yz < 4; ++yz) a4[yz] = radd(rmul(cv[yz][ch], wx), rmul(cv[4 + yz][ch], ux));
      const Real b0 = radd(rmul(a4[0], wy), rmul(a4[2], uy));
      const Real b1 = radd(rmul(a4[1], wy), rmul(a4[3], uy));
      out[4 * i + ch] = radd(rmul(b0, wz), rmul(b1, uz));
    }
  }
}

template <typename Real, typename Store>
__global__ void trilinear_scatter_kernel(GridP<Real> g, const Real* __restrict__ n,
                                         const int64_t* __restrict__ corners, int64_t count,
                                         const Real* __restrict__ dout, Real* __restrict__ grad,
                                         int* __restrict__ status) {
  PGB_FOR(i, count) {
    const Real wx = frac_ref(n[3 * i]), wy = frac_ref(n[3 * i + 1]), wz = frac_ref(n[3 * i + 2]);
    const Real ux = rsub(Real(1), wx), uy = rsub(Real(1), wy), uz = rsub(Real(1), wz);
    Real dv[4];
#pragma unroll
    for (int ch = 0; ch < 4; ++ch) dv[ch] = dout[4 * i + ch];
#pragma unroll
    for (int corner = 0; corner < 8; ++corner) {
      const Real sz = (corner & 1) ? uz : wz;
      const Real sy = (corner & 2) ? uy : wy;
      const Real sx = (corner & 4) ? ux : wx;
      uint64_t c;
      if (!corner_cell(g, corners + 24 * i + 3 * corner, c, status)) continue;
      Real cv[4];
      if (g.clip) CellIO<Store>::load(g.cells, c, cv);
      Real gv[4];
      bool any = false;
#pragma unroll
      for (int ch = 0; ch < 4; ++ch) {
        gv[ch] = rmul(rmul(rmul(dv[ch], sz), sy), sx);
        if (g.clip && !in01(cv[ch])) gv[ch] = Real(0);
        any |= gv[ch] != Real(0);
      }
      if (any) grad_add(grad, c, gv);
    }
  }
}

// src/grid_functions.py:198-212: coordinates (i - ceil(s/2) + 1) * pd in fp32 and the
// integer meshgrid, one thread per cell.
__global__ void grid_coords_kernel(int X, int Y, int Z, float pd, float* __restrict__ coords,
                                   int64_t* __restrict__ mesh) {
  const int64_t total = (int64_t)X * Y * Z;
  const int cx = (X + 1) / 2, cy = (Y + 1) / 2, cz = (Z + 1) / 2;  // ceil(s / 2)
  PGB_FOR(i, total) {
    const int k = (int)(i % Z);
    const int64_t ij = i / Z;
    const int j = (int)(ij % Y);
    const int a = (int)(ij / Y);
    if (coords) {
      coords[3 * i + 0] = rmul((float)(a - cx + 1), pd);
      coords[3 * i + 1] = rmul((float)(j - cy + 1), pd);
      coords[3 * i + 2] = rmul((float)(k - cz + 1), pd);
    }
    if (mesh) {
      mesh[3 * i + 0] = a;
      mesh[3 * i + 1] = j;
      mesh[3 * i + 2] = k;
    }
  }
}

// Gather / scatter of whole cells at caller-supplied int64 indices.
template <typename Real, typename Store>
__global__ void gather_cells_kernel(GridP<Real> g, const int64_t* __restrict__ idx, int64_t count,
                                    Real* __restrict__ vals, int* __restrict__ status) {
  PGB_FOR(i, count) {
    uint64_t c;
    Real cv[4] = {Real(0), Real(0), Real(0), Real(0)};
    if (corner_cell(g, idx + 3 * i, c, status)) CellIO<Store>::load(g.cells, c, cv);
#pragma unroll
    for (int ch = 0; ch < 4; ++ch) vals[4 * i + ch] = g.clip ? clamp01(cv[ch]) : cv[ch];
  }
}

template <typename Real, typename Store>
__global__ void scatter_cells_kernel(GridP<Real> g, const int64_t* __restrict__ idx, int64_t count,
                                     const Real* __restrict__ dv, Real* __restrict__ grad,
                                     int* __restrict__ status) {
  PGB_FOR(i, count) {
    uint64_t c;
    if (!corner_cell(g, idx + 3 * i, c, status)) continue;
    Real cv[4];
    if (g.clip) CellIO<Store>::load(g.cells, c, cv);
    Real gv[4];
    bool any = false;
#pragma unroll
    for (int ch = 0; ch < 4; ++ch) {
      gv[ch] = (g.clip && !in01(cv[ch])) ? Real(0) : dv[4 * i + ch];
      any |= gv[ch] != Real(0);
    }
    if (any) grad_add(grad, c, gv);
  }
}

// --------------------------------------------------------------- compositing
// src/ray_sampling.py:172-192 over [M,S,4] samples, one warp per ray, 256-sample chunks.
template <typename Real>
__device__ __forceinline__ void load_sample(const Real* p, Real v[4]) {
  v[0] = p[0]; v[1] = p[1]; v[2] = p[2]; v[3] = p[3];
}
template <>
__device__ __forceinline__ void load_sample<float>(const float* p, float v[4]) {
  const float4 q = *reinterpret_cast<const float4*>(p);
  v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
}

constexpr int kCompK = 8;

// Exclusive transmittance of every sample of a register chunk from the chunk's starting
// T; returns T after the chunk.
template <typename Real, int K>
__device__ __forceinline__ Real scan_chunk(const Real v[K][4], Real T, int lane, Real Ts[K]) {
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const Real incl = warp_incl_prod(Real(1) - v[k][3], lane);
    Real excl = __shfl_up_sync(kFull, incl, 1);
    if (lane == 0) excl = Real(1);
    Ts[k] = T * excl;
    T *= __shfl_sync(kFull, incl, kWarp - 1);
  }
  return T;
}

template <typename Real>
__device__ __forceinline__ void load_comp_chunk(const Real* base, int S, int c, int lane,
                                                Real v[kCompK][4]) {
#pragma unroll
  for (int k = 0; k < kCompK; ++k) {
    const int s = (c * kCompK + k) * kWarp + lane;
    if (s < S) load_sample(base + 4 * (int64_t)s, v[k]);
    else v[k][0] = v[k][1] = v[k][2] = v[k][3] = Real(0);
  }
}

template <typename Real, bool BWD>
__global__ void __launch_bounds__(256) composite_kernel(const Real* __restrict__ samples,
                                                        int64_t M, int S, const Real* __restrict__ dout,
                                                        Real* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int nchunks = (S + kWarp * kCompK - 1) / (kWarp * kCompK);
  for (int64_t m = gw; m < M; m += nw) {
    const Real* base = samples + (int64_t)4 * S * m;
    Real v[kCompK][4], Ts[kCompK];
    Real acc[4] = {Real(0), Real(0), Real(0), Real(0)};
    Real T = Real(1), Tstart = Real(1);
    for (int c = 0; c < nchunks; ++c) {
      if (lane == c) Tstart = T;
      load_comp_chunk(base, S, c, lane, v);
      T = scan_chunk<Real, kCompK>(v, T, lane, Ts);
      if (!BWD) {
#pragma unroll
        for (int k = 0; k < kCompK; ++k) {
          const Real w = v[k][3] * Ts[k];
          acc[0] += w * v[k][0];
          acc[1] += w * v[k][1];
          acc[2] += w * v[k][2];
          acc[3] += w;
        }
      }
    }
    if (!BWD) {
      Real px[4];
#pragma unroll
      for (int ch = 0; ch < 4; ++ch) px[ch] = warp_sum(acc[ch]);
      if (lane < 4) out[4 * m + lane] = pick4(px, lane);
      continue;
    }
    Real g[4];
#pragma unroll
    for (int ch = 0; ch < 4; ++ch) g[ch] = dout[4 * m + ch];
    Real* obase = out + (int64_t)4 * S * m;
    Real carry = Real(0);
    for (int c = nchunks - 1; c >= 0; --c) {
      if (c != nchunks - 1) {
        load_comp_chunk(base, S, c, lane, v);
        scan_chunk<Real, kCompK>(v, __shfl_sync(kFull, Tstart, c), lane, Ts);
      }
#pragma unroll
      for (int k = kCompK - 1; k >= 0; --k) {
        const Real al = v[k][3];
        const Real G = g[0] * v[k][0] + g[1] * v[k][1] + g[2] * v[k][2] + g[3];
        Real fa = G * al, fb = Real(1) - al;
        warp_suffix_affine(fa, fb, lane);
        const Real S_here = fa + fb * carry;
        Real S_after = __shfl_down_sync(kFull, S_here, 1);
        if (lane == kWarp - 1) S_after = carry;
        carry = __shfl_sync(kFull, S_here, 0);
        const int s = (c * kCompK + k) * kWarp + lane;
        if (s < S) {
          const Real w = al * Ts[k];
          Real* o = obase + 4 * (int64_t)s;
          o[0] = g[0] * w;
          o[1] = g[1] * w;
          o[2] = g[2] * w;
          o[3] = Ts[k] * (G - S_after);
        }
      }
    }
  }
}

// --------------------------------------------------------------- fused-path index view
template <typename Real, int MODE>
__global__ void render_indices_kernel(const RenderArgs<Real> a, int64_t* __restrict__ idx_out,
                                      uint8_t* __restrict__ inb_out) {
  const int64_t total = a.R * (int64_t)a.S;
  const int dims[3] = {a.g.X, a.g.Y, a.g.Z};
  PGB_FOR(i, total) {
    const int64_t r = i / a.S;
    const int s = (int)(i - r * a.S);
    Ray<Real> ray;
    load_ray(a, r, ray, false);
    Real nx, ny, nz;
    sample_coords(a, ray, s, nx, ny, nz);
    if (MODE == PGB_NEAREST) {
      long long idx[3];
      bool inb;
      nearest_index(nx, ny, nz, dims, idx, inb);
      if (idx_out) {
        idx_out[3 * i + 0] = idx[0];
        idx_out[3 * i + 1] = idx[1];
        idx_out[3 * i + 2] = idx[2];
      }
      if (inb_out) inb_out[i] = inb ? 1 : 0;
    } else {
      const Real n[3] = {nx, ny, nz};
      long long c[3], f[3];
#pragma unroll
      for (int ax = 0; ax < 3; ++ax) {
        c[ax] = floor_mod(to_i64(rceil(n[ax])), dims[ax]);
        f[ax] = floor_mod(to_i64(rfloor(n[ax])), dims[ax]);
      }
      if (idx_out) {
#pragma unroll
        for (int corner = 0; corner < 8; ++corner) {
          int64_t* o = idx_out + 24 * i + 3 * corner;
          o[0] = (corner & 4) ? f[0] : c[0];
          o[1] = (corner & 2) ? f[1] : c[1];
          o[2] = (corner & 1) ? f[2] : c[2];
        }
      }
      if (inb_out) inb_out[i] = float_in_bounds(nx, ny, nz, dims) ? 1 : 0;
    }
  }
}

// (255 * rgba).round().clip(0, 255) as uint8, written transposed (src/visualization.py:148-152)
__global__ void rgba_to_image_kernel(const float* __restrict__ rgba, int res, uint8_t* __restrict__ out) {
  const int64_t n = (int64_t)res * res;
  PGB_FOR(i, n) {
    const int64_t a = i / res, b = i - a * res;  // out[a][b] = ray b * res + a
    const float* p = rgba + 4 * (b * res + a);
#pragma unroll
    for (int ch = 0; ch < 4; ++ch) {
      const float v = fminf(fmaxf(rintf(rmul(p[ch], 255.0f)), 0.0f), 255.0f);
      out[4 * i + ch] = (uint8_t)v;
    }
  }
}

__global__ void fill_zero_kernel(uint4* __restrict__ p, int64_t n16, uint8_t* __restrict__ tail,
                                 int tail_bytes) {
  PGB_FOR(i, n16) p[i] = make_uint4(0u, 0u, 0u, 0u);
  if (blockIdx.x == 0 && (int)threadIdx.x < tail_bytes) tail[threadIdx.x] = 0;
}

// Zeroes the marked units of a gradient buffer and clears the marks (clear_marked_warp),
// every warp of the grid taking rounds of 32 mark words.
__global__ void clear_marked_kernel(uint4* __restrict__ grad, int64_t total16, int unit_shift,
                                    uint32_t* __restrict__ marks, int64_t words) {
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  clear_marked_warp(grad, total16, unit_shift, marks, words, warp, warps, threadIdx.x & 31);
}

}  // namespace

// ================================================================ launchers
int op_generate_rays(const float* T, int C, int64_t Rc, float fov, const float* images, int H, int W,
                     const float* uv, int even_side, float* dirs, float* pixels, int* status,
                     cudaStream_t s) {
  generate_rays_kernel<<<blocks_for((int64_t)C * Rc), kThreads, 0, s>>>(
      T, C, Rc, fov, images, H, W, uv, even_side, dirs, pixels, status);
  return after_launch();
}

int op_sample_points(const float* T, int C, int64_t Rc, const float* dirs, int S, float delta,
                     float* out, cudaStream_t s) {
  const int64_t total = (int64_t)C * Rc * S;
  sample_points_kernel<<<blocks_for(total), kThreads, 0, s>>>(T, Rc, S, dirs, delta, total, out);
  return after_launch();
}

int op_coords_min(const float* coords, int64_t count, float* out, cudaStream_t s) {
  int* o = reinterpret_cast<int*>(out);
  min_init_kernel<<<1, 32, 0, s>>>(o);
  int st = after_launch();
  if (st) return st;
  const unsigned blocks = std::min<unsigned>(blocks_for(count, 4), 152u * 8u);
  coords_min_kernel<<<blocks, kThreads, 0, s>>>(coords, count, o);
  st = after_launch();
  if (st) return st;
  min_finish_kernel<<<1, 32, 0, s>>>(o);
  return after_launch();
}

int op_normalize(const float* samples, int64_t count, const float* gmin, float pd, float* out,
                 cudaStream_t s) {
  normalize_kernel<<<blocks_for(count), kThreads, 0, s>>>(samples, count, gmin, pd, out);
  return after_launch();
}

template <typename Real, typename Store>
static int nearest_gather_t(const GridP<Real>& g, const void* n, int64_t count, void* vals,
                            uint8_t* inb, int64_t* idx, cudaStream_t s) {
  nearest_gather_kernel<Real, Store><<<blocks_for(count), kThreads, 0, s>>>(
      g, (const Real*)n, count, (Real*)vals, inb, idx);
  return after_launch();
}
template <typename Real, typename Store>
static int nearest_scatter_t(const GridP<Real>& g, const void* n, int64_t count, const void* dv,
                             void* grad, cudaStream_t s) {
  nearest_scatter_kernel<Real, Store><<<blocks_for(count), kThreads, 0, s>>>(
      g, (const Real*)n, count, (const Real*)dv, (Real*)grad);
  return after_launch();
}
template <typename Real, typename Store>
static int trilinear_gather_t(const GridP<Real>& g, const void* n, const int64_t* corners,
                              int64_t count, void* out, int* status, cudaStream_t s) {
  trilinear_gather_kernel<Real, Store><<<blocks_for(count), kThreads, 0, s>>>(
      g, (const Real*)n, corners, count, (Real*)out, status);
  return after_launch();
}
template <typename Real, typename Store>
static int trilinear_scatter_t(const GridP<Real>& g, const void* n, const int64_t* corners,
                               int64_t count, const void* dout, void* grad, int* status,
                               cudaStream_t s) {
  trilinear_scatter_kernel<Real, Store><<<blocks_for(count), kThreads, 0, s>>>(
      g, (const Real*)n, corners, count, (const Real*)dout, (Real*)grad, status);
  return after_launch();
}

int op_nearest_gather_f32(const GridP<float>& g, int bf16, const void* n, int64_t count, void* vals,
                          uint8_t* inb, int64_t* idx, cudaStream_t s) {
  return bf16 ? nearest_gather_t<float, __nv_bfloat16>(g, n, count, vals, inb, idx, s)
              : nearest_gather_t<float, float>(g, n, count, vals, inb, idx, s);
}
int op_nearest_gather_f64(const GridP<double>& g, const void* n, int64_t count, void* vals,
                          uint8_t* inb, int64_t* idx, cudaStream_t s) {
  return nearest_gather_t<double, double>(g, n, count, vals, inb, idx, s);
}
int op_nearest_scatter_f32(const GridP<float>& g, int bf16, const void* n, int64_t count,
                           const void* dv, void* grad, cudaStream_t s) {
  return bf16 ? nearest_scatter_t<float, __nv_bfloat16>(g, n, count, dv, grad, s)
              : nearest_scatter_t<float, float>(g, n, count, dv, grad, s);
}
int op_nearest_scatter_f64(const GridP<double>& g, const void* n, int64_t count, const void* dv,
                           void* grad, cudaStream_t s) {
  return nearest_scatter_t<double, double>(g, n, count, dv, grad, s);
}
int op_trilinear_gather_f32(const GridP<float>& g, int bf16, const void* n, const int64_t* corners,
                            int64_t count, void* out, int* status, cudaStream_t s) {
  return bf16 ? trilinear_gather_t<float, __nv_bfloat16>(g, n, corners, count, out, status, s)
              : trilinear_gather_t<float, float>(g, n, corners, count, out, status, s);
}
int op_trilinear_gather_f64(const GridP<double>& g, const void* n, const int64_t* corners,
                            int64_t count, void* out, int* status, cudaStream_t s) {
  return trilinear_gather_t<double, double>(g, n, corners, count, out, status, s);
}
int op_trilinear_scatter_f32(const GridP<float>& g, int bf16, const void* n, const int64_t* corners,
                             int64_t count, const void* dout, void* grad, int* status,
                             cudaStream_t s) {
  return bf16 ? trilinear_scatter_t<float, __nv_bfloat16>(g, n, corners, count, dout, grad, status, s)
              : trilinear_scatter_t<float, float>(g, n, corners, count, dout, grad, status, s);
}
int op_trilinear_scatter_f64(const GridP<double>& g, const void* n, const int64_t* corners,
                             int64_t count, const void* dout, void* grad, int* status,
                             cudaStream_t s) {
  return trilinear_scatter_t<double, double>(g, n, corners, count, dout, grad, status, s);
}

int op_grid_coords(const int dims[3], float pd, float* coords, int64_t* mesh, cudaStream_t s) {
  grid_coords_kernel<<<blocks_for((int64_t)dims[0] * dims[1] * dims[2]), kThreads, 0, s>>>(
      dims[0], dims[1], dims[2], pd, coords, mesh);
  return after_launch();
}

template <typename Real, typename Store>
static int gather_cells_t(const GridP<Real>& g, const int64_t* idx, int64_t count, void* vals,
                          int* status, cudaStream_t s) {
  gather_cells_kernel<Real, Store><<<blocks_for(count), kThreads, 0, s>>>(g, idx, count, (Real*)vals, status);
  return after_launch();
}
template <typename Real, typename Store>
static int scatter_cells_t(const GridP<Real>& g, const int64_t* idx, int64_t count, const void* dv,
                           void* grad, int* status, cudaStream_t s) {
  scatter_cells_kernel<Real, Store><<<blocks_for(count), kThreads, 0, s>>>(
      g, idx, count, (const Real*)dv, (Real*)grad, status);
  return after_launch();
}
int op_gather_cells_f32(const GridP<float>& g, int bf16, const int64_t* idx, int64_t count, void* vals,
                        int* status, cudaStream_t s) {
  return bf16 ? gather_cells_t<float, __nv_bfloat16>(g, idx, count, vals, status, s)
              : gather_cells_t<float, float>(g, idx, count, vals, status, s);
}
int op_gather_cells_f64(const GridP<double>& g, const int64_t* idx, int64_t count, void* vals,
                        int* status, cudaStream_t s) {
  return gather_cells_t<double, double>(g, idx, count, vals, status, s);
}
int op_scatter_cells_f32(const GridP<float>& g, int bf16, const int64_t* idx, int64_t count,
                         const void* dv, void* grad, int* status, cudaStream_t s) {
  return bf16 ? scatter_cells_t<float, __nv_bfloat16>(g, idx, count, dv, grad, status, s)
              : scatter_cells_t<float, float>(g, idx, count, dv, grad, status, s);
}
int op_scatter_cells_f64(const GridP<double>& g, const int64_t* idx, int64_t count, const void* dv,
                         void* grad, int* status, cudaStream_t s) {
  return scatter_cells_t<double, double>(g, idx, count, dv, grad, status, s);
}

int op_corner_indices(const void* n, int f64, int64_t count, int64_t* out, cudaStream_t s) {
  if (f64) corner_indices_kernel<double><<<blocks_for(count), kThreads, 0, s>>>((const double*)n, count, out);
  else corner_indices_kernel<float><<<blocks_for(count), kThreads, 0, s>>>((const float*)n, count, out);
  return after_launch();
}

int op_in_bounds(const void* idx, int kind, int64_t count, const int dims[3], uint8_t* out,
                 cudaStream_t s) {
  const unsigned b = blocks_for(count);
  if (kind == PGB_INDEX_F32)
    in_bounds_kernel<float><<<b, kThreads, 0, s>>>((const float*)idx, count, dims[0], dims[1], dims[2], out);
  else if (kind == PGB_INDEX_F64)
    in_bounds_kernel<double><<<b, kThreads, 0, s>>>((const double*)idx, count, dims[0], dims[1], dims[2], out);
  else
    in_bounds_kernel<long long><<<b, kThreads, 0, s>>>((const long long*)idx, count, dims[0], dims[1], dims[2], out);
  return after_launch();
}

int op_wrap(int64_t* idx, int64_t count, const int dims[3], cudaStream_t s) {
  wrap_kernel<<<blocks_for(count), kThreads, 0, s>>>(idx, count, dims[0], dims[1], dims[2]);
  return after_launch();
}

int op_composite(const void* samples, int f64, int64_t M, int S, const void* dout, void* out,
                 int bwd, cudaStream_t s) {
  const unsigned b = blocks_for(M * kWarp);
  if (f64) {
    if (bwd) composite_kernel<double, true><<<b, kThreads, 0, s>>>((const double*)samples, M, S, (const double*)dout, (double*)out);
    else composite_kernel<double, false><<<b, kThreads, 0, s>>>((const double*)samples, M, S, nullptr, (double*)out);
  } else {
    if (bwd) composite_kernel<float, true><<<b, kThreads, 0, s>>>((const float*)samples, M, S, (const float*)dout, (float*)out);
    else composite_kernel<float, false><<<b, kThreads, 0, s>>>((const float*)samples, M, S, nullptr, (float*)out);
  }
  return after_launch();
}
int composite_max_samples() { return kMaxChunks * kWarp * kCompK; }

// Normalised coordinates (p - origin) / pd of every sample of every ray, as the fused
// kernels compute them: out[(r * S + s) * 3 + axis].
template <typename Real>
__global__ void render_coords_kernel(const RenderArgs<Real> a, Real* __restrict__ out) {
  const int64_t total = a.R * (int64_t)a.S;
  PGB_FOR(i, total) {
    const int64_t r = i / a.S;
    const int s = (int)(i - r * a.S);
    Ray<Real> ray;
    load_ray(a, r, ray, false);
    Real nx, ny, nz;
    sample_coords(a, ray, s, nx, ny, nz);
    out[3 * i + 0] = nx;
    out[3 * i + 1] = ny;
    out[3 * i + 2] = nz;
  }
}

int op_render_coords_f32(const RenderArgs<float>& a, float* out, cudaStream_t s) {
  render_coords_kernel<float><<<blocks_for(a.R * (int64_t)a.S), kThreads, 0, s>>>(a, out);
  return after_launch();
}
int op_render_coords_f64(const RenderArgs<double>& a, double* out, cudaStream_t s) {
  render_coords_kernel<double><<<blocks_for(a.R * (int64_t)a.S), kThreads, 0, s>>>(a, out);
  return after_launch();
}

template <typename Real>
static int render_indices_t(const RenderArgs<Real>& a, int mode, int64_t* idx, uint8_t* inb,
                            cudaStream_t s) {
  const unsigned b = blocks_for(a.R * (int64_t)a.S);
  if (mode == PGB_NEAREST) render_indices_kernel<Real, PGB_NEAREST><<<b, kThreads, 0, s>>>(a, idx, inb);
  else render_indices_kernel<Real, PGB_TRILINEAR><<<b, kThreads, 0, s>>>(a, idx, inb);
  return after_launch();
}
int op_render_indices_f32(const RenderArgs<float>& a, int mode, int64_t* idx, uint8_t* inb, cudaStream_t s) {
  return render_indices_t(a, mode, idx, inb, s);
}
int op_render_indices_f64(const RenderArgs<double>& a, int mode, int64_t* idx, uint8_t* inb, cudaStream_t s) {
  return render_indices_t(a, mode, idx, inb, s);
}

int op_rgba_to_image(const float* rgba, int res, uint8_t* out, cudaStream_t s) {
  rgba_to_image_kernel<<<blocks_for((int64_t)res * res), kThreads, 0, s>>>(rgba, res, out);
  return after_launch();
}

int op_clear_marked(void* grad, int cell_bytes, int64_t num_cells, uint32_t* marks, cudaStream_t s) {
  const int64_t words = mark_words(num_cells);
  // log2 of the 16-byte slots per unit: a cell is 1 (fp32 gradient) or 2 (fp64) slots
  const int unit_shift = (cell_bytes == 32 ? 1 : 0) + kMarkCellsLog2;
  const int64_t total16 = num_cells * cell_bytes / 16;
  // one thread per word: each warp takes 32 consecutive words
  clear_marked_kernel<<<blocks_for(words), kThreads, 0, s>>>((uint4*)grad, total16, unit_shift,
                                                            marks, words);
  return after_launch();
}

int op_fill_zero(void* p, int64_t bytes, cudaStream_t s) {
  const int64_t n16 = bytes / 16;
  const int tail = (int)(bytes - n16 * 16);
  fill_zero_kernel<<<blocks_for(n16, 4), kThreads, 0, s>>>(
      (uint4*)p, n16, (uint8_t*)p + n16 * 16, tail);
  return after_launch();
}

}  // namespace pgb
