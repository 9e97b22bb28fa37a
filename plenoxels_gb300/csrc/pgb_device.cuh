// Device-side building blocks shared by every kernel of the library.
//
// Arithmetic on the index path is written with explicitly rounded intrinsics so that
// nvcc cannot contract a*b+c into an FMA: the reference (PyTorch CPU) rounds after
// every elementwise op, and voxel indices must come out bit-identical.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include "plenoxels_gb300.h"
#include "pgb_host.h"

namespace pgb {

constexpr int kWarp = 32;
constexpr unsigned kFull = 0xffffffffu;

// ---------------------------------------------------------------- exact arithmetic
__device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float rsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float rdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float rsqrt_exact(float a) { return __fsqrt_rn(a); }
__device__ __forceinline__ float rfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double rsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double rdiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double rsqrt_exact(double a) { return __dsqrt_rn(a); }
__device__ __forceinline__ double rfma(double a, double b, double c) { return __fma_rn(a, b, c); }

// round half to even (torch.round), floor, ceil, trunc
__device__ __forceinline__ float rround(float a) { return rintf(a); }
__device__ __forceinline__ double rround(double a) { return rint(a); }
__device__ __forceinline__ float rfloor(float a) { return floorf(a); }
__device__ __forceinline__ double rfloor(double a) { return floor(a); }
__device__ __forceinline__ float rceil(float a) { return ceilf(a); }
__device__ __forceinline__ double rceil(double a) { return ceil(a); }
__device__ __forceinline__ float rtrunc(float a) { return truncf(a); }
__device__ __forceinline__ double rtrunc(double a) { return trunc(a); }

// clamp(x, 0, 1) as torch.clamp (min then max order is irrelevant for 0 <= 1)
template <typename Real>
__device__ __forceinline__ Real clamp01(Real x) {
  return x < Real(0) ? Real(0) : (x > Real(1) ? Real(1) : x);
}
template <typename Real>
__device__ __forceinline__ bool in01(Real x) { return x >= Real(0) && x <= Real(1); }

// Python-style floor modulo for a positive modulus (src/grid_functions.py:75-77).
__device__ __forceinline__ long long floor_mod(long long a, long long m) {
  long long r = a % m;
  return r < 0 ? r + m : r;
}

// ---------------------------------------------------------------- counter hash
// splitmix64 finaliser (Steele, Lea, Flood: "Fast splittable pseudorandom number
// generators", 2014). The library's uniform(seed, a, b) = top 24 bits of
// mix(mix(mix(seed) ^ a) ^ b) * 2^-24: exact in float and double, reproducible on the host.
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
__host__ __device__ __forceinline__ uint64_t hash_stream(uint64_t seed, uint64_t a) {
  return mix64(mix64(seed) ^ a);
}
__host__ __device__ __forceinline__ float hash_to_unit(uint64_t h, uint32_t b) {
  return (float)(uint32_t)(mix64(h ^ (uint64_t)b) >> 40) * 5.9604644775390625e-08f;  // 2^-24
}

// ---------------------------------------------------------------- cell storage
// A cell is four channels R, G, B, alpha. Load returns "Real" channels.
template <typename Store> struct CellIO;

template <> struct CellIO<float> {
  using Real = float;
  static constexpr int kBytes = 16;
  __device__ __forceinline__ static void load(const void* cells, uint64_t c, float v[4]) {
    const float4 q = __ldg(reinterpret_cast<const float4*>(cells) + c);
    v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
  }
};

template <> struct CellIO<__nv_bfloat16> {
  using Real = float;
  static constexpr int kBytes = 8;
  __device__ __forceinline__ static void load(const void* cells, uint64_t c, float v[4]) {
    const uint2 q = __ldg(reinterpret_cast<const uint2*>(cells) + c);
    v[0] = __uint_as_float(q.x << 16);
    v[1] = __uint_as_float(q.x & 0xffff0000u);
    v[2] = __uint_as_float(q.y << 16);
    v[3] = __uint_as_float(q.y & 0xffff0000u);
  }
};

template <> struct CellIO<double> {
  using Real = double;
  static constexpr int kBytes = 32;
  __device__ __forceinline__ static void load(const void* cells, uint64_t c, double v[4]) {
    const double2* p = reinterpret_cast<const double2*>(cells) + 2 * c;
    const double2 a = __ldg(p), b = __ldg(p + 1);
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
  }
};

// Gradient accumulation into a dense [X,Y,Z,4] buffer of Real.
__device__ __forceinline__ void grad_add(float* grad, uint64_t c, const float g[4]) {
  atomicAdd(reinterpret_cast<float4*>(grad) + c, make_float4(g[0], g[1], g[2], g[3]));
}
__device__ __forceinline__ void grad_add(double* grad, uint64_t c, const double g[4]) {
  double* p = grad + 4 * c;
  atomicAdd(p + 0, g[0]);
  atomicAdd(p + 1, g[1]);
  atomicAdd(p + 2, g[2]);
  atomicAdd(p + 3, g[3]);
}

// ---------------------------------------------------------------- warp scans
// Inclusive prefix product over lanes (lane 0 first).
template <typename Real>
__device__ __forceinline__ Real warp_incl_prod(Real x, int lane) {
#pragma unroll
  for (int d = 1; d < kWarp; d <<= 1) {
    const Real y = __shfl_up_sync(kFull, x, d);
    if (lane >= d) x *= y;
  }
  return x;
}

// Inclusive suffix scan of affine maps f_l(s) = a_l + b_l * s composed towards lane 31:
// after the call lane l holds F_l = f_l o f_{l+1} o ... o f_31 as (a, b).
template <typename Real>
__device__ __forceinline__ void warp_suffix_affine(Real& a, Real& b, int lane) {
#pragma unroll
  for (int d = 1; d < kWarp; d <<= 1) {
    const Real a2 = __shfl_down_sync(kFull, a, d);
    const Real b2 = __shfl_down_sync(kFull, b, d);
    if (lane + d < kWarp) {
      a = a + b * a2;
      b = b * b2;
    }
  }
}

template <typename Real>
__device__ __forceinline__ Real warp_sum(Real x) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) x += __shfl_xor_sync(kFull, x, d);
  return x;
}

// A running sum of loss terms kept in an 8-byte slot. For fp64 kernels a plain double.
// For fp32 kernels an unevaluated pair hi + lo of floats, each term added with Knuth's
// TwoSum (the rounding error of hi + x is exact and goes to lo), ~48 bits in all: the
// sums stay in fp32 arithmetic, since GB300's fp64 rate is a small fraction of its fp32
// rate and the loss reductions sit on the kernels' critical path.
template <typename Real>
struct LossSum {
  double v = 0.0;
  __device__ __forceinline__ void add(double x) { v += x; }
  __device__ __forceinline__ void add(const LossSum& o) { v += o.v; }
  __device__ __forceinline__ double value() const { return v; }
  __device__ __forceinline__ void store(double* slot) const { *slot = v; }
  __device__ __forceinline__ void store_volatile(double* slot) const {
    *(volatile double*)slot = v;
  }
  __device__ __forceinline__ static LossSum load_volatile(const double* slot) {
    LossSum s;
    s.v = *(const volatile double*)slot;
    return s;
  }
  __device__ __forceinline__ static LossSum load_cg(const double* slot) {
    LossSum s;
    s.v = __ldcg(slot);
    return s;
  }
  __device__ __forceinline__ LossSum shfl_xor(int d) const {
    LossSum s;
    s.v = __shfl_xor_sync(kFull, v, d);
    return s;
  }
};

template <>
struct LossSum<float> {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float s = hi + x;
    if (isinf(s)) {  // an infinite sum carries no error term (inf - inf would make it NaN)
      hi = s;
      lo = 0.f;
      return;
    }
    const float b = s - hi;
    lo += (hi - (s - b)) + (x - b);
    hi = s;
  }
  __device__ __forceinline__ void add(const LossSum& o) {
    add(o.hi);
    lo += o.lo;
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
  __device__ __forceinline__ void store(double* slot) const {
    *reinterpret_cast<float2*>(slot) = make_float2(hi, lo);
  }
  __device__ __forceinline__ void store_volatile(double* slot) const {
    volatile float* q = reinterpret_cast<volatile float*>(slot);
    q[0] = hi;
    q[1] = lo;
  }
  __device__ __forceinline__ static LossSum load_volatile(const double* slot) {
    const volatile float* q = reinterpret_cast<const volatile float*>(slot);
    LossSum s;
    s.hi = q[0];
    s.lo = q[1];
    return s;
  }
  __device__ __forceinline__ static LossSum load_cg(const double* slot) {
    const float2 p = __ldcg(reinterpret_cast<const float2*>(slot));
    LossSum s;
    s.hi = p.x;
    s.lo = p.y;
    return s;
  }
  __device__ __forceinline__ LossSum shfl_xor(int d) const {
    LossSum s;
    s.hi = __shfl_xor_sync(kFull, hi, d);
    s.lo = __shfl_xor_sync(kFull, lo, d);
    return s;
  }
};

// Gradient marks (layout in pgb_host.h): the unit of a cell.
__device__ __forceinline__ uint64_t mark_unit_of(uint64_t cell) { return cell >> kMarkCellsLog2; }

// Zeroing of the marked units of a gradient buffer, by one warp of `warps` (this one is
// `warp`): bit b of mark word w marks unit 32 w + b, i.e. the 16-byte slots
// (32 w + b) << unit_shift onwards (unit_shift: log2 of the 16-byte slots per unit). The
// warp takes 32 consecutive words per round (one coalesced load, one word per lane) and
// clears them; then, for every word that had marks, it zeroes the word's slots as
// consecutive 16-byte stores (512 B per warp store), lanes of unmarked units skipping
// theirs, so the stores stay coalesced however the marks are spread.
__device__ __forceinline__ void clear_marked_warp(uint4* __restrict__ grad, int64_t total16,
                                                  int unit_shift, uint32_t* __restrict__ marks,
                                                  int64_t words, int64_t warp, int64_t warps,
                                                  int lane) {
  const int slots = 32 << unit_shift;  // 16-byte slots under one word
  for (int64_t base = warp * 32; base < words; base += warps * 32) {
    const int64_t w = base + lane;
    const uint32_t mine = w < words ? marks[w] : 0u;
    if (mine != 0u) marks[w] = 0u;
    uint32_t pending = __ballot_sync(kFull, mine != 0u);
    while (pending != 0u) {
      const int src = __ffs(pending) - 1;
      pending &= pending - 1u;
      const uint32_t m = __shfl_sync(kFull, mine, src);
      const int64_t first = (base + src) * (int64_t)slots;
      for (int s = lane; s < slots; s += 32) {
        const int64_t at = first + s;
        if (((m >> (s >> unit_shift)) & 1u) && at < total16) grad[at] = make_uint4(0u, 0u, 0u, 0u);
      }
    }
  }
}

template <typename Real>
__device__ __forceinline__ LossSum<Real> warp_sum(LossSum<Real> x) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) x.add(x.shfl_xor(d));
  return x;
}

}  // namespace pgb
