// Device-memory probes, a measurement helper built as its own library (libpgb_probes.so)
// beside the renderer: the rate at which this GPU serves independent random 32 B sectors
// (reads, and float4 atomic adds) out of a buffer larger than L2. The fused kernels read
// one grid cell per trilinear corner and add one gradient cell per corner at positions
// with little reuse across rays, so this rate, not the streaming copy bandwidth, is what
// random cell traffic runs against. The benchmark reports it next to the copy-bandwidth
// roofline. No counterpart in the reference.
#include <algorithm>

#include "pgb_device.cuh"
#include "pgb_probes.h"

namespace pgb {
namespace {

constexpr int kProbeUnroll = 8;  // independent accesses in flight per thread

// Random slot of `slots` 16 B slots for access i (a 32-bit mix; every slot < slots).
__device__ __forceinline__ uint64_t probe_slot(uint64_t seed, uint64_t i, uint64_t slots) {
  return (mix64(seed ^ i) >> 11) % slots;
}

__global__ void probe_reads_kernel(const float4* __restrict__ table, uint64_t slots, int64_t n,
                                   uint64_t seed, float* __restrict__ sink) {
  float acc = 0.f;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x * kProbeUnroll;
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * kProbeUnroll; i < n; i += stride) {
    float4 v[kProbeUnroll];
#pragma unroll
    for (int u = 0; u < kProbeUnroll; ++u)
      v[u] = i + u < n ? __ldg(table + probe_slot(seed, (uint64_t)(i + u), slots)) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int u = 0; u < kProbeUnroll; ++u) acc += v[u].x + v[u].w;
  }
  if (acc == -1.0f) sink[0] = acc;  // keeps the loads; the table never sums to -1
}

__global__ void probe_atomics_kernel(float4* table, uint64_t slots, int64_t n, uint64_t seed) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x * kProbeUnroll;
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * kProbeUnroll; i < n; i += stride) {
#pragma unroll
    for (int u = 0; u < kProbeUnroll; ++u)
      if (i + u < n) atomicAdd(table + probe_slot(seed, (uint64_t)(i + u), slots), make_float4(1.f, 1.f, 1.f, 1.f));
  }
}

int launch_status() { return cudaGetLastError() == cudaSuccess ? PGB_OK : PGB_ERR_LAUNCH; }

unsigned probe_blocks() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return (unsigned)std::max(1, sms) * 8u;
}

}  // namespace
}  // namespace pgb

using namespace pgb;

extern "C" {

int pgb_probe_random_reads(const void* table, int64_t table_bytes, int64_t num_reads, uint64_t seed,
                           float* sink, pgb_stream_t stream) {
  if (num_reads < 0 || table_bytes < 0) return PGB_ERR_ARG;
  if (num_reads == 0) return PGB_OK;
  if (!table || !sink || table_bytes < 16) return PGB_ERR_ARG;
  if (((uintptr_t)table % 16) != 0) return PGB_ERR_ALIGN;
  probe_reads_kernel<<<probe_blocks(), 256, 0, stream>>>(
      static_cast<const float4*>(table), (uint64_t)(table_bytes / 16), num_reads, seed, sink);
  return launch_status();
}

int pgb_probe_random_atomics(void* table, int64_t table_bytes, int64_t num_updates, uint64_t seed,
                             pgb_stream_t stream) {
  if (num_updates < 0 || table_bytes < 0) return PGB_ERR_ARG;
  if (num_updates == 0) return PGB_OK;
  if (!table || table_bytes < 16) return PGB_ERR_ARG;
  if (((uintptr_t)table % 16) != 0) return PGB_ERR_ALIGN;
  probe_atomics_kernel<<<probe_blocks(), 256, 0, stream>>>(
      static_cast<float4*>(table), (uint64_t)(table_bytes / 16), num_updates, seed);
  return launch_status();
}

}  // extern "C"
