// Host-side declarations shared by the translation units of the library (not part of
// the public C ABI, which is include/plenoxels_gb300.h).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "plenoxels_gb300.h"

namespace pgb {

template <typename Real> struct RenderArgs;

// Counts one kernel launch and converts the launch status into a PGB status.
int after_launch();

// Most warps the fused training kernel may use (size of its per-warp loss table).
constexpr int kMaxTrainWarps = 32768;
// Samples per chunk are 32 * K; a ray may span at most this many chunks.
constexpr int kMaxChunks = 32;
// Largest samples-per-ray the fused kernels accept.
constexpr int kMaxSamples = kMaxChunks * 32 * 8;

int launch_render_f32(const RenderArgs<float>& a, int mode, int phase, cudaStream_t s);
int launch_render_bf16(const RenderArgs<float>& a, int mode, int phase, cudaStream_t s);
int launch_render_f64(const RenderArgs<double>& a, int mode, int phase, cudaStream_t s);
// Log-sum transmittance form (fp32 arithmetic over fp32 or BF16 cells).
int launch_render_logt_f32(const RenderArgs<float>& a, int mode, int phase, cudaStream_t s);
int launch_render_logt_bf16(const RenderArgs<float>& a, int mode, int phase, cudaStream_t s);

// Slots per lane (K) used for a ray of S samples: one chunk up to 512 samples,
// 256-sample chunks beyond.
inline int pick_slots(int S) {
#ifdef PGB_FORCE_SLOTS
  if (S <= 32 * kMaxChunks * PGB_FORCE_SLOTS) return PGB_FORCE_SLOTS;
#endif
  if (S <= 64) return 2;
  if (S <= 128) return 4;
  if (S <= 256) return 8;
  if (S <= 512) return 16;
  return 8;
}

}  // namespace pgb
