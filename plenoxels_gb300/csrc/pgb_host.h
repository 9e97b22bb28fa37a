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

// Gradient marks: bit u % 32 of word u / 32 marks unit u = cell >> kMarkCellsLog2, a unit
// some step wrote. Units of 4 cells (64 B of fp32 gradient, two whole sectors): a 256^3
// trilinear step took 0.1014 ms per step with them, 0.1011 ms with 2-cell units and
// 0.1074 ms with 1-cell units, whose clear writes half the bytes but as half sectors and
// whose marks touch twice the words.
#ifndef PGB_MARK_CELLS_LOG2
#define PGB_MARK_CELLS_LOG2 2
#endif
constexpr int kMarkCellsLog2 = PGB_MARK_CELLS_LOG2;
// Words of the mark bitmap of a gradient of num_cells cells.
inline int64_t mark_words(int64_t num_cells) {
  const int64_t units = (num_cells + (1 << kMarkCellsLog2) - 1) >> kMarkCellsLog2;
  return (units + 31) / 32;
}

int launch_render_f32(const RenderArgs<float>& a, int mode, int phase, cudaStream_t s);
int launch_render_bf16(const RenderArgs<float>& a, int mode, int phase, cudaStream_t s);
int launch_render_f64(const RenderArgs<double>& a, int mode, int phase, cudaStream_t s);
// Log-sum transmittance form (fp32 arithmetic over fp32 or BF16 cells).
int launch_render_logt_f32(const RenderArgs<float>& a, int mode, int phase, cudaStream_t s);
int launch_render_logt_bf16(const RenderArgs<float>& a, int mode, int phase, cudaStream_t s);

// Slots per lane (K) of a chunk of 32 * K samples. A requested chunk size (32 * K for K
// in 1, 2, 4, 8, 16) is raised until a ray spans at most kMaxChunks chunks. Without one:
// when rays can stop at the first chunk whose transmittance reaches 0 (clip on, no beta
// term), short chunks (32 samples for trilinear lookup, 64 for nearest) skip the most
// samples behind opaque cells (measured on GB300: 256^3 grid, 8192 rays x 256 samples,
// trilinear step 0.175 ms with one 256-sample chunk, 0.133 ms with 32-sample chunks);
// otherwise a ray up to 512 samples is a single chunk and longer rays use 256-sample
// chunks.
inline int pick_slots(int S, int chunk_samples = 0, bool early_stop = false,
                      int mode = PGB_TRILINEAR) {
#ifdef PGB_FORCE_SLOTS
  if (S <= 32 * kMaxChunks * PGB_FORCE_SLOTS) return PGB_FORCE_SLOTS;
#endif
  if (chunk_samples <= 0 && early_stop) chunk_samples = mode == PGB_NEAREST ? 64 : 32;
  if (chunk_samples > 0) {
    int k = 1;
    while (k < 16 && 32 * k < chunk_samples) k *= 2;
    while (k < 16 && (S + 32 * k - 1) / (32 * k) > kMaxChunks) k *= 2;
    return k;
  }
  if (S <= 64) return 2;
  if (S <= 128) return 4;
  if (S <= 256) return 8;
  if (S <= 512) return 16;
  return 8;
}

}  // namespace pgb
