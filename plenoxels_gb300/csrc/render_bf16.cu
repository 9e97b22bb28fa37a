// BF16 grid storage: cells are widened to fp32 at load; compositing and gradients are fp32.
#include "render_launch.cuh"

namespace pgb {
int launch_render_bf16(const RenderArgs<float>& a, int mode, int phase, cudaStream_t s) {
  return launch_render_t<float, __nv_bfloat16>(a, mode, phase, s);
}
}  // namespace pgb
