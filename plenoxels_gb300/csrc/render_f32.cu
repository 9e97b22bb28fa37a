// fp32 grid storage: fp32 lookup, compositing and gradients.
#include "render_launch.cuh"

namespace pgb {
int launch_render_f32(const RenderArgs<float>& a, int mode, int phase, cudaStream_t s) {
  return launch_render_t<float, float>(a, mode, phase, s);
}
}  // namespace pgb
