// Fused render kernels with the compensated log-sum transmittance over fp32 cells:
// T_s = exp(sum of log(1 - alpha) before s), the precision form's alternative to the
// reference's product scan.
#include "render_launch.cuh"

namespace pgb {
int launch_render_logt_f32(const RenderArgs<float>& a, int mode, int phase, cudaStream_t s) {
  return launch_render_t<float, float, true>(a, mode, phase, s);
}
}  // namespace pgb
