// Fused render kernels with the compensated log-sum transmittance over BF16 cells (fp32
// arithmetic), the precision form.
#include "render_launch.cuh"

namespace pgb {
int launch_render_logt_bf16(const RenderArgs<float>& a, int mode, int phase, cudaStream_t s) {
  return launch_render_t<float, __nv_bfloat16, true>(a, mode, phase, s);
}
}  // namespace pgb
