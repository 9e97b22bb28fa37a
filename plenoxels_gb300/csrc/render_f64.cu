// fp64 grid storage and arithmetic, for finite-difference and fp64-oracle checks.
#include "render_launch.cuh"

namespace pgb {
int launch_render_f64(const RenderArgs<double>& a, int mode, int phase, cudaStream_t s) {
  return launch_render_t<double, double>(a, mode, phase, s);
}
}  // namespace pgb
