// Window stage kernels for 7-orbital windows (split for parallel builds).
#include "stage_launch.cuh"

namespace ffgb {
template int launch_win_stage<7>(const WinStageParams&, int, int, bool, cudaStream_t);
}  // namespace ffgb
