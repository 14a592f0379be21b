// Explicit instantiations of the sector kernel (split for parallel builds).
#include "launch.cuh"

namespace ffgb {
template int launch_sector<float, 15>(const SectorParams<float>&, int, int, int, cudaStream_t);
}  // namespace ffgb
