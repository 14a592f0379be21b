// Explicit instantiations of the sector kernel (split for parallel builds).
#include "launch.cuh"

namespace ffgb {
template int launch_sector<float, 15>(const SectorParams<float>&, long long, int, int, cudaStream_t, int*);
}  // namespace ffgb
