// Explicit instantiations of the sector kernel (split for parallel builds).
#include "launch.cuh"

namespace ffgb {
template int launch_sector<float, 13>(const SectorParams<float>&, long long, int, int, cudaStream_t, int*);
template int launch_sector<float, 14>(const SectorParams<float>&, long long, int, int, cudaStream_t, int*);
}  // namespace ffgb
