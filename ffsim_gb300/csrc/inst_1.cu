// Explicit instantiations of the sector kernel (split for parallel builds).
#include "launch.cuh"

namespace ffgb {
template int launch_sector<float, 9>(const SectorParams<float>&, long long, int, int, cudaStream_t, int*);
template int launch_sector<float, 10>(const SectorParams<float>&, long long, int, int, cudaStream_t, int*);
template int launch_sector<float, 11>(const SectorParams<float>&, long long, int, int, cudaStream_t, int*);
template int launch_sector<float, 12>(const SectorParams<float>&, long long, int, int, cudaStream_t, int*);
}  // namespace ffgb
