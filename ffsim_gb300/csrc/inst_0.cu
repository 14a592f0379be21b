// Explicit instantiations of the sector kernel (split for parallel builds).
#include "launch.cuh"

namespace ffgb {
template int launch_sector<double, 0>(const SectorParams<double>&, long long, int, int, cudaStream_t, int*);
template int launch_sector<float, 0>(const SectorParams<float>&, long long, int, int, cudaStream_t, int*);
template int launch_sector<float, 1>(const SectorParams<float>&, long long, int, int, cudaStream_t, int*);
template int launch_sector<float, 2>(const SectorParams<float>&, long long, int, int, cudaStream_t, int*);
template int launch_sector<float, 3>(const SectorParams<float>&, long long, int, int, cudaStream_t, int*);
template int launch_sector<float, 4>(const SectorParams<float>&, long long, int, int, cudaStream_t, int*);
template int launch_sector<float, 5>(const SectorParams<float>&, long long, int, int, cudaStream_t, int*);
template int launch_sector<float, 6>(const SectorParams<float>&, long long, int, int, cudaStream_t, int*);
template int launch_sector<float, 7>(const SectorParams<float>&, long long, int, int, cudaStream_t, int*);
template int launch_sector<float, 8>(const SectorParams<float>&, long long, int, int, cudaStream_t, int*);
}  // namespace ffgb
