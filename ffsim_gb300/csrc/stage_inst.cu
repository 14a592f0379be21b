// Window-stage kernels of window size WIN_B for classes WIN_K0..WIN_K1
// (compiled once per range, see _build.py).
#include "stage_launch.cuh"

namespace ffgb {

#define FFGB_WIN_INST(K)                                                                              \
  template int launch_win_bk<WIN_B, K>(const WinJob&, int, bool, int, long long, cudaStream_t, int*);

#if WIN_K0 <= 0 && 0 <= WIN_K1
FFGB_WIN_INST(0)
#endif
#if WIN_K0 <= 1 && 1 <= WIN_K1 && 1 <= WIN_B
FFGB_WIN_INST(1)
#endif
#if WIN_K0 <= 2 && 2 <= WIN_K1 && 2 <= WIN_B
FFGB_WIN_INST(2)
#endif
#if WIN_K0 <= 3 && 3 <= WIN_K1 && 3 <= WIN_B
FFGB_WIN_INST(3)
#endif
#if WIN_K0 <= 4 && 4 <= WIN_K1 && 4 <= WIN_B
FFGB_WIN_INST(4)
#endif
#if WIN_K0 <= 5 && 5 <= WIN_K1 && 5 <= WIN_B
FFGB_WIN_INST(5)
#endif
#if WIN_K0 <= 6 && 6 <= WIN_K1 && 6 <= WIN_B
FFGB_WIN_INST(6)
#endif
#if WIN_K0 <= 7 && 7 <= WIN_K1 && 7 <= WIN_B
FFGB_WIN_INST(7)
#endif
#if WIN_K0 <= 8 && 8 <= WIN_K1 && 8 <= WIN_B
FFGB_WIN_INST(8)
#endif

}  // namespace ffgb
