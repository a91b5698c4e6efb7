// Instantiation unit of the mixed-radix pass kernel (fft_mixed.cuh):
// 64-bit fixed point (FX), forward, lengths 40, 80, 160, 320, 640.
#include "fft_mixed.cuh"

namespace pg {
namespace fast {

template <class P, int SIGN>
int launch_mixed_five(int N, const FastArgs& a, bool row_in, bool row_out, cudaStream_t s) {
  switch (N) {
    case 40: return launch_mixed_n<P, SIGN, 40>(a, row_in, row_out, s);
    case 80: return launch_mixed_n<P, SIGN, 80>(a, row_in, row_out, s);
    case 160: return launch_mixed_n<P, SIGN, 160>(a, row_in, row_out, s);
    case 320: return launch_mixed_n<P, SIGN, 320>(a, row_in, row_out, s);
    case 640: return launch_mixed_n<P, SIGN, 640>(a, row_in, row_out, s);
  }
  return -1;
}

template int launch_mixed_five<FX, -1>(int, const FastArgs&, bool, bool, cudaStream_t);

}  // namespace fast
}  // namespace pg
