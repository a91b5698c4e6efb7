// Instantiation unit of the radix-8 pass kernel for paired c2r passes (two
// real lines combined before the transform, IO kind 3 in fft_fast.cuh), 64-bit fixed point (FX), backward,
// 16..4096-point lines, default tile heights.
#include "fft_fast.cuh"

namespace pg {
namespace fast {

template <class P, int SIGN>
int launch_gio_pinv(int N, const FastArgs& a, bool row_in, bool row_out, cudaStream_t s) {
  const bool col = !(row_in && row_out);
  switch (N) {
    case 16: return launch4<P, SIGN, 16, 128, 3>(a, row_in, row_out, s);
    case 32: return launch4<P, SIGN, 32, 64, 3>(a, row_in, row_out, s);
    case 64: return launch4<P, SIGN, 64, 32, 3>(a, row_in, row_out, s);
    case 128: return launch4<P, SIGN, 128, 16, 3>(a, row_in, row_out, s);
    case 256: return launch4<P, SIGN, 256, 8, 3>(a, row_in, row_out, s);
    case 512: return col ? launch4<P, SIGN, 512, 8, 3>(a, row_in, row_out, s)
                         : launch4<P, SIGN, 512, 4, 3>(a, row_in, row_out, s);
    case 1024: return col ? launch4<P, SIGN, 1024, 4, 3>(a, row_in, row_out, s)
                          : launch4<P, SIGN, 1024, 2, 3>(a, row_in, row_out, s);
    case 2048: return launch4<P, SIGN, 2048, 2, 3>(a, row_in, row_out, s);
    case 4096: return launch4<P, SIGN, 4096, 1, 3>(a, row_in, row_out, s);
  }
  return -1;
}

template int launch_gio_pinv<FX, 1>(int, const FastArgs&, bool, bool, cudaStream_t);

}  // namespace fast
}  // namespace pg
