// Instantiation unit of the radix-8 pass kernel for paired REDFT01 passes
// (two real lines combined before the transform, IO kind 4 in fft_fast.cuh),
// 64-bit fixed point (FX): 16..512-point lines, lines contiguous on both sides
// or on neither.
#include "fft_fast.cuh"

namespace pg {
namespace fast {

template <class P, int SIGN>
int launch_dct_pinv(int N, const FastArgs& a, bool row_in, bool row_out, cudaStream_t s) {
  if (row_in != row_out) return -1;
  switch (N) {
    case 16: return launch4<P, SIGN, 16, 128, 4>(a, row_in, row_out, s);
    case 32: return launch4<P, SIGN, 32, 64, 4>(a, row_in, row_out, s);
    case 64: return launch4<P, SIGN, 64, 32, 4>(a, row_in, row_out, s);
    case 128: return launch4<P, SIGN, 128, 16, 4>(a, row_in, row_out, s);
    case 256: return launch4<P, SIGN, 256, 8, 4>(a, row_in, row_out, s);
    case 512: return row_in ? launch4<P, SIGN, 512, 4, 4>(a, row_in, row_out, s)
                            : launch4<P, SIGN, 512, 8, 4>(a, row_in, row_out, s);
  }
  return -1;
}

template int launch_dct_pinv<FX, 1>(int, const FastArgs&, bool, bool, cudaStream_t);

}  // namespace fast
}  // namespace pg
