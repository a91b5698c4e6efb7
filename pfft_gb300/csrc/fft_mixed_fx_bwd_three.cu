// Instantiation unit of the mixed-radix pass kernel (fft_mixed.cuh):
// 64-bit fixed point (FX), backward, lengths 24, 48, 96, 192, 384, 768.
#include "fft_mixed.cuh"

namespace pg {
namespace fast {

template <class P, int SIGN>
int launch_mixed_three(int N, const FastArgs& a, bool row_in, bool row_out, cudaStream_t s) {
  switch (N) {
    case 24: return launch_mixed_n<P, SIGN, 24>(a, row_in, row_out, s);
    case 48: return launch_mixed_n<P, SIGN, 48>(a, row_in, row_out, s);
    case 96: return launch_mixed_n<P, SIGN, 96>(a, row_in, row_out, s);
    case 192: return launch_mixed_n<P, SIGN, 192>(a, row_in, row_out, s);
    case 384: return launch_mixed_n<P, SIGN, 384>(a, row_in, row_out, s);
    case 768: return launch_mixed_n<P, SIGN, 768>(a, row_in, row_out, s);
  }
  return -1;
}

template int launch_mixed_three<FX, 1>(int, const FastArgs&, bool, bool, cudaStream_t);

}  // namespace fast
}  // namespace pg
