// Instantiation unit of the register-resident pass kernel, 64-bit fixed point (FX) (see fft_fast.cuh).
#include "fft_fast.cuh"

namespace pg {
namespace fast {

template <class P, int SIGN>
int launch_small(int N, const FastArgs& a, bool row_in, bool row_out, cudaStream_t s) {
  const bool col = !(row_in && row_out);
  switch (N) {
    case 16: return launch4<P, SIGN, 16, 128>(a, row_in, row_out, s);
    case 32: return launch4<P, SIGN, 32, 64>(a, row_in, row_out, s);
    case 64: return launch4<P, SIGN, 64, 32>(a, row_in, row_out, s);
    case 128: return launch4<P, SIGN, 128, 16>(a, row_in, row_out, s);
    case 256: return launch4<P, SIGN, 256, 8>(a, row_in, row_out, s);
    case 512: {
      const int L = a.fastL ? a.fastL : (col ? 8 : 4);
      if (L == 16) return launch4<P, SIGN, 512, 16>(a, row_in, row_out, s);
      if (L == 2) return launch4<P, SIGN, 512, 2>(a, row_in, row_out, s);
      return L == 8 ? launch4<P, SIGN, 512, 8>(a, row_in, row_out, s) : launch4<P, SIGN, 512, 4>(a, row_in, row_out, s);
    }
  }
  return -1;
}

template int launch_small<FX, 1>(int, const FastArgs&, bool, bool, cudaStream_t);

}  // namespace fast
}  // namespace pg
