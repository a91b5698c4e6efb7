// Instantiation unit of the register-resident pass kernel, 64-bit fixed point (FX) (see fft_fast.cuh).
#include "fft_fast.cuh"

namespace pg {
namespace fast {

template <class P, int SIGN>
int launch_large(int N, const FastArgs& a, bool row_in, bool row_out, cudaStream_t s) {
  const bool col = !(row_in && row_out);
  switch (N) {
    case 1024: {
      const int L = a.fastL ? a.fastL : (col ? 4 : 2);
      if (L == 8) return launch4<P, SIGN, 1024, 8>(a, row_in, row_out, s);
      return L == 4 ? launch4<P, SIGN, 1024, 4>(a, row_in, row_out, s) : launch4<P, SIGN, 1024, 2>(a, row_in, row_out, s);
    }
    case 2048:
      return a.fastL == 4 ? launch4<P, SIGN, 2048, 4>(a, row_in, row_out, s) : launch4<P, SIGN, 2048, 2>(a, row_in, row_out, s);
    case 4096:
      return a.fastL == 2 ? launch4<P, SIGN, 4096, 2>(a, row_in, row_out, s) : launch4<P, SIGN, 4096, 1>(a, row_in, row_out, s);
  }
  return -1;
}

template int launch_large<FX, -1>(int, const FastArgs&, bool, bool, cudaStream_t);

}  // namespace fast
}  // namespace pg
