// Twiddle tables W_M^m = exp(-2*pi*i*m/M), m < M, one per (M, arithmetic),
// and the tables of the radix-8 / mixed-radix kernels (kinds in pass.h).
// Computed once on the host in long double (octant-folded argument) and kept
// in device memory until pfft_cleanup().
#include <math.h>
#include <string.h>
#include <map>
#include <mutex>
#include <utility>
#include <vector>
#include "core.h"

namespace pg {

namespace {
std::mutex g_mu;
std::map<std::pair<int, int>, void*> g_tables;

// cos and sin of 2*pi*k/M with the argument folded into [0, pi/4]
void cis(long long k, long long M, long double* c, long double* s) {
  k %= M;
  if (k < 0) k += M;
  // angle = 2*pi*k/M ; octant index from 8k/M
  long long k8 = 8 * k;
  int oct = (int)(k8 / M);
  const long double pi = 3.141592653589793238462643383279502884L;
  // fractional part within the octant, mirrored for odd octants
  long long rem = k8 - (long long)oct * M;  // 0 <= rem < M
  long double phi;
  if (oct & 1)
    phi = (pi / 4) * (long double)(M - rem) / (long double)M;
  else
    phi = (pi / 4) * (long double)rem / (long double)M;
  long double a = cosl(phi), b = sinl(phi);
  long double cc, ss;
  switch (oct) {
    case 0: cc = a; ss = b; break;
    case 1: cc = b; ss = a; break;
    case 2: cc = -b; ss = a; break;
    case 3: cc = -a; ss = b; break;
    case 4: cc = -a; ss = -b; break;
    case 5: cc = -b; ss = -a; break;
    case 6: cc = b; ss = -a; break;
    default: cc = a; ss = -b; break;
  }
  *c = cc;
  *s = ss;
}
}  // namespace

namespace {
// packed float-float entry of w = c + i s: high pair (c, c, -s, s) into h,
// low pair into l
void packed_entry(long double c, long double s, float* h, float* l) {
  const float rh = (float)c, ih = (float)s;
  const float rl = (float)(c - (long double)rh), il = (float)(s - (long double)ih);
  h[0] = rh; h[1] = rh; h[2] = -ih; h[3] = ih;
  l[0] = rl; l[1] = rl; l[2] = -il; l[3] = il;
}
// v * 2^62 rounded to an integer, split as hi * 2^32 + lo, lo in [-2^31, 2^31)
void fx_split(long double v, int* hl) {
  const long long x = llroundl(ldexpl(v, 62));
  const long long hi = (x + (1ll << 31)) >> 32;
  hl[0] = (int)hi;
  hl[1] = (int)(x - hi * (1ll << 32));
}
}  // namespace

const void* twiddle_table(int M, int arith, cudaError_t* err) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto key = std::make_pair(M, arith);
  auto it = g_tables.find(key);
  if (it != g_tables.end()) return it->second;
  const bool fx = arith == TW_FX_FWD_STG || arith == TW_FX_BWD_STG || arith == TW_FX_FWD || arith == TW_FX_BWD;
  const bool staged = arith == TW_F32_STG || arith == TW_DFP_FWD_STG || arith == TW_DFP_BWD_STG ||
                      arith == TW_FX_FWD_STG || arith == TW_FX_BWD_STG;
  const bool packed = arith == TW_DFP_FWD || arith == TW_DFP_BWD || arith == TW_DFP_FWD_STG || arith == TW_DFP_BWD_STG;
  const bool bwd = arith == TW_DFP_BWD || arith == TW_DFP_BWD_STG || arith == TW_FX_BWD_STG || arith == TW_FX_BWD;
  if (staged && (M < 16 || (M & (M - 1)))) {
    if (err) *err = cudaErrorInvalidValue;
    return nullptr;
  }
  // entry j of the table: exponent m of W_M^m
  std::vector<long long> expo;
  if (staged) {
    int p8 = 8;
    while (p8 * 8 <= M) p8 *= 8;
    const int q = M / p8;
    for (int Ns = 8; Ns < p8; Ns *= 8)
      for (int r = 1; r < 8; r++)
        for (int k = 0; k < Ns; k++) expo.push_back((long long)k * r * (M / (Ns * 8)));
    for (int r = 1; r < q; r++)
      for (int j = 0; j < M / q; j++) expo.push_back((long long)j * r);
  } else {
    for (int m = 0; m < M; m++) expo.push_back(m);
  }
  const size_t n = expo.size();
  size_t bytes;
  if (packed || fx)
    bytes = n * (packed ? 32 : 24);
  else if (arith == ARITH_F32 || arith == TW_F32_STG)
    bytes = n * 8;
  else
    bytes = n * (size_t)arith_sm_bytes(arith);
  std::vector<unsigned char> host(bytes > 0 ? bytes : 16);
  for (size_t j = 0; j < n; j++) {
    long double c, s;
    cis(expo[j], M, &c, &s);
    s = -s;  // forward direction
    if (fx) {
      if (bwd) s = -s;
      int a[4], ns[2];
      fx_split(c, a);
      fx_split(s, a + 2);
      fx_split(-s, ns);
      memcpy(&host[j * 16], a, 16);
      memcpy(&host[n * 16 + j * 8], ns, 8);
    } else if (packed) {
      if (bwd) s = -s;
      float h[4], l[4];
      packed_entry(c, s, h, l);
      memcpy(&host[j * 16], h, 16);
      memcpy(&host[(n + j) * 16], l, 16);
    } else if (arith == ARITH_F32 || arith == TW_F32_STG) {
      float v[2] = {(float)c, (float)s};
      memcpy(&host[j * 8], v, 8);
    } else if (arith == ARITH_F64) {
      double v[2] = {(double)c, (double)s};
      memcpy(&host[j * 16], v, 16);
    } else {
      float ch = (float)c, sh = (float)s;
      float v[4] = {ch, (float)(c - (long double)ch), sh, (float)(s - (long double)sh)};
      memcpy(&host[j * 16], v, 16);
    }
  }
  void* d = nullptr;
  cudaError_t e = cudaMalloc(&d, host.size());
  if (e == cudaSuccess) e = cudaMemcpy(d, host.data(), host.size(), cudaMemcpyHostToDevice);
  if (err) *err = e;
  if (e != cudaSuccess) {
    if (d) cudaFree(d);
    return nullptr;
  }
  g_tables[key] = d;
  return d;
}

void twiddle_release_all() {
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto& kv : g_tables) cudaFree(kv.second);
  g_tables.clear();
}

}  // namespace pg
