// Twiddle tables W_M^m = exp(-2*pi*i*m/M), m < M, one per (M, arithmetic).
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

const void* twiddle_table(int M, int arith, cudaError_t* err) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto key = std::make_pair(M, arith);
  auto it = g_tables.find(key);
  if (it != g_tables.end()) return it->second;
  size_t esz = arith_sm_bytes(arith);
  std::vector<unsigned char> host((size_t)M * esz);
  for (int m = 0; m < M; m++) {
    long double c, s;
    cis(m, M, &c, &s);
    s = -s;  // forward direction
    if (arith == ARITH_F32) {
      float v[2] = {(float)c, (float)s};
      memcpy(&host[(size_t)m * esz], v, 8);
    } else if (arith == ARITH_F64) {
      double v[2] = {(double)c, (double)s};
      memcpy(&host[(size_t)m * esz], v, 16);
    } else {
      float ch = (float)c, sh = (float)s;
      float v[4] = {ch, (float)(c - (long double)ch), sh, (float)(s - (long double)sh)};
      memcpy(&host[(size_t)m * esz], v, 16);
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
