// colpass_bench: times the 1024-point column transforms of the library (FP32
// CUDA-core pass and tcgen05 split-precision pass) on a column set of the
// Y-pass shape: `planes` planes of 1024 x 512 complex columns (row stride 512),
// transformed in place, so the bytes moved are read + write of the set.
//   colpass_bench [planes=128] [reps=5] [which: 0 fp32, 1 tc, 2 both]
// Prints the time per pass and the bandwidth; exit status 0 on success.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "fft.h"

using namespace gethi;

int main(int argc, char **argv)
{
  const int planes = argc > 1 ? std::atoi(argv[1]) : 128;
  const int reps = argc > 2 ? std::atoi(argv[2]) : 5;
  const int which = argc > 3 ? std::atoi(argv[3]) : 2;
  if (planes < 1 || planes > 1024 || reps < 1) {
    std::fprintf(stderr, "usage: colpass_bench [planes 1..1024] [reps] [0|1|2]\n");
    return 2;
  }
  const long n = 1024, m = 512;
  const size_t elems = (size_t)planes * n * m;
  float2 *buf = nullptr, *twN = nullptr, *dtw = nullptr;
  uint4 *dbm = nullptr;
  int *err = nullptr;
  if (cudaMalloc(&buf, elems * sizeof(float2)) != cudaSuccess) return 1;
  std::vector<float2> h(elems);
  unsigned s = 1;
  for (size_t i = 0; i < elems; i++) {
    s = s * 1664525u + 1013904223u;
    const float a = (s >> 8) * (1.f / 16777216.f) - 0.5f;
    s = s * 1664525u + 1013904223u;
    h[i] = make_float2(a, (s >> 8) * (1.f / 16777216.f) - 0.5f);
  }
  cudaMemcpy(buf, h.data(), elems * sizeof(float2), cudaMemcpyHostToDevice);
  std::vector<uint16_t> bm;
  std::vector<float2> tw;
  tc_tables((int)n, bm, tw);
  cudaMalloc(&dbm, bm.size() * 2);
  cudaMalloc(&dtw, tw.size() * sizeof(float2));
  cudaMalloc(&err, sizeof(int));
  cudaMemset(err, 0, sizeof(int));
  cudaMemcpy(dbm, bm.data(), bm.size() * 2, cudaMemcpyHostToDevice);
  cudaMemcpy(dtw, tw.data(), tw.size() * sizeof(float2), cudaMemcpyHostToDevice);
  std::vector<float2> t(n);
  for (int k = 0; k < n; k++) t[k] = make_float2((float)std::cos(2 * M_PI * k / n), (float)std::sin(2 * M_PI * k / n));
  cudaMalloc(&twN, n * sizeof(float2));
  cudaMemcpy(twN, t.data(), n * sizeof(float2), cudaMemcpyHostToDevice);
  DevCfg c;
  std::memset(&c, 0, sizeof(c));
  c.n = (int)n;
  c.m = (int)m;
  c.dk = 1.f;
  ColGeom g;
  g.base = buf;
  g.cpp = m;
  g.pstride = n * m;
  g.cstride = 1;
  g.estride = m;
  g.ncols = (long)planes * m;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  int rc = 0;
  for (int tc = 0; tc < 2; tc++) {
    if (which != 2 && which != tc) continue;
    c.tc_bmat = tc ? dbm : nullptr;
    c.tc_tw = dtw;
    c.tc_err = err;
    cudaError_t e = col_pass(c, g, 0, 0, 0, nullptr, twN, nullptr, nullptr, 0);  // warm-up
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
      std::fprintf(stderr, "%s\n", cudaGetErrorString(e));
      return 1;
    }
    cudaEventRecord(a);
    for (int r = 0; r < reps; r++) col_pass(c, g, 0, 0, 0, nullptr, twN, nullptr, nullptr, 0);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    ms /= reps;
    std::printf("%s: %.3f ms per pass, %.1f GB/s (read + write %.2f GB)\n", tc ? "tc_split" : "fp32", ms,
                2.0 * elems * sizeof(float2) / ms / 1e6, 2.0 * elems * sizeof(float2) / 1e9);
  }
  int flag = 0;
  cudaMemcpy(&flag, err, sizeof(int), cudaMemcpyDeviceToHost);
  if (flag || cudaGetLastError() != cudaSuccess) rc = 1;
  cudaFree(buf);
  cudaFree(twN);
  cudaFree(dtw);
  cudaFree(dbm);
  cudaFree(err);
  return rc;
}
