// Column passes (Z, Y) of the 3D c2r on the tcgen05 tensor cores, split precision
// (fft_precision=tc_split).
//
// A 1024-point column transform is two batches of 32-point DFTs (1024 = 32 x 32,
// Cooley-Tukey with the twiddles W_1024^{n2 k1} between them):
//   stage 1: y[n2][k1] = sum_{n1} W_32^{n1 k1} x[32 n1 + n2]
//   stage 2: X[k1 + 32 k2] = sum_{n2} W_32^{n2 k2} (W_1024^{n2 k1} y[n2][k1])
// Each batch is a real GEMM D[rows x 64] = A[rows x 64] B[64 x 64]: a row of A is
// one 32-point sequence with (re, im) interleaved along K, B is the 32-point DFT
// in real 2x2-block form.  Operands are FP16 pairs a = a_hi + a_lo (11 + 11
// significant bits) and D = A_hi B_hi + A_hi B_lo + A_lo B_hi accumulates in FP32
// in TMEM; the dropped A_lo B_lo and the split residuals are ~2^-22 relative.  Each
// transform is scaled by a power of two (exact) so that FP16 cannot overflow.
//
// A tile = 4 adjacent columns, handled by a "slot" of 128 threads (one sequence
// per thread and stage, one M=128 MMA).  A CTA of 4 independent slots (own
// operand buffers, TMEM columns, mbarrier and named barrier; shared DFT tables)
// runs per SM, persistent over tiles, so that one slot's loads overlap another's
// MMAs (a kernel that allocates TMEM is resident once per SM).  Rows are ordered (sequence index, column), so a
// warp's global loads and stores cover 8 runs of 4 adjacent columns (one 32-byte
// sector each).  Every wait on the
// MMA-completion barrier is bounded (1 s of the GPU's global timer): on expiry the kernel records an error,
// waits once more (bounded) for the MMAs in flight, frees its TMEM and returns.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "common.cuh"
#include "fft.h"
#include "modes.cuh"
#include "tc.cuh"

namespace gethi {
namespace {

constexpr int kL = 1024, kTX = 4, kThreads = 128, kSlots = 4;  // kThreads per slot
constexpr uint32_t kLBO = 128, kSBO = 1024;     // K-adjacent core matrices contiguous; 8 rows = 1 KB
constexpr uint32_t kABytes = 128 * 128;         // 128 rows x 64 halves
constexpr uint32_t kBBytes = 64 * 128;          // 64 rows (outputs) x 64 halves (inputs)
constexpr uint32_t kTwBytes = kL * 8;           // inter-stage twiddles (float2)
constexpr size_t kSmem = 2 * kBBytes + kTwBytes + kSlots * 2 * kABytes;
constexpr uint32_t kTmemCols = 128;             // two 128 x 64 FP32 accumulators per slot
constexpr uint64_t kWaitNs = 1000000000ull;      // 1 s bound on every MMA-completion wait
constexpr float kStage2Scale = 1.f / 32.f;      // folded into the twiddle table

__device__ __forceinline__ uint32_t core_off(int r, int j) { return (r >> 3) * kSBO + j * kLBO + (r & 7) * 16; }


// element (column, e): input with the per-mode factor of the pass
template <int MODE>
__device__ __forceinline__ float2 factor_in(const DevCfg &c, float2 x, int e, int f, int ky, int kx, float fcol)
{
  if constexpr (MODE == 1) {
    if (f > 0) {
      x = cscale(x, vfac_over_k2(c, e, ky, kx));
      if (f == 2) x = cmul_i(cscale(x, 2 * e == c.n ? 0.f : kval(e, c.n, c.dk)));
    }
  } else if constexpr (MODE == 4) {
    x = cmul_i(cscale(x, fcol));
  } else if constexpr (MODE == 5) {
    x = cmul_i(cscale(x, 2 * e == c.n ? 0.f : kval(e, c.n, c.dk)));
  }
  return x;
}

// named barrier of one slot (ids 1..kSlots; 0 is __syncthreads)
__device__ __forceinline__ void slot_sync(int slot)
{
  asm volatile("bar.sync %0, %1;" ::"r"(slot + 1), "r"(kThreads) : "memory");
}

// x = hi + lo for the two components of v, packed as half2 (re in the low half)
__device__ __forceinline__ void split2(float2 v, uint32_t &hi, uint32_t &lo)
{
  const __half2 h = __floats2half2_rn(v.x, v.y);
  const float2 hf = __half22float2(h);
  const __half2 l = __floats2half2_rn(v.x - hf.x, v.y - hf.y);
  hi = *reinterpret_cast<const uint32_t *>(&h);
  lo = *reinterpret_cast<const uint32_t *>(&l);
}

template <int MODE>
__global__ void __launch_bounds__(kThreads *kSlots, 1)
    tc_col_kernel(DevCfg c, ColGeom g, int nout, const float2 *__restrict__ src, const uint4 *__restrict__ bmat,
                  const float2 *__restrict__ tw, float2 *out1, float2 *out2, int *err)
{
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint64_t mbar[kSlots];
  __shared__ uint32_t tslot;
  __shared__ float red[kSlots][kThreads / 32];
  __shared__ int fail[kSlots];

  const int slot = threadIdx.x / kThreads, t = threadIdx.x % kThreads, w = t >> 5, lane = t & 31;
  const int c4 = t & 3;  // column within the tile
  const int q = t >> 2;  // stage 1: n2 of the sequence; stage 2: k1
  unsigned char *Bhi = sm;
  float2 *stw = reinterpret_cast<float2 *>(sm + 2 * kBBytes);
  unsigned char *Ahi = sm + 2 * kBBytes + kTwBytes + slot * 2 * kABytes, *Alo = Ahi + kABytes;

  for (int i = threadIdx.x; i < (int)(2 * kBBytes / 16); i += kThreads * kSlots)
    reinterpret_cast<uint4 *>(Bhi)[i] = bmat[i];
  for (int i = threadIdx.x; i < kL; i += kThreads * kSlots) stw[i] = tw[i];
  if (threadIdx.x < 32) tc::tmem_alloc(&tslot, kTmemCols * kSlots);
  if (t == 0) {
    tc::mbar_init(&mbar[slot], 1);
    fail[slot] = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tm = tslot + kTmemCols * slot;           // this slot's accumulator columns
  const uint32_t trow = tm + ((uint32_t)(32 * w) << 16);  // this thread's row (TMEM lane t)
  const uint32_t a_hi = tc::smem_addr(Ahi), a_lo = tc::smem_addr(Alo), b_hi = tc::smem_addr(Bhi),
                 b_lo = b_hi + kBBytes;
  constexpr uint32_t idesc = tc::idesc_f16_f32(128, 64);
  uint64_t *bar = &mbar[slot];
  uint32_t phase = 0;
  bool alive = true;

  // operands staged by the slot's threads -> its 12 MMAs -> result in TMEM
  auto gemm = [&]() -> bool {
    tc::fence_proxy_async();
    tc::fence_before_sync();
    slot_sync(slot);
    if (t == 0) {  // two independent accumulation chains: hi*hi, and the hi*lo + lo*hi corrections
      tc::fence_after_sync();
#pragma unroll
      for (int kk = 0; kk < 4; kk++) {
        const uint64_t ah = tc::smem_desc(a_hi + 256 * kk, kLBO, kSBO), al = tc::smem_desc(a_lo + 256 * kk, kLBO, kSBO);
        const uint64_t bh = tc::smem_desc(b_hi + 256 * kk, kLBO, kSBO), bl = tc::smem_desc(b_lo + 256 * kk, kLBO, kSBO);
        tc::mma_f16(tm, ah, bh, idesc, kk > 0);
        tc::mma_f16(tm + 64, ah, bl, idesc, kk > 0);
        tc::mma_f16(tm + 64, al, bh, idesc, 1);
      }
      tc::mma_commit(bar);
    }
    if (!tc::mbar_wait(bar, phase, kWaitNs)) fail[slot] = 1;
    slot_sync(slot);
    const bool ok = fail[slot] == 0;
    if (!ok) {
      if (t == 0) atomicExch(err, 1);
      tc::mbar_wait(bar, phase, kWaitNs);  // let MMAs still in flight finish before TMEM is freed
    }
    phase ^= 1;
    tc::fence_after_sync();
    return ok;
  };

  const long ntiles = g.ncols / kTX, tstep = (long)gridDim.x * kSlots;
  const long es32 = 32 * g.estride;
  // element (q + 32 n1) of this thread's column in a tile
  auto column = [&](long tile) -> const float2 * {
    const long col = tile * kTX + c4;
    return g.base + (col / g.cpp) * g.pstride + (col % g.cpp) * g.cstride + (long)q * g.estride;
  };
  float2 x[32];  // x[n1] = element 32 n1 + q of the column
  long tile = (long)blockIdx.x * kSlots + slot;
  if constexpr (MODE != 1) {
    if (tile < ntiles) {
      const float2 *p = column(tile);
#pragma unroll
      for (int n1 = 0; n1 < 32; n1++, p += es32) x[n1] = *p;
    }
  }
  for (; alive && tile < ntiles; tile += tstep) {
    const long col = tile * kTX + c4;
    const long cb = (col / g.cpp) * g.pstride + (col % g.cpp) * g.cstride;
    const int ky = (int)(col / c.m), kx = (int)(col % c.m);  // Z-pass columns (MODE 1)
    float fcol = 0.f;
    if constexpr (MODE == 4) fcol = kval(kx, c.n, c.dk);
    if constexpr (MODE == 1) {
#pragma unroll
      for (int n1 = 0; n1 < 16; n1++) {
        const int e = 32 * n1 + q;  // e < N/2, partner e + N/2 = 32 (n1 + 16) + q
        if (src) {
          x[n1] = mode_value(c, e, ky, kx, FIELD_DENS, src);
          x[n1 + 16] = mode_value(c, e + kL / 2, ky, kx, FIELD_DENS, src);
        } else {
          const uint4 o = philox_for_pair(c, e, ky, kx);
          x[n1] = mode_from_words(c, e, ky, kx, o.x, o.y);
          x[n1 + 16] = mode_from_words(c, e + kL / 2, ky, kx, o.z, o.w);
        }
      }
    }
    const int nf = MODE == 1 ? nout : 1;
    for (int f = 0; f < nf && alive; f++) {
      // power-of-two scale of this transform: |component| < 2^9 on input
      float mx = 0.f;
#pragma unroll
      for (int n1 = 0; n1 < 32; n1++) {
        const float2 y = factor_in<MODE>(c, x[n1], 32 * n1 + q, f, ky, kx, fcol);
        mx = fmaxf(mx, fmaxf(fabsf(y.x), fabsf(y.y)));
      }
#pragma unroll
      for (int s = 16; s > 0; s >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, s));
      if (lane == 0) red[slot][w] = mx;
      slot_sync(slot);
      mx = fmaxf(fmaxf(red[slot][0], red[slot][1]), fmaxf(red[slot][2], red[slot][3]));
      int ex = 0;
      frexpf(mx, &ex);
      const float s_in = ldexpf(1.f, 9 - ex), s_out = ldexpf(1.f, ex - 4);

      // stage-1 operand: this thread's row, K chunk j holds x[4j .. 4j+3]
#pragma unroll
      for (int j = 0; j < 8; j++) {
        uint32_t hw[4], lw[4];
#pragma unroll
        for (int u = 0; u < 4; u++)
          split2(cscale(factor_in<MODE>(c, x[4 * j + u], 32 * (4 * j + u) + q, f, ky, kx, fcol), s_in), hw[u], lw[u]);
        *reinterpret_cast<uint4 *>(Ahi + core_off(t, j)) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
        *reinterpret_cast<uint4 *>(Alo + core_off(t, j)) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
      }
      if constexpr (MODE != 1) {  // the next tile's column loads overlap this tile's MMAs
        if (tile + tstep < ntiles) {
          const float2 *p = column(tile + tstep);
#pragma unroll
          for (int n1 = 0; n1 < 32; n1++, p += es32) x[n1] = *p;
        }
      }
      if (!(alive = gemm())) break;

      // stage-1 result (k1 = 0..31 of sequence n2 = q), twiddles, stage-2 operand:
      // row 4 k1 + c4, K position 2 q.  Half of the warp writes k1 = 2p first and
      // the other half k1 = 2p + 1, so that a store covers all 32 banks.
      {
        const int sw = (lane >> 4) & 1;
        const uint32_t kofs = (q >> 2) * kLBO + (q & 3) * 4 + c4 * 16;
#pragma unroll
        for (int h = 0; h < 4; h++) {
          float v[16], u[16];
          tc::tmem_ld16(trow + 16 * h, v);
          tc::tmem_ld16(trow + 64 + 16 * h, u);
#pragma unroll
          for (int i = 0; i < 16; i++) v[i] += u[i];
#pragma unroll
          for (int pp = 0; pp < 4; pp++) {
            const int k1 = 8 * h + 2 * pp;
            uint32_t h0, l0, h1, l1;
            split2(cmul(make_float2(v[4 * pp], v[4 * pp + 1]), stw[32 * k1 + q]), h0, l0);
            split2(cmul(make_float2(v[4 * pp + 2], v[4 * pp + 3]), stw[32 * (k1 + 1) + q]), h1, l1);
            const uint32_t o = (k1 >> 1) * kSBO + kofs;
            *reinterpret_cast<uint32_t *>(Ahi + o + 64 * sw) = sw ? h1 : h0;
            *reinterpret_cast<uint32_t *>(Alo + o + 64 * sw) = sw ? l1 : l0;
            *reinterpret_cast<uint32_t *>(Ahi + o + 64 * (1 - sw)) = sw ? h0 : h1;
            *reinterpret_cast<uint32_t *>(Alo + o + 64 * (1 - sw)) = sw ? l0 : l1;
          }
        }
      }
      if (!(alive = gemm())) break;

      // stage-2 result: X[q + 32 k2] of column c4
      {
        float2 *o = (MODE == 1 ? (f == 0 ? g.base : (f == 1 ? out1 : out2)) : (out1 ? out1 : g.base)) + cb +
                    (long)q * g.estride;
#pragma unroll
        for (int h = 0; h < 4; h++) {
          float v[16], u[16];
          tc::tmem_ld16(trow + 16 * h, v);
          tc::tmem_ld16(trow + 64 + 16 * h, u);
#pragma unroll
          for (int i = 0; i < 8; i++, o += es32) *o = make_float2((v[2 * i] + u[2 * i]) * s_out, (v[2 * i + 1] + u[2 * i + 1]) * s_out);
        }
      }
      tc::fence_before_sync();
      slot_sync(slot);  // TMEM and the operand buffers are free for the next transform
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tslot, kTmemCols * kSlots);
  }
}

template <int MODE>
cudaError_t launch(const DevCfg &c, const ColGeom &g, int nout, const float2 *src, float2 *out1, float2 *out2,
                   cudaStream_t st)
{
  auto kern = tc_col_kernel<MODE>;
  static int blocks_per_sm[8] = {0};
  int &bps = blocks_per_sm[MODE];
  if (!bps) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, kThreads * kSlots, kSmem);
    if (e != cudaSuccess) return e;
    if (bps < 1) return cudaErrorInvalidConfiguration;
    if (std::getenv("GETHI_TC_VERBOSE")) {
      cudaFuncAttributes fa;
      cudaFuncGetAttributes(&fa, kern);
      int o0 = 0, o16 = 0, o32 = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o0, kern, kThreads * kSlots, 0);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o16, kern, kThreads * kSlots, 16384);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o32, kern, kThreads * kSlots, 32768);
      std::fprintf(stderr,
                   "tc_col_kernel<%d>: %d CTAs per SM (regs %d, static smem %zu, local %zu, maxthreads %d, "
                   "maxdyn %d, carveout %d; occ smem 0/16K/32K: %d %d %d)\n",
                   MODE, bps, fa.numRegs, fa.sharedSizeBytes, fa.localSizeBytes, fa.maxThreadsPerBlock,
                   fa.maxDynamicSharedSizeBytes, fa.preferredShmemCarveout, o0, o16, o32);
    }
  }
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long ntiles = g.ncols / kTX;
  const long grid = std::min<long>((ntiles + kSlots - 1) / kSlots, (long)sms * bps);
  kern<<<(unsigned)grid, kThreads * kSlots, kSmem, st>>>(c, g, nout, src, c.tc_bmat, c.tc_tw, out1, out2, c.tc_err);
  return cudaGetLastError();
}

}  // namespace

// Failure detection of the bounded waits: one warp waits on an mbarrier that
// nothing ever arrives on (no asynchronous copy or MMA is issued), through the
// same bounded wait the tensor-core passes use, and raises the context's error
// flag when the wait expires, as an expired MMA-completion wait does.
__global__ void wait_selftest_kernel(int *err, uint64_t limit_ns)
{
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) tc::mbar_init(&bar, 1);
  __syncthreads();
  if (threadIdx.x == 0 && !tc::mbar_wait(&bar, 0, limit_ns)) atomicExch(err, 1);
  __syncthreads();
}

cudaError_t wait_selftest(int *err, uint64_t limit_ns, cudaStream_t st)
{
  wait_selftest_kernel<<<1, 32, 0, st>>>(err, limit_ns);
  return cudaGetLastError();
}

bool tc_col_supported(const DevCfg &c, const ColGeom &g, int nyq)
{
  return c.tc_bmat && !nyq && c.n == kL && g.cstride == 1 && g.ncols % kTX == 0 && g.cpp % kTX == 0;
}

cudaError_t tc_col_pass(const DevCfg &c, const ColGeom &g, int mode, int nout, const float2 *src, float2 *out1,
                        float2 *out2, cudaStream_t st)
{
  switch (mode) {
    case 0: return launch<0>(c, g, nout, src, out1, out2, st);
    case 1: return launch<1>(c, g, nout, src, out1, out2, st);
    case 4: return launch<4>(c, g, nout, src, out1, out2, st);
    case 5: return launch<5>(c, g, nout, src, out1, out2, st);
    default: return cudaErrorInvalidValue;
  }
}

// The 32-point backward DFT y_k = sum_n e^{+2 pi i k n/32} x_n as a real 64 x 64
// matrix B[q = 2n + s][p = 2k + u] (s, u: 0 re, 1 im), split into FP16 hi and lo
// and laid out as the kernel's shared-memory operand (row p, K-major core
// matrices); the inter-stage twiddles e^{+2 pi i n2 k1/1024} / 32 at [k1][n2].
bool tc_tables(int n, std::vector<uint16_t> &bmat, std::vector<float2> &tw)
{
  if (n != kL) return false;
  bmat.assign(2 * kBBytes / 2, 0);
  for (int p = 0; p < 64; p++)
    for (int qk = 0; qk < 64; qk++) {
      const int k = p >> 1, u = p & 1, nn = qk >> 1, s = qk & 1;
      const int r = (k * nn) & 31;
      const double a = 2 * M_PI * r / 32.0, cs = std::cos(a), sn = std::sin(a);
      const double b = u == 0 ? (s == 0 ? cs : -sn) : (s == 0 ? sn : cs);
      const float bf = (float)b;
      const __half hi = __float2half_rn(bf);
      const __half lo = __float2half_rn(bf - __half2float(hi));
      const size_t off = ((p >> 3) * kSBO + (qk >> 3) * kLBO + (p & 7) * 16 + (qk & 7) * 2) / 2;
      bmat[off] = __half_as_ushort(hi);
      bmat[kBBytes / 2 + off] = __half_as_ushort(lo);
    }
  tw.resize(kL);  // [k1][n2]: a warp's 8 sequences n2 read 8 consecutive entries for one k1
  for (int k1 = 0; k1 < 32; k1++)
    for (int n2 = 0; n2 < 32; n2++) {
      const double a = 2 * M_PI * ((n2 * k1) % kL) / kL;
      tw[32 * k1 + n2] = make_float2((float)(std::cos(a) * kStage2Scale), (float)(std::sin(a) * kStage2Scale));
    }
  return true;
}

size_t tc_table_bytes() { return 2 * kBBytes; }

}  // namespace gethi
