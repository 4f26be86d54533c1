// 3D complex-to-real FFT of the GetHI fields on GB300, FP32.
//
// Replaces fftw_wrap (src/fourier.c:78-99, fftwf_plan_dft_c2r_3d, sign +1,
// unnormalised) plus the normalisation loop (src/fourier.c:397-412), the
// Gaussian variance (src/fourier.c:24-76) and, for velocity_mode=spectral,
// the radial projection of the velocity.
//
// Layout in HBM ("split half spectrum"): for kx < N/2 the modes live in
// main[kz][ky][kx] (row length m = N/2 complex, rows 16-byte aligned); the
// kx = N/2 (Nyquist) plane lives in nyq[kz][ky].  The transform is three
// passes, each one read and one write of the field:
//   pass Z: inverse c2c along kz of every (ky,kx) column.  The modes are drawn
//           on the fly (Philox, or an uploaded spectrum) and, in the same
//           kernel, up to three fields are transformed from them: delta,
//           phi = delta f0 H0/k^2 and i k_z phi.  Along a z column k_x and k_y
//           are constant, so the Z-transformed v_x and v_y are i k_x and i k_y
//           times the Z-transformed phi and need no transform of their own;
//   pass Y: inverse c2c along ky (v_x, v_y: phi times i k_x or i k_y on load);
//   pass X: per (z,y) row the N-point c2r is an N/2-point complex FFT of
//           Z[k] = (X_k + X*_{m-k}) + i e^{2 pi i k/N} (X_k - X*_{m-k}); the result
//           (x[2j], x[2j+1]) overwrites the row in place, so the real field is a
//           compact N^3 float grid with the same bytes as main.  For the
//           spectral velocity one X kernel transforms v_x, v_y, v_z and writes
//           v_r = v . (x - x_obs)/|x - x_obs| once.
// Only Re X_0 and Re X_{N/2} enter the x c2r, i.e. the result is the real part
// of the full inverse DFT of the Hermitian-extended spectrum (the reference
// draws the kx=0 and kx=N/2 planes without Hermitian symmetry).
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdio>
#include <type_traits>

#include "common.cuh"
#include "fft.h"
#include "dfloat.cuh"
#include "modes.cuh"
#include "tc.cuh"

namespace gethi {

// ---------------------------------------------------------------------------
// column passes (Z and Y)
// element (col, e) of a column set lives at base + (col/cpp) pstride + (col%cpp) cstride + e estride
//   MODE 0: out = FFT(in)                   (in = g.base, out = out1 or in place)
//   MODE 1: draw delta_k and write FFT(delta) to g.base, and (nout >= 2)
//           FFT(phi) to out1, (nout == 3) FFT(i kz phi) to out2
//   MODE 4: out = FFT(i kx in)  (kx of the column; 0 on the Nyquist plane)
//   MODE 5: out = FFT(i ky in)  (ky of the element; 0 at the Nyquist index)
// ---------------------------------------------------------------------------
template <int L, int P, int TX, class Rad, int MODE>
__global__ void __launch_bounds__(TX *(L / P), TX *(L / P) >= 512 ? 1 : 2)
    col_pass_kernel(DevCfg c, ColGeom g, int nyq, int nout, const float2 *__restrict__ src,
                    const float2 *__restrict__ tw, float2 *out1, float2 *out2)
{
  constexpr int T = L / P;
  constexpr int R0 = radix_first(Rad{}), RL = radix_last(Rad{});
  extern __shared__ float2 smem[];
  const int tid = threadIdx.x, cl = tid % TX, t = tid / TX;
  const long col = (long)blockIdx.x * TX + cl;
  const bool active = col < g.ncols;
  const long cb = (col / g.cpp) * g.pstride + (col % g.cpp) * g.cstride;
  const int ky = nyq ? (int)col : (int)(col / c.m), kx = nyq ? c.m : (int)(col % c.m);  // MODE 1 columns
  float2 v[P];
  if constexpr (MODE == 1) {
    float2 d[P];
    static_assert(R0 % 2 == 0, "modes kz and kz + N/2 sit in first-stage slots r and r + R0/2");
#pragma unroll
    for (int j = 0; j < P / R0; j++)
#pragma unroll
      for (int r = 0; r < R0 / 2; r++) {
        const int e = t + T * j + (L / R0) * r;  // e < N/2; its partner e + N/2 is slot r + R0/2
        float2 lo = make_float2(0.f, 0.f), hi = lo;
        if (active) {
          if (src) {
            lo = mode_value(c, e, ky, kx, FIELD_DENS, src);
            hi = mode_value(c, e + L / 2, ky, kx, FIELD_DENS, src);
          } else {
            const uint4 o = philox_for_pair(c, e, ky, kx);
            lo = mode_from_words(c, e, ky, kx, o.x, o.y);
            hi = mode_from_words(c, e + L / 2, ky, kx, o.z, o.w);
          }
        }
        d[j * R0 + r] = lo;
        d[j * R0 + r + R0 / 2] = hi;
      }
#pragma unroll
    for (int i = 0; i < P; i++) v[i] = d[i];
#pragma unroll 1
    for (int f = 0; f < nout; f++) {
      if (f > 0) {
#pragma unroll
        for (int j = 0; j < P / R0; j++)
#pragma unroll
          for (int r = 0; r < R0; r++) {
            const int e = t + T * j + (L / R0) * r;
            const float s = vfac_over_k2(c, e, ky, kx);
            float2 x = cscale(d[j * R0 + r], s);
            if (f == 2) x = cmul_i(cscale(x, 2 * e == c.n ? 0.f : kval(e, c.n, c.dk)));
            v[j * R0 + r] = x;
          }
        __syncthreads();  // the previous transform's last shared-memory reads are done
      }
      stockham_run<L, P>(v, smem + cl, TX, t, tw, Rad{});
      float2 *o = f == 0 ? g.base : (f == 1 ? out1 : out2);
      if (active) {
#pragma unroll
        for (int j = 0; j < P / RL; j++)
#pragma unroll
          for (int r = 0; r < RL; r++) o[cb + (long)(t + T * j + (L / RL) * r) * g.estride] = v[j * RL + r];
      }
    }
  } else {
    float2 *o = out1 ? out1 : g.base;
    float fcol = 0.f;
    if constexpr (MODE == 4) fcol = nyq ? 0.f : kval((int)(col % c.m), c.n, c.dk);
#pragma unroll
    for (int j = 0; j < P / R0; j++)
#pragma unroll
      for (int r = 0; r < R0; r++) {
        const int e = t + T * j + (L / R0) * r;
        float2 x = active ? g.base[cb + (long)e * g.estride] : make_float2(0.f, 0.f);
        if constexpr (MODE == 4) x = cmul_i(cscale(x, fcol));
        if constexpr (MODE == 5) x = cmul_i(cscale(x, 2 * e == c.n ? 0.f : kval(e, c.n, c.dk)));
        v[j * R0 + r] = x;
      }
    stockham_run<L, P>(v, smem + cl, TX, t, tw, Rad{});
    if (active) {
#pragma unroll
      for (int j = 0; j < P / RL; j++)
#pragma unroll
        for (int r = 0; r < RL; r++) o[cb + (long)(t + T * j + (L / RL) * r) * g.estride] = v[j * RL + r];
    }
  }
}

// ---------------------------------------------------------------------------
// Y pass with TMA-staged column tiles (MODE 0: out = FFT(in); 4: FFT(i kx in);
// 5: FFT(i ky in)).  A tile is TX adjacent kx columns of one kz plane, L rows of
// ky: in HBM L rows of TX complex values (row stride N/2 complex), in shared
// memory the same [row][column] layout the Stockham exchanges use.  A persistent
// CTA walks its tiles; one thread issues the tensor-map copies of a tile (L/256
// boxes of 256 rows, complete_tx on the buffer's mbarrier).  With NBUF = 2 the
// next tile's copies are issued before the current tile is transformed; with
// NBUF = 1 they are issued once it is transformed and the other CTAs on the SM
// cover the wait.  The first Stockham stage reads the tile from shared memory;
// the buffer then serves as the exchange buffer of that tile's later stages, and
// the last stage stores straight to HBM.  Every wait is bounded by 1 s of the
// global timer: on expiry the CTA raises *err, waits (again bounded) for its
// copies in flight and stops.
// ---------------------------------------------------------------------------
constexpr uint64_t kTmaWaitNs = 1000000000ull;

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar)
{
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
      ::"r"(tc::smem_addr(dst)), "l"(map), "r"(x), "r"(y), "r"(z), "r"(tc::smem_addr(bar))
      : "memory");
}

template <int L, int P, int TX, int MINB, int NBUF, class Rad, int MODE>
__global__ void __launch_bounds__(TX *(L / P), MINB)
    col_tma_kernel(DevCfg c, const __grid_constant__ CUtensorMap map, long ntiles, const float2 *__restrict__ tw,
                   float2 *out, int *err)
{
  constexpr int T = L / P;
  constexpr int R0 = radix_first(Rad{}), RL = radix_last(Rad{});
  constexpr int BOX = L < 256 ? L : 256;
  constexpr uint32_t kTileBytes = (uint32_t)(L * TX * sizeof(float2));
  extern __shared__ float2 smem_raw[];  // NBUF tiles of [L][TX], from a 128-byte boundary
  float2 *smem = smem_raw + ((128u - (tc::smem_addr(smem_raw) & 127u)) & 127u) / sizeof(float2);
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ int stop;
  const int tid = threadIdx.x, cl = tid % TX, t = tid / TX;
  const int m = c.m, n = c.n;
  const long tiles_per_plane = m / TX;
  auto issue = [&](long tile, int b) {
    const int kz = (int)(tile / tiles_per_plane), kx0 = (int)(tile % tiles_per_plane) * TX;
    tc::mbar_arrive_expect_tx(&bar[b], kTileBytes);
#pragma unroll
    for (int r0 = 0; r0 < L; r0 += BOX) tma_load_3d(smem + b * L * TX + r0 * TX, &map, 2 * kx0, r0, kz, &bar[b]);
  };
  if (tid == 0) {
    tc::mbar_init(&bar[0], 1);
    tc::mbar_init(&bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    stop = 0;
    if ((long)blockIdx.x < ntiles) issue(blockIdx.x, 0);
  }
  __syncthreads();
  uint32_t phase[2] = {0u, 0u};
  int b = 0;
  for (long tile = blockIdx.x; tile < ntiles; tile += gridDim.x, b = NBUF == 2 ? b ^ 1 : 0) {
    const long next = tile + gridDim.x;
    if (NBUF == 2 && tid == 0 && next < ntiles) issue(next, b ^ 1);  // b^1 was released at the end of the last tile
    if (tid == 0 && !tc::mbar_wait(&bar[b], phase[b], kTmaWaitNs)) {
      if (err) atomicExch(err, 1);
      stop = 1;
    }
    __syncthreads();
    if (stop) break;
    phase[b] ^= 1u;
    float2 *sb = smem + b * L * TX;
    const int kz = (int)(tile / tiles_per_plane), kx = (int)(tile % tiles_per_plane) * TX + cl;
    float fcol = 0.f;
    if constexpr (MODE == 4) fcol = kval(kx, n, c.dk);
    float2 v[P];
#pragma unroll
    for (int j = 0; j < P / R0; j++)
#pragma unroll
      for (int r = 0; r < R0; r++) {
        const int e = t + T * j + (L / R0) * r;
        float2 x = sb[e * TX + cl];
        if constexpr (MODE == 4) x = cmul_i(cscale(x, fcol));
        if constexpr (MODE == 5) x = cmul_i(cscale(x, 2 * e == n ? 0.f : kval(e, n, c.dk)));
        v[j * R0 + r] = x;
      }
    stockham_run<L, P>(v, sb + cl, TX, t, tw, Rad{});  // its first exchange follows a barrier
    float2 *o = out + (long)kz * n * m + kx;
#pragma unroll
    for (int j = 0; j < P / RL; j++)
#pragma unroll
      for (int r = 0; r < RL; r++) o[(long)(t + T * j + (L / RL) * r) * m] = v[j * RL + r];
    // the buffer's generic-proxy accesses are ordered before the tensor copies that refill it
    tc::fence_proxy_async();
    __syncthreads();
    if (NBUF == 1 && tid == 0 && next < ntiles) issue(next, 0);  // one buffer: reloaded once transformed
  }
  if (stop && tid == 0) {  // copies still in flight must land before the CTA's shared memory is released
    for (int k = 0; k < 2; k++) tc::mbar_wait(&bar[k], phase[k], kTmaWaitNs);
  }
}

// ---------------------------------------------------------------------------
// row pass (X): c2r of every (z,y) row
//   EPI 0: write the real row in place (x scale), per-block sum and sum of squares
//   EPI 3: write the real row in place (x scale)
//   EPI 2: rows of v_x (in0), v_y (in1), v_z (in2) -> v_r = sum_j v_j u_j into vr
// ---------------------------------------------------------------------------
// c2r of one row held in shared memory (srow, skewed slots): Z[k] at the
// first-stage positions, then the M-point inverse FFT; srow is reused as the
// exchange buffer
// SKEWIN: the input row sits in the skewed slots (loaded point by point); false:
// in natural order (a bulk copy), which the reads of k and M - k by consecutive
// threads take without bank conflicts as well
template <int M, int P, class Rad, bool SKEWIN = true>
__device__ __forceinline__ void row_c2r_smem(float2 *v, float2 *srow, float2 xm, int t, const float2 *__restrict__ twN,
                                             const float2 *__restrict__ twM)
{
  constexpr int T = M / P;
  constexpr int R0 = radix_first(Rad{});
#pragma unroll
  for (int j = 0; j < P / R0; j++)
#pragma unroll
    for (int r = 0; r < R0; r++) {
      const int k = t + T * j + (M / R0) * r;
      float2 a = srow[sm_slot<SKEWIN>(k, 1)], b = k == 0 ? xm : srow[sm_slot<SKEWIN>(M - k, 1)];
      if (k == 0) {
        a.y = 0.f;
        b.y = 0.f;
      }
      float2 s = make_float2(a.x + b.x, a.y - b.y);  // a + conj(b)
      float2 d = make_float2(a.x - b.x, a.y + b.y);  // a - conj(b)
      v[j * R0 + r] = cadd(s, cmul_i(cmul(__ldg(&twN[k]), d)));
    }
  stockham_run<M, P, true>(v, srow, 1, t, twM, Rad{});
}

// asynchronous copy of one float2 from global to shared memory (cp.async, no
// register staging); completed by cp_async_wait_all
__device__ __forceinline__ void cp_async8(float2 *dst, const float2 *src)
{
  const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all()
{
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// one row of M complex points into shared memory (skewed slots), asynchronously
template <int M, int P>
__device__ __forceinline__ void row_load_async(float2 *srow, const float2 *__restrict__ grow, bool active, int t)
{
  constexpr int T = M / P;
#pragma unroll
  for (int j = 0; j < P; j++) {
    float2 *d = &srow[sm_slot<true>(t + T * j, 1)];
    if (active) cp_async8(d, grow + t + T * j);
    else *d = make_float2(0.f, 0.f);
  }
}

template <int M, int P, int RW, class Rad>
__device__ __forceinline__ void row_c2r(float2 *v, float2 *srow, const float2 *__restrict__ grow, float2 xm,
                                        bool active, int t, const float2 *__restrict__ twN,
                                        const float2 *__restrict__ twM)
{
  row_load_async<M, P>(srow, grow, active, t);
  cp_async_wait_all();
  __syncthreads();
  row_c2r_smem<M, P, Rad>(v, srow, xm, t, twN, twM);
}

// v_r of one row: v . (x - x_obs) accumulated over the components (x in the
// two cells 2e, 2e + 1 of point e), then divided by |x - x_obs| once
template <int M, int P, int RL>
__device__ __forceinline__ void vr_accumulate(const DevCfg &c, int comp, const float2 *v, float2 *acc, int t, float y,
                                              float z)
{
  constexpr int T = M / P;
#pragma unroll
  for (int j = 0; j < P / RL; j++)
#pragma unroll
    for (int r = 0; r < RL; r++) {
      const int e = t + T * j + (M / RL) * r;
      const float2 x = v[j * RL + r];
      if (comp == 0) {
        const float x0 = c.dxf * (2 * e + 0.5f) - c.pos_obsf, x1 = c.dxf * (2 * e + 1.5f) - c.pos_obsf;
        acc[j * RL + r] = make_float2(x.x * x0, x.y * x1);
      } else {
        const float w = comp == 1 ? y : z;
        acc[j * RL + r] = make_float2(fmaf(x.x, w, acc[j * RL + r].x), fmaf(x.y, w, acc[j * RL + r].y));
      }
    }
}

template <int M, int P, int RL>
__device__ __forceinline__ void vr_store(const DevCfg &c, const float2 *acc, float *vrow_f, int t, float y, float z,
                                         float scale)
{
  constexpr int T = M / P;
  float2 *vrow = reinterpret_cast<float2 *>(vrow_f);
  const float yz = y * y + z * z;
#pragma unroll
  for (int j = 0; j < P / RL; j++)
#pragma unroll
    for (int r = 0; r < RL; r++) {
      const int e = t + T * j + (M / RL) * r;
      const float x0 = c.dxf * (2 * e + 0.5f) - c.pos_obsf, x1 = c.dxf * (2 * e + 1.5f) - c.pos_obsf;
      const float s0 = scale * rsqrtf(fmaf(x0, x0, yz)), s1 = scale * rsqrtf(fmaf(x1, x1, yz));
      vrow[e] = make_float2(acc[j * RL + r].x * s0, acc[j * RL + r].y * s1);
    }
}

template <int M, int P, int RW, class Rad, int EPI>
__global__ void __launch_bounds__(RW *(M / P), EPI == 2 ? 512 / (RW * (M / P)) : 3) row_pass_kernel(DevCfg c, RowIn in, long nrows,
                                                               const float2 *__restrict__ twN,
                                                               const float2 *__restrict__ twM, float scale,
                                                               float *vr, double2 *partials)
{
  constexpr int T = M / P;
  constexpr int RL = radix_last(Rad{});
  extern __shared__ float2 smem[];
  const int tid = threadIdx.x, rl = tid / T, t = tid % T;
  const long row = (long)blockIdx.x * RW + rl;
  const bool active = row < nrows;
  float2 *srow = smem + rl * sm_len<M, true>();
  float2 v[P];
  if constexpr (EPI == 2) {
    // the three component rows of this row index go to three shared-memory
    // regions at once, so all their loads are in flight together
    float2 *sr[3];
    float2 xm[3];
#pragma unroll
    for (int comp = 0; comp < 3; comp++) {
      sr[comp] = smem + (comp * RW + rl) * sm_len<M, true>();
      row_load_async<M, P>(sr[comp], in.main[comp] + row * (long)M, active, t);
      xm[comp] = active ? in.nyq[comp][row] : make_float2(0.f, 0.f);
    }
    cp_async_wait_all();
    __syncthreads();
    float2 acc[P];
    const int iy = (int)(row % c.n), iz = (int)(row / c.n);
    const float y = c.dxf * (iy + 0.5f) - c.pos_obsf, z = c.dxf * (iz + 0.5f) - c.pos_obsf;
    // v . (x - x_obs) accumulated over the components, divided by |x - x_obs| once
#pragma unroll 1
    for (int comp = 0; comp < 3; comp++) {
      row_c2r_smem<M, P, Rad>(v, sr[comp], xm[comp], t, twN, twM);
      vr_accumulate<M, P, RL>(c, comp, v, acc, t, y, z);
    }
    if (active) vr_store<M, P, RL>(c, acc, vr + row * (long)c.n, t, y, z, scale);
  } else {
    float2 *grow = in.main[0] + row * (long)M;
    row_c2r<M, P, RW, Rad>(v, srow, grow, active ? in.nyq[0][row] : make_float2(0.f, 0.f), active, t, twN, twM);
    df s1 = df_f(0.f), s2 = df_f(0.f);
    if (active) {
      // per-thread sums in FP32 with Neumaier compensation, carried as double-float pairs
      float a1 = 0.f, c1 = 0.f, a2 = 0.f, c2 = 0.f;
      auto nsum = [](float &acc, float &comp, float val) {
        float s = acc + val;
        comp += fabsf(acc) >= fabsf(val) ? (acc - s) + val : (val - s) + acc;
        acc = s;
      };
#pragma unroll
      for (int j = 0; j < P / RL; j++)
#pragma unroll
        for (int r = 0; r < RL; r++) {
          const int e = t + T * j + (M / RL) * r;
          const float2 x = cscale(v[j * RL + r], scale);
          grow[e] = x;
          if constexpr (EPI == 0) {
            nsum(a1, c1, x.x);
            nsum(a1, c1, x.y);
            nsum(a2, c2, x.x * x.x);  // float squares, src/fourier.c:51
            nsum(a2, c2, x.y * x.y);
          }
        }
      s1 = two_sum(a1, c1);
      s2 = two_sum(a2, c2);
    }
    if constexpr (EPI == 0) {
      // warp reduction in double-float (FP32 TwoSum, ~48 bits); FP64 only for the block's
      // final sum (on GB300 a per-thread FP64 reduction cost the pass ~1.5 ms at 1024^3)
      __shared__ float red[4][32];
      for (int o = 16; o > 0; o >>= 1) {
        const df t1 = {__shfl_xor_sync(0xffffffffu, s1.hi, o), __shfl_xor_sync(0xffffffffu, s1.lo, o)};
        const df t2 = {__shfl_xor_sync(0xffffffffu, s2.hi, o), __shfl_xor_sync(0xffffffffu, s2.lo, o)};
        s1 = df_add(s1, t1);
        s2 = df_add(s2, t2);
      }
      const int w = tid >> 5, lane = tid & 31, nw = (RW * T + 31) >> 5;
      __syncthreads();
      if (lane == 0) {
        red[0][w] = s1.hi;
        red[1][w] = s1.lo;
        red[2][w] = s2.hi;
        red[3][w] = s2.lo;
      }
      __syncthreads();
      if (tid == 0) {
        double a = 0, b = 0;
        for (int i = 0; i < nw; i++) {
          a += (double)red[0][i] + (double)red[1][i];
          b += (double)red[2][i] + (double)red[3][i];
        }
        partials[blockIdx.x] = make_double2(a, b);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Fused v_r X pass, persistent, rows staged by bulk copies: a CTA walks groups
// of RW rows; one thread copies the group's three component rows (RW x 3 copies
// of N/2 complex, cp.async.bulk completing on one mbarrier) into natural-order
// slots of the skewed row buffers, which the c2r's Stockham exchanges then use.
// Along a row y and z are constant and the c2r is linear, so the y and z terms
// of v . (x - x_obs) are combined in the spectrum, W = y V_y + z V_z, and a row
// takes two transforms (V_x and W) instead of three.  Once a group is stored the
// buffers are refilled with the CTA's next group; the other CTAs on the SM cover
// that wait.  Waits are bounded by 1 s of the global timer (on expiry: *err
// raised, copies in flight awaited, stop).
// ---------------------------------------------------------------------------
template <int M, int P, int RW, int MINB, class Rad>
__global__ void __launch_bounds__(RW *(M / P), MINB)
    row_vel_bulk_kernel(DevCfg c, RowIn in, long ngroups, const float2 *__restrict__ twN,
                        const float2 *__restrict__ twM, float scale, float *vr, int *err)
{
  constexpr int T = M / P, RL = radix_last(Rad{}), SL = sm_len<M, true>();
  constexpr uint32_t kRowBytes = M * sizeof(float2);
  extern __shared__ float2 smem_raw[];  // [comp][row of the group][SL], from a 128-byte boundary
  float2 *smem = smem_raw + ((128u - (tc::smem_addr(smem_raw) & 127u)) & 127u) / sizeof(float2);
  __shared__ __align__(8) uint64_t bar;
  __shared__ int stop;
  const int tid = threadIdx.x, rl = tid / T, t = tid % T;
  auto issue = [&](long g) {
    tc::mbar_arrive_expect_tx(&bar, 3 * RW * kRowBytes);
#pragma unroll
    for (int comp = 0; comp < 3; comp++)
#pragma unroll
      for (int r = 0; r < RW; r++)
        tc::bulk_g2s(smem + (comp * RW + r) * SL, in.main[comp] + (g * RW + r) * (long)M, kRowBytes, &bar);
  };
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    stop = 0;
    if ((long)blockIdx.x < ngroups) issue(blockIdx.x);
  }
  __syncthreads();
  uint32_t phase = 0;
  float2 *sr[3];
#pragma unroll
  for (int comp = 0; comp < 3; comp++) sr[comp] = smem + (comp * RW + rl) * SL;
  for (long g = blockIdx.x; g < ngroups; g += gridDim.x) {
    const long row = g * RW + rl;
    float2 xm[3];
#pragma unroll
    for (int comp = 0; comp < 3; comp++) xm[comp] = in.nyq[comp][row];
    if (tid == 0 && !tc::mbar_wait(&bar, phase, kTmaWaitNs)) {
      if (err) atomicExch(err, 1);
      stop = 1;
    }
    __syncthreads();
    if (stop) break;
    phase ^= 1u;
    float2 v[P], acc[P];
    const int iy = (int)(row % c.n), iz = (int)(row / c.n);
    const float y = c.dxf * (iy + 0.5f) - c.pos_obsf, z = c.dxf * (iz + 0.5f) - c.pos_obsf;
    // W = y V_y + z V_z into the V_y buffer (natural order), Nyquist terms likewise
#pragma unroll
    for (int j = 0; j < P; j++) {
      const int k = t + T * j;
      const float2 a = sr[1][k], b = sr[2][k];
      sr[1][k] = make_float2(fmaf(y, a.x, z * b.x), fmaf(y, a.y, z * b.y));
    }
    const float2 xmw = make_float2(fmaf(y, xm[1].x, z * xm[2].x), fmaf(y, xm[1].y, z * xm[2].y));
    __syncthreads();
    row_c2r_smem<M, P, Rad, false>(v, sr[0], xm[0], t, twN, twM);
    vr_accumulate<M, P, RL>(c, 0, v, acc, t, y, z);
    row_c2r_smem<M, P, Rad, false>(v, sr[1], xmw, t, twN, twM);
#pragma unroll
    for (int i = 0; i < P; i++) acc[i] = make_float2(acc[i].x + v[i].x, acc[i].y + v[i].y);
    vr_store<M, P, RL>(c, acc, vr + row * (long)c.n, t, y, z, scale);
    tc::fence_proxy_async();  // this group's accesses before the copies that refill the buffers
    __syncthreads();
    if (tid == 0 && g + (long)gridDim.x < ngroups) issue(g + gridDim.x);
  }
  if (stop && tid == 0) tc::mbar_wait(&bar, phase, kTmaWaitNs);
}

// ---------------------------------------------------------------------------
// Density X pass, persistent, rows staged by bulk copies (as the v_r pass): the
// real row is written back in place, and each thread's FP32 sums of delta and
// delta^2 (Neumaier-compensated, src/fourier.c:43-54) run over all its groups.
// Block b writes partials[b] and zeroes partials[b + k gridDim.x] < npartials,
// the entries of the launch shape that had one block per row group.
// ---------------------------------------------------------------------------
template <int M, int P, int RW, int MINB, class Rad>
__global__ void __launch_bounds__(RW *(M / P), MINB)
    row_den_bulk_kernel(DevCfg c, float2 *main, const float2 *__restrict__ nyq, long ngroups,
                        const float2 *__restrict__ twN, const float2 *__restrict__ twM, float scale,
                        double2 *partials, long npartials, int *err)
{
  constexpr int T = M / P, RL = radix_last(Rad{}), SL = sm_len<M, true>();
  constexpr uint32_t kRowBytes = M * sizeof(float2);
  extern __shared__ float2 smem_raw[];  // [row of the group][SL], from a 128-byte boundary
  float2 *smem = smem_raw + ((128u - (tc::smem_addr(smem_raw) & 127u)) & 127u) / sizeof(float2);
  __shared__ __align__(8) uint64_t bar;
  __shared__ int stop;
  __shared__ float red[4][32];
  const int tid = threadIdx.x, rl = tid / T, t = tid % T;
  auto issue = [&](long g) {
    tc::mbar_arrive_expect_tx(&bar, RW * kRowBytes);
#pragma unroll
    for (int r = 0; r < RW; r++) tc::bulk_g2s(smem + r * SL, main + (g * RW + r) * (long)M, kRowBytes, &bar);
  };
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    stop = 0;
    if ((long)blockIdx.x < ngroups) issue(blockIdx.x);
  }
  __syncthreads();
  uint32_t phase = 0;
  float2 *srow = smem + rl * SL;
  float a1 = 0.f, c1 = 0.f, a2 = 0.f, c2 = 0.f;
  auto nsum = [](float &acc, float &comp, float val) {
    float s = acc + val;
    comp += fabsf(acc) >= fabsf(val) ? (acc - s) + val : (val - s) + acc;
    acc = s;
  };
  for (long g = blockIdx.x; g < ngroups; g += gridDim.x) {
    const long row = g * RW + rl;
    const float2 xm = nyq[row];
    if (tid == 0 && !tc::mbar_wait(&bar, phase, kTmaWaitNs)) {
      if (err) atomicExch(err, 1);
      stop = 1;
    }
    __syncthreads();
    if (stop) break;
    phase ^= 1u;
    float2 v[P];
    row_c2r_smem<M, P, Rad, false>(v, srow, xm, t, twN, twM);
    float2 *grow = main + row * (long)M;
#pragma unroll
    for (int j = 0; j < P / RL; j++)
#pragma unroll
      for (int r = 0; r < RL; r++) {
        const int e = t + T * j + (M / RL) * r;
        const float2 x = cscale(v[j * RL + r], scale);
        grow[e] = x;
        nsum(a1, c1, x.x);
        nsum(a1, c1, x.y);
        nsum(a2, c2, x.x * x.x);  // float squares, src/fourier.c:51
        nsum(a2, c2, x.y * x.y);
      }
    tc::fence_proxy_async();  // this group's accesses before the copies that refill the buffers
    __syncthreads();
    if (tid == 0 && g + (long)gridDim.x < ngroups) issue(g + gridDim.x);
  }
  if (stop && tid == 0) tc::mbar_wait(&bar, phase, kTmaWaitNs);
  // warp reduction in double-float, FP64 for the block's sum
  df s1 = two_sum(a1, c1), s2 = two_sum(a2, c2);
  for (int o = 16; o > 0; o >>= 1) {
    const df t1 = {__shfl_xor_sync(0xffffffffu, s1.hi, o), __shfl_xor_sync(0xffffffffu, s1.lo, o)};
    const df t2 = {__shfl_xor_sync(0xffffffffu, s2.hi, o), __shfl_xor_sync(0xffffffffu, s2.lo, o)};
    s1 = df_add(s1, t1);
    s2 = df_add(s2, t2);
  }
  const int w = tid >> 5, lane = tid & 31, nw = (RW * T + 31) >> 5;
  __syncthreads();
  if (lane == 0) {
    red[0][w] = s1.hi;
    red[1][w] = s1.lo;
    red[2][w] = s2.hi;
    red[3][w] = s2.lo;
  }
  __syncthreads();
  if (tid == 0) {
    double a = 0, b = 0;
    for (int i = 0; i < nw; i++) {
      a += (double)red[0][i] + (double)red[1][i];
      b += (double)red[2][i] + (double)red[3][i];
    }
    partials[blockIdx.x] = make_double2(a, b);
  }
  for (long i = blockIdx.x + (long)gridDim.x * (1 + tid); i < npartials; i += (long)gridDim.x * blockDim.x)
    partials[i] = make_double2(0.0, 0.0);
}

// Kahan-compensated FP64 sum of the per-block partials -> stats = (mean, sigma^2)
__global__ void finish_sigma_kernel(const double2 *__restrict__ partials, int np, double ncells, double *stats)
{
  __shared__ double sh[4][256];
  double a = 0, ca = 0, b = 0, cb = 0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) {
    double2 p = partials[i];
    double y = p.x - ca, t = a + y;
    ca = (t - a) - y;
    a = t;
    y = p.y - cb;
    t = b + y;
    cb = (t - b) - y;
    b = t;
  }
  sh[0][threadIdx.x] = a;
  sh[1][threadIdx.x] = -ca;
  sh[2][threadIdx.x] = b;
  sh[3][threadIdx.x] = -cb;
  __syncthreads();
  if (threadIdx.x == 0) {
    double A = 0, CA = 0, B = 0, CB = 0;
    for (int i = 0; i < (int)blockDim.x; i++) {
      for (int q = 0; q < 2; q++) {
        double y = sh[q][i] - CA, t = A + y;
        CA = (t - A) - y;
        A = t;
        y = sh[2 + q][i] - CB;
        t = B + y;
        CB = (t - B) - y;
        B = t;
      }
    }
    double mean = A / ncells;
    stats[0] = mean;
    stats[1] = B / ncells - mean * mean;  // src/fourier.c:74
  }
}

// ---------------------------------------------------------------------------
// Gaussianised spectrum on the grid (gaussianise=1):
//   xi(x) = c2r(P~/V), xi_G = ln(1 + xi) in FP64, P_G = (V/N^3) c2r(xi_G),
// where c2r(xi_G) is the forward DFT because xi_G is real and even.
// ---------------------------------------------------------------------------
// P~(|k|)/V on the split half spectrum (imaginary parts zero)
__global__ void pack_pk_kernel(DevCfg c, float2 *main, float2 *nyq, float inv_vol)
{
  const int n = c.n, m = c.m;
  const long total = (long)n * n * (m + 1);
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const int kk = (int)(i % (m + 1));
    const long rest = i / (m + 1);
    const int jj = (int)(rest % n), ii = (int)(rest / n);
    float kz = kval(ii, n, c.dk), ky = kval(jj, n, c.dk), kx = kval(kk, n, c.dk);
    float k2 = kx * kx + ky * ky + kz * kz;
    float p = 0.f;
    if (k2 > 0.f) {
      p = pk_lookup(c, 0.5f * log10f(k2));
      if (c.do_smoothing) p *= expf(-c.r2_smooth * k2);  // src/fourier.c:294-295
    }
    const float2 v = make_float2(p * inv_vol, 0.f);
    if (kk < m) main[rest * m + kk] = v;
    else nyq[rest] = v;
  }
}

// xi (real, compact N^3) -> half grid of ln(1 + xi) packed as a half spectrum
__global__ void log_xi_kernel(DevCfg c, const float *__restrict__ xi, float2 *main, float2 *nyq)
{
  const int n = c.n, m = c.m;
  const long total = (long)n * n * (m + 1);
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const int x = (int)(i % (m + 1));
    const long row = i / (m + 1);
    double v = (double)xi[row * n + x];
    v = v > -1.0 + 1e-12 ? v : -1.0 + 1e-12;
    const float2 g = make_float2((float)log1p(v), 0.f);  // the log transform in FP64
    if (x < m) main[row * m + x] = g;
    else nyq[row] = g;
  }
}

// standalone mode generator (inspection): reference layout [kz][ky][N/2+1]
__global__ void modes_kernel(DevCfg c, float2 *out)
{
  const long h = c.m + 1;
  const long total = (long)c.n * c.n * h;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    int kk = (int)(i % h);
    long rest = i / h;
    int jj = (int)(rest % c.n), ii = (int)(rest / c.n);
    out[i] = mode_value(c, ii, jj, kk, FIELD_DENS, nullptr);
  }
}

// ---------------------------------------------------------------------------
// launch plumbing
// ---------------------------------------------------------------------------
template <int L> struct ColPlan;
template <int M> struct RowPlan;
template <int M> struct RowPlanV;
// columns: L = N; P points per thread, TX columns per block.  At 2048 points a column of the
// spectrum steps 16 MB per element, so wide tiles (512 threads) keep the pages touched per byte low
template <> struct ColPlan<2048> { static constexpr int P = 32, TX = 8; using R = Radices<32, 8, 8>; };
template <> struct ColPlan<1024> { static constexpr int P = 32, TX = 8; using R = Radices<32, 32>; };
template <> struct ColPlan<512> { static constexpr int P = 32, TX = 16; using R = Radices<32, 16>; };
template <> struct ColPlan<384> { static constexpr int P = 24, TX = 16; using R = Radices<8, 8, 6>; };
template <> struct ColPlan<256> { static constexpr int P = 16, TX = 16; using R = Radices<16, 16>; };
template <> struct ColPlan<128> { static constexpr int P = 16, TX = 16; using R = Radices<16, 8>; };
template <> struct ColPlan<64> { static constexpr int P = 8, TX = 16; using R = Radices<8, 8>; };
template <> struct ColPlan<32> { static constexpr int P = 8, TX = 16; using R = Radices<8, 4>; };
template <> struct ColPlan<24> { static constexpr int P = 12, TX = 16; using R = Radices<12, 2>; };
template <> struct ColPlan<16> { static constexpr int P = 4, TX = 16; using R = Radices<4, 4>; };
// half-width column tiles (a second launch shape for the autotuner) at the ensemble sizes
template <int L> struct ColPlanNarrow;
template <> struct ColPlanNarrow<384> { static constexpr int P = 24, TX = 8; using R = Radices<8, 8, 6>; };
template <> struct ColPlanNarrow<256> { static constexpr int P = 16, TX = 8; using R = Radices<16, 16>; };
template <> struct ColPlanNarrow<128> { static constexpr int P = 16, TX = 8; using R = Radices<16, 8>; };
template <int L> constexpr bool has_narrow() { return L == 128 || L == 256 || L == 384; }
// columns of the drawing Z pass (modes kept in registers for up to three transforms)
template <int L> struct ColPlanGen : ColPlan<L> {};
template <> struct ColPlanGen<2048> { static constexpr int P = 16, TX = 4; using R = Radices<16, 16, 8>; };
template <> struct ColPlanGen<1024> { static constexpr int P = 16, TX = 8; using R = Radices<16, 16, 4>; };  // TX 4: 12.45 ms, 8: 12.03 ms at 1024^3
template <> struct ColPlanGen<512> { static constexpr int P = 16, TX = 8; using R = Radices<16, 16, 2>; };
// rows: M = N/2 (single field)
template <> struct RowPlan<1024> { static constexpr int P = 32, RW = 4; using R = Radices<32, 8, 4>; };
template <> struct RowPlan<512> { static constexpr int P = 32, RW = 16; using R = Radices<32, 16>; };
template <> struct RowPlan<256> { static constexpr int P = 16, RW = 16; using R = Radices<16, 16>; };
template <> struct RowPlan<192> { static constexpr int P = 24, RW = 16; using R = Radices<8, 8, 3>; };
template <> struct RowPlan<128> { static constexpr int P = 16, RW = 16; using R = Radices<16, 8>; };
template <> struct RowPlan<64> { static constexpr int P = 8, RW = 32; using R = Radices<8, 8>; };
template <> struct RowPlan<32> { static constexpr int P = 8, RW = 32; using R = Radices<8, 4>; };
template <> struct RowPlan<16> { static constexpr int P = 4, RW = 32; using R = Radices<4, 4>; };
template <> struct RowPlan<12> { static constexpr int P = 12, RW = 32; using R = Radices<12>; };
template <> struct RowPlan<8> { static constexpr int P = 8, RW = 32; using R = Radices<8>; };
// rows of the fused velocity pass (an accumulator per point: fewer points per thread)
template <> struct RowPlanV<1024> { static constexpr int P = 16, RW = 2; using R = Radices<16, 16, 4>; };
template <> struct RowPlanV<512> { static constexpr int P = 16, RW = 4; using R = Radices<16, 16, 2>; };
template <> struct RowPlanV<256> { static constexpr int P = 16, RW = 8; using R = Radices<16, 16>; };
template <> struct RowPlanV<192> { static constexpr int P = 24, RW = 16; using R = Radices<8, 8, 3>; };
template <> struct RowPlanV<128> { static constexpr int P = 16, RW = 16; using R = Radices<16, 8>; };
template <> struct RowPlanV<64> { static constexpr int P = 8, RW = 16; using R = Radices<8, 8>; };
template <> struct RowPlanV<32> { static constexpr int P = 8, RW = 32; using R = Radices<8, 4>; };
template <> struct RowPlanV<16> { static constexpr int P = 4, RW = 32; using R = Radices<4, 4>; };
template <> struct RowPlanV<12> { static constexpr int P = 12, RW = 32; using R = Radices<12>; };
template <> struct RowPlanV<8> { static constexpr int P = 8, RW = 32; using R = Radices<8>; };

template <int L, int MODE, class PL>
static cudaError_t launch_col_plan(const DevCfg &c, const ColGeom &g, int nyq, int nout, const float2 *src,
                                   const float2 *tw, float2 *out1, float2 *out2, cudaStream_t st)
{
  constexpr int threads = PL::TX * (L / PL::P);
  const size_t sm = sizeof(float2) * PL::TX * L;
  auto kern = col_pass_kernel<L, PL::P, PL::TX, typename PL::R, MODE>;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    attr = true;
  }
  long blocks = (g.ncols + PL::TX - 1) / PL::TX;
  kern<<<(unsigned)blocks, threads, sm, st>>>(c, g, nyq, nout, src, tw, out1, out2);
  return cudaGetLastError();
}

template <int L, int MODE>
static cudaError_t launch_col(const DevCfg &c, const ColGeom &g, int nyq, int nout, const float2 *src,
                              const float2 *tw, float2 *out1, float2 *out2, cudaStream_t st)
{
  if constexpr (has_narrow<L>()) {
    if (c.col_variant == 1) return launch_col_plan<L, MODE, ColPlanNarrow<L>>(c, g, nyq, nout, src, tw, out1, out2, st);
  }
  using PL = typename std::conditional<MODE == 1, ColPlanGen<L>, ColPlan<L>>::type;
  return launch_col_plan<L, MODE, PL>(c, g, nyq, nout, src, tw, out1, out2, st);
}

// TMA-staged Y passes: tile plans per column length
template <int L> struct TmaPlan { static constexpr bool ok = false; };
// One buffer per CTA and two CTAs per SM measured faster than two buffers in one
// CTA (Y passes at 1024^3: 6.20 against 7.47 ms; register-loaded tiles 7.11 ms):
// the transform of a 64 KB tile outlasts its load, so the second CTA's
// transform is what hides the first one's copies.
template <> struct TmaPlan<1024> { static constexpr bool ok = true; static constexpr int P = 32, TX = 8, MINB = 2, NBUF = 1; using R = Radices<32, 32>; };
template <> struct TmaPlan<256> { static constexpr bool ok = true; static constexpr int P = 16, TX = 8, MINB = 4, NBUF = 1; using R = Radices<16, 16>; };
template <> struct TmaPlan<512> { static constexpr bool ok = true; static constexpr int P = 32, TX = 8, MINB = 4, NBUF = 1; using R = Radices<32, 16>; };

// the driver's tensor-map encoder, looked up once (thread-safe static initialisation)
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
    cudaDriverEntryPointQueryResult q;
    void *p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    cudaGetLastError();
    return nullptr;
  }();
  return fn;
}

// the Y-pass column set of a split half spectrum: columns (kz, kx < N/2), elements along ky
static bool y_geometry(const DevCfg &c, const ColGeom &g, int nyq)
{
  return !nyq && g.cstride == 1 && g.cpp == c.m && g.estride == c.m && g.pstride == (long)c.n * c.m &&
         g.ncols == (long)c.n * c.m;
}

template <int L, int MODE>
static cudaError_t launch_col_tma(const DevCfg &c, const ColGeom &g, const float2 *tw, float2 *out, cudaStream_t st)
{
  using PL = TmaPlan<L>;
  constexpr int threads = PL::TX * (L / PL::P);
  constexpr int box = L < 256 ? L : 256;
  const size_t sm = PL::NBUF * sizeof(float2) * PL::TX * L + 128;
  auto kern = col_tma_kernel<L, PL::P, PL::TX, PL::MINB, PL::NBUF, typename PL::R, MODE>;
  static int bps = 0;
  if (!bps) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, threads, sm);
    if (e != cudaSuccess) return e;
    if (bps < 1) return cudaErrorInvalidConfiguration;
  }
  auto encode = tensor_map_encoder();
  if (!encode) return cudaErrorNotSupported;
  CUtensorMap map;
  const cuuint64_t dims[3] = {(cuuint64_t)2 * c.m, (cuuint64_t)c.n, (cuuint64_t)c.n};
  const cuuint64_t strides[2] = {(cuuint64_t)c.m * sizeof(float2), (cuuint64_t)c.n * c.m * sizeof(float2)};
  const cuuint32_t boxd[3] = {2 * PL::TX, box, 1}, estr[3] = {1, 1, 1};
  if (encode(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void *)g.base, dims, strides, boxd, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return cudaErrorInvalidValue;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long ntiles = (long)c.n * (c.m / PL::TX);
  const long grid = ntiles < (long)sms * bps ? ntiles : (long)sms * bps;
  kern<<<(unsigned)grid, threads, sm, st>>>(c, map, ntiles, tw, out, c.tc_err);
  return cudaGetLastError();
}

template <int L>
static bool col_tma(const DevCfg &c, const ColGeom &g, int nyq, int mode, const float2 *tw, float2 *out1,
                    cudaStream_t st, cudaError_t &e)
{
  if constexpr (!TmaPlan<L>::ok) {
    return false;
  } else {
    if (c.col_variant != 0 || !y_geometry(c, g, nyq) || (mode != 0 && mode != 4 && mode != 5)) return false;
    if ((reinterpret_cast<uintptr_t>(g.base) & 15) || !tensor_map_encoder()) return false;
    float2 *out = out1 ? out1 : g.base;
    e = mode == 0 ? launch_col_tma<L, 0>(c, g, tw, out, st)
                  : (mode == 4 ? launch_col_tma<L, 4>(c, g, tw, out, st) : launch_col_tma<L, 5>(c, g, tw, out, st));
    return true;
  }
}

template <int M, int EPI, class PL>
static cudaError_t launch_row(const DevCfg &c, const RowIn &in, const float2 *twN, const float2 *twM, float scale,
                              float *vr, double2 *partials, cudaStream_t st)
{
  constexpr int threads = PL::RW * (M / PL::P);
  const size_t sm = sizeof(float2) * PL::RW * sm_len<M, true>() * (EPI == 2 ? 3 : 1);
  auto kern = row_pass_kernel<M, PL::P, PL::RW, typename PL::R, EPI>;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    attr = true;
  }
  const long nrows = (long)c.n * c.n;
  long blocks = (nrows + PL::RW - 1) / PL::RW;
  kern<<<(unsigned)blocks, threads, sm, st>>>(c, in, nrows, twN, twM, scale, vr, partials);
  return cudaGetLastError();
}

// persistent bulk-copy v_r X pass: plans per row length (N/2 complex points).
// 32 points per thread won at 512- and 1024-point rows (1024^3: v_r 4.20 -> 3.60 ms,
// density 1.86 -> 1.69 ms; 2048^3: 39.0 -> 32.9 and 17.4 -> 15.2 ms) and lost at
// 256-point rows (512^3: 0.39 -> 0.51 and 0.20 -> 0.23 ms)
template <int M> struct VelBulkPlan { static constexpr bool ok = false; };
template <> struct VelBulkPlan<128> { static constexpr bool ok = true; static constexpr int P = 16, RW = 16, MINB = 4; using R = Radices<16, 8>; };
template <> struct VelBulkPlan<256> { static constexpr bool ok = true; static constexpr int P = 16, RW = 8, MINB = 4; using R = Radices<16, 16>; };
template <> struct VelBulkPlan<512> { static constexpr bool ok = true; static constexpr int P = 32, RW = 4, MINB = 4; using R = Radices<32, 16>; };
template <> struct VelBulkPlan<1024> { static constexpr bool ok = true; static constexpr int P = 32, RW = 2, MINB = 4; using R = Radices<32, 32>; };

template <int M>
static bool row_vel_bulk(const DevCfg &c, const RowIn &in, const float2 *twN, const float2 *twM, float scale,
                         float *vr, cudaStream_t st, cudaError_t &e)
{
  if constexpr (!VelBulkPlan<M>::ok) {
    return false;
  } else {
    using PL = VelBulkPlan<M>;
    if (c.col_variant != 0) return false;
    for (int k = 0; k < 3; k++)
      if (reinterpret_cast<uintptr_t>(in.main[k]) & 15) return false;
    constexpr int threads = PL::RW * (M / PL::P);
    const size_t sm = sizeof(float2) * 3 * PL::RW * sm_len<M, true>() + 128;
    auto kern = row_vel_bulk_kernel<M, PL::P, PL::RW, PL::MINB, typename PL::R>;
    static int bps = 0;
    if (!bps) {
      e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, threads, sm);
      if (e != cudaSuccess) return true;
      if (bps < 1) {
        e = cudaErrorInvalidConfiguration;
        return true;
      }
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long ngroups = (long)c.n * c.n / PL::RW;
    const long grid = ngroups < (long)sms * bps ? ngroups : (long)sms * bps;
    kern<<<(unsigned)grid, threads, sm, st>>>(c, in, ngroups, twN, twM, scale, vr, c.tc_err);
    e = cudaGetLastError();
    return true;
  }
}

// persistent bulk-copy density X pass
template <int M> struct DenBulkPlan { static constexpr bool ok = false; };
template <> struct DenBulkPlan<128> { static constexpr bool ok = true; static constexpr int P = 16, RW = 16, MINB = 8; using R = Radices<16, 8>; };
template <> struct DenBulkPlan<256> { static constexpr bool ok = true; static constexpr int P = 16, RW = 8, MINB = 8; using R = Radices<16, 16>; };
template <> struct DenBulkPlan<512> { static constexpr bool ok = true; static constexpr int P = 32, RW = 4, MINB = 8; using R = Radices<32, 16>; };
template <> struct DenBulkPlan<1024> { static constexpr bool ok = true; static constexpr int P = 32, RW = 2, MINB = 8; using R = Radices<32, 32>; };

template <int M>
static bool row_den_bulk(const DevCfg &c, const RowIn &in, const float2 *twN, const float2 *twM, float scale,
                         double2 *partials, long npartials, cudaStream_t st, cudaError_t &e)
{
  if constexpr (!DenBulkPlan<M>::ok) {
    return false;
  } else {
    using PL = DenBulkPlan<M>;
    if (c.col_variant != 0 || !partials || (reinterpret_cast<uintptr_t>(in.main[0]) & 15)) return false;
    constexpr int threads = PL::RW * (M / PL::P);
    const size_t sm = sizeof(float2) * PL::RW * sm_len<M, true>() + 128;
    auto kern = row_den_bulk_kernel<M, PL::P, PL::RW, PL::MINB, typename PL::R>;
    static int bps = 0;
    if (!bps) {
      e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, threads, sm);
      if (e != cudaSuccess) return true;
      if (bps < 1) {
        e = cudaErrorInvalidConfiguration;
        return true;
      }
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long ngroups = (long)c.n * c.n / PL::RW;
    long grid = ngroups < (long)sms * bps ? ngroups : (long)sms * bps;
    grid = grid < npartials ? grid : npartials;
    kern<<<(unsigned)grid, threads, sm, st>>>(c, in.main[0], in.nyq[0], ngroups, twN, twM, scale, partials,
                                              npartials, c.tc_err);
    e = cudaGetLastError();
    return true;
  }
}

long row_pass_blocks(int n)
{
  long nrows = (long)n * n;
  int rw = 0;
  switch (n / 2) {
    case 1024: rw = RowPlan<1024>::RW; break;
    case 512: rw = RowPlan<512>::RW; break;
    case 256: rw = RowPlan<256>::RW; break;
    case 192: rw = RowPlan<192>::RW; break;
    case 128: rw = RowPlan<128>::RW; break;
    case 64: rw = RowPlan<64>::RW; break;
    case 32: rw = RowPlan<32>::RW; break;
    case 16: rw = RowPlan<16>::RW; break;
    case 12: rw = RowPlan<12>::RW; break;
    case 8: rw = RowPlan<8>::RW; break;
    default: return -1;
  }
  return (nrows + rw - 1) / rw;
}

bool fft_supported(int n)
{
  switch (n) {
    case 16: case 24: case 32: case 64: case 128: case 256: case 384: case 512: case 1024: case 2048: return true;
    default: return false;
  }
}

#define GETHI_COL_CASE(LV, MV) \
  case LV: return launch_col<LV, MV>(c, g, nyq, nout, src, tw, out1, out2, st);
#define GETHI_COL_DISPATCH(MV)                                                                        \
  switch (c.n) {                                                                                      \
    GETHI_COL_CASE(2048, MV) GETHI_COL_CASE(1024, MV) GETHI_COL_CASE(512, MV) GETHI_COL_CASE(384, MV) \
    GETHI_COL_CASE(256, MV) GETHI_COL_CASE(128, MV) GETHI_COL_CASE(64, MV) GETHI_COL_CASE(32, MV)     \
    GETHI_COL_CASE(24, MV) GETHI_COL_CASE(16, MV)                                                     \
    default: return cudaErrorInvalidValue;                                                            \
  }

cudaError_t col_pass(const DevCfg &c, const ColGeom &g, int nyq, int mode, int nout, const float2 *src,
                     const float2 *tw, float2 *out1, float2 *out2, cudaStream_t st)
{
  if (tc_col_supported(c, g, nyq)) return tc_col_pass(c, g, mode, nout, src, out1, out2, st);
  cudaError_t te = cudaSuccess;
  if (c.n == 1024 && col_tma<1024>(c, g, nyq, mode, tw, out1, st, te)) return te;
  if (c.n == 512 && col_tma<512>(c, g, nyq, mode, tw, out1, st, te)) return te;
  if (c.n == 256 && col_tma<256>(c, g, nyq, mode, tw, out1, st, te)) return te;
  switch (mode) {
    case 0: GETHI_COL_DISPATCH(0)
    case 1: GETHI_COL_DISPATCH(1)
    case 4: GETHI_COL_DISPATCH(4)
    case 5: GETHI_COL_DISPATCH(5)
    default: return cudaErrorInvalidValue;
  }
}

#define GETHI_ROW_CASE(MV, EPIV, PLAN) \
  case MV: return launch_row<MV, EPIV, PLAN<MV>>(c, in, twN, twM, scale, vr, partials, st);
#define GETHI_ROW_DISPATCH(EPIV, PLAN)                                                                        \
  switch (c.m) {                                                                                              \
    GETHI_ROW_CASE(1024, EPIV, PLAN) GETHI_ROW_CASE(512, EPIV, PLAN) GETHI_ROW_CASE(256, EPIV, PLAN)          \
    GETHI_ROW_CASE(192, EPIV, PLAN) GETHI_ROW_CASE(128, EPIV, PLAN) GETHI_ROW_CASE(64, EPIV, PLAN)            \
    GETHI_ROW_CASE(32, EPIV, PLAN) GETHI_ROW_CASE(16, EPIV, PLAN) GETHI_ROW_CASE(12, EPIV, PLAN)              \
    GETHI_ROW_CASE(8, EPIV, PLAN)                                                                             \
    default: return cudaErrorInvalidValue;                                                                    \
  }

cudaError_t row_pass(const DevCfg &c, const RowIn &in, const float2 *twN, const float2 *twM, float scale, int epi,
                     float *vr, double2 *partials, cudaStream_t st)
{
  cudaError_t be = cudaSuccess;
  const long np = row_pass_blocks(c.n);
  if (epi == 0 && c.m == 128 && row_den_bulk<128>(c, in, twN, twM, scale, partials, np, st, be)) return be;
  if (epi == 0 && c.m == 256 && row_den_bulk<256>(c, in, twN, twM, scale, partials, np, st, be)) return be;
  if (epi == 0 && c.m == 512 && row_den_bulk<512>(c, in, twN, twM, scale, partials, np, st, be)) return be;
  if (epi == 0 && c.m == 1024 && row_den_bulk<1024>(c, in, twN, twM, scale, partials, np, st, be)) return be;
  if (epi == 2 && c.m == 128 && row_vel_bulk<128>(c, in, twN, twM, scale, vr, st, be)) return be;
  if (epi == 2 && c.m == 256 && row_vel_bulk<256>(c, in, twN, twM, scale, vr, st, be)) return be;
  if (epi == 2 && c.m == 512 && row_vel_bulk<512>(c, in, twN, twM, scale, vr, st, be)) return be;
  if (epi == 2 && c.m == 1024 && row_vel_bulk<1024>(c, in, twN, twM, scale, vr, st, be)) return be;
  switch (epi) {
    case 0: GETHI_ROW_DISPATCH(0, RowPlan)
    case 2: GETHI_ROW_DISPATCH(2, RowPlanV)
    case 3: GETHI_ROW_DISPATCH(3, RowPlan)
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t finish_sigma(const double2 *partials, int np, double ncells, double *stats, cudaStream_t st)
{
  finish_sigma_kernel<<<1, 256, 0, st>>>(partials, np, ncells, stats);
  return cudaGetLastError();
}

cudaError_t pack_pk(const DevCfg &c, float2 *main, float2 *nyq, float inv_vol, cudaStream_t st)
{
  pack_pk_kernel<<<152 * 16, 256, 0, st>>>(c, main, nyq, inv_vol);
  return cudaGetLastError();
}

cudaError_t log_xi(const DevCfg &c, const float *xi, float2 *main, float2 *nyq, cudaStream_t st)
{
  log_xi_kernel<<<152 * 16, 256, 0, st>>>(c, xi, main, nyq);
  return cudaGetLastError();
}

cudaError_t gen_modes(const DevCfg &c, float2 *out, int kind, cudaStream_t st)
{
  (void)kind;
  modes_kernel<<<1024, 256, 0, st>>>(c, out);
  return cudaGetLastError();
}

}  // namespace gethi
