// shdom_tc.cuh -- tensor-core (tcgen05) dense transform GEMM for sm_103a.
//
// The spherical-harmonic <-> discrete-ordinate transforms are linear maps
// with a fixed coefficient matrix: C[p][n] = sum_k A[p][k] B[n][k], where A
// is the per-point field (SOURCE [npts][nlm] or the ordinate radiances
// [npts][nang]) and B the masked transform matrix stored [N][K] (K-major).
// FP32 accuracy is kept with the three-product split of TF32 operands:
// A = Ah + Al, B = Bh + Bl (Ah, Bh, Al, Bl rounded to nearest TF32),
// C ~= Ah Bh + Ah Bl + Al Bh.  With split = 0 only Ah Bh is formed (the
// reduced-precision variant).
//
// The tensor cores accumulate a chunk of 32 K-elements into a fresh FP32
// accumulator in tensor memory; the chunks are summed on the CUDA cores in
// FP32 with round-to-nearest.  Measured on a 128x128x64 cloud field
// (NMU=16/NPHI=32) against the FP32 CUDA-core transforms: one accumulator
// over the whole K reduction gave radiances low by 5e-6 (relative) after one
// iteration and by 1.8e-4 after 30 -- a one-signed error that the source
// iteration carries through the scattering orders; with chunked sums the
// same run is low by 3e-7 after one iteration and 1.0e-5 after 30.
//
// Stages of 32 K-elements (one 128-byte swizzle row) are brought in by TMA
// (cp.async.bulk.tensor, SWIZZLE_128B) on a 2-4 stage mbarrier pipeline.
// Every wait is bounded; on expiry the kernel records an error, lets its
// loads and MMAs finish, and leaves after releasing its tensor memory.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace shdom {
namespace tc {

constexpr int BM = 128, BK = 32;
constexpr int kWaitLimit = 1 << 22;

struct Epilogue {
  int M, N;          // rows (points), logical columns
  int mode;          // 0: C = max(0, acc); 1: radiance (masked by nr), fluxes from A
  float *C;          // mode 0 output, row stride ldc
  int ldc;
  float *R;          // mode 1 radiance [M][nlm]
  int nlm;
  const int *nr;
  float *fluxes;     // mode 1 fluxes [M][2]: FP32 sums of the ordinates (the A columns) with these weights
  const float *fluxw;
  int ncol_down;     // columns below this are downward ordinates
  int *err;
  int split;
  const int *rowmap;  // output point of each A row (A holds a compacted subset of the points), or null
  const uint8_t *stk; // mode 0: Stokes component per output column (only I, 0, is clamped), or null (all I)
  int ldr;            // mode 1: row stride of R (nlm, or 3 nlm for I, Q, U rows); columns are masked by (col mod nlm) < nr
  int wait_limit;     // polls of a pipeline wait before the kernel gives up (kWaitLimit; 0 in the abort-path test)
};

__device__ __forceinline__ uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int limit = kWaitLimit) {
  for (int i = 0; i < limit; ++i) {
    uint32_t ok;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}
__device__ __forceinline__ void tma_load(uint32_t dst, const CUtensorMap *map, uint32_t bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(map), "r"(x), "r"(y), "r"(bar)
      : "memory");
}
// Shared-memory matrix descriptor: K-major operand in the 128-byte swizzle
// layout written by TMA (8-row groups of 128-byte rows, 1024 bytes apart).
__device__ __forceinline__ uint64_t sdesc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;            // leading byte offset (unused for this layout)
  d |= (uint64_t)(1024 >> 4) << 32;  // stride byte offset: next 8-row group
  d |= (uint64_t)1 << 46;            // descriptor version
  d |= (uint64_t)2 << 61;            // 128-byte swizzle
  return d;
}
__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accum) {
  asm volatile("{ .reg .pred p; setp.ne.b32 p, %4, 0; tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p; }" ::"r"(dtmem),
               "l"(a), "l"(b), "r"(idesc), "r"(accum));
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 16 columns of this warp's 32 tensor-memory lanes into registers (async;
// complete after tcgen05.wait::ld).
__device__ __forceinline__ void tmem_ld16(uint32_t ta, uint32_t *r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(ta));
}
// Orders later uses of 16 registers after the preceding volatile asm (the wait).
__device__ __forceinline__ void reg_fence16(uint32_t *r) {
  asm volatile(""
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                 "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15]));
}

// Persistent kernel: CTA i takes the tiles i, i + gridDim.x, ... of the
// (row tile, N tile) grid, N tile fastest, so the N tiles of one row tile
// run at the same time on neighbouring CTAs and A comes from DRAM once.  A
// tile is a 128-row block of A against a BN-column block of B (BN a
// multiple of 32, at most 128 so that the FP32 sums stay in registers).
// The chunks of all the CTA's tiles form one pipeline, so loads for the
// next tile start while the current one is in the tensor cores and its
// results are stored.
//
// Warp roles (448 threads):
//   warp 0 lane 0  TMA producer: A chunk (128 x 32 fp32) and the B hi / lo
//                  chunks (BN x 32) into stage g % S;
//   warp 1 lane 0  MMA issuer: the chunk's 3 (or 1) x BK/8 tcgen05.mma into a
//                  FRESH accumulator (tensor-memory buffer g % 2, BN columns);
//                  warp 1 also owns the tensor-memory allocation;
//   warps 2..5     split: one row of the chunk per thread, into TF32 high (in
//                  place) and low parts (and, for the ordinate-to-harmonic
//                  direction, the row's ordinates into the two hemispheric
//                  flux sums in FP32);
//   warps 6..13    accumulate: read chunk g's partial product from tensor
//                  memory and add it into FP32 registers (each thread: one
//                  row, half of the BN columns); after a tile's last chunk,
//                  store its results (while the tensor cores work on the
//                  next tile).
// Summing the per-chunk partial products on the CUDA cores (round to
// nearest) keeps the tensor-core accumulation chains 32 K-elements long.
template <int BN>
struct Cfg {
  static constexpr int HALF = BN / 2;
  static constexpr int A_BYTES = BM * BK * 4, B_BYTES = BN * BK * 4;
  static constexpr int STAGE = 2 * A_BYTES + 2 * B_BYTES;
  static constexpr int kFluxTab = 16 * 1024;  // down and up flux weights, K padded to 32 (K <= 2048)
  static constexpr int S = (227 * 1024 - 2048 - kFluxTab) / STAGE > 4 ? 4 : (227 * 1024 - 2048 - kFluxTab) / STAGE;
  static constexpr uint32_t TCOLS = 2 * BN <= 256 ? 256u : 512u;
  static constexpr size_t smem() { return (size_t)S * STAGE + 256 + kFluxTab + 1024; }
};
constexpr int kThreads = 448;

// Round to TF32, nearest with ties away from zero (the rounding of
// cvt.rna.tf32.f32), on the integer pipe: add half of the dropped range to
// the magnitude bits and clear the 13 low bits.  Finite inputs.
__device__ __forceinline__ float tf32_rna_bits(float x) {
  return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xffffe000u);
}

template <int BN>
__global__ void __launch_bounds__(kThreads, 1) k_tc_gemm(const __grid_constant__ CUtensorMap tmA,
                                                         const __grid_constant__ CUtensorMap tmBh,
                                                         const __grid_constant__ CUtensorMap tmBl, int K, int ntn,
                                                         int ntiles, Epilogue g) {
  using C = Cfg<BN>;
  constexpr int S = C::S, HALF = C::HALF, A_BYTES = C::A_BYTES, B_BYTES = C::B_BYTES, STAGE = C::STAGE;
  extern __shared__ uint8_t smem_raw[];
  const uint32_t base0 = saddr(smem_raw);
  const uint32_t pad = (1024u - (base0 & 1023u)) & 1023u;
  uint8_t *smem = smem_raw + pad;
  const uint32_t sbase = base0 + pad;
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + S * STAGE);
  // barriers: full[S], split[S], empty[S], accfull[2], accempty[2], fin
  const uint32_t full0 = saddr(&bars[0]), split0 = saddr(&bars[S]), empty0 = saddr(&bars[2 * S]);
  const uint32_t accf0 = saddr(&bars[3 * S]), acce0 = saddr(&bars[3 * S + 2]), fin = saddr(&bars[3 * S + 4]);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(&bars[3 * S + 5]);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(&bars[3 * S + 6]);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int KB = (K + BK - 1) / BK, kpad = KB * BK;
  float *fw = reinterpret_cast<float *>(smem + S * STAGE + 256);  // [2][kpad]: down, up weights
  if (g.mode == 1)
    for (int i = tid; i < kpad; i += blockDim.x) {
      const float w = i < K ? g.fluxw[i] : 0.f;
      fw[i] = i < g.ncol_down ? w : 0.f;
      fw[kpad + i] = i < g.ncol_down ? 0.f : w;
    }
  const int mine = blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  const int G = mine * KB;  // chunks of all this CTA's tiles
  auto tile_origin = [&](int gc, int &m0, int &n0) {
    const int t = (int)blockIdx.x + (gc / KB) * (int)gridDim.x;
    n0 = (t % ntn) * BN;
    m0 = (t / ntn) * BM;
  };

  if (tid == 0) {
    for (int i = 0; i < S; ++i) {
      mbar_init(full0 + 8 * i, 1);
      mbar_init(split0 + 8 * i, 4);
      mbar_init(empty0 + 8 * i, 1);
    }
    mbar_init(accf0, 1); mbar_init(accf0 + 8, 1);
    mbar_init(acce0, 8); mbar_init(acce0 + 8, 8);
    mbar_init(fin, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(tslot)), "r"(C::TCOLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tslot;

  if (warp == 0) {
    // ---------------------------------------------------------- producer
    if (lane == 0) {
      int issued = 0;
      for (int gc = 0; gc < G && !*abort_flag; ++gc) {
        const int s = gc % S;
        if (gc >= S && !mbar_wait(empty0 + 8 * s, ((gc / S) - 1) & 1, g.wait_limit)) { *abort_flag = 1; break; }
        int m0, n0;
        tile_origin(gc, m0, n0);
        const int kx = (gc % KB) * BK;
        const uint32_t st = sbase + s * STAGE;
        mbar_expect_tx(full0 + 8 * s, A_BYTES + 2 * B_BYTES);
        tma_load(st, &tmA, full0 + 8 * s, kx, m0);
        tma_load(st + 2 * A_BYTES, &tmBh, full0 + 8 * s, kx, n0);
        tma_load(st + 2 * A_BYTES + B_BYTES, &tmBl, full0 + 8 * s, kx, n0);
        issued = gc + 1;
      }
      // Every load issued has landed before the shared memory is released:
      // the last S issued stages' phases (already complete unless the
      // consumers gave up before waiting on them).  Unconditional, since
      // a consumer may give up after this thread left its loop; the full
      // limit here, whatever the pipeline's.
      for (int gc = issued > S ? issued - S : 0; gc < issued; ++gc)
        mbar_wait(full0 + 8 * (gc % S), (gc / S) & 1, kWaitLimit);
    }
  } else if (warp == 1) {
    // ---------------------------------------------------------- MMA issuer
    if (lane == 0) {
      const uint32_t idesc =
          (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
      for (int gc = 0; gc < G; ++gc) {
        const int s = gc % S, b = gc & 1;
        if (*abort_flag) break;
        if (!mbar_wait(split0 + 8 * s, (gc / S) & 1, g.wait_limit)) { *abort_flag = 1; break; }
        if (gc >= 2 && !mbar_wait(acce0 + 8 * b, ((gc >> 1) - 1) & 1, g.wait_limit)) { *abort_flag = 1; break; }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t st = sbase + s * STAGE, dt = tmem + (uint32_t)(b * BN);
#pragma unroll
        for (int ks = 0; ks < BK / 8; ++ks) {
          const uint32_t off = ks * 32;  // 8 tf32 elements
          const uint64_t dah = sdesc(st + off), dal = sdesc(st + A_BYTES + off);
          const uint64_t dbh = sdesc(st + 2 * A_BYTES + off), dbl = sdesc(st + 2 * A_BYTES + B_BYTES + off);
          if (g.split) {
            // small terms first, while the fresh accumulator is small
            mma_tf32(dt, dal, dbh, idesc, ks > 0 ? 1u : 0u);
            mma_tf32(dt, dah, dbl, idesc, 1u);
            mma_tf32(dt, dah, dbh, idesc, 1u);
          } else {
            mma_tf32(dt, dah, dbh, idesc, ks > 0 ? 1u : 0u);
          }
        }
        mma_commit(empty0 + 8 * s);
        mma_commit(accf0 + 8 * b);
      }
      // every MMA issued has finished before tensor memory is released (the
      // full limit here, whatever the pipeline's)
      mma_commit(fin);
      mbar_wait(fin, 0, kWaitLimit);
    }
  } else if (warp < 6) {
    // ---------------------------------------------------------- split
    const int srow = tid - 64;  // 0..127
    const int swz = srow & 7;
    float fd = 0.f, fu = 0.f;
    bool flux = false;
    if (G > 0) {
      int m0, n0;
      tile_origin(0, m0, n0);
      flux = g.mode == 1 && n0 == 0;
    }
    for (int gc = 0; gc < G; ++gc) {
      const int s = gc % S, c = gc % KB;
      const bool go = !*abort_flag && mbar_wait(full0 + 8 * s, (gc / S) & 1, g.wait_limit);
      if (!__all_sync(0xffffffffu, go)) { *abort_flag = 1; break; }
      uint8_t *arow = smem + s * STAGE + (srow >> 3) * 1024 + swz * 128;
      float4 v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) v[u] = *reinterpret_cast<const float4 *>(arow + ((u ^ swz) << 4));
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        // u is the logical 16-byte unit of the row; (u ^ swz) its place in the 128-byte swizzle row
        float4 h, l;
        h.x = tf32_rna_bits(v[u].x); l.x = tf32_rna_bits(v[u].x - h.x);
        h.y = tf32_rna_bits(v[u].y); l.y = tf32_rna_bits(v[u].y - h.y);
        h.z = tf32_rna_bits(v[u].z); l.z = tf32_rna_bits(v[u].z - h.z);
        h.w = tf32_rna_bits(v[u].w); l.w = tf32_rna_bits(v[u].w - h.w);
        *reinterpret_cast<float4 *>(arow + ((u ^ swz) << 4)) = h;
        *reinterpret_cast<float4 *>(arow + A_BYTES + ((u ^ swz) << 4)) = l;
      }
      if (flux) {
        // down / up weights of the chunk's 32 ordinates (zero past K): broadcast reads
        const float4 *wd = reinterpret_cast<const float4 *>(fw + c * BK);
        const float4 *wu = reinterpret_cast<const float4 *>(fw + kpad + c * BK);
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const float4 a = wd[u], b = wu[u];
          fd = fmaf(a.x, v[u].x, fd); fd = fmaf(a.y, v[u].y, fd); fd = fmaf(a.z, v[u].z, fd); fd = fmaf(a.w, v[u].w, fd);
          fu = fmaf(b.x, v[u].x, fu); fu = fmaf(b.y, v[u].y, fu); fu = fmaf(b.z, v[u].z, fu); fu = fmaf(b.w, v[u].w, fu);
        }
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(split0 + 8 * s) : "memory");
      if (flux && c == KB - 1) {
        // the tile's fluxes are complete once its last chunk is split
        int m0, n0;
        tile_origin(gc, m0, n0);
        const int frow = m0 + srow;
        if (frow < g.M) {
          const size_t fp = g.rowmap ? (size_t)g.rowmap[frow] : (size_t)frow;
          g.fluxes[2 * fp] = fd;
          g.fluxes[2 * fp + 1] = fu;
        }
        fd = 0.f; fu = 0.f;
      }
      if (c == KB - 1 && gc + 1 < G) {
        int m0, n0;
        tile_origin(gc + 1, m0, n0);
        flux = g.mode == 1 && n0 == 0;  // one N tile of a row tile forms its fluxes
      }
    }
  } else {
    // ---------------------------------------------------------- accumulate
    const int lg = warp & 3, half = (warp - 6) >> 2;
    float acc[HALF];
#pragma unroll
    for (int j = 0; j < HALF; ++j) acc[j] = 0.f;
    for (int gc = 0; gc < G; ++gc) {
      const int b = gc & 1;
      const bool go = !*abort_flag && mbar_wait(accf0 + 8 * b, (gc >> 1) & 1, g.wait_limit);
      if (!__all_sync(0xffffffffu, go)) { *abort_flag = 1; break; }
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t ta = tmem + ((uint32_t)(lg * 32) << 16) + (uint32_t)(b * BN + half * HALF);
      // two loads in flight per wait
#pragma unroll
      for (int c0 = 0; c0 < HALF; c0 += 32) {
        uint32_t r[32];
        tmem_ld16(ta + (uint32_t)c0, r);
        if (c0 + 16 < HALF) tmem_ld16(ta + (uint32_t)(c0 + 16), r + 16);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        reg_fence16(r);
        if (c0 + 16 < HALF) reg_fence16(r + 16);
#pragma unroll
        for (int j = 0; j < 32; ++j)
          if (c0 + j < HALF) acc[c0 + j] += __uint_as_float(r[j]);
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(acce0 + 8 * b) : "memory");
      if (gc % KB == KB - 1) {
        int m0, n0;
        tile_origin(gc, m0, n0);
        const int arow = m0 + lg * 32 + lane;
        if (arow < g.M) {
          const int row = g.rowmap ? g.rowmap[arow] : arow;
          const int cb = n0 + half * HALF;
          if (g.mode == 0) {
            float *out = g.C + (size_t)row * g.ldc;
#pragma unroll
            for (int j = 0; j < HALF; j += 4) {
              const int col = cb + j;
              float4 v = make_float4(fmaxf(acc[j], 0.f), fmaxf(acc[j + 1], 0.f), fmaxf(acc[j + 2], 0.f),
                                     fmaxf(acc[j + 3], 0.f));
              if (g.stk) {  // polarized: the Q and U ordinate sources keep their sign
                if (col < g.N && g.stk[col]) v.x = acc[j];
                if (col + 1 < g.N && g.stk[col + 1]) v.y = acc[j + 1];
                if (col + 2 < g.N && g.stk[col + 2]) v.z = acc[j + 2];
                if (col + 3 < g.N && g.stk[col + 3]) v.w = acc[j + 3];
              }
              if (col + 3 < g.N) {
                *reinterpret_cast<float4 *>(out + col) = v;  // col and ldc are multiples of 4
              } else {
                if (col < g.N) out[col] = v.x;
                if (col + 1 < g.N) out[col + 1] = v.y;
                if (col + 2 < g.N) out[col + 2] = v.z;
              }
            }
          } else {
            const int nrp = g.nr[row];
            float *out = g.R + (size_t)row * (g.ldr ? g.ldr : g.nlm);
#pragma unroll
            for (int j = 0; j < HALF; ++j) {
              const int col = cb + j;
              const int jt = col < g.nlm ? col : col % g.nlm;
              if (col < g.N) out[col] = (jt < nrp) ? acc[j] : 0.f;
            }
          }
        }
#pragma unroll
        for (int j = 0; j < HALF; ++j) acc[j] = 0.f;
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (*abort_flag && tid == 0) atomicCAS(g.err, 0, 6);
  if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(C::TCOLS));
}

template <int BN>
inline size_t smem_bytes() { return Cfg<BN>::smem(); }

}  // namespace tc
}  // namespace shdom
