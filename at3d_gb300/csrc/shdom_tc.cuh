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
};

__device__ __forceinline__ uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (int i = 0; i < kWaitLimit; ++i) {
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

// One CTA: a 128-row tile of A against a BN-column tile of B (BN a multiple
// of 32, at most 256).  The N tiles of one row tile are adjacent in launch
// order (blockIdx.x), so they run together and A comes from DRAM once.
//
// Warp roles (320 threads):
//   warp 0 lane 0  TMA producer: A chunk (128 x 32 fp32) and the B hi / lo
//                  chunks (BN x 32) into stage c % S;
//   warp 1 lane 0  MMA issuer: the chunk's 3 (or 1) x BK/8 tcgen05.mma into a
//                  FRESH accumulator (TMEM buffer c % 2, BN columns each);
//                  warp 1 also owns the tensor-memory allocation;
//   warps 2..9     split and accumulate: split chunk c of A into TF32 high
//                  (in place) and low parts (and, for the ordinate-to-
//                  harmonic direction, add its ordinates into the two
//                  hemispheric flux sums in FP32), then read chunk c-1's
//                  partial product from tensor memory and add it into FP32
//                  registers (each thread: one row, half of the BN columns).
// Summing the per-chunk partial products on the CUDA cores (round to
// nearest) keeps the tensor-core accumulation chains 32 K-elements long.
template <int BN>
struct Cfg {
  static constexpr int HALF = BN / 2;
  static constexpr int A_BYTES = BM * BK * 4, B_BYTES = BN * BK * 4;
  static constexpr int STAGE = 2 * A_BYTES + 2 * B_BYTES;
  static constexpr int S = (227 * 1024 - 2048) / STAGE > 4 ? 4 : (227 * 1024 - 2048) / STAGE;
  static constexpr uint32_t TCOLS = 2 * BN <= 256 ? 256u : 512u;
  static constexpr size_t smem() { return (size_t)S * STAGE + 256 + 1024; }
};
constexpr int kThreads = 320;

template <int BN>
__global__ void __launch_bounds__(kThreads, 1) k_tc_gemm(const __grid_constant__ CUtensorMap tmA,
                                                         const __grid_constant__ CUtensorMap tmBh,
                                                         const __grid_constant__ CUtensorMap tmBl, int K,
                                                         Epilogue g) {
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
  const int n0 = blockIdx.x * BN, m0 = blockIdx.y * BM;
  const int KB = (K + BK - 1) / BK;

  if (tid == 0) {
    for (int i = 0; i < S; ++i) {
      mbar_init(full0 + 8 * i, 1);
      mbar_init(split0 + 8 * i, 8);
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
      for (int c = 0; c < KB && !*abort_flag; ++c) {
        const int s = c % S;
        if (c >= S && !mbar_wait(empty0 + 8 * s, ((c / S) - 1) & 1)) { *abort_flag = 1; break; }
        const uint32_t st = sbase + s * STAGE;
        mbar_expect_tx(full0 + 8 * s, A_BYTES + 2 * B_BYTES);
        tma_load(st, &tmA, full0 + 8 * s, c * BK, m0);
        tma_load(st + 2 * A_BYTES, &tmBh, full0 + 8 * s, c * BK, n0);
        tma_load(st + 2 * A_BYTES + B_BYTES, &tmBl, full0 + 8 * s, c * BK, n0);
        issued = c + 1;
      }
      if (*abort_flag) {
        // let the loads still in flight land before the shared memory is released
        for (int c = issued > S ? issued - S : 0; c < issued; ++c) mbar_wait(full0 + 8 * (c % S), (c / S) & 1);
      }
    }
  } else if (warp == 1) {
    // ---------------------------------------------------------- MMA issuer
    if (lane == 0) {
      const uint32_t idesc =
          (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
      for (int c = 0; c < KB; ++c) {
        const int s = c % S, b = c & 1;
        if (*abort_flag) break;
        if (!mbar_wait(split0 + 8 * s, (c / S) & 1)) { *abort_flag = 1; break; }
        if (c >= 2 && !mbar_wait(acce0 + 8 * b, ((c >> 1) - 1) & 1)) { *abort_flag = 1; break; }
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
      // every MMA issued has finished before tensor memory is released
      mma_commit(fin);
      mbar_wait(fin, 0);
    }
  } else {
    // ---------------------------------------------------------- split + accumulate
    const int e = tid - 64;                 // 0..255
    const int srow = e >> 1, sh = e & 1;    // split: row of the tile, half of its 32 elements
    const int lg = warp & 3, half = (warp - 2) >> 2;
    const int row = m0 + lg * 32 + lane;    // accumulate: this thread's TMEM lane
    float acc[HALF];
#pragma unroll
    for (int j = 0; j < HALF; ++j) acc[j] = 0.f;
    float fd = 0.f, fu = 0.f;
    auto consume = [&](int c) -> bool {
      const int b = c & 1;
      if (!__all_sync(0xffffffffu, mbar_wait(accf0 + 8 * b, (c >> 1) & 1))) return false;
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t ta = tmem + ((uint32_t)(lg * 32) << 16) + (uint32_t)(b * BN + half * HALF);
#pragma unroll
      for (int c0 = 0; c0 < HALF; c0 += 16) {
        uint32_t r[16];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
            : "r"(ta + (uint32_t)c0));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int j = 0; j < 16; ++j) acc[c0 + j] += __uint_as_float(r[j]);
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(acce0 + 8 * b) : "memory");
      return true;
    };
    bool ok = true;
    for (int c = 0; c < KB; ++c) {
      const int s = c % S;
      const bool go = !*abort_flag && mbar_wait(full0 + 8 * s, (c / S) & 1);
      if (!__all_sync(0xffffffffu, go)) { ok = false; break; }
      uint8_t *arow = smem + s * STAGE + (srow >> 3) * 1024 + (srow & 7) * 128;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int j = sh * 4 + u;                       // logical 16-byte unit of the row
        const int off = ((j ^ (srow & 7)) << 4);        // its place in the 128-byte swizzle row
        float4 v = *reinterpret_cast<float4 *>(arow + off), h, l;
        uint32_t t;
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(v.x)); h.x = __uint_as_float(t);
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(v.y)); h.y = __uint_as_float(t);
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(v.z)); h.z = __uint_as_float(t);
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(v.w)); h.w = __uint_as_float(t);
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(v.x - h.x)); l.x = __uint_as_float(t);
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(v.y - h.y)); l.y = __uint_as_float(t);
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(v.z - h.z)); l.z = __uint_as_float(t);
        asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(v.w - h.w)); l.w = __uint_as_float(t);
        *reinterpret_cast<float4 *>(arow + off) = h;
        *reinterpret_cast<float4 *>(arow + A_BYTES + off) = l;
        if (g.mode == 1) {
          const int col = c * BK + j * 4;
          const float vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int cc = col + q;
            if (cc < K) {
              const float w = __ldg(&g.fluxw[cc]) * vv[q];
              if (cc < g.ncol_down) fd += w; else fu += w;
            }
          }
        }
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(split0 + 8 * s) : "memory");
      if (c >= 1 && !consume(c - 1)) { ok = false; break; }
    }
    if (ok && KB > 0) ok = consume(KB - 1);
    if (!ok) {
      *abort_flag = 1;
    } else {
      if (g.mode == 1) {
        fd += __shfl_xor_sync(0xffffffffu, fd, 1);
        fu += __shfl_xor_sync(0xffffffffu, fu, 1);
        const int frow = m0 + srow;
        if (sh == 0 && n0 == 0 && frow < g.M) {
          g.fluxes[2 * (size_t)frow] = fd;
          g.fluxes[2 * (size_t)frow + 1] = fu;
        }
      }
      if (row < g.M) {
        const int cb = n0 + half * HALF;
        if (g.mode == 0) {
          float *out = g.C + (size_t)row * g.ldc;
#pragma unroll
          for (int j = 0; j < HALF; j += 4) {
            const int col = cb + j;
            const float4 v = make_float4(fmaxf(acc[j], 0.f), fmaxf(acc[j + 1], 0.f), fmaxf(acc[j + 2], 0.f),
                                         fmaxf(acc[j + 3], 0.f));
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
          float *out = g.R + (size_t)row * g.nlm;
#pragma unroll
          for (int j = 0; j < HALF; ++j) {
            const int col = cb + j;
            if (col < g.nlm) out[col] = (col < nrp) ? acc[j] : 0.f;
          }
        }
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
