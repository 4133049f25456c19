// shdom_tc.cuh -- tensor-core (tcgen05) dense transform GEMM for sm_103a.
//
// The spherical-harmonic <-> discrete-ordinate transforms are linear maps
// with a fixed coefficient matrix: C[p][n] = sum_k A[p][k] B[n][k], where A
// is the per-point field (SOURCE [npts][nlm] or the ordinate radiances
// [npts][nang]) and B the masked transform matrix stored [N][K] (K-major).
// FP32 accuracy is kept with the three-product split of TF32 operands:
// A = Ah + Al, B = Bh + Bl (Ah, Bh rounded to TF32), C ~= Ah Bh + Ah Bl + Al Bh
// accumulated in FP32 in tensor memory.  With split = 0 only Ah Bh is formed
// (the reduced-precision variant).
//
// Per CTA: one 128-row tile of A, one BN-column tile of B; 128 threads.
// Stages of 32 K-elements (one 128-byte swizzle row) are brought in by TMA
// (cp.async.bulk.tensor, SWIZZLE_128B) on a two-stage mbarrier pipeline;
// all threads split A into hi/lo in shared memory; thread 0 issues the
// tcgen05.mma instructions (M=128, N=BN, K=8) and commits to mbarriers; the
// four warps read their 32 TMEM lanes with tcgen05.ld for the epilogue.
// Every wait is bounded; on expiry the kernel records an error and leaves
// after releasing its tensor memory.
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
  int mode;          // 0: C = max(0, acc); 1: radiance (masked by nr) + fluxes
  float *C;          // mode 0 output, row stride ldc
  int ldc;
  float *R;          // mode 1 radiance [M][nlm]
  int nlm;
  const int *nr;
  float *fluxes;     // mode 1 fluxes [M][2] (columns nlm, nlm+1)
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

// BN (the N tile, a multiple of 16 in [16, 256]) is a launch argument; the
// dynamic shared memory must hold smem_bytes(BN).
__global__ void __launch_bounds__(128, 1) k_tc_gemm(const __grid_constant__ CUtensorMap tmA,
                                                    const __grid_constant__ CUtensorMap tmBh,
                                                    const __grid_constant__ CUtensorMap tmBl, int K, int BN,
                                                    Epilogue g) {
  const int A_BYTES = BM * BK * 4, B_BYTES = BN * BK * 4;
  const int STAGE = 2 * A_BYTES + 2 * B_BYTES;
  extern __shared__ uint8_t smem_raw[];
  const uint32_t base0 = saddr(smem_raw);
  const uint32_t pad = (1024u - (base0 & 1023u)) & 1023u;
  uint8_t *smem = smem_raw + pad;
  const uint32_t sbase = base0 + pad;
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + 2 * STAGE);
  const uint32_t full0 = saddr(&bars[0]), empty0 = saddr(&bars[2]), accbar = saddr(&bars[4]);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(&bars[5]);
  int *abort_flag = reinterpret_cast<int *>(&bars[6]);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int KB = (K + BK - 1) / BK;

  if (tid == 0) {
    mbar_init(full0, 1); mbar_init(full0 + 8, 1);
    mbar_init(empty0, 1); mbar_init(empty0 + 8, 1);
    mbar_init(accbar, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(tslot)), "r"(256));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tslot;
  // instruction descriptor: D f32, A/B tf32, K-major both, N = BN, M = 128
  const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);

  auto issue = [&](int kb) {
    const int s = kb & 1;
    const uint32_t st = sbase + s * STAGE;
    mbar_expect_tx(full0 + 8 * s, A_BYTES + 2 * B_BYTES);
    tma_load(st, &tmA, full0 + 8 * s, kb * BK, m0);
    tma_load(st + 2 * A_BYTES, &tmBh, full0 + 8 * s, kb * BK, n0);
    tma_load(st + 2 * A_BYTES + B_BYTES, &tmBl, full0 + 8 * s, kb * BK, n0);
  };
  int issued = 0;  // loads issued by thread 0 (only thread 0 reads it)
  if (tid == 0) {
    issue(0);
    issued = 1;
    if (KB > 1) { issue(1); issued = 2; }
  }
  for (int kb = 0; kb < KB; ++kb) {
    const int s = kb & 1;
    const uint32_t par = (kb >> 1) & 1;
    if (!mbar_wait(full0 + 8 * s, par)) *abort_flag = 1;
    __syncthreads();
    if (*abort_flag) break;
    // split the fp32 A tile into TF32 high part (in place) and remainder
    float4 *ah = reinterpret_cast<float4 *>(smem + s * STAGE);
    float4 *al = reinterpret_cast<float4 *>(smem + s * STAGE + A_BYTES);
#pragma unroll 4
    for (int i = tid; i < A_BYTES / 16; i += 128) {
      float4 v = ah[i], h, l;
      uint32_t t;
      asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(v.x)); h.x = __uint_as_float(t); l.x = v.x - h.x;
      asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(v.y)); h.y = __uint_as_float(t); l.y = v.y - h.y;
      asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(v.z)); h.z = __uint_as_float(t); l.z = v.z - h.z;
      asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(v.w)); h.w = __uint_as_float(t); l.w = v.w - h.w;
      ah[i] = h;
      al[i] = l;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t st = sbase + s * STAGE;
#pragma unroll
      for (int ks = 0; ks < BK / 8; ++ks) {
        const uint32_t off = ks * 32;  // 8 tf32 elements
        const uint64_t dah = sdesc(st + off), dal = sdesc(st + A_BYTES + off);
        const uint64_t dbh = sdesc(st + 2 * A_BYTES + off), dbl = sdesc(st + 2 * A_BYTES + B_BYTES + off);
        mma_tf32(tmem, dah, dbh, idesc, (kb > 0 || ks > 0) ? 1u : 0u);
        if (g.split) {
          mma_tf32(tmem, dah, dbl, idesc, 1u);
          mma_tf32(tmem, dal, dbh, idesc, 1u);
        }
      }
      mma_commit(empty0 + 8 * s);
      if (kb + 2 < KB) {
        if (!mbar_wait(empty0 + 8 * s, par)) *abort_flag = 1;
        else { issue(kb + 2); issued = kb + 3; }
      }
    }
  }
  if (tid == 0) {
    mma_commit(accbar);
    if (*abort_flag) {
      // let every load still in flight land before the shared memory is released
      // (only the last load of each stage can be outstanding)
      for (int kb = issued > 2 ? issued - 2 : 0; kb < issued; ++kb) mbar_wait(full0 + 8 * (kb & 1), (kb >> 1) & 1);
    }
  }
  bool ok = mbar_wait(accbar, 0);
  __syncthreads();
  if (!ok || *abort_flag) {
    if (tid == 0) atomicCAS(g.err, 0, 6);
  } else {
    asm volatile("tcgen05.fence::after_thread_sync;");
    const int row = m0 + warp * 32 + lane;
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 16) {
      uint32_t r[16];
      const uint32_t ta = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
            "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(ta));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (row < g.M) {
        if (g.mode == 0) {
          float *out = g.C + (size_t)row * g.ldc;
#pragma unroll
          for (int j = 0; j < 16; j += 4) {
            const int col = n0 + c0 + j;
            const float4 v = make_float4(fmaxf(__uint_as_float(r[j]), 0.f), fmaxf(__uint_as_float(r[j + 1]), 0.f),
                                         fmaxf(__uint_as_float(r[j + 2]), 0.f), fmaxf(__uint_as_float(r[j + 3]), 0.f));
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
          for (int j = 0; j < 16; ++j) {
            const int col = n0 + c0 + j;
            const float v = __uint_as_float(r[j]);
            if (col < g.nlm) out[col] = (col < nrp) ? v : 0.f;
            else if (col < g.nlm + 2) g.fluxes[2 * (size_t)row + (col - g.nlm)] = v;
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(256));
}

inline size_t smem_bytes(int BN) { return (size_t)2 * (2 * BM * BK * 4 + 2 * BN * BK * 4) + 64 + 1024; }

}  // namespace tc
}  // namespace shdom
