// 5th-generation tensor cores (tcgen05) for the trailing update of the FP32
// Newton-matrix LU: A22 -= L21 * U12 with K = 32 (one LU panel).
//
// The product runs as 3xTF32: each FP32 operand x is split into a TF32 head
// h = rna_tf32(x) and a tail l = x - h (exact in FP32), and
// L21*U12 ~= Lh*Uh + Lh*Ul + Ll*Uh, accumulated in FP32 in tensor memory
// (TMEM).  The dropped Ll*Ul term and the truncation of the tails are
// ~2^-21 relative, the level of FP32 arithmetic, so the factors keep the
// accuracy of the CUDA-core FP32 update.
//
// Per 128-row tile of L21: the threads stage the split tile in shared
// memory, one thread issues the tcgen05.mma instructions (M = 128, N <= 256
// per instruction, K = 8 each), a tcgen05.commit arrives on an mbarrier,
// and every warp reads its 32 TMEM lanes back (tcgen05.ld) and subtracts the
// product from A22 in global memory.  Operands use the K-major layout
// without swizzle: 8-row x 16-byte core matrices, element (r, k) at byte
//   (r / 8) * 1024 + (k / 4) * 128 + (r % 8) * 16 + (k % 4) * 4
// (LBO = 128 B between K-adjacent core matrices, SBO = 1024 B between
// 8-row groups), so each K = 8 step advances the descriptors by 256 B.
#pragma once
#include "ucl_common.cuh"

namespace ucl {

constexpr int TC_TMEM_COLS = 512;       // most accumulator columns a CTA allocates
constexpr int TC_M = 128;               // rows per tcgen05.mma
constexpr unsigned TC_WAIT_LIMIT = 1u << 22;  // bounded mbarrier polling

// Tensor-core state of one CTA (shared memory).
struct TcState {
  unsigned long long mbar;  // MMA-completion mbarrier
  unsigned tmem;            // TMEM base address from tcgen05.alloc
  unsigned phase;           // parity of the next mbarrier phase to wait for
  int err;                  // set when a bounded wait gave up
  unsigned cols;            // TMEM columns held (a power of two, 32..512)
};

// TMEM columns the trailing updates of an n x n FP32 factorisation need:
// the widest update is the first one, n - 32 columns padded to 16, and the
// allocation is a power of two of at least 32.  Sizing it to n lets more
// than one CTA hold TMEM on an SM where shared memory allows it.
__host__ __device__ constexpr unsigned tc_cols_for(int n) {
  return ((n - 32 + 15) & ~15) <= 32 ? 32u : ((n - 32 + 15) & ~15) <= 64 ? 64u
       : ((n - 32 + 15) & ~15) <= 128 ? 128u : ((n - 32 + 15) & ~15) <= 256 ? 256u : 512u;
}

__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

// warp-collective: allocate `cols` columns, address to *dst
__device__ __forceinline__ void tc_alloc(unsigned* dst, unsigned cols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst)),
               "r"(cols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
// warp-collective
__device__ __forceinline__ void tc_dealloc(unsigned taddr, unsigned cols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols)
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// make this thread's generic-proxy shared-memory writes visible to the
// tensor core (async proxy)
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_init(unsigned long long* mbar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(mbar)), "r"(count) : "memory");
}
// wait for the phase with the given parity; false if the limit ran out
__device__ __forceinline__ bool mbar_wait(unsigned long long* mbar, unsigned parity) {
  const unsigned a = smem_addr(mbar);
  for (unsigned it = 0; it < TC_WAIT_LIMIT; ++it) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// shared-memory matrix descriptor: K-major, no swizzle (sm_100 family format:
// start >> 4 in bits 0-13, LBO >> 4 in 16-29, SBO >> 4 in 32-45, version 1
// in bits 46-47, layout type 0)
__device__ __forceinline__ unsigned long long tc_desc(unsigned saddr, unsigned lbo, unsigned sbo) {
  return (unsigned long long)((saddr >> 4) & 0x3FFFu) | ((unsigned long long)((lbo >> 4) & 0x3FFFu) << 16) |
         ((unsigned long long)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// instruction descriptor, kind::tf32: D f32 (bits 4-5 = 1), A and B tf32
// (bits 7-9, 10-12 = 2), both K-major, N >> 3 in bits 17-22, M >> 4 in 24-28
__device__ __forceinline__ unsigned tc_idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((unsigned)(N >> 3) << 17) | ((unsigned)(M >> 4) << 24);
}
__device__ __forceinline__ void tc_mma_tf32(unsigned dtmem, unsigned long long adesc, unsigned long long bdesc,
                                            unsigned idesc, unsigned accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// arrive on the mbarrier once all previously issued MMAs of this thread end
__device__ __forceinline__ void tc_commit(unsigned long long* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_addr(mbar))
               : "memory");
}
// 32 lanes x 8 consecutive columns of TMEM -> 8 registers per thread
// (issue only; the values are valid after tc_ld_wait)
__device__ __forceinline__ void tc_ld8(unsigned taddr, unsigned* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
      : "r"(taddr)
      : "memory");
}
__device__ __forceinline__ void tc_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// CTA prologue / epilogue of kernels that use the tensor cores: TMEM
// allocation by warp 0, mbarrier set-up by thread 0.  All threads call.
__device__ __forceinline__ void tc_setup(TcState* tc, unsigned cols = TC_TMEM_COLS) {
  if ((threadIdx.x >> 5) == 0) tc_alloc(&tc->tmem, cols);
  if (threadIdx.x == 0) {
    tc->cols = cols;
    mbar_init(&tc->mbar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    tc->phase = 0;
    tc->err = 0;
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
}
__device__ __forceinline__ void tc_teardown(TcState* tc) {
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if ((threadIdx.x >> 5) == 0) tc_dealloc(tc->tmem, tc->cols);
}

// TF32 head (round to nearest, ties away) of x, as an FP32 value
__device__ __forceinline__ float tf32_head(float x) {
  unsigned r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// byte offset of element (r, k), 0 <= k < 32, in a K-major no-swizzle tile
__device__ __forceinline__ unsigned tc_off(int r, int k) {
  return (unsigned)((r >> 3) * 1024 + (k >> 2) * 128 + (r & 7) * 16 + (k & 3) * 4);
}

// store 4 consecutive K values (k0 % 4 == 0) of row r, split into head and
// tail tiles
__device__ __forceinline__ void tc_put4(char* head, char* tail, int r, int k0, float a, float b, float c, float d) {
  const float4 h = make_float4(tf32_head(a), tf32_head(b), tf32_head(c), tf32_head(d));
  const float4 l = make_float4(a - h.x, b - h.y, c - h.z, d - h.w);
  const unsigned o = tc_off(r, k0);
  *reinterpret_cast<float4*>(head + o) = h;
  *reinterpret_cast<float4*>(tail + o) = l;
}

// Shared-memory bytes of the staging: A tile (128 rows) and B (np rows),
// head and tail each.
__host__ __device__ constexpr size_t tc_stage_bytes(int np) {
  return (size_t)2 * TC_M * 128 + (size_t)2 * np * 128;
}

// A22 -= L21 * U12 on the tensor cores.
//   A       row-major n x n (global); A22 starts at (r0g, c0g)
//   R, nc   rows and columns of A22
//   lsrc    L21 in shared memory, row i at lsrc + i * ldl (32 values)
//   bh, bl  U12 already staged as B (np rows = nc rounded up to 16, zero
//           padded), head and tail
//   ah, al  staging for one 128-row tile of L21
// All threads call this; returns false if a bounded wait gave up.
__device__ bool tc_trailing_update(float* __restrict__ A, int n, int r0g, int c0g, int R, int nc,
                                   const float* lsrc, int ldl, char* ah, char* al, const char* bh, const char* bl,
                                   TcState* tc) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int np = (nc + 15) & ~15;
  bool ok = true;
  for (int m0 = 0; m0 < R; m0 += TC_M) {
    // stage the split 128 x 32 tile of L21 (rows past R are zero)
    for (int t = tid; t < TC_M * 8; t += NT) {
      const int r = t >> 3, k4 = (t & 7) * 4;
      const int gr = m0 + r;
      float a = 0.f, b = 0.f, c = 0.f, d = 0.f;
      if (gr < R) {
        const float* s = lsrc + (size_t)gr * ldl + k4;
        a = s[0]; b = s[1]; c = s[2]; d = s[3];
      }
      tc_put4(ah, al, r, k4, a, b, c, d);
    }
    fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      const unsigned a_h = smem_addr(ah), a_l = smem_addr(al), b_h = smem_addr(bh), b_l = smem_addr(bl);
      for (int c0 = 0; c0 < np; c0 += 256) {
        const int N = min(256, np - c0);
        const unsigned idesc = tc_idesc_tf32(TC_M, N);
        const unsigned boff = (unsigned)(c0 / 8) * 1024u;
        const unsigned d = tc->tmem + (unsigned)c0;
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
          const unsigned ko = (unsigned)kk * 256u;
          tc_mma_tf32(d, tc_desc(a_h + ko, 128, 1024), tc_desc(b_h + boff + ko, 128, 1024), idesc, kk > 0);
          tc_mma_tf32(d, tc_desc(a_h + ko, 128, 1024), tc_desc(b_l + boff + ko, 128, 1024), idesc, 1);
          tc_mma_tf32(d, tc_desc(a_l + ko, 128, 1024), tc_desc(b_h + boff + ko, 128, 1024), idesc, 1);
        }
      }
      tc_commit(&tc->mbar);
    }
    // epilogue: warp w reads TMEM lanes 32*(w%4).. (its sub-partition),
    // columns of half w/4, and updates its row of A22 in chunks of 32
    // columns; the row segment of each chunk is loaded before it is needed
    // (the first one while the MMAs run)
    const int q = warp & 3, half = warp >> 2;
    const int cw = np / 2;  // multiple of 8
    const int row = m0 + q * 32 + lane;
    const bool live = row < R;
    const bool vec = ((n & 3) == 0) && ((c0g & 3) == 0);
    float* dst = A + (size_t)(r0g + (live ? row : 0)) * n + c0g;
    const int cbeg = half * cw, cend = (half + 1) * cw;
    float cv[32];
    auto load_chunk = [&](int c) {
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int cc = c + 4 * u;
        if (live && cc < cend && cc + 4 <= nc && vec) {
          const float4 x = *reinterpret_cast<const float4*>(dst + cc);
          cv[4 * u] = x.x; cv[4 * u + 1] = x.y; cv[4 * u + 2] = x.z; cv[4 * u + 3] = x.w;
        } else {
#pragma unroll
          for (int i = 0; i < 4; ++i) cv[4 * u + i] = (live && cc < cend && cc + i < nc) ? dst[cc + i] : 0.f;
        }
      }
    };
    load_chunk(cbeg);
    const bool done = mbar_wait(&tc->mbar, tc->phase);
    tc_fence_after();
    if (!done) {
      // give the MMAs in flight one more bounded wait before TMEM is reused
      mbar_wait(&tc->mbar, tc->phase);
      ok = false;
      if (tid == 0) tc->err = 1;
    } else {
      for (int c = cbeg; c < cend; c += 32) {
        unsigned d[32];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          if (c + 8 * u < cend) tc_ld8(tc->tmem + ((unsigned)(q * 32) << 16) + (unsigned)(c + 8 * u), d + 8 * u);
          else {
#pragma unroll
            for (int i = 0; i < 8; ++i) d[8 * u + i] = 0u;
          }
        }
        tc_ld_wait();
        float out[32];
#pragma unroll
        for (int i = 0; i < 32; ++i) out[i] = cv[i] - __uint_as_float(d[i]);
        if (c + 32 < cend) load_chunk(c + 32);
        if (live) {
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const int cc = c + 4 * u;
            if (cc < cend && cc + 4 <= nc && vec) {
              *reinterpret_cast<float4*>(dst + cc) =
                  make_float4(out[4 * u], out[4 * u + 1], out[4 * u + 2], out[4 * u + 3]);
            } else {
#pragma unroll
              for (int i = 0; i < 4; ++i)
                if (cc < cend && cc + i < nc) dst[cc + i] = out[4 * u + i];
            }
          }
        }
      }
    }
    tc_fence_before();
    __syncthreads();
    if (tid == 0) tc->phase ^= 1u;
    __syncthreads();
    if (!ok) break;
  }
  return ok;
}

}  // namespace ucl
