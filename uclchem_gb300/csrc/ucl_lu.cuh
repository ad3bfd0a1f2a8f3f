// Dense LU with partial pivoting and triangular solves for one system per
// CTA (the Newton matrix P = I - h*gamma*J of the BDF corrector; the
// reference factors it with LINPACK DGEFA/DGESL, dvode.f90:11982-12160).
//
// Storage is row-major (P[i*n + j]) so that row interchanges, panel loads and
// the register-tiled trailing update are all coalesced.  The blocked
// right-looking algorithm:
//   for each panel of NB columns:
//     factor the (n-k0) x NB panel in registers (one barrier per column:
//     warp max-reductions of |v|, candidates exchanged in shared memory);
//     apply the panel's interchanges to the columns outside it;
//     U12 = L11^-1 A12 (one thread per column, registers);
//     A22 -= L21 * U12 (register tiles of TM x TN, operands in shared memory).
// The composite row permutation is kept as perm[] so a solve gathers the
// right-hand side in one parallel pass; the inverses of the 32 x 32 diagonal
// blocks of L turn each forward block step into a small GEMV, and compact
// copies of the diagonal blocks of U are solved from registers.
#pragma once
#include "ucl_common.cuh"
#include "ucl_tc.cuh"

namespace ucl {

// integer scratch block_lu needs in shared memory: [0] pivot, [1..NB]
// interchanges, [39] count and [40..] (dst, src) pairs of <= 2*NB moved rows
constexpr int LU_NB_MAX = 32;
constexpr int LU_SI_INTS = 40 + 4 * LU_NB_MAX + 8;

template <typename T>
struct LuCfg;
template <>
struct LuCfg<float> {
  static constexpr int NB = 32, TM = 8, TN = 8;
};
template <>
struct LuCfg<double> {
  static constexpr int NB = 16, TM = 4, TN = 4;
};
static_assert(LuCfg<float>::NB <= LU_NB_MAX && LuCfg<double>::NB <= LU_NB_MAX, "LU scratch too small");


// P = I + con * J over an n x n row-major matrix: 16-byte vector loads issued
// eight at a time per thread so the memory round trips overlap (J is often
// no longer in L2 when P is re-formed).  n*n must be a multiple of the
// vector width (n even).
template <typename T>
__device__ void form_newton_matrix(const T* __restrict__ J, T* __restrict__ P, int n, T con) {
  using V = typename Vec2<T>::type;
  constexpr int W = Vec2<T>::W;
  constexpr int U = 8;
  const int nv = (n * n) / W;
  const V* __restrict__ Jv = reinterpret_cast<const V*>(J);
  V* __restrict__ Pv = reinterpret_cast<V*>(P);
  int i = threadIdx.x;
  for (; i + (U - 1) * NT < nv; i += U * NT) {
    V a[U];
#pragma unroll
    for (int u = 0; u < U; ++u) a[u] = Jv[i + u * NT];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      T* e = reinterpret_cast<T*>(&a[u]);
#pragma unroll
      for (int w = 0; w < W; ++w) e[w] *= con;
      Pv[i + u * NT] = a[u];
    }
  }
  for (; i < nv; i += NT) {
    V a = Jv[i];
    T* e = reinterpret_cast<T*>(&a);
#pragma unroll
    for (int w = 0; w < W; ++w) e[w] *= con;
    Pv[i] = a;
  }
  for (int t = nv * W + threadIdx.x; t < n * n; t += NT) P[t] = con * J[t];
  __syncthreads();
  for (int d = threadIdx.x; d < n; d += NT) P[(size_t)d * n + d] += (T)1;
  __syncthreads();
}

// Shared-memory layout of block_lu: the factored panel (L11/L21, rows of
// LDP = NB+1), the U12 block row, the per-warp pivot candidates (double
// buffered), and the panel's position maps.
// FP32 factorisations of n <= TC_MAX_N run the trailing update on the tensor
// cores (the staging of the split operands must fit in shared memory).
constexpr int TC_MAX_N = 352;

template <typename T>
struct LuSmem {
  static constexpr int NB = LuCfg<T>::NB, LDP = NB + 1;
  __host__ __device__ static constexpr size_t al(size_t b) { return (b + 127) & ~(size_t)127; }
  __host__ __device__ static constexpr bool tc_ok(int n) { return sizeof(T) == 4 && n <= TC_MAX_N; }
  __host__ __device__ static constexpr int np(int n) { return (n + 15) & ~15; }
  __host__ __device__ static constexpr size_t sp(int) { return 0; }
  // U12 block row (CUDA-core update) or the tensor-core operand staging:
  // A tile head, A tile tail, B head, B tail
  __host__ __device__ static constexpr size_t su(int n) { return al((size_t)n * LDP * sizeof(T)); }
  __host__ __device__ static constexpr size_t su_bytes(int n) {
    return tc_ok(n) ? tc_stage_bytes(np(n)) : (size_t)NB * n * sizeof(T);
  }
  __host__ __device__ static constexpr size_t crow(int n) { return su(n) + al(su_bytes(n)); }
  __host__ __device__ static constexpr size_t ckey(int n) { return crow(n) + (size_t)2 * NWARP * NB * sizeof(T); }
  __host__ __device__ static constexpr size_t maps(int n) { return ckey(n) + (size_t)2 * NWARP * 4 * sizeof(unsigned); }
  // (the diagonal-block inversion after the factorisation reuses the area
  // for NWARP staged 32 x 33 tiles)
  __host__ __device__ static constexpr size_t tiles() { return (size_t)NWARP * 32 * 33 * sizeof(T); }
  __host__ __device__ static constexpr size_t maps_bytes(int n) { return al((size_t)(2 * n + NB) * sizeof(int)); }
  __host__ __device__ static constexpr size_t bytes(int n) {
    return maps(n) + maps_bytes(n) + 16 > tiles() ? maps(n) + maps_bytes(n) + 16 : tiles();
  }
};

// shared-memory bytes the LU needs for an n x n matrix
template <typename T>
__host__ __device__ constexpr size_t lu_smem_bytes(int n) {
  return LuSmem<T>::bytes(n);
}

// correctly rounded reciprocal (the same value as 1 / x)
__device__ __forceinline__ float recip_rn(float x) { return __frcp_rn(x); }
__device__ __forceinline__ double recip_rn(double x) { return __drcp_rn(x); }

// |v| as an unsigned key whose integer order is the order of |v|
__device__ __forceinline__ unsigned long long abs_key(double v) {
  return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
}
__device__ __forceinline__ unsigned long long abs_key(float v) {
  return (unsigned long long)(__float_as_uint(v) & 0x7fffffffu);
}
// warp maximum of a key (keys of floats fit in 32 bits)
template <typename T>
__device__ __forceinline__ unsigned long long warp_max_key(unsigned long long k) {
  if (sizeof(T) == 4) return __reduce_max_sync(0xffffffffu, (unsigned)k);
  const unsigned hi = __reduce_max_sync(0xffffffffu, (unsigned)(k >> 32));
  const unsigned lo = __reduce_max_sync(0xffffffffu, (unsigned)(k >> 32) == hi ? (unsigned)k : 0u);
  return ((unsigned long long)hi << 32) | lo;
}

// Factor the m x nb panel at (k0, k0) with partial pivoting, rows held in
// registers: thread t owns panel rows t + NT*s (s < RPT).  Rows are not
// moved while the panel is factored; the pivot row of each column is
// recorded and, after the panel, row_at/pos_of are built from the
// LINPACK-order interchanges (DGEFA's ipvt).  One barrier per column: every
// warp publishes its best candidate (|v| key, row, and the row's values) in
// a double-buffered slot, then every warp reduces the NWARP candidates
// itself.  Ties go to the lowest lane / warp.  Zero pivot: no elimination,
// info = column + 1.
// Rows are written back to A (panel columns, final positions) and to the
// shared panel sp for the U12 solve and the trailing update.
template <typename T, int RPT>
__device__ __forceinline__ int panel_factor(T* __restrict__ A, int n, int k0, int nb, int m, char* smem,
                                            int info) {
  constexpr int NB = LuCfg<T>::NB, LDP = NB + 1;
  using V = typename Vec2<T>::type;
  constexpr int W = Vec2<T>::W;
  T* sp = (T*)(smem + LuSmem<T>::sp(n));
  T* crow = (T*)(smem + LuSmem<T>::crow(n));              // [2][NWARP][NB]
  unsigned* ckey = (unsigned*)(smem + LuSmem<T>::ckey(n));  // [2][NWARP][4]
  int* row_at = (int*)(smem + LuSmem<T>::maps(n));
  int* pos_of = row_at + n;
  int* piv = pos_of + n;  // [NB] pivot row chosen for each column
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const bool vec = (n % W) == 0;
  T a[RPT][NB];
  bool done[RPT];
#pragma unroll
  for (int s = 0; s < RPT; ++s) {
    const int i = tid + NT * s;
    done[s] = i >= m;
    const T* src = A + (size_t)(k0 + i) * n + k0;
    if (i < m && vec && nb == NB) {
#pragma unroll
      for (int j = 0; j < NB; j += W) {
        const V v = *reinterpret_cast<const V*>(src + j);
        const T* e = reinterpret_cast<const T*>(&v);
#pragma unroll
        for (int w = 0; w < W; ++w) a[s][j + w] = e[w];
      }
    } else {
#pragma unroll
      for (int j = 0; j < NB; ++j) a[s][j] = (i < m && j < nb) ? src[j] : (T)0;
    }
    if (i < m) { row_at[i] = i; pos_of[i] = i; }
  }
#pragma unroll
  for (int c = 0; c < NB; ++c) {
    if (c < nb) {
      const int buf = c & 1;
      // this thread's best row, then the warp's (key, row, values)
      unsigned long long bk = 0;
      int bs = 0;
#pragma unroll
      for (int s = 0; s < RPT; ++s) {
        // live rows key |v| + 1 (order kept), finished rows 0
        const unsigned long long k = done[s] ? 0ull : abs_key(a[s][c]) + 1ull;
        if (k > bk) { bk = k; bs = s; }
      }
      const unsigned long long wk = warp_max_key<T>(bk);
      const int owner = __ffs(__ballot_sync(0xffffffffu, bk == wk)) - 1;
      if (lane == owner) {
        T* dst = crow + (size_t)(buf * NWARP + warp) * NB;
#pragma unroll
        for (int j = (c / W) * W; j < NB; j += W) {
          V v;
          T* e = reinterpret_cast<T*>(&v);
#pragma unroll
          for (int w = 0; w < W; ++w) {
            T x = a[0][j + w];
#pragma unroll
            for (int s = 1; s < RPT; ++s)
              if (bs == s) x = a[s][j + w];
            e[w] = x;
          }
          *reinterpret_cast<V*>(dst + j) = v;
        }
        unsigned* kk = ckey + (buf * NWARP + warp) * 4;
        kk[0] = (unsigned)wk;
        kk[1] = (unsigned)(wk >> 32);
        kk[2] = (unsigned)(tid + NT * bs);
      }
      __syncthreads();
      // winner over the warps
      unsigned long long ck = 0;
      int crow_i = 0;
      if (lane < NWARP) {
        const uint4 kk = *reinterpret_cast<const uint4*>(ckey + (buf * NWARP + lane) * 4);
        ck = ((unsigned long long)kk.y << 32) | kk.x;
        crow_i = (int)kk.z;
      }
      const unsigned long long mk = warp_max_key<T>(ck);
      const int ww = __ffs(__ballot_sync(0xffffffffu, lane < NWARP && ck == mk)) - 1;
      const int pi = __shfl_sync(0xffffffffu, crow_i, ww);
      if (tid == 0) piv[c] = pi;
      if (mk == 1ull) {
        // zero pivot column: nothing is eliminated (DGEFA).  A zero row
        // other than the one at position c may be taken as the pivot row;
        // the factors of a singular matrix are not used (info != 0).
        if (info == 0) info = k0 + c + 1;
#pragma unroll
        for (int s = 0; s < RPT; ++s)
          if (tid + NT * s == pi) done[s] = true;
      } else {
        const T* pr = crow + (size_t)(buf * NWARP + ww) * NB;
        T prow[NB];
        const int c0 = (c / W) * W;
        if (NB % W == 0) {
#pragma unroll
          for (int j = c0; j < NB; j += W) {
            const V v = *reinterpret_cast<const V*>(pr + j);
            const T* e = reinterpret_cast<const T*>(&v);
#pragma unroll
            for (int w = 0; w < W; ++w) prow[j + w] = e[w];
          }
        }
        const T inv = recip_rn(prow[c]);
#pragma unroll
        for (int s = 0; s < RPT; ++s) {
          if (done[s]) continue;
          if (tid + NT * s == pi) { done[s] = true; continue; }
          const T l = a[s][c] * inv;
          a[s][c] = l;
#pragma unroll
          for (int j = c + 1; j < NB; ++j) a[s][j] -= l * prow[j];
        }
      }
    }
  }
  __syncthreads();
  // the interchanges of the panel in LINPACK order: position maps
  if (tid == 0) {
    for (int c = 0; c < nb; ++c) {
      const int pi = piv[c];
      const int q = pos_of[pi], r2 = row_at[c];
      row_at[c] = pi;
      row_at[q] = r2;
      pos_of[pi] = c;
      pos_of[r2] = q;
    }
  }
  __syncthreads();
  // rows to their final positions, in A and in the shared panel
#pragma unroll
  for (int s = 0; s < RPT; ++s) {
    const int i = tid + NT * s;
    if (i >= m) continue;
    const int fp = pos_of[i];
    T* dst = A + (size_t)(k0 + fp) * n + k0;
    if (vec && nb == NB) {
#pragma unroll
      for (int j = 0; j < NB; j += W) {
        V v;
        T* e = reinterpret_cast<T*>(&v);
#pragma unroll
        for (int w = 0; w < W; ++w) e[w] = a[s][j + w];
        *reinterpret_cast<V*>(dst + j) = v;
      }
    } else {
#pragma unroll
      for (int j = 0; j < NB; ++j)
        if (j < nb) dst[j] = a[s][j];
    }
#pragma unroll
    for (int j = 0; j < NB; ++j)
      if (j < nb) sp[fp * LDP + j] = a[s][j];
  }
  return info;
}

// Factor A (row-major n x n, global) in place.  perm[i] = original row of
// row i after pivoting.  Returns 0 or (first zero pivot index + 1).
// s_i: LU_SI_INTS ints of shared scratch; scr: 2*NB*n elements of global
// scratch for the row interchanges outside the panel; perm: shared [n].
// tc: tensor-core state of the CTA (TMEM + mbarrier) or nullptr for the
// CUDA-core trailing update.
// Not inlined (nor dev_rhs, dev_jac): inside the 255-register solver kernel
// each then gets a register allocation of its own; measured on 152 grid
// models, 272 -> 265 us per BDF step, the factorisation 637 -> 516 us (the
// triangular solve is faster inlined).
template <typename T>
__device__ __noinline__ int block_lu(T* __restrict__ A, int n, int* __restrict__ perm_out, char* smem, int* s_i,
                         T* __restrict__ scr, int* perm, TcState* tc = nullptr) {
  constexpr int NB = LuCfg<T>::NB, TM = LuCfg<T>::TM, TN = LuCfg<T>::TN;
  constexpr int LDP = NB + 1;
  T* sp = (T*)(smem + LuSmem<T>::sp(n));   // panel [m x LDP]
  T* su = (T*)(smem + LuSmem<T>::su(n));   // U12 [NB x ncols]
  const int* row_at = (const int*)(smem + LuSmem<T>::maps(n));
  const int tid = threadIdx.x;
  int info = 0;
  // perm lives in shared memory while factoring
  for (int i = tid; i < n; i += NT) perm[i] = i;
  for (int k0 = 0; k0 < n; k0 += NB) {
    const int nb = min(NB, n - k0);
    const int m = n - k0;
    const int ncols = n - k0 - nb;
    if (tid == 0) s_i[39] = 0;
    __syncthreads();
    if (m <= NT) info = panel_factor<T, 1>(A, n, k0, nb, m, smem, info);
    else if (m <= 2 * NT) info = panel_factor<T, 2>(A, n, k0, nb, m, smem, info);
    else info = panel_factor<T, (MAX_NEQ + NT - 1) / NT>(A, n, k0, nb, m, smem, info);
    // composite permutation and the list of moved rows (dst <- src), <= 2*nb
    int* mv = s_i + 40;
    int pv[(MAX_NEQ + NT - 1) / NT];
#pragma unroll
    for (int s = 0; s < (MAX_NEQ + NT - 1) / NT; ++s) {
      const int i = tid + NT * s;
      if (i < m) {
        const int src = row_at[i];
        pv[s] = perm[k0 + src];
        if (src != i) {
          const int q = atomicAdd(&s_i[39], 1);
          mv[2 * q] = k0 + i;
          mv[2 * q + 1] = k0 + src;
        }
      }
    }
    __syncthreads();
#pragma unroll
    for (int s = 0; s < (MAX_NEQ + NT - 1) / NT; ++s)
      if (tid + NT * s < m) perm[k0 + tid + NT * s] = pv[s];
    {
      // the same interchanges in the columns outside the panel, as one
      // gather through scr: a warp per moved row, 16-byte row segments
      using V = typename Vec2<T>::type;
      constexpr int W = Vec2<T>::W;
      const int lane = tid & 31, warp = tid >> 5;
      const int m2 = s_i[39];
      const bool vec = (n % W) == 0;
      for (int pass = 0; pass < 2; ++pass) {
        if (vec) {
          // 4 rows per warp at a time, all loads issued before the stores
          constexpr int RU = 4, CU = 3;
          for (int q0 = warp * RU; q0 < m2; q0 += NWARP * RU)
            for (int jb = 0; jb < n; jb += 32 * W * CU) {
              V v[RU][CU];
#pragma unroll
              for (int u = 0; u < RU; ++u) {
                const int q = q0 + u;
                const T* src = q < m2 ? (pass == 0 ? A + (size_t)mv[2 * q + 1] * n : scr + (size_t)q * n) : A;
#pragma unroll
                for (int t = 0; t < CU; ++t) {
                  const int j = jb + (lane + 32 * t) * W;
                  if (q < m2 && j < n && (j < k0 || j >= k0 + nb)) v[u][t] = *reinterpret_cast<const V*>(src + j);
                }
              }
#pragma unroll
              for (int u = 0; u < RU; ++u) {
                const int q = q0 + u;
                T* dst = q < m2 ? (pass == 0 ? scr + (size_t)q * n : A + (size_t)mv[2 * q] * n) : A;
#pragma unroll
                for (int t = 0; t < CU; ++t) {
                  const int j = jb + (lane + 32 * t) * W;
                  if (q < m2 && j < n && (j < k0 || j >= k0 + nb)) *reinterpret_cast<V*>(dst + j) = v[u][t];
                }
              }
            }
        } else {
          for (int q = warp; q < m2; q += NWARP) {
            const T* src = pass == 0 ? A + (size_t)mv[2 * q + 1] * n : scr + (size_t)q * n;
            T* dst = pass == 0 ? scr + (size_t)q * n : A + (size_t)mv[2 * q] * n;
            for (int j = lane; j < n; j += 32)
              if (j < k0 || j >= k0 + nb) dst[j] = src[j];
          }
        }
        __syncthreads();
      }
    }
    __syncthreads();
    if (ncols > 0) {
      const bool use_tc = tc != nullptr && LuSmem<T>::tc_ok(n) && nb == NB;
      char* bh = (char*)su + 2 * TC_M * 128;
      char* bl = bh + (size_t)LuSmem<T>::np(ncols) * 128;
      // U12 = L11^-1 A12
      for (int jj = tid; jj < ncols; jj += NT) {
        T x[NB];
        // the whole column of A12 first (independent loads), then the
        // forward substitution with L11 from shared memory
#pragma unroll
        for (int q = 0; q < NB; ++q) x[q] = q < nb ? A[(size_t)(k0 + q) * n + k0 + nb + jj] : (T)0;
#pragma unroll
        for (int q = 1; q < NB; ++q) {
          if (q < nb) {
            T v = x[q];
#pragma unroll
            for (int p = 0; p < q; ++p) v -= sp[q * LDP + p] * x[p];
            x[q] = v;
          }
        }
#pragma unroll
        for (int q = 0; q < NB; ++q)
          if (q < nb) A[(size_t)(k0 + q) * n + k0 + nb + jj] = x[q];
        if constexpr (sizeof(T) == 4) {
          if (use_tc) {
            // B operand of the tensor-core update: row jj = column jj of U12
#pragma unroll
            for (int q = 0; q < NB; q += 4) tc_put4(bh, bl, jj, q, x[q], x[q + 1], x[q + 2], x[q + 3]);
            continue;
          }
        }
#pragma unroll
        for (int q = 0; q < NB; ++q)
          if (q < nb) su[q * ncols + jj] = x[q];
      }
      if (use_tc) {
        // zero rows of B past ncols (N is padded to a multiple of 16)
        for (int t = tid; t < (LuSmem<T>::np(ncols) - ncols) * 8; t += NT) {
          const int r = ncols + (t >> 3), k4 = (t & 7) * 4;
          tc_put4(bh, bl, r, k4, 0.f, 0.f, 0.f, 0.f);
        }
      }
      __syncthreads();
      if constexpr (sizeof(T) == 4) {
        if (use_tc) {
          if (!tc_trailing_update(A, n, k0 + nb, k0 + nb, m - nb, ncols, sp + nb * LDP, LDP, (char*)su,
                                  (char*)su + TC_M * 128, bh, bl, tc))
            info = n + 1;
          __syncthreads();
          continue;
        }
      }
      // A22 -= L21 * U12
      const int R = m - nb;
      const int TR = (R + TM - 1) / TM, TC = (ncols + TN - 1) / TN;
      for (int t = tid; t < TR * TC; t += NT) {
        const int ti = t / TC, tj = t - ti * TC;
        const int r0 = ti * TM, j0 = tj * TN;
        T acc[TM][TN];
        using V = typename Vec2<T>::type;
        constexpr int W = Vec2<T>::W;
        const bool full = (r0 + TM <= R) && (j0 + TN <= ncols) && (n % W == 0);
        if (full) {
#pragma unroll
          for (int a = 0; a < TM; ++a)
#pragma unroll
            for (int b = 0; b < TN; b += W) {
              const V v = *reinterpret_cast<const V*>(A + (size_t)(k0 + nb + r0 + a) * n + k0 + nb + j0 + b);
              const T* e = reinterpret_cast<const T*>(&v);
#pragma unroll
              for (int w = 0; w < W; ++w) acc[a][b + w] = e[w];
            }
        } else {
#pragma unroll
          for (int a = 0; a < TM; ++a)
#pragma unroll
            for (int b = 0; b < TN; ++b) {
              const int r = r0 + a, j = j0 + b;
              acc[a][b] = (r < R && j < ncols) ? A[(size_t)(k0 + nb + r) * n + k0 + nb + j] : (T)0;
            }
        }
        for (int q = 0; q < nb; ++q) {
          T av[TM], bv[TN];
#pragma unroll
          for (int a = 0; a < TM; ++a) av[a] = (r0 + a < R) ? sp[(nb + r0 + a) * LDP + q] : (T)0;
          if (j0 + TN <= ncols && (ncols % W) == 0) {
#pragma unroll
            for (int b = 0; b < TN; b += W) {
              const V v = *reinterpret_cast<const V*>(su + q * ncols + j0 + b);
              const T* e = reinterpret_cast<const T*>(&v);
#pragma unroll
              for (int w = 0; w < W; ++w) bv[b + w] = e[w];
            }
          } else {
#pragma unroll
            for (int b = 0; b < TN; ++b) bv[b] = (j0 + b < ncols) ? su[q * ncols + j0 + b] : (T)0;
          }
#pragma unroll
          for (int a = 0; a < TM; ++a)
#pragma unroll
            for (int b = 0; b < TN; ++b) acc[a][b] -= av[a] * bv[b];
        }
        if (full) {
#pragma unroll
          for (int a = 0; a < TM; ++a)
#pragma unroll
            for (int b = 0; b < TN; b += W) {
              V v;
              T* e = reinterpret_cast<T*>(&v);
#pragma unroll
              for (int w = 0; w < W; ++w) e[w] = acc[a][b + w];
              *reinterpret_cast<V*>(A + (size_t)(k0 + nb + r0 + a) * n + k0 + nb + j0 + b) = v;
            }
        } else {
#pragma unroll
          for (int a = 0; a < TM; ++a)
#pragma unroll
            for (int b = 0; b < TN; ++b) {
              const int r = r0 + a, j = j0 + b;
              if (r < R && j < ncols) A[(size_t)(k0 + nb + r) * n + k0 + nb + j] = acc[a][b];
            }
        }
      }
    }
    __syncthreads();
  }
  for (int i = tid; i < n; i += NT) perm_out[i] = perm[i];
  __syncthreads();
  return info;
}

// elements per n x n matrix slot in batched workspaces: n*n rounded up to a
// multiple of 4, so every slot starts 16-byte aligned (the vector loads of
// the LU and the Newton-matrix formation) for any n
__host__ __device__ constexpr size_t mat_stride(int n) { return ((size_t)n * n + 3) & ~(size_t)3; }

// elements of the diagonal-block inverses of an n x n factorisation
__host__ __device__ constexpr size_t dinv_elems(int n) { return (size_t)((n + 31) / 32) * 2 * 1024; }

// Diagonal 32 x 32 blocks of the factors in the form the block solves use,
// after block_lu: dinv[(2*b + 0)*1024 + i*32 + j] = (L_bb^-1)[i][j] (unit
// lower, |l| <= 1, so its inverse is well conditioned), and
// dinv[(2*b + 1)*1024 + ...] = U_bb itself (upper part, contiguous) with the
// reciprocal of the pivot on the diagonal: U blocks carry the conditioning
// of P, so they are applied by substitution, which is backward stable (an
// explicit U_bb^-1 measurably loosened element conservation of the FP32
// solve).  Rows and columns past n are the identity.  One warp per block:
// lane j forms column j of L_bb^-1 by substitution against the block staged
// in shared memory.  tile: shared, NWARP * 32 * 33 elements.
template <typename T>
__device__ void lu_diag_inverses(const T* __restrict__ A, int n, T* __restrict__ dinv, T* tile) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nblk = (n + 31) / 32;
  T* t = tile + warp * 32 * 33;
  for (int job = warp; job < 2 * nblk; job += NWARP) {
    const int b = job >> 1, k0 = b * 32, nb = min(32, n - k0);
    const bool upper = job & 1;
#pragma unroll 8
    for (int r = 0; r < 32; ++r)
      t[r * 33 + lane] = (r < nb && lane < nb) ? A[(size_t)(k0 + r) * n + k0 + lane] : (T)(r == lane ? 1 : 0);
    __syncwarp();
    T y[32];
    if (!upper) {
#pragma unroll
      for (int i = 0; i < 32; ++i) {
        T v = (i == lane) ? (T)1 : (T)0;
#pragma unroll
        for (int q = 0; q < i; ++q) v -= t[i * 33 + q] * y[q];
        y[i] = v;
      }
    } else {
#pragma unroll
      for (int i = 0; i < 32; ++i) {
        const T u = t[i * 33 + lane];
        y[i] = lane > i ? u : lane == i ? (T)1 / u : (T)0;
      }
    }
    T* d = dinv + (size_t)job * 1024;
#pragma unroll
    for (int i = 0; i < 32; ++i) d[i * 32 + lane] = y[i];
    __syncwarp();
  }
}

// Solve (LU) x = b with the factors, the row permutation and the diagonal
// blocks prepared by lu_diag_inverses.
// Forward over the 32-row blocks of L, then backward over those of U; per
// block: r = b_blk - (off-diagonal block row) . x with 4 rows per warp,
// lane-strided 16-byte loads (independent of x, so they are all in flight
// at once) and warp sums; then warp 0 forms x_blk = L_bb^-1 r (a GEMV) or
// solves U_bb x_blk = r from registers.  Two barriers per block.
// tmp: shared [n]; rbuf: shared [32].
// The right-hand side comes in and the solution goes out as FP64 y (shared):
// the system solved is (LU) x = W y and y <- W^-1 x, with W = diag(ws) and
// W^-1 = diag(wis) (both nullptr: no scaling).
template <typename T>
__device__ void block_lusolve(const T* __restrict__ A, int n, const int* __restrict__ perm,
                              const T* __restrict__ dinv, double* y, const double* ws, const double* wis, T* tmp,
                              T* rbuf) {
  using V = typename Vec2<T>::type;
  constexpr int W = Vec2<T>::W;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nblk = (n + 31) / 32;
  const bool vec = (n % W) == 0;
  for (int i = tid; i < n; i += NT) {
    const int p = perm[i];
    tmp[i] = (T)(ws ? ws[p] * y[p] : y[p]);
  }
  __syncthreads();
  for (int pass = 0; pass < 2; ++pass) {
    for (int step = 0; step < nblk; ++step) {
      const int b = pass == 0 ? step : nblk - 1 - step;
      const int k0 = b * 32, nb = min(32, n - k0);
      const int c0 = pass == 0 ? 0 : k0 + nb, c1 = pass == 0 ? k0 : n;
      T drow[32];
      if (warp == 0) {
        const V* dv = reinterpret_cast<const V*>(dinv + (size_t)(2 * b + pass) * 1024 + lane * 32);
#pragma unroll
        for (int u = 0; u < 32 / W; ++u) {
          const V v = dv[u];
          const T* e = reinterpret_cast<const T*>(&v);
#pragma unroll
          for (int w = 0; w < W; ++w) drow[u * W + w] = e[w];
        }
      }
      T s[4] = {(T)0, (T)0, (T)0, (T)0};
      const int r0 = warp * 4;
      if (vec) {
        // c0, c1 are multiples of W here (block edges, n % W == 0)
        for (int j = c0 + lane * W; j < c1; j += 32 * W) {
          const V xv = *reinterpret_cast<const V*>(tmp + j);
          const T* xe = reinterpret_cast<const T*>(&xv);
          V av[4];
#pragma unroll
          for (int a = 0; a < 4; ++a)
            if (r0 + a < nb) av[a] = *reinterpret_cast<const V*>(A + (size_t)(k0 + r0 + a) * n + j);
#pragma unroll
          for (int a = 0; a < 4; ++a)
            if (r0 + a < nb) {
              const T* e = reinterpret_cast<const T*>(&av[a]);
#pragma unroll
              for (int w = 0; w < W; ++w) s[a] += e[w] * xe[w];
            }
        }
      } else {
        for (int j = c0 + lane; j < c1; j += 32) {
          const T xj = tmp[j];
#pragma unroll
          for (int a = 0; a < 4; ++a)
            if (r0 + a < nb) s[a] += A[(size_t)(k0 + r0 + a) * n + j] * xj;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int a = 0; a < 4; ++a) s[a] += __shfl_xor_sync(0xffffffffu, s[a], o);
      if (lane < 4) {
        const int r = r0 + lane;
        const T sv = lane == 0 ? s[0] : lane == 1 ? s[1] : lane == 2 ? s[2] : s[3];
        rbuf[r] = r < nb ? tmp[k0 + r] - sv : (T)0;
      }
      __syncthreads();
      if (warp == 0) {
        T v;
        if (pass == 0) {
          v = (T)0;
#pragma unroll
          for (int j = 0; j < 32; ++j) v += drow[j] * rbuf[j];
        } else {
          // back substitution on the block held in registers (drow = row
          // `lane` of U_bb, reciprocal pivot on the diagonal)
          v = rbuf[lane];
#pragma unroll
          for (int q = 31; q >= 0; --q) {
            if (lane == q) v *= drow[q];
            const T xq = __shfl_sync(0xffffffffu, v, q);
            if (lane < q) v -= drow[q] * xq;
          }
        }
        if (lane < nb) tmp[k0 + lane] = v;
      }
      __syncthreads();
    }
  }
  for (int i = tid; i < n; i += NT) y[i] = wis ? (double)tmp[i] * wis[i] : (double)tmp[i];
  __syncthreads();
}

}  // namespace ucl

