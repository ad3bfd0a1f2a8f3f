// Dense LU with partial pivoting and triangular solves for one system per
// CTA (the Newton matrix P = I - h*gamma*J of the BDF corrector; the
// reference factors it with LINPACK DGEFA/DGESL, dvode.f90:11982-12160).
//
// Storage is row-major (P[i*n + j]) so that row interchanges, panel loads and
// the register-tiled trailing update are all coalesced.  The blocked
// right-looking algorithm:
//   for each panel of NB columns:
//     factor the (n-k0) x NB panel in shared memory (warp pivot search,
//     row swap, scaling, rank-1 updates);
//     swap the same rows in the columns outside the panel;
//     U12 = L11^-1 A12 (one thread per column, registers);
//     A22 -= L21 * U12 (register tiles of TM x TN, operands in shared memory).
// The composite row permutation is kept as perm[] so a solve gathers the
// right-hand side in one parallel pass.
#pragma once
#include "ucl_common.cuh"

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

template <typename T>
struct Vec2;
template <>
struct Vec2<float> { using type = float4; static constexpr int W = 4; };
template <>
struct Vec2<double> { using type = double2; static constexpr int W = 2; };

// P = I + con * J over an n x n row-major matrix: 16-byte vector loads issued
// four at a time so the L2 round trips overlap.  n*n must be a multiple of
// the vector width (n even).
template <typename T>
__device__ void form_newton_matrix(const T* __restrict__ J, T* __restrict__ P, int n, T con) {
  using V = typename Vec2<T>::type;
  constexpr int W = Vec2<T>::W;
  const int nv = (n * n) / W;
  const V* __restrict__ Jv = reinterpret_cast<const V*>(J);
  V* __restrict__ Pv = reinterpret_cast<V*>(P);
  int i = threadIdx.x;
  for (; i + 3 * NT < nv; i += 4 * NT) {
    V a[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) a[u] = Jv[i + u * NT];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
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

// shared-memory bytes the LU needs for an n x n matrix
template <typename T>
__host__ __device__ constexpr size_t lu_smem_bytes(int n) {
  return sizeof(T) * ((size_t)n * (LuCfg<T>::NB + 1) + (size_t)LuCfg<T>::NB * n) + 64;
}

// Factor A (row-major n x n, global) in place.  perm[i] = original row of
// row i after pivoting.  Returns 0 or (first zero pivot index + 1).
template <typename T>
__device__ int block_lu(T* __restrict__ A, int n, int* __restrict__ perm_out, char* smem, int* s_i,
                         T* __restrict__ scr, int* perm) {
  constexpr int NB = LuCfg<T>::NB, TM = LuCfg<T>::TM, TN = LuCfg<T>::TN;
  constexpr int LDP = NB + 1;
  T* sp = (T*)smem;                  // panel [m x LDP]
  T* su = sp + (size_t)n * LDP;      // U12 [NB x ncols]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int info = 0;
  // perm lives in shared memory while factoring (it is updated per column)
  for (int i = tid; i < n; i += NT) perm[i] = i;
  __syncthreads();
  for (int k0 = 0; k0 < n; k0 += NB) {
    const int nb = min(NB, n - k0);
    const int m = n - k0;
    const int ncols = n - k0 - nb;
    {
      const int tot = m * nb;
      int idx = tid;
      for (; idx + 3 * NT < tot; idx += 4 * NT) {
        T v[4];
        int rr[4], cc[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          rr[u] = (idx + u * NT) / nb;
          cc[u] = idx + u * NT - rr[u] * nb;
          v[u] = A[(size_t)(k0 + rr[u]) * n + k0 + cc[u]];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) sp[rr[u] * LDP + cc[u]] = v[u];
      }
      for (; idx < tot; idx += NT) {
        const int r = idx / nb, c = idx - r * nb;
        sp[r * LDP + c] = A[(size_t)(k0 + r) * n + k0 + c];
      }
    }
    __syncthreads();
    for (int c = 0; c < nb; ++c) {
      if (warp == 0) {
        T best = (T)-1;
        int bi = c;
        for (int r = c + lane; r < m; r += 32) {
          const T v = fabs(sp[r * LDP + c]);
          if (v > best) { best = v; bi = r; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const T ov = __shfl_xor_sync(0xffffffffu, best, o);
          const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
          if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
        }
        if (lane == 0) s_i[0] = bi;
      }
      __syncthreads();
      const int p = s_i[0];
      const T pv = sp[p * LDP + c];
      if (pv == (T)0) {
        if (info == 0) info = k0 + c + 1;
        if (tid == 0) s_i[1 + c] = c;
        __syncthreads();
        continue;
      }
      if (p != c) {
        for (int j = tid; j < nb; j += NT) {
          const T t = sp[p * LDP + j];
          sp[p * LDP + j] = sp[c * LDP + j];
          sp[c * LDP + j] = t;
        }
        if (tid == 0) {
          const int t = perm[k0 + p];
          perm[k0 + p] = perm[k0 + c];
          perm[k0 + c] = t;
          s_i[1 + c] = p;  // remember the interchange for the other columns
        }
      } else if (tid == 0) {
        s_i[1 + c] = c;
      }
      __syncthreads();
      const T inv = (T)1 / sp[c * LDP + c];
      T prow[NB];
#pragma unroll
      for (int j = 0; j < NB; ++j) prow[j] = (j > c && j < nb) ? sp[c * LDP + j] : (T)0;
      for (int r = c + 1 + tid; r < m; r += NT) {
        T* row = sp + r * LDP;
        const T l = row[c] * inv;
        row[c] = l;
#pragma unroll
        for (int j = 0; j < NB; ++j)
          if (j > c && j < nb) row[j] -= l * prow[j];
      }
      __syncthreads();
    }
    // panel back to A
    for (int idx = tid; idx < m * nb; idx += NT) {
      const int r = idx / nb, c = idx - r * nb;
      A[(size_t)(k0 + r) * n + k0 + c] = sp[r * LDP + c];
    }
    __syncthreads();
    // the same interchanges in the columns outside the panel, applied as one
    // gather: thread 0 composes the nb transpositions into dst <- src row
    // pairs (s_i[40..]), then all threads stage the source rows in scr and
    // write them back (independent, coalesced row segments).
    int* mv_dst = s_i + 40;  // <= 2*NB moved rows
    if (tid == 0) {
      int cnt = 0;
      int rows[2 * NB], src[2 * NB];
      for (int c = 0; c < nb; ++c) {
        const int a = k0 + c, b = k0 + s_i[1 + c];
        if (a == b) continue;
        int ia = -1, ib = -1;
        for (int q = 0; q < cnt; ++q) { if (rows[q] == a) ia = q; if (rows[q] == b) ib = q; }
        if (ia < 0) { rows[cnt] = a; src[cnt] = a; ia = cnt++; }
        if (ib < 0) { rows[cnt] = b; src[cnt] = b; ib = cnt++; }
        const int t = src[ia]; src[ia] = src[ib]; src[ib] = t;
      }
      int m2 = 0;
      for (int q = 0; q < cnt; ++q)
        if (src[q] != rows[q]) { mv_dst[2 * m2] = rows[q]; mv_dst[2 * m2 + 1] = src[q]; ++m2; }
      s_i[39] = m2;
    }
    __syncthreads();
    {
      const int m2 = s_i[39];
      const int w = n - nb;  // columns outside the panel
      const int tot = m2 * w;
      for (int idx = tid; idx < tot; idx += 4 * NT) {
        T v[4];
        size_t dst[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int id = idx + u * NT;
          const int q = id / w, jj0 = id - q * w;
          const int jj = jj0 < k0 ? jj0 : jj0 + nb;
          dst[u] = (size_t)q * n + jj;
          v[u] = id < tot ? A[(size_t)mv_dst[2 * q + 1] * n + jj] : (T)0;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (idx + u * NT < tot) scr[dst[u]] = v[u];
      }
      __syncthreads();
      for (int idx = tid; idx < tot; idx += 4 * NT) {
        T v[4];
        size_t dst[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int id = idx + u * NT;
          const int q = id / w, jj0 = id - q * w;
          const int jj = jj0 < k0 ? jj0 : jj0 + nb;
          dst[u] = (size_t)mv_dst[2 * q] * n + jj;
          v[u] = id < tot ? scr[(size_t)q * n + jj] : (T)0;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (idx + u * NT < tot) A[dst[u]] = v[u];
      }
    }
    __syncthreads();
    if (ncols > 0) {
      // U12 = L11^-1 A12
      for (int jj = tid; jj < ncols; jj += NT) {
        T x[NB];
#pragma unroll
        for (int q = 0; q < NB; ++q) {
          if (q < nb) {
            T v = A[(size_t)(k0 + q) * n + k0 + nb + jj];
            for (int p = 0; p < q; ++p) v -= sp[q * LDP + p] * x[p];
            x[q] = v;
          }
        }
#pragma unroll
        for (int q = 0; q < NB; ++q) {
          if (q < nb) {
            A[(size_t)(k0 + q) * n + k0 + nb + jj] = x[q];
            su[q * ncols + jj] = x[q];
          }
        }
      }
      __syncthreads();
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

// s - row[0:nb] . x[0:nb], with 16-byte loads of the row when aligned
template <typename T>
__device__ __forceinline__ T dot_sub(const T* __restrict__ row, const T* x, int nb, T s, int n) {
  using V = typename Vec2<T>::type;
  constexpr int W = Vec2<T>::W;
  if ((n % W) == 0 && (nb % W) == 0) {
    const V* rv = reinterpret_cast<const V*>(row);
    V buf[32 / W];
#pragma unroll
    for (int u = 0; u < 32 / W; ++u)
      if (u * W < nb) buf[u] = rv[u];
#pragma unroll
    for (int u = 0; u < 32 / W; ++u)
      if (u * W < nb) {
        const T* e = reinterpret_cast<const T*>(&buf[u]);
#pragma unroll
        for (int w = 0; w < W; ++w) s -= e[w] * x[u * W + w];
      }
    return s;
  }
  for (int q = 0; q < nb; ++q) s -= row[q] * x[q];
  return s;
}

// Solve (LU) x = b in place, x in shared memory (precision T), perm from
// block_lu.  tmp: shared [n]; tile: shared [32 x 33] staging of the diagonal
// blocks.  Per 32-row block: warp 0 solves the diagonal block from the
// staged tile while the others wait; then all threads update the remaining
// rows (16-byte row loads) and, in the same phase, stage the next diagonal
// block, so the two load latencies overlap.
template <typename T>
__device__ void block_lusolve(const T* __restrict__ A, int n, const int* __restrict__ perm, T* x,
                                           T* tmp, T* tile) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nblk = (n + 31) / 32;
  auto stage = [&](int k0, bool upper) {
    const int nb = min(32, n - k0);
    for (int idx = tid; idx < 32 * 32; idx += NT) {
      const int r = idx >> 5, c = idx & 31;
      const bool in = r < nb && c < nb && (upper ? c >= r : c < r);
      tile[r * 33 + c] = in ? A[(size_t)(k0 + r) * n + k0 + c] : (T)0;
    }
  };
  for (int i = tid; i < n; i += NT) tmp[i] = x[perm[i]];
  stage(0, false);
  __syncthreads();
  // forward: unit lower
  for (int bk = 0; bk < nblk; ++bk) {
    const int k0 = bk * 32, nb = min(32, n - k0);
    if (warp == 0) {
      T xi = lane < nb ? tmp[k0 + lane] : (T)0;
#pragma unroll
      for (int q = 0; q < 31; ++q) {
        const T xq = __shfl_sync(0xffffffffu, xi, q);
        if (lane > q) xi -= tile[lane * 33 + q] * xq;
      }
      if (lane < nb) tmp[k0 + lane] = xi;
    }
    __syncthreads();
    for (int i = k0 + nb + tid; i < n; i += NT) tmp[i] = dot_sub<T>(A + (size_t)i * n + k0, tmp + k0, nb, tmp[i], n);
    if (bk + 1 < nblk) stage(k0 + 32, false);
    else stage((nblk - 1) * 32, true);
    __syncthreads();
  }
  // backward: upper
  for (int bk = nblk - 1; bk >= 0; --bk) {
    const int k0 = bk * 32, nb = min(32, n - k0);
    if (warp == 0) {
      T xi = lane < nb ? tmp[k0 + lane] : (T)0;
#pragma unroll
      for (int q = 31; q >= 0; --q) {
        if (q < nb) {
          if (lane == q) xi = xi / tile[q * 33 + q];
          const T xq = __shfl_sync(0xffffffffu, xi, q);
          if (lane < q) xi -= tile[lane * 33 + q] * xq;
        }
      }
      if (lane < nb) tmp[k0 + lane] = xi;
    }
    __syncthreads();
    for (int i = tid; i < k0; i += NT) tmp[i] = dot_sub<T>(A + (size_t)i * n + k0, tmp + k0, nb, tmp[i], n);
    if (bk > 0) stage(k0 - 32, true);
    __syncthreads();
  }
  for (int i = tid; i < n; i += NT) x[i] = tmp[i];
  __syncthreads();
}

}  // namespace ucl

