// Warp-level dense LU with partial pivoting and triangular solves on column-major matrices in shared memory
// (the factorization LAPACK dgetrf computes, with 0-based pivots), used by the batched Newton algebra and by the
// persistent integrator.
#pragma once
#include <cuda_runtime.h>

namespace sfgb {

__device__ __forceinline__ unsigned long long abs_key(double x)
{
  return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}
__device__ __forceinline__ unsigned long long abs_key(float x)
{
  return (unsigned long long)((unsigned)__float_as_int(x) & 0x7fffffffu);
}

// Right-looking LU with partial pivoting of an m x m column-major matrix in shared memory, one warp.
// Pivot rows are 0-based. Returns info (0, or k+1 for an exactly zero pivot at step k).
template <typename F>
__device__ __forceinline__ int warp_lu(F *A, int m, int *piv)
{
  const int lane = threadIdx.x & 31;
  int info = 0;
  for (int k = 0; k < m; ++k) {
    // pivot: first index of the largest |A[i,k]|, i >= k (as idamax); magnitudes are compared as the integer bit
    // patterns of |x|, which order finite non-negative values like the values themselves
    unsigned long long best = 0ull;
    int bi = m;
    for (int i = k + lane; i < m; i += 32) {
      const unsigned long long key = abs_key(A[i + k * m]);
      if (bi == m || key > best) { best = key; bi = i; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (oi < m && (bi >= m || ob > best || (ob == best && oi < bi))) { best = ob; bi = oi; }
    }
    if (lane == 0) piv[k] = bi;
    if (bi != k)
      for (int j = lane; j < m; j += 32) {
        const F t = A[k + j * m];
        A[k + j * m] = A[bi + j * m];
        A[bi + j * m] = t;
      }
    __syncwarp();
    const F pv = A[k + k * m];
    if (pv == (F)0) {
      if (!info) info = k + 1;
      continue;
    }
    const F inv = (F)1 / pv;
    for (int i = k + 1 + lane; i < m; i += 32) A[i + k * m] *= inv;
    __syncwarp();
    // trailing update, flattened over (i, j) so every lane has work
    const int r = m - k - 1;
    const int tot = r * r;
    for (int t = lane; t < tot; t += 32) {
      const int jj = t / r, ii = t - jj * r;
      const int i = k + 1 + ii, j = k + 1 + jj;
      A[i + j * m] -= A[i + k * m] * A[k + j * m];
    }
    __syncwarp();
  }
  return info;
}

// Solve (LU) x = b in place on x (shared memory), one warp.
template <typename F>
__device__ __forceinline__ void warp_lu_solve(const F *LU, int m, const int *piv, F *x)
{
  const int lane = threadIdx.x & 31;
  if (lane == 0)
    for (int k = 0; k < m; ++k) {
      const int p = piv[k];
      if (p != k) { const F t = x[k]; x[k] = x[p]; x[p] = t; }
    }
  __syncwarp();
  for (int j = 0; j < m; ++j) {
    const F xj = x[j];
    for (int i = j + 1 + lane; i < m; i += 32) x[i] -= LU[i + j * m] * xj;
    __syncwarp();
  }
  for (int j = m - 1; j >= 0; --j) {
    if (lane == 0) x[j] /= LU[j + j * m];
    __syncwarp();
    const F xj = x[j];
    for (int i = lane; i < j; i += 32) x[i] -= LU[i + j * m] * xj;
    __syncwarp();
  }
}

// warp_lu for repeated solves: returns the final row permutation (perm[i]: the original row that ends in row i)
// instead of LAPACK's interchanges, and the reciprocals of U's diagonal (the 1 / pivot the factorization computes
// anyway), so that a solve applies the permutation while loading its right-hand side and multiplies instead of
// dividing on its serial backward sweep.
template <typename F>
__device__ __forceinline__ int warp_lu_pd(F *A, int m, int *perm, F *dinv)
{
  const int lane = threadIdx.x & 31;
  for (int i = lane; i < m; i += 32) perm[i] = i;
  __syncwarp();
  int info = 0;
  for (int k = 0; k < m; ++k) {
    unsigned long long best = 0ull;
    int bi = m;
    for (int i = k + lane; i < m; i += 32) {
      const unsigned long long key = abs_key(A[i + k * m]);
      if (bi == m || key > best) { best = key; bi = i; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (oi < m && (bi >= m || ob > best || (ob == best && oi < bi))) { best = ob; bi = oi; }
    }
    if (bi != k) {
      if (lane == 0) {
        const int t = perm[k];
        perm[k] = perm[bi];
        perm[bi] = t;
      }
      for (int j = lane; j < m; j += 32) {
        const F t = A[k + j * m];
        A[k + j * m] = A[bi + j * m];
        A[bi + j * m] = t;
      }
    }
    __syncwarp();
    const F pv = A[k + k * m];
    const F inv = (F)1 / pv;
    if (lane == 0) dinv[k] = inv;
    if (pv == (F)0) {
      if (!info) info = k + 1;
      continue;
    }
    for (int i = k + 1 + lane; i < m; i += 32) A[i + k * m] *= inv;
    __syncwarp();
    const int r = m - k - 1;
    const int tot = r * r;
    for (int t = lane; t < tot; t += 32) {
      const int jj = t / r, ii = t - jj * r;
      const int i = k + 1 + ii, j = k + 1 + jj;
      A[i + j * m] -= A[i + k * m] * A[k + j * m];
    }
    __syncwarp();
  }
  return info;
}

// Solve (LU) x = b with the factors of warp_lu_pd, x holding the permuted right-hand side (x[i] = b[perm[i]]).
template <typename F>
__device__ __forceinline__ void warp_lu_solve_pd(const F *LU, int m, const F *dinv, F *x)
{
  const int lane = threadIdx.x & 31;
  __syncwarp();
  for (int j = 0; j < m; ++j) {
    const F xj = x[j];
    for (int i = j + 1 + lane; i < m; i += 32) x[i] -= LU[i + j * m] * xj;
    __syncwarp();
  }
  for (int j = m - 1; j >= 0; --j) {
    const F xj = x[j] * dinv[j];
    for (int i = lane; i < j; i += 32) x[i] -= LU[i + j * m] * xj;
    __syncwarp();
    if (lane == 0) x[j] = xj;  // after the barrier: no lane still reads x[j]
  }
  __syncwarp();
}

}  // namespace sfgb
