// Batched dense Newton algebra: LU factorization of A = gamma_h * J - I with partial pivoting and the matching
// triangular solves, one warp per matrix, the matrix held in shared memory.
//
// Replaces the scipy LAPACK calls of HomogeneousReactor (reactors.py:340-356): dgetrf on (prefactor*J - I) and
// dgetrs per Newton iteration. The FP32 variant factorizes the same matrix in single precision (FP32 pipe) and
// recovers FP64 accuracy in the solve by residual refinement r = b - A x with A in FP64.
#include "sf_internal.h"
#include "warp_lu.cuh"

namespace sfgb {

namespace {

constexpr int kWarpsPerCta = 4;

__global__ void lu64_kernel(int n, int m, const double *J, const double *gh, double *outA, double *outLU, int *piv,
                            int *info)
{
  extern __shared__ __align__(16) unsigned char sm[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t mm = (size_t)m * m;
  double *A = reinterpret_cast<double *>(sm) + (size_t)w * mm;
  int *pv = reinterpret_cast<int *>(reinterpret_cast<double *>(sm) + (size_t)kWarpsPerCta * mm) + w * m;
  for (int s = blockIdx.x * kWarpsPerCta + w; s < n; s += gridDim.x * kWarpsPerCta) {
    const double g = gh[s];
    const double *Js = J + s * mm;
    for (size_t e = lane; e < mm; e += 32) {
      const int col = (int)(e / m), row = (int)(e - (size_t)col * m);
      const double v = g * Js[e] - (row == col ? 1. : 0.);
      A[e] = v;
      if (outA) outA[s * mm + e] = v;
    }
    __syncwarp();
    const int inf = warp_lu(A, m, pv);
    for (size_t e = lane; e < mm; e += 32) outLU[s * mm + e] = A[e];
    for (int k = lane; k < m; k += 32) piv[(size_t)s * m + k] = pv[k];
    if (info && lane == 0) info[s] = inf;
    __syncwarp();
  }
}

__global__ void lu32_kernel(int n, int m, const double *J, const double *gh, double *outA, float *outLU, int *piv,
                            int *info)
{
  extern __shared__ __align__(16) unsigned char sm[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t mm = (size_t)m * m;
  float *A = reinterpret_cast<float *>(sm) + (size_t)w * mm;
  int *pv = reinterpret_cast<int *>(reinterpret_cast<float *>(sm) + (size_t)kWarpsPerCta * mm) + w * m;
  for (int s = blockIdx.x * kWarpsPerCta + w; s < n; s += gridDim.x * kWarpsPerCta) {
    const double g = gh[s];
    const double *Js = J + s * mm;
    for (size_t e = lane; e < mm; e += 32) {
      const int col = (int)(e / m), row = (int)(e - (size_t)col * m);
      const double v = g * Js[e] - (row == col ? 1. : 0.);
      A[e] = (float)v;
      outA[s * mm + e] = v;
    }
    __syncwarp();
    const int inf = warp_lu(A, m, pv);
    for (size_t e = lane; e < mm; e += 32) outLU[s * mm + e] = A[e];
    for (int k = lane; k < m; k += 32) piv[(size_t)s * m + k] = pv[k];
    if (info && lane == 0) info[s] = inf;
    __syncwarp();
  }
}

__global__ void solve64_kernel(int n, int m, const double *LU, const int *piv, const double *b, double *x)
{
  extern __shared__ __align__(16) unsigned char sm[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t mm = (size_t)m * m;
  double *L = reinterpret_cast<double *>(sm) + (size_t)w * (mm + m);
  double *xs = L + mm;
  int *pv = reinterpret_cast<int *>(reinterpret_cast<double *>(sm) + (size_t)kWarpsPerCta * (mm + m)) + w * m;
  for (int s = blockIdx.x * kWarpsPerCta + w; s < n; s += gridDim.x * kWarpsPerCta) {
    for (size_t e = lane; e < mm; e += 32) L[e] = LU[s * mm + e];
    for (int k = lane; k < m; k += 32) {
      xs[k] = b[(size_t)s * m + k];
      pv[k] = piv[(size_t)s * m + k];
    }
    __syncwarp();
    warp_lu_solve(L, m, pv, xs);
    for (int k = lane; k < m; k += 32) x[(size_t)s * m + k] = xs[k];
    __syncwarp();
  }
}

// FP32 triangular solves + FP64 residual refinement (r = b - A x, x += LU32^-1 r).
__global__ void solve32_kernel(int n, int m, const double *A, const float *LU, const int *piv, int refine,
                               const double *b, double *x)
{
  extern __shared__ __align__(16) unsigned char sm[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t mm = (size_t)m * m;
  const size_t per = mm / 2 + 2 * (size_t)m + 2;  // doubles per warp: fp32 LU, x (fp64), r (fp32 in fp64 slots)
  double *base = reinterpret_cast<double *>(sm) + (size_t)w * per;
  float *L = reinterpret_cast<float *>(base);
  double *xs = base + (mm + 1) / 2;
  float *rs = reinterpret_cast<float *>(xs + m);
  int *pv = reinterpret_cast<int *>(reinterpret_cast<double *>(sm) + (size_t)kWarpsPerCta * per) + w * m;
  for (int s = blockIdx.x * kWarpsPerCta + w; s < n; s += gridDim.x * kWarpsPerCta) {
    for (size_t e = lane; e < mm; e += 32) L[e] = LU[s * mm + e];
    for (int k = lane; k < m; k += 32) {
      rs[k] = (float)b[(size_t)s * m + k];
      pv[k] = piv[(size_t)s * m + k];
    }
    __syncwarp();
    warp_lu_solve(L, m, pv, rs);
    for (int k = lane; k < m; k += 32) xs[k] = (double)rs[k];
    __syncwarp();
    const double *As = A + s * mm;
    for (int it = 0; it < refine; ++it) {
      // residual in FP64, rows over lanes
      for (int i = lane; i < m; i += 32) {
        double r = b[(size_t)s * m + i];
        for (int j = 0; j < m; ++j) r = fma(-As[i + (size_t)j * m], xs[j], r);
        rs[i] = (float)r;
      }
      __syncwarp();
      warp_lu_solve(L, m, pv, rs);
      for (int k = lane; k < m; k += 32) xs[k] += (double)rs[k];
      __syncwarp();
    }
    for (int k = lane; k < m; k += 32) x[(size_t)s * m + k] = xs[k];
    __syncwarp();
  }
}

int grid_for(int n)
{
  int dev, nsm;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const long long need = ((long long)n + kWarpsPerCta - 1) / kWarpsPerCta;
  return (int)std::max<long long>(1, std::min<long long>(need, (long long)nsm * 8));
}

}  // namespace
}  // namespace sfgb

using namespace sfgb;

extern "C" {

int sf_newton_lu_batch(int n, int m, const double *J, const double *gamma_h, int precision, double *out_A,
                       void *out_lu, int *out_piv, int *out_info, void *stream)
{
  if (n < 0 || m < 1 || m > 80 || (n > 0 && (!J || !gamma_h || !out_lu || !out_piv))) {
    set_error("sf_newton_lu_batch: bad argument (1 <= m <= 80)");
    return SF_ERR_INVALID_ARGUMENT;
  }
  if (precision == 1 && !out_A) {
    set_error("sf_newton_lu_batch: precision 1 needs out_A for the refinement");
    return SF_ERR_INVALID_ARGUMENT;
  }
  if (n == 0) return SF_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t mm = (size_t)m * m;
  if (precision == 0) {
    const size_t smem = kWarpsPerCta * (mm * 8 + m * 4);
    try {
      ensure_dynamic_smem((const void *)lu64_kernel, smem);
    } catch (sf_error &e) {
      set_error(e.what());
      return e.code;
    }
    lu64_kernel<<<grid_for(n), 32 * kWarpsPerCta, smem, st>>>(n, m, J, gamma_h, out_A, (double *)out_lu, out_piv,
                                                              out_info);
  } else if (precision == 1) {
    const size_t smem = kWarpsPerCta * (mm * 4 + m * 4);
    try {
      ensure_dynamic_smem((const void *)lu32_kernel, smem);
    } catch (sf_error &e) {
      set_error(e.what());
      return e.code;
    }
    lu32_kernel<<<grid_for(n), 32 * kWarpsPerCta, smem, st>>>(n, m, J, gamma_h, out_A, (float *)out_lu, out_piv,
                                                              out_info);
  } else {
    set_error("sf_newton_lu_batch: precision must be 0 or 1");
    return SF_ERR_INVALID_ARGUMENT;
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(cudaGetErrorString(e));
    return SF_ERR_CUDA;
  }
  return SF_OK;
}

int sf_newton_solve_batch(int n, int m, const double *A, const void *lu, const int *piv, int precision, int refine,
                          const double *b, double *out_x, void *stream)
{
  if (n < 0 || m < 1 || m > 80 || (n > 0 && (!lu || !piv || !b || !out_x))) {
    set_error("sf_newton_solve_batch: bad argument");
    return SF_ERR_INVALID_ARGUMENT;
  }
  if (n == 0) return SF_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t mm = (size_t)m * m;
  if (precision == 0) {
    const size_t smem = kWarpsPerCta * ((mm + m) * 8 + m * 4);
    try {
      ensure_dynamic_smem((const void *)solve64_kernel, smem);
    } catch (sf_error &e) {
      set_error(e.what());
      return e.code;
    }
    solve64_kernel<<<grid_for(n), 32 * kWarpsPerCta, smem, st>>>(n, m, (const double *)lu, piv, b, out_x);
  } else if (precision == 1) {
    if (!A) {
      set_error("sf_newton_solve_batch: precision 1 needs A");
      return SF_ERR_INVALID_ARGUMENT;
    }
    const size_t per = mm / 2 + 2 * (size_t)m + 2;
    const size_t smem = kWarpsPerCta * (per * 8 + m * 4);
    try {
      ensure_dynamic_smem((const void *)solve32_kernel, smem);
    } catch (sf_error &e) {
      set_error(e.what());
      return e.code;
    }
    solve32_kernel<<<grid_for(n), 32 * kWarpsPerCta, smem, st>>>(n, m, A, (const float *)lu, piv, refine, b, out_x);
  } else {
    set_error("sf_newton_solve_batch: precision must be 0 or 1");
    return SF_ERR_INVALID_ARGUMENT;
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(cudaGetErrorString(e));
    return SF_ERR_CUDA;
  }
  return SF_OK;
}

}  // extern "C"
