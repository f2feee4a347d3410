// Eigenvalues of a small real nonsymmetric matrix by one warp, in shared memory: Householder reduction to upper
// Hessenberg form followed by the implicit double-shift (Francis) QR iteration with deflation. Only eigenvalues
// are computed (the active block is updated, not the full Schur form). This is the published algorithm of
// Golub & Van Loan, "Matrix Computations", sections 7.4-7.5 (Householder Hessenberg reduction, Francis QR step,
// deflation by negligible subdiagonal entries, exceptional shifts after 10 and 20 stalled iterations), written for
// a warp: reflector applications run over lanes.
//
// It replaces the LAPACK dgeev call Griffon makes per flamelet Jacobian block for the pseudo-transient
// continuation time step (flamelet_kernels.cpp:1329-1341).
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace sfgb {

__device__ __forceinline__ double warp_sum_all(double v)
{
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Reduce the n x n column-major matrix A (leading dimension n) to upper Hessenberg form in place.
// v: n doubles of shared work space.
__device__ void warp_hessenberg(double *A, int n, double *v)
{
  const int lane = threadIdx.x & 31;
  for (int k = 0; k + 2 < n; ++k) {
    // Householder vector for x = A[k+1:n, k]
    double ss = 0.;
    for (int i = k + 2 + lane; i < n; i += 32) ss += A[i + k * n] * A[i + k * n];
    ss = warp_sum_all(ss);
    const double x0 = A[(k + 1) + k * n];
    if (ss == 0.) continue;  // already in Hessenberg form below the subdiagonal
    const double alpha = -copysign(sqrt(x0 * x0 + ss), x0);
    // v = x - alpha e1, beta = 2 / (v^T v)
    for (int i = k + 1 + lane; i < n; i += 32) v[i] = (i == k + 1) ? x0 - alpha : A[i + k * n];
    __syncwarp();
    const double vtv = (x0 - alpha) * (x0 - alpha) + ss;
    const double beta = 2. / vtv;
    // left: A[k+1:, j] -= beta v (v^T A[k+1:, j]) for j >= k
    for (int j = k; j < n; ++j) {
      double s = 0.;
      for (int i = k + 1 + lane; i < n; i += 32) s += v[i] * A[i + j * n];
      s = warp_sum_all(s) * beta;
      for (int i = k + 1 + lane; i < n; i += 32) A[i + j * n] -= s * v[i];
      __syncwarp();
    }
    // right: A[i, k+1:] -= beta (A[i, k+1:] v) v^T for all rows i
    for (int i = lane; i < n; i += 32) {
      double s = 0.;
      for (int l = k + 1; l < n; ++l) s += A[i + l * n] * v[l];
      s *= beta;
      for (int l = k + 1; l < n; ++l) A[i + l * n] -= s * v[l];
    }
    __syncwarp();
    for (int i = k + 2 + lane; i < n; i += 32) A[i + k * n] = 0.;
    __syncwarp();
  }
}

// Apply the reflector P = I - beta v v^T (v of length nr <= 3, v[0] = 1) to rows r0..r0+nr-1 of H over columns
// c0..c1, and to columns r0..r0+nr-1 over rows c2..c3.
__device__ __forceinline__ void apply_reflector(double *H, int n, const double *v, int nr, double beta, int r0, int c0,
                                                int c1, int c2, int c3)
{
  const int lane = threadIdx.x & 31;
  for (int j = c0 + lane; j <= c1; j += 32) {
    double s = 0.;
    for (int a = 0; a < nr; ++a) s += v[a] * H[(r0 + a) + j * n];
    s *= beta;
    for (int a = 0; a < nr; ++a) H[(r0 + a) + j * n] -= s * v[a];
  }
  __syncwarp();
  for (int i = c2 + lane; i <= c3; i += 32) {
    double s = 0.;
    for (int a = 0; a < nr; ++a) s += H[i + (r0 + a) * n] * v[a];
    s *= beta;
    for (int a = 0; a < nr; ++a) H[i + (r0 + a) * n] -= s * v[a];
  }
  __syncwarp();
}

// Householder reflector mapping (x, y[, z]) to a multiple of e1: v = [1, y/(x-a), z/(x-a)], beta.
__device__ __forceinline__ int house3(double x, double y, double z, int nr, double *v, double *beta)
{
  const double nrm = sqrt(x * x + y * y + (nr == 3 ? z * z : 0.));
  if (nrm == 0.) {
    *beta = 0.;
    v[0] = 1.;
    v[1] = 0.;
    v[2] = 0.;
    return 0;
  }
  const double a = -copysign(nrm, x);
  const double d = x - a;
  v[0] = 1.;
  v[1] = y / d;
  v[2] = nr == 3 ? z / d : 0.;
  const double vv = 1. + v[1] * v[1] + v[2] * v[2];
  *beta = 2. / vv;
  return 1;
}

// Largest real part of the eigenvalues of the n x n matrix A (destroyed). Returns false if the QR iteration did not
// converge within its iteration budget (the largest real part of the diagonal found so far is returned then).
__device__ bool warp_max_real_eig(double *A, int n, double *work, double *out_max)
{
  warp_hessenberg(A, n, work);
  double *H = A;
  double vmax = -INFINITY;
  int hi = n - 1, iter = 0, total = 0;
  const int budget = 40 * n;
  bool ok = true;
  double v[3];
  while (hi >= 0) {
    if (total > budget) {
      ok = false;
      for (int i = 0; i <= hi; ++i) vmax = fmax(vmax, H[i + i * n]);
      break;
    }
    // find the start lo of the unreduced block ending at hi
    int lo = hi;
    while (lo > 0) {
      const double sub = fabs(H[lo + (lo - 1) * n]);
      double s = fabs(H[(lo - 1) + (lo - 1) * n]) + fabs(H[lo + lo * n]);
      if (s == 0.) s = 1.;
      if (sub <= 2.220446049250313e-16 * s) {
        H[lo + (lo - 1) * n] = 0.;
        break;
      }
      --lo;
    }
    if (lo == hi) {
      vmax = fmax(vmax, H[hi + hi * n]);
      --hi;
      iter = 0;
      continue;
    }
    if (lo == hi - 1) {
      const double a = H[(hi - 1) + (hi - 1) * n], b = H[(hi - 1) + hi * n];
      const double c = H[hi + (hi - 1) * n], d = H[hi + hi * n];
      const double tr = 0.5 * (a + d), det = a * d - b * c;
      const double disc = tr * tr - det;
      if (disc >= 0.) {
        const double r = sqrt(disc);
        vmax = fmax(vmax, tr + r);
      } else {
        vmax = fmax(vmax, tr);
      }
      hi -= 2;
      iter = 0;
      continue;
    }
    ++iter;
    ++total;
    // double shift from the trailing 2x2 block (exceptional shift after 10 and 20 stalled iterations)
    double s, t;
    if (iter == 10 || iter == 20) {
      const double w = fabs(H[hi + (hi - 1) * n]) + fabs(H[(hi - 1) + (hi - 2) * n]);
      s = 1.5 * w;
      t = w * w;
    } else {
      const int mm = hi - 1;
      s = H[mm + mm * n] + H[hi + hi * n];
      t = H[mm + mm * n] * H[hi + hi * n] - H[mm + hi * n] * H[hi + mm * n];
    }
    double x = H[lo + lo * n] * H[lo + lo * n] + H[lo + (lo + 1) * n] * H[(lo + 1) + lo * n] - s * H[lo + lo * n] + t;
    double y = H[(lo + 1) + lo * n] * (H[lo + lo * n] + H[(lo + 1) + (lo + 1) * n] - s);
    double z = H[(lo + 1) + lo * n] * H[(lo + 2) + (lo + 1) * n];
    for (int k = lo - 1; k <= hi - 3; ++k) {
      double beta;
      house3(x, y, z, 3, v, &beta);
      if (beta != 0.) {
        const int c0 = k < lo ? lo : k;
        const int r1 = k + 4 < hi ? k + 4 : hi;
        apply_reflector(H, n, v, 3, beta, k + 1, c0, hi, lo, r1);
      }
      x = H[(k + 2) + (k + 1) * n];
      y = H[(k + 3) + (k + 1) * n];
      if (k < hi - 3) z = H[(k + 4) + (k + 1) * n];
    }
    double beta;
    house3(x, y, 0., 2, v, &beta);
    if (beta != 0.) apply_reflector(H, n, v, 2, beta, hi - 1, hi - 2, hi, lo, hi);
  }
  *out_max = vmax;
  return ok;
}

}  // namespace sfgb
