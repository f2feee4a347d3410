// Largest real part of the eigenvalues of a small real nonsymmetric matrix, by one warp, in shared memory:
// Parlett-Reinsch balancing (diagonal similarity by powers of two, exact in floating point), Householder reduction
// to upper Hessenberg form, then the implicit double-shift (Francis) QR iteration with deflation on the active
// window only (eigenvalues, no Schur vectors). Published algorithms: B. N. Parlett and C. Reinsch, "Balancing a
// matrix for calculation of eigenvalues and eigenvectors", Numer. Math. 13 (1969); G. H. Golub and C. F. Van Loan,
// "Matrix Computations", sections 7.4-7.5 (Hessenberg reduction, Francis step, deflation, exceptional shifts).
//
// GB300 issues FP64 at a fixed cost per warp instruction whatever the number of active lanes, so the warp
// layout keeps lanes busy: column-parallel Hessenberg updates (no per-column reductions), reflectors in the
// tau form (one reciprocal) in the Hessenberg reduction, unit-scaled reflectors (one reciprocal square root) in
// the QR sweeps, and a lane-parallel deflation scan.
//
// Replaces the LAPACK dgeev call Griffon makes per flamelet Jacobian block for the pseudo-transient
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

// Both sums of two per-lane values in every lane, with five FP64 additions per lane instead of ten: the first
// exchange leaves the half-sums of a in lanes 0-15 and of b in lanes 16-31, and each half then reduces its own.
__device__ __forceinline__ void warp_sum_pair(double &a, double &b)
{
  const int lane = threadIdx.x & 31;
  const bool lo = lane < 16;
  double v = lo ? a : b;
  v += __shfl_xor_sync(0xffffffffu, lo ? b : a, 16);
  for (int o = 8; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  a = __shfl_sync(0xffffffffu, v, 0);
  b = __shfl_sync(0xffffffffu, v, 16);
}

__device__ __forceinline__ double warp_max_all(double v)
{
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// x * 2^k for fac = 2^k, on the integer pipe where that is exact: a normal x whose product stays normal gets k added to
// its exponent field, a zero is unchanged; anything else (subnormal, infinite, NaN, leaving the normal range) is
// multiplied as before.
__device__ __forceinline__ double scale_pow2(double x, int k, double fac)
{
  const long long b = __double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7ff);
  if (e == 0 && (b & 0x7fffffffffffffffLL) == 0) return x;
  if (e == 0 || e == 0x7ff || e + k <= 0 || e + k >= 0x7ff) return x * fac;
  return __longlong_as_double(b + ((long long)k << 52));
}

// Parlett-Reinsch balancing with radix 2 (scaling only): repeat until no row/column pair changes by more than
// 5%, at most `max_sweeps` sweeps. Column-major A, leading dimension n.
// GB300 issues FP64 at one warp instruction per 76 cycles per scheduler, so the scalings by powers of two (exact)
// run on the integer pipe: non-negative finite doubles order like their bit patterns, and a factor 4 or 1/4 on a
// normal value is a change of 2 in its exponent field. The results are those of the plain FP64 form bit for bit;
// values near the ends of the exponent range take the FP64 form.
__device__ void warp_balance(double *A, int n, int max_sweeps = 32)
{
  const int lane = threadIdx.x & 31;
  constexpr long long kExp1 = 1LL << 52;
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    bool changed = false;
    for (int i = 0; i < n; ++i) {
      double c = 0., r = 0.;
      for (int j = lane; j < n; j += 32)
        if (j != i) {
          c += fabs(A[j + i * n]);
          r += fabs(A[i + j * n]);
        }
      warp_sum_pair(c, r);
      // c, r >= 0: zero when the bit pattern is zero, not finite when the exponent field is all ones
      const long long cb = __double_as_longlong(c), rb = __double_as_longlong(r);
      const int ce = (int)(cb >> 52), re = (int)(rb >> 52);
      if (cb == 0 || rb == 0 || ce == 0x7ff || re == 0x7ff) continue;
      // the scaling f = 2^m: the smallest m >= 0 with c 4^m >= r / 2, else the m < 0 that brings c below 2 r
      int m = 0;
      const double s = c + r;
      if (ce > 4 && ce < 0x7f0 && re > 4 && re < 0x7f0) {
        long long cc = cb;
        const long long g1 = rb - kExp1, g2 = rb + kExp1;  // r / 2, 2 r
        for (int t = 0; t < 1100 && cc < g1; ++t) {
          cc += 2 * kExp1;
          ++m;
        }
        for (int t = 0; t < 1100 && cc >= g2; ++t) {
          cc -= 2 * kExp1;
          --m;
        }
        c = __longlong_as_double(cc);
      } else {
        double g = r * 0.5;
        for (int t = 0; t < 1100 && c < g; ++t) {
          c *= 4.;
          ++m;
        }
        g = r * 2.;
        for (int t = 0; t < 1100 && c >= g; ++t) {
          c *= 0.25;
          --m;
        }
      }
      const bool normal = m >= -1000 && m <= 1000;
      const double f = normal ? __longlong_as_double((long long)(1023 + m) << 52) : ldexp(1., m);
      const double fi = normal ? __longlong_as_double((long long)(1023 - m) << 52) : 1. / f;
      // (c + r) / f < 0.95 s, with (c + r) / f formed exactly on the exponent field where it stays normal
      const double t = c + r, lim = 0.95 * s;
      const int te = (int)(__double_as_longlong(t) >> 52);
      const bool fits = normal && te > 0 && te < 0x7ff && te - m > 0 && te - m < 0x7ff;
      const bool shrink = fits ? (__double_as_longlong(t) - (long long)m * kExp1) < __double_as_longlong(lim)
                               : (normal ? t * fi : t / f) < lim;
      if (shrink) {
        changed = true;
        for (int j = lane; j < n; j += 32) {
          if (normal) {
            A[i + j * n] = scale_pow2(A[i + j * n], -m, fi);
            A[j + i * n] = scale_pow2(A[j + i * n], m, f);
          } else {
            A[i + j * n] *= fi;
            A[j + i * n] *= f;
          }
        }
        __syncwarp();
      }
    }
    if (!changed) break;
  }
}

// Sufficient test that every eigenvalue of the n x n column-major A has real part below `cutoff`, by Gershgorin's
// theorem under the best diagonal scaling: if the comparison matrix M = diag(cutoff - a_ii) - |offdiag(A)| is a
// nonsingular M-matrix, some x > 0 has M x > 0, and then every Gershgorin disc of X^-1 A X (X = diag(x)) lies left
// of the cutoff. A Z-matrix is a nonsingular M-matrix iff its LU factorization without pivoting has positive
// pivots (all leading principal minors positive; A. Berman and R. J. Plemmons, "Nonnegative Matrices in the
// Mathematical Sciences", ch. 6). Each pivot must stay above 1e-10 of the diagonal entry it starts from, far above
// the rounding of the elimination, so a pass holds for the exact matrix. A is overwritten with M's partial
// factors; dg: n doubles of shared work. Lanes over rows (contiguous in column-major storage); a zero entry of
// the pivot row is skipped by the whole warp, which exploits the sparsity of chemistry Jacobians.
__device__ bool warp_hmatrix_below(double *A, int n, double cutoff, double *dg)
{
  const int lane = threadIdx.x & 31;
  bool ok = true;
  for (int e = lane; e < n * n; e += 32) {
    const int c = e / n, r = e - c * n;
    const double a = A[e];
    if (r == c) {
      const double m = cutoff - a;
      A[e] = m;
      dg[r] = m;
      ok = ok && m > 0.;  // false for NaN too
    } else {
      A[e] = -fabs(a);
    }
  }
  if (!__all_sync(0xffffffffu, ok)) return false;
  __syncwarp();
  for (int k = 0; k < n; ++k) {
    const double p = A[k + k * n];
    if (!(p > 1e-10 * dg[k])) return false;  // the same value in every lane: a warp-uniform exit
    const double ip = 1. / p;
    for (int i = k + 1 + lane; i < n; i += 32) {
      const double l = A[i + k * n] * ip;
      for (int j = k + 1; j < n; ++j) {
        const double mkj = A[k + j * n];
        if (mkj != 0.) A[i + j * n] -= l * mkj;
      }
    }
    __syncwarp();
  }
  return true;
}

// The same test for the unreduced upper Hessenberg block H[lo..hi, lo..hi] of a QR iterate: every eigenvalue of
// the block has real part below `cutoff` if its comparison matrix (diag(cutoff - h_ii), -|h_ij| elsewhere, zero
// below the subdiagonal) is a nonsingular M-matrix. A Hessenberg LU without pivoting eliminates one row per
// column, so the test keeps one row vector (r: hi + 1 doubles of shared work, lanes over columns) and costs
// O(m^2) for a block of m rows, against O(m^2) per double-shift QR sweep over the block.
__device__ bool warp_hess_hmatrix_below(const double *H, int n, int lo, int hi, double cutoff, double *r)
{
  const int lane = threadIdx.x & 31;
  for (int j = lo + lane; j <= hi; j += 32) r[j] = j == lo ? cutoff - H[lo + lo * n] : -fabs(H[lo + j * n]);
  __syncwarp();
  for (int k = lo; k <= hi; ++k) {
    const double dgk = cutoff - H[k + k * n];
    const double p = r[k];
    if (!(dgk > 0.) || !(p > 1e-10 * dgk)) return false;  // the same values in every lane: a warp-uniform exit
    if (k == hi) break;
    const double l = -fabs(H[(k + 1) + k * n]) / p;  // multiplier of row k + 1 (its only entry below the pivot)
    __syncwarp();
    for (int j = k + 1 + lane; j <= hi; j += 32) {
      const double m = j == k + 1 ? cutoff - H[(k + 1) + (k + 1) * n] : -fabs(H[(k + 1) + j * n]);
      r[j] = m - l * r[j];
    }
    __syncwarp();
  }
  return true;
}

// Upper bound of the real parts of the eigenvalues by Gershgorin's theorem applied to rows and to columns.
__device__ double warp_gershgorin_bound(const double *A, int n)
{
  const int lane = threadIdx.x & 31;
  double br = -INFINITY, bc = -INFINITY;
  for (int i = lane; i < n; i += 32) {
    double rs = 0., cs = 0.;
    for (int j = 0; j < n; ++j)
      if (j != i) {
        rs += fabs(A[i + j * n]);
        cs += fabs(A[j + i * n]);
      }
    br = fmax(br, A[i + i * n] + rs);
    bc = fmax(bc, A[i + i * n] + cs);
  }
  return fmin(warp_max_all(br), warp_max_all(bc));
}

// Reduce the n x n column-major A to upper Hessenberg form in place. v: n doubles, s: n doubles of shared work.
__device__ void warp_hessenberg(double *A, int n, double *v, double *s)
{
  const int lane = threadIdx.x & 31;
  for (int k = 0; k + 2 < n; ++k) {
    double ss = 0.;
    for (int i = k + 2 + lane; i < n; i += 32) ss += A[i + k * n] * A[i + k * n];
    ss = warp_sum_all(ss);
    if (ss == 0.) continue;  // already zero below the subdiagonal
    const double x0 = A[(k + 1) + k * n];
    const double nrm = sqrt(x0 * x0 + ss);
    const double alpha = -copysign(nrm, x0);
    const double tau = 1. / (nrm * (nrm + fabs(x0)));  // 2 / (u^T u) for u = x - alpha e1
    for (int i = k + 1 + lane; i < n; i += 32) v[i] = (i == k + 1) ? x0 - alpha : A[i + k * n];
    __syncwarp();
    // left: A[k+1:, j] -= tau u (u^T A[k+1:, j]), lanes over columns j > k; column k becomes alpha e1
    for (int j = k + 1 + lane; j < n; j += 32) {
      double d = 0.;
      for (int i = k + 1; i < n; ++i) d += v[i] * A[i + j * n];
      d *= tau;
      for (int i = k + 1; i < n; ++i) A[i + j * n] -= d * v[i];
    }
    if (lane == 0) A[(k + 1) + k * n] = alpha;
    for (int i = k + 2 + lane; i < n; i += 32) A[i + k * n] = 0.;
    __syncwarp();
    // right: A[i, k+1:] -= tau (A[i, k+1:] u) u^T, lanes over rows
    for (int i = lane; i < n; i += 32) {
      double d = 0.;
      for (int l = k + 1; l < n; ++l) d += A[i + l * n] * v[l];
      d *= tau;
      for (int l = k + 1; l < n; ++l) A[i + l * n] -= d * v[l];
    }
    __syncwarp();
  }
  (void)s;
}

// Householder reflector P = I - v v^T mapping (x, y[, z]) to a multiple of e1: v = u / sqrt(beta) with
// u = (x + sign(x) ||.||, y, z) and beta = u^T u / 2 = ||.|| (||.|| + |x|), so |v|^2 = 2. Normalizing u by one
// reciprocal square root (instead of a square root and a reciprocal for tau = 1/beta) also drops the tau
// multiplication from every application. Returns false when (x, y, z) is zero (P = I).
template <int NR>
__device__ __forceinline__ bool house3(double x, double y, double z, double *v)
{
  const double nn = x * x + y * y + (NR == 3 ? z * z : 0.);
  if (nn == 0.) return false;
  const double nrm = sqrt(nn);
  const double r = rsqrt(nrm * (nrm + fabs(x)));
  v[0] = (x + copysign(nrm, x)) * r;
  v[1] = y * r;
  v[2] = NR == 3 ? z * r : 0.;
  return true;
}

// Apply P = I - v v^T (v of length NR <= 3) to rows r0..r0+NR-1 of H over columns c0..c1, and to columns
// r0..r0+NR-1 over rows c2..c3.
template <int NR>
__device__ __forceinline__ void apply_reflector(double *H, int n, const double *v, int r0, int c0, int c1, int c2,
                                                int c3)
{
  const int lane = threadIdx.x & 31;
  for (int j = c0 + lane; j <= c1; j += 32) {
    double s = v[0] * H[r0 + j * n] + v[1] * H[(r0 + 1) + j * n];
    if (NR == 3) s += v[2] * H[(r0 + 2) + j * n];
    H[r0 + j * n] -= s * v[0];
    H[(r0 + 1) + j * n] -= s * v[1];
    if (NR == 3) H[(r0 + 2) + j * n] -= s * v[2];
  }
  __syncwarp();
  for (int i = c2 + lane; i <= c3; i += 32) {
    double s = H[i + r0 * n] * v[0] + H[i + (r0 + 1) * n] * v[1];
    if (NR == 3) s += H[i + (r0 + 2) * n] * v[2];
    H[i + r0 * n] -= s * v[0];
    H[i + (r0 + 1) * n] -= s * v[1];
    if (NR == 3) H[i + (r0 + 2) * n] -= s * v[2];
  }
  __syncwarp();
}

// Start of the unreduced block ending at row hi: the largest lo <= hi with H[lo, lo-1] negligible (set to zero), or
// 0. Lanes test the subdiagonals in parallel, 32 rows at a time from the bottom.
__device__ __forceinline__ int warp_find_lo(double *H, int n, int hi)
{
  const int lane = threadIdx.x & 31;
  for (int top = hi; top > 0; top -= 32) {
    const int r = top - lane;  // candidate row, r >= 1
    bool neg = false;
    if (r >= 1) {
      const double sub = fabs(H[r + (r - 1) * n]);
      double s = fabs(H[(r - 1) + (r - 1) * n]) + fabs(H[r + r * n]);
      if (s == 0.) s = 1.;
      neg = sub <= 2.220446049250313e-16 * s;
    }
    const unsigned m = __ballot_sync(0xffffffffu, neg);
    if (m) {
      const int first = __ffs(m) - 1;  // lowest lane = largest row
      const int lo = top - first;
      if (lane == 0) H[lo + (lo - 1) * n] = 0.;
      __syncwarp();
      return lo;
    }
  }
  return 0;
}

// Largest real part of the eigenvalues of the n x n matrix A (destroyed; A is balanced first). work: 2n doubles
// of shared memory. If cutoff is given and the balanced matrix's Gershgorin bound is <= cutoff, the function
// returns that bound instead of running QR (every eigenvalue is then known to have real part <= cutoff).
// With a cutoff the QR iteration also stops early: after every second sweep on an unreduced block, the block is
// tested with warp_hess_hmatrix_below, and a block whose eigenvalues are all proven left of the cutoff is set aside
// without computing them. The returned maximum then covers only the eigenvalues computed, so it is exact whenever
// it exceeds the cutoff, and at most the cutoff otherwise, which is all max(lambda_max - cutoff, 0) needs.
// Returns false if the QR iteration did not converge within its budget (the largest real part of the diagonal
// found so far is returned then).
__device__ bool warp_max_real_eig(double *A, int n, double *work, double *out_max, double cutoff = -INFINITY)
{
  warp_balance(A, n);
  __syncwarp();
  const double gb = warp_gershgorin_bound(A, n);
  if (gb <= cutoff) {
    *out_max = gb;
    return true;
  }
  warp_hessenberg(A, n, work, work + n);
  double *H = A;
  double vmax = -INFINITY;
  int hi = n - 1, iter = 0, total = 0;
  const int budget = 40 * n;
  bool ok = true;
  double u[3];
  while (hi >= 0) {
    if (total > budget) {
      ok = false;
      for (int i = 0; i <= hi; ++i) vmax = fmax(vmax, H[i + i * n]);
      break;
    }
    const int lo = hi > 0 ? warp_find_lo(H, n, hi) : 0;
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
      vmax = fmax(vmax, disc >= 0. ? tr + sqrt(disc) : tr);
      hi -= 2;
      iter = 0;
      continue;
    }
    // the early exit: a block whose eigenvalues all lie left of the cutoff is done
    if (cutoff > -INFINITY && (iter & 1) && warp_hess_hmatrix_below(H, n, lo, hi, cutoff, work)) {
      hi = lo - 1;
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
      if (house3<3>(x, y, z, u)) {
        const int c0 = k < lo ? lo : k;
        const int r1 = k + 4 < hi ? k + 4 : hi;
        apply_reflector<3>(H, n, u, k + 1, c0, hi, lo, r1);
      }
      x = H[(k + 2) + (k + 1) * n];
      y = H[(k + 3) + (k + 1) * n];
      if (k < hi - 3) z = H[(k + 4) + (k + 1) * n];
    }
    if (house3<2>(x, y, 0., u)) apply_reflector<2>(H, n, u, hi - 1, hi - 2, hi, lo, hi);
  }
  *out_max = vmax;
  return ok;
}

}  // namespace sfgb
