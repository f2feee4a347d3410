// Device building blocks of the Griffon hot path on sm_103a.
//
// Execution model: one *state group* of G lanes (G = 8, 16 or 32) evaluates one thermochemical state at a time.
// Lanes split species (thermodynamics, gathers by species) and reactions (rate evaluation), and a static gather
// program assembles Jacobian entries with one FP64 FMA per item. The packed mechanism is copied into shared
// memory once per CTA with a bulk-async (TMA) copy; every state group keeps its own scratch area in shared memory.
// Reference formulas: src/spitfire/griffon/src/thermodynamics_kernels.cpp, chemistry_kernels.cpp,
// rates_sensitivities_exact.cpp (file:line in comments below).
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "exp_table.h"
#include "sf_mech.h"

namespace sfgb {

// -------------------------------------------------------------------------------------------- error reporting
// Device-side error word (one int per mechanism, allocated with it): kernels never trap; a failed bounded wait or
// an invalid input records a code there and the kernel returns. sf_device_status() (host) reads and clears it.
enum { DEVERR_BULK_TIMEOUT = 1, DEVERR_BAD_ARG = 2, DEVERR_WAIT_TIMEOUT = 3 };

__device__ __forceinline__ void report_error(int *status, int code)
{
  if (status) atomicCAS(status, 0, code);
}

// --------------------------------------------------------------------------------- bulk copy into shared memory
__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Copy `bytes` (multiple of 16, both addresses 16-byte aligned) from global to shared memory through the TMA
// engine (cp.async.bulk) and wait for it on an mbarrier. The wait is bounded: on timeout the error word is set,
// a second bounded wait gives the copy a chance to land, and the function reports failure.
__device__ inline bool stage_to_smem(void *dst, const void *src, uint32_t bytes, uint64_t *bar, int *status)
{
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
    constexpr uint32_t kChunk = 16384;
    for (uint32_t off = 0; off < bytes; off += kChunk) {
      const uint32_t n = bytes - off < kChunk ? bytes - off : kChunk;
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
              smem_addr((char *)dst + off)),
          "l"((const char *)src + off), "r"(n), "r"(smem_addr(bar))
          : "memory");
    }
  }
  bool done = false;
  for (int it = 0; it < (1 << 22) && !done; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(0)
        : "memory");
    done = ok != 0;
  }
  if (!done) {
    report_error(status, DEVERR_BULK_TIMEOUT);
    for (int it = 0; it < (1 << 22) && !done; ++it) {
      uint32_t ok;
      asm volatile(
          "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
          : "=r"(ok)
          : "r"(smem_addr(bar)), "r"(0)
          : "memory");
      done = ok != 0;
    }
  }
  __syncthreads();
  return done;
}

// ----------------------------------------------------------------------------------------------- state groups
template <int G>
struct Group {
  int lane;       // 0..G-1
  unsigned mask;  // lanes of this group within the warp
  __device__ __forceinline__ Group()
  {
    const int wl = threadIdx.x & 31;
    lane = wl & (G - 1);
    mask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (wl & ~(G - 1)));
  }
  __device__ __forceinline__ void sync() const { __syncwarp(mask); }
  __device__ __forceinline__ double sum(double v) const
  {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o, G);
    return v;
  }
};

struct Blob {
  const double *d;
  const int *i;
};

// Scratch of one state interleaved with the states of the other 31 lanes of its warp (thread-per-state kernels):
// element i of this lane's state lives at p[32 i], so the lanes of a warp touch one contiguous 256-byte row.
// The state-group kernels use a plain double * into their shared-memory area instead; the device code below is
// written for either.
struct ScrStrided {
  double *p;  // base + lane
  __device__ __forceinline__ double &operator[](int i) const { return p[(size_t)i << 5]; }
  __device__ __forceinline__ ScrStrided operator+(int o) const { return ScrStrided{p + ((size_t)o << 5)}; }
};

__device__ __forceinline__ Blob blob_at(const DevMech &m, const void *base)
{
  Blob b;
  b.d = (const double *)base;
  b.i = (const int *)((const char *)base + (size_t)m.blob_doubles * 8);
  return b;
}

// ----------------------------------------------------------------------------------------- thermodynamics
// One species at temperature T: cp (clamped outside [Tmin, Tmax]), h (linear extrapolation outside), dcp/dT
// (zero outside), Gibbs energy g and B = d(g/RT)/dT-like term of the reverse-rate sensitivity
// (thermodynamics_kernels.cpp:45-131, 183-260, 262-351; chemistry_kernels.cpp:56-97;
//  rates_sensitivities_exact.cpp:83-124).
struct SpeciesThermo {
  double cp, h, dcp, g, dB;
};

__device__ __forceinline__ SpeciesThermo species_thermo(const DevMech &m, Blob b, int k, double T, double logT,
                                                        double invT, bool want_sens)
{
  SpeciesThermo s;
  const double *c = b.d + m.d_nasa + 15 * k;
  const double invmw = b.d[m.d_invmw + k];
  if (m.all_nasa7 || b.i[m.i_thermo + k] == 2) {
    const double tmin = b.d[m.d_tmin + k], tmax = b.d[m.d_tmax + k];
    // polynomial for g and dB: chosen by Tmid only
    const int gb = (T <= c[0]) ? 8 : 1;
    const double *a = c + gb;
    const double a6 = (T <= c[0]) ? c[13] : c[6];
    const double a7 = (T <= c[0]) ? c[14] : c[7];
    s.g = a6 + T * (a[0] - a7 - a[0] * logT - T * (a[1] + T * (a[2] + T * (a[3] + T * a[4]))));
    // cp / h / dcp on the clamped temperature
    const double tt = fmin(fmax(T, tmin), tmax);
    const bool inside = (T >= tmin) && (T <= tmax);
    const int hb = (tt <= c[0]) ? 8 : 1;
    const double *p = c + hb;
    const double p6 = (tt <= c[0]) ? c[13] : c[6];
    const double cpm = p[0] + tt * (2. * p[1] + tt * (6. * p[2] + tt * (12. * p[3] + 20. * tt * p[4])));
    s.cp = invmw * cpm;
    const double hm = p6 + tt * (p[0] + tt * (p[1] + tt * (2. * p[2] + tt * (3. * p[3] + tt * 4. * p[4]))));
    s.h = invmw * (inside ? hm : hm + cpm * (T - tt));
    if (want_sens) {
      s.dcp = inside ? invmw * (2. * p[1] + tt * (12. * p[2] + tt * (36. * p[3] + 80. * tt * p[4]))) : 0.;
      s.dB = m.invRu * ((a[0] - m.Ru) * invT + a[1] + T * (2 * a[2] + T * (3 * a[3] + T * 4 * a[4])) + a6 * invT * invT);
    } else {
      s.dcp = 0.;
      s.dB = 0.;
    }
  } else {
    // constant cp: c = [T0, h0, s0, cp, log T0] (thermodynamics_kernels.cpp:60-63, chemistry_kernels.cpp:88-89)
    s.cp = invmw * c[3];
    s.h = invmw * (c[1] + c[3] * (T - c[0]));
    s.g = c[1] + c[3] * (T - c[0]) - T * (c[2] + c[3] * (logT - c[4]));
    s.dcp = 0.;
    s.dB = want_sens ? invT * (b.d[m.d_mw + k] * m.invRu * (c[3] - invT * (c[3] * c[0] - c[1])) - 1) : 0.;
  }
  return s;
}

__device__ __forceinline__ double ipow(double x, int n)
{
  double r = 1.;
  for (int i = 0; i < n; ++i) r *= x;
  return r;
}

// ------------------------------------------------------------------------------- table-driven exponential
// e^x by Tang's table-driven method (P. T. P. Tang, "Table-driven implementation of the exponential function in
// IEEE floating-point arithmetic", ACM TOMS 15(2), 1989), written for FP64 throughput:
//   x = (64 m + j) ln2/64 + r, |r| <= ln2/128: N = 64 m + j is the nearest integer to x 64/ln2 (one FMA against
//   1.5 2^52, whose low word is then N), and r = (x - N L1) - N L2 with L1 + L2 = ln2/64 (the first FMA is exact:
//   x and N L1 are multiples of the ulp of L1, and |r| < 2^-7);
//   e^r - 1 = p(r), its Taylor polynomial of degree 6 (truncation below 3e-20 on |r| <= ln2/128);
//   e^x = 2^m (T_j + T_j p), T_j = 2^(j/64) as a head and a tail (the blob's table, 16-byte pairs), the power of two
//   applied to the exponent field while the result stays normal (|x| < 708), else by two exact factors.
// Against a 113-bit reference on 2M arguments over the whole range: at most 0.51 ulp for normal results (CUDA's exp:
// 0.86-0.88), 99.8 % correctly rounded; about 11.7 warp FP64 instructions per call against 15.0 for CUDA's exp
// (throughput loops on a GB300). NaN in, NaN out; beyond the range, 0 or +inf.
__device__ __forceinline__ double exp_parts(double x, double &r, int &N)
{
  const double tm = fma(x, kExpInvL, 0x1.8p52);
  N = __double2loint(tm);
  const double Nd = tm - 0x1.8p52;
  r = fma(-Nd, kExpL2, fma(-Nd, kExpL1, x));
  return Nd;
}

__device__ __forceinline__ double exp_finish(double x, double y, int N)
{
  const long long ax = __double_as_longlong(x) & 0x7fffffffffffffffll;
  if (ax < 0x4086200000000000ll)  // |x| < 708: the result is normal
    return __longlong_as_double(__double_as_longlong(y) + (long long)(N >> 6) * (1ll << 52));
  if (x != x) return x;
  if (x > 709.8) return __longlong_as_double(0x7ff0000000000000ll);
  if (x < -745.2) return 0.;
  const int m = N >> 6, m1 = m / 2, m2 = m - m1;  // both factors normal
  return y * __longlong_as_double((long long)(1023 + m1) << 52) * __longlong_as_double((long long)(1023 + m2) << 52);
}

__device__ __forceinline__ double tab_exp(double x, const double *tab)
{
  double r;
  int N;
  exp_parts(x, r, N);
  double q = fma(r, 1. / 720., 1. / 120.);
  q = fma(r, q, 1. / 24.);
  q = fma(r, q, 1. / 6.);
  q = fma(r, q, 0.5);
  const double p = fma(q, r * r, r);
  const double2 t = reinterpret_cast<const double2 *>(tab)[N & 63];
  return exp_finish(x, t.x + fma(t.x, p, t.y), N);
}

// exp(-g/RT) of one species as m 2^k, formed once per state so that the equilibrium factor of every reversible
// reaction, exp(-sum_i nu_i g_i/RT), becomes a product of mantissas and an exact power-of-two scaling instead of one
// exponential per reaction. With x = -g/RT = (64 k + j) ln2/64 + r (the reduction of tab_exp):
//   m = 2^(j/64) e^r in [1, 2) (to rounding), and the reciprocal mantissa 2^(-j/64) e^-r = m^-1 (the factor of a
//   product: every m^-1 2^-k is e^-x), from the same reduction: 2^(-j/64) = T_(64-j) / 2 for j > 0, and e^r, e^-r
//   from the even and odd parts of the polynomial, without a division.
// The power of two stays an integer (k = N >> 6), so any |x| below 2^31 ln2/64 = 2.3e7, where N fits an int, is
// represented exactly; g/RT of a species is at most a few thousand even at 10 K.
template <class S>
__device__ __forceinline__ void store_gibbs_factor(S scr, const ScratchLayout &L, int i, double gRT, const double *tab)
{
  const double x = -gRT;
  double r;
  int N;
  exp_parts(x, r, N);
  const double r2 = r * r;
  const double E = r2 * fma(r2, fma(r2, 1. / 720., 1. / 24.), 0.5);          // r^2/2 + r^4/24 + r^6/720
  const double O = fma(r * r2, fma(r2, 1. / 120., 1. / 6.), r);              // r + r^3/6 + r^5/120
  const int j = N & 63;
  const double2 t = reinterpret_cast<const double2 *>(tab)[j];
  const double2 u = reinterpret_cast<const double2 *>(tab)[(64 - j) & 63];
  const double ui = j ? 0.5 : 1.;                                             // exact
  const double ep = O + E, em = E - O;                                        // e^r - 1, e^-r - 1
  scr[L.gm + i] = t.x + fma(t.x, ep, t.y);
  scr[L.gmi + i] = ui * (u.x + fma(u.x, em, u.y));
  scr[L.gk + i] = __longlong_as_double((long long)(N >> 6));
}

// x 2^K, exact unless the result leaves the normal range; |K| beyond 2044 already takes any factor of a rate
// expression to 0 or infinity.
__device__ __forceinline__ double scale_pow2(double x, long long K)
{
  const int k = (int)(K < -2044 ? -2044 : (K > 2046 ? 2046 : K));
  const int k1 = k / 2, k2 = k - k1;  // both within [-1022, 1023]
  const double f1 = __longlong_as_double((long long)(k1 + 1023) << 52);
  const double f2 = __longlong_as_double((long long)(k2 + 1023) << 52);
  return x * f1 * f2;
}

// A small integer (a stoichiometric coefficient or a sum of them) as a double: from the blob's table when within
// -32..31 (a shared-memory load), else converted.
__device__ __forceinline__ double small_int(const double *table, int k)
{
  return (unsigned)(k + 32) < 64u ? table[k + 32] : (double)k;
}

// ------------------------------------------------------------------------------------------ reaction phase
// Per-state quantities every reaction needs.
struct StateCtx {
  double T, logT, invT, rho, invRho, mmw, invM, ct;
  double port, invport;  // p_ref / (R T) and its reciprocal
  int option;  // rates-sensitivity option: 0 / 2 exact, 1 without third-body/falloff derivatives
};

// Product of C_j^nu_j over a reactant/product list, with the factor of list position `at` differentiated
// with respect to Y of that species (nu * rho/M * C^(nu-1)); at < 0: no differentiation.
template <class SC>
__device__ __forceinline__ double mass_action(const int *lst, int n, const SC &C, const double *invmw_d,
                                              double rho, int at)
{
  double v = 1.;
  for (int j = 0; j < n; ++j) {
    const int e = lst[j];
    const int s = e & 0xFFFF, nu = e >> 16;
    const double c = C[s];
    if (j == at)
      v *= nu * rho * invmw_d[s] * ipow(c, nu - 1);
    else
      v *= ipow(c, nu);
  }
  return v;
}

// Mass-action factors of a reactant or product list of at most three entries, formed once per reaction: the
// product P = prod_i C_i^nu_i and, per list position j, g_j = d P / d Y_j / rho = nu_j / M_j C_j^(nu_j - 1)
// prod_{i != j} C_i^nu_i (C_i = rho Y_i / M_i). The Jacobian slots of the reaction then cost one multiply each.
struct MassAction3 {
  double P, g0, g1, g2;
  __device__ __forceinline__ double g(int j) const { return j == 0 ? g0 : (j == 1 ? g1 : g2); }
};

template <class SC>
__device__ __forceinline__ MassAction3 mass_action3(const int *lst, int n, const SC &C, const double *invmw_d)
{
  double p[3], d[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    p[j] = 1.;
    d[j] = 0.;
    if (j < n) {
      const int e = lst[j];
      const int sp = e & 0xFFFF, nu = e >> 16;
      const double c = C[sp];
      const double im = invmw_d[sp];
      if (nu == 1) {
        p[j] = c;
        d[j] = im;
      } else {
        const double cm = ipow(c, nu - 1);
        p[j] = cm * c;
        d[j] = (double)nu * im * cm;
      }
    }
  }
  MassAction3 o;
  if (n <= 1) {
    o.P = p[0];
    o.g0 = d[0];
    o.g1 = o.g2 = 0.;
  } else if (n == 2) {
    o.P = p[0] * p[1];
    o.g0 = d[0] * p[1];
    o.g1 = p[0] * d[1];
    o.g2 = 0.;
  } else {
    const double t = p[0] * p[1];
    o.P = t * p[2];
    o.g0 = d[0] * (p[1] * p[2]);
    o.g1 = d[1] * (p[0] * p[2]);
    o.g2 = d[2] * t;
  }
  return o;
}

// Special-order rate law (chemistry_kernels.cpp:316-325) and its Y derivative for order-list position `at`
// (rates_sensitivities_exact.cpp:177-261).
template <class SC>
__device__ __forceinline__ double special_orders(const DevMech &m, Blob b, int r, const SC &C, double rho, int at,
                                                 bool last_closure)
{
  const int o0 = b.i[m.i_ord_off + r], o1 = b.i[m.i_ord_off + r + 1];
  const double *invmw_d = b.d + m.d_invmw;
  double v = 1.;
  for (int j = o0; j < o1; ++j) {
    const int e = b.i[m.i_ord + j];
    const int s = e & 0xFFFF;
    const bool nz = (e >> 16) != 0;
    const double ord = b.d[m.d_ord + j];
    const double c = C[s];
    if (j - o0 == at) {
      if (last_closure)
        v *= ord * rho * invmw_d[s] * pow(fmax(c, 1.e-16), ord - 1.);
      else if (ord > 1)
        v *= ord * rho * invmw_d[s] * pow(fmax(c, 1.e-16), ord - 1.);
      else
        v *= ord * rho * invmw_d[s] / pow(fmax(c, 1.e-16), 1. - ord);
    } else if (nz) {
      v *= last_closure ? pow(c, ord) : pow(fmax(c, 0.), ord);
    }
  }
  return v;
}

template <bool JAC>
struct RxnOut {
  double q;
};

// Evaluate reaction r. Always writes q[r]; with JAC also dq/drho, dq/dT, the sparse slot derivatives D (scaled by
// 1/rho), the dense coefficients alpha, beta (scaled by 1/rho) and E_r = sum_i c_ir * eh_i.
template <bool JAC, class S>
__device__ __forceinline__ void eval_reaction(const DevMech &m, Blob b, const ScratchLayout &L, S scr,
                                              const StateCtx &s, int r, double *Eacc_a, double *Eacc_b)
{
  const int info = b.i[m.i_info + r];
  const int kind = (info >> RI_KIND_SHIFT) & 7;
  const int kform = (info >> RI_KFORM_SHIFT) & 7;
  const bool rev = (info >> RI_REV_BIT) & 1;
  const bool has_ord = (info >> RI_ORD_BIT) & 1;
  const double *kc = b.d + m.d_kf + 3 * r;
  const auto C = scr + L.C;
  const auto y = scr + L.y;
  const double *invmw_d = b.d + m.d_invmw;
  // forward rate constant (chemistry_kernels.cpp:140-157)
  double kf;
  switch (kform) {
  case 0: kf = kc[0]; break;
  case 1: kf = kc[0] * s.T; break;
  case 2: kf = kc[0] * s.T * s.T; break;
  case 3: kf = kc[0] * s.invT; break;
  default: kf = kc[0] * tab_exp(kc[1] * s.logT - kc[2] * s.invT, b.d + m.d_exptab); break;
  }
  const double dlogkf = s.invT * (kc[1] + kc[2] * s.invT);
  // third-body / falloff factor (chemistry_kernels.cpp:158-314; rates_sensitivities_exact.cpp:826-1000)
  double Ctbaf = 1., dCdrho = 0., dCdT = 0., K = 0.;
  if (kind != 1) {
    const int t0 = b.i[m.i_tb_off + r], t1 = b.i[m.i_tb_off + r + 1];
    double sumtb = 0.;
    for (int j = t0; j < t1; ++j) sumtb += b.d[m.d_tbeff + j] * y[b.i[m.i_tb + j]];
    const double beff = b.d[m.d_beff + r];
    const double M = beff * s.ct + s.rho * sumtb;
    const double dMdrho = beff * s.invM + sumtb;
    if (kind == 2) {
      Ctbaf = M;
      K = 1.;
      dCdrho = dMdrho;
    } else {
      const int f = b.i[m.i_fall + r];
      const double *kp = b.d + m.d_kp + 3 * f;
      const double kpf = kp[0] * tab_exp(kp[1] * s.logT - kp[2] * s.invT, b.d + m.d_exptab) / kf;
      const double pr = kpf * M;
      const double dlogk = s.invT * (kp[1] + kp[2] * s.invT) - dlogkf;
      if (kind == 3) {
        Ctbaf = pr / (1. + pr);
        if (JAC) {
          dCdT = Ctbaf / (1. + pr) * dlogk;
          K = kpf / ((1. + pr) * (1. + pr));
        }
      } else {
        const double *tr = b.d + m.d_troe + 4 * f;
        const int terms = (info >> RI_TROE_SHIFT) & 7;
        double fc = 0., dfc = 0.;
        if (terms & 1) {
          const double e1 = tab_exp(-s.T / tr[1], b.d + m.d_exptab);
          fc += (1 - tr[0]) * e1;
          dfc += (tr[0] - 1) / tr[1] * e1;
        }
        if (terms & 2) {
          const double e2 = tab_exp(-s.T / tr[2], b.d + m.d_exptab);
          fc += tr[0] * e2;
          dfc += -tr[0] / tr[2] * e2;
        }
        if (terms & 4) {
          const double e3 = tab_exp(-s.invT * tr[3], b.d + m.d_exptab);
          fc += e3;
          dfc += e3 * tr[3] * s.invT * s.invT;
        }
        if (!JAC) {
          // chemistry_kernels.cpp:280-312: F = 10^(log10 Fc / (1 + f1^2)), no clamp on Fc
          const double lfc = log10(fc);
          const double lpc = log10(fmax(pr, 1.e-300)) + (-0.4 - 0.67 * lfc);
          const double f1 = lpc / ((0.75 - 1.27 * lfc) - 0.14 * lpc);
          Ctbaf = tab_exp(2.302585092994046 * (lfc / (1 + f1 * f1)), b.d + m.d_exptab) * pr / (1 + pr);
        } else {
          // rates_sensitivities_exact.cpp:949-985: F = Fc^g with Fc clamped at 1e-300
          const double l10pr = log10(fmax(pr, 1.e-300));
          const double lnfc = log(fmax(fc, 1.e-300));
          const double l10fc = lnfc * 0.43429448190325176;
          const double a = l10pr - 0.67 * l10fc - 0.4;
          const double bb = -0.14 * l10pr - 1.1762 * l10fc + 0.806;
          const double gt = 1 / (1 + (a / bb) * (a / bb));
          const double F = tab_exp(gt * lnfc, b.d + m.d_exptab);
          Ctbaf = F * pr / (1 + pr);
          const double ln10 = 2.302585092994046;
          const double dFdT = F * (gt / fc * dfc + lnfc * (-2.0 * gt * gt / ln10 * a / (bb * bb * bb) *
                                                          ((bb + 0.14 * a) * dlogk - (0.67 * bb - 1.1762 * a) * dfc / fc)));
          dCdT = 1. / (1. + 1. / pr) * dFdT + F * pr / ((1. + pr) * (1. + pr)) * dlogk;
          K = kpf * (-2.0 / (1. + pr) * F * lnfc * gt * gt / ln10 * a / (bb * bb * bb) * (bb + 0.14 * a) +
                     F / ((1. + pr) * (1 + pr)));
        }
      }
      if (JAC) dCdrho = K * dMdrho;
    }
  }
  const bool orders = has_ord && !(JAC && s.option == 1);
  const int ro0 = b.i[m.i_reac_off + r], nre = b.i[m.i_reac_off + r + 1] - ro0;
  const int po0 = b.i[m.i_prod_off + r], npr = b.i[m.i_prod_off + r + 1] - po0;
  const int *rl = b.i + m.i_reac + ro0;
  const int *pl = b.i + m.i_prod + po0;
  double Rf, kr = 0., Rr = 0.;
  const int sums = b.i[m.i_sums + r];
  const int sum_nu = (int)(short)(sums & 0xFFFF);
  // lists of at most three entries (every reaction of common mechanisms) use the factored form
  const bool short_lists = !orders && nre <= 3 && npr <= 3;
  MassAction3 mr, mp;
  mp.P = mp.g0 = mp.g1 = mp.g2 = 0.;
  if (orders) {
    Rf = kf * special_orders(m, b, r, C, s.rho, -1, false);
  } else {
    if (short_lists) {
      mr = mass_action3(rl, nre, C, invmw_d);
      Rf = kf * mr.P;
    } else {
      Rf = kf * mass_action(rl, nre, C, invmw_d, s.rho, -1);
    }
    // rates of a special-order reaction have no reverse part (chemistry_kernels.cpp:316-326)
    if (rev && !has_ord) {
      // kr = kf exp(sum_nu ln(p_ref/RT) - sum_i nu_i g_i/RT) (chemistry_kernels.cpp:327-341), with
      // exp(-g_i/RT) = gm_i 2^gk_i
      const int n0 = b.i[m.i_net_off + r], n1 = b.i[m.i_net_off + r + 1];
      double mant = 1.;
      long long K = 0;
      for (int j = n0; j < n1; ++j) {
        const int e = b.i[m.i_net + j];
        const int sp = e & 0xFFFF, nu = (e >> 16) - 128;
        const double mi = scr[(nu > 0 ? L.gm : L.gmi) + sp];
        const int a = nu > 0 ? nu : -nu;
        mant *= a == 1 ? mi : ipow(mi, a);
        K += (long long)nu * __double_as_longlong(scr[L.gk + sp]);
      }
      const double pw = sum_nu >= 0 ? ipow(s.port, sum_nu) : ipow(s.invport, -sum_nu);
      kr = scale_pow2(kf * pw * mant, K);
      if (short_lists) {
        mp = mass_action3(pl, npr, C, invmw_d);
        Rr = kr * mp.P;
      } else {
        Rr = kr * mass_action(pl, npr, C, invmw_d, s.rho, -1);
      }
    }
  }
  const double Rnet = Rf - Rr;
  scr[L.q + r] = Rnet * Ctbaf;
  if (!JAC) return;

  const double *smallint = b.d + m.d_smallint;
  const double sum_reac_nu = small_int(smallint, (sums >> 16) & 0xFF),
               sum_prod_nu = small_int(smallint, (sums >> 24) & 0xFF);
  double dRdrho, dRdT;
  if (orders) {
    double sumo = 0.;
    const int o0 = b.i[m.i_ord_off + r], o1 = b.i[m.i_ord_off + r + 1];
    for (int j = o0; j < o1; ++j)
      if (b.i[m.i_ord + j] >> 16) sumo += b.d[m.d_ord + j];
    dRdrho = Rf * s.invRho * sumo;
    dRdT = Rf * dlogkf;
  } else {
    double dKc = 0.;
    if (rev && !has_ord) {
      const int n0 = b.i[m.i_net_off + r], n1 = b.i[m.i_net_off + r + 1];
      for (int j = n0; j < n1; ++j) {
        const int e = b.i[m.i_net + j];
        dKc -= small_int(smallint, (e >> 16) - 128) * scr[L.dB + (e & 0xFFFF)];
      }
    }
    dRdrho = (Rf * sum_reac_nu - Rr * sum_prod_nu) * s.invRho;
    dRdT = Rf * dlogkf - Rr * (dlogkf - dKc);
  }
  const bool tbaf = s.option != 1;
  scr[L.dqdrho + r] = dRdrho * Ctbaf + (tbaf ? dCdrho * Rnet : 0.);
  scr[L.dqdT + r] = dRdT * Ctbaf + (tbaf ? dCdT * Rnet : 0.);
  // d q / d Y_k / rho through the third-body concentration: rho * Rnet * K * eff_k / rho
  const double RK = tbaf ? Rnet * K : 0.;
  // sparse slots: D_j = d q / d Y_k / rho for the slot's species k
  const int ns = m.ns;
  const int s0 = b.i[m.i_slot_off + r], s1 = b.i[m.i_slot_off + r + 1];
  const int tb0 = b.i[m.i_tb_off + r];
  for (int j = s0; j < s1; ++j) {
    const int e = b.i[m.i_slot + j];
    const int rp = ((e >> 16) & 15) - 1, pp = ((e >> 20) & 15) - 1, tp = ((e >> 24) & 15) - 1;
    const int op = ((unsigned)e >> 28) - 1;
    double v = 0.;  // d (Rf - Rr) / d Y_k / rho
    if (orders) {
      if (op >= 0) {
        const int oe = b.i[m.i_ord + b.i[m.i_ord_off + r] + op];
        if (oe >> 16) v = kf * special_orders(m, b, r, C, s.rho, op, false) * s.invRho;
      }
    } else if (short_lists) {
      if (rp >= 0) v += kf * mr.g(rp);
      if (pp >= 0 && kr != 0.) v -= kr * mp.g(pp);
    } else {
      if (rp >= 0) v += kf * mass_action(rl, nre, C, invmw_d, s.rho, rp) * s.invRho;
      if (pp >= 0 && kr != 0.) v -= kr * mass_action(pl, npr, C, invmw_d, s.rho, pp) * s.invRho;
    }
    double Dv = Ctbaf * v;
    if (tp >= 0) Dv += RK * b.d[m.d_tbeff + tb0 + tp];
    scr[L.D + j] = Dv;
  }
  const int di = b.i[m.i_dense + r];
  double Er = 0.;
  {
    const int n0 = b.i[m.i_net_off + r], n1 = b.i[m.i_net_off + r + 1];
    for (int j = n0; j < n1; ++j) Er += b.d[m.d_netc + j] * scr[L.eh + (b.i[m.i_net + j] & 0xFFFF)];
  }
  scr[L.E + r] = Er;
  if (di >= 0) {
    // closure species ns-1 and third-body terms common to every Y column (all divided by rho)
    double closure = 0.;
    if (orders) {
      const int o0 = b.i[m.i_ord_off + r], o1 = b.i[m.i_ord_off + r + 1];
      for (int j = o0; j < o1; ++j) {
        const int oe = b.i[m.i_ord + j];
        if ((oe & 0xFFFF) == ns - 1 && (oe >> 16))
          closure -= kf * special_orders(m, b, r, C, s.rho, j - o0, true) * s.invRho;
      }
    } else if (short_lists) {
      for (int j = 0; j < nre; ++j)
        if ((rl[j] & 0xFFFF) == ns - 1) closure -= kf * mr.g(j);
      if (kr != 0.)
        for (int j = 0; j < npr; ++j)
          if ((pl[j] & 0xFFFF) == ns - 1) closure += kr * mp.g(j);
    } else {
      for (int j = 0; j < nre; ++j)
        if ((rl[j] & 0xFFFF) == ns - 1) closure -= kf * mass_action(rl, nre, C, invmw_d, s.rho, j) * s.invRho;
      if (kr != 0.)
        for (int j = 0; j < npr; ++j)
          if ((pl[j] & 0xFFFF) == ns - 1) closure += kr * mass_action(pl, npr, C, invmw_d, s.rho, j) * s.invRho;
    }
    double beta = Ctbaf * closure;
    if (tbaf && kind != 1) {
      const int t1 = b.i[m.i_tb_off + r + 1];
      for (int j = tb0; j < t1; ++j)
        if (b.i[m.i_tb + j] == ns - 1) beta -= RK * b.d[m.d_tbeff + j];
    }
    const double alpha = (kind != 1) ? RK * b.d[m.d_beff + r] : 0.;
    scr[L.alpha + di] = alpha;
    scr[L.beta + di] = beta;
    *Eacc_a += Er * alpha;
    *Eacc_b += Er * beta;
  }
}

// ------------------------------------------------------------------------------------------ gather programs
// Execute a gather program for one state: every lane runs prog.len items (see sf_mech.h). Destination kinds:
// DST_SCRATCH / DST_TROW write scratch[index]; DST_JBLOCK calls jw(row, col, value).
// Items are processed in batches of U (each lane's item count is padded to a multiple of GATHER_UNROLL): the
// operands of a whole batch are loaded before its FMAs, and the next batch's items while they run. This is sound
// because no program reads a scratch location that it writes (checked when the program is built), so no load
// can overtake a store it depends on.

// One lane per state reads its scratch from global memory and gains most from loads in flight; the lane groups
// (scratch in shared memory or L2) take half the batch, which keeps their larger kernels free of register spills.
__host__ __device__ constexpr int default_unroll(int G) { return G == 1 ? GATHER_UNROLL : GATHER_UNROLL / 2; }

template <class S>
__device__ __forceinline__ double gather_operand(uint32_t ref, const double *blobd, const S &scr)
{
  return (ref & REF_SCRATCH) ? scr[ref & ~REF_SCRATCH] : blobd[ref];
}

template <int G, int U = default_unroll(G), class JW, class S>
__device__ __forceinline__ void run_program(const DevProgram &prog, int lane, const double *blobd, S scr,
                                            JW &jw)
{
  static_assert(GATHER_UNROLL % U == 0, "batch must divide the program padding");
  const uint4 *it = reinterpret_cast<const uint4 *>(prog.items) + lane;
  uint4 x[U];
#pragma unroll
  for (int u = 0; u < U; ++u) x[u] = prog.len > 0 ? __ldg(it + u * G) : make_uint4(0, 0, 0, F_NOP);
  double acc = 0.;
  for (int j = 0; j < prog.len; j += U) {
    double a[U], bv[U], c0[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      a[u] = gather_operand(x[u].x, blobd, scr);
      bv[u] = gather_operand(x[u].y, blobd, scr);
      const uint32_t ii = x[u].w & INIT_MASK;
      c0[u] = ((x[u].w & F_START) && ii) ? scr[ii - 1] : 0.;
    }
    uint4 y[U];
    const bool more = j + U < prog.len;
#pragma unroll
    for (int u = 0; u < U; ++u) y[u] = more ? __ldg(it + (j + U + u) * G) : make_uint4(0, 0, 0, F_NOP);
    bool stop = false;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (x[u].w & F_NOP) {
        stop = true;  // padding only follows a lane's last real item
      } else {
        if (x[u].w & F_START) acc = c0[u];
        acc = fma(a[u], bv[u], acc);
        if (x[u].w & F_END) {
          const uint32_t kindd = x[u].z & DST_KIND_MASK;
          if (kindd == DST_JBLOCK)
            jw(x[u].z & 0x7FFF, (x[u].z >> 15) & 0x7FFF, acc);
          else
            scr[x[u].z & ~DST_KIND_MASK] = acc;
        }
      }
    }
    if (stop) break;
#pragma unroll
    for (int u = 0; u < U; ++u) x[u] = y[u];
  }
}

struct NoJ {
  __device__ __forceinline__ void operator()(int, int, double) const {}
};

}  // namespace sfgb
