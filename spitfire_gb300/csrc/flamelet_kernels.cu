// Flamelet kernels: the flamelet right-hand side (adiabatic or with heat loss) and its block-tridiagonal ("BTDDOD": block diagonal,
// diagonal off-diagonals) Jacobian for a batch of flamelets with different grids, and the block-Thomas algebra.
//
// Reference: src/spitfire/griffon/src/flamelet_kernels.cpp:31-90 (stencils, COO indices), :1039-1218
// (flamelet_rhs), :1220-1409 (flamelet_jacobian); src/btddod_matrix_kernels.cpp:19-465.
//
// Points of all flamelets are flattened: flamelet f owns interior points offsets_z[f] .. offsets_z[f+1]-1. One state
// group evaluates one point (isobaric chemistry via reactor_eval, then the mixture-fraction stencils). The
// block-Thomas factorization and solve are sequential in mixture fraction; they run from both ends of a flamelet
// toward its middle block, two CTAs (factorization) or two warps (solve) per flamelet, parallel within each block.
#include "reactor_eval.cuh"
#include "sf_internal.h"
#include "eig_device.cuh"

namespace sfgb {
namespace {

struct FlmParams {
  DevMech m;
  const void *blob;
  int *status;
  ScratchLayout L;
  Progs pg;
  int n_flamelets, n_points;
  const int *offz;        // device [nf+1]
  const long long *offv;  // device [nf+1]
  double pressure;
  const double *oxy, *fuel;  // [nf][ns]
  const double *cmajor, *csub, *csup, *mc, *nc, *chi;
  int eflux, vcp;
  const double *state;
  double *out_rhs;
  double *out_values;
  int scale_offset;
  int rates_option;
  double prefactor;
  const double *prefactors;  // device [nf] or null: each flamelet's own prefactor of scale_offset
  double *eflux_store;  // if set: the enthalpy-flux diagonal correction is stored here (per point) instead
  const int *active;    // device [nf] or null: flamelets with active[f] == 0 are skipped
  // nonadiabatic flamelets: convection / radiation temperature and coefficient per interior point (null: adiabatic)
  const double *Tconv, *hconv, *Trad, *hrad;
  int scaled_heat_loss;
  int groups_per_cta;
};

__device__ __forceinline__ int find_flamelet(const int *offz, int nf, int p)
{
  int lo = 0, hi = nf - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (offz[mid] <= p) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// cp of the mixture at a state [T, Y_0..Y_{ns-2}] (lanes over species, group reduction)
template <int G>
__device__ __forceinline__ double cp_of_state(const DevMech &m, const Blob &b, const Group<G> &grp, const double *st)
{
  const int ns = m.ns;
  const double T = st[0], logT = log(T), invT = 1. / T;
  double ys = 0., cp = 0.;
  for (int i = grp.lane; i < ns - 1; i += G) {
    const SpeciesThermo th = species_thermo(m, b, i, T, logT, invT, false);
    cp += st[1 + i] * th.cp;
    ys += st[1 + i];
  }
  ys = grp.sum(ys);
  cp = grp.sum(cp);
  const SpeciesThermo thn = species_thermo(m, b, ns - 1, T, logT, invT, false);
  return cp + (1. - ys) * thn.cp;
}

struct BlockWriter {
  double *blk;  // column-major ns x ns
  int ns;
  const double *cmaj;  // [ns] of this point
  int scale;
  double pref;
  __device__ __forceinline__ void operator()(int row, int col, double v) const
  {
    double x = v + (row == col ? cmaj[row] : 0.);
    if (scale) x = pref * x - (row == col ? 1. : 0.);
    blk[col * ns + row] = x;
  }
};

// Heat loss of a nonadiabatic flamelet point (flamelet_kernels.cpp:1121-1138, :1290-1320): the isobaric reactor's
// diathermal terms with unit surface-to-volume ratio and this point's convection (Tc, hc) and radiation (Tr, hr)
// parameters, q = hc (Tc - T) + hr sigma (Tr^4 - T^4) entering dT/dt as q / (rho cp). With use_scaled_heat_loss the
// coefficients are divided by (max T - Tc) and (max T^4 - Tr^4), max T over the flamelet's interior points (held
// constant in the Jacobian, as the reference does). The reference adds the Y-column terms in a loop that runs two
// columns past the end of its primitive Jacobian (flamelet_kernels.cpp:1316-1319); here they stop at the last Y
// column.
template <int G>
__device__ __forceinline__ void heat_loss_cfg(const FlmParams &p, const Group<G> &grp, int pt, int z0, int nzi,
                                              ReactorCfg &cfg)
{
  if (!p.Tconv) {
    cfg.heat = 0;
    return;
  }
  const double Tc = p.Tconv[pt], Tr = p.Trad[pt];
  double hc = p.hconv[pt], hr = p.hrad[pt];
  if (p.scaled_heat_loss) {
    double mx = -1.;
    for (int j = grp.lane; j < nzi; j += G) mx = fmax(mx, p.state[(size_t)(z0 + j) * p.m.ns]);
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(grp.mask, mx, o, G));
    const double Tr4 = Tr * Tr * Tr * Tr;
    hc = hc / (mx - Tc);
    hr = hr / (mx * mx * mx * mx - Tr4);
  }
  cfg.heat = 2;
  cfg.Tc = Tc;
  cfg.hc = hc;
  cfg.Tr = Tr;
  cfg.eps = hr;
  cfg.SoV = 1.;
}

template <int G, bool JAC>
__global__ void __launch_bounds__(256) flamelet_point_kernel(const FlmParams p)
{
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint64_t bar;
  const DevMech &m = p.m;
  if (!stage_to_smem(smem, p.blob, m.blob_bytes, &bar, p.status)) return;
  const Blob b = blob_at(m, smem);
  const ScratchLayout &L = p.L;
  const int gid = threadIdx.x / G;
  // per group: Griffon scratch + ns doubles for the (unused) right-hand side of the Jacobian evaluation
  double *scr = reinterpret_cast<double *>(smem + m.blob_bytes) + (size_t)gid * ((JAC ? L.total : L.total_rhs) + m.ns + 2);
  const Group<G> grp;
  const int lane = grp.lane;
  const int ns = m.ns;
  ReactorCfg cfg{};
  cfg.configuration = 0;
  cfg.heat = 0;
  cfg.option = JAC ? p.rates_option : 0;
  NoJ noj;
  for (int pt = blockIdx.x * p.groups_per_cta + gid; pt < p.n_points; pt += gridDim.x * p.groups_per_cta) {
    const int f = find_flamelet(p.offz, p.n_flamelets, pt);
    const double pref = p.prefactors ? p.prefactors[f] : p.prefactor;
    if (p.active && !p.active[f]) continue;
    const int z0 = p.offz[f], nzi = p.offz[f + 1] - z0;
    const int iz = pt - z0;
    heat_loss_cfg<G>(p, grp, pt, z0, nzi, cfg);
    const double *st = p.state + (size_t)pt * ns;
    const double *oxy = p.oxy + (size_t)f * ns;
    const double *fuel = p.fuel + (size_t)f * ns;
    const double *sm1 = iz == 0 ? oxy : st - ns;
    const double *sp1 = iz == nzi - 1 ? fuel : st + ns;
    const double mcf = p.mc[pt], ncf = p.nc[pt], chi = p.chi[pt];
    if (!JAC) {
      double *out = p.out_rhs + (size_t)pt * ns;
      reactor_eval<G, false, default_unroll(G), false>(m, b, L, scr, grp, st, p.pressure, cfg, p.pg, out, noj);
      // enthalpy-flux and variable-cp terms of the temperature equation (flamelet_kernels.cpp:1141-1206)
      double cp = 0.;
      for (int i = lane; i < ns; i += G) cp += scr[L.y + i] * scr[L.cpv + i];
      cp = grp.sum(cp);
      const double dTdZ = mcf * sm1[0] + ncf * sp1[0];
      double extra = 0.;
      if (p.eflux) {
        const double cpn = scr[L.cpv + ns - 1];
        double s = 0.;
        for (int j = lane; j < ns - 1; j += G) s += (scr[L.cpv + j] - cpn) * (mcf * sm1[1 + j] + ncf * sp1[1 + j]);
        s = grp.sum(s);
        extra += 0.5 * chi / cp * dTdZ * s;
      }
      if (p.vcp) {
        const double cpm = cp_of_state<G>(m, b, grp, sm1);
        const double cpp = cp_of_state<G>(m, b, grp, sp1);
        extra += 0.5 * chi * (mcf * cpm + ncf * cpp) / cp * dTdZ;
      }
      grp.sync();
      // mixture-fraction diffusion (flamelet_kernels.cpp:1208-1217)
      const double *cma = p.cmajor + (size_t)pt * ns, *csb = p.csub + (size_t)pt * ns, *csp = p.csup + (size_t)pt * ns;
      for (int i = lane; i < ns; i += G) {
        double v = out[i] + (i == 0 ? extra : 0.);
        v += cma[i] * st[i] + csb[i] * sm1[i] + csp[i] * sp1[i];
        out[i] = v;
      }
      grp.sync();
    } else {
      // block of this point in the flamelet's BTDDOD value array
      double *vals = p.out_values + p.offv[f];
      double *blk = vals + (size_t)iz * ns * ns;
      BlockWriter bw{blk, ns, p.cmajor + (size_t)pt * ns, p.scale_offset, pref};
      double *rhs_tmp = scr + L.total;
      reactor_eval<G, true, default_unroll(G), false>(m, b, L, scr, grp, st, p.pressure, cfg, p.pg, rhs_tmp, bw);
      if (p.eflux) {
        // approximate diagonal correction of the enthalpy-flux term (flamelet_kernels.cpp:1350-1381)
        double cp = 0., cps = 0.;
        for (int i = lane; i < ns; i += G) {
          cp += scr[L.y + i] * scr[L.cpv + i];
          cps += scr[L.y + i] * scr[L.dcp + i];
        }
        cp = grp.sum(cp);
        cps = grp.sum(cps);
        const double cpm = cp_of_state<G>(m, b, grp, sm1);
        const double cpp = cp_of_state<G>(m, b, grp, sp1);
        const double dTdZ = mcf * sm1[0] + ncf * sp1[0];
        const double dcpdZ = mcf * cpm + ncf * cpp;
        const double f1 = 0.5 * chi / cp * dTdZ * dcpdZ;
        grp.sync();
        if (lane == 0) {
          const double corr = (p.scale_offset ? pref : 1.) * f1 / cp * cps;
          if (p.eflux_store)
            p.eflux_store[(size_t)pt * ns] = corr;
          else
            blk[0] -= corr;
        }
      } else if (p.eflux_store && lane == 0) {
        p.eflux_store[(size_t)pt * ns] = 0.;
      }
      // off-diagonals: sub row iz (iz >= 1) and super row iz (iz <= nzi-2) (flamelet_kernels.cpp:1383-1394)
      const long long sub_off = (long long)nzi * ns * ns, sup_off = sub_off + (long long)(nzi - 1) * ns;
      const double sc = p.scale_offset ? pref : 1.;
      for (int q = lane; q < ns; q += G) {
        if (iz >= 1) vals[sub_off + (long long)(iz - 1) * ns + q] = sc * p.csub[(size_t)pt * ns + q];
        if (iz <= nzi - 2) vals[sup_off + (long long)iz * ns + q] = sc * p.csup[(size_t)pt * ns + q];
      }
      grp.sync();
    }
  }
}

// Pseudo-time-step eigenvalue bound (flamelet_kernels.cpp:1329-1341): for each point, max(max Re(lambda) - d, 0)
// of the transformed isobaric chemistry block (the block before the diffusion diagonal and the enthalpy-flux
// correction are added), d the flamelet's diffusion term, written to all ns entries of the point; then the held-back
// enthalpy-flux correction is applied to the block. One warp per point, the block in shared memory. The result is
// exactly 0 whenever every eigenvalue lies left of d; the scaled-Gershgorin (M-matrix) test proves that for a large
// share of the points at a small fraction of the QR iteration's cost, which then runs only for the rest.
__global__ void flamelet_expeig_kernel(int n_points, int nf, int ns, const int *offz, const long long *offv,
                                       double *values, const double *cmajor, double diffterm,
                                       const double *diffterm_f, const int *active, double *expeig, int *status,
                                       int warps, int *next_point)
{
  extern __shared__ __align__(16) unsigned char smem[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double *A = reinterpret_cast<double *>(smem) + (size_t)w * (ns * ns + 2 * ns);
  double *work = A + ns * ns;
  // points are taken dynamically (whether a point needs the QR iteration is known only once it is examined)
  for (;;) {
    int pt = 0;
    if (lane == 0) pt = atomicAdd(next_point, 1);
    pt = __shfl_sync(0xffffffffu, pt, 0);
    if (pt >= n_points) break;
    const int f = find_flamelet(offz, nf, pt);
    if (active && !active[f]) continue;
    const int iz = pt - offz[f];
    const double d = diffterm_f ? diffterm_f[f] : diffterm;
    double *blk = values + offv[f] + (size_t)iz * ns * ns;
    auto load = [&]() {
      for (int e = lane; e < ns * ns; e += 32) {
        const int col = e / ns, row = e - col * ns;
        A[e] = blk[e] - (row == col ? cmajor[(size_t)pt * ns + row] : 0.);
      }
      __syncwarp();
    };
    load();
    double mx = d;
    bool ok = true;
    if (!warp_hmatrix_below(A, ns, d, work)) {
      __syncwarp();
      load();
      ok = warp_max_real_eig(A, ns, work, &mx, d);
    }
    if (!ok && lane == 0) report_error(status, DEVERR_WAIT_TIMEOUT);
    const double corr = expeig[(size_t)pt * ns];
    __syncwarp();
    const double e = fmax(mx - d, 0.);
    for (int q = lane; q < ns; q += 32) expeig[(size_t)pt * ns + q] = e;
    if (lane == 0) blk[0] -= corr;
    __syncwarp();
  }
}

// ------------------------------------------------------------------------------- block-Thomas (BTDDOD) algebra
// The reference factorization (btddod_matrix_kernels.cpp:19-80) eliminates downward from the first block:
// LU(D_0); for i >= 1: L_i = diag(sub_{i-1}) D_{i-1}^-1 (the reference solves D_{i-1} X = I with dgetrs),
// D_i <- D_i - L_i diag(sup_{i-1}), LU(D_i). Its chain of nzi dependent block steps is the critical path of a
// flamelet, so this factorization is twisted: with m = nzi/2, one CTA eliminates blocks 0..m-1 downward exactly as
// above, a second CTA eliminates blocks nzi-1..m+1 upward (T_{nzi-1} = D_{nzi-1}; U_i = diag(sup_{i-1}) T_i^-1;
// T_{i-1} = D_{i-1} - U_i diag(sub_{i-1})), and block m receives both: M = D_m - L_m diag(sup_{m-1})
// - U_{m+1} diag(sub_m). Same flops, half the chain, and as stable for these block-diagonally dominant matrices.
// Every eliminated block is inverted once (the multiplier blocks need the inverse anyway), by Gauss-Jordan
// elimination with one CTA barrier per column, and the inverse is what the solve applies.
// Storage: values block i holds the inverse of the eliminated block i; l_values block i holds L_i for
// 1 <= i <= m and U_i for m < i < nzi (block 0 unused).
constexpr int kFactorThreads = 512;  // 16 warps: warp 0 runs the pivot look-ahead, 12 update the block
static_assert(kFactorThreads >= 64 && kFactorThreads % 32 == 0, "the elimination needs updating warps");

// Inverse of the n x n row-major matrix in S by Gauss-Jordan elimination with partial pivoting (G. H. Golub and
// C. F. Van Loan, "Matrix Computations", section 3.2; rows are not moved, the pivot order is recorded). Phase k
// maps the source buffer to the destination (S and D alternate): with pivot row p, ip = 1/S[p][k] and
// f_i = S[i][k] ip,
//   D[p][j] = S[p][j] ip,   D[i][j] = S[i][j] - f_i S[p][j]   (j != k),   D[p][k] = ip,   D[i][k] = -f_i.
// The other warps update the block while warp 0 forms column k+1 of D and, before the phase's barrier, chooses the
// next pivot among the unused rows (largest magnitude, lowest row on ties, as idamax) and its multipliers: one
// barrier per column. Returns the buffer Z holding the inverse permuted: inverse(r, c) = Z[piv[r]][pinv[c]], where
// pinv[piv[k]] = k. ws: 2n + 2 doubles (the negated multipliers and pivot reciprocals of two phases); used: n ints.
// A pivot column of zeros gives ip = 0 (a singular block; the output is then not an inverse). n <= 128.
__device__ double *cta_gj_inverse(double *S, double *D, int n, int *piv, int *pinv, double *ws, int *used)
{
  const int tid = threadIdx.x, nt = blockDim.x, warp = tid >> 5, lane = tid & 31;
  double *ipb = ws + 2 * n;
  // The updating warps leave warp 0's scheduler partition (warps 4, 8, ... share it; warps are dealt to the four
  // partitions by warp index) to warp 0 alone, so that its serial look-ahead does not queue for the FP64 unit
  // behind their updates. Elements are dealt to the updating threads in row-major order with incremental indices.
  const int nw = nt >> 5;
  const int uw = (warp & 3) ? warp - (warp >> 2) - 1 : -1;
  const int ustride = 32 * (nw - (nw + 3) / 4);
  const int ut = uw * 32 + lane;
  const int i0 = ut / n, j0 = ut - (ut / n) * n, di = ustride / n, dj = ustride - (ustride / n) * n;
  // warp 0: choose the pivot of column j among the unused rows from the lane-held column values v (row lane+32s),
  // publish it with its multipliers for phase j
  auto choose = [&](int j, const double (&v)[4]) {
    unsigned long long best = 0ull;
    int bp = n;
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const int i = lane + 32 * s;
      if (i < n && !used[i]) {
        const unsigned long long key = (unsigned long long)__double_as_longlong(v[s]) & 0x7fffffffffffffffull;
        if (bp == n || key > best) { best = key; bp = i; }
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bp, o);
      if (oi < n && (bp >= n || ob > best || (ob == best && oi < bp))) { best = ob; bp = oi; }
    }
    double pv = 0.;
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const double t = __shfl_sync(0xffffffffu, v[s], bp & 31);
      if ((bp >> 5) == s) pv = t;
    }
    const double ip = pv != 0. ? 1. / pv : 0.;
    const double nip = -ip;
    double *f = ws + (j & 1) * n;  // the negated multipliers -f_i
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const int i = lane + 32 * s;
      if (i < n) f[i] = v[s] * nip;
    }
    if (lane == 0) {
      ipb[j & 1] = ip;
      piv[j] = bp;
      pinv[bp] = j;
      used[bp] = 1;
    }
    __syncwarp();
  };
  if (warp == 0) {
    for (int i = lane; i < n; i += 32) used[i] = 0;
    __syncwarp();
    double v[4];
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const int i = lane + 32 * s;
      v[s] = i < n ? S[i * n] : 0.;
    }
    choose(0, v);
  }
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    const int p = piv[k];
    const double ip = ipb[k & 1];
    const double *nf = ws + (k & 1) * n;  // -f_i
    const double *Sp = S + (size_t)p * n;
    if (warp == 0) {
      if (k + 1 < n) {
        const int j = k + 1;
        const double spj = Sp[j];
        double v[4];
#pragma unroll
        for (int s = 0; s < 4; ++s) {
          const int i = lane + 32 * s;
          double val = 0.;
          if (i < n) {
            val = S[i * n + j] + nf[i] * spj;
            if (i == p) val = spj * ip;
            D[i * n + j] = val;
          }
          v[s] = val;
        }
        choose(j, v);
      }
    } else if (uw >= 0) {
      const int kn = k + 1;
      int i = i0, j = j0;
      for (int e = ut; e < n * n; e += ustride) {
        if (j != kn) {  // column k+1 is warp 0's
          // one FMA per element and warp; the column-k value is a select, the pivot row (in at most two of a warp's
          // iterations) a multiplication
          const double nfi = nf[i];
          double val = S[e] + nfi * Sp[j];
          if (j == k) val = nfi;
          if (i == p) val = j == k ? ip : Sp[j] * ip;
          D[e] = val;
        }
        i += di;
        j += dj;
        if (j >= n) {
          j -= n;
          ++i;
        }
      }
    }
    __syncthreads();
    double *t = S;
    S = D;
    D = t;
  }
  return S;
}

// Shared-memory bytes of the factorization kernels: two row-major blocks, the elimination's multipliers and pivot
// reciprocals, three index arrays.
inline size_t factor_smem_bytes(int ns)
{
  return (size_t)2 * ns * ns * 8 + (size_t)(2 * ns + 2) * 8 + (size_t)3 * ns * 4 + 16;
}

struct FactorShared {
  double *buf0, *buf1, *ws;
  int *piv, *pinv, *used;
  __device__ FactorShared(unsigned char *smem, int ns)
  {
    buf0 = reinterpret_cast<double *>(smem);
    buf1 = buf0 + (size_t)ns * ns;
    ws = buf1 + (size_t)ns * ns;
    piv = reinterpret_cast<int *>(ws + 2 * ns + 2);
    pinv = piv + ns;
    used = pinv + ns;
  }
};

// One CTA per (flamelet, half): even CTAs eliminate blocks 0..m-1 downward, odd CTAs blocks nzi-1..m+1 upward.
// Each half ends with the multiplier block that feeds block m (L_m, or U_{m+1}); btddod_middle_kernel then forms
// and inverts block m.
__global__ void __launch_bounds__(kFactorThreads) btddod_factor_kernel(int nf, int ns, const int *offz,
                                                                       const long long *offv, double *values,
                                                                       double *lvals, int *perms, const int *active)
{
  extern __shared__ __align__(16) unsigned char smem[];
  const int f = blockIdx.x >> 1;
  const bool down = (blockIdx.x & 1) == 0;
  if (f >= nf || (active && !active[f])) return;
  const int z0 = offz[f], nb = offz[f + 1] - z0, m = nb / 2;
  const int len = down ? m : nb - 1 - m;
  if (len <= 0) return;
  const int bs2 = ns * ns;
  double *vals = values + offv[f];
  double *lv = lvals + (size_t)z0 * bs2;
  int *pv = perms + (size_t)z0 * ns;
  const double *sub = vals + (size_t)nb * bs2;
  const double *sup = sub + (size_t)(nb - 1) * ns;
  FactorShared sh(smem, ns);
  double *cur = sh.buf0, *other = sh.buf1;  // cur: the block to invert (row-major)
  const int tid = threadIdx.x, nt = blockDim.x;
  {
    const double *D0 = vals + (size_t)(down ? 0 : nb - 1) * bs2;
    for (int e = tid; e < bs2; e += nt) {
      const int c = e / ns, r = e - c * ns;
      cur[r * ns + c] = D0[e];
    }
  }
  __syncthreads();
  for (int t = 0; t < len; ++t) {
    const int i = down ? t : nb - 1 - t;
    double *Z = cta_gj_inverse(cur, other, ns, sh.piv, sh.pinv, sh.ws, sh.used);
    double *nxt = Z == cur ? other : cur;  // the buffer the elimination no longer needs
    // multiplier: downward L_{i+1} = diag(sub_i) D_i^-1 at block i+1; upward U_i = diag(sup_{i-1}) T_i^-1 at block
    // i. Then the next block of the chain: D_{i+1} - L_{i+1} diag(sup_i), or D_{i-1} - U_i diag(sub_{i-1}).
    const double *rs = down ? sub + (size_t)i * ns : sup + (size_t)(i - 1) * ns;
    const double *cs = down ? sup + (size_t)i * ns : sub + (size_t)(i - 1) * ns;
    double *Di = vals + (size_t)i * bs2;
    double *Lm = lv + (size_t)(down ? i + 1 : i) * bs2;
    const double *Dn = vals + (size_t)(down ? i + 1 : i - 1) * bs2;
    const bool more = t + 1 < len;
    for (int e = tid; e < bs2; e += nt) {  // e: column-major index of the global arrays
      const int c = e / ns, r = e - c * ns;
      const double inv = Z[sh.piv[r] * ns + sh.pinv[c]];
      Di[e] = inv;
      const double l = inv * rs[r];
      Lm[e] = l;
      if (more) nxt[r * ns + c] = Dn[e] + (-cs[c]) * l;
    }
    for (int k = tid; k < ns; k += nt) pv[(size_t)i * ns + k] = sh.piv[k];
    __syncthreads();
    cur = nxt;
    other = Z;
  }
}

// Block m of each flamelet: M = D_m - L_m diag(sup_{m-1}) - U_{m+1} diag(sub_m) (terms present when m >= 1 and
// m + 1 < nzi), then its inverse. One CTA per flamelet, after btddod_factor_kernel.
__global__ void __launch_bounds__(kFactorThreads) btddod_middle_kernel(int nf, int ns, const int *offz,
                                                                       const long long *offv, double *values,
                                                                       const double *lvals, int *perms,
                                                                       const int *active)
{
  extern __shared__ __align__(16) unsigned char smem[];
  const int f = blockIdx.x;
  if (f >= nf || (active && !active[f])) return;
  const int z0 = offz[f], nb = offz[f + 1] - z0, m = nb / 2;
  const int bs2 = ns * ns;
  double *vals = values + offv[f];
  const double *lv = lvals + (size_t)z0 * bs2;
  const double *sub = vals + (size_t)nb * bs2;
  const double *sup = sub + (size_t)(nb - 1) * ns;
  FactorShared sh(smem, ns);
  double *Dm = vals + (size_t)m * bs2;
  const double *La = m >= 1 ? lv + (size_t)m * bs2 : nullptr;
  const double *Ub = m + 1 < nb ? lv + (size_t)(m + 1) * bs2 : nullptr;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < bs2; e += nt) {
    const int c = e / ns, r = e - c * ns;
    double v = Dm[e];
    if (La) v = v + (-sup[(size_t)(m - 1) * ns + c]) * La[e];
    if (Ub) v = v + (-sub[(size_t)m * ns + c]) * Ub[e];
    sh.buf0[r * ns + c] = v;
  }
  __syncthreads();
  const double *Z = cta_gj_inverse(sh.buf0, sh.buf1, ns, sh.piv, sh.pinv, sh.ws, sh.used);
  for (int e = tid; e < bs2; e += nt) {
    const int c = e / ns, r = e - c * ns;
    Dm[e] = Z[sh.piv[r] * ns + sh.pinv[c]];
  }
  int *pv = perms + (size_t)(z0 + m) * ns;
  for (int k = tid; k < ns; k += nt) pv[k] = sh.piv[k];
}

// Per-lane asynchronous 8-byte copies global -> shared (cp.async, completion tracked by commit groups; no
// mbarrier wait is involved).
__device__ __forceinline__ void async_copy_doubles(double *dst, const double *src, int n)
{
  const int lane = threadIdx.x & 31;
  for (int e = lane; e < n; e += 32)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_addr(dst + e)), "l"(src + e) : "memory");
  asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void async_wait_all_but_one() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Register-distributed vector of a warp: element k lives in lane k % 32, register k / 32 (R registers).
template <int R>
__device__ __forceinline__ double vec_get(const double (&v)[R], int k)
{
  double out = 0.;
#pragma unroll
  for (int s = 0; s < R; ++s) {
    const double t = __shfl_sync(0xffffffffu, v[s], k & 31);
    if ((k >> 5) == s) out = t;
  }
  return out;
}

template <int R>
__device__ __forceinline__ void vec_load(double (&v)[R], const double *src, int ns)
{
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int s = 0; s < R; ++s) {
    const int k = lane + 32 * s;
    v[s] = k < ns ? src[k] : 0.;
  }
}

template <int R>
__device__ __forceinline__ void vec_store(double *dst, const double (&v)[R], int ns)
{
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int s = 0; s < R; ++s) {
    const int k = lane + 32 * s;
    if (k < ns) dst[k] = v[s];
  }
}

// acc -= B y for the column-major ns x ns block B (shared memory) and register-distributed y.
template <int R>
__device__ __forceinline__ void vec_sub_matvec(const double *B, const double (&y)[R], int ns, double (&acc)[R])
{
  const int lane = threadIdx.x & 31;
  for (int c = 0; c < ns; ++c) {
    const double yc = vec_get<R>(y, c);
#pragma unroll
    for (int s = 0; s < R; ++s) {
      const int k = lane + 32 * s;
      if (k < ns) acc[s] += (-B[k + c * ns]) * yc;
    }
  }
}

// v <- B v for the column-major ns x ns block B (shared memory) and register-distributed v.
template <int R>
__device__ __forceinline__ void vec_apply(const double *B, int ns, double (&v)[R])
{
  const int lane = threadIdx.x & 31;
  double acc[R];
#pragma unroll
  for (int s = 0; s < R; ++s) acc[s] = 0.;
  for (int c = 0; c < ns; ++c) {
    const double vc = vec_get<R>(v, c);
#pragma unroll
    for (int s = 0; s < R; ++s) {
      const int k = lane + 32 * s;
      if (k < ns) acc[s] += B[k + c * ns] * vc;
    }
  }
#pragma unroll
  for (int s = 0; s < R; ++s) v[s] = acc[s];
}

// Matrices of one warp's sweep, staged into shared memory: with two buffers the next block is copied while the
// current one is used; with one (large blocks) each is copied when needed.
struct SweepBuffers {
  double *b0, *b1;
  bool dbl;
  int bs2;
  __device__ __forceinline__ double *slot(int k) const { return (k & 1) ? b1 : b0; }  // parity, also for k < 0
  template <class Src>
  __device__ __forceinline__ const double *get(int t, int last, int step, Src src)
  {
    // blocks t, t + step, ... up to `last` inclusive are fetched in this order
    __syncwarp();
    if (dbl) {
      if (t != last) {
        async_copy_doubles(slot(t + step), src(t + step), bs2);
        async_wait_all_but_one();
      } else {
        async_wait_all();
      }
    } else {
      async_copy_doubles(b0, src(t), bs2);
      async_wait_all();
    }
    __syncwarp();
    return dbl ? slot(t) : b0;
  }
  template <class Src>
  __device__ __forceinline__ void prime(int t, Src src)
  {
    if (dbl) async_copy_doubles(slot(t), src(t), bs2);
  }
};

// Solve with the twisted factors (the reference's btddod_matrix_kernels.cpp:82-119 sweeps, run from both ends):
// one CTA of two warps per flamelet, warp 0 over blocks 0..m-1, warp 1 over blocks nzi-1..m+1, m = nzi/2.
//   downward  y_0 = b_0, y_i = b_i - L_i y_{i-1};       upward  z_{nzi-1} = b_{nzi-1}, z_i = b_i - U_{i+1} z_{i+1}
//   middle    x_m = M^-1 (b_m - L_m y_{m-1} - U_{m+1} z_{m+1})
//   back      x_i = D_i^-1 (y_i - sup_i o x_{i+1}) for i < m;   x_i = T_i^-1 (z_i - sub_{i-1} o x_{i-1}) for i > m.
// Every block step is a matrix-vector product (the factors hold the inverses). Vectors stay in registers; y and z are
// parked in out_x until the back substitution overwrites them.
template <int R>
__global__ void __launch_bounds__(64) btddod_solve_kernel(int nf, int ns, const int *offz, const long long *offv,
                                                          const double *values, const double *lvals,
                                                          const int *perms, const double *rhs, double *x,
                                                          const int *active, int double_buffer)
{
  extern __shared__ __align__(16) unsigned char smem[];
  const int f = blockIdx.x;
  if (f >= nf || (active && !active[f])) return;
  const int warp = threadIdx.x >> 5;
  const bool down = warp == 0;
  const int z0 = offz[f], nb = offz[f + 1] - z0, m = nb / 2;
  const int len = down ? m : nb - 1 - m;
  const int bs2 = ns * ns;
  double *sm = reinterpret_cast<double *>(smem);
  const int nbuf = double_buffer ? 2 : 1;
  SweepBuffers sb{sm + (size_t)(warp * nbuf) * bs2, sm + (size_t)(warp * nbuf + nbuf - 1) * bs2, double_buffer != 0,
                  bs2};
  double *feed = sm + (size_t)(2 * nbuf) * bs2;  // 2 ns doubles: -L_m y_{m-1} and -U_{m+1} z_{m+1}
  double *xmid = feed + 2 * ns;                  // ns doubles
  const double *vals = values + offv[f];
  const double *lv = lvals + (size_t)z0 * bs2;
  (void)perms;  // the pivot order of each block's elimination; the stored inverses need none
  const double *sub = vals + (size_t)nb * bs2;
  const double *sup = sub + (size_t)(nb - 1) * ns;
  const double *b = rhs + (size_t)z0 * ns;
  double *xs = x + (size_t)z0 * ns;
  auto blk = [&](int t) { return down ? t : nb - 1 - t; };
  // ---- sweeps toward block m: step t (1 <= t <= len) applies multiplier block blk(t) (+1 upward); step len feeds m
  auto lsrc = [&](int t) { return lv + (size_t)(down ? t : nb - t) * bs2; };
  double y[R];
#pragma unroll
  for (int s = 0; s < R; ++s) y[s] = 0.;
  if (len > 0) {
    sb.prime(1, lsrc);
    vec_load<R>(y, b + (size_t)blk(0) * ns, ns);
    vec_store<R>(xs + (size_t)blk(0) * ns, y, ns);
    for (int t = 1; t <= len; ++t) {
      const double *B = sb.get(t, len, 1, lsrc);
      double acc[R];
      if (t < len) {
        vec_load<R>(acc, b + (size_t)blk(t) * ns, ns);
      } else {
#pragma unroll
        for (int s = 0; s < R; ++s) acc[s] = 0.;
      }
      vec_sub_matvec<R>(B, y, ns, acc);
#pragma unroll
      for (int s = 0; s < R; ++s) y[s] = acc[s];
      if (t < len) vec_store<R>(xs + (size_t)blk(t) * ns, y, ns);
    }
  }
  vec_store<R>(feed + (size_t)warp * ns, y, ns);  // zero when this half is empty
  __syncthreads();
  // ---- block m
  auto fsrc = [&](int i) { return vals + (size_t)i * bs2; };
  if (down) {
    sb.prime(m, fsrc);
    const double *F = sb.get(m, m, 1, fsrc);  // single fetch (t == last)
    double v[R], f0[R], f1[R];
    vec_load<R>(v, b + (size_t)m * ns, ns);
    vec_load<R>(f0, feed, ns);
    vec_load<R>(f1, feed + ns, ns);
#pragma unroll
    for (int s = 0; s < R; ++s) v[s] = (v[s] + f0[s]) + f1[s];
    vec_apply<R>(F, ns, v);
    vec_store<R>(xs + (size_t)m * ns, v, ns);
    vec_store<R>(xmid, v, ns);
  }
  __syncthreads();
  if (len == 0) return;
  // ---- back substitution away from block m: blocks blk(len-1), ..., blk(0)
  double xn[R];
  vec_load<R>(xn, xmid, ns);
  auto bsrc = [&](int t) { return vals + (size_t)blk(t) * bs2; };
  sb.prime(len - 1, bsrc);
  for (int t = len - 1; t >= 0; --t) {
    const double *F = sb.get(t, 0, -1, bsrc);
    const int i = blk(t);
    const double *cpl = down ? sup + (size_t)i * ns : sub + (size_t)(i - 1) * ns;
    double v[R];
    vec_load<R>(v, xs + (size_t)i * ns, ns);
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int s = 0; s < R; ++s) {
      const int k = lane + 32 * s;
      if (k < ns) v[s] = v[s] - cpl[k] * xn[s];
    }
    vec_apply<R>(F, ns, v);
    vec_store<R>(xs + (size_t)i * ns, v, ns);
#pragma unroll
    for (int s = 0; s < R; ++s) xn[s] = v[s];
  }
}

// Block-triangular solves with the inverses of a block-diagonal factorization (btddod_matrix_kernels.cpp:386-428):
//   lower  x_0 = F_0 b_0,               x_i = F_i (b_i - sub_{i-1} o x_{i-1})
//   upper  x_{nb-1} = F_{nb-1} b_{nb-1}, x_i = F_i (b_i - sup_i o x_{i+1})
// One warp per flamelet; F_i (column-major inverses, [points][ns*ns]) are streamed into shared memory one block
// ahead, the vector stays in registers.
template <int R>
__global__ void __launch_bounds__(32) btddod_triangle_solve_kernel(int nf, int ns, const int *offz,
                                                                   const long long *offv, const double *inverses,
                                                                   const double *values, const double *rhs, double *x,
                                                                   int upper, const int *active, int double_buffer)
{
  extern __shared__ __align__(16) unsigned char smem[];
  const int f = blockIdx.x;
  if (f >= nf || (active && !active[f])) return;
  const int z0 = offz[f], nb = offz[f + 1] - z0;
  const int bs2 = ns * ns;
  double *sm = reinterpret_cast<double *>(smem);
  SweepBuffers sb{sm, sm + (double_buffer ? bs2 : 0), double_buffer != 0, bs2};
  const double *vals = values + offv[f];
  const double *sub = vals + (size_t)nb * bs2;
  const double *sup = sub + (size_t)(nb - 1) * ns;
  const double *b = rhs + (size_t)z0 * ns;
  double *xs = x + (size_t)z0 * ns;
  auto blk = [&](int t) { return upper ? nb - 1 - t : t; };
  auto fsrc = [&](int t) { return inverses + (size_t)(z0 + blk(t)) * bs2; };
  const int lane = threadIdx.x & 31;
  double xp[R];
#pragma unroll
  for (int s = 0; s < R; ++s) xp[s] = 0.;
  sb.prime(0, fsrc);
  for (int t = 0; t < nb; ++t) {
    const double *F = sb.get(t, nb - 1, 1, fsrc);
    const int i = blk(t);
    double v[R];
    vec_load<R>(v, b + (size_t)i * ns, ns);
    if (t > 0) {
      const double *cpl = upper ? sup + (size_t)i * ns : sub + (size_t)(i - 1) * ns;
#pragma unroll
      for (int s = 0; s < R; ++s) {
        const int k = lane + 32 * s;
        if (k < ns) v[s] = v[s] - cpl[k] * xp[s];
      }
    }
    vec_apply<R>(F, ns, v);
    vec_store<R>(xs + (size_t)i * ns, v, ns);
#pragma unroll
    for (int s = 0; s < R; ++s) xp[s] = v[s];
  }
}

// Inverse of every ns x ns column-major block of a list (btddod_matrix_kernels.cpp:364-373 factors each block of a
// block-diagonal matrix): one CTA per block, Gauss-Jordan with partial pivoting as in the block-Thomas
// factorization. pivots receives each block's pivot order.
__global__ void __launch_bounds__(kFactorThreads) blockdiag_inverse_kernel(int n_blocks, int ns, const double *blocks,
                                                                           double *out_inv, int *pivots)
{
  extern __shared__ __align__(16) unsigned char smem[];
  const int blkid = blockIdx.x;
  if (blkid >= n_blocks) return;
  const int bs2 = ns * ns;
  FactorShared sh(smem, ns);
  const double *A = blocks + (size_t)blkid * bs2;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < bs2; e += nt) {
    const int c = e / ns, r = e - c * ns;
    sh.buf0[r * ns + c] = A[e];
  }
  __syncthreads();
  const double *Z = cta_gj_inverse(sh.buf0, sh.buf1, ns, sh.piv, sh.pinv, sh.ws, sh.used);
  double *O = out_inv + (size_t)blkid * bs2;
  for (int e = tid; e < bs2; e += nt) {
    const int c = e / ns, r = e - c * ns;
    O[e] = Z[sh.piv[r] * ns + sh.pinv[c]];
  }
  for (int k = tid; k < ns; k += nt) pivots[(size_t)blkid * ns + k] = sh.piv[k];
}

// y_i = B_i x_i for every block of a list (btddod_matrix_kernels.cpp:167-177, and :375-384 with the inverses of a
// block-diagonal factorization): one thread per row.
__global__ void blockdiag_matvec_kernel(int n_blocks, int ns, const double *blocks, const double *x, double *y)
{
  const long long total = (long long)n_blocks * ns;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const long long bi = t / ns;
    const int r = (int)(t - bi * ns);
    const double *B = blocks + (size_t)bi * ns * ns;
    const double *xs = x + (size_t)bi * ns;
    double v = 0.;
    for (int c = 0; c < ns; ++c) v += B[r + c * ns] * xs[c];
    y[t] = v;
  }
}

// A <- matrix_scale*A + diag_scale*B over the BTDDOD values, B a block diagonal [points][ns*ns]
// (btddod_matrix_kernels.cpp:430-446): grid (chunks, flamelets), one value per thread per chunk step.
__global__ void btddod_scale_block_diag_kernel(int nf, int ns, const int *offz, const long long *offv, double *values,
                                               double ms, const double *bdiag, double ds, const int *active)
{
  const int f = blockIdx.y;
  if (f >= nf || (active && !active[f])) return;
  const int z0 = offz[f], nb = offz[f + 1] - z0;
  const long long bs2 = (long long)ns * ns;
  const long long ne = (long long)ns * (nb * ns + 2 * (nb - 1));
  double *vals = values + offv[f];
  const double *bd = bdiag + (size_t)z0 * bs2;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += (long long)gridDim.x * blockDim.x) {
    double v = __dmul_rn(vals[e], ms);
    if (e < nb * bs2) v = __dadd_rn(v, __dmul_rn(bd[e], ds));
    vals[e] = v;
  }
}

// y = A x (btddod_matrix_kernels.cpp:121-160): one thread per row of every point of every flamelet.
__global__ void btddod_matvec_kernel(int n_points, int nf, int ns, const int *offz, const long long *offv,
                                     const double *values, const double *x, double *y, const int *active)
{
  const long long total = (long long)n_points * ns;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int pt = (int)(t / ns), r = (int)(t - (long long)pt * ns);
    const int f = find_flamelet(offz, nf, pt);
    if (active && !active[f]) continue;
    const int z0 = offz[f], nb = offz[f + 1] - z0, iz = pt - z0;
    const double *vals = values + offv[f];
    const double *D = vals + (size_t)iz * ns * ns;
    const double *xs = x + (size_t)z0 * ns;
    double v = 0.;
    for (int c = 0; c < ns; ++c) v += D[r + c * ns] * xs[(size_t)iz * ns + c];
    const double *sub = vals + (size_t)nb * ns * ns;
    const double *sup = sub + (size_t)(nb - 1) * ns;
    if (iz >= 1) v += sub[(size_t)(iz - 1) * ns + r] * xs[(size_t)(iz - 1) * ns + r];
    if (iz <= nb - 2) v += sup[(size_t)iz * ns + r] * xs[(size_t)(iz + 1) * ns + r];
    y[t] = v;
  }
}

// A <- matrix_scale*A + diag_scale*diag(d) (btddod_matrix_kernels.cpp:448-465): grid (chunks, flamelets), one
// value per thread per chunk step, the diagonal entries of the blocks getting the added term.
__global__ void btddod_scale_diag_kernel(int nf, int ns, const int *offz, const long long *offv, double *values,
                                         double ms, const double *diag, double ds, const int *active)
{
  const int f = blockIdx.y;
  if (f >= nf || (active && !active[f])) return;
  const int z0 = offz[f], nb = offz[f + 1] - z0;
  const long long bs2 = (long long)ns * ns;
  const long long ne = (long long)ns * (nb * ns + 2 * (nb - 1));
  double *vals = values + offv[f];
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += (long long)gridDim.x * blockDim.x) {
    double v = __dmul_rn(vals[e], ms);
    if (e < nb * bs2) {
      const long long iz = e / bs2, rem = e - iz * bs2;
      if (rem % (ns + 1) == 0) v = __dadd_rn(v, __dmul_rn(ds, diag[(size_t)(z0 + iz) * ns + rem / (ns + 1)]));
    }
    vals[e] = v;
  }
}

int launch_points(HostMech &hm, FlmParams &p, bool jac, cudaStream_t st)
{
  const int G = 32;
  const auto &progs = hm.programs_for(G);
  p.m = hm.dm;
  p.blob = hm.d_blob;
  p.status = hm.d_status;
  p.L = hm.sl;
  p.pg.w = progs.progs[0];
  p.pg.full = progs.progs[1];
  p.pg.j = progs.progs[2];
  int dev, smem_max, nsm;
  CUDA_THROW(cudaGetDevice(&dev));
  CUDA_THROW(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  CUDA_THROW(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const size_t per = (size_t)((jac ? hm.sl.total : hm.sl.total_rhs) + hm.dm.ns + 2) * 8;
  const size_t avail = (size_t)smem_max - hm.dm.blob_bytes - 64;
  int groups = (int)std::min<size_t>(avail / per, 256 / G);
  if (groups < 1) throw sf_error(SF_ERR_UNSUPPORTED, "mechanism too large for the flamelet kernels");
  p.groups_per_cta = groups;
  const size_t smem = hm.dm.blob_bytes + per * groups;
  void (*k)(const FlmParams) = jac ? flamelet_point_kernel<32, true> : flamelet_point_kernel<32, false>;
  ensure_dynamic_smem((const void *)k, smem);
  const int bps = std::max(1, (int)((size_t)smem_max / smem));
  const int grid = (int)std::max<long long>(1, std::min<long long>(((long long)p.n_points + groups - 1) / groups,
                                                                   (long long)nsm * bps));
  k<<<grid, groups * G, smem, st>>>(p);
  CUDA_THROW(cudaGetLastError());
  return SF_OK;
}

void fill(FlmParams &p, const sf_flamelet_batch *fb)
{
  if (!fb || fb->n_flamelets < 1 || !fb->offsets_z || !fb->offsets_v || !fb->offsets_z_host || !fb->oxy_state ||
      !fb->fuel_state || !fb->cmajor || !fb->csub || !fb->csup || !fb->mcoeff || !fb->ncoeff || !fb->chi)
    throw sf_error(SF_ERR_INVALID_ARGUMENT, "bad flamelet batch");
  p.n_flamelets = fb->n_flamelets;
  p.n_points = fb->offsets_z_host[fb->n_flamelets];
  for (int f = 0; f < fb->n_flamelets; ++f)
    if (fb->offsets_z_host[f + 1] - fb->offsets_z_host[f] < 2)
      throw sf_error(SF_ERR_INVALID_ARGUMENT, "every flamelet needs at least two interior points");
  p.offz = fb->offsets_z;
  p.offv = fb->offsets_v;
  p.pressure = fb->pressure;
  p.oxy = fb->oxy_state;
  p.fuel = fb->fuel_state;
  p.cmajor = fb->cmajor;
  p.csub = fb->csub;
  p.csup = fb->csup;
  p.mc = fb->mcoeff;
  p.nc = fb->ncoeff;
  p.chi = fb->chi;
  if (fb->T_convection || fb->h_convection || fb->T_radiation || fb->h_radiation) {
    if (!fb->T_convection || !fb->h_convection || !fb->T_radiation || !fb->h_radiation)
      throw sf_error(SF_ERR_INVALID_ARGUMENT, "nonadiabatic flamelets need all four heat-loss arrays");
    p.Tconv = fb->T_convection;
    p.hconv = fb->h_convection;
    p.Trad = fb->T_radiation;
    p.hrad = fb->h_radiation;
    p.scaled_heat_loss = fb->use_scaled_heat_loss ? 1 : 0;
  }
  p.eflux = fb->include_enthalpy_flux;
  p.vcp = fb->include_variable_cp;
  p.active = fb->active;
  p.prefactors = fb->prefactor;
}

template <class F>
int guarded(F f)
{
  try {
    return f();
  } catch (sf_error &e) {
    set_error(e.what());
    return e.code;
  }
}

int check_launch()
{
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(cudaGetErrorString(e));
    return SF_ERR_CUDA;
  }
  return SF_OK;
}

template <int R>
int launch_solve(int nf, int ns, const int *offz, const long long *offv, const double *values,
                 const double *l_values, const int *pivots, const double *rhs, double *out_x, const int *active,
                 cudaStream_t st)
{
  int dev, smem_max;
  CUDA_THROW(cudaGetDevice(&dev));
  CUDA_THROW(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  // two warps, each with two staged blocks (one when four do not fit), plus the middle block's feed vectors
  const size_t extra = (size_t)3 * ns * 8;
  const int dbl = (size_t)4 * ns * ns * 8 + extra <= (size_t)smem_max ? 1 : 0;
  const size_t smem = (size_t)(dbl ? 4 : 2) * ns * ns * 8 + extra;
  if (smem > (size_t)smem_max)
    throw sf_error(SF_ERR_UNSUPPORTED, "block size too large for the shared-memory block-Thomas solve");
  ensure_dynamic_smem((const void *)btddod_solve_kernel<R>, smem);
  btddod_solve_kernel<R><<<nf, 64, smem, st>>>(nf, ns, offz, offv, values, l_values, pivots, rhs, out_x, active,
                                               dbl);
  return check_launch();
}

template <int R>
int launch_triangle(int nf, int ns, const int *offz, const long long *offv, const double *inverses,
                    const double *values, const double *rhs, double *out_x, int upper, const int *active,
                    cudaStream_t st)
{
  int dev, smem_max;
  CUDA_THROW(cudaGetDevice(&dev));
  CUDA_THROW(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  const int dbl = (size_t)2 * ns * ns * 8 <= (size_t)smem_max ? 1 : 0;
  const size_t smem = (size_t)(dbl ? 2 : 1) * ns * ns * 8;
  if (smem > (size_t)smem_max)
    throw sf_error(SF_ERR_UNSUPPORTED, "block size too large for the shared-memory triangular solve");
  ensure_dynamic_smem((const void *)btddod_triangle_solve_kernel<R>, smem);
  btddod_triangle_solve_kernel<R><<<nf, 32, smem, st>>>(nf, ns, offz, offv, inverses, values, rhs, out_x, upper,
                                                         active, dbl);
  return check_launch();
}

}  // namespace
}  // namespace sfgb

using namespace sfgb;

extern "C" {

int sf_btddod_blockdiag_factor_batch(int n_blocks, int ns, const double *blocks, double *out_inverses,
                                     int *out_pivots, void *stream)
{
  if (n_blocks < 0 || ns < 1 || ns > 128 || (n_blocks > 0 && (!blocks || !out_inverses || !out_pivots))) {
    set_error("sf_btddod_blockdiag_factor_batch: bad argument");
    return SF_ERR_INVALID_ARGUMENT;
  }
  if (n_blocks == 0) return SF_OK;
  const size_t smem = factor_smem_bytes(ns);
  return guarded([&] {
    int dev, smem_max;
    CUDA_THROW(cudaGetDevice(&dev));
    CUDA_THROW(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    if (smem > (size_t)smem_max)
      throw sf_error(SF_ERR_UNSUPPORTED, "block size too large for the shared-memory block inverse");
    ensure_dynamic_smem((const void *)blockdiag_inverse_kernel, smem);
    blockdiag_inverse_kernel<<<n_blocks, kFactorThreads, smem, (cudaStream_t)stream>>>(n_blocks, ns, blocks,
                                                                                        out_inverses, out_pivots);
    return check_launch();
  });
}

int sf_btddod_blockdiag_matvec_batch(int n_blocks, int ns, const double *blocks, const double *x, double *out_y,
                                     void *stream)
{
  if (n_blocks < 0 || ns < 1 || (n_blocks > 0 && (!blocks || !x || !out_y))) {
    set_error("sf_btddod_blockdiag_matvec_batch: bad argument");
    return SF_ERR_INVALID_ARGUMENT;
  }
  if (n_blocks == 0) return SF_OK;
  const long long rows = (long long)n_blocks * ns;
  const int grid = (int)std::max<long long>(1, std::min<long long>((rows + 255) / 256, 152LL * 16));
  blockdiag_matvec_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(n_blocks, ns, blocks, x, out_y);
  return check_launch();
}

int sf_btddod_triangle_solve_batch(int nf, int ns, const int *offz, const long long *offv, const int *offz_host,
                                   const double *inverses, const double *values, const double *rhs, double *out_x,
                                   int upper, const int *active, void *stream)
{
  if (nf < 1 || ns < 1 || ns > 128 || !offz || !offv || !inverses || !values || !rhs || !out_x) {
    set_error("sf_btddod_triangle_solve_batch: bad argument");
    return SF_ERR_INVALID_ARGUMENT;
  }
  (void)offz_host;
  cudaStream_t st = (cudaStream_t)stream;
  const int up = upper ? 1 : 0;
  return guarded([&] {
    if (ns <= 32) return launch_triangle<1>(nf, ns, offz, offv, inverses, values, rhs, out_x, up, active, st);
    if (ns <= 64) return launch_triangle<2>(nf, ns, offz, offv, inverses, values, rhs, out_x, up, active, st);
    if (ns <= 96) return launch_triangle<3>(nf, ns, offz, offv, inverses, values, rhs, out_x, up, active, st);
    return launch_triangle<4>(nf, ns, offz, offv, inverses, values, rhs, out_x, up, active, st);
  });
}

int sf_btddod_scale_and_add_block_diagonal_batch(int nf, int ns, const int *offz, const long long *offv,
                                                 const int *offz_host, double *values, double ms,
                                                 const double *block_diag, double ds, const int *active,
                                                 void *stream)
{
  if (nf < 1 || ns < 1 || nf > 65535 || !offz || !offv || !offz_host || !values || !block_diag) {
    set_error("sf_btddod_scale_and_add_block_diagonal_batch: bad argument");
    return SF_ERR_INVALID_ARGUMENT;
  }
  long long max_ne = 0;
  for (int f = 0; f < nf; ++f) {
    const long long nb = offz_host[f + 1] - offz_host[f];
    max_ne = std::max(max_ne, (long long)ns * (nb * ns + 2 * (nb - 1)));
  }
  const int chunks = (int)std::max<long long>(1, std::min<long long>((max_ne + 1023) / 1024, 1024));
  btddod_scale_block_diag_kernel<<<dim3(chunks, nf), 256, 0, (cudaStream_t)stream>>>(nf, ns, offz, offv, values, ms,
                                                                                     block_diag, ds, active);
  return check_launch();
}

int sf_flamelet_stencils(const sf_mech *mech, const double *dz, int nzi, const double *chi, const double *invLe,
                         double *cmaj, double *csub, double *csup, double *mc, double *nc)
{
  if (!mech || !dz || !chi || !invLe || !cmaj || !csub || !csup || !mc || !nc || nzi < 1) {
    set_error("sf_flamelet_stencils: bad argument");
    return SF_ERR_INVALID_ARGUMENT;
  }
  const int ns = mech->m.dm.ns;
  for (int i = 0; i < nzi; ++i) {  // flamelet_kernels.cpp:31-48
    const double dzt = dz[i] + dz[i + 1];
    for (int l = 0; l < ns; ++l) {
      cmaj[i * ns + l] = -chi[1 + i] / (dz[i] * dz[i + 1]) * invLe[l];
      csub[i * ns + l] = chi[1 + i] / (dzt * dz[i]) * invLe[l];
      csup[i * ns + l] = chi[1 + i] / (dzt * dz[i + 1]) * invLe[l];
    }
    nc[i] = 1 / (dz[i] + dz[i + 1]);
    mc[i] = -nc[i];
  }
  return SF_OK;
}

int sf_flamelet_jac_indices(const sf_mech *mech, int nzi, int *rows, int *cols)
{
  if (!mech || !rows || !cols || nzi < 1) {
    set_error("sf_flamelet_jac_indices: bad argument");
    return SF_ERR_INVALID_ARGUMENT;
  }
  const int ns = mech->m.dm.ns;
  int idx = 0;  // flamelet_kernels.cpp:50-90
  for (int iz = 0; iz < nzi; ++iz)
    for (int iq = 0; iq < ns; ++iq)
      for (int jq = 0; jq < ns; ++jq) {
        rows[idx] = iz * ns + jq;
        cols[idx] = iz * ns + iq;
        ++idx;
      }
  for (int iz = 1; iz < nzi; ++iz)
    for (int iq = 0; iq < ns; ++iq) {
      rows[idx] = iz * ns + iq;
      cols[idx] = iz * ns + iq - ns;
      ++idx;
    }
  for (int iz = 0; iz < nzi - 1; ++iz)
    for (int iq = 0; iq < ns; ++iq) {
      rows[idx] = iz * ns + iq;
      cols[idx] = iz * ns + iq + ns;
      ++idx;
    }
  return SF_OK;
}

int sf_flamelet_rhs_batch(const sf_mech *mech, const sf_flamelet_batch *fb, const double *state, double *out_rhs,
                          void *stream)
{
  return guarded([&] {
    if (!mech || !state || !out_rhs) throw sf_error(SF_ERR_INVALID_ARGUMENT, "bad argument");
    FlmParams p{};
    fill(p, fb);
    p.state = state;
    p.out_rhs = out_rhs;
    return launch_points(const_cast<HostMech &>(mech->m), p, false, (cudaStream_t)stream);
  });
}

size_t sf_flamelet_jac_workspace_size(const sf_mech *mech, int eigenvalues)
{
  return mech && eigenvalues ? 256 : 0;
}

int sf_flamelet_jac_batch(const sf_mech *mech, const sf_flamelet_batch *fb, const double *state, int rates_option,
                          int scale_and_offset, double prefactor, double diffterm, double *out_expeig,
                          double *out_values, void *workspace, size_t workspace_bytes, void *stream)
{
  return guarded([&] {
    if (!mech || !state || !out_values) throw sf_error(SF_ERR_INVALID_ARGUMENT, "bad argument");
    if (out_expeig && (!workspace || workspace_bytes < sf_flamelet_jac_workspace_size(mech, 1)))
      throw sf_error(SF_ERR_WORKSPACE, "eigenvalue bounds need the workspace sf_flamelet_jac_workspace_size reports");
    if (rates_option < 0 || rates_option > 2)
      throw sf_error(SF_ERR_INVALID_ARGUMENT, "rates option must be 0, 1 or 2");
    if (out_expeig && scale_and_offset)
      throw sf_error(SF_ERR_INVALID_ARGUMENT, "eigenvalue bounds need scale_and_offset = 0 (as flamelet.py calls it)");
    FlmParams p{};
    fill(p, fb);
    p.state = state;
    p.out_values = out_values;
    p.scale_offset = scale_and_offset;
    p.rates_option = rates_option;
    p.prefactor = prefactor;
    p.eflux_store = out_expeig;
    HostMech &hm = const_cast<HostMech &>(mech->m);
    cudaStream_t st = (cudaStream_t)stream;
    launch_points(hm, p, true, st);
    if (out_expeig) {
      const int ns = hm.dm.ns;
      int dev, smem_max, nsm;
      CUDA_THROW(cudaGetDevice(&dev));
      CUDA_THROW(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
      CUDA_THROW(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
      const size_t per = (size_t)(ns * ns + 2 * ns) * 8;
      const int warps = (int)std::min<size_t>(8, (size_t)smem_max / per);
      if (warps < 1) throw sf_error(SF_ERR_UNSUPPORTED, "block too large for the eigenvalue kernel");
      ensure_dynamic_smem((const void *)flamelet_expeig_kernel, per * warps);
      int per_sm = 0;
      CUDA_THROW(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, flamelet_expeig_kernel, 32 * warps,
                                                               per * warps));
      const int grid = (int)std::max<long long>(1, std::min<long long>((long long)nsm * std::max(1, per_sm),
                                                                       ((long long)p.n_points + warps - 1) / warps));
      // the points are handed out by an atomic counter in the caller's workspace, zeroed on the stream first
      int *counter = static_cast<int *>(workspace);
      CUDA_THROW(cudaMemsetAsync(counter, 0, sizeof(int), st));
      flamelet_expeig_kernel<<<grid, 32 * warps, per * warps, st>>>(p.n_points, p.n_flamelets, ns, p.offz, p.offv,
                                                                    out_values, p.cmajor, diffterm, fb->diffterm,
                                                                    fb->active, out_expeig, hm.d_status, warps,
                                                                    counter);
      CUDA_THROW(cudaGetLastError());
    }
    return SF_OK;
  });
}

int sf_btddod_factor_batch(int nf, int ns, const int *offz, const long long *offv, const int *offz_host,
                           double *values, double *l_values, int *pivots, const int *active, void *stream)
{
  if (nf < 1 || ns < 1 || ns > 128 || !offz || !offv || !values || !l_values || !pivots) {
    set_error("sf_btddod_factor_batch: bad argument");
    return SF_ERR_INVALID_ARGUMENT;
  }
  (void)offz_host;
  const size_t smem = factor_smem_bytes(ns);
  return guarded([&] {
    int dev, smem_max;
    CUDA_THROW(cudaGetDevice(&dev));
    CUDA_THROW(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    if (smem > (size_t)smem_max)
      throw sf_error(SF_ERR_UNSUPPORTED, "block size too large for the shared-memory block-Thomas factorization");
    if ((long long)nf * 2 > 0x7fffffffLL) throw sf_error(SF_ERR_INVALID_ARGUMENT, "too many flamelets");
    int nsm;
    CUDA_THROW(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    // Each CTA is bound by its SM's FP64 unit. When every CTA can have an SM of its own, ask for more than half an
    // SM's shared memory so that no two CTAs share one (the block scheduler may otherwise pair them).
    const size_t smem_launch = 2LL * nf <= nsm ? std::max(smem, (size_t)smem_max / 2 + 1024) : smem;
    ensure_dynamic_smem((const void *)btddod_factor_kernel, smem_launch);
    ensure_dynamic_smem((const void *)btddod_middle_kernel, smem);
    cudaStream_t st = (cudaStream_t)stream;
    btddod_factor_kernel<<<2 * nf, kFactorThreads, smem_launch, st>>>(nf, ns, offz, offv, values, l_values, pivots,
                                                                      active);
    CUDA_THROW(cudaGetLastError());
    btddod_middle_kernel<<<nf, kFactorThreads, smem, st>>>(nf, ns, offz, offv, values, l_values, pivots, active);
    return check_launch();
  });
}

int sf_btddod_solve_batch(int nf, int ns, const int *offz, const long long *offv, const int *offz_host,
                          const double *values, const double *l_values, const int *pivots, const double *rhs,
                          double *out_x, const int *active, void *stream)
{
  if (nf < 1 || ns < 1 || ns > 128 || !offz || !offv || !values || !l_values || !pivots || !rhs || !out_x) {
    set_error("sf_btddod_solve_batch: bad argument");
    return SF_ERR_INVALID_ARGUMENT;
  }
  (void)offz_host;
  cudaStream_t st = (cudaStream_t)stream;
  return guarded([&] {
    if (ns <= 32) return launch_solve<1>(nf, ns, offz, offv, values, l_values, pivots, rhs, out_x, active, st);
    if (ns <= 64) return launch_solve<2>(nf, ns, offz, offv, values, l_values, pivots, rhs, out_x, active, st);
    if (ns <= 96) return launch_solve<3>(nf, ns, offz, offv, values, l_values, pivots, rhs, out_x, active, st);
    return launch_solve<4>(nf, ns, offz, offv, values, l_values, pivots, rhs, out_x, active, st);
  });
}

int sf_btddod_matvec_batch(int nf, int ns, const int *offz, const long long *offv, const int *offz_host,
                           const double *values, const double *x, double *out_y, const int *active, void *stream)
{
  if (nf < 1 || ns < 1 || !offz || !offv || !offz_host || !values || !x || !out_y) {
    set_error("sf_btddod_matvec_batch: bad argument");
    return SF_ERR_INVALID_ARGUMENT;
  }
  const int npts = offz_host[nf];
  const long long rows = (long long)npts * ns;
  const int grid = (int)std::max<long long>(1, std::min<long long>((rows + 255) / 256, 152LL * 16));
  btddod_matvec_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(npts, nf, ns, offz, offv, values, x, out_y, active);
  return check_launch();
}

int sf_btddod_scale_and_add_diagonal_batch(int nf, int ns, const int *offz, const long long *offv,
                                           const int *offz_host, double *values, double ms, const double *diag,
                                           double ds, const int *active, void *stream)
{
  if (nf < 1 || ns < 1 || nf > 65535 || !offz || !offv || !offz_host || !values || !diag) {
    set_error("sf_btddod_scale_and_add_diagonal_batch: bad argument");
    return SF_ERR_INVALID_ARGUMENT;
  }
  long long max_ne = 0;
  for (int f = 0; f < nf; ++f) {
    const long long nb = offz_host[f + 1] - offz_host[f];
    max_ne = std::max(max_ne, (long long)ns * (nb * ns + 2 * (nb - 1)));
  }
  const int chunks = (int)std::max<long long>(1, std::min<long long>((max_ne + 1023) / 1024, 1024));
  btddod_scale_diag_kernel<<<dim3(chunks, nf), 256, 0, (cudaStream_t)stream>>>(nf, ns, offz, offv, values, ms, diag,
                                                                               ds, active);
  return check_launch();
}

}  // extern "C"
