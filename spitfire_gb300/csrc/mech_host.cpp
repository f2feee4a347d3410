// Host side of the mechanism: Griffon's finalize derivations, packing into the device blob, and the construction
// of the load-balanced gather programs used by the Jacobian kernels.
//
// Derivations restated from src/spitfire/griffon/src/chemistry_setup.cpp:
//   NASA7 storage scaled by R and 1/2, 1/6, 1/12, 1/20          (:102-130)
//   third-body efficiencies stored as invM*(eff - default)        (:406-419)
//   net stoichiometry over species in ascending index order       (:459-541), 2 <= n_net <= 8 enforced
//   dense/sparse sensitivity classification                       (:543-602)
//   rate-constant temperature form and Troe term flags            (:670-730)
#include "sf_internal.h"
#include "exp_table.h"

#include <algorithm>
#include <cmath>
#include <map>
#include <numeric>
#include <stdexcept>
#include <string>

namespace sfgb {

static int pack_sp(int s, int hi) { return (s & 0xFFFF) | (hi << 16); }

HostMech::~HostMech()
{
  for (auto &kv : programs) {
    for (auto &p : kv.second.progs)
      if (p.items) cudaFree((void *)p.items);
  }
  if (d_blob) cudaFree(d_blob);
  if (d_status) cudaFree(d_status);
  for (cudaEvent_t e : events) cudaEventDestroy(e);
  if (copy_stream) cudaStreamDestroy(copy_stream);
}

void HostMech::build(const sf_mech_desc *d)
{
  const int ns = d->n_species, nr = d->n_reactions;
  if (ns < 2 || ns > kMaxSpecies) throw sf_error(SF_ERR_INVALID_ARGUMENT, "n_species must be in [2, 1024]");
  if (nr < 0) throw sf_error(SF_ERR_INVALID_ARGUMENT, "n_reactions < 0");
  DevMech &m = dm;
  m = DevMech{};
  m.ns = ns;
  m.nr = nr;
  m.Ru = d->gas_constant;
  m.invRu = 1. / d->gas_constant;
  m.pref = d->ref_pressure;

  // ---------------- species
  invmw.resize(ns);
  mw.assign(d->molecular_weights, d->molecular_weights + ns);
  for (int i = 0; i < ns; ++i) invmw[i] = 1. / mw[i];
  std::vector<double> nasa(ns * 15, 0.), tmin(ns), tmax(ns);
  std::vector<int> thermo(ns);
  m.all_nasa7 = 1;
  for (int k = 0; k < ns; ++k) {
    const double *t = d->thermo_coefs + 20 * k;
    double *c = &nasa[15 * k];
    thermo[k] = d->thermo_kind[k];
    if (thermo[k] == SF_THERMO_NASA7) {
      tmin[k] = t[0];
      tmax[k] = t[2];
      c[0] = t[1];
      for (int j = 0; j < 7; ++j) c[1 + j] = t[10 + j] * m.Ru;
      for (int j = 0; j < 7; ++j) c[8 + j] = t[3 + j] * m.Ru;
      c[2] /= 2.; c[3] /= 6.; c[4] /= 12.; c[5] /= 20.;
      c[9] /= 2.; c[10] /= 6.; c[11] /= 12.; c[12] /= 20.;
    } else if (thermo[k] == SF_THERMO_CONST) {
      m.all_nasa7 = 0;
      tmin[k] = t[0];
      tmax[k] = t[1];
      c[0] = t[2]; c[1] = t[3]; c[2] = t[4]; c[3] = t[5];
      c[4] = std::log(t[2]);
    } else {
      throw sf_error(SF_ERR_UNSUPPORTED, "NASA9 thermodynamics is not supported by the GPU kernels");
    }
  }

  // ---------------- reactions
  rx.clear();
  rx.resize(nr);
  int n_fall = 0, n_dense = 0;
  for (int r = 0; r < nr; ++r) {
    HRxn &x = rx[r];
    x.kind = d->rxn_kind[r];
    if (x.kind < SF_RXN_SIMPLE || x.kind > SF_RXN_TROE)
      throw sf_error(SF_ERR_MECHANISM, "reaction " + std::to_string(r) + ": unknown kind");
    x.reversible = d->rxn_reversible[r] != 0;
    for (int j = 0; j < 3; ++j) x.kf[j] = d->rxn_kfwd[3 * r + j];
    if (x.kind >= SF_RXN_LINDEMANN) {
      for (int j = 0; j < 3; ++j) x.kp[j] = d->rxn_kflf[3 * r + j];
      x.fall = n_fall++;
    }
    if (x.kind == SF_RXN_TROE)
      for (int j = 0; j < 4; ++j) x.troe[j] = d->rxn_troe[4 * r + j];
    x.beff = x.kind != SF_RXN_SIMPLE ? d->rxn_default_eff[r] : 0.;
    for (int i = d->reac_offsets[r]; i < d->reac_offsets[r + 1]; ++i) {
      x.reac.push_back(d->reac_species[i]);
      x.reac_nu.push_back(d->reac_stoich[i]);
    }
    for (int i = d->prod_offsets[r]; i < d->prod_offsets[r + 1]; ++i) {
      x.prod.push_back(d->prod_species[i]);
      x.prod_nu.push_back(d->prod_stoich[i]);
    }
    if (x.kind != SF_RXN_SIMPLE)
      for (int i = d->eff_offsets[r]; i < d->eff_offsets[r + 1]; ++i) {
        const int s = d->eff_species[i];
        x.tb.push_back(s);
        x.tbeff.push_back(invmw[s] * (d->eff_values[i] - x.beff));
      }
    if (d->order_offsets && d->order_offsets[r + 1] > d->order_offsets[r]) {
      x.has_orders = true;
      for (int i = d->order_offsets[r]; i < d->order_offsets[r + 1]; ++i) {
        x.ord.push_back(d->order_species[i]);
        x.ord_val.push_back(d->order_values[i]);
      }
    }
    for (const auto *v : {&x.reac, &x.prod, &x.tb, &x.ord})
      for (int s : *v)
        if (s < 0 || s >= ns) throw sf_error(SF_ERR_MECHANISM, "reaction " + std::to_string(r) + ": bad species index");
    std::map<int, int> net;
    x.sum_nu = 0;
    for (size_t i = 0; i < x.reac.size(); ++i) { net[x.reac[i]] += x.reac_nu[i]; x.sum_nu += x.reac_nu[i]; }
    for (size_t i = 0; i < x.prod.size(); ++i) { net[x.prod[i]] -= x.prod_nu[i]; x.sum_nu -= x.prod_nu[i]; }
    for (auto &kv : net)
      if (kv.second != 0) { x.net.push_back(kv.first); x.net_nu.push_back(kv.second); }
    if (x.net.size() < 2 || x.net.size() > (size_t)kMaxNet)
      throw sf_error(SF_ERR_MECHANISM, "reaction " + std::to_string(r) + ": bad number of net reacting species (n < 2 or n > 8)");
    x.sum_reac_nu = 0;
    for (int v : x.reac_nu) x.sum_reac_nu += std::abs(v);
    x.sum_prod_nu = 0;
    for (int v : x.prod_nu) x.sum_prod_nu += std::abs(v);
    // coefficients and their sums are read through the device's table of small integers
    if (x.sum_reac_nu > 127 || x.sum_prod_nu > 127)
      throw sf_error(SF_ERR_MECHANISM, "reaction " + std::to_string(r) + ": stoichiometric coefficients above 127");
    if (std::abs(x.kf[2]) < 1.e-6) {
      if (std::abs(x.kf[1]) < 1.e-6) x.kform = 0;
      else if (std::abs(x.kf[1] - 1) < 1.e-6) x.kform = 1;
      else if (std::abs(x.kf[1] - 2) < 1.e-6) x.kform = 2;
      else if (std::abs(x.kf[1] + 1) < 1.e-6) x.kform = 3;
      else x.kform = 4;
    } else x.kform = 4;
    if (x.kind == SF_RXN_TROE) {
      x.troe_terms = (std::abs(x.troe[1]) > 1.e-8 ? 1 : 0) | (std::abs(x.troe[2]) > 1.e-8 ? 2 : 0) |
                     (std::abs(x.troe[3]) > 1.e-8 ? 4 : 0);
      if (!x.troe_terms) throw sf_error(SF_ERR_MECHANISM, "no troe terms flagged for evaluation");
    }
    // Jacobian slots: every species other than the last whose Y column receives a sparse contribution from this
    // reaction (reactants, products, third bodies, special-order species). The closure species ns-1 contributes
    // a constant to every column (beta), third-body/falloff reactions a term proportional to u_s (alpha).
    auto pos = [](const std::vector<int> &v, int s) {
      for (size_t i = 0; i < v.size(); ++i) if (v[i] == s) return (int)i;
      return -1;
    };
    std::vector<int> slots;
    for (const auto *v : {&x.reac, &x.prod, &x.tb, &x.ord})
      for (int s : *v)
        if (s != ns - 1 && std::find(slots.begin(), slots.end(), s) == slots.end()) slots.push_back(s);
    std::sort(slots.begin(), slots.end());
    x.slots.clear();
    for (int s : slots) {
      const int rp = pos(x.reac, s);
      const int pp = pos(x.prod, s);
      const int tp = pos(x.tb, s);
      const int op = pos(x.ord, s);
      if (rp < 0 && pp < 0 && tp < 0 && op < 0) continue;
      x.slots.push_back(s | ((rp + 1) << 16) | ((pp + 1) << 20) | ((tp + 1) << 24) | ((op + 1) << 28));
    }
    bool last_involved = false;
    for (const auto *v : {&x.reac, &x.prod, &x.tb, &x.ord})
      for (int s : *v) if (s == ns - 1) last_involved = true;
    x.dense = (x.kind != SF_RXN_SIMPLE) || last_involved;
    x.dense_idx = x.dense ? n_dense++ : -1;
  }
  // Device order: reactions grouped by kind and, within a kind, by their number of Jacobian slots (stable).
  // Lanes of a state group take reactions in strides of the group width, so the per-reaction slot loop of a
  // group iteration then runs about as many times for every lane. Per-reaction outputs map back through i_orig.
  std::vector<int> order(nr);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    if (rx[a].kind != rx[b].kind) return rx[a].kind < rx[b].kind;
    return rx[a].slots.size() < rx[b].slots.size();
  });
  {
    std::vector<HRxn> sorted(nr);
    for (int k = 0; k < nr; ++k) sorted[k] = std::move(rx[order[k]]);
    rx = std::move(sorted);
    n_fall = 0;
    n_dense = 0;
    for (HRxn &x : rx) {
      x.fall = x.kind >= SF_RXN_LINDEMANN ? n_fall++ : -1;
      x.dense_idx = x.dense ? n_dense++ : -1;
    }
  }
  orig_index = order;
  m.n_fall = n_fall;
  m.n_dense = n_dense;

  // ---------------- pack the blob
  std::vector<double> D;
  std::vector<int> I;
  auto dsec = [&](int n) { const int o = (int)D.size(); D.resize(D.size() + std::max(n, 0), 0.); return o; };
  auto isec = [&](int n) { const int o = (int)I.size(); I.resize(I.size() + std::max(n, 0), 0); return o; };
  m.d_nasa = dsec(15 * ns);
  std::copy(nasa.begin(), nasa.end(), D.begin() + m.d_nasa);
  m.d_tmin = dsec(ns);
  m.d_tmax = dsec(ns);
  m.d_invmw = dsec(ns);
  m.d_mw = dsec(ns);
  m.d_u = dsec(ns);
  for (int i = 0; i < ns; ++i) {
    D[m.d_tmin + i] = tmin[i];
    D[m.d_tmax + i] = tmax[i];
    D[m.d_invmw + i] = invmw[i];
    D[m.d_mw + i] = mw[i];
    D[m.d_u + i] = invmw[i] - invmw[ns - 1];
  }
  m.d_kf = dsec(3 * nr);
  m.d_kp = dsec(3 * n_fall);
  m.d_troe = dsec(4 * n_fall);
  m.d_beff = dsec(nr);
  for (int r = 0; r < nr; ++r) {
    const HRxn &x = rx[r];
    for (int j = 0; j < 3; ++j) D[m.d_kf + 3 * r + j] = x.kf[j];
    if (x.fall >= 0) {
      for (int j = 0; j < 3; ++j) D[m.d_kp + 3 * x.fall + j] = x.kp[j];
      for (int j = 0; j < 4; ++j) D[m.d_troe + 4 * x.fall + j] = x.troe[j];
    }
    D[m.d_beff + r] = x.beff;
  }
  int ntb = 0, nnet = 0, nord = 0, nslot = 0, nreac = 0, nprod = 0;
  for (const auto &x : rx) {
    ntb += (int)x.tb.size(); nnet += (int)x.net.size(); nord += (int)x.ord.size(); nslot += (int)x.slots.size();
    nreac += (int)x.reac.size(); nprod += (int)x.prod.size();
  }
  m.n_slots = nslot;
  m.n_net_total = nnet;
  m.d_tbeff = dsec(ntb);
  m.d_netc = dsec(nnet);
  m.d_ord = dsec(nord);
  m.d_one = dsec(1);
  D[m.d_one] = 1.;
  m.d_smallint = dsec(64);
  for (int k = 0; k < 64; ++k) D[m.d_smallint + k] = k - 32;
  while (D.size() % 2) D.push_back(0.);  // 16-byte boundary: the table is read as (head, tail) pairs
  m.d_exptab = dsec(128);
  std::copy(kExpTable, kExpTable + 128, D.begin() + m.d_exptab);
  m.i_info = isec(nr);
  m.i_orig = isec(nr);
  for (int r = 0; r < nr; ++r) I[m.i_orig + r] = orig_index[r];
  m.i_sums = isec(nr);
  m.i_fall = isec(nr);
  m.i_dense = isec(nr);
  m.i_reac_off = isec(nr + 1); m.i_reac = isec(nreac);
  m.i_prod_off = isec(nr + 1); m.i_prod = isec(nprod);
  m.i_net_off = isec(nr + 1); m.i_net = isec(nnet);
  m.i_tb_off = isec(nr + 1); m.i_tb = isec(ntb);
  m.i_ord_off = isec(nr + 1); m.i_ord = isec(nord);
  m.i_slot_off = isec(nr + 1); m.i_slot = isec(nslot);
  m.i_thermo = isec(ns);
  for (int i = 0; i < ns; ++i) I[m.i_thermo + i] = thermo[i];
  int cr = 0, cp = 0, cn = 0, ct = 0, co = 0, cs = 0;
  net_entry_of.assign(nr, std::vector<int>());
  slot_entry_of.assign(nr, std::vector<int>());
  for (int r = 0; r < nr; ++r) {
    const HRxn &x = rx[r];
    I[m.i_info + r] = (x.kind << RI_KIND_SHIFT) | (x.kform << RI_KFORM_SHIFT) | (x.troe_terms << RI_TROE_SHIFT) |
                      (x.reversible ? 1 << RI_REV_BIT : 0) | (x.has_orders ? 1 << RI_ORD_BIT : 0) |
                      (x.dense ? 1 << RI_DENSE_BIT : 0);
    I[m.i_sums + r] = (x.sum_nu & 0xFFFF) | ((x.sum_reac_nu & 0xFF) << 16) | ((x.sum_prod_nu & 0xFF) << 24);
    I[m.i_fall + r] = x.fall;
    I[m.i_dense + r] = x.dense_idx;
    I[m.i_reac_off + r] = cr;
    for (size_t i = 0; i < x.reac.size(); ++i) I[m.i_reac + cr++] = pack_sp(x.reac[i], x.reac_nu[i]);
    I[m.i_prod_off + r] = cp;
    for (size_t i = 0; i < x.prod.size(); ++i) I[m.i_prod + cp++] = pack_sp(x.prod[i], x.prod_nu[i]);
    I[m.i_net_off + r] = cn;
    for (size_t i = 0; i < x.net.size(); ++i) {
      I[m.i_net + cn] = pack_sp(x.net[i], x.net_nu[i] + 128);
      D[m.d_netc + cn] = -x.net_nu[i] * mw[x.net[i]];
      net_entry_of[r].push_back(cn);
      ++cn;
    }
    I[m.i_tb_off + r] = ct;
    for (size_t i = 0; i < x.tb.size(); ++i) {
      I[m.i_tb + ct] = x.tb[i];
      D[m.d_tbeff + ct] = x.tbeff[i];
      ++ct;
    }
    I[m.i_ord_off + r] = co;
    for (size_t i = 0; i < x.ord.size(); ++i) {
      I[m.i_ord + co] = pack_sp(x.ord[i], std::abs(x.ord_val[i]) > 1.e-12 ? 1 : 0);
      D[m.d_ord + co] = x.ord_val[i];
      ++co;
    }
    I[m.i_slot_off + r] = cs;
    for (size_t i = 0; i < x.slots.size(); ++i) {
      I[m.i_slot + cs] = x.slots[i];
      slot_entry_of[r].push_back(cs);
      ++cs;
    }
  }
  I[m.i_reac_off + nr] = cr; I[m.i_prod_off + nr] = cp; I[m.i_net_off + nr] = cn;
  I[m.i_tb_off + nr] = ct; I[m.i_ord_off + nr] = co; I[m.i_slot_off + nr] = cs;
  while (D.size() % 2) D.push_back(0.);  // 16-byte boundary for the int section
  while (I.size() % 4) I.push_back(0);   // 16-byte total
  m.blob_doubles = (int)D.size();
  m.blob_ints = (int)I.size();
  m.blob_bytes = m.blob_doubles * 8 + m.blob_ints * 4;
  host_dbl = D;
  host_int = I;

  // ---------------- scratch layout (RHS-only path uses the prefix up to total_rhs)
  ScratchLayout &L = sl;
  int o = 0;
  auto take = [&](int n) { const int r = o; o += (n + 1) & ~1; return r; };
  L.misc = take(16);
  L.y = take(ns); L.C = take(ns); L.eh = take(ns); L.cpv = take(ns); L.w = take(ns);
  L.gm = take(ns); L.gmi = take(ns); L.gk = take(ns);
  L.q = take(nr);
  L.total_rhs = o;
  L.dB = take(ns); L.dcp = take(ns); L.Srho = take(ns); L.ST = take(ns); L.P = take(ns); L.Q = take(ns);
  L.trow = take(ns);
  L.dqdrho = take(nr); L.dqdT = take(nr); L.E = take(nr);
  L.alpha = take(n_dense); L.beta = take(n_dense);
  L.D = take(nslot);
  L.total = o;

  // ---------------- upload
  CUDA_THROW(cudaMalloc(&d_blob, m.blob_bytes));
  std::vector<unsigned char> bytes(m.blob_bytes);
  std::memcpy(bytes.data(), D.data(), D.size() * 8);
  std::memcpy(bytes.data() + D.size() * 8, I.data(), I.size() * 4);
  CUDA_THROW(cudaMemcpy(d_blob, bytes.data(), m.blob_bytes, cudaMemcpyHostToDevice));
  CUDA_THROW(cudaMalloc(&d_status, 16));
  CUDA_THROW(cudaMemset(d_status, 0, 16));
  CUDA_THROW(cudaGetDevice(&device));
  // every gather program the kernels use, built here so that no evaluation call builds or allocates one
  for (int G : {1, 8, 16, 32}) build_programs(G);
}

const HostMech::Programs &HostMech::programs_for(int G) const
{
  auto it = programs.find(G);
  if (it == programs.end()) throw sf_error(SF_ERR_INVALID_ARGUMENT, "no gather program for this lane width");
  return it->second;
}

void ensure_dynamic_smem(const void *kernel, size_t bytes)
{
  static std::mutex mu;
  static std::map<std::pair<const void *, int>, size_t> set;
  int dev;
  CUDA_THROW(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  size_t &cur = set[{kernel, dev}];
  if (bytes <= cur) return;
  CUDA_THROW(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  cur = bytes;
}

// ------------------------------------------------------------------------------------------ gather programs
namespace {
struct Entry {
  std::vector<std::pair<uint32_t, uint32_t>> items;  // (a, b)
  uint32_t init;  // scratch index + 1, or 0
  uint32_t dst;
};

// The device runner loads operands ahead of the stores of earlier items, so a program must never read a scratch
// location that it writes (as a destination or through an entry's initial value).
void check_no_read_after_write(const std::vector<Entry> &entries)
{
  std::vector<uint32_t> written;
  for (const Entry &e : entries)
    if ((e.dst & DST_KIND_MASK) != DST_JBLOCK) written.push_back(e.dst & ~DST_KIND_MASK);
  std::sort(written.begin(), written.end());
  auto is_written = [&](uint32_t idx) { return std::binary_search(written.begin(), written.end(), idx); };
  for (const Entry &e : entries) {
    if (e.init && is_written(e.init - 1)) throw sf_error(SF_ERR_MECHANISM, "internal: gather program reads what it writes");
    for (auto &it : e.items)
      for (uint32_t ref : {it.first, it.second})
        if ((ref & REF_SCRATCH) && is_written(ref & ~REF_SCRATCH))
          throw sf_error(SF_ERR_MECHANISM, "internal: gather program reads what it writes");
  }
}

// Assignment of entries to G lanes and the interleaved item array, each lane's items padded with no-ops to a
// multiple of the device runner's batch. G > 1: longest-processing-time assignment (balanced lanes). G = 1 (one
// lane per state): entries in destination order, Jacobian entries column-major, so that each thread writes its
// Jacobian block sequentially through memory.
std::vector<GatherItem> schedule(std::vector<Entry> &entries, int G, int *len_out)
{
  check_no_read_after_write(entries);
  std::vector<int> order(entries.size());
  std::iota(order.begin(), order.end(), 0);
  if (G == 1) {
    auto key = [&](int e) {
      const uint32_t d = entries[e].dst;
      const uint64_t kind = d & DST_KIND_MASK;
      const uint64_t pos = kind == DST_JBLOCK ? (uint64_t)((d >> 15) & 0x7FFF) << 15 | (d & 0x7FFF)
                                              : (uint64_t)(d & ~DST_KIND_MASK);
      return kind << 32 | pos;
    };
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return key(a) < key(b); });
  } else {
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return entries[a].items.size() > entries[b].items.size(); });
  }
  std::vector<std::vector<int>> lane(G);
  std::vector<size_t> load(G, 0);
  for (int e : order) {
    if (entries[e].items.empty()) continue;
    int best = 0;
    for (int l = 1; l < G; ++l) if (load[l] < load[best]) best = l;
    lane[best].push_back(e);
    load[best] += entries[e].items.size();
  }
  size_t len = 0;
  for (int l = 0; l < G; ++l) len = std::max(len, load[l]);
  len = (len + GATHER_UNROLL - 1) / GATHER_UNROLL * GATHER_UNROLL;
  std::vector<GatherItem> out(len * G, GatherItem{0, 0, 0, F_NOP});
  for (int l = 0; l < G; ++l) {
    size_t j = 0;
    for (int e : lane[l]) {
      const Entry &E = entries[e];
      for (size_t k = 0; k < E.items.size(); ++k, ++j) {
        GatherItem it;
        it.a = E.items[k].first;
        it.b = E.items[k].second;
        it.dst = E.dst;
        it.flags = (k == 0 ? F_START | (E.init & INIT_MASK) : 0) | (k + 1 == E.items.size() ? F_END : 0);
        out[j * G + l] = it;
      }
    }
  }
  *len_out = (int)len;
  return out;
}
}  // namespace

void HostMech::build_programs(int G)
{
  if (programs.count(G)) return;
  const int ns = dm.ns, nr = dm.nr;
  const ScratchLayout &L = sl;
  auto S = [](int idx) { return REF_SCRATCH | (uint32_t)idx; };
  auto B = [](int idx) { return (uint32_t)idx; };
  // species -> list of (reaction, net entry) in increasing reaction order
  std::vector<std::vector<std::pair<int, int>>> by_species(ns);
  for (int r = 0; r < nr; ++r)
    for (size_t i = 0; i < rx[r].net.size(); ++i) by_species[rx[r].net[i]].push_back({r, net_entry_of[r][i]});
  Programs P;
  // program 0: production rates only  w_i = sum_r c_ir q_r
  {
    std::vector<Entry> E;
    for (int i = 0; i < ns; ++i) {
      Entry e{{}, 0, DST_SCRATCH | (uint32_t)(L.w + i)};
      for (auto &re : by_species[i]) e.items.push_back({B(dm.d_netc + re.second), S(L.q + re.first)});
      E.push_back(e);
    }
    auto items = schedule(E, G, &P.progs[0].len);
    P.host_items[0] = items;
  }
  // program 1: w, S_rho, S_T, P, Q for all species
  {
    std::vector<Entry> E;
    for (int i = 0; i < ns; ++i) {
      Entry ew{{}, 0, DST_SCRATCH | (uint32_t)(L.w + i)};
      Entry er{{}, 0, DST_SCRATCH | (uint32_t)(L.Srho + i)};
      Entry et{{}, 0, DST_SCRATCH | (uint32_t)(L.ST + i)};
      Entry ep{{}, 0, DST_SCRATCH | (uint32_t)(L.P + i)};
      Entry eq{{}, 0, DST_SCRATCH | (uint32_t)(L.Q + i)};
      for (auto &re : by_species[i]) {
        const uint32_t c = B(dm.d_netc + re.second);
        ew.items.push_back({c, S(L.q + re.first)});
        er.items.push_back({c, S(L.dqdrho + re.first)});
        et.items.push_back({c, S(L.dqdT + re.first)});
        const int di = rx[re.first].dense_idx;
        if (di >= 0) {
          ep.items.push_back({c, S(L.alpha + di)});
          eq.items.push_back({c, S(L.beta + di)});
        }
      }
      for (Entry *e : {&ew, &er, &et, &ep, &eq}) E.push_back(*e);
    }
    auto items = schedule(E, G, &P.progs[1].len);
    P.host_items[1] = items;
  }
  // program 2: the Y block (rows/cols 0..ns-2) and the T-row sums
  {
    std::vector<std::vector<std::vector<std::pair<int, int>>>> contrib(ns);  // [row][col] -> (net entry, slot)
    for (int i = 0; i < ns; ++i) contrib[i].resize(ns - 1);
    std::vector<std::vector<std::pair<int, int>>> tcontrib(ns - 1);  // [col] -> (reaction, slot)
    for (int r = 0; r < nr; ++r) {
      const HRxn &x = rx[r];
      for (size_t j = 0; j < x.slots.size(); ++j) {
        const int s = x.slots[j] & 0xFFFF;
        tcontrib[s].push_back({r, slot_entry_of[r][j]});
        for (size_t i = 0; i < x.net.size(); ++i) {
          contrib[x.net[i]][s].push_back({net_entry_of[r][i], slot_entry_of[r][j]});
        }
      }
    }
    for (int variant = 2; variant <= 3; ++variant) {
      // variant 2: reactor Y block (species rows 0..ns-2) + T-row sums; variant 3: every species row (the
      // (ns+1)^2 sensitivity block of prod_rates_primitive_sensitivities)
      const int nrows = variant == 2 ? ns - 1 : ns;
      std::vector<Entry> E;
      for (int i = 0; i < nrows; ++i)
        for (int k = 0; k < ns - 1; ++k) {
          Entry e{{}, (uint32_t)(L.Q + i + 1), DST_JBLOCK | (uint32_t)i | ((uint32_t)k << 15)};
          e.items.push_back({S(L.P + i), B(dm.d_u + k)});
          for (auto &c : contrib[i][k]) e.items.push_back({B(dm.d_netc + c.first), S(L.D + c.second)});
          E.push_back(e);
        }
      if (variant == 2)
        for (int k = 0; k < ns - 1; ++k) {
          Entry e{{}, 0, DST_TROW | (uint32_t)(L.trow + k)};
          for (auto &c : tcontrib[k]) e.items.push_back({S(L.E + c.first), S(L.D + c.second)});
          E.push_back(e);
        }
      auto items = schedule(E, G, &P.progs[variant].len);
      P.host_items[variant] = items;
    }
  }
  for (int k = 0; k < 4; ++k) {
    P.progs[k].G = G;
    const auto &items = P.host_items[k];
    GatherItem *dptr = nullptr;
    const size_t bytes = std::max<size_t>(items.size(), 1) * sizeof(GatherItem);
    CUDA_THROW(cudaMalloc(&dptr, bytes));
    if (!items.empty()) CUDA_THROW(cudaMemcpy(dptr, items.data(), items.size() * sizeof(GatherItem), cudaMemcpyHostToDevice));
    P.progs[k].items = dptr;
  }
  programs.emplace(G, std::move(P));
}

}  // namespace sfgb
