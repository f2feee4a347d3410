// Shared host/device definitions: the packed mechanism ("blob") and the gather programs.
//
// A built mechanism lives on the device as one contiguous, 16-byte aligned buffer: a double section followed by
// an int section. Kernels copy the whole buffer into shared memory once per CTA (one bulk-async copy) and read
// every mechanism coefficient from there. The offsets below are in elements of their section.
#pragma once
#include <cstdint>

namespace sfgb {

constexpr int kMaxSpecies = 1024;   // species indices are stored in 16 bits in the gather programs
constexpr int kMaxNet = 8;          // Griffon's NSR (combustion_kernels.h:518)

// per-reaction packed info word (int section, o_info)
enum : int {
  RI_KIND_SHIFT = 0,     // 3 bits: 1 simple, 2 third-body, 3 Lindemann, 4 Troe
  RI_KFORM_SHIFT = 3,    // 3 bits: 0 const, 1 linear, 2 quadratic, 3 reciprocal, 4 Arrhenius
  RI_TROE_SHIFT = 6,     // 3 bits: which of the three F_cent terms are present
  RI_REV_BIT = 9,
  RI_ORD_BIT = 10,       // special (non-elementary) orders
  RI_DENSE_BIT = 11,     // has a Jacobian contribution to every Y column (alpha/beta terms)
};

struct DevMech {
  int ns, nr;
  int n_dense;      // reactions with a dense Jacobian part
  int n_fall;       // Lindemann + Troe
  int n_slots;      // total sparse Jacobian slots over all reactions
  int n_net_total;
  int all_nasa7;    // 1 if every species is NASA7 (else some are constant-cp)
  int blob_doubles; // size of the double section
  int blob_ints;    // size of the int section
  int blob_bytes;   // total, multiple of 16
  double Ru, invRu, pref;

  // ---- double section offsets ----
  int d_nasa;    // [ns][15] Griffon NASA7 storage (chemistry_setup.cpp:102-130); const-cp: [T0, h0, s0, cp, ...]
  int d_tmin, d_tmax, d_invmw, d_mw, d_u;  // [ns]; u_s = 1/M_s - 1/M_{ns-1}
  int d_kf;      // [nr][3] A, b, Ea/R
  int d_kp;      // [n_fall][3]
  int d_troe;    // [n_fall][4]
  int d_beff;    // [nr] default third-body efficiency
  int d_tbeff;   // [tb entries] invM*(eff - default)
  int d_netc;    // [net entries] -nu*M (coefficient of q_r in w_i)
  int d_ord;     // [order entries] special orders
  int d_one;     // 1.0
  int d_smallint;  // [64] the integer k - 32 at index k (stoichiometric coefficients without conversions); kept
                   // small because every kernel stages the blob into shared memory
  int d_exptab;    // [128] 2^(j/64) as (head, tail) pairs, j = 0..63, for the table-driven exponential; even offset

  // ---- int section offsets ----
  int i_info;    // [nr]
  int i_orig;    // [nr] index of each device-order reaction in the order the mechanism was described
  int i_sums;    // [nr] sum_nu (low 16 bits, signed) | sum_reac_nu << 16 (8 bits) | sum_prod_nu << 24
  int i_fall;    // [nr] falloff index or -1
  int i_dense;   // [nr] dense index or -1
  int i_reac_off, i_reac;   // [nr+1], entries: species | nu << 16
  int i_prod_off, i_prod;   // [nr+1], entries: species | nu << 16
  int i_net_off, i_net;     // [nr+1], entries: species | (nu + 128) << 16
  int i_tb_off, i_tb;       // [nr+1], entries: species
  int i_ord_off, i_ord;     // [nr+1], entries: species | nonzero << 16
  int i_slot_off, i_slot;   // [nr+1], entries: species | (rpos+1) << 16 | (ppos+1) << 20 | (tpos+1) << 24 | (opos+1) << 28
  int i_thermo;             // [ns] 1 const-cp, 2 NASA7
};

// ---------------------------------------------------------------------------------------- gather programs
// A gather program computes many sums  acc = init + sum_k a_k * b_k  with one FMA per item, spread over the G
// lanes of a state group in a static, load-balanced schedule: item j of lane l sits at items[j*G + l] and every
// lane executes exactly `len` items, so the loop has no divergence. Operand references name a double either in
// the mechanism blob (shared memory) or in the state's scratch area.
struct GatherItem {
  uint32_t a;      // operand ref
  uint32_t b;      // operand ref
  uint32_t dst;    // destination (see DST_*), valid on END items
  uint32_t flags;  // START | END | NOP, init ref in the low 24 bits (0 = start from zero)
};
constexpr uint32_t REF_SCRATCH = 0x80000000u;  // else blob double table
constexpr uint32_t F_START = 0x80000000u, F_END = 0x40000000u, F_NOP = 0x20000000u;
constexpr uint32_t INIT_MASK = 0x00FFFFFFu;    // scratch index + 1 of the initial value
constexpr uint32_t DST_SCRATCH = 0u << 30, DST_JBLOCK = 1u << 30, DST_TROW = 2u << 30;
constexpr uint32_t DST_KIND_MASK = 3u << 30;
constexpr int GATHER_UNROLL = 8;  // items per batch of the device runner; each lane's item count is a multiple

// Per-state scratch layout (doubles), shared by every kernel of one mechanism.
struct ScratchLayout {
  int y, C, dB, eh, cpv, dcp;          // species arrays [ns]
  int gm, gmi, gk;                     // [ns] exp(-g/RT) = gm * 2^gk (gk as integer bits), gmi = 1 / gm
  int w, Srho, ST, P, Q, trow;         // gather destinations [ns]
  int q, dqdrho, dqdT, E;              // reaction arrays [nr]
  int alpha, beta;                     // [n_dense]
  int D;                               // [n_slots]
  int misc;                            // 16 scalars
  int total;                           // doubles per state
  int total_rhs;                       // doubles per state needed by the RHS-only path (prefix of the layout)
};

struct DevProgram {
  const GatherItem *items;  // device
  int len;                  // items per lane
  int G;                    // lanes per group
};

}  // namespace sfgb
