// Internal host-side declarations of the spitfire_gb300 library.
#pragma once
#include <cuda_runtime.h>

#include <array>
#include <cstring>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/spitfire_gb300.h"
#include "sf_mech.h"

namespace sfgb {

struct sf_error : std::runtime_error {
  int code;
  sf_error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

#define CUDA_THROW(call)                                                                                         \
  do {                                                                                                           \
    cudaError_t _e = (call);                                                                                     \
    if (_e != cudaSuccess)                                                                                       \
      throw ::sfgb::sf_error(SF_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e));                   \
  } while (0)

struct HRxn {
  int kind = 1, kform = 4, troe_terms = 0, fall = -1, dense_idx = -1;
  bool reversible = true, has_orders = false, dense = false;
  double kf[3] = {0, 0, 0}, kp[3] = {0, 0, 0}, troe[4] = {0, 0, 0, 0}, beff = 0;
  std::vector<int> reac, reac_nu, prod, prod_nu, net, net_nu, tb, ord, slots;
  std::vector<double> tbeff, ord_val;
  int sum_nu = 0, sum_reac_nu = 0, sum_prod_nu = 0;
};

struct HostMech {
  DevMech dm{};
  ScratchLayout sl{};
  std::vector<double> host_dbl, mw, invmw;
  std::vector<int> host_int;
  std::vector<HRxn> rx;               // device order (see build)
  std::vector<int> orig_index;        // device reaction -> index in the description
  std::vector<std::vector<int>> net_entry_of, slot_entry_of;
  void *d_blob = nullptr;
  int *d_status = nullptr;  // device error word of kernels using this mechanism
  int device = 0;
  int tune[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // launch shapes chosen by the autotuner (sf_tune_knob), 0 = default
  cudaStream_t copy_stream = nullptr;      // host-buffer entry points: device-to-host copies overlapping compute
  std::vector<cudaEvent_t> events;         // their chunk-completion events (created on first use)
  std::mutex host_batch_mutex;             // serializes the host-buffer calls that share the two above

  struct Programs {
    DevProgram progs[4]{};  // 0: w only, 1: w/S_rho/S_T/P/Q, 2: Y block + T row, 3: all species rows (sens)
    std::vector<GatherItem> host_items[4];
  };
  std::map<int, Programs> programs;

  void build(const sf_mech_desc *d);
  const Programs &programs_for(int G) const;  // the gather programs of lane width G (1, 8, 16 or 32), built by build()
  ~HostMech();

 private:
  void build_programs(int G);
};

// Launch helpers implemented in the .cu files (return an sf_status code).
int launch_rates(const HostMech &m, int n, const double *T, const double *rho, const double *Y, double *w,
                 cudaStream_t st);
void set_error(const std::string &msg);
// Raise a kernel's dynamic shared-memory limit to `bytes` on the current device, once per (kernel, device) and
// size: cudaFuncSetAttribute is a host-side call the launchers would otherwise repeat on every launch.
void ensure_dynamic_smem(const void *kernel, size_t bytes);
// Thread-per-state chemistry kernels: warps that can be resident at once, and the bytes of interleaved scratch a
// launch of n states takes (at most one slot per resident warp).
size_t tps_resident_warps(const HostMech &hm);
// sf_reactor_jac_batch with an explicit lane width G (8, 16 or 32; no workspace). Throws sf_error.
void reactor_jac_lanes(const sf_mech *mech, const sf_reactor_params *rp, int rates_option, int n, const double *q,
                       const double *pressures, double *out_rhs, double *out_jac, int G, cudaStream_t st);
// Parameter adjoint of closed adiabatic reactors (sf_rate_param_adjoint_batch) with `wsets` adjoint vector sets per
// state: w [n_items][wsets][stages][neq], out [n_items][wsets][2 nr] (accumulated). Throws sf_error.
void launch_rate_param_adjoint(const HostMech &hm, int configuration, double pressure, int n_items, int wsets,
                               int stages, const double *q, const double *pressures, const double *w, double *out,
                               cudaStream_t st);
size_t tps_scratch_bytes(const HostMech &hm, int mode, long long n);

}  // namespace sfgb

struct sf_mech {
  sfgb::HostMech m;
};
