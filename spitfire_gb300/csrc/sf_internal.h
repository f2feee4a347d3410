// Internal host-side declarations of the spitfire_gb300 library.
#pragma once
#include <cuda_runtime.h>

#include <array>
#include <cstring>
#include <map>
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
  // work counter of the dynamically scheduled kernels (zeroed on the launching stream before each launch; like
  // the scratch below it serves one stream at a time)
  int *d_work_counter = nullptr;
  int device = 0;
  int tune[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // launch shapes chosen by the autotuner (sf_tune_knob), 0 = default
  double *tps_scratch = nullptr;           // interleaved scratch of the thread-per-state kernels
  size_t tps_scratch_bytes = 0;
  cudaStream_t copy_stream = nullptr;      // host-buffer entry points: device-to-host copies overlapping compute
  std::vector<cudaEvent_t> events;         // their chunk-completion events (created on first use)

  struct Programs {
    DevProgram progs[4]{};  // 0: w only, 1: w/S_rho/S_T/P/Q, 2: Y block + T row, 3: all species rows (sens)
    std::vector<GatherItem> host_items[4];
  };
  std::map<int, Programs> programs;

  void build(const sf_mech_desc *d);
  const Programs &programs_for(int G);
  ~HostMech();
};

// Launch helpers implemented in the .cu files (return an sf_status code).
int launch_rates(const HostMech &m, int n, const double *T, const double *rho, const double *Y, double *w,
                 cudaStream_t st);
void set_error(const std::string &msg);
void ensure_tps_scratch(HostMech &m);

}  // namespace sfgb

struct sf_mech {
  sfgb::HostMech m;
};
