/*
 * spitfire_gb300 -- C ABI of the GB300 (sm_103a) Griffon chemistry hot path.
 *
 * Every entry point takes plain pointers and sizes. Batched entry points take DEVICE pointers (memory the
 * caller allocated on the current CUDA device), a CUDA stream passed as `void *` (a cudaStream_t; NULL is the
 * legacy default stream) and, where a kernel needs global scratch memory, a caller-provided workspace whose
 * size the matching *_workspace_size function reports. No batched entry point allocates device memory.
 * Entry points return 0 (SF_OK) or a status code; sf_last_error() gives the message of the last failure in
 * the calling thread. Per-item numerical outcomes (e.g. an integration that hit its step cap) are reported in
 * device int arrays, not by the return code.
 *
 * Array layouts (all FP64 unless stated; "state-major" = one contiguous row per state):
 *   mass fractions   Y[n][ns]
 *   reactor state    isochoric q[n][ns+1] = [rho, T, Y_0..Y_{ns-2}]; isobaric q[n][ns] = [T, Y_0..Y_{ns-2}]
 *   Jacobians        one column-major neq x neq block per state, blocks contiguous: J[n][neq*neq]
 *   rate sensitivity one column-major (ns+1) x (ns+1) block per state (columns rho, T, Y_0..Y_{ns-2};
 *                    last row unused), as Griffon's prod_rates_primitive_sensitivities writes it
 *   flamelet values  per flamelet, Griffon's BTDDOD layout: nzi column-major ns x ns diagonal blocks, then
 *                    (nzi-1)*ns sub-diagonal values, then (nzi-1)*ns super-diagonal values
 *
 * Reference interfaces replaced (paths within sandialabs/Spitfire):
 *   src/spitfire/griffon/griffon.pyx            -- Cython class PyCombustionKernels and py_btddod_* functions
 *   src/spitfire/griffon/include/combustion_kernels.h and btddod_matrix_kernels.h -- the C++ engine
 */
#ifndef SPITFIRE_GB300_H
#define SPITFIRE_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------------------------------------------- status */
enum sf_status {
  SF_OK = 0,
  SF_ERR_INVALID_ARGUMENT = 1, /* bad size, null pointer, unknown option */
  SF_ERR_MECHANISM = 2,        /* mechanism rejected (e.g. 2 <= n_net <= 8 violated, unknown enum) */
  SF_ERR_CUDA = 3,             /* a CUDA runtime call failed */
  SF_ERR_UNSUPPORTED = 4,      /* feature not available on this path (e.g. NASA9 thermo on the GPU) */
  SF_ERR_WORKSPACE = 5,        /* workspace missing or smaller than *_workspace_size reported */
  SF_ERR_NO_DEVICE = 6         /* no CUDA device */
};

/* Message of the last failing call in this thread (empty string if none). */
const char *sf_last_error(void);
/* Library version string. */
const char *sf_version(void);

/* ------------------------------------------------------------------------------------- mechanism description */
/* Thermodynamic model codes (combustion_kernels.h:43-49 CpType). */
enum sf_thermo_kind { SF_THERMO_CONST = 1, SF_THERMO_NASA7 = 2, SF_THERMO_NASA9 = 3 };
/* Reaction rate types (combustion_kernels.h:59-66 RateType). */
enum sf_rxn_kind { SF_RXN_SIMPLE = 1, SF_RXN_THIRD_BODY = 2, SF_RXN_LINDEMANN = 3, SF_RXN_TROE = 4 };

/*
 * Flat mechanism description: the data Spitfire passes to Griffon through the 16 mechanism_* setters
 * (griffon.pyx:234-551, combustion_kernels.h:293-379), gathered into arrays. Species indices refer to the phase
 * order. Within a reaction, reactants, products, efficiencies and special orders must be listed in ascending
 * species-NAME order (the std::map<std::string,...> order Griffon iterates in, chemistry_setup.cpp:361-392).
 *
 * thermo_coefs[k*20 + j]:
 *   NASA7: [Tmin, Tmid, Tmax, low a0..a6, high a0..a6]              (raw coefficients, not multiplied by R)
 *   CONST: [Tmin, Tmax, T0, h0, s0, cp, 0...]
 * NASA9 species carry their coefficient list in nasa9_coefs with nasa9_offsets[k]..nasa9_offsets[k+1]
 * (Cantera's flattened form: [n_regions, Tlo, Thi, a0..a8, Tlo, Thi, ...]); nasa9_offsets may be NULL if no
 * species is NASA9.
 * Rate constants: k = A T^b exp(-Ea_over_R / T); kfwd is the (high-pressure) forward rate, kflf the low-pressure
 * rate of falloff reactions. troe = [A, T3, T1, T2].
 */
typedef struct sf_mech_desc {
  int n_species;
  int n_reactions;
  int n_elements;
  double gas_constant;       /* J/kmol/K */
  double ref_pressure;       /* Pa */
  double ref_temperature;    /* K */
  const double *molecular_weights; /* [n_species] kg/kmol */
  const int *thermo_kind;          /* [n_species] sf_thermo_kind */
  const double *thermo_coefs;      /* [n_species*20] */
  const int *nasa9_offsets;        /* [n_species+1] or NULL */
  const double *nasa9_coefs;

  const int *rxn_kind;          /* [n_reactions] sf_rxn_kind */
  const int *rxn_reversible;    /* [n_reactions] 0/1 */
  const double *rxn_kfwd;       /* [n_reactions*3] A, b, Ea/R */
  const double *rxn_kflf;       /* [n_reactions*3] (falloff only) */
  const double *rxn_troe;       /* [n_reactions*4] (Troe only) */
  const double *rxn_default_eff;/* [n_reactions] (third-body / falloff only) */
  const int *reac_offsets;      /* [n_reactions+1] */
  const int *reac_species;
  const int *reac_stoich;
  const int *prod_offsets;      /* [n_reactions+1] */
  const int *prod_species;
  const int *prod_stoich;       /* positive integers */
  const int *eff_offsets;       /* [n_reactions+1] third-body efficiencies */
  const int *eff_species;
  const double *eff_values;
  const int *order_offsets;     /* [n_reactions+1] special (non-elementary) orders; a reaction with any entry
                                   here is a *_with_special_orders reaction */
  const int *order_species;
  const double *order_values;
} sf_mech_desc;

typedef struct sf_mech sf_mech; /* opaque: host tables + device blob on one CUDA device */

/* Build a mechanism from a description, running Griffon's ReactionRateData::finalize derivations
 * (chemistry_setup.cpp:459-732) and uploading the packed blob to the current device.
 * Replaces PyCombustionKernels.__cinit__ + mechanism_* setters (griffon.pyx:225-551). */
int sf_mech_create(const sf_mech_desc *desc, sf_mech **out_mech);
/* Replaces PyCombustionKernels.__dealloc__ (griffon.pyx:228-229). */
int sf_mech_destroy(sf_mech *mech);
/* Device error word of the kernels that use this mechanism: 0, or the first code a kernel recorded
 * (1 shared-memory staging timed out, 2 invalid input, 3 a bounded wait ran out). Synchronizes the device.
 * clear != 0 resets it. Returns -1 on a CUDA failure. */
int sf_device_status(const sf_mech *mech, int clear);
/* Sizes of a built mechanism; counts[0..5] = reactions by kind: simple, three-body, Lindemann, Troe, dense
 * (Jacobian rows that need the dense term), special-order. Any output pointer may be NULL. */
int sf_mech_info(const sf_mech *mech, int *n_species, int *n_reactions, int *counts6);

/* Launch shapes of the kernels that use a mechanism, as chosen by an autotuner (spitfire_gb300/autotune.py times
 * the candidates on the device). 0 restores the built-in choice. Knobs and values:
 *   SF_TUNE_GROUP_{RATES,SENS,RHS,JAC}: lanes per state of the batched kernels, 8, 16 or 32, or 1 for the
 *     thread-per-state kernels (each lane one state, scratch interleaved across the warp in the caller's
 *     workspace, whose size sf_chem_workspace_size reports; no knob allocates anything);
 *   SF_TUNE_INTEGRATE_WARPS: warps (reactors) per block of sf_integrate_batch, 1..8 (0: as many as fit);
 *   SF_TUNE_INTEGRATE_SCRATCH: where each integrating warp keeps its data: 3 all in shared memory; 1 its Griffon
 *     scratch in global memory (L2-resident), so that more warps fit per SM; 2 also its iteration matrix and FP32
 *     factors (0: the built-in choice, 2);
 *   SF_TUNE_TPS_CTAS: resident 4-warp blocks per SM of the thread-per-state kernels, 1..16 (0: as many as fit);
 *     fewer keep more of their interleaved scratch in L2.
 * The integrator knobs do not change results; the lane-group width changes the order of per-species sums, so those
 * results agree to rounding. No reference counterpart.
 * Concurrency: a mechanism holds no scratch, so calls on one sf_mech may run on several streams at once, each with
 * its own workspace. Set knobs while no call that uses the mechanism is being issued. */
enum sf_tune_knob {
  SF_TUNE_GROUP_RATES = 0, SF_TUNE_GROUP_SENS = 1, SF_TUNE_GROUP_RHS = 2, SF_TUNE_GROUP_JAC = 3,
  SF_TUNE_INTEGRATE_WARPS = 4, SF_TUNE_INTEGRATE_SCRATCH = 5, SF_TUNE_TPS_CTAS = 6, SF_TUNE_KNOBS = 7
};
int sf_mech_set_tuning(sf_mech *mech, int knob, int value);
int sf_mech_get_tuning(const sf_mech *mech, int knob, int *value);
/* Per-state scratch of the kernels (doubles: right-hand side only, and with the Jacobian) and the size of the
 * mechanism blob staged into shared memory; any output pointer may be NULL. */
int sf_mech_layout(const sf_mech *mech, int *scratch_rhs_doubles, int *scratch_total_doubles, long long *blob_bytes);

/* ------------------------------------------------------------------------------------------- thermodynamics */
/* what: 0 cp_mix[n], 1 cv_mix[n], 2 enthalpy_mix[n], 3 energy_mix[n], 4 species_cp[n][ns], 5 species_cv[n][ns],
 *       6 species_enthalpies[n][ns], 7 species_energies[n][ns], 8 mixture_molecular_weight[n],
 *       9 dcp/dT mix[n] (cp_sens_T), 10 dcp/dT species[n][ns]
 * Replaces griffon.pyx:684-761 (cp_mix, cv_mix, species_cp, ..., dcpdT_species). */
int sf_thermo_batch(const sf_mech *mech, int what, int n, const double *T, const double *Y, double *out,
                    void *stream);

/* --------------------------------------------------------------------------------------------------- kinetics */
/* Device workspace of the batched chemistry calls below, in bytes, for n states: the thread-per-state kernels
 * (lanes-per-state knob 1) interleave each warp's per-state scratch in it, at most one slot per warp that can be
 * resident (GRI-3.0 Jacobians: about 1.2 GB for a full device); the lane-group kernels keep their scratch in shared
 * memory and need none (0; the workspace pointer may then be NULL). The size depends on the mechanism's current
 * knobs: query it after tuning. One workspace must not be used by two calls that run at the same time. */
enum sf_chem_kind { SF_CHEM_RATES = 0, SF_CHEM_SENS = 1, SF_CHEM_RHS = 2, SF_CHEM_JAC = 3 };
size_t sf_chem_workspace_size(const sf_mech *mech, int kind, int n);

/* Production rates w[n][ns] (kg/m^3/s) at (T, rho, Y).
 * Replaces PyCombustionKernels.production_rates (griffon.pyx:763-768 -> chemistry_kernels.cpp:29-33). Note the
 * Cython wrapper passes its first positional argument as T; this entry point names T and rho explicitly. */
int sf_production_rates_batch(const sf_mech *mech, int n, const double *T, const double *rho, const double *Y,
                              double *out_w, void *workspace, size_t workspace_bytes, void *stream);

/* Production rates and their sensitivities to (rho, T, Y_0..Y_{ns-2}), out_sens[n][(ns+1)^2].
 * option: 0 exact dense, 2 exact sparse (identical values), 1 no third-body/falloff sensitivities.
 * Replaces prod_rates_primitive_sensitivities (griffon.pyx:773-783 -> chemistry_kernels.cpp:464-483). */
int sf_rates_sens_batch(const sf_mech *mech, int n, const double *rho, const double *T, const double *Y, int option,
                        double *out_w, double *out_sens, void *workspace, size_t workspace_bytes, void *stream);

/* ------------------------------------------------------------------------------------------ reactor kernels */
/* Reactor parameters shared by every state of one batched call (the scalar arguments of
 * reactor_rhs_isobaric / reactor_rhs_isochoric, griffon.pyx:788-866). */
typedef struct sf_reactor_params {
  int configuration;        /* 0 isobaric (q = [T, Y]), 1 isochoric (q = [rho, T, Y]) */
  int heat_transfer;        /* 0 adiabatic, 1 isothermal, 2 diathermal */
  int open;                 /* 0 closed, 1 open (mass exchange with a feed) */
  double pressure;          /* isobaric: thermodynamic pressure (Pa) */
  double inflow_density;    /* isochoric open reactors */
  double inflow_temperature;
  const double *inflow_Y;   /* DEVICE pointer [ns] or NULL when closed */
  double tau;               /* residence time */
  double fluid_temperature; /* convection temperature */
  double surface_temperature; /* radiation temperature */
  double h_convection;
  double eps_radiation;
  double surface_area_to_volume;
} sf_reactor_params;

/* Reactor right-hand sides and Jacobians of n states held in HOST memory, as the reference's
 * reactor_jac_isochoric / reactor_jac_isobaric take them (griffon.pyx:807-866): the states (and optional per-state
 * pressures) are copied in on `stream`, the Jacobians computed in chunks of chunk_states states (<= 0: one wave of
 * the thread-per-state kernel's resident warps when the autotuner selected it, else half the batch), and each
 * chunk's results copied back on a second stream while the next chunk computes. `stream` is ordered after the last
 * copy. Pinned host buffers let the copies run asynchronously. workspace: DEVICE, at least
 * sf_reactor_jac_host_workspace_size bytes (device copies of inputs and outputs plus the kernel's workspace).
 * Calls on one mechanism from several host threads take turns while they issue their work; their copies back share
 * the mechanism's copy stream. */
size_t sf_reactor_jac_host_workspace_size(const sf_mech *mech, const sf_reactor_params *params, int n);
int sf_reactor_jac_host_batch(const sf_mech *mech, const sf_reactor_params *params, int rates_option, int n,
                              const double *q_host, const double *pressures_host, double *out_rhs_host,
                              double *out_jac_host, int chunk_states, void *workspace, size_t workspace_bytes,
                              void *stream);

/* Right-hand side of n reactors (state-major q, out_rhs). If pressures is non-NULL (isobaric) it gives one
 * pressure per state and overrides params->pressure.
 * Replaces reactor_rhs_isobaric / reactor_rhs_isochoric (isobaric_reactor_kernels.cpp:170-219,
 * isochoric_reactor_kernels.cpp:184-242). */
int sf_reactor_rhs_batch(const sf_mech *mech, const sf_reactor_params *params, int n, const double *q,
                         const double *pressures, double *out_rhs, void *workspace, size_t workspace_bytes,
                         void *stream);

/* Right-hand side and analytical Jacobian (column-major neq x neq per state). rates_option as in
 * sf_rates_sens_batch. Replaces reactor_jac_isobaric / reactor_jac_isochoric (isobaric_reactor_kernels.cpp:221-343,
 * isochoric_reactor_kernels.cpp:244-333). workspace: sf_chem_workspace_size(mech, SF_CHEM_JAC, n) bytes, as for
 * the rates calls. */
int sf_reactor_jac_batch(const sf_mech *mech, const sf_reactor_params *params, int rates_option, int n,
                         const double *q, const double *pressures, double *out_rhs, double *out_jac, void *workspace,
                         size_t workspace_bytes, void *stream);

/* The same evaluation in the plain single-state GPU form: one thread per state, the mechanism read from global
 * memory, Griffon's per-reaction dense scatter into a per-state scratch Jacobian. It exists as the comparison
 * point for the batched kernels; results are the same to rounding. Needs workspace of
 * sf_reactor_jac_plain_workspace_size bytes. */
size_t sf_reactor_jac_plain_workspace_size(const sf_mech *mech, int n);
int sf_reactor_jac_plain_batch(const sf_mech *mech, const sf_reactor_params *params, int n, const double *q,
                               const double *pressures, double *out_rhs, double *out_jac, void *workspace,
                               size_t workspace_bytes, void *stream);

/* Size of the fixed device scratch used by sf_reactor_jac_plain_batch_static: 32 MiB on each device. */
#define SF_PLAIN_STATIC_SCRATCH_BYTES (32u << 20)

/* sf_reactor_jac_plain_batch without any allocation. No counterpart in the reference: it is for callers that
 * cannot allocate device memory where they evaluate Jacobians (a host code whose memory manager owns every
 * device allocation and forbids raw cudaMalloc, or a caller that must not allocate while it records work on its
 * streams). Instead of a caller-provided workspace, the per-state scratch comes from a fixed array of
 * SF_PLAIN_STATIC_SCRATCH_BYTES in device global memory that the library holds on every device that loads it,
 * until the process exits; inputs and outputs are still the caller's. The first call on a device looks up that
 * array's device address (a runtime query, no allocation), so make the first call on each device before any
 * stream capture. Batches whose scratch does not fit (n * per-state scratch > 32 MiB; about 600 GRI-3.0 states or
 * 8000 h2-burke states) are rejected with SF_ERR_WORKSPACE and a message giving the limit. All calls on a device
 * share the array: two calls that run at the same time on the GPU (e.g. on different streams) overwrite each
 * other's scratch and give wrong results; serialize them. Each call rewrites all scratch it reads, so contents
 * left by an earlier call do no harm. The looked-up address is kept for the life of the process: after a
 * cudaDeviceReset of that device, which unloads this library's device code, do not call this entry point again. */
int sf_reactor_jac_plain_batch_static(const sf_mech *mech, const sf_reactor_params *params, int n, const double *q,
                                      const double *pressures, double *out_rhs, double *out_jac, void *stream);

/* ------------------------------------------------------------------------------------------- Newton algebra */
/* Factor the Newton iteration matrices A_k = gamma_h[k] * J_k - I (m x m column-major, n of them).
 * precision: 0 FP64 LU with partial pivoting (as LAPACK dgetrf, reactors.py:340-344); 1 FP32 LU of the same
 * matrix (A itself kept in FP64 for the residual refinement of sf_newton_solve_batch).
 * out_A[n][m*m] receives A in FP64; out_lu receives the factors: FP64 [n][m*m] (precision 0) or FP32 [n][m*m]
 * (precision 1, pass it as a double* of n*m*m/2 doubles); out_piv[n][m] pivots (0-based). out_info[n] (may be
 * NULL) gets 0 or k+1 for an exactly zero pivot at step k.
 * Replaces scipy dgetrf in HomogeneousReactor._lapack_setup_wrapper (reactors.py:340-344). */
int sf_newton_lu_batch(int n, int m, const double *J, const double *gamma_h, int precision, double *out_A,
                       void *out_lu, int *out_piv, int *out_info, void *stream);
/* Solve A_k x_k = b_k with the factors of sf_newton_lu_batch. precision 1 runs FP32 triangular solves with
 * `refine` FP64 residual-refinement sweeps r = b - A x (A from out_A). Replaces scipy dgetrs
 * (reactors.py:354-356). */
int sf_newton_solve_batch(int n, int m, const double *A, const void *lu, const int *piv, int precision, int refine,
                          const double *b, double *out_x, void *stream);

/* --------------------------------------------------------------------------------------- batched integration */
/* Controls of HomogeneousReactor.integrate / odesolve (reactors.py:429-611, integrator.py:229-713) with the
 * reference defaults: ESDIRK64 (KennedyCarpenterS6P4Q3), simple Newton with frozen Jacobian, PI controller. */
typedef struct sf_integrate_params {
  double first_time_step;           /* 1e-6 */
  double max_time_step;             /* 1e6 */
  double transient_tolerance;       /* 1e-10 (PI target error) */
  double nonlinear_tolerance;       /* 1e-12 */
  int minimum_time_step_count;      /* 40 */
  int maximum_time_step_count;      /* hard cap on accepted steps (the reference default is unbounded) */
  int max_nonlinear_iter;           /* 20 */
  int maximum_steps_per_jacobian;   /* 1 */
  double stop_at_time;              /* > 0: stop (and land exactly) at this time; <= 0: none */
  double delta_temperature_ignition;/* > 0: stop when T > T0 + delta (compute_ignition_delay) */
  double minimum_allowable_residual;/* ignition stop: residual below this marks "will not ignite" */
  double stop_at_steady;            /* > 0: stop when residual < this */
  int linear_precision;             /* 0 FP64 LU, 1 FP32 LU + FP64 refinement */
  int refine_sweeps;                /* refinement sweeps for linear_precision 1 */
  int rates_option;                 /* 0 dense exact (default), 2 sparse exact */
  int max_attempts;                 /* cap on step attempts (accepted + failed) per reactor */
  /* Time-dependent reactor parameters (reactors.py:253-341): when time_table is non-NULL (DEVICE
   * [time_points][time_width], time_points >= 2, values at integration-local times time_t0 + j time_dt), each
   * parameter whose sf_time_param bit is set in time_columns is the table's interpolant (cubic Lagrange on four
   * table points, held constant beyond the ends) in place of its value in sf_reactor_params. The columns hold the
   * set parameters in the order of their bits, the ns feed mass fractions of SF_TIME_FEED_Y last. As in the
   * reference's closures (reactors.py:279-282, :335-341, :538-592), each right-hand side takes the parameters at
   * its own time and each Jacobian those of the most recent right-hand side, or those at time_jac_t0 before the
   * first one. The feed density has no column: the reference evaluates it once, at t = 0. Mass-transfer columns
   * act on open reactors only, heat-transfer ones on diathermal reactors only. NULL: none. */
  const double *time_table;
  int time_points, time_width, time_columns;
  double time_t0, time_dt, time_jac_t0;
  /* Optional output of sf_integrate_batch / sf_integrate_record_batch with delta_temperature_ignition > 0: DEVICE
   * [n], the time at which T first reaches T0 + delta, from the cubic Hermite interpolant of T over the accepted
   * step that crossed it (end values and the right-hand side's dT/dt at both ends; the first crossing in the step).
   * NaN where T never reaches it. No reference counterpart: the reference's delay is the end time of that step
   * (reactors.py:774-790, the integrators' out_t), which this refines without changing the steps. NULL: none. */
  double *ignition_time_interp;
} sf_integrate_params;

/* Parameters a time table of sf_integrate_params may hold, as bits of time_columns. */
enum sf_time_param {
  SF_TIME_FEED_T = 1,      /* feed temperature */
  SF_TIME_MIXING_TAU = 2,  /* mixing (residence) time */
  SF_TIME_CONV_T = 4,      /* convection (fluid) temperature */
  SF_TIME_CONV_H = 8,      /* convection coefficient */
  SF_TIME_RAD_T = 16,      /* radiation (surface) temperature */
  SF_TIME_RAD_EPS = 32,    /* radiative emissivity */
  SF_TIME_FEED_Y = 64      /* feed mass fractions (ns columns) */
};

/* Per-reactor outcome codes written to out_status. */
enum sf_integrate_status {
  SF_INT_RUNNING = 0, SF_INT_DONE = 1, SF_INT_IGNITED = 2, SF_INT_STEADY = 3, SF_INT_MAX_STEPS = 4,
  SF_INT_NAN = 5, SF_INT_NO_IGNITION = 6, SF_INT_RECORD_FULL = 7
};

size_t sf_integrate_workspace_size(const sf_mech *mech, const sf_reactor_params *params, int n);
/* Integrate n independent reactors of the same configuration and feed from q0 (state-major; isobaric reactors
 * may each have their own pressure). One persistent launch works through the batch: each warp takes the next
 * unfinished reactor from a queue, so reactors with 10x more steps do not stall the rest. Outputs: final states
 * out_q, final time out_t, per-reactor counters out_counts[n][4] = steps, Newton iterations, Jacobian setups,
 * failed steps, and status codes. out_t of an ignition run is the ignition delay (the end time of the first
 * accepted step with T > T0 + delta, reactors.py:774-790). */
int sf_integrate_batch(const sf_mech *mech, const sf_reactor_params *params, const sf_integrate_params *iparams,
                       int n, const double *q0, const double *pressures, double *out_q, double *out_t,
                       int *out_counts, int *out_status, void *workspace, size_t workspace_bytes, void *stream);

/* The plain single-state GPU form of sf_integrate_batch, kept as its comparison point: one thread per reactor runs
 * the same step logic serially over Griffon's plain per-state evaluation (dense derivative scatter, as
 * sf_reactor_jac_plain_batch) and a serial LU, with all its data in the workspace (DEVICE, at least
 * sf_integrate_plain_workspace_size bytes). Closed adiabatic reactors. */
size_t sf_integrate_plain_workspace_size(const sf_mech *mech, const sf_reactor_params *params, int n);
int sf_integrate_plain_batch(const sf_mech *mech, const sf_reactor_params *params, const sf_integrate_params *iparams,
                             int n, const double *q0, const double *pressures, double *out_q, double *out_t,
                             int *out_counts, int *out_status, void *workspace, size_t workspace_bytes,
                             void *stream);

/* sf_integrate_batch that also records every accepted step for adjoint sensitivities: trajectory is DEVICE
 * [n][capacity_steps][2 + 6*neq] doubles, per step (t_n, dt_n, Y_1..Y_6) with Y_1 = y_n and Y_2..Y_6 the converged
 * ESDIRK64 stage values (in the integrator's order). A reactor that needs more steps than the capacity stops with
 * SF_INT_RECORD_FULL. No reference counterpart (the reference computes no parameter sensitivities). */
int sf_integrate_record_batch(const sf_mech *mech, const sf_reactor_params *params, const sf_integrate_params *iparams,
                              int n, const double *q0, const double *pressures, double *out_q, double *out_t,
                              int *out_counts, int *out_status, void *workspace, size_t workspace_bytes,
                              double *trajectory, int capacity_steps, void *stream);

/* ------------------------------------------------------------------------------------------ rate parameters */
/* Parameter adjoint of the closed adiabatic reactor right-hand side f(q; theta), theta = (ln A_r, E_a,r) per
 * reaction (forward, or high-pressure for falloff, Arrhenius coefficients; E_a in J/kmol), reactions in the
 * mechanism's internal order (simple, three-body, Lindemann, Troe, as the setters were called):
 *   out_grad[i][2r] += sum_s w_is^T df/d ln A_r (q_is),  out_grad[i][2r+1] += sum_s w_is^T df/d E_a,r (q_is)
 * for items i < n_items and stages s < stages; q and w are DEVICE [n_items][stages][neq] (isobaric [T, Y] or
 * isochoric [rho, T, Y] per params->configuration), pressures DEVICE [n_items] (isobaric; NULL = params->pressure),
 * out_grad DEVICE [n_items][2*n_reactions], accumulated. No reference counterpart. */
int sf_rate_param_adjoint_batch(const sf_mech *mech, const sf_reactor_params *params, int n_items, int stages,
                                const double *q, const double *pressures, const double *w, double *out_grad,
                                void *stream);

/* Outputs of sf_adjoint_batch. SF_ADJ_T_END: the temperature at the end of the recorded integration.
 * SF_ADJ_TAU_S: the smoothed ignition delay, the ESDIRK64 quadrature of the time spent below T0 + 400 K,
 *   tau_s = sum_n h_n sum_s b_s g(T_ns),  g(T) = 1 - 1 / (1 + exp(-(T - T0 - 400 K) / 20 K)). */
enum sf_adjoint_output { SF_ADJ_T_END = 0, SF_ADJ_TAU_S = 1 };
/* Gradients of recorded closed adiabatic integrations (sf_integrate_record_batch) by the discrete adjoint of their
 * ESDIRK64 step sequences: for every reactor and output, d/d ln A_r and d/d E_a,r of every reaction (forward, or
 * high-pressure for falloff, Arrhenius coefficients; E_a in J/kmol) and d/d q0. Backwards over the recorded steps,
 * all reactors at once: stage Jacobians at the recorded stages, the transposed stage systems
 * (I - h gamma J_s^T) w_s = c_s with c_s = h b_s lam' + h sum_{l>s} a_ls Ybar_l + h gamma qd_s, Ybar_s = J_s^T w_s +
 * qd_s, lam = lam' + sum_s Ybar_s (lam' the adjoint with the entries the step's clamp of negative values acted on
 * zeroed, qd_s the quadrature term of tau_s), and the parameter adjoint sum_s w_s^T df/dtheta (Y_s).
 * trajectory DEVICE [n][capacity_steps][2 + 6 neq] and counts DEVICE [n][4] as sf_integrate_record_batch wrote
 * them; pressures DEVICE [n] (isobaric; NULL = params->pressure); T0 DEVICE [n], each reactor's initial
 * temperature (needed by SF_ADJ_TAU_S, else may be NULL); output_kinds HOST [n_outputs] (1..8 of
 * sf_adjoint_output). out_grad_theta DEVICE [n][n_outputs][2 n_reactions] (d/d ln A_r at 2r, d/d E_a,r at 2r+1,
 * reactions in the order the mechanism was described), out_grad_q0 DEVICE [n][n_outputs][neq] or NULL; both
 * overwritten. The call reads the step counts back once (a synchronization of `stream`). workspace: DEVICE,
 * sf_adjoint_workspace_size bytes. No reference counterpart (the reference computes no sensitivities). */
size_t sf_adjoint_workspace_size(const sf_mech *mech, const sf_reactor_params *params, int n, int n_outputs);
int sf_adjoint_batch(const sf_mech *mech, const sf_reactor_params *params, int n, const double *trajectory,
                     int capacity_steps, const int *counts, const double *pressures, const double *T0,
                     int n_outputs, const int *output_kinds, double *out_grad_theta, double *out_grad_q0,
                     void *workspace, size_t workspace_bytes, void *stream);

/* ------------------------------------------------------------------------------------------------ flamelets */
/* Stencil coefficients (flamelet_kernels.cpp:31-48); host pointers, host computation (setup only). */
int sf_flamelet_stencils(const sf_mech *mech, const double *dz, int nzi, const double *chi,
                         const double *inv_lewis, double *out_cmajor, double *out_csub, double *out_csup,
                         double *out_mcoeff, double *out_ncoeff);
/* COO indices of the BTDDOD Jacobian (flamelet_kernels.cpp:50-90); host pointers. */
int sf_flamelet_jac_indices(const sf_mech *mech, int nzi, int *out_rows, int *out_cols);

/* A batch of adiabatic flamelets, each with its own grid size; arrays are concatenated over flamelets.
 * offsets_z[f] is the first interior point of flamelet f in point-indexed arrays (state has ns values per point,
 * chi one per point, stencils ns per point, m/n one per point); offsets_z[n_flamelets] = total points.
 * Value arrays use offsets_v[f] = offset of flamelet f's BTDDOD value block (ns*(nzi*ns + 2*(nzi-1)) each). */
typedef struct sf_flamelet_batch {
  int n_flamelets;
  const int *offsets_z;     /* DEVICE [n_flamelets+1] */
  const long long *offsets_v; /* DEVICE [n_flamelets+1] */
  const int *offsets_z_host;  /* HOST copy of offsets_z */
  double pressure;
  const double *oxy_state;  /* DEVICE [n_flamelets][ns] boundary state [T, Y_0..Y_{ns-2}] at Z = 0 */
  const double *fuel_state; /* DEVICE [n_flamelets][ns] boundary state at Z = 1 */
  const double *cmajor, *csub, *csup; /* DEVICE [points][ns] */
  const double *mcoeff, *ncoeff, *chi; /* DEVICE [points] */
  int include_enthalpy_flux;
  int include_variable_cp;
  const double *diffterm;   /* DEVICE [n_flamelets] diffusion term of each flamelet for the eigenvalue bound of
                               sf_flamelet_jac_batch, or NULL to use its scalar diffterm argument for all */
  const int *active;        /* DEVICE [n_flamelets] or NULL: flamelets with active[f] == 0 are left untouched */
  /* Nonadiabatic flamelets (flamelet_kernels.cpp:1121-1138, :1290-1320): DEVICE [points] convection temperature and
   * coefficient, radiation temperature and emissivity per interior point, all NULL for adiabatic flamelets. With
   * use_scaled_heat_loss the coefficients are divided by (max T - T_conv) and (max T^4 - T_rad^4), max T over each
   * flamelet's interior points. */
  const double *T_convection, *h_convection, *T_radiation, *h_radiation;
  int use_scaled_heat_loss;
  const double *prefactor;  /* DEVICE [n_flamelets] or NULL: each flamelet's own prefactor of the scale_and_offset
                               form of sf_flamelet_jac_batch (prefactor * J - I, e.g. gamma * dt of its own time
                               step), in place of the scalar argument */
} sf_flamelet_batch;

/* Flamelet residual for every flamelet of the batch (flamelet_kernels.cpp:1039-1218). */
int sf_flamelet_rhs_batch(const sf_mech *mech, const sf_flamelet_batch *fb, const double *state, double *out_rhs,
                          void *stream);
/* BTDDOD Jacobian values (flamelet_kernels.cpp:1220-1409, rates options 0/1/2, exact transform).
 * If scale_and_offset, J <- prefactor*J - I on the diagonal blocks (flamelet_kernels.cpp:1395-1408). If
 * out_expeig is non-NULL it receives, for every row of a point, max(max Re(lambda) - d, 0) over the eigenvalues
 * lambda of that point's diagonal block without the diffusion diagonal (block - diag(cmajor)), d = fb->diffterm[f]
 * or the scalar diffterm, computed by balancing, Householder-Hessenberg reduction and Francis double-shift QR on
 * one warp (exactly 0 without QR when the balanced block's Gershgorin bound is <= d); this replaces the dgeev call
 * at flamelet_kernels.cpp:1329-1341. scale_and_offset must be 0 when out_expeig is requested. */
int sf_flamelet_jac_batch(const sf_mech *mech, const sf_flamelet_batch *fb, const double *state, int rates_option,
                          int scale_and_offset, double prefactor, double diffterm, double *out_expeig,
                          double *out_values, void *workspace, size_t workspace_bytes, void *stream);
/* Workspace of sf_flamelet_jac_batch: 256 bytes when eigenvalue bounds are requested (the eigenvalue kernel hands
 * out points with a counter there, zeroed on the stream before each launch), else 0. */
size_t sf_flamelet_jac_workspace_size(const sf_mech *mech, int eigenvalues);

/* The four block-Thomas functions take `active`: DEVICE int [n_flamelets] or NULL; flamelets with active[f] == 0
 * are left untouched (their values, factors and outputs keep what they held).
 * Block-Thomas factorization of a batch of BTDDOD matrices, in place (btddod_matrix_kernels.cpp:19-80), twisted:
 * with m = nzi/2, blocks 0..m-1 are eliminated downward as the reference does (L_i = diag(sub_{i-1}) D_{i-1}^-1,
 * D_i <- D_i - L_i diag(sup_{i-1})), blocks nzi-1..m+1 upward (U_i = diag(sup_{i-1}) D_i^-1,
 * D_{i-1} <- D_{i-1} - U_i diag(sub_{i-1})), and block m takes both updates; the two halves run concurrently, which
 * halves a flamelet's chain of dependent block steps. With nzi <= 2 this is the reference's order exactly.
 * Each eliminated block is inverted by Gauss-Jordan elimination with partial pivoting (the multiplier blocks need
 * the inverse; the reference forms it with dgetrs on the identity).
 * values: DEVICE, layout per flamelet as above, its diagonal blocks overwritten with the inverses of the eliminated
 * blocks; l_values: DEVICE output of nzi*ns*ns per flamelet at point offset offsets_z[f]*ns*ns (block i: L_i for
 * 1 <= i <= m, U_i for m < i < nzi); pivots: DEVICE int [points][ns], the pivot row of each elimination step of
 * each block (the reference stores LAPACK swap indices there; neither solve needs them with these factors). The
 * factors are read only by sf_btddod_solve_batch. ns <= 128 and 2*ns*ns doubles must fit in the shared memory of
 * one block (ns <= 119 on GB300). */
int sf_btddod_factor_batch(int n_flamelets, int ns, const int *offsets_z, const long long *offsets_v,
                           const int *offsets_z_host, double *values, double *l_values, int *pivots,
                           const int *active, void *stream);
/* Solve with the factors of sf_btddod_factor_batch (btddod_matrix_kernels.cpp:82-119, its two sweeps run from both
 * ends toward block m and back). rhs and out_x are point-major [points][ns] (they must not alias). */
int sf_btddod_solve_batch(int n_flamelets, int ns, const int *offsets_z, const long long *offsets_v,
                          const int *offsets_z_host, const double *values, const double *l_values,
                          const int *pivots, const double *rhs, double *out_x, const int *active, void *stream);
/* y = A x for a batch of BTDDOD matrices (btddod_matrix_kernels.cpp:121-160). */
int sf_btddod_matvec_batch(int n_flamelets, int ns, const int *offsets_z, const long long *offsets_v,
                           const int *offsets_z_host, const double *values, const double *x, double *out_y,
                           const int *active, void *stream);
/* A <- matrix_scale*A + diag_scale*diag(d) (btddod_matrix_kernels.cpp:448-465). */
int sf_btddod_scale_and_add_diagonal_batch(int n_flamelets, int ns, const int *offsets_z,
                                           const long long *offsets_v, const int *offsets_z_host, double *values,
                                           double matrix_scale, const double *diagonal, double diag_scale,
                                           const int *active, void *stream);

/* Block-diagonal algebra (the reference's py_btddod_blockdiag_* and *_fulltriangle_* functions, griffon.pyx:1019-1069,
 * btddod_matrix_kernels.cpp:167-177 and :364-428). A block-diagonal factorization here is the list of the blocks'
 * inverses, and its "solve" is the block-diagonal product with them.
 * Inverse of every column-major ns x ns block of blocks[n_blocks][ns*ns] into out_inverses (same layout) by
 * Gauss-Jordan elimination with partial pivoting; out_pivots[n_blocks][ns] receives each block's pivot order (the
 * reference stores LAPACK swap indices there; nothing here reads them). All pointers DEVICE; ns <= 119 on GB300. */
int sf_btddod_blockdiag_factor_batch(int n_blocks, int ns, const double *blocks, double *out_inverses,
                                     int *out_pivots, void *stream);
/* y_i = B_i x_i for every block (btddod_blockdiag_matvec, and btddod_blockdiag_solve when B holds the inverses of
 * sf_btddod_blockdiag_factor_batch). blocks DEVICE [n_blocks][ns*ns] column-major, x and out_y DEVICE
 * [n_blocks][ns] (must not alias). */
int sf_btddod_blockdiag_matvec_batch(int n_blocks, int ns, const double *blocks, const double *x, double *out_y,
                                     void *stream);
/* Block-triangular solves of BTDDOD matrices with the inverses of their diagonal blocks (btddod_lowerfulltriangle_solve
 * with upper = 0: x_0 = D_0^-1 b_0, x_i = D_i^-1 (b_i - sub_{i-1} o x_{i-1}); btddod_upperfulltriangle_solve with
 * upper = 1: x_{nzi-1} = D_{nzi-1}^-1 b_{nzi-1}, x_i = D_i^-1 (b_i - sup_i o x_{i+1})). inverses DEVICE
 * [points][ns*ns] (from sf_btddod_blockdiag_factor_batch on each flamelet's diagonal blocks), values the BTDDOD
 * values (only sub / sup are read), rhs and out_x DEVICE [points][ns] (must not alias). */
int sf_btddod_triangle_solve_batch(int n_flamelets, int ns, const int *offsets_z, const long long *offsets_v,
                                   const int *offsets_z_host, const double *inverses, const double *values,
                                   const double *rhs, double *out_x, int upper, const int *active, void *stream);
/* A <- matrix_scale*A + diag_scale*B (btddod_matrix_kernels.cpp:430-446), B a block diagonal DEVICE
 * [points][ns*ns] (column-major blocks) added to each flamelet's diagonal blocks. */
int sf_btddod_scale_and_add_block_diagonal_batch(int n_flamelets, int ns, const int *offsets_z,
                                                 const long long *offsets_v, const int *offsets_z_host,
                                                 double *values, double matrix_scale, const double *block_diag,
                                                 double diag_scale, const int *active, void *stream);

/* Steady flamelet solvers for every flamelet of a batch, each with its own iteration count, line search, Jacobian
 * reuse and (psitc) pseudo-time steps and restarts: Flamelet.steady_solve_newton (flamelet.py:1352-1485) and
 * Flamelet.steady_solve_psitc (flamelet.py:1487-1703), which a Python caller runs one flamelet at a time. Both
 * replace the per-flamelet solver loop of Flamelet.compute_steady_state (flamelet.py:1705-1778) for a batch.
 * Every vector operation, norm and per-flamelet decision runs on the device; the call synchronizes `stream` a few
 * times per iteration to read whether any flamelet still iterates, needs a new Jacobian, cuts its step or
 * restarts. state: DEVICE [points][ns] in/out, the initial guess on entry; on return each flamelet's last iterate,
 * clamped at 0 (as the reference's solvers return it). active: DEVICE int [n_flamelets] or NULL; inactive
 * flamelets are not iterated (their state is still clamped) and report converged 0. fb->active, fb->prefactor and
 * fb->diffterm are ignored. Norms are the reference's: the infinity norm of the residual with the temperature rows
 * divided by 1e3. out_converged, out_iterations: DEVICE int [n_flamelets]; out_min_ds (psitc, DEVICE
 * [n_flamelets] or NULL): the smallest pseudo-time step of each flamelet where it stopped (the reference's psitc
 * returns it and compute_steady_state starts its ESDIRK fallback from 1e-2 of it). Factors and Jacobians live in
 * the workspace (sf_flamelet_steady_workspace_size bytes, DEVICE, 256-byte aligned); a call uses it alone.
 *
 * Newton: damped Newton with a Jacobian reused until a line search cut; the line search halves the step (at most
 * 12 times, while alpha > 1e-3) while the new residual norm exceeds max_factor_line_search times the old one. A
 * flamelet fails on a non-finite step or residual, a residual above max_allowed_residual, or a state value below
 * min_allowable_state_var; it converges when its residual norm is <= tolerance within max_iterations. */
size_t sf_flamelet_steady_workspace_size(const sf_mech *mech, const sf_flamelet_batch *fb);
int sf_flamelet_steady_newton_batch(const sf_mech *mech, const sf_flamelet_batch *fb, double *state,
                                    const int *active, double tolerance, int max_iterations,
                                    double max_factor_line_search, double max_allowed_residual,
                                    double min_allowable_state_var, int rates_option, int *out_converged,
                                    int *out_iterations, void *workspace, size_t workspace_bytes, void *stream);
/* psitc: pseudo-transient continuation, (ds^-1 I - J) dx = r with a per-row pseudo-time step ds refreshed with every
 * Jacobian: ds <- min(ds_safety / (expeig + 1e-16), ds_ramp * ds, ds_max), expeig the eigenvalue bound of
 * sf_flamelet_jac_batch with diffterm[f] (DEVICE [n_flamelets], the reference's diffusion_factor * max(chi) of each
 * flamelet), and on a flamelet's first Jacobian (or every one with global_ds) the flamelet's smallest ds on all its
 * rows. The Jacobian is refreshed after 8 uses or while the residual norm exceeds 1e-2, and after a line search
 * cut. A failure (non-finite step or residual, residual above max_allowed_residual, state below
 * min_allowable_state_var) restarts the flamelet from its initial guess with ds_init divided by ds_init_decrease
 * (adaptive_restart), until a failure at restart depth > max_recursion_depth ends it unconverged. */
int sf_flamelet_steady_psitc_batch(const sf_mech *mech, const sf_flamelet_batch *fb, double *state,
                                   const int *active, const double *diffterm, double tolerance, int max_iterations,
                                   double min_allowable_state_var, double ds_init, double ds_init_decrease,
                                   int global_ds, double ds_safety, double ds_ramp, double ds_max,
                                   double max_factor_line_search, double max_allowed_residual,
                                   int max_recursion_depth, int adaptive_restart, int rates_option,
                                   int *out_converged, int *out_iterations, double *out_min_ds, void *workspace,
                                   size_t workspace_bytes, void *stream);

/* One ESDIRK64 step attempt (time/methods.py:441-612 with SimpleNewtonSolver, time/nonlinear.py:185-268) of every
 * running flamelet of a batch, each with its own step size: the transient flamelet integration of Flamelet.integrate
 * (flamelet.py:1046-1213) without its step-size control, which the caller keeps (one call per attempt):
 *   - where setup[f] (any_setup != 0 when any is set): the iteration matrix gamma dt_f J - I and its block-Thomas
 *     factors, kept in the workspace for the following attempts (pass the same workspace to every attempt);
 *   - k_0 = F(state); for s = 1..5 the implicit stage Y_s = state + dt (gamma F(Y_s) + sum_{j<s} a_sj k_j) by the
 *     simplified Newton iteration with those factors, at most max_nonlinear_iter iterations, converged when the
 *     weighted infinity norm of its residual (temperature rows divided by 1e3) is below nonlinear_tolerance;
 *   - the step dt sum_s b_s k_s and the error estimate dt sum_s (b_s - bhat_s) k_s.
 * A running flamelet whose step is finite gets state <- max(state + step, 0). Per flamelet (DEVICE [n_flamelets]):
 * out_err the weighted norm of the error estimate, out_step_norm that of the step, out_nonfinite 1.0 if the step has
 * a non-finite entry, out_nl_ok 0 if a stage's Newton iteration did not converge; inout_newton += iterations.
 * state DEVICE [points][ns] in/out; dt DEVICE [n_flamelets]; run, setup DEVICE int [n_flamelets]. The arithmetic
 * is evaluated with one rounding per operation in the order of the reference's vector expressions. The call reads
 * back one flag per Newton iteration (whether any flamelet still iterates). workspace: DEVICE,
 * sf_flamelet_esdirk_workspace_size bytes. */
size_t sf_flamelet_esdirk_workspace_size(const sf_mech *mech, const sf_flamelet_batch *fb);
int sf_flamelet_esdirk_attempt_batch(const sf_mech *mech, const sf_flamelet_batch *fb, double *state,
                                     const double *dt, const int *run, const int *setup, int any_setup,
                                     double nonlinear_tolerance, int max_nonlinear_iter, int rates_option,
                                     double *out_err, double *out_step_norm, double *out_nonfinite, int *out_nl_ok,
                                     int *inout_newton, void *workspace, size_t workspace_bytes, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* SPITFIRE_GB300_H */
