// Entry points whose kernels are not in this build yet: they report SF_ERR_UNSUPPORTED.
#include "sf_internal.h"
using namespace sfgb;
extern "C" {
static int nyi(const char *f) { set_error(std::string(f) + ": not available in this build"); return SF_ERR_UNSUPPORTED; }
int sf_flamelet_stencils(const sf_mech *, const double *, int, const double *, const double *, double *, double *,
                         double *, double *, double *) { return nyi("sf_flamelet_stencils"); }
int sf_flamelet_jac_indices(const sf_mech *, int, int *, int *) { return nyi("sf_flamelet_jac_indices"); }
int sf_flamelet_rhs_batch(const sf_mech *, const sf_flamelet_batch *, const double *, double *, void *) { return nyi("sf_flamelet_rhs_batch"); }
int sf_flamelet_jac_batch(const sf_mech *, const sf_flamelet_batch *, const double *, int, int, double, double, double *,
                          double *, void *) { return nyi("sf_flamelet_jac_batch"); }
int sf_btddod_factor_batch(int, int, const int *, const long long *, const int *, double *, double *, int *, void *) { return nyi("sf_btddod_factor_batch"); }
int sf_btddod_solve_batch(int, int, const int *, const long long *, const int *, const double *, const double *,
                          const int *, const double *, double *, void *) { return nyi("sf_btddod_solve_batch"); }
int sf_btddod_matvec_batch(int, int, const int *, const long long *, const double *, const double *, double *, void *) { return nyi("sf_btddod_matvec_batch"); }
int sf_btddod_scale_and_add_diagonal_batch(int, int, const int *, const long long *, const int *, double *, double,
                                           const double *, double, void *) { return nyi("sf_btddod_scale_and_add_diagonal_batch"); }
}
