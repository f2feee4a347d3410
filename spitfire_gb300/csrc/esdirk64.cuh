// ESDIRK64 (Kennedy and Carpenter, S6P4Q3) tableau as spitfire/time/methods.py:464-500 gives it, shared by the
// batched integrator (integrate_kernels.cu) and the plain one-thread-per-reactor form (plain_kernels.cu).
#pragma once

namespace sfgb {
namespace {

constexpr double kGamma = 0.25;
// ESDIRK64 stage coefficients a_sj (methods.py:464-500)
__constant__ double c_a[6][6] = {
    {0., 0., 0., 0., 0., 0.},
    {0.25, 0.25, 0., 0., 0., 0.},
    {8611. / 62500., -1743. / 31250., 0.25, 0., 0., 0.},
    {5012029. / 34652500., -654441. / 2922500., 174375. / 388108., 0.25, 0., 0.},
    {15267082809. / 155376265600., -71443401. / 120774400., 730878875. / 902184768., 2285395. / 8070912., 0.25, 0.},
    {82889. / 524892., 0., 15625. / 83664., 69875. / 102672., -2260. / 8211., 0.25}};
// stage times c_s = sum_j a_sj, summed left to right as numpy does for methods.py:500 (self.c)
__constant__ double c_c[6] = {
    0.,
    0.25 + 0.25,
    8611. / 62500. + -1743. / 31250. + 0.25,
    5012029. / 34652500. + -654441. / 2922500. + 174375. / 388108. + 0.25,
    15267082809. / 155376265600. + -71443401. / 120774400. + 730878875. / 902184768. + 2285395. / 8070912. + 0.25,
    82889. / 524892. + 0. + 15625. / 83664. + 69875. / 102672. + -2260. / 8211. + 0.25};
__constant__ double c_b[6] = {82889. / 524892., 0., 15625. / 83664., 69875. / 102672., -2260. / 8211., 0.25};
__constant__ double c_bh[6] = {4586570599. / 29645900160., 0., 178811875. / 945068544., 814220225. / 1159782912.,
                               -3700637. / 11593932., 61727. / 225920.};

}  // namespace
}  // namespace sfgb
