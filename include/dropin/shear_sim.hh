// Stand-in for the reference's esim/sb/main/shear_sim.hh: put this
// directory first on a reference driver's include path (and build the driver
// from a directory that does not hold the reference's own shear_sim.hh) to
// run it on the GPU through libstzg.so.  It brings the drop-in classes of
// stzg_shear_sim.hh into the global namespace under the reference's names.
#ifndef STZG_DROPIN_SHEAR_SIM_HH
#define STZG_DROPIN_SHEAR_SIM_HH

// the standard headers the reference's header chain provides to drivers
// (stz_model.hh:4-7, tgmg.hh:4-10)
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>

#include "../stzg_shear_sim.hh"

// shear_sim.hh:16, the smoothing cut-off of initialize_random
const double gaussian_fac = 5.;

using stzg::c_field;
using stzg::shear_sim;
using stzg::stz_dynamics;
using stzg::stz_dynamics_linear;
using stzg::stz_dynamics_linear_athermal;
using stzg::stz_dynamics_nonlinear;
using stzg::stz_dynamics_nonlinear_athermal;
using stzg::vec;

#endif
