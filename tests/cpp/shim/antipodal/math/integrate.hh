// Test stand-in for the antipodal reference's integrator configuration (src/antipodal/math/integrate.hh of that
// project), for building tests/cpp/frontend_run.cc where the reference's headers are not installed.
#pragma once

namespace antipodal
{
struct integrate_config
{
    int min_depth = 0;
    int max_depth = 10;
    double tol = 1e-6;
};
} // namespace antipodal
