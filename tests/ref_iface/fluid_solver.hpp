// Test-only stand-in for the reference's abstract solver interface (mworchel/fluid-2d
// src/fluid_solver.hpp:8-25): one pure virtual solve() over host grids with the same
// parameter list, so include/fluid_solver_gb300.hpp can be built without the checkout.
#pragma once

#include "grid.hpp"

class fluid_solver {
public:
    virtual ~fluid_solver() = default;
    virtual void solve(grid<float>& density, grid<float> const& density_source, float const diffusion_rate,
                       grid<float>& u, grid<float>& v, grid<float> const& u_source,
                       grid<float> const& v_source, float const viscosity, float const dt) = 0;
};
