// Builds the header-only adapter against the reference's own fluid_solver.hpp and
// grid.hpp and drives it exactly as the reference's simulation::update does
// (src/simulation.cpp:53-59). Exit 0 on success, 3 when no CUDA device is present
// (the adapter must then throw rather than silently do nothing), 1 on failure.
#include <cmath>
#include <cstdio>
#include <memory>
#include <stdexcept>

#include "fluid_solver_gb300.hpp"

int main(int argc, char** argv) {
    const std::size_t n = 34;
    const int steps = argc > 1 ? std::atoi(argv[1]) : 3;
    const bool gauss_seidel = argc > 2 && argv[2][0] == 'g';
    std::unique_ptr<fluid_solver> solver;
    try {
        if (gauss_seidel)
            solver = std::make_unique<fluid_solver_gb300_gauss_seidel>();
        else
            solver = std::make_unique<fluid_solver_gb300>(n, n);
    } catch (const std::runtime_error& e) {
        std::printf("create failed: %s\n", e.what());
        return 3;
    }
    grid<float> d(n, n, 0.f), ds(n, n, 0.f), u(n, n, 0.f), v(n, n, 0.f), us(n, n, 0.f), vs(n, n, 0.f);
    for (std::size_t i = 10; i < 20; ++i)
        for (std::size_t j = 12; j < 18; ++j) {
            ds(i, j) = 100.f;
            us(i, j) = 2.f;
            vs(i, j) = -1.f;
        }
    double mass = 0;
    for (int s = 0; s < steps; ++s) solver->solve(d, ds, 1e-4f, u, v, us, vs, 1e-4f, 0.1f);
    for (std::size_t i = 1; i + 1 < n; ++i)
        for (std::size_t j = 1; j + 1 < n; ++j) mass += d(i, j);
    std::printf("mass %.6f\n", mass);
    return (mass > 0 && std::isfinite(mass)) ? 0 : 1;
}
