// fluid_solver_gb300 — header-only drop-in for the reference's fluid_solver_gpu.
//
// Implements the reference's abstract interface
//     class fluid_solver { virtual void solve(grid<float>& density, ...) = 0; }
// (mworchel/fluid-2d src/fluid_solver.hpp:8-25) on top of the C ABI in fluid2d_gb300.h.
// Include it from the reference's source tree (it needs that tree's fluid_solver.hpp
// and grid.hpp on the include path) and link libfluid2d_gb300.so. The one-line change
// in the reference's simulation.cpp:21-23 is
//     m_solver = std::make_unique<fluid_solver_gb300>(config.height, config.width);
//
// Semantics are those of fluid_solver_gpu::solve (fluid_solver_gpu.cu:222-258): the
// call uploads the host grids, runs one step, downloads density/u/v and returns when
// they are written. Unlike the reference, failures are not silent: a failed call throws
// std::runtime_error carrying the library's message.
#pragma once

#include <cstddef>
#include <stdexcept>
#include <string>

#include "fluid2d_gb300.h"
#include "fluid_solver.hpp"

class fluid_solver_gb300 : public fluid_solver {
public:
    // rows/cols include the boundary, as fluid_solver_gpu(rows, cols)
    // (fluid_solver_gpu.cuh:14). The reference hard-codes 15 diffusion and 20 pressure
    // sweeps (fluid_solver_gpu.cu:238, 245-247, 252); they are the defaults here.
    fluid_solver_gb300(std::size_t rows, std::size_t cols, int diffuse_iterations = 15,
                       int pressure_iterations = 20) {
        fs_config cfg;
        check(fs_config_init(&cfg, (int)rows, (int)cols));
        cfg.diffuse_iterations = diffuse_iterations;
        cfg.pressure_iterations = pressure_iterations;
        check(fs_create(&cfg, &m_handle));
    }

    explicit fluid_solver_gb300(const fs_config& cfg) { check(fs_create(&cfg, &m_handle)); }

    fluid_solver_gb300(const fluid_solver_gb300&) = delete;
    fluid_solver_gb300& operator=(const fluid_solver_gb300&) = delete;

    ~fluid_solver_gb300() override { fs_destroy(m_handle); }

    void solve(grid<float>& density_grid, grid<float> const& density_source_grid, float const diffusion_rate,
               grid<float>& horizontal_velocity_grid, grid<float>& vertical_velocity_grid,
               grid<float> const& horizontal_velocity_source_grid,
               grid<float> const& vertical_velocity_source_grid, float const viscosity, float const dt) override {
        check(fs_solve_host(m_handle, density_grid.data(), density_source_grid.data(), diffusion_rate,
                            horizontal_velocity_grid.data(), vertical_velocity_grid.data(),
                            horizontal_velocity_source_grid.data(), vertical_velocity_source_grid.data(),
                            viscosity, dt));
    }

    fs_solver* handle() const { return m_handle; }

private:
    static void check(int rc) {
        if (rc != FS_OK) throw std::runtime_error(std::string("fluid2d_gb300: ") + fs_last_error());
    }

    fs_solver* m_handle = nullptr;
};

// Drop-in for the reference's fluid_solver_cpu (src/fluid_solver_cpu.hpp:11-50): the host
// solver's method (in-place Gauss-Seidel, corner-averaging fills, 20 + 20 sweeps,
// src/fluid_solver_cpu.cpp:6-31), run on the GPU with bit-identical results. Like the
// reference class it is default-constructed and takes its size from the grids passed to
// solve(); the device state is created on the first call and again when the size
// changes. Square grids up to fs_gauss_seidel_max_size() a side.
// simulation.cpp:18-20 becomes
//     m_solver = std::make_unique<fluid_solver_gb300_gauss_seidel>();
class fluid_solver_gb300_gauss_seidel : public fluid_solver {
public:
    fluid_solver_gb300_gauss_seidel() = default;
    fluid_solver_gb300_gauss_seidel(const fluid_solver_gb300_gauss_seidel&) = delete;
    fluid_solver_gb300_gauss_seidel& operator=(const fluid_solver_gb300_gauss_seidel&) = delete;
    ~fluid_solver_gb300_gauss_seidel() override { fs_destroy(m_handle); }

    void solve(grid<float>& density_grid, grid<float> const& density_source_grid, float const diffusion_rate,
               grid<float>& horizontal_velocity_grid, grid<float>& vertical_velocity_grid,
               grid<float> const& horizontal_velocity_source_grid,
               grid<float> const& vertical_velocity_source_grid, float const viscosity, float const dt) override {
        const int n = (int)density_grid.rows();
        if (!m_handle || n != m_n) {
            fs_destroy(m_handle);
            m_handle = nullptr;
            fs_config cfg;
            check(fs_config_init(&cfg, n, n));
            cfg.method = FS_METHOD_GAUSS_SEIDEL;
            cfg.diffuse_iterations = 20;
            cfg.pressure_iterations = 20;
            cfg.smooth = 0;
            check(fs_create(&cfg, &m_handle));
            m_n = n;
        }
        check(fs_solve_host(m_handle, density_grid.data(), density_source_grid.data(), diffusion_rate,
                            horizontal_velocity_grid.data(), vertical_velocity_grid.data(),
                            horizontal_velocity_source_grid.data(), vertical_velocity_source_grid.data(),
                            viscosity, dt));
    }

    fs_solver* handle() const { return m_handle; }

private:
    static void check(int rc) {
        if (rc != FS_OK) throw std::runtime_error(std::string("fluid2d_gb300: ") + fs_last_error());
    }

    fs_solver* m_handle = nullptr;
    int m_n = 0;
};
