/*
 * fluid2d_gb300 — C ABI of a GB300-native (sm_103a) solver step for mworchel/fluid-2d.
 *
 * The reference exposes one operation, the abstract
 *     fluid_solver::solve(density, density_src, diffusion_rate,
 *                         u, v, u_src, v_src, viscosity, dt)
 * (src/fluid_solver.hpp:16-24), implemented on the GPU by fluid_solver_gpu
 * (src/fluid_solver_gpu.cuh:9-70, src/fluid_solver_gpu.cu:209-404). This header is the
 * drop-in boundary for that operation: plain C, plain pointers and sizes, no C++ or
 * torch types. A header-only adapter implementing the reference's class interface on top
 * of it is in include/fluid_solver_gb300.hpp.
 *
 * Grids are row-major float32 arrays of rows*cols values, element (i, j) at i*cols + j,
 * rows and cols INCLUDING the one-cell boundary — the layout of the reference's
 * grid<float> (src/grid.hpp:60-69) and the (rows, cols) the reference's GPU solver is
 * constructed with (src/fluid_solver_gpu.cuh:14, src/simulation.cpp:22).
 *
 * Every function returns an int status (FS_OK on success). The reference reports no
 * errors at all (its solve() is void and ignores every cudaError_t); here a failed CUDA
 * call, a bad argument, a non-finite result or an unconverged pressure solve each has a
 * code, and fs_last_error() gives a message for the calling thread's last failure.
 *
 * Threading: a solver handle owns one CUDA stream on one device and is used by one host
 * thread at a time. fs_solve_host() is synchronous like the reference; fs_step() and
 * the upload/download calls are asynchronous on the handle's stream until fs_sync().
 */
#ifndef FLUID2D_GB300_H
#define FLUID2D_GB300_H

#if defined(__GNUC__)
#define FS_API __attribute__((visibility("default")))
#else
#define FS_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define FS_OK 0
#define FS_ERR_ARG 1          /* invalid argument (null pointer, size < 3, bad enum) */
#define FS_ERR_CUDA 2         /* a CUDA runtime call failed; see fs_last_error() */
#define FS_ERR_NONFINITE 3    /* the step produced a NaN or Inf (state is still updated) */
#define FS_ERR_NOT_CONVERGED 4/* residual-driven pressure solve hit its iteration cap */
#define FS_ERR_TIMEOUT 5      /* a bounded host wait ran out */
#define FS_ERR_NOMEM 6        /* device or pinned host allocation failed */
#define FS_ERR_STATE 7        /* call not valid in the handle's current state */

/* Pressure warm start for the projection (the reference always starts from zero:
 * p_buffer.clear(0), src/fluid_solver_gpu.cu:364). */
#define FS_WARM_ZERO 0
#define FS_WARM_PREVIOUS 1
#define FS_WARM_LEARNED 2 /* network corrections of the pressure (fs_set_network): of the previous
                            pressure with a fixed sweep count; with a residual target, of the
                            current pressure every learned_cycle_iterations sweeps */

/* Solution method of the step. FS_METHOD_JACOBI is the reference's CUDA solver
 * (fluid_solver_gpu, src/fluid_solver_gpu.cu:209-404). FS_METHOD_GAUSS_SEIDEL reproduces
 * the reference's host solver (fluid_solver_cpu, src/fluid_solver_cpu.cpp:6-215) bit for
 * bit: in-place lexicographic sweeps, corner-averaging fills, no smoothing. It needs a
 * square grid of at most fs_gauss_seidel_max_size() cells a side, pressure from zero and a
 * fixed iteration count; the host solver uses 20 diffusion and 20 pressure sweeps
 * (src/fluid_solver_cpu.cpp:14,24). */
#define FS_METHOD_JACOBI 0
#define FS_METHOD_GAUSS_SEIDEL 1

typedef struct fs_solver fs_solver;

typedef struct fs_config {
    int rows;                  /* grid rows including the boundary, >= 3 */
    int cols;                  /* grid cols including the boundary, >= 3 */
    int diffuse_iterations;    /* Jacobi sweeps per diffusion; reference: 15 (fluid_solver_gpu.cu:238) */
    int pressure_iterations;   /* Jacobi sweeps per projection; reference: 20 (fluid_solver_gpu.cu:247) */
    int smooth;                /* 1: 5-point density smoothing after advection (fluid_solver_gpu.cu:240) */
    int sweeps_per_pass;       /* temporal-blocking depth (sweeps per HBM pass), 0 = tuned default */
    int tile_rows;             /* stencil region height: 64 or 128, 0 = tuned default */
    int use_graph;             /* 1: replay each step as a captured CUDA graph */
    int device;                /* CUDA device ordinal, -1 = the calling thread's current device */
    int warm_start;            /* FS_WARM_ZERO or FS_WARM_PREVIOUS */
    float pressure_tolerance;  /* > 0: run the pressure solve to this relative residual (tested
                                  after every second pass of sweeps_per_pass sweeps and after
                                  the last pass the cap allows) */
    int pressure_max_iterations; /* iteration cap when pressure_tolerance > 0 */
    int check_finite;          /* 1: flag NaN/Inf in the step's outputs (FS_ERR_NONFINITE) */
    int capture;               /* 1: keep each projection's divergence and starting pressure
                                  for fs_capture_view (training-data generation) */
    int method;                /* FS_METHOD_JACOBI (default) or FS_METHOD_GAUSS_SEIDEL */
    int learned_cycles;        /* FS_WARM_LEARNED with a residual target: most network
                                  corrections per projection, each followed by Jacobi sweeps;
                                  0 = as many as pressure_max_iterations allows. Steps stop at
                                  convergence (read on the host after each segment). */
    int learned_cycle_iterations; /* Jacobi sweeps after each correction; 0 = 256 */
    int learned_grid;          /* coarse grid side of the network, 32 or 64; 0 = 32 */
    int learned_defect;        /* FS_WARM_LEARNED with a residual target, steps driven from the host:
                                  1 (default) = mixed-precision defect correction (the pressure
                                  kept as two FP32 parts, each cycle solving for a correction of
                                  the residual of their sum, formed in double-float arithmetic);
                                  0 = corrections of the FP32 pressure */
} fs_config;

typedef struct fs_stats {
    long long steps;                 /* solver steps completed */
    long long kernel_launches;       /* kernels of this library launched so far */
    int launches_per_step;           /* kernels per step in the current plan */
    int passes_per_step;             /* HBM passes of the stencil kernels per step */
    int sweeps_per_pass;             /* temporal-blocking depth in use */
    int tile_rows;                   /* stencil region height in use */
    int pressure_iterations_last[2]; /* sweeps used by the two projections of the last step */
    double pressure_residual_last[2];/* their final relative residuals (residual mode only) */
    int nonfinite;                   /* 1 if a NaN/Inf was flagged since the last check */
    long long learned_used;          /* network corrections kept (they lowered the residual) */
    long long learned_fallback;      /* corrections rejected: the uncorrected pressure was better */
} fs_stats;

/* Device view of the resident state, for zero-copy use by other CUDA code. Each field
 * is rows x pitch floats (pitch >= cols, a multiple of 32); element (i, j) at i*pitch + j. */
typedef struct fs_device_view {
    float* density;
    float* u;
    float* v;
    float* density_source;
    float* u_source;
    float* v_source;
    int rows, cols, pitch;
    void* stream; /* cudaStream_t */
} fs_device_view;

/* Fill *cfg with the reference GPU solver's behaviour for a rows x cols grid:
 * 15 diffusion sweeps, 20 pressure sweeps, smoothing on, zero warm start. */
FS_API int fs_config_init(fs_config* cfg, int rows, int cols);

/* Replaces fluid_solver_gpu::fluid_solver_gpu(rows, cols) (fluid_solver_gpu.cu:209-218):
 * allocates the device state for one grid. */
FS_API int fs_create(const fs_config* cfg, fs_solver** out);

/* Largest grid side (rows = cols, boundary included) that FS_METHOD_GAUSS_SEIDEL accepts
 * on the calling thread's current device (16384). Grids whose field fits one SM's shared
 * memory (234 a side on a GB300) run each solve in one CTA; larger ones run it as a tiled
 * wavefront over the whole GPU. Writes 0 when no device is usable. */
FS_API int fs_gauss_seidel_max_size(int* n);

/* Device-resident simulation driver: the reference's simulation::add_*_source and
 * simulation::update (src/simulation.cpp:44-64) on the handle's source grids, so a frame
 * loop never moves a field through host memory. A source event adds value * cols * rows
 * (float arithmetic, in that order, as simulation.cpp:45,49-50) to cell (i, j) of the
 * density source, or the horizontal / vertical velocity sources. */
#define FS_SOURCE_DENSITY 0
#define FS_SOURCE_VELOCITY 1
typedef struct fs_source_event {
    int step;     /* fs_run_script: the step (0-based within the call) it belongs to */
    int kind;     /* FS_SOURCE_DENSITY or FS_SOURCE_VELOCITY */
    int i, j;     /* cell (row, column), boundary included */
    float value;  /* density, or horizontal velocity */
    float value2; /* vertical velocity (FS_SOURCE_VELOCITY) */
} fs_source_event;

/* simulation::add_density_source / add_velocity_source (simulation.cpp:44-51), on the
 * device, asynchronous on the handle's stream. */
FS_API int fs_add_density_source(fs_solver* s, int i, int j, float value);
FS_API int fs_add_velocity_source(fs_solver* s, int i, int j, float horizontal, float vertical);
/* simulation::update (simulation.cpp:53-64): one step with the accumulated sources, then
 * the three source grids cleared. Asynchronous. */
FS_API int fs_update(fs_solver* s, float diffusion_rate, float viscosity, float dt);
/* nsteps updates driven by a script: before step k the events with step == k are added
 * in array order (events must be sorted by step; steps outside [0, nsteps) are an
 * error), then the step runs and the sources are cleared. Asynchronous. */
FS_API int fs_run_script(fs_solver* s, const fs_source_event* events, int count, int nsteps,
                         float diffusion_rate, float viscosity, float dt);

/* Replaces fluid_solver_gpu::~fluid_solver_gpu (fluid_solver_gpu.cu:220). NULL is a no-op. */
FS_API int fs_destroy(fs_solver* s);

/* Message for the calling thread's last failed call ("" when none). */
FS_API const char* fs_last_error(void);

/* Replaces fluid_solver_gpu::solve (fluid_solver_gpu.cu:222-258), argument for
 * argument: uploads density/u/v and the three source grids from host memory, runs one
 * step, downloads density/u/v, and returns when they are written. Host buffers may be
 * pageable; pinned buffers (fs_host_alloc) copy faster. On grids of 2^20 cells and more
 * the copies overlap the step (density first and diffusing while u and v upload; the new
 * density downloading while the velocity is projected); the results are those of
 * fs_upload + fs_upload_sources + fs_step + fs_download. On failure no copy from or into
 * the host buffers is still in flight when the call returns. */
FS_API int fs_solve_host(fs_solver* s, float* density, const float* density_source, float diffusion_rate,
                  float* u, float* v, const float* u_source, const float* v_source, float viscosity,
                  float dt);

/* Device-resident stepping (no per-step host round trip). */
FS_API int fs_upload(fs_solver* s, const float* density, const float* u, const float* v);
FS_API int fs_upload_sources(fs_solver* s, const float* density_source, const float* u_source,
                      const float* v_source);
FS_API int fs_step(fs_solver* s, float diffusion_rate, float viscosity, float dt, int nsteps);
FS_API int fs_download(fs_solver* s, float* density, float* u, float* v);
FS_API int fs_sync(fs_solver* s);

/* Bound of the grid-wide barrier wait in a residual-driven pressure solve
 * (pressure_tolerance > 0), in polls of about 120 ns; 0 restores the default (2^24 polls,
 * about 2 s). When a wait runs out the solve stops, the step's velocity is left
 * unprojected and fs_sync / fs_step return FS_ERR_TIMEOUT; the handle stays usable.
 * The reference has no bounded waits (it has no grid-wide synchronisation at all). */
FS_API int fs_set_barrier_poll_limit(fs_solver* s, unsigned polls);

FS_API int fs_get_stats(const fs_solver* s, fs_stats* out);
FS_API int fs_device_view_get(fs_solver* s, fs_device_view* out);

/* Learned warm start (FS_WARM_LEARNED): load the network's FP32 parameters (8 layers x
 * (32x9x32 weights [co][tap][ci] + 32 biases) = FS_NET_PARAMS floats, host memory). The
 * grid must be square with an interior divisible by FS_NET_GRID. The network runs on a
 * G x G coarse grid (G = FS_NET_GRID or FS_NET_GRID_MAX, config learned_grid) on block
 * sums of the pressure's residual; its correction
 * is post-smoothed on the coarse grid, interpolated and added where it brings the
 * pressure closer to the solution (see fs_config.learned_cycles). */
#define FS_NET_GRID 32
#define FS_NET_GRID_MAX 64
#define FS_NET_PARAMS (8 * (32 * 9 * 32 + 32))
FS_API int fs_set_network(fs_solver* s, const float* params, long long count);

/* Device pointers (rows x pitch, see fs_device_view) to the divergence and the starting
 * pressure of projection `slot` (0 or 1) of the last step, and to its final pressure;
 * requires cfg.capture (divergence, start) and a warm-start mode (final). */
FS_API int fs_capture_view(fs_solver* s, int slot, float** div, float** p_start, float** p_final);

/* Device-to-device copy on a stream (helper for callers holding raw device pointers). */
FS_API int fs_memcpy_device(void* dst, const void* src, unsigned long long bytes, void* stream);

/* Headless render kernels on device fields (rows x pitch floats), for the
 * reference's display path without its SFML window:
 *   fs_render_density: RGBA8 image, rows*cols*4 bytes, as grid_to_image_kernel
 *     (src/density_grid_renderer.cu:10-29);
 *   fs_render_velocity_lines: 2 vertices per cell in sf::Vertex layout (x, y floats,
 *     RGBA bytes, u, v texture floats = 20 bytes), as velocity_to_lines_kernel
 *     (src/velocity_grid_renderer.cu:8-44). Outputs are device buffers. */
FS_API int fs_render_density(const float* density, int rows, int cols, int pitch, float mr, float mg, float mb,
                             void* rgba, void* stream);
FS_API int fs_render_velocity_lines(const float* u, const float* v, int rows, int cols, int pitch, float hscale,
                                    float vscale, void* vertices, void* stream);

/* Checkpoint / resume (no counterpart in the reference). File layout, little endian:
 *   char magic[8] = "FS2DCKP1"; int32 rows, cols, warm_valid, reserved; int64 steps;
 *   then rows*cols float32 each of density, u, v, sources (3), warm-start pressures (2).
 * fs_checkpoint_load needs a handle of the same rows/cols; it restores the state, the
 * sources, the warm-start pressures and the step counter. */
FS_API int fs_checkpoint_save(fs_solver* s, const char* path);
FS_API int fs_checkpoint_load(fs_solver* s, const char* path);

/* Single stages of the step on the resident state, for kernel-level checks. The
 * stage runs with the handle's sweep counts and leaves its result in the state. */
#define FS_STAGE_DIFFUSE_DENSITY 1  /* add_sources + diffuse (fluid_solver_gpu.cu:237-238) */
#define FS_STAGE_ADVECT_DENSITY 2   /* forward advection + smooth (fluid_solver_gpu.cu:239-240) */
#define FS_STAGE_DIFFUSE_VELOCITY 3 /* add_sources + diffuse u, v (fluid_solver_gpu.cu:243-246) */
#define FS_STAGE_PROJECT 4          /* project (fluid_solver_gpu.cu:358-404) */
#define FS_STAGE_ADVECT_VELOCITY 5  /* backtrace advection of u, v (fluid_solver_gpu.cu:248-251) */
FS_API int fs_stage(fs_solver* s, int stage, float rate, float dt);

/* Autotuner: times whole steps of candidate stencil tilings (region height 64/128 x
 * blocking depth 2..16) for cfg's grid and sweep plan on the device (on a smooth
 * velocity field with divergence everywhere, so that residual-target solves do real
 * work) and writes the
 * fastest into cfg->tile_rows / cfg->sweeps_per_pass. With a cache_path the choice is
 * looked up first and stored after tuning (key: device, SM count, rows, cols, kd, kp,
 * tolerance, warm start). No counterpart in the reference (fixed 32x32 launches,
 * kernel_launcher.hpp:14-16). best_ms (nullable) receives the time per step. */
FS_API int fs_autotune(fs_config* cfg, float diffusion_rate, float viscosity, float dt, int steps,
                       const char* cache_path, double* best_ms);

/* Autotuner for batches: the same search (region heights 64 and 128; depths 2, 4, ..., 16
 * and those that split cfg->pressure_iterations into two, three or four equal passes)
 * over whole steps of a batch of `count` grids of rows[k] x cols[k], each on a smooth
 * divergent tuning state, `steps` timed steps after one warm-up step per candidate; the
 * fastest goes into cfg->tile_rows / cfg->sweeps_per_pass for fs_batch_create. With
 * cache_path the choice is looked up first and stored after tuning (key: device, SM
 * count, a hash of the shapes, kd, kp). No counterpart in the reference. */
FS_API int fs_batch_autotune(fs_config* cfg, int count, const int* rows, const int* cols, float diffusion_rate,
                             float viscosity, float dt, int steps, const char* cache_path, double* best_ms);

/* Batches: many independent grids of uneven size advanced together. No counterpart
 * in the reference (which steps one grid per fluid_solver_gpu object). Every sub-step
 * of the step is one launch over all grids; the step is replayed as a CUDA graph.
 * Grids share dt, the rates, the sweep counts and the config (cfg->rows/cols are
 * ignored; rows[k], cols[k] give grid k, boundary included). Residual-driven pressure
 * and warm starts are not available for batches. */
typedef struct fs_batch fs_batch;
FS_API int fs_batch_create(const fs_config* cfg, int count, const int* rows, const int* cols, fs_batch** out);
FS_API int fs_batch_destroy(fs_batch* b);
FS_API int fs_batch_upload(fs_batch* b, int index, const float* density, const float* u, const float* v);
FS_API int fs_batch_upload_sources(fs_batch* b, int index, const float* density_source, const float* u_source,
                                   const float* v_source);
FS_API int fs_batch_step(fs_batch* b, float diffusion_rate, float viscosity, float dt, int nsteps);
FS_API int fs_batch_download(fs_batch* b, int index, float* density, float* u, float* v);
FS_API int fs_batch_sync(fs_batch* b);
FS_API int fs_batch_get_stats(const fs_batch* b, fs_stats* out);
FS_API int fs_batch_stream(fs_batch* b, void** stream);

/* Per-kernel timing of one step. The step is captured in the shape of the timed graph —
 * the same launches on the same streams, the density branch beside the main stream —
 * with an event-record node around every launch on the stream it runs on, and replayed
 * once (steps whose results are read on the host, learned residual solves, run eagerly). For each kernel kind: the launch count and summed event time, the part of both
 * that ran on the density branch (concurrently with the main stream, so the main
 * stream's total ms - branch_ms never exceeds the step), the algorithmic bytes of the
 * per-sweep model (each input field read once and each output written once per sweep,
 * the cost of the reference's one-kernel-per-sweep design) and the pass bytes (each
 * array a launch itself reads or writes, once: what a temporally blocked pass must move
 * through HBM). The state advances by one step. */
#define FS_KIND_STENCIL 0   /* diffusion / pressure passes (temporally blocked) */
#define FS_KIND_SPLAT 1     /* forward density advection */
#define FS_KIND_FINISH 2    /* density fill + smoothing */
#define FS_KIND_ADVECT 3    /* velocity backtrace advection */
#define FS_KIND_MEMSET 4    /* accumulator clear (a memset node, not a kernel) */
#define FS_KIND_GRADIENT 5  /* gradient subtract + reflecting fills after a multi-pass projection */
#define FS_NUM_KINDS 6
typedef struct fs_kernel_times {
    int launches[FS_NUM_KINDS];
    double ms[FS_NUM_KINDS];
    double algorithmic_bytes[FS_NUM_KINDS];
    double pass_bytes[FS_NUM_KINDS];
    int branch_launches[FS_NUM_KINDS];
    double branch_ms[FS_NUM_KINDS];
} fs_kernel_times;
FS_API int fs_profile_step(fs_solver* s, float diffusion_rate, float viscosity, float dt, fs_kernel_times* out);

/* Pressure projection that allocates nothing. No counterpart in the reference.
 *
 * For callers that cannot call cudaMalloc: code running inside a host framework that
 * owns all device memory (a fixed pool or budget), plug-ins whose host application hands
 * them device buffers but no allocator, and frame loops that must not allocate after
 * start-up. fs_create() allocates, so they cannot use a handle.
 *
 * Projects (u, v) -> (u_out, v_out) with `iterations` Jacobi sweeps from zero pressure:
 * the same result as fs_stage(FS_STAGE_PROJECT) on a handle created with
 * pressure_iterations = iterations and warm_start = FS_WARM_ZERO. All four arrays are
 * the caller's device buffers of rows x pitch floats (element (i, j) at i*pitch + j,
 * rows/cols including the boundary); no output may overlap an input or the other output
 * (FS_ERR_ARG). Work is queued on `stream` (a cudaStream_t; NULL = default stream) and is
 * asynchronous.
 *
 * Scratch (divergence and two pressure buffers) lives in a fixed file-scope device
 * array of 3 x FS_NOALLOC_MAX_CELLS floats (12 MiB) that every GPU loading this library
 * holds until process exit; rows * pitch above FS_NOALLOC_MAX_CELLS is rejected with
 * FS_ERR_ARG. The first call on a device looks up that array's address and caches it;
 * make that first call before any stream capture begins on the device.
 * After cudaDeviceReset() on a device the cached
 * address is stale and further calls on that device are not supported. All calls share
 * the array, so calls that may overlap on the GPU race and must be serialised by the
 * caller. */
#define FS_NOALLOC_MAX_CELLS 1048576
FS_API int fs_project_noalloc(const float* u, const float* v, float* u_out, float* v_out, int rows, int cols,
                              int pitch, int iterations, void* stream);

/* 3x3 convolution building block of the learned pressure warm start (no counterpart
 * in the reference). Activations are NHWC BF16 with 32 channels; output (H x W), input
 * (H x W) or (H/2 x W/2) nearest-upsampled when up = 1; zero padding. y = act(conv(x) +
 * bias + skip), act = ReLU when relu = 1; y (BF16) and/or yf (FP32) receive it.
 * use_tensor_cores = 1 runs the tcgen05 implicit GEMM with `wpk` (weights packed by
 * fs_conv_pack_weights); 0 runs the CUDA-core reference with the FP32 weights `w32`
 * ([co][tap][ci], 32 x 9 x 32). All pointers are device pointers; `err` (nullable) is
 * set if a tensor-core wait gave up. */
FS_API int fs_conv_pack_weights(const float* w32, void* wpk, void* stream);
/* The whole 8-layer network of the learned warm start on `images` 32 x 32 grids in one
 * launch (one CTA per grid, activations in shared memory, every conv on tcgen05):
 * x0 (images x 32 x 32 x 32 BF16 NHWC), wpk (8 x 9216 packed weights, fs_conv_pack_weights
 * of each layer), params (the FP32 parameters, 8 x 9248: weights then 32 biases per
 * layer), e1 (scratch of x0's size), y (FP32 output, images x 32 x 32 x 32). Same
 * results as the layer-by-layer fs_conv3x3 sequence. */
FS_API int fs_net_infer32(const void* x0, const void* wpk, const float* params, void* e1, float* y, int images,
                          int* err, void* stream);
FS_API int fs_conv3x3(const void* x, const void* wpk, const float* w32, const float* bias, const void* skip,
                      void* y, float* yf, int H, int W, int img_h, int up, int relu, int use_tensor_cores,
                      int* err, void* stream);

/* Remaining building blocks of the learned warm start (no counterpart in the reference),
 * on device pointers, NHWC with 32 channels, images stacked along rows:
 *   avgpool2 (BF16, rows_out x w_out output) and its backward (FP32, dx = dy/4 broadcast);
 *   upsample2_bwd: dlow = 2x2 block sums of dup; relu_bwd: dz = (da + da2) * (a > 0),
 *   FP32 and BF16 copies; weight_grad: dw += sum_p dz x im2col(x), db += sum_p dz (CUDA
 *   cores, FP32 atomics); flip_weights: weights of the backward-data convolution;
 *   mse: loss on channel 0 and its gradient (per-CTA partial sums of squared error);
 *   adam: one Adam step on FP32 weights (frozen mask nullable);
 *   restrict: block sums of the Poisson residual of p_prev (null = zero) over the G x G
 *   network grid into work (G*G floats), their RMS into *scale, network input channel 0 =
 *   sums / scale (BF16, G*G*32), optional block means of p_prev into pc;
 *   prolong: p_out = p_prev + bilinear interpolation of channel 0 of y times scale*kappa. */
FS_API int fs_net_avgpool2(const void* x, void* y, int rows_out, int w_out, void* stream);
FS_API int fs_net_avgpool2_bwd(const float* dy, float* dx, int rows_in, int w_in, void* stream);
FS_API int fs_net_upsample2_bwd(const float* dup, float* dlow, int rows_low, int w_low, void* stream);
FS_API int fs_net_relu_bwd(const float* da, const float* da2, const void* a, float* dz, void* dzb, long long n,
                           int relu, void* stream);
FS_API int fs_net_weight_grad(const float* dz, const void* x, float* dw, float* db, int H, int W, int img_h, int up,
                              void* stream);
/* The weight gradient on the tensor cores: dw += sum_p dz x im2col(x) and db += sum_p dz
 * from the BF16 copy dzb of dz, as a tcgen05 implicit GEMM over the pixels (FP32
 * accumulation in tensor memory), per-CTA partial sums in `work` (work_floats floats;
 * fs_net_weight_grad_tc_work_floats() is enough for any size on the current device)
 * and a fixed-order reduction, so the result is deterministic. `err` as in fs_conv3x3. */
FS_API long long fs_net_weight_grad_tc_work_floats(int H, int W);
FS_API int fs_net_weight_grad_tc(const void* dzb, const void* x, float* dw, float* db, float* work,
                                 long long work_floats, int H, int W, int img_h, int up, int* err, void* stream);
FS_API int fs_net_flip_weights(const float* w, float* wt, void* stream);
FS_API int fs_net_mse(const float* y, const float* target, float* dy, float* loss_part, long long n, void* stream);
FS_API int fs_net_adam(float* w, const float* g, float* m, float* v, long long n, float lr, float b1, float b2,
                       float eps, int step, const unsigned char* frozen, void* stream);
FS_API int fs_net_restrict(const float* div, const float* p_prev, int rows, int cols, int pitch, int G, float* work,
                           float* scale, void* xin, float* pc, void* stream);
FS_API int fs_net_prolong(const float* y, const float* p_prev, float* p_out, int rows, int cols, int pitch, int G,
                          const float* scale, float kappa, void* stream);

/* Pinned host memory helpers (page-locked; fastest fs_solve_host / upload / download). */
FS_API int fs_host_alloc(void** ptr, unsigned long long bytes);
FS_API int fs_host_free(void* ptr);

/* Library build identification: "fluid2d_gb300 <version> sm_103a". */
FS_API const char* fs_version(void);

#ifdef __cplusplus
}
#endif

#endif /* FLUID2D_GB300_H */
