/*
 * tinyfluids_gb300 -- C ABI of the GB300 (sm_103a) tinyfluids time step.
 *
 * A drop-in for the reference's hot path, tinyfluids/jax_tinyfluids:
 * the first-order Godunov / HLL update of the 3D compressible Euler
 * equations (fluid.py) and its run-to-time loop (time_integration.py).
 *
 * Conventions shared by every entry point:
 *  - A state is a device array of 5 * nx * ny * nz float32 in the
 *    reference's layout [var][x][y][z], z contiguous, var order
 *    rho, vx, vy, vz, p (fluid.py:10-22).  Conserved states use
 *    rho, mx, my, mz, E.
 *  - The caller owns all device memory; no entry point allocates device
 *    memory for states or buffers (a t_final loop instantiates and caches a
 *    CUDA graph, whose resources the CUDA driver holds).  Inputs are never
 *    modified; outputs must not alias inputs.
 *  - `stream` is a cudaStream_t (NULL = legacy default stream).  Work is
 *    enqueued asynchronously unless stated otherwise.  The fused step
 *    kernels are launched with programmatic stream serialization: each waits
 *    for the work before it, and lets the next launch start early, so a
 *    caller's kernel launched after them with that attribute must call
 *    cudaGridDependencySynchronize() before reading their output (ordinary
 *    launches, copies and events are ordered as usual).
 *  - Every function returns a tf_status; tf_last_error() describes the last
 *    failure on the calling thread.
 *
 * The reference has no FFI of its own (it is a JAX program); each entry
 * point cites the reference function whose inputs, outputs and semantics it
 * reproduces.
 */
#ifndef TINYFLUIDS_GB300_H
#define TINYFLUIDS_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define TF_ABI_VERSION 1

typedef enum tf_status {
  TF_OK = 0,
  TF_ERR_ARG = 1,          /* invalid argument (shape, pointer, value) */
  TF_ERR_CUDA = 2,         /* a CUDA runtime call failed */
  TF_ERR_NONFINITE = 3,    /* the max wave speed became NaN/Inf/0: state blew up */
  TF_ERR_TIMEOUT = 4,      /* a bounded device-side wait gave up */
  TF_ERR_UNSUPPORTED = 5   /* valid request this build does not implement */
} tf_status;

/* flags */
#define TF_FLAG_OPEN_BOUNDARIES 1u /* fluid.py:571-572 handle_boundaries=True */
#define TF_FLAG_EXACT 2u           /* reference op order, bit-identical to the oracle */
#define TF_FLAG_IN_CONSERVED 4u    /* tf_evolve_along_axis, fast policy: input is conserved */
#define TF_FLAG_OUT_CONSERVED 8u   /* tf_evolve_along_axis, fast policy: output is conserved */
#define TF_FLAG_HOST_LOOP 16u      /* tf_time_integration, t_final loop: test the condition on
                                      the host once per chunk of steps instead of in a CUDA
                                      graph's device-side while node */

/*
 * Device-resident control block of a run (64 bytes, caller-allocated device
 * memory, tf_ctl_bytes()).  The run-to-time loop keeps t, dt and the
 * iteration count here so that no host synchronisation is needed per step
 * (the reference keeps them in the carry of lax.while_loop,
 * time_integration.py:63-92).
 */
typedef struct tf_ctl {
  float t;            /* simulated time reached */
  float dt;           /* CFL dt of the current state (fluid.py:502) */
  float t_final;      /* loop runs while t < t_final (time_integration.py:85-87) */
  float cfl_dx;       /* C_CFL * dx rounded to float */
  unsigned ws_bits;   /* internal: running max wave speed (float bits) */
  unsigned done;      /* internal: finished-CTA counter */
  int iter;           /* steps taken (the reference's num_iterations) */
  int active;         /* nonzero while the loop condition holds */
  int max_steps;      /* < 0: unbounded */
  int status;         /* TF_OK or a device-detected tf_status */
  float max_speed;    /* max wave speed of the current state */
  int reserved[5];
} tf_ctl;

/* Tile of the fused step kernel; NULL = built-in choice: the y-marching
 * 8-row tile for a fast (or diagnostics / conserved) step on a grid with an
 * even nz and at least 2^17 cells (open boundaries: a fast step on at least
 * 2^27 cells) where it computes no more cells than the x-marching tile, else
 * the x-marching tile (8 rows up to 2^21 cells, 16 above; always 16 for
 * conserved input or output); the chunk length (lx) for about nine waves of
 * resident CTAs in chunks of >= 16 planes (y-marching: <= 64), shorter chunks
 * for grids that would not fill one wave.  tf_resolve_tile reports the
 * choice. */
typedef struct tf_tile_config {
  int rows;    /* x-marching: grid rows (y) per tile incl. the 1-cell ring: 8, 16 or 32
                  (rows/2 warps); y-marching: 8 or 16 (rows/2 x rows per CTA, one warp each) */
  int lx;      /* planes per CTA along the marching axis (x or y; >= 1; 0 = heuristic) */
  int loader;  /* 0 = auto (x-marching, per-thread loads), 1 = x-marching with per-thread
                  loads, 2 = x-marching with TMA-staged planes (needs nz % 4 == 0 and 16-byte
                  aligned states; falls back otherwise), 3 = the y-marching tile (x rows
                  across warps, z pairs per lane, input by cp.async) */
} tf_tile_config;

/* The tile a fused step with these dimensions and flags runs (tile NULL: the
 * built-in choice), written to *out with lx resolved; no counterpart in the
 * reference (introspection of this library's tiling). */
int tf_resolve_tile(int nx, int ny, int nz, unsigned flags, const tf_tile_config *tile,
                    tf_tile_config *out);

int tf_abi_version(void);
const char *tf_status_string(int status);
const char *tf_last_error(void);
unsigned long long tf_ctl_bytes(void);

/* fluid.py:30-67 conserved_state_from_primitive.  W, U: 5*ncells floats. */
int tf_conserved_from_primitive(const float *W, float *U, long long ncells, float gamma,
                                void *stream);

/* fluid.py:71-103 primitive_state_from_conserved. */
int tf_primitive_from_conserved(const float *U, float *W, long long ncells, float gamma,
                                void *stream);

/* fluid.py:427-504 _cfl_time_step.  Writes ctl->dt = C_CFL*dx/max_speed and
 * ctl->max_speed (device), resets the rest of ctl. */
int tf_cfl_time_step(const float *W, int nx, int ny, int nz, float dx, float gamma,
                     float cfl, tf_ctl *ctl, void *stream);

/* fluid.py:562-578 _evolve_state: one split step with a given dt.  dt is
 * read from dt_dev (device float) when non-NULL, else dt_host.  flags:
 * TF_FLAG_OPEN_BOUNDARIES, TF_FLAG_EXACT; or TF_FLAG_IN_CONSERVED |
 * TF_FLAG_OUT_CONSERVED together (fast arithmetic, 16-row tiles): a conserved
 * state in and out, equal bit for bit to the three conserved fast sweeps.
 * tile may be NULL. */
int tf_evolve_state(const float *W_in, float *W_out, int nx, int ny, int nz, float dx,
                    float dt_host, const float *dt_dev, float gamma, unsigned flags,
                    const tf_tile_config *tile, void *stream);

/* Diagnostics (the headless form of scaling_jax.py:75-82 plot_results, which
 * shows rho and p on the plane z = n//2, plus conserved totals); no reference
 * C counterpart.
 *
 * tf_evolve_state_diag: tf_evolve_state (same arguments and result, per-thread
 * loads) that in the same pass writes totals[0..4] = sums over all cells of the
 * NEW state's conserved variables (rho, rho vx, rho vy, rho vz, E per
 * fluid.py:30-67; float32 per thread, float64 across threads; not multiplied
 * by the cell volume) and, when slice is non-NULL, slice[0][x][y] = rho and
 * slice[1][x][y] = p of the plane z = z_slice (2*nx*ny floats).  totals (5
 * device doubles) is zeroed by the call.
 *
 * tf_diagnostics: the same outputs for any stored primitive state in one
 * read pass (float64 sums per thread). */
int tf_evolve_state_diag(const float *W_in, float *W_out, int nx, int ny, int nz, float dx,
                         float dt_host, const float *dt_dev, float gamma, unsigned flags,
                         const tf_tile_config *tile, double *totals, float *slice, int z_slice,
                         void *stream);
int tf_diagnostics(const float *W, int nx, int ny, int nz, float gamma, double *totals,
                   float *slice, int z_slice, void *stream);

/* Verification hooks of the checked build (compiled with TF_CHECKED=1; the
 * product build returns TF_ERR_UNSUPPORTED / -1).  In a checked build the
 * fused step range-checks every global load and store (out-of-range accesses
 * are counted and skipped) and adds 1 to write_counts[cell] (ncells int32 of
 * device memory, cell = (x*ny + y)*nz + z) for every cell it stores.  No
 * reference counterpart (the reference has no race or bounds checking). */
int tf_debug_checked(void);
/* Step cap of the device-side t_final loop for loops started from now on
 * (cap <= 0 or above the default restores the default 2^24): lets a test
 * run a loop into its bound. */
int tf_debug_set_graph_loop_cap(int cap);
/* The simulated time tf_time_integration loops start from (default 0, the
 * reference's, time_integration.py:66; t0 must be finite and >= 0): lets a
 * test start a loop where float32 t no longer advances by dt and see the
 * stall reported.  No reference counterpart (a test hook). */
int tf_debug_set_loop_start_time(float t0);
/* on != 0: fused steps use the 64-bit addressing form that grids of 2^31 or
 * more cells take (both tiles), on every grid, so a test can check that form
 * on small grids; 0 restores the default.  No reference counterpart. */
int tf_debug_force_64bit_offsets(int on);
int tf_debug_reset(int *write_counts, long long ncells);
long long tf_debug_oob_count(void);
/* The adjoint sweep of tf_adjoint_sweep computed one thread per cell with
 * both faces' VJPs recomputed (the form the marching x / y adjoint kernels
 * replace), on any axis: lets a test check that the marching kernels give
 * the same bits.  No reference counterpart. */
int tf_debug_adjoint_sweep_per_cell(const float *U, const float *lam_out, float *lam_in, int nx,
                                    int ny, int nz, float dx, float dt, float gamma, int axis,
                                    void *stream);

/* time_integration.py:94-128 (plain branch): while t < t_final: dt = CFL dt;
 * W = step(W, dt); t += dt; iter += 1.  max_steps >= 0 also bounds the loop
 * (0 = t_final only is NOT implied: pass -1 for unbounded).  fixed_dt > 0
 * replaces the CFL dt (the fixed-dt form used for differentiation).
 * work: scratch state of the same size (ping-pong).  The final state is in
 * W_out; ctl holds t, iter and status.  If iters_host is non-NULL the call
 * blocks until the loop ends and stores the iteration count there.
 * A known step count (max_steps >= 0) enqueues that many predicated steps.
 * A t_final loop (max_steps < 0) runs as one CUDA graph whose while node
 * repeats {steps, condition} on the device until the loop condition fails,
 * float32 t no longer advances (TF_ERR_NONFINITE: the reference would loop
 * forever) or 2^24 steps have run short of t_final (TF_ERR_TIMEOUT):
 * nothing waits on the host.  TF_FLAG_HOST_LOOP instead tests the condition
 * on the host once per chunk of steps. */
int tf_time_integration(const float *W_in, float *W_out, float *work, tf_ctl *ctl, int nx,
                        int ny, int nz, float dx, float t_final, float gamma, float cfl,
                        int max_steps, float fixed_dt, unsigned flags,
                        const tf_tile_config *tile, int *iters_host, void *stream);

/* Device workspace bytes of tf_time_integration_host for `count` states of
 * nx*ny*nz cells: two slots of three states and one control block per state
 * (0 for invalid arguments). */
unsigned long long tf_host_runs_workspace_bytes(int nx, int ny, int nz, int count);

/* time_integration.py:94-128 called with HOST arrays, for a stream of
 * `count` independent states of one grid size: each W_in_host[k] is copied to
 * the device, run with exactly tf_time_integration's loop and arguments, and
 * its final state copied to W_out_host[k].  The copies of one state overlap
 * the runs of its neighbours (two device slots; one copy stream each way, the
 * runs on `stream`), so with pinned host memory the stream runs at about the
 * device's step rate instead of the sum of copy and step times (pageable
 * memory works, without the overlap).  Blocks until every output is in host
 * memory.  iters_host (count ints, may be NULL) receives each run's iteration
 * count; a device-side error is reported with the index of its state.  Inputs
 * may repeat; an output may share memory with its own or earlier inputs (in
 * place), not with a later state's input (TF_ERR_ARG).  workspace: device
 * memory of tf_host_runs_workspace_bytes bytes, 256-byte aligned. */
int tf_time_integration_host(const float *const *W_in_host, float *const *W_out_host, int count,
                             int nx, int ny, int nz, float dx, float t_final, float gamma,
                             float cfl, int max_steps, float fixed_dt, unsigned flags,
                             const tf_tile_config *tile, void *workspace,
                             unsigned long long workspace_bytes, int *iters_host, void *stream);

/* Per-sweep form of fluid.py:508-557 (_evolve_state_along_axis), axis 0..2:
 * reads W_in, writes W_out.  TF_FLAG_OPEN_BOUNDARIES applies the
 * fluid.py:571-572 remap to the input (use it for the x sweep only).
 * TF_FLAG_EXACT: reference op order on primitive states.  Otherwise the fast
 * arithmetic, with TF_FLAG_IN_CONSERVED / TF_FLAG_OUT_CONSERVED selecting a
 * conserved input/output; x (prim->cons), y (cons->cons), z (cons->prim)
 * then reproduce the fused fast step bit for bit. */
int tf_evolve_along_axis(const float *W_in, float *W_out, int nx, int ny, int nz, float dx,
                         float dt_host, const float *dt_dev, float gamma, int axis,
                         unsigned flags, void *stream);

/* ---- the reference's building blocks (exact op order) ----
 * vel is the reference's flux_direction_index (1 = x, 2 = y, 3 = z).
 * Left/right states are full [5][ncells] arrays (the reference passes
 * roll(W, +1, axis) and W). */

/* fluid.py:106-117 speed_of_sound: c = sqrt(gamma*p/rho), n values. */
int tf_speed_of_sound(const float *rho, const float *p, float *c, long long n, float gamma,
                      void *stream);

/* fluid.py:208-259 _euler_flux along vel. */
int tf_euler_flux(const float *W, float *F, long long ncells, float gamma, int vel, void *stream);

/* fluid.py:121-160 get_wave_speeds: S- and S+ per interface. */
int tf_wave_speeds(const float *WL, const float *WR, float *s_minus, float *s_plus,
                   long long ncells, float gamma, int vel, void *stream);

/* fluid.py:164-195 get_max_wave_speeds: max(max|S+|, max|S-|) into
 * ctl->max_speed (ctl is reset first). */
int tf_max_wave_speeds(const float *WL, const float *WR, long long ncells, float gamma, int vel,
                       tf_ctl *ctl, void *stream);

/* fluid.py:263-305 _hll_solver: HLL flux of each (left, right) pair. */
int tf_hll_flux(const float *WL, const float *WR, float *F, long long ncells, float gamma,
                int vel, void *stream);

/* fluid.py:335-413 open boundaries with num_ghost_cells ghost cells, on the
 * axes whose bits (1 = x, 2 = y, 4 = z) are set in lo_axes (left boundary)
 * and hi_axes (right boundary); _open_boundaries is lo = hi = 7. */
int tf_open_boundaries(const float *W, float *out, int nx, int ny, int nz, int num_ghost_cells,
                       unsigned lo_axes, unsigned hi_axes, void *stream);

/* ---- adjoint of the fixed-dt step (conserved variables) ----
 * Adjoint of one periodic sweep along axis (0..2) of the fast scheme:
 * given the sweep's input U (conserved) and lam_out = dL/dU', writes
 * lam_in = dL/dU.  A step's adjoint is axis 2, 1, 0 in turn, each with the
 * input state of that forward sweep.  No reference counterpart (the
 * reference relies on JAX autodiff of fluid.py). */
int tf_adjoint_sweep(const float *U, const float *lam_out, float *lam_in, int nx, int ny, int nz,
                     float dx, float dt, float gamma, int axis, void *stream);
int tf_adjoint_sweep_f64(const double *U, const double *lam_out, double *lam_in, int nx, int ny,
                         int nz, double dx, double dt, double gamma, int axis, void *stream);

/* FP64 forward sweep of the same scheme on conserved states (for the
 * finite-difference check of the adjoint). */
int tf_sweep_conserved_f64(const double *U, double *out, int nx, int ny, int nz, double dx,
                           double dt, double gamma, int axis, void *stream);

/* Largest grid (nx*ny*nz cells) tf_time_integration_noalloc accepts. */
#define TF_NOALLOC_MAX_CELLS (1 << 18)

/* The run loop of tf_time_integration for callers that cannot allocate device
 * memory (a host runtime that owns the device heap, allocator-free callbacks,
 * memory reserved up front): the work state and control block come from a
 * fixed scratch array compiled into the library (about 5 MiB per GPU that
 * loads it, held until exit), so the caller passes only W_in and W_out, and
 * nothing is allocated.  Grids above TF_NOALLOC_MAX_CELLS cells are rejected
 * with TF_ERR_ARG, and so are states whose bytes overlap each other or the
 * scratch.  The run uses tf_time_integration's built-in tile choice.  The
 * first call on a device looks up the scratch's device address and caches it
 * for the life of the process; make that first call before any stream
 * capture, and do not use the entry point across a cudaDeviceReset (which
 * invalidates the address).  All calls share the one scratch array, which
 * keeps the previous call's contents (each call re-initialises the control
 * block it uses): calls that may overlap on the GPU (other streams, other
 * threads) race and must be serialised by the caller.
 * Errors found on the device (TF_ERR_NONFINITE, TF_ERR_TIMEOUT): a t_final run
 * (max_steps < 0) checks the loop on the host and always reports them; a run
 * of a known step count is asynchronous and reports them only when iters_host
 * is non-NULL (the call then waits for the run).  No counterpart in the
 * reference (it has no allocation control). */
int tf_time_integration_noalloc(const float *W_in, float *W_out, int nx, int ny, int nz,
                                float dx, float t_final, float gamma, float cfl, int max_steps,
                                float fixed_dt, unsigned flags, int *iters_host, void *stream);

/* ---- batches: many independent instances, each with its own dt ---- */

/* One instance of a batch (host struct; all pointers are device memory).  The
 * loop per instance is time_integration.py:63-92 with the CFL dt of
 * fluid.py:427-504 (or fixed_dt > 0), bounded by t_final and/or max_steps. */
typedef struct tf_instance {
  const float *W_in; /* initial primitive state [5][nx][ny][nz] */
  float *W_out;      /* final state */
  float *work;       /* scratch state, same size; may equal W_in (W_in is then overwritten) */
  tf_ctl *ctl;       /* this instance's control block (t, dt, iter, status) */
  int nx, ny, nz;
  unsigned flags;    /* TF_FLAG_OPEN_BOUNDARIES */
  float dx, gamma, cfl;
  float t_final;     /* +inf when only max_steps bounds the loop */
  float fixed_dt;    /* > 0: fixed dt instead of the CFL dt */
  int max_steps;     /* < 0: unbounded (t_final must be finite) */
  int lx;            /* x planes per tile, 0 = default */
  int reserved;
} tf_instance;

typedef struct tf_batch_config {
  int rows;          /* grid rows per tile: 8, 16 or 32 (see tf_tile_config) */
  int exact;         /* nonzero: reference op order */
  int persistent;    /* nonzero: one persistent launch for all steps; else one launch per step */
  int ctas_per_sm;   /* persistent grid = ctas_per_sm * SMs (0 = occupancy limit) */
  unsigned long long wait_limit; /* bounded spin before TF_ERR_TIMEOUT (0 = default) */
} tf_batch_config;

/* Device workspace bytes for a batch of `count` instances (256-byte aligned). */
unsigned long long tf_batch_workspace_bytes(int count);

/* Validates the instances, builds the tile tables and uploads them to the
 * workspace (synchronises `stream` once).  No reference counterpart: the
 * reference advances one state per call (time_integration.py:94-128). */
int tf_batch_prepare(const tf_instance *inst, int count, const tf_batch_config *cfg,
                     void *workspace, unsigned long long workspace_bytes, void *stream);

/* Enqueues `steps` step slots of a prepared batch, starting at step_base
 * (0: also initialises every ctl and computes the first dt).  Asynchronous
 * and capturable in a CUDA graph.  Each instance's result is in its W_out and
 * its t/iter/status in its ctl. */
int tf_batch_run(void *workspace, int step_base, int steps, void *stream);

/* Batch-level device error (TF_ERR_TIMEOUT if a bounded wait gave up); syncs. */
int tf_batch_error(void *workspace, int *error_host, void *stream);

/* Forgets the host-side plan of a workspace. */
int tf_batch_release(void *workspace);

/* ---- initial states, built on the device (W: 5*n^3 floats, n^3 grid,
 * 1 <= n <= 65535; computed in float32) ---- */

/* scaling_jax.py:23-41 setup_ics(n, k): rho = 0.125, p = 0.1, u = 0; rho = p = 1
 * on [n/2-k, n/2+k)^3.  The caller uses dx = 1/(n-1) like the reference. */
int tf_ics_injection_cube(float *W, int n, int num_injection_cells, void *stream);

/* Spherical overpressure on the unit periodic cube (cell centres (i+0.5)/n):
 * p = p_in for r < radius around the centre else p_out, u = 0,
 * rho = rho0*(1 + noise*U(-1,1)) from a counter-based hash of seed.  No
 * reference counterpart (benchmark initial state). */
int tf_ics_overpressure(float *W, int n, unsigned long long seed, double radius, double p_in,
                        double p_out, double rho0, double noise, void *stream);

/* Shear layer: rho=2, vx=+0.5 for |y-0.5|<0.25, else rho=1, vx=-0.5; p=2.5;
 * vy = amplitude*sin(4 pi x)*a with a ~ N(0,1) per cell (seeded hash); vz=0.
 * No reference counterpart (benchmark initial state). */
int tf_ics_shear_layer(float *W, int n, unsigned long long seed, double amplitude, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* TINYFLUIDS_GB300_H */
