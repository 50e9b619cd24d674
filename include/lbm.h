/*
 * lbm.h -- C ABI of the GB300 D2Q9 lattice-Boltzmann engine (liblbm_gb300.so).
 *
 * Drop-in for the step path of the lbm-wgpu crate (PPLUSCHT/LBM): construct a
 * grid, set and clear barrier cells, set inlet velocity and viscosity, step N
 * times, read back rho / ux / uy / curl.  Every entry point below names the
 * reference interface it replaces (paths relative to the reference tree).
 *
 * Conventions
 *   - Every function returns an int status: LBM_OK (0) or an LBM_ERR_* code;
 *     lbm_last_error() returns a thread-local message for the last failure.
 *   - The caller owns every host array passed in or out; the library owns all
 *     device memory of a simulation.  Host arrays are row-major, x fastest,
 *     index = x + y * nx, row 0 first (the reference's index(), lbm.rs:1517).
 *   - A handle is used by one host thread at a time.  Work is queued on the
 *     handle's CUDA stream; functions that return data to the host
 *     synchronise that stream, lbm_step does not (use lbm_synchronize).
 *   - Population order is the reference's (set_equil, lbm.rs:632-640):
 *     0 nw, 1 n, 2 ne, 3 w, 4 rest, 5 e, 6 sw, 7 s, 8 se; north is row - 1.
 */
#ifndef LBM_GB300_H
#define LBM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct lbm_sim lbm_sim;

/* status codes */
#define LBM_OK 0
#define LBM_ERR_ARG 1      /* invalid argument */
#define LBM_ERR_CUDA 2     /* CUDA runtime error (message has the CUDA error) */
#define LBM_ERR_NOMEM 3    /* device or host allocation failed */
#define LBM_ERR_STATE 4    /* non-finite density detected by the step kernel */

/* edge modes */
#define LBM_EDGE_REF 0     /* the reference: walls on rows 0 and ny-1, column 0 and
                              the last row never streamed, linear-index neighbours */
#define LBM_EDGE_CHANNEL 1 /* column 0 frozen equilibrium inlet at (1, u_in, 0),
                              zero-gradient outflow at column nx-1, periodic top/bottom */

/* population storage */
#define LBM_STORE_F32 0
/* The 16-bit modes store the deviation of each population from the rest
 * weights, f_i - w_i, and collide in f32 arithmetic; with
 * lbm_set_storage_reference(sim, 1) the deviation from the equilibrium of
 * the lattice's inlet velocity instead, f_i - f_i^eq(1, (u_in, 0)). */
#define LBM_STORE_F16 1    /* binary16 deviations, f32 arithmetic */
#define LBM_STORE_BF16 2   /* bfloat16 deviations, f32 arithmetic */
#define LBM_STORE_F64 3    /* f64 storage and arithmetic (oracle-grade runs) */

/* readback fields (lbm_read_field) */
#define LBM_FIELD_RHO 0        /* density */
#define LBM_FIELD_JX 1         /* x momentum: the reference's "ux" summary (ux.wgsl:41) */
#define LBM_FIELD_JY 2         /* y momentum (north positive): the reference's "uy" (uy.wgsl:41) */
#define LBM_FIELD_UX 3         /* velocity jx / rho */
#define LBM_FIELD_UY 4         /* velocity jy / rho */
#define LBM_FIELD_CURL 5       /* curl.wgsl:49 on momenta, 10*(...)/rho; 0 in column 0
                                  and the last row */
#define LBM_FIELD_VORTICITY 6  /* central-difference dx(uy) - dy(ux) of velocities */
#define LBM_FIELD_SPEED 7      /* |u| */

/* Message of the last failed call on this thread ("" if none). */
const char* lbm_last_error(void);

/* Library version string. */
const char* lbm_version(void);

/* LBM::new (lbm-wgpu/src/lbm.rs:726): allocate an nx x ny grid on the
 * current CUDA device with relaxation rate omega, barrier = init_barrier
 * (lbm.rs:595-605) in LBM_EDGE_REF (no walls in LBM_EDGE_CHANNEL), state =
 * set_equil(0.1, 0, 1) (lbm.rs:740).  nx, ny >= 3; ny <= 65535; the padded grid
 * (nx rounded up to 32, times ny) below 2^29 cells. */
int lbm_create(uint32_t nx, uint32_t ny, float omega, int edge_mode, int storage, lbm_sim** out);

/* Drop of LBM: free all device memory of the handle. */
int lbm_destroy(lbm_sim* sim);

/* Dimensions and mode of a handle (any pointer may be NULL). */
int lbm_get_info(const lbm_sim* sim, uint32_t* nx, uint32_t* ny, int* edge_mode, int* storage);

/* Queue the handle's work on a CUDA stream (a cudaStream_t passed as void*;
 * NULL is CUDA's legacy default stream).  A new handle uses its own
 * non-blocking stream, which lbm_get_stream returns.  The new stream waits,
 * on the device, for the work already queued on the previous one (unless
 * either is being captured into a graph: the caller orders them then), so
 * the previous stream must still exist when the handle leaves it. */
int lbm_set_stream(lbm_sim* sim, void* cuda_stream);
int lbm_get_stream(const lbm_sim* sim, void** cuda_stream);

/* Step kernel variant and launch shape; every variant gives identical
 * results.  kernel 0: one cell per thread, rows_per_thread rows each;
 * 1: the same with the next row's loads issued before the current row's
 * collision; 2, 3, 4, 5: row segments staged in shared memory by the
 * bulk-copy engine with a ring of 5, 4, 6, 8 stages, a producer warp and 8
 * consumer warps per 256-column strip (rows_per_thread is then the minimum
 * band height); 6, 7, 8: the same with rings of 8, 6, 4 stages and two cells
 * per consumer thread (channel mode; reference mode runs one); 9, 10: rings
 * of 4, 6 stages and four cells per consumer thread, 2 consumer warps per
 * strip (channel mode with f16 / bf16 storage; otherwise as 8); 11, 12, 13:
 * rings of 5, 6, 7 stages, two cells per thread and 512-column strips
 * (channel mode with f16 / bf16 storage; otherwise as 7).  Defaults: 3
 * for f32, 11 for f16 / bf16 (7 below 1024 columns), with rows_per_thread 8 for kernels 0 / 1 and a
 * band floor of 2 rows for the staged kernels; f64 storage always uses
 * kernel 0.  No counterpart in the reference, whose dispatch is fixed at
 * 256-wide 1-D workgroups (lbm.rs:102-106). */
int lbm_set_tuning(lbm_sim* sim, int rows_per_thread, int kernel);

/* draw_shape / draw_barrier_updates (lbm.rs:1337-1356, barrier_draw.wgsl:13-17):
 * npairs (location, value) pairs; value 1 sets a solid cell, any other value
 * clears it; locations >= nx*ny clamp to the last cell (the shader's clamped
 * store).  Pairs apply in order: the last pair for a cell wins. */
int lbm_set_barrier(lbm_sim* sim, const uint32_t* idx_val_pairs, size_t npairs);

/* reset_barrier (lbm.rs:1362-1365): the two wall rows in LBM_EDGE_REF, all
 * fluid in LBM_EDGE_CHANNEL. */
int lbm_reset_barrier(lbm_sim* sim);

/* Whole-mask upload / download: one byte per cell, nonzero = solid, dense
 * nx-wide rows (the reference uploads whole barrier buffers in reset_barrier,
 * lbm.rs:1364).  lbm_set_mask copies the bytes to the device and bit-packs
 * them there; it returns once `mask` has been read, with the packing queued on
 * the handle's stream. */
int lbm_set_mask(lbm_sim* sim, const uint8_t* mask);
int lbm_get_mask(lbm_sim* sim, uint8_t* mask);

/* update_omega_buffer (lbm.rs:1358-1360). */
int lbm_set_omega(lbm_sim* sim, float omega);

/* WASMInteraction::update_viscosity + lib.rs:181-186: omega = 1/(3 nu + 0.5). */
int lbm_set_viscosity(lbm_sim* sim, float nu);

/* custom_speed (lbm.rs:1090-1102) when reset_field != 0: the whole field is
 * re-initialised to set_equil(ux, 0, 1) and the step count restarts at 0.
 * With reset_field == 0 only the inlet changes: in LBM_EDGE_CHANNEL the frozen
 * inlet column, in LBM_EDGE_REF column 0 (its de-facto inlet).  In the 16-bit
 * modes with the inlet storage reference (lbm_set_storage_reference) the
 * inlet velocity is also the storage's reference state: a new one without a
 * reset re-expresses every stored word against it (one pass over both
 * buffer sets; its rounding is part of the state). */
int lbm_set_inlet_velocity(lbm_sim* sim, float ux, int reset_field);

/* 16-bit storage only (no reference counterpart: the reference stores f32).
 * inlet = 0 (the default) keeps the words relative to the rest weights w_q,
 * f_i - w_i; inlet = 1 keeps them relative to the inlet equilibrium, which
 * makes them small wherever the flow is near the inlet velocity (several
 * times less rounding error in a moving flow, a few per cent slower: one
 * fused operation more per direction, bounced words re-expressed for their
 * new direction).  Switching re-expresses the stored state; a no-op for
 * f32 / f64.  The setting travels with checkpoints. */
int lbm_set_storage_reference(lbm_sim* sim, int inlet);
int lbm_get_storage_reference(const lbm_sim* sim, int* inlet);

/* Rounding of the words each step stores (16-bit storage only; no reference
 * counterpart).  LBM_ROUND_NEAREST (the default) rounds to nearest even.
 * LBM_ROUND_STOCHASTIC rounds each word up or down with probabilities set by
 * its distance to the two neighbouring 16-bit values (the hardware's
 * cvt.rs conversions), so rounding adds no bias. Round-to-nearest gives a
 * steady flow the same error every step, and that error accumulates. The
 * random bits are a hash of (seed, step index, row + row origin, column
 * pair, direction): runs are deterministic, and graph replays, row-range
 * steps, checkpoints and kernel variants give identical states.
 * Initialisation, uploads and re-expression still round to nearest.
 * LBM_ERR_ARG for stochastic rounding with f32 / f64 storage.  The setting
 * travels with checkpoints.  The step index comes from a counter in device
 * memory that every step call advances in stream order, so graphs replay
 * with fresh indices: lbm_step's own and a caller's capture alike. */
#define LBM_ROUND_NEAREST 0
#define LBM_ROUND_STOCHASTIC 1
int lbm_set_rounding(lbm_sim* sim, int mode, uint32_t seed);
int lbm_get_rounding(const lbm_sim* sim, int* mode, uint32_t* seed);

/* Row origin of the stochastic-rounding hash: row y hashes as y + origin
 * (default 0).  A lattice that holds rows [y0, y1) of a larger one (a slab)
 * sets the origin so its rounding matches the undivided lattice.  Travels
 * with checkpoints. */
int lbm_set_row_origin(lbm_sim* sim, int32_t origin);
int lbm_get_row_origin(const lbm_sim* sim, int32_t* origin);

/* reset_to_equilibrium (lbm.rs:1076-1088): set_equil(0.1, 0, 1) everywhere. */
int lbm_reset_to_equilibrium(lbm_sim* sim);

/* set_equil (lbm.rs:611-643) per cell at (rho, ux + nx_i, uy + ny_i), where
 * nx_i, ny_i are seeded uniform noise in [-noise_amp, noise_amp) from a
 * splitmix64 hash of (seed, cell, component).  Step count restarts at 0. */
int lbm_init_equilibrium(lbm_sim* sim, float rho, float ux, float uy, float noise_amp, uint64_t seed);
/* The same with the caller's noise: set_equil per cell at (rho, ux +
 * noise[i], uy + noise[nx ny + i]), i = x + y nx, from 2 nx ny floats of
 * host memory (NULL: no noise).  Returns once `noise` has been read. */
int lbm_init_equilibrium_noise(lbm_sim* sim, float rho, float ux, float uy, const float* noise);

/* single_cell (lbm.rs:1482-1515): rest state with population `direction` set
 * to 4.0 at the reference's cell for that direction. */
int lbm_single_cell(lbm_sim* sim, int direction);

/* iterate (lbm.rs:1065-1068) without the draw: n fused collide+stream steps.
 * The density / momentum buffers hold the moments of the last step's
 * collision (the reference's density_bg after iterate). Asynchronous. */
int lbm_step(lbm_sim* sim, uint32_t n);

/* One step taken in row ranges, for a lattice split into y-slabs: a call
 * computes rows [y0, y1) of the next step (same results as lbm_step), and
 * the call with LBM_ROWS_COMPLETE in `flags` completes it (the step count and
 * buffer parity advance then).  A slab computes its edge rows first, starts
 * sending them, and overlaps that with its interior rows.  Until the step is
 * complete, lbm_rows_read / lbm_rows_write address the rows being written,
 * and only they, further lbm_step_rows calls, lbm_set_stream and
 * lbm_synchronize are accepted (others return LBM_ERR_STATE).  Rows that no
 * call of the step covers keep stale values.  LBM_ROWS_MOMENTS: these rows
 * also write their moments; read_field then reflects the step only if every
 * call of it asked for them.  Plain launches, no graphs.  No counterpart in
 * the reference (one lattice per adapter, driver.rs:14-40). */
#define LBM_ROWS_COMPLETE 1
#define LBM_ROWS_MOMENTS 2
int lbm_step_rows(lbm_sim* sim, uint32_t y0, uint32_t y1, int flags);

/* lbm_step replays CUDA graphs captured on first use: a call of 2 to 64
 * steps is captured whole and replayed by later calls of the same length;
 * longer calls replay runs of 16 steps (per buffer parity, recaptured when
 * omega, the step kernel, the launch shape, the stream or the closure
 * change).  On by default; results are the same either way.  Not on the
 * legacy default stream, which cannot be captured, nor while the caller is
 * capturing the lattice's stream.  enable = 0 turns it off and frees the
 * graphs.  Steps recorded in a caller's own capture are plain launches
 * that replay from the buffer parity they were recorded at: record an even
 * number of steps, from a state that has taken at least one step since its
 * last initialisation or edit (that step collides in place), and the
 * graph can be replayed any number of times.  The host-side step count
 * advances once, by the recorded steps, not per replay. */
int lbm_set_graphs(lbm_sim* sim, int enable);

/* Wait for queued work; returns LBM_ERR_STATE if a step saw a non-finite density. */
int lbm_synchronize(lbm_sim* sim);

/* set_summary + calculate_summary (lbm.rs:1051-1063) with a real readback:
 * nx*ny floats of LBM_FIELD_* into out. */
int lbm_read_field(lbm_sim* sim, int field, float* out);
/* The same into a DEVICE array of nx * ny floats, queued on the handle's
 * stream without synchronising (for on-device averaging of large grids).
 * No counterpart in the reference. */
int lbm_read_field_device(lbm_sim* sim, int field, float* device_out);

/* Current populations (the reference's set compute_step%2 plus the rest plane
 * "origin"): 9 * nx * ny values, plane-major, reference order. */
int lbm_read_populations(lbm_sim* sim, float* out);
int lbm_read_populations_f64(lbm_sim* sim, double* out);

/* The same f32 populations into a DEVICE array of 9 * nx * ny floats, queued
 * on the handle's stream without synchronising (for on-device consumers such
 * as the closure's training samples).  No counterpart in the reference. */
int lbm_read_populations_device(lbm_sim* sim, float* device_out);

/* Upload populations (9 planes, reference order) to both buffer sets, as
 * custom_speed / single_cell upload states (lbm.rs:1092-1095); the step
 * count restarts at 0.  Returns once `in` has been read (the caller may reuse
 * it); the conversion into the buffer sets is queued on the handle's stream. */
int lbm_write_populations(lbm_sim* sim, const float* in);
int lbm_write_populations_f64(lbm_sim* sim, const double* in);

/* get_compute_num (lbm.rs:1170-1172): steps since the last re-initialisation. */
int lbm_step_count(const lbm_sim* sim, uint64_t* out);

/* Kernels launched by this handle so far (instrumentation). */
int lbm_launch_count(const lbm_sim* sim, uint64_t* out);

/* Force on the solid cells (drag out[0] along +x, lift out[1] north
 * positive) by momentum exchange on the half-way bounce-back links of the last
 * collision: sum over streamed cells x and directions p with a solid
 * neighbour x + c_p of 2 f_p*(x) c_p, in f64.  LBM_ERR_STATE before the first
 * step.  No counterpart in the reference. */
int lbm_read_force(lbm_sim* sim, double out[2]);

/* FP64 sums over fluid cells of rho, jx, jy from the last step's moments
 * (global mass and momentum; no counterpart in the reference). */
int lbm_conservation(lbm_sim* sim, double out[3]);

/* The same FP64 fluid sums for callers that cannot allocate device memory
 * (an application that owns all device memory through its own pool, a
 * real-time loop that cannot afford cudaMalloc's implicit synchronisation):
 * no handle, no allocation.  No counterpart in the reference.
 *   rho, jx, jy: device arrays of f32 moments, row pitch `pitch` elements;
 *   solid: device array, one byte per cell (nonzero = excluded) with the
 *          same row pitch `pitch` (cell (x, y) at solid[y * pitch + x]), or
 *          NULL (every cell counts);
 *   out: device pointer to 3 doubles (sum rho, sum jx, sum jy);
 *   stream: cudaStream_t as void* (NULL = the legacy default stream).
 * Its scratch is a fixed 96 KiB array in the library's device image (present
 * on every GPU that loads the library until exit), which limits ny * pitch to
 * 2^28 cells; larger inputs return LBM_ERR_ARG before any device work.  All
 * calls share that array, so calls that overlap on the GPU race: serialise
 * them.  The first call on a device resolves the array's address there; make
 * it before any stream capture.  The address is kept per CUDA context: after
 * cudaDeviceReset (or any other end of the device's context) the next call
 * resolves it again, and should again come before any capture.  Errors are
 * reported by lbm_last_error(). */
int lbm_conservation_noalloc(const float* rho, const float* jx, const float* jy, const uint8_t* solid, uint32_t nx,
                             uint32_t ny, uint32_t pitch, double* out, void* stream);

/* Halo rows for a lattice split into y-slabs across devices (no counterpart
 * in the reference, which runs one lattice on one adapter).  Copies rows
 * y .. y + nrows - 1 of the moving-population planes selected by slot_mask
 * (bit s = slot s: 0 nw, 1 n, 2 ne, 3 w, 4 e, 5 sw, 6 s, 7 se) of the state
 * the next step pulls from, in the storage's own words (4, 2 or 8 bytes;
 * 16-bit words are relative to the lattice's storage reference, so lattices
 * that exchange rows must share it and, with the inlet reference, the inlet
 * velocity),
 * planes in slot order, each nrows * nx words row-major.  on_device != 0:
 * `out` / `in` is device memory and the copy is queued on the lattice's
 * stream; otherwise host memory and the call synchronises. */
int lbm_rows_read(lbm_sim* sim, uint32_t y, uint32_t nrows, uint32_t slot_mask, void* out, int on_device);
int lbm_rows_write(lbm_sim* sim, uint32_t y, uint32_t nrows, uint32_t slot_mask, const void* in, int on_device);
/* Bytes per stored population (4 f32, 2 f16 / bf16, 8 f64). */
int lbm_storage_bytes(const lbm_sim* sim, uint32_t* bytes);

#ifdef __cplusplus
}
#endif

#endif /* LBM_GB300_H */
