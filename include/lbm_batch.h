/* Batched lattices: many independent D2Q9 channel domains advanced together.
 *
 * No counterpart in the reference (lbm-wgpu drives one lattice per `Lbm`
 * object, lbm.rs).  Each domain behaves exactly like an lbm_sim created with
 * LBM_EDGE_CHANNEL and the same storage: frozen equilibrium inlet at its own
 * u_in on column 0, zero-gradient outflow, periodic top/bottom, half-way
 * bounce-back from its own mask, its own omega.
 * One lbm_batch_step advances every domain by one step in ONE persistent
 * kernel launch over a table of (domain, 256-column strip, row band) tiles;
 * runs of 20 steps are replayed from a CUDA graph captured on first use.
 * Results are bit-identical to advancing each domain through lbm_sim.
 *
 * Storage: LBM_STORE_F32, LBM_STORE_F16, LBM_STORE_BF16.  Every call is
 * ordered on the batch's own stream; reads synchronise it.  Status codes and
 * lbm_last_error() as in lbm.h. */
#ifndef LBM_GB300_BATCH_H
#define LBM_GB300_BATCH_H

#include <stddef.h>
#include <stdint.h>

#include "lbm.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct lbm_batch lbm_batch;

/* count domains; domain d is nx[d] x ny[d] (3..65535 rows, nx*ny < 2^28) with
 * relaxation omega[d] in (0, 2) and inlet velocity u_in[d].  All domains start
 * at equilibrium rho = 1, ux = u_in[d], uy = 0, no solids. */
int lbm_batch_create(uint32_t count, const uint32_t* nx, const uint32_t* ny, const float* omega, const float* u_in,
                     int storage, lbm_batch** out);
int lbm_batch_destroy(lbm_batch* batch);

/* Number of domains, total cells, steps since the last initialisation. */
int lbm_batch_info(const lbm_batch* batch, uint32_t* count, uint64_t* cells, uint64_t* steps);

/* The batch's own CUDA stream (cudaStream_t as void*), for callers that
 * order or time their work against it. */
int lbm_batch_get_stream(const lbm_batch* batch, void** stream);

/* Replace domain d's solid mask: nx*ny bytes, row-major, nonzero = solid. */
int lbm_batch_set_mask(lbm_batch* batch, uint32_t domain, const uint8_t* mask);

/* Every domain to equilibrium at rho = 1, ux = u_in[d], uy = 0 with seeded
 * uniform noise of amplitude noise_amp on ux and uy (seed + d for domain d,
 * the generator of lbm_init_equilibrium); step count back to 0. */
int lbm_batch_init_equilibrium(lbm_batch* batch, float noise_amp, uint64_t seed);

/* Advance every domain n steps (asynchronous). */
int lbm_batch_step(lbm_batch* batch, uint32_t n);

/* Wait for the batch's stream; LBM_ERR_STATE as lbm_synchronize. */
int lbm_batch_synchronize(lbm_batch* batch);

/* Domain d's LBM_FIELD_* (nx*ny floats) / populations (9 planes, reference
 * direction order, f32). */
int lbm_batch_read_field(lbm_batch* batch, uint32_t domain, int field, float* out);
int lbm_batch_read_populations(lbm_batch* batch, uint32_t domain, float* out);

/* FP64 sums over each domain's fluid cells of the last step's density and
 * momenta (as lbm_conservation per lattice): out[3 d .. 3 d + 2] = (mass,
 * x momentum, y momentum) of domain d, 3 * count doubles; synchronises.
 * Domains sharded across ranks add these up with one all-reduce; nothing
 * else crosses between ranks. */
int lbm_batch_conservation(lbm_batch* batch, double* out);

/* Rounding of the stored words (lbm_set_rounding): LBM_ROUND_NEAREST (the
 * default) or, for f16 / bf16 batches, LBM_ROUND_STOCHASTIC.  Domain d then
 * rounds exactly as a single lattice of its size with seed `seed + d`; the
 * step index is the batch's.  LBM_ERR_ARG for stochastic rounding of an
 * f32 batch. */
int lbm_batch_set_rounding(lbm_batch* batch, int mode, uint32_t seed);
int lbm_batch_get_rounding(const lbm_batch* batch, int* mode, uint32_t* seed);

/* Fix the schedule by hand: variant 0..5 = (ring stages, cells per thread,
 * strip columns) (5,1,256) (6,1,256) (5,2,256) (8,2,256) (6,2,512)
 * (4,2,512), the 512-column strips for f16 / bf16 only (f32 runs variants 4
 * and 5 with 256-column strips); dynamic 0 = tiles sorted longest first and dealt
 * round-robin to the persistent CTAs, 1 = CTAs take tiles from an atomic
 * counter, 2 = dealt as 0 with each CTA's tiles run through one bulk-copy
 * ring (the next tile's first rows are staged while the current one ends);
 * rows_per_bucket[3] = target band height for domains of height
 * <= 128, <= 256 and taller (NULL keeps the current ones). */
int lbm_batch_set_schedule(lbm_batch* batch, int variant, int dynamic, const int* rows_per_bucket);

/* Time the candidate schedules on this batch (each for steps_per_trial steps
 * after a warm-up; the state advances meanwhile) and keep the fastest.  The
 * trials and the choice are written as JSON into report (report_len bytes,
 * truncated; may be NULL). */
int lbm_batch_autotune(lbm_batch* batch, uint32_t steps_per_trial, char* report, size_t report_len);

#ifdef __cplusplus
}
#endif

#endif /* LBM_GB300_BATCH_H */
