/* Checkpoint and resume of a lattice.
 *
 * The reference keeps no checkpoints (its state lives in GPU buffers for the
 * life of the page, lbm.rs:32-98).  A checkpoint here holds the exact device
 * state, so that a lattice loaded from it continues bit for bit as the saved
 * one would have: both buffer sets and the rest plane in their storage words
 * (f32, f64, or the 16-bit words relative to the rest weights, or with
 * store_inlet = 1 to the equilibrium of the saved inlet velocity u_in), which
 * buffer is current and whether
 * it is materialised, the step count, omega, the inlet velocity, the solid
 * mask and, when the learned closure is on, its per-cell records.
 *
 * Layout (little-endian): a 96-byte header
 *   char magic[8] = "LBMGB3CK"; u32 version = 2, nx, ny; i32 edge, storage;
 *   f32 omega, u_in, drift; u64 steps; u32 cur, materialised, closure,
 *   elem_bytes; u64 payload_bytes; u32 crc32 (zlib's CRC-32 of the header
 *   with this field zero, continued over the payload); u32 store_inlet
 *   (lbm_set_storage_reference); u32 rounding, rounding_seed
 *   (lbm_set_rounding); i32 row_origin (lbm_set_row_origin); u32 reserved
 * then the payload, every plane dense row-major (nx * ny, row 0 first):
 *   mask (u8 per cell); buffer 0 (8 planes, direction slots 0..3 = nw, n, ne,
 *   w and 4..7 = e, sw, s, se); buffer 1 (8 planes); rest plane; closure
 *   records (2 x binary16 per cell) when closure != 0.
 * A checkpoint loads into a lattice of the same size, edge mode and storage. */
#ifndef LBM_GB300_CHECKPOINT_H
#define LBM_GB300_CHECKPOINT_H

#include <stddef.h>

#include "lbm.h"

#ifdef __cplusplus
extern "C" {
#endif

int lbm_checkpoint_size(const lbm_sim* sim, size_t* bytes);
/* Into a caller buffer of at least lbm_checkpoint_size bytes (synchronises). */
int lbm_checkpoint_save(lbm_sim* sim, void* buf, size_t len);
/* From a buffer; LBM_ERR_ARG, before any device work, on a size / mode
 * mismatch, a CRC error, or a header field out of range (cur, materialised
 * closure and store_inlet must be 0 or 1; rounding 0, or 1 with 16-bit
 * storage; omega in (0, 2); u_in finite; drift finite and > 0). */
int lbm_checkpoint_load(lbm_sim* sim, const void* buf, size_t len);

/* Host only (no device work, no lattice): check a checkpoint buffer as
 * lbm_checkpoint_load does before it touches a lattice (magic, version,
 * header ranges, a grid, edge mode, storage and element size the engine
 * knows, the payload size those imply, the CRC) and, when `info` is not
 * NULL, report what it holds.  LBM_ERR_ARG when any check fails. */
typedef struct lbm_checkpoint_info {
  uint32_t nx, ny;
  int edge, storage;
  float omega, u_in, drift;
  uint64_t steps;
  int closure, store_inlet;
  int rounding;            /* LBM_ROUND_NEAREST / LBM_ROUND_STOCHASTIC */
  uint32_t rounding_seed;
  int32_t row_origin;
} lbm_checkpoint_info;
int lbm_checkpoint_inspect(const void* buf, size_t len, lbm_checkpoint_info* info);
/* The same through a file. */
int lbm_checkpoint_write(lbm_sim* sim, const char* path);
int lbm_checkpoint_read(lbm_sim* sim, const char* path);

#ifdef __cplusplus
}
#endif

#endif /* LBM_GB300_CHECKPOINT_H */
