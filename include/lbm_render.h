/* Headless readout of a lattice: the reference's summary statistics, colour
 * maps and frame, without any graphics API.
 *
 * The reference computes a summary statistic per cell (summary_stats/*.wgsl,
 * selected by SummaryStat, lbm.rs:10-16), maps it to a colour
 * (color_map/*.wgsl, ColorMap, lbm.rs:20-24; solid cells black) and draws one
 * quad per cell into the window's swapchain (render.wgsl, vertex buffer
 * lbm.rs:108-114, draw lbm.rs:1140-1160).  Here the same values are produced
 * on the device from the lattice's moments: the frame is a plain buffer of
 * width x height pixels, pixel (px, py) showing cell
 * (floor((px + 1/2) nx / width), floor((py + 1/2) ny / height)), row 0 at the
 * top.  The frame is what the fragment shader outputs (linear RGB in [0, 1]);
 * the RGBA8 variant optionally applies the sRGB transfer function, as an sRGB
 * swapchain format would (the reference takes whatever format the platform
 * lists first).
 *
 * Curl of cells the reference's pass skips (column 0, the last row) is 0
 * here; the reference leaves whatever its output buffer held there. */
#ifndef LBM_GB300_RENDER_H
#define LBM_GB300_RENDER_H

#include <stdint.h>

#include "lbm.h"

/* SummaryStat */
#define LBM_STAT_CURL 0
#define LBM_STAT_UX 1  /* raw momentum jx (ux.wgsl) */
#define LBM_STAT_UY 2  /* raw momentum jy (uy.wgsl) */
#define LBM_STAT_RHO 3 /* 4 clamp(0.15 rho, 0, 1) - 0.5 (rho.wgsl) */
#define LBM_STAT_SPEED 4 /* clamp(5 |j|, 0, 1) - 0.5 (speed.wgsl) */

/* ColorMap */
#define LBM_CMAP_INFERNO 0
#define LBM_CMAP_VIRIDIS 1
#define LBM_CMAP_JET 2

#ifdef __cplusplus
extern "C" {
#endif

/* The statistic of every cell after the last step (nx * ny floats, host). */
int lbm_summary(lbm_sim* sim, int stat, float* out);

/* One frame into host memory: rgb (width * height * 3 floats) and / or rgba
 * (width * height * 4 bytes, sRGB-encoded when srgb != 0); either may be NULL. */
int lbm_render(lbm_sim* sim, int stat, int cmap, uint32_t width, uint32_t height, float* rgb, uint8_t* rgba,
               int srgb);

/* One frame into a DEVICE buffer of width * height * 3 floats, queued on the
 * lattice's stream without synchronising. */
int lbm_render_device(lbm_sim* sim, int stat, int cmap, uint32_t width, uint32_t height, float* rgb);

#ifdef __cplusplus
}
#endif

#endif /* LBM_GB300_RENDER_H */
