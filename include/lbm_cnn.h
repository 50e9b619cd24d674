/* Learned closure: training kernels of the per-cell relaxation-time network.
 *
 * No counterpart in the reference (lbm-wgpu relaxes every cell with one
 * uniform omega, lbm.rs:1358-1360).  A small CNN (3x3 convolutions,
 * 4 -> 32 -> 32 -> 32 -> 1, ReLU between) maps the coarse flow state to a
 * per-cell relaxation-time correction delta_tau = LBM_CNN_DT_MAX * sigmoid(z);
 * it is trained on coarse-grained trajectories of fine-grid runs of this
 * engine.  Every pointer below is DEVICE memory; work is queued on `stream`
 * (a cudaStream_t, NULL = legacy default stream) and nothing synchronises.
 * Status codes and lbm_last_error() as in lbm.h.
 *
 * Tensors are [N, C, H, W] f32, weights [Cout, Cin, 3, 3] with tap (ky, kx)
 * reading input (y + ky - 1, x + kx - 1), zero padding outside the image. */
#ifndef LBM_GB300_CNN_H
#define LBM_GB300_CNN_H

#include <stddef.h>
#include <stdint.h>

#include "lbm.h"

/* input feature scaling and the output range */
#define LBM_CNN_S_RHO 50.0f  /* feature 0 = (rho - 1) * S_RHO */
#define LBM_CNN_S_U 10.0f    /* features 1, 2 = ux * S_U, uy * S_U (uy positive north) */
#define LBM_CNN_DT_MAX 0.25f /* delta_tau = DT_MAX * sigmoid(z) */

#ifdef __cplusplus
extern "C" {
#endif

/* y = act(conv3x3(x) + bias); cin <= 32, cout 32 or 1; relu != 0 applies max(., 0). */
int lbm_cnn_conv_forward(const float* x, int n, int cin, int h, int w, const float* weight, const float* bias,
                         int cout, int relu, float* y, void* stream);

/* Input gradient of a layer with cin == 32: grad_in from the gradient w.r.t.
 * its output; `out` is the layer's ReLU output (gradient masked where out <= 0)
 * or NULL for a layer without ReLU. */
int lbm_cnn_conv_backward_data(const float* grad_out, const float* out, int n, int cin, int h, int w,
                               const float* weight, int cout, float* grad_in, void* stream);

/* Weight and bias gradients (overwritten, not accumulated), summed over the
 * batch in a fixed order; scratch of lbm_cnn_weight_scratch_bytes(cin, cout). */
int lbm_cnn_conv_backward_weight(const float* in, const float* grad_out, const float* out, int n, int cin, int h,
                                 int w, int cout, float* grad_weight, float* grad_bias, float* scratch,
                                 size_t scratch_bytes, void* stream);
size_t lbm_cnn_weight_scratch_bytes(int cin, int cout);

/* Closure loss of network outputs z [n, 1, h, w] against sample coefficients
 * coef [n, 3, h, w] (A, B, C per cell): the sum over cells of
 * A dt^2 - 2 B dt + C with dt = delta_tau(z), divided by norm, written as one
 * double to *loss_out; grad_z (may be NULL) receives its gradient.
 * scratch: 608 doubles. */
int lbm_cnn_closure_loss(const float* z, const float* coef, int n, int h, int w, float norm, float* grad_z,
                         double* scratch, double* loss_out, void* stream);

/* One Adam step (Kingma & Ba) on n parameters; t >= 1 is the step number. */
int lbm_cnn_adam(float* param, const float* grad, float* m, float* v, int n, int t, float lr, float beta1,
                 float beta2, float eps, void* stream);

/* Training sample of one snapshot of a fine run: pops [9, hf, wf] are its
 * populations (reference direction order), solid_fine [hf, wf] its mask.
 * For the coarse grid of (hf / factor) x (wf / factor) cells (Favre averages
 * over each block's fluid cells; a block is solid when fewer than half its
 * cells are fluid) it writes feat [4, H, W] (scaled rho - 1, Ux, Uy and the
 * solid flag), coef [3, H, W] and solid_coarse [H, W].  coef holds, per cell,
 * the eddy-viscosity fit of the subgrid stress tau_ij = <rho u_i u_j> / <rho>
 * - U_i U_j against the coarse strain rate S (central differences of U, y
 * periodic): the squared residual |tau^d + (2/3) dt S^d|^2 of the deviatoric
 * parts is A dt^2 - 2 B dt + C.  Zero where the cell is solid, on the first or
 * last column, or next to a solid.  scratch: 6 * H * W floats. */
int lbm_cnn_closure_sample(const float* pops, const uint8_t* solid_fine, int hf, int wf, int factor, float* feat,
                           float* coef, float* scratch, uint8_t* solid_coarse, void* stream);

/* ---- the closure on a lattice (LBM_EDGE_CHANNEL, f32 / f16 / bf16 storage) ----
 *
 * Network parameters: LBM_CNN_PARAMS floats packed layer by layer, each
 * layer's weights [cout][cin][3][3] followed by its biases; stored on the
 * device in BF16 (round to nearest even).  The inference evaluates the
 * network on the lattice's current moments in one fused kernel (all four
 * layers per 16 x 16 tile in shared memory, f32 accumulation) and stores per
 * cell (delta_tau, |u|) as two binary16 values.  While enabled, every step
 * relaxes a fluid cell with omega = 1 / (1 / omega_sim + delta_tau) as long
 * as its speed stays within drift * max(|u|_predicted, 0.01) of the predicted
 * one; a cell that drifts further (or has no prediction yet) takes the plain
 * BGK step, and is counted. */
#define LBM_CNN_PARAMS 19969

int lbm_closure_set_weights(lbm_sim* sim, const float* params, size_t n);
int lbm_closure_enable(lbm_sim* sim, float drift);
int lbm_closure_disable(lbm_sim* sim);
/* Predict from the moments of the last step (queued on the lattice's stream). */
int lbm_closure_infer(lbm_sim* sim);
/* Inference kernel: 0 (default) the tensor-core kernel (tcgen05.mma, BF16
 * operands, f32 accumulation in tensor memory), 1 the CUDA-core kernel (BF16
 * weights widened to f32).  Both evaluate the same network. */
int lbm_closure_set_inference(lbm_sim* sim, int kernel);
/* Current records as nx * ny floats each (either pointer may be NULL). */
int lbm_closure_read(lbm_sim* sim, float* dtau, float* speed);
/* Cell-steps that fell back to plain BGK since the last reset. */
int lbm_closure_fallback_count(lbm_sim* sim, uint64_t* out, int reset);

#ifdef __cplusplus
}
#endif

#endif /* LBM_GB300_CNN_H */
