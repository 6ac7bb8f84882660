/*
 * augur_field2d.h — C ABI of the reference's production 2D scatter-field model around the
 * isolated 2D PM plan: ScatterField(net="unet", potential=True, kernel=True, pp>0,
 * verlet=True) (scripts/scatter_field.py:28-67, 221-261, 551-688).
 *
 * One force evaluation (ScatterField._force / _grid_force, :591-666) is:
 *   augur_field2d_scatter                 x[0:3] = [m, m vx, m vy] * in_scale / h^2
 *   augur_pm_set_kernel_mlp + augur_pm_poisson(x[0])   kernel acceleration (kernel_acc)
 *   augur_field2d_inputs                  x[3:5] = kernel acceleration, x[5:] = previous field
 *   augur_unet2d_forward                  field = UNet(x)
 *   augur_field2d_accel                   grid acceleration -grad(field[0]) + kernel acceleration
 *   augur_pm_gather + augur_pm_pair_acc   at the bodies, plus the pair term
 *   augur_field2d_finish                  momentum fix and mask
 * and augur_field2d_drift / augur_field2d_kick are the velocity-Verlet halves of _step.
 *
 * Layouts: grids channels-first (C, G, G) float32 per scene (torch NCHW with B = 1), x the
 * fastest axis; force grids float4 (a_x, a_y, 0, phi) per cell; bodies (N, 2) float32.
 * All calls are asynchronous on `stream` and return 0 or a negative AUGUR_E* status
 * (include/augur_pm.h). fp32 throughout, as the reference's default (non-autocast) path.
 */
#ifndef AUGUR_FIELD2D_H
#define AUGUR_FIELD2D_H

#include <stddef.h>
#include <stdint.h>

#include "augur_pm.h"

#ifdef __cplusplus
extern "C" {
#endif

/*
 * Three-channel CIC scatter, ScatterField.scatter (:237-250): out3 (3, G, G) receives
 * [m*mask, m*mask*vx, m*mask*vy] * in_scale / h^2 with the fp32 corner weights of _corners
 * (:179-182); corners off the grid [-extent/2, extent/2)^2 are dropped (:208). Deterministic:
 * every corner contribution is rounded to a per-channel fixed point (2^-e, e chosen from the
 * largest |value| so that N of them fit in 61 bits) and summed with integer atomics.
 * work: augur_field2d_scatter_work_bytes(grid) bytes of device memory, 8-byte aligned.
 */
size_t augur_field2d_scatter_work_bytes(int grid);
int augur_field2d_scatter(const float *pos, const float *vel, const float *mass, const float *mask,
                          int64_t n, int grid, double extent, double in_scale, float *out3,
                          void *work, void *stream);

/* x[3], x[4] = lanes a_x, a_y of force4 (G*G float4); x[5 .. 5+cf) = field (cf, G, G), or 0 if NULL. */
int augur_field2d_inputs(const float *force4, const float *field, int cf, int grid, float *x,
                         void *stream);

/*
 * The reference's UNet (:28-67): inp = Conv(cin, width); enc[0..levels] = (Conv, GELU, Conv,
 * GELU) at resolutions grid / 2^l, each after avg_pool2d(2) of the previous one; dec[l] for l =
 * levels-1 .. 0 = the same block on cat(nearest-upsampled h, enc output l) (2 width channels);
 * out = Conv(width, cout), no activation. 3x3 convolutions, zero padding 1, exact (erf) GELU.
 * params: fp32 device array in torch's parameter order (inp.weight, inp.bias, enc.0.0.weight,
 * enc.0.0.bias, enc.0.2.weight, enc.0.2.bias, ..., dec.*, out.weight, out.bias), each conv weight
 * (out, in, 3, 3); augur_unet2d_param_count gives its length. augur_unet2d_prepare rewrites it
 * once into the kernels' layout (per convolution [in][tap][32 outputs, zero-padded] then 32
 * biases; augur_unet2d_prepared_count floats, 16-byte aligned), which augur_unet2d_forward reads.
 * x (batch, cin, G, G) -> y (batch, cout, G, G): the batch's scenes run in the same launches
 * (grid z = scene). Needs cin <= 64, width <= 32, cout <= 32, batch <= 65535 and grid divisible
 * by 2^levels; work: augur_unet2d_work_bytes(grid, width, levels, batch) bytes.
 */
int64_t augur_unet2d_param_count(int cin, int cout, int width, int levels);
int64_t augur_unet2d_prepared_count(int cin, int cout, int width, int levels);
int augur_unet2d_prepare(const float *params, int cin, int cout, int width, int levels,
                         float *prepared, void *stream);
size_t augur_unet2d_work_bytes(int grid, int width, int levels, int batch);
int augur_unet2d_forward(const float *prepared, int cin, int cout, int width, int levels, int grid,
                         int batch, const float *x, float *y, void *work, size_t work_bytes,
                         void *stream);

/*
 * force4_out (G*G float4, 16-byte aligned) = (-d phi/dx + k_x, -d phi/dy + k_y, 0, 0) with
 * central differences over 2h and zero padding (ScatterField.neg_grad, :551-555); k = lanes
 * a_x, a_y of force4_kernel (the kernel acceleration), or 0 if NULL.
 */
int augur_field2d_accel(const float *phi, const float *force4_kernel, int grid, double h,
                        float *force4_out, void *stream);

/*
 * acc_out = (acc_grid + acc_pair - momfix * sum(m mask a) / max(sum(m mask), 1e-9)) * mask
 * (:608-615); acc_pair may be NULL. The sums are FP64 in a fixed order.
 * work: augur_field2d_finish_work_bytes() bytes (8-byte aligned) when momfix is set.
 */
size_t augur_field2d_finish_work_bytes(void);
int augur_field2d_finish(const float *acc_grid, const float *acc_pair, const float *mass,
                         const float *mask, int64_t n, int momfix, float *acc_out, void *work,
                         void *stream);

/*
 * Velocity Verlet (ScatterField._step, :677-688):
 *   drift: pos_out = pos + dt vel + (dt^2/2) acc,  vel_pred = vel + dt acc
 *   kick:  dv = (dt/2) (acc0 + acc1),  vel_out = vel + dv  (dv_out may be NULL)
 */
int augur_field2d_drift(const float *pos, const float *vel, const float *acc, int64_t n, double dt,
                        float *pos_out, float *vel_pred, void *stream);
int augur_field2d_kick(const float *vel, const float *acc0, const float *acc1, int64_t n, double dt,
                       float *vel_out, float *dv_out, void *stream);

/*
 * Chunked large-N tick of the 2D model (Sim, scripts/scatter_bh_1b.py:107-146): unit-mass
 * bodies whose state (pos, momentum; (N, 2) each) is stored as fp32, fp16 or bf16 and widened
 * per body, with the relativistic speed v = p ms / sqrt(1 + |p ms|^2 / c^2)
 * (scripts/scatter_bh.py:22-23); drift = (pos + dt v) rounded to the position type. One tick is
 *   augur_tick2d_drift_scatter(drift = 1)  out3 = scatter of [1, vx, vy] * in_scale / h^2 at the
 *                                          drifted positions (the state is not written)
 *   grid force as above (kernel acceleration, U-Net on [out3, kernel acc, field], -grad + kernel)
 *   augur_tick2d_mean_acc                  abar = sum_cells acc * rho * h^2 / in_scale / N (FP64)
 *   augur_tick2d_gather_kick(drift = 1, kick = dt)   stores the drifted pos (from the same,
 *                                          not yet kicked momentum), then mom += kick (gather(acc,
 *                                          pos) - abar) / ms
 * and init_kick is the same with drift = 0 and kick = dt/2; augur_tick2d_drift stores the drift
 * alone. The scatter is deterministic: contributions are rounded to a fixed point bounded by
 * |v| < c and N, summed in int64 (one channel per CTA in shared memory for grid <= 160, then one
 * flush per CTA). fp32 arithmetic follows torch's operation order without contractions.
 * Non-finite state (NaN or infinite positions or momenta) is outside the tick's contract: no
 * error is reported, and such a body's fixed-point contribution is undefined (where the
 * reference's float grid would turn NaN). Callers that can produce non-finite state check it
 * themselves (for example with torch.isfinite on the state between ticks).
 * work: augur_tick2d_work_bytes(grid) bytes, 8-byte aligned.
 */
#define AUGUR_DTYPE_F32  0
#define AUGUR_DTYPE_F16  1
#define AUGUR_DTYPE_BF16 2
size_t augur_tick2d_work_bytes(int grid);
int augur_tick2d_drift_scatter(const void *pos, const void *mom, int64_t n, int pos_type,
                               int mom_type, double mom_scale, double c, double dt, int drift,
                               int grid, double extent, double in_scale, float *out3, void *work,
                               void *stream);
int augur_tick2d_drift(void *pos, const void *mom, int64_t n, int pos_type, int mom_type,
                       double mom_scale, double c, double dt, void *stream);
int augur_tick2d_mean_acc(const float *force4, const float *rho, int grid, double cell_mass,
                          int64_t n, float *abar, void *work, void *stream);
int augur_tick2d_gather_kick(const float *force4, void *pos, void *mom, int64_t n, int pos_type,
                             int mom_type, double mom_scale, double kick_dt, const float *abar,
                             int grid, double extent, int drift, double c, double dt,
                             void *stream);

#ifdef __cplusplus
}
#endif

#endif
