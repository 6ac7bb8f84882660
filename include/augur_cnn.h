/*
 * augur_cnn.h — C ABI of the scatter-field grid CNN (sm_103a).
 *
 * Network: the reference's LocalNet (scripts/scatter_field.py:15-26) in 3D — Conv3d 3x3x3,
 * zero padding 1, widths 2 -> 32 -> 32 -> 32 -> 32 -> 3, GELU (erf form), residual middle
 * layers, zero-initialised output layer (:135-136). Its input is the CIC density and PM
 * potential grids cast to BF16; its output, a 3-channel force correction, is added to the
 * PM force grid before the CIC gather (the role of the net output in
 * ScatterField._grid_force, :646-663).
 *
 * Layouts: activations channels-last BF16 (B, G, G, G, C); force grids float4 (a_x, a_y,
 * a_z, phi) per cell; weights fp32 w[n][tap][c] with tap = (dz*3 + dy)*3 + dx, which is
 * torch's Conv3d weight (n, c, dz, dy, dx) with the channel axis moved last.
 * All calls are asynchronous on `stream` and return 0 or a negative AUGUR_E* status.
 * Tensor-core waits are bounded: a stall sets bit 4 of *err (AUGUR_ETIMEDOUT on check).
 */
#ifndef AUGUR_CNN_H
#define AUGUR_CNN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/*
 * tcgen05 implicit-GEMM 3x3x3 convolution over 32 input channels (16 for layer 3).
 *   layer 0: 32 -> 32 forward, out0 = resid + gelu(conv + bias) (bf16), out1 = conv + bias (bf16, may be NULL)
 *   layer 1: 32 -> 3 output layer, out0 (float4 grid) lanes 0..2 += out_scale * (conv + bias)
 *   layer 2: data gradient of a 32 -> 32 layer: out0 = resid + conv^T (fp32; resid may be NULL),
 *            out1 = out0 * gelu'(zprev) (bf16)
 *   layer 3: data gradient of the output layer (in: 16-channel padded output gradient), as layer 2
 * w_umma: weights prepared by augur_cnn_prep_weights for that layer.
 * stats (layer 1 only, may be NULL): stats[0] += sum |correction|^2, stats[1] += sum |force|^2
 * of the grid before the correction, over all voxels (doubles; the fallback monitor's
 * correction-size check without another pass over the grid).
 * Replaces the nn.Conv3d calls of LocalNet.forward / autograd backward.
 */
int augur_cnn_conv_tc(int layer, const void *in, const void *w_umma, const float *bias, const void *resid,
                      const void *zprev, void *out0, void *out1, int batch, int grid, float out_scale,
                      unsigned *err, double *stats, void *stream);

/* Input layer 2 -> 32 on the CUDA cores: z0 = conv(x) + bias, h0 = gelu(z0), both bf16. */
int augur_cnn_conv_in(const void *x, const float *w, const float *bias, int batch, int grid, void *z0, void *h0,
                      void *stream);

/*
 * Input layer 2 -> 32 on tcgen05 (K = 54 padded to 64, A operand built in shared memory):
 * h0 = gelu(conv(x) + bias) bf16; z0 (may be NULL) = conv(x) + bias bf16. w_umma: a zeroed
 * 64 x 32 bf16 buffer filled by augur_cnn_prep_weights(w, 32, 2, 2, 32, 0, w_umma) (weights
 * rounded to bf16, unlike augur_cnn_conv_in's fp32 weights).
 */
int augur_cnn_conv_in_tc(const void *x, const void *w_umma, const float *bias, int batch, int grid, void *z0,
                         void *h0, unsigned *err, void *stream);

/*
 * Weight and bias gradients (fixed-order reduction of per-CTA partial sums; the reference's
 * autograd through nn.Conv3d, scripts/train_scatter_field.py:224-228):
 *   kind 0: 32 -> 32 layer on tcgen05, h (bf16, 32 ch) and dz (bf16, 32 ch)
 *   kind 1: output layer on the CUDA cores, h3 (bf16, 32 ch) and the output gradient as a float4
 *           grid (4 channels, the 4th must be zero)
 *   kind 2: input layer on the CUDA cores, x (bf16, 2 ch) and dz0 (bf16, 32 ch)
 *   kind 3: output layer on tcgen05, h3 (bf16, 32 ch) and the 16-channel bf16 output gradient
 *           written by augur_cnn_pack_dout (channels 3..15 zero)
 *   kind 4: kind 0 on the CUDA cores (the same sums in another order)
 * out receives N*27*CIN weight gradients in w[n][tap][c] order, then N bias gradients (N = 4 for
 * the output layer, whose 4th channel is zero). partial: scratch of max_parts * (N*27*CIN + N)
 * floats. err: error word of the tensor-core kinds (bit 4: a bounded wait ran out), may be NULL
 * for kinds 1, 2 and 4.
 */
int augur_cnn_wgrad(int kind, const void *h, const void *dz, int batch, int grid, float *partial, int max_parts,
                    float *out, unsigned *err, void *stream);

/*
 * Tries of every bounded pipeline wait in the tensor-core kernels launched after this call
 * (process-wide; the default is 2^20 = 1048576). Returns the previous value, so a caller can
 * restore it. A kernel whose wait runs out leaves its loops, waits (with a fixed bound) for its
 * own copies and MMAs in flight, frees its TMEM and raises bit 4 of its error word; with 0 tries
 * every pipeline wait gives up at once, which exercises that path. No counterpart in the reference.
 */
unsigned augur_cnn_set_wait_budget(unsigned tries);

/*
 * fp32 w[n][tap][c] (n < n_out, c < c_in) -> bf16 tensor-core operand with cin_pad
 * reduction channels and n_pad output channels; flip = 1 builds the data-gradient operand
 * (taps mirrored, input and output channels exchanged). cin_pad >= 16: the layout of
 * augur_cnn_conv_tc (per dx, K = (dz, channel), N = (dy, output channel)); cin_pad = 2: the
 * input layer's (K = (tap, channel) padded to 64, into a zeroed 64 x n_pad buffer).
 */
int augur_cnn_prep_weights(const float *w, int n_out, int c_in, int cin_pad, int n_pad, int flip, void *out,
                           void *stream);

/* x (nvox, 2) bf16 = (log(1 + rho_scale * rho), phi_scale * force4.w). */
int augur_cnn_input(const float *rho, const float *force4, int64_t nvox, float rho_scale, float phi_scale, void *x,
                    void *stream);

/* AdamW step on a flat fp32 parameter vector (torch.optim.AdamW semantics). */
int augur_cnn_adamw(float *p, const float *g, float *m, float *v, int n, float lr, float b1, float b2, float eps,
                    float wd, int step, void *stream);

/* field4 lanes 0..2 += CIC scatter of grad (n, 3) at pos (n, 3): the transpose of the gather. */
int augur_cnn_gather_transpose(const float *pos, const float *grad, int64_t n, int grid, double extent,
                               float *field4, void *stream);

/* (nvox) float4 lanes 0..2 -> (nvox, 16) bf16 scaled, channels 3..15 zero. */
int augur_cnn_pack_dout(const float *field4, int64_t nvox, float scale, void *out16, void *stream);

/* dz = dh * gelu'(z) elementwise (n values; dh fp32, z and dz bf16). */
int augur_cnn_gelu_bwd(const float *dh, const void *z, int64_t n, void *dz, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* AUGUR_CNN_H */
