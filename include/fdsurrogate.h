/* fdsurrogate.h - C ABI of the learned surrogate's CUDA kernels (libfdlbm.so).
 *
 * The reference has no learned component; nothing here replaces reference
 * code.  These are the training and inference kernels of a small convolutional
 * U-Net that advances (psi, u_x, u_y) by a fixed number of lattice steps given
 * the solid mask (the network is defined in fingering_dynamics_gb300/surrogate.py;
 * a float64 numpy restatement is the test oracle).
 *
 * Conventions: every pointer is device memory; activations are NHWC bfloat16
 * with the channel dimension innermost (P = N*H*W pixels); conv weights are
 * bfloat16 [Cout][3][3][Cin] ("same" zero padding, stride 1); channel counts
 * are multiples of 16; accumulation is FP32.  Calls are asynchronous on
 * `stream` and return FD_OK (0) or a negative fd_status (fdlbm.h), with the
 * message in fd_last_error().
 */
#ifndef FDSURROGATE_H
#define FDSURROGATE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum sg_act { SG_ACT_NONE = 0, SG_ACT_GELU = 1 };

/* z = conv3x3(x, w) + bias (bias may be NULL); y = act(z).  z may be NULL
 * (not stored); y may equal z when act == SG_ACT_NONE.  Implicit GEMM on the
 * tensor cores (M = P pixels, N = Cout, K = 9*Cin). */
int sg_conv3x3(const void* x, int N, int H, int W, int Cin, const void* w, const float* bias, int Cout, int act,
               void* z, void* y, void* stream);

/* sg_conv3x3 on the fifth-generation tensor cores (tcgen05.mma, operands in
 * shared memory through matrix descriptors, accumulator in tensor memory);
 * same arguments and results.  sg_tc_status reads (and optionally clears) its
 * device error word: bit 0 = an mbarrier wait gave up. */
int sg_conv3x3_tc(const void* x, int N, int H, int W, int Cin, const void* w, const float* bias, int Cout, int act,
                  void* z, void* y, void* stream);
int sg_tc_status(unsigned* out, int clear);

/* sg_conv3x3_tc fed by the tensor memory accelerator: one thread loads the
 * operands as tensor-map boxes (zero fill outside the image = the padding) into
 * a ring of stages and issues the MMAs as each lands.  Same arguments and
 * results; needs W a multiple of 128 and Cin, Cout multiples of 16
 * (FD_ERR_SHAPE otherwise).  Its waits share sg_tc_status's error word. */
int sg_conv3x3_tma(const void* x, int N, int H, int W, int Cin, const void* w, const float* bias, int Cout, int act,
                   void* z, void* y, void* stream);

/* sg_conv3x3_tma as a persistent kernel with warp-specialised roles: one
 * thread issues the boxes and MMAs of the CTA's tiles through one ring, two
 * accumulator buffers in tensor memory let four epilogue warps finish a tile
 * while the next one is multiplied.  Same arguments, results and shape rule. */
int sg_conv3x3_tma_ws(const void* x, int N, int H, int W, int Cin, const void* w, const float* bias, int Cout,
                      int act, void* z, void* y, void* stream);

/* wt[ci][ky][kx][co] = w[co][2-ky][2-kx][ci]: the weights of the data-gradient
 * convolution (dx = sg_conv3x3(dz, wt)). */
int sg_flip_weights(const void* w, int Cin, int Cout, void* wt, void* stream);

/* dw[co][ky][kx][ci] = sum_p dz[p][co] x[p + (ky-1, kx-1)][ci] (FP32 out,
 * overwritten), split over `splits` pixel ranges whose FP32 partial sums go
 * to `partial` (splits*Cout*9*Cin floats) and are added in a fixed order:
 * the result does not depend on scheduling.  splits <= 0 picks a split. */
int sg_conv3x3_wgrad(const void* x, const void* dz, int N, int H, int W, int Cin, int Cout, float* dw,
                     float* partial, size_t partial_floats, int splits, void* stream);

/* sg_conv3x3_wgrad on the fifth-generation tensor cores: D[co][ci] per tap
 * with K = pixels, both operands MN-major tensor-map boxes (dz and the x halo
 * of a kernel row), accumulators in tensor memory; the same FP32 partials
 * added in a fixed order.  Same arguments and result; needs W a multiple of
 * 128 and Cin, Cout multiples of 16 (FD_ERR_SHAPE otherwise); splits <= 0
 * picks the most CTAs that fill two waves of one per SM, within what
 * `partial` holds. */
int sg_conv3x3_wgrad_tc(const void* x, const void* dz, int N, int H, int W, int Cin, int Cout, float* dw,
                        float* partial, size_t partial_floats, int splits, void* stream);

/* Floats of `partial` that sg_conv3x3_wgrad and sg_conv3x3_wgrad_tc need with splits <= 0. */
size_t sg_wgrad_partial_floats(int N, int H, int W, int Cin, int Cout);

/* db[c] = sum_p dz[p][c] (FP32, fixed order; partial: sg_bias_partial_floats). */
int sg_bias_grad(const void* dz, size_t P, int C, float* db, float* partial, void* stream);
size_t sg_bias_partial_floats(int C);

/* dz = dy * GELU'(z) (tanh form), n elements. */
int sg_gelu_bwd(const void* dy, const void* z, size_t n, void* dz, void* stream);

/* 2x2 mean pooling of x (N,H,W,C) -> y (N,H/2,W/2,C) and its backward. */
int sg_pool2(const void* x, int N, int H, int W, int C, void* y, void* stream);
int sg_pool2_bwd(const void* dy, int N, int H, int W, int C, void* dx, void* stream);

/* Nearest 2x upsampling of x (N,h,w,C) into channels [coff, coff+C) of y
 * (N,2h,2w,Cy), and its backward (dx = sum of the 4 copies). */
int sg_up2(const void* x, int N, int h, int w, int C, void* y, int Cy, int coff, void* stream);
int sg_up2_bwd(const void* dy, int N, int h, int w, int Cy, int coff, int C, void* dx, void* stream);

/* dst[p][coff + c] = src[p][c] (c < Cs): a skip connection into a concatenation. */
int sg_copy_channels(const void* src, size_t P, int Cs, void* dst, int Cd, int coff, void* stream);

/* dst[p][c] += src[p][coff + c] (c < C): the skip connection's gradient. */
int sg_add_channels(const void* src, size_t P, int Cs, int coff, int C, void* dst, void* stream);

/* Masked MSE of prediction = x[..., 0:3] + out[..., 0:3] against target =
 * xn[..., 0:3] over pixels whose solid channel x[..., 3] is 0 (all three
 * tensors NHWC with C channels).  dout (C channels, zero beyond 3) =
 * d loss / d out; loss_partial receives per-block sums (sg_loss_blocks()
 * floats) of squared error and of fluid pixels, added by the caller. */
int sg_masked_mse(const void* x, const void* out, const void* xn, size_t P, int C, void* dout, float* loss_partial,
                  float inv_count, void* stream);
int sg_loss_blocks(void);

/* Decoupled-weight-decay Adam on FP32 master weights w (n), writing the
 * bfloat16 copy w16 (may be NULL); step >= 1. */
int sg_adamw(float* w, void* w16, const float* g, float* m, float* v, size_t n, float lr, float beta1, float beta2,
             float eps, float weight_decay, int step, void* stream);

/* FP32 -> bfloat16 (round to nearest even), n elements. */
int sg_to_bf16(const float* src, size_t n, void* dst, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FDSURROGATE_H */
