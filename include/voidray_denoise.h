/*
 * voidray_denoise.h — C ABI of the learned denoiser of the GB300 backend.
 *
 * No counterpart in voidray: the reference only accumulates samples
 * (voidray_renderer/src/render/iterative.rs:11-55).  The denoiser is a small
 * U-Net over the renderer's radiance, albedo and normal buffers
 * (vr_render_aov_device): 4 levels of 32/64/128/256 channels, two 3x3
 * convolutions + ReLU per level, 2x2 average pooling down, nearest 2x
 * upsampling + skip concatenation up, a 3x3 output convolution.  Weights and
 * activations are bf16, products accumulate in fp32 on the tensor cores; the
 * optimiser (Adam) keeps fp32 master weights.  Training and inference run on
 * the library's own kernels.
 *
 * Input features (9 channels, stored padded to 16): log1p of the radiance
 * divided by (albedo + 0.01), the albedo, the normal.  The network predicts
 * the log1p of the demodulated radiance; the output is multiplied back by
 * (albedo + 0.01).  Loss (vr_denoiser_set_loss): the mean absolute error of
 * that prediction, or the relative MSE (y - t)^2 / (y^2 + 0.01) of the
 * remodulated radiance y against the target t, the denominator held constant
 * (the form suited to noisy rendered targets).
 *
 * Shares vr_status and vr_last_error() with voidray_gpu.h.
 */
#ifndef VOIDRAY_DENOISE_H
#define VOIDRAY_DENOISE_H

#include <stdint.h>

#include "voidray_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct vr_denoiser vr_denoiser;

typedef struct vr_denoiser_info {
    uint64_t param_count;      /* fp32 parameters, padded tensors included     */
    uint64_t steps;            /* Adam steps taken                              */
    uint64_t workspace_bytes;  /* device activation/gradient workspace held    */
    double flops_per_pixel;    /* forward FLOPs per full-resolution pixel      */
    uint32_t num_layers;
    uint32_t input_channels;   /* 9                                             */
} vr_denoiser_info;

/* One 3x3 convolution of the network: input = concat(src1 (upsampled 2x when
 * up1), src2), weights [cout][9][c1+c2] at w_offset, bias [cout] at b_offset
 * (offsets in floats into the parameter vector). */
typedef struct vr_denoiser_layer {
    uint32_t c1, c2, up1, cout, relu, level;
    uint64_t w_offset, b_offset;
} vr_denoiser_layer;

/* Creates the network on the current device with He-normal weights drawn
 * from `seed` (zero biases). */
vr_status vr_denoiser_create(uint64_t seed, vr_denoiser** out);
vr_status vr_denoiser_destroy(vr_denoiser* net);
vr_status vr_denoiser_info_get(const vr_denoiser* net, vr_denoiser_info* info);
vr_status vr_denoiser_layer_get(uint32_t index, vr_denoiser_layer* layer);
/* Training loss of later gradient / train-step calls (default L1_LOG). */
#define VR_DN_LOSS_L1_LOG 0
#define VR_DN_LOSS_RELMSE 1
vr_status vr_denoiser_set_loss(vr_denoiser* net, int32_t kind);
/* Convolutions on mma.sync (default) or on tcgen05 + TMEM with TMA operand
 * staging (forward and backward-data; the weight gradient stays on
 * mma.sync). */
#define VR_DN_BACKEND_MMA_SYNC 0
#define VR_DN_BACKEND_TCGEN05 1
vr_status vr_denoiser_set_backend(vr_denoiser* net, int32_t backend);
/* Synchronises, returns and clears the device status of the tcgen05 kernels
 * (VR_ERR_TIMEOUT when a bounded wait ran out). */
vr_status vr_denoiser_status(vr_denoiser* net, uint32_t* flags);
/* fp32 parameter vector (count must equal param_count).  set_params also
 * resets the optimiser state. */
vr_status vr_denoiser_get_params(vr_denoiser* net, float* host, uint64_t count);
vr_status vr_denoiser_set_params(vr_denoiser* net, const float* host, uint64_t count);

/* Denoises one image: rgba/albedo/normal are RGBA f32 device buffers of
 * width x height holding per-pixel sums, multiplied by `scale` (1/samples for
 * raw sums, 1 for means) before use.  Writes the denoised radiance (alpha 1)
 * to out_rgba (device, width x height x 4; may not alias the inputs).  Any
 * width and height: the network runs on the image padded to multiples of 8.
 * A handle owns one activation workspace (kept and reused by every call that
 * fits in it): calls on one handle from different streams must be ordered by
 * the caller; use one handle per stream for concurrent work. */
vr_status vr_denoise_device(vr_denoiser* net, const float* rgba, const float* albedo, const float* normal,
                            float scale, float* out_rgba, uint32_t width, uint32_t height, void* stream);

/* Denoises `batch` images of width x height at once ([batch][height][width][4]
 * f32 device buffers); image i is scaled by scales[i] (host array of batch
 * floats).  Same result per image as vr_denoise_device; one launch sequence
 * for the whole batch. */
vr_status vr_denoise_batch_device(vr_denoiser* net, const float* rgba, const float* albedo, const float* normal,
                                  const float* scales, float* out_rgba, uint32_t batch, uint32_t width,
                                  uint32_t height, void* stream);

/* Loss and gradients of a batch of `batch` crops (width, height multiples of
 * 8): inputs as vr_denoise_device (scaled by scale_in), target radiance
 * scaled by scale_target, all [batch][height][width][4] f32 on the device.
 * loss_host (optional) receives the mean loss per pixel and colour channel; grads_host
 * (optional, param_count floats) the gradient.  No parameter update. */
vr_status vr_denoiser_gradients_device(vr_denoiser* net, const float* rgba, const float* albedo,
                                       const float* normal, const float* target, float scale_in,
                                       float scale_target, uint32_t batch, uint32_t width, uint32_t height,
                                       float* loss_host, float* grads_host, void* stream);
/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) at learning rate lr on
 * the same batch layout.  loss_host (optional) synchronises and receives the
 * loss before the update. */
vr_status vr_denoiser_train_step_device(vr_denoiser* net, const float* rgba, const float* albedo,
                                        const float* normal, const float* target, float scale_in,
                                        float scale_target, uint32_t batch, uint32_t width, uint32_t height,
                                        float lr, float* loss_host, void* stream);

/* Single kernels, bf16 tensors as uint16 bit patterns (NHWC, channels
 * multiples of 16, h and w even when up1):
 * out = conv3x3(concat(up1 ? upsample2x(src1) : src1, src2), weight) + bias,
 * then ReLU when relu, then zero where mask <= 0 (mask optional), written
 * as bf16 to out_bf16 or as f32 to out_f32 (exactly one of them). */
vr_status vr_dn_conv3x3_device(const uint16_t* src1, uint32_t c1, int32_t up1, const uint16_t* src2, uint32_t c2,
                               const uint16_t* weight, const float* bias, const uint16_t* mask, uint16_t* out_bf16,
                               float* out_f32, uint32_t cout, uint32_t n, uint32_t h, uint32_t w, int32_t relu,
                               void* stream);
/* The same convolution on the tcgen05 tensor cores (no upsample; Cout a
 * multiple of 16, split into tiles of at most 256).  status_device
 * (optional) gets bit 1 / 2 when a bounded wait inside the kernel ran out. */
vr_status vr_dn_conv3x3_tc_device(const uint16_t* src1, uint32_t c1, const uint16_t* src2, uint32_t c2,
                                  const uint16_t* weight, const float* bias, const uint16_t* mask,
                                  uint16_t* out_bf16, float* out_f32, uint32_t cout, uint32_t n, uint32_t h,
                                  uint32_t w, int32_t relu, uint32_t* status_device, void* stream);
/* dw[co][tap][ci] += sum over pixels of dz[p][co] * input(p + tap)[ci]. */
vr_status vr_dn_conv3x3_wgrad_device(const uint16_t* dz, const uint16_t* src1, uint32_t c1, int32_t up1,
                                     const uint16_t* src2, uint32_t c2, float* dw, uint32_t cout, uint32_t n,
                                     uint32_t h, uint32_t w, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* VOIDRAY_DENOISE_H */
