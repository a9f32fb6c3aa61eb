// dn_kernels.h — launch interface of the denoiser's BF16 kernels.
//
// Activations are NHWC bf16 (channels innermost, 16-byte rows of 8 channels),
// weights [Cout][3*3][Cin] bf16 with an fp32 master copy; accumulation is fp32
// on the tensor cores (mma.sync m16n8k16).  Every channel count is a multiple
// of 16, images are N x H x W with H and W multiples of 8.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace dn {

using bf16 = __nv_bfloat16;

// 3x3 convolution, stride 1, zero padding 1, as an implicit GEMM
// (M = N*H*W pixels, N = Cout, K = 9*(C1+C2)).  The input is the channel
// concatenation [src1, src2]; with up1 set, src1 is an (H/2, W/2) tensor read
// through a nearest-neighbour 2x upsample.  Epilogue: + bias (optional),
// ReLU (optional), multiply by (mask > 0) (optional; the ReLU backward of the
// layer that produced the input), then store bf16 or fp32.
struct ConvArgs {
    const bf16* src1;
    const bf16* src2;
    const bf16* weight;  // [Cout][9][C1+C2]
    const float* bias;   // [Cout] or null
    const bf16* mask;    // [P][Cout] or null
    bf16* out;           // [P][Cout] (bf16) or null
    float* out_f32;      // [P][Cout] (fp32) or null
    int n, h, w;         // output image size (= full-resolution input size)
    int c1, c2, cout;
    int up1, relu;
};

// Weight gradient dw[co][tap][ci] += sum_p dz[p][co] * x(p + tap)[ci] over all
// pixels, with x read exactly as ConvArgs reads its input.  dw is fp32.
struct WgradArgs {
    const bf16* dz;      // [P][Cout]
    const bf16* src1;
    const bf16* src2;
    float* dw;           // [Cout][9][C1+C2]
    int n, h, w;
    int c1, c2, cout;
    int up1;
    int pix_per_split;   // multiple of 32
    float* db;           // optional [Cout]: the bias gradient (sum of dz over pixels) is added here too
};

cudaError_t conv3x3(const ConvArgs& a, cudaStream_t st);
// The same convolution on the 5th-generation tensor cores (tcgen05.mma,
// TMEM accumulator, TMA operand staging; dn_tc.cu): forward and
// backward-data (mask epilogue); no upsampled source (materialise it with
// upsample2 first); Cout a multiple of 16 split into tiles of at most 256.
// `status` (optional device word) receives bit 1 / 2 when a bounded wait ran out.
bool conv3x3_tc_supported(const ConvArgs& a);
cudaError_t conv3x3_tc(const ConvArgs& a, uint32_t* status, cudaStream_t st);
// out[n][y][x][c] = in[n][y/2][x/2][c] (nearest 2x upsample, (h, w) = output size)
cudaError_t upsample2(const bf16* in, bf16* out, int n, int h, int w, int c, cudaStream_t st);
cudaError_t conv3x3_wgrad(const WgradArgs& a, cudaStream_t st);
// db[c] += sum_p dz[p][c]
cudaError_t bias_grad(const bf16* dz, int p, int c, float* db, cudaStream_t st);
// 2x2 average pool (fp32 mean, rounded once)
cudaError_t avgpool2(const bf16* in, bf16* out, int n, int h, int w, int c, cudaStream_t st);
// dz[p][c] = (dcat[p][coff + c] + dpool[p/2][c] / 4) * (act[p][c] > 0), full resolution
cudaError_t skip_bwd(const bf16* dcat, int ccat, int coff, const bf16* dpool, const bf16* act, bf16* dz, int n,
                     int h, int w, int c, cudaStream_t st);
// dz[q][c] = (sum of the 2x2 fine pixels dcat[.][c], c < c1) * (act[q][c] > 0), coarse resolution (hc, wc)
cudaError_t up_bwd(const bf16* dcat, int ccat, const bf16* act, bf16* dz, int n, int hc, int wc, int c1,
                   cudaStream_t st);
// Network input from renderer buffers (RGBA f32, n images of width x height,
// sums scaled by scales[image] (device) or, when scales is null, by `scale`):
// ch 0-2 log1p(radiance / (albedo + DEMOD_EPS)), 3-5 albedo, 6-8 normal,
// 9-15 zero; pixels outside the image (padding to h x w) zero.
constexpr float DEMOD_EPS = 0.01f;
cudaError_t preprocess(const float4* rad, const float4* alb, const float4* nrm, float scale, const float* scales,
                       int n, int img_h, int img_w, int h, int w, bf16* x0, cudaStream_t st);
// out[p][0..2] (log irradiance) -> rgba = expm1(clamp(o, 0, 80)) * (albedo + DEMOD_EPS), alpha 1
cudaError_t postprocess(const float* out, int cout, const float4* alb, float scale, const float* scales, int n,
                        int img_h, int img_w, int h, int w, float4* rgba, cudaStream_t st);
// Loss against the target radiance; writes the gradient (bf16, [P][cout],
// zero beyond channel 2, scaled by inv_count) and adds the loss sum to *loss_sum.
constexpr int LOSS_L1_LOG = 0;  // L1 of the log-demodulated prediction
constexpr int LOSS_RELMSE = 1;  // relative MSE of the remodulated radiance
cudaError_t loss(const float* out, int cout, const float4* target, const float4* alb, float scale_target,
                 float scale_alb, int n, int h, int w, float inv_count, int kind, bf16* grad, float* loss_sum,
                 cudaStream_t st);
cudaError_t adam(float* w, float* g, float* m, float* v, size_t n, float lr, float b1, float b2, float eps, float bc1,
                 float bc2, cudaStream_t st);
// w16 = bf16(w32); wt16[ci][tap][co] = bf16(w32[co][8 - tap][ci]) (the bwd-data weights)
cudaError_t cast_flip(const float* w32, bf16* w16, bf16* wt16, int cout, int cin, cudaStream_t st);

}  // namespace dn
