// dn_kernels.cu — BF16 kernels of the U-Net denoiser (tensor cores through
// mma.sync m16n8k16 with fp32 accumulation; cp.async multi-stage pipelines
// feeding XOR-swizzled shared-memory tiles read with ldmatrix).
//
//   k_conv3x3        implicit-GEMM 3x3 convolution: forward (bias + ReLU
//                    epilogue) and, with flipped weights and a ReLU mask,
//                    backward-data; the input may be the concatenation of an
//                    upsampled coarse tensor and a skip tensor (fused gather)
//   k_conv3x3_wgrad  weight gradient, pixel range split across CTAs, fp32
//                    atomics into the gradient buffer
//   glue             2x2 average pool, skip / upsample backward, bias grad,
//                    pre/post-processing, L1 loss, Adam, weight cast + flip
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>

#include "dn_kernels.h"

namespace dn {
namespace {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// 16-byte async copy global -> shared; src_size 0 writes zeros (padding)
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, bool valid) {
    const int n = valid ? 16 : 0;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(n));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

__device__ __forceinline__ void ldsm_x4(uint32_t a, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(a));
}
__device__ __forceinline__ void ldsm_x2(uint32_t a, uint32_t& r0, uint32_t& r1) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n" : "=r"(r0), "=r"(r1) : "r"(a));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t a, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(a));
}
__device__ __forceinline__ void ldsm_x2_t(uint32_t a, uint32_t& r0, uint32_t& r1) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];\n" : "=r"(r0), "=r"(r1) : "r"(a));
}

// D += A(16x16, row) * B(16x8, col), bf16 in, fp32 accumulate
__device__ __forceinline__ void mma_bf16(float* d, const uint32_t* a, const uint32_t* b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Shared tiles are rows of CPR 16-byte chunks; chunk c of row r is stored at
// chunk c ^ swz(r), so the 8 rows one ldmatrix phase reads hit 8 different
// 16-byte bank groups.
template <int CPR>
__device__ __forceinline__ int swz(int row) {
    return (row / (8 / CPR)) & (CPR - 1);
}

struct Pix {
    int n, y, x;
};
__device__ __forceinline__ Pix pix_of(int p, int h, int w) {
    Pix r;
    const int hw = h * w;
    r.n = p / hw;
    const int q = p - r.n * hw;
    r.y = q / w;
    r.x = q - r.y * w;
    return r;
}

// Address of input channels [c, c+8) of pixel (n, yy, xx) of the
// concatenated (and optionally upsampled) convolution input.
__device__ __forceinline__ const bf16* in_addr(const bf16* src1, const bf16* src2, int c1, int c2, int up1, int h,
                                               int w, int n, int yy, int xx, int c) {
    if (c < c1) {
        const int hs = up1 ? (h >> 1) : h, ws = up1 ? (w >> 1) : w;
        const int ys = up1 ? (yy >> 1) : yy, xs = up1 ? (xx >> 1) : xx;
        return src1 + ((size_t)(n * hs + ys) * ws + xs) * c1 + c;
    }
    return src2 + ((size_t)(n * h + yy) * w + xx) * c2 + (c - c1);
}

// ---------------------------------------------------------------- conv ----
// CTA tile 128 pixels x BN output channels, K step BK (one tap, BK input
// channels), 3-stage cp.async pipeline, 8 warps as 4 (M) x 2 (N).
template <int BK, int BN>
__global__ void __launch_bounds__(256) k_conv3x3(const ConvArgs a) {
    constexpr int BM = 128, STAGES = 3, CPR = BK / 8, NT = BN / 16;
    constexpr int A_CH = BM * CPR, B_CH = BN * CPR;
    constexpr int A_IT = A_CH / 256;
    constexpr int B_IT = (B_CH + 255) / 256;
    __shared__ __align__(128) bf16 sA[STAGES][BM * BK];
    __shared__ __align__(128) bf16 sB[STAGES][BN * BK];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = warp & 3, wn = warp >> 2;
    const int P = a.n * a.h * a.w;
    const int pbase = blockIdx.x * BM, nbase = blockIdx.y * BN;
    const int cin = a.c1 + a.c2;
    const int kct = cin / BK, nk = 9 * kct;

    Pix ap[A_IT];
    bool ain[A_IT];
#pragma unroll
    for (int i = 0; i < A_IT; ++i) {
        const int p = pbase + (tid + i * 256) / CPR;
        ain[i] = p < P;
        ap[i] = pix_of(ain[i] ? p : 0, a.h, a.w);
    }
    auto load = [&](int stage, int kt) {
        const int tap = kt / kct, c0 = (kt - tap * kct) * BK;
        const int dy = tap / 3 - 1, dx = tap % 3 - 1;
#pragma unroll
        for (int i = 0; i < A_IT; ++i) {
            const int idx = tid + i * 256, row = idx / CPR, ch = idx % CPR;
            const int yy = ap[i].y + dy, xx = ap[i].x + dx;
            const bool ok = ain[i] && yy >= 0 && yy < a.h && xx >= 0 && xx < a.w;
            const bf16* src = ok ? in_addr(a.src1, a.src2, a.c1, a.c2, a.up1, a.h, a.w, ap[i].n, yy, xx, c0 + ch * 8)
                                 : a.weight;
            cp_async16(smem_u32(&sA[stage][row * BK + ((ch ^ swz<CPR>(row)) << 3)]), src, ok);
        }
#pragma unroll
        for (int i = 0; i < B_IT; ++i) {
            const int idx = tid + i * 256;
            if ((B_CH % 256) != 0 && idx >= B_CH) break;
            const int row = idx / CPR, ch = idx % CPR;
            const int co = nbase + row;
            const bool ok = co < a.cout;
            const bf16* src = ok ? a.weight + (size_t)co * 9 * cin + tap * cin + c0 + ch * 8 : a.weight;
            cp_async16(smem_u32(&sB[stage][row * BK + ((ch ^ swz<CPR>(row)) << 3)]), src, ok);
        }
    };

    float acc[2][NT][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < NT; ++j)
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[i][j][k] = 0.0f;

#pragma unroll
    for (int s = 0; s < STAGES - 1; ++s) {
        if (s < nk) load(s, s);
        cp_commit();
    }
    for (int kt = 0; kt < nk; ++kt) {
        cp_wait<STAGES - 2>();
        __syncthreads();
        if (kt + STAGES - 1 < nk) load((kt + STAGES - 1) % STAGES, kt + STAGES - 1);
        cp_commit();
        const bf16* tA = sA[kt % STAGES];
        const bf16* tB = sB[kt % STAGES];
#pragma unroll
        for (int kk = 0; kk < BK; kk += 16) {
            uint32_t af[2][4], bfr[NT][2];
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                const int row = wm * 32 + mt * 16 + (lane & 15);
                const int ch = (kk >> 3) + (lane >> 4);
                ldsm_x4(smem_u32(tA + row * BK + ((ch ^ swz<CPR>(row)) << 3)), af[mt][0], af[mt][1], af[mt][2],
                        af[mt][3]);
            }
            if constexpr (NT == 1) {
                const int row = wn * 8 + (lane & 7);
                const int ch = (kk >> 3) + ((lane >> 3) & 1);
                ldsm_x2(smem_u32(tB + row * BK + ((ch ^ swz<CPR>(row)) << 3)), bfr[0][0], bfr[0][1]);
            } else {
#pragma unroll
                for (int j = 0; j < NT / 2; ++j) {
                    const int row = wn * (BN / 2) + j * 16 + (lane & 7) + ((lane >> 4) << 3);
                    const int ch = (kk >> 3) + ((lane >> 3) & 1);
                    ldsm_x4(smem_u32(tB + row * BK + ((ch ^ swz<CPR>(row)) << 3)), bfr[2 * j][0], bfr[2 * j][1],
                            bfr[2 * j + 1][0], bfr[2 * j + 1][1]);
                }
            }
#pragma unroll
            for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                for (int nt = 0; nt < NT; ++nt) mma_bf16(acc[mt][nt], af[mt], bfr[nt]);
        }
    }
    cp_wait<0>();

    // epilogue: fragment element (r, c) at row lane/4 (+8), column 2*(lane%4) (+1)
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
            const int col = nbase + wn * (BN / 2) + nt * 8 + 2 * (lane & 3);
            if (col >= a.cout) continue;
            float b0 = 0.0f, b1 = 0.0f;
            if (a.bias) {
                b0 = a.bias[col];
                b1 = a.bias[col + 1];
            }
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
                const int p = pbase + wm * 32 + mt * 16 + (lane >> 2) + 8 * hh;
                if (p >= P) continue;
                float v0 = acc[mt][nt][2 * hh] + b0, v1 = acc[mt][nt][2 * hh + 1] + b1;
                if (a.relu) {
                    v0 = fmaxf(v0, 0.0f);
                    v1 = fmaxf(v1, 0.0f);
                }
                const size_t o = (size_t)p * a.cout + col;
                if (a.mask) {
                    const __nv_bfloat162 m = *reinterpret_cast<const __nv_bfloat162*>(a.mask + o);
                    if (!(__bfloat162float(m.x) > 0.0f)) v0 = 0.0f;
                    if (!(__bfloat162float(m.y) > 0.0f)) v1 = 0.0f;
                }
                if (a.out_f32) {
                    *reinterpret_cast<float2*>(a.out_f32 + o) = make_float2(v0, v1);
                } else {
                    __nv_bfloat162 r;
                    r.x = __float2bfloat16_rn(v0);
                    r.y = __float2bfloat16_rn(v1);
                    *reinterpret_cast<__nv_bfloat162*>(a.out + o) = r;
                }
            }
        }
}

// --------------------------------------------------------------- wgrad ----
// GEMM per tap: M = Cout (tile BM), N = Cin (tile BN), K = pixels (step 32).
// Both operands sit in shared memory pixel-major (K rows); ldmatrix.trans
// turns them into the row-major A and column-major B fragments.  4 warps as
// 2 (M) x 2 (N).
template <int BM, int BN>
__global__ void __launch_bounds__(128) k_conv3x3_wgrad(const WgradArgs a) {
    constexpr int BK = 32, STAGES = 3, CPA = BM / 8, CPB = BN / 8, MT = BM / 32, NT = BN / 16;
    constexpr int A_CH = BK * CPA, B_CH = BK * CPB;
    __shared__ __align__(128) bf16 sA[STAGES][BK * BM];
    __shared__ __align__(128) bf16 sB[STAGES][BK * BN];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = warp & 1, wn = warp >> 1;
    const int P = a.n * a.h * a.w;
    const int cin = a.c1 + a.c2;
    const int co0 = blockIdx.x * BM;
    const int tap = blockIdx.y % 9, ci0 = (blockIdx.y / 9) * BN;
    const int dy = tap / 3 - 1, dx = tap % 3 - 1;
    const int pb = blockIdx.z * a.pix_per_split;
    const int pe = min(P, pb + a.pix_per_split);
    if (pb >= pe) return;
    const int nk = (pe - pb + BK - 1) / BK;

    auto load = [&](int stage, int kt) {
        const int p0 = pb + kt * BK;
        for (int idx = tid; idx < A_CH; idx += 128) {
            const int row = idx / CPA, ch = idx % CPA;
            const int p = p0 + row, co = co0 + ch * 8;
            const bool ok = p < pe && co < a.cout;
            const bf16* src = ok ? a.dz + (size_t)p * a.cout + co : a.dz;
            cp_async16(smem_u32(&sA[stage][row * BM + ((ch ^ swz<CPA>(row)) << 3)]), src, ok);
        }
        for (int idx = tid; idx < B_CH; idx += 128) {
            const int row = idx / CPB, ch = idx % CPB;
            const int p = p0 + row;
            bool ok = p < pe;
            const bf16* src = a.dz;
            if (ok) {
                const Pix q = pix_of(p, a.h, a.w);
                const int yy = q.y + dy, xx = q.x + dx;
                ok = yy >= 0 && yy < a.h && xx >= 0 && xx < a.w;
                if (ok) src = in_addr(a.src1, a.src2, a.c1, a.c2, a.up1, a.h, a.w, q.n, yy, xx, ci0 + ch * 8);
            }
            cp_async16(smem_u32(&sB[stage][row * BN + ((ch ^ swz<CPB>(row)) << 3)]), src, ok);
        }
    };

    float acc[MT][NT][4];
#pragma unroll
    for (int i = 0; i < MT; ++i)
#pragma unroll
        for (int j = 0; j < NT; ++j)
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[i][j][k] = 0.0f;

#pragma unroll
    for (int s = 0; s < STAGES - 1; ++s) {
        if (s < nk) load(s, s);
        cp_commit();
    }
    for (int kt = 0; kt < nk; ++kt) {
        cp_wait<STAGES - 2>();
        __syncthreads();
        if (kt + STAGES - 1 < nk) load((kt + STAGES - 1) % STAGES, kt + STAGES - 1);
        cp_commit();
        const bf16* tA = sA[kt % STAGES];
        const bf16* tB = sB[kt % STAGES];
#pragma unroll
        for (int kk = 0; kk < BK; kk += 16) {
            uint32_t af[MT][4], bfr[NT][2];
            const int i4 = lane >> 3;
#pragma unroll
            for (int mt = 0; mt < MT; ++mt) {
                const int krow = kk + (lane & 7) + ((i4 >> 1) << 3);
                const int ch = (wm * (BM / 2) + mt * 16 + ((i4 & 1) << 3)) >> 3;
                ldsm_x4_t(smem_u32(tA + krow * BM + ((ch ^ swz<CPA>(krow)) << 3)), af[mt][0], af[mt][1], af[mt][2],
                          af[mt][3]);
            }
            if constexpr (NT == 1) {
                const int krow = kk + (lane & 7) + (((lane >> 3) & 1) << 3);
                const int ch = (wn * (BN / 2)) >> 3;
                ldsm_x2_t(smem_u32(tB + krow * BN + ((ch ^ swz<CPB>(krow)) << 3)), bfr[0][0], bfr[0][1]);
            } else {
                const int krow = kk + (lane & 7) + ((i4 & 1) << 3);
                const int ch = (wn * (BN / 2) + ((i4 >> 1) << 3)) >> 3;
                ldsm_x4_t(smem_u32(tB + krow * BN + ((ch ^ swz<CPB>(krow)) << 3)), bfr[0][0], bfr[0][1], bfr[1][0],
                          bfr[1][1]);
            }
#pragma unroll
            for (int mt = 0; mt < MT; ++mt)
#pragma unroll
                for (int nt = 0; nt < NT; ++nt) mma_bf16(acc[mt][nt], af[mt], bfr[nt]);
        }
    }
    cp_wait<0>();

#pragma unroll
    for (int mt = 0; mt < MT; ++mt)
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
            const int ci = ci0 + wn * (BN / 2) + nt * 8 + 2 * (lane & 3);
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
                const int co = co0 + wm * (BM / 2) + mt * 16 + (lane >> 2) + 8 * hh;
                if (co >= a.cout) continue;
                float* d = a.dw + ((size_t)co * 9 + tap) * cin + ci;
                atomicAdd(d, acc[mt][nt][2 * hh]);
                atomicAdd(d + 1, acc[mt][nt][2 * hh + 1]);
            }
        }
}

// ---------------------------------------------------------------- glue ----
// db[c] += sum over pixels of dz[p][c].  Each thread sums 8 channels (one
// 16-byte load) of every (256 / (C / 8))-th pixel of the block's rows, four
// loads in flight; the block reduces per channel in shared memory and adds
// one float per channel.  C is a multiple of 8 up to 256.
__global__ void __launch_bounds__(256) k_bias_grad(const bf16* __restrict__ dz, int P, int C, int rows,
                                                    float* __restrict__ db) {
    __shared__ float red[256 * 8];
    const int tpp = C >> 3;              // threads per pixel
    const int slots = blockDim.x / tpp;  // pixels per step
    const int g = threadIdx.x % tpp, slot = threadIdx.x / tpp;
    const int p0 = blockIdx.x * rows, p1 = min(P, p0 + rows);
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (slot < slots) {
        const uint4* base = reinterpret_cast<const uint4*>(dz) + g;
        int p = p0 + slot;
        for (; p + 3 * slots < p1; p += 4 * slots) {
            uint4 v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) v[u] = __ldg(base + (size_t)(p + u * slots) * tpp);
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const bf16* h = reinterpret_cast<const bf16*>(&v[u]);
#pragma unroll
                for (int j = 0; j < 8; ++j) acc[j] += __bfloat162float(h[j]);
            }
        }
        for (; p < p1; p += slots) {
            const uint4 v = __ldg(base + (size_t)p * tpp);
            const bf16* h = reinterpret_cast<const bf16*>(&v);
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[j] += __bfloat162float(h[j]);
        }
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) red[threadIdx.x * 8 + j] = acc[j];
    __syncthreads();
    if (threadIdx.x < C) {  // one thread per channel: sum over the pixel slots
        const int cg = threadIdx.x >> 3, cj = threadIdx.x & 7;
        float s = 0.0f;
        for (int k = 0; k < slots; ++k) s += red[(k * tpp + cg) * 8 + cj];
        atomicAdd(&db[threadIdx.x], s);
    }
}

union V8 {
    uint4 u;
    bf16 h[8];
};

__global__ void k_avgpool2(const bf16* __restrict__ in, bf16* __restrict__ out, int n, int h, int w, int c) {
    const int hc = h >> 1, wc = w >> 1, c8 = c >> 3;
    const size_t total = (size_t)n * hc * wc * c8;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int ch = (int)(i % c8);
        size_t q = i / c8;
        const int x = (int)(q % wc);
        q /= wc;
        const int y = (int)(q % hc);
        const int nn = (int)(q / hc);
        float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
        for (int d = 0; d < 4; ++d) {
            const int yy = 2 * y + (d >> 1), xx = 2 * x + (d & 1);
            V8 v;
            v.u = *reinterpret_cast<const uint4*>(in + ((size_t)(nn * h + yy) * w + xx) * c + ch * 8);
#pragma unroll
            for (int k = 0; k < 8; ++k) s[k] += __bfloat162float(v.h[k]);
        }
        V8 o;
#pragma unroll
        for (int k = 0; k < 8; ++k) o.h[k] = __float2bfloat16_rn(s[k] * 0.25f);
        *reinterpret_cast<uint4*>(out + ((size_t)(nn * hc + y) * wc + x) * c + ch * 8) = o.u;
    }
}

__global__ void k_upsample2(const uint4* __restrict__ in, uint4* __restrict__ out, int n, int h, int w, int c8) {
    const size_t total = (size_t)n * h * w * c8;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int ch = (int)(i % c8);
        const size_t p = i / c8;
        const int x = (int)(p % w);
        const int y = (int)((p / w) % h);
        const int nn = (int)(p / ((size_t)w * h));
        out[i] = in[(((size_t)nn * (h >> 1) + (y >> 1)) * (w >> 1) + (x >> 1)) * c8 + ch];
    }
}

__global__ void k_skip_bwd(const bf16* __restrict__ dcat, int ccat, int coff, const bf16* __restrict__ dpool,
                           const bf16* __restrict__ act, bf16* __restrict__ dz, int n, int h, int w, int c) {
    const int c8 = c >> 3, hc = h >> 1, wc = w >> 1;
    const size_t total = (size_t)n * h * w * c8;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int ch = (int)(i % c8);
        const size_t p = i / c8;
        const int x = (int)(p % w);
        const int y = (int)((p / w) % h);
        const int nn = (int)(p / ((size_t)w * h));
        V8 a, b, m, o;
        a.u = *reinterpret_cast<const uint4*>(dcat + p * ccat + coff + ch * 8);
        b.u = *reinterpret_cast<const uint4*>(dpool + ((size_t)(nn * hc + (y >> 1)) * wc + (x >> 1)) * c + ch * 8);
        m.u = *reinterpret_cast<const uint4*>(act + p * c + ch * 8);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const float v = __bfloat162float(a.h[k]) + 0.25f * __bfloat162float(b.h[k]);
            o.h[k] = __float2bfloat16_rn(__bfloat162float(m.h[k]) > 0.0f ? v : 0.0f);
        }
        *reinterpret_cast<uint4*>(dz + p * c + ch * 8) = o.u;
    }
}

__global__ void k_up_bwd(const bf16* __restrict__ dcat, int ccat, const bf16* __restrict__ act,
                         bf16* __restrict__ dz, int n, int hc, int wc, int c1) {
    const int c8 = c1 >> 3, h = hc * 2, w = wc * 2;
    const size_t total = (size_t)n * hc * wc * c8;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int ch = (int)(i % c8);
        const size_t q = i / c8;
        const int x = (int)(q % wc);
        const int y = (int)((q / wc) % hc);
        const int nn = (int)(q / ((size_t)wc * hc));
        float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
        for (int d = 0; d < 4; ++d) {
            const int yy = 2 * y + (d >> 1), xx = 2 * x + (d & 1);
            V8 v;
            v.u = *reinterpret_cast<const uint4*>(dcat + ((size_t)(nn * h + yy) * w + xx) * ccat + ch * 8);
#pragma unroll
            for (int k = 0; k < 8; ++k) s[k] += __bfloat162float(v.h[k]);
        }
        V8 m, o;
        m.u = *reinterpret_cast<const uint4*>(act + q * c1 + ch * 8);
#pragma unroll
        for (int k = 0; k < 8; ++k) o.h[k] = __float2bfloat16_rn(__bfloat162float(m.h[k]) > 0.0f ? s[k] : 0.0f);
        *reinterpret_cast<uint4*>(dz + q * c1 + ch * 8) = o.u;
    }
}

__device__ __forceinline__ float finite_or_zero(float v) {
    // NaN -> 0, +-inf -> +-1e30 (keeps log1p finite)
    if (!(v == v)) return 0.0f;
    return fminf(fmaxf(v, -1e30f), 1e30f);
}

__global__ void k_preprocess(const float4* __restrict__ rad, const float4* __restrict__ alb,
                             const float4* __restrict__ nrm, float scale_all, const float* __restrict__ scales, int n,
                             int ih, int iw, int h, int w, bf16* __restrict__ x0) {
    const size_t total = (size_t)n * h * w;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < total; p += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(p % w);
        const int y = (int)((p / w) % h);
        const int nn = (int)(p / ((size_t)w * h));
        V8 lo, hi;
#pragma unroll
        for (int k = 0; k < 8; ++k) lo.h[k] = hi.h[k] = __float2bfloat16_rn(0.0f);
        if (y < ih && x < iw) {
            const float scale = scales ? scales[nn] : scale_all;
            const size_t s = ((size_t)nn * ih + y) * iw + x;
            const float4 r = rad[s], a = alb[s], q = nrm[s];
            const float ar = finite_or_zero(a.x * scale), ag = finite_or_zero(a.y * scale),
                        ab = finite_or_zero(a.z * scale);
            const float rr = fmaxf(finite_or_zero(r.x * scale), 0.0f);
            const float rg = fmaxf(finite_or_zero(r.y * scale), 0.0f);
            const float rb = fmaxf(finite_or_zero(r.z * scale), 0.0f);
            lo.h[0] = __float2bfloat16_rn(log1pf(rr / (ar + DEMOD_EPS)));
            lo.h[1] = __float2bfloat16_rn(log1pf(rg / (ag + DEMOD_EPS)));
            lo.h[2] = __float2bfloat16_rn(log1pf(rb / (ab + DEMOD_EPS)));
            lo.h[3] = __float2bfloat16_rn(ar);
            lo.h[4] = __float2bfloat16_rn(ag);
            lo.h[5] = __float2bfloat16_rn(ab);
            lo.h[6] = __float2bfloat16_rn(finite_or_zero(q.x * scale));
            lo.h[7] = __float2bfloat16_rn(finite_or_zero(q.y * scale));
            hi.h[0] = __float2bfloat16_rn(finite_or_zero(q.z * scale));
        }
        uint4* o = reinterpret_cast<uint4*>(x0 + p * 16);
        o[0] = lo.u;
        o[1] = hi.u;
    }
}

__global__ void k_postprocess(const float* __restrict__ out, int cout, const float4* __restrict__ alb,
                              float scale_all, const float* __restrict__ scales, int n, int ih, int iw, int h, int w,
                              float4* __restrict__ rgba) {
    const size_t total = (size_t)n * ih * iw;
    for (size_t s = blockIdx.x * (size_t)blockDim.x + threadIdx.x; s < total; s += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(s % iw);
        const int y = (int)((s / iw) % ih);
        const int nn = (int)(s / ((size_t)iw * ih));
        const float* o = out + (((size_t)nn * h + y) * w + x) * cout;
        const float scale = scales ? scales[nn] : scale_all;
        const float4 a = alb[s];
        float4 r;
        r.x = expm1f(fminf(fmaxf(o[0], 0.0f), 80.0f)) * (finite_or_zero(a.x * scale) + DEMOD_EPS);
        r.y = expm1f(fminf(fmaxf(o[1], 0.0f), 80.0f)) * (finite_or_zero(a.y * scale) + DEMOD_EPS);
        r.z = expm1f(fminf(fmaxf(o[2], 0.0f), 80.0f)) * (finite_or_zero(a.z * scale) + DEMOD_EPS);
        r.w = 1.0f;
        rgba[s] = r;
    }
}

// kind LOSS_L1_LOG: |o - log1p(t / (albedo + eps))|, gradient sign(d) / count.
// kind LOSS_RELMSE: (y - t)^2 / (max(y, 0)^2 + 0.01) with y = expm1(min(o, 20))
// * (albedo + eps), the relative error the renders are measured in, normalised
// by the prediction held constant (the target is itself a noisy render, and a
// noisy denominator would bias the fit); gradient
// 2 (y - t) / (max(y, 0)^2 + 0.01) * (albedo + eps) * exp(o) / count.
__global__ void k_loss(const float* __restrict__ out, int cout, const float4* __restrict__ tgt,
                       const float4* __restrict__ alb, float st, float sa, size_t total, float inv_count, int kind,
                       bf16* __restrict__ grad, float* __restrict__ loss) {
    __shared__ float red[256];
    float s = 0.0f;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < total; p += (size_t)gridDim.x * blockDim.x) {
        const float4 t = tgt[p], a = alb[p];
        const float tv[3] = {t.x, t.y, t.z}, av[3] = {a.x, a.y, a.z};
        const float* o = out + p * cout;
        bf16* g = grad + p * cout;
        for (int c = 0; c < cout; ++c) {
            float gv = 0.0f;
            if (c < 3) {
                const float tc = fmaxf(finite_or_zero(tv[c] * st), 0.0f);
                const float ae = finite_or_zero(av[c] * sa) + DEMOD_EPS;
                if (kind == LOSS_RELMSE) {
                    // exp(20) * 1.01 is far above any radiance the tracer
                    // produces; the cap keeps the square and gradient finite
                    const float e = expf(fminf(o[c], 20.0f));
                    const float y = (e - 1.0f) * ae;
                    const float yp = fmaxf(y, 0.0f);
                    const float den = 1.0f / (yp * yp + 0.01f);
                    const float r = y - tc;
                    s += r * r * den;
                    gv = o[c] < 20.0f ? 2.0f * r * den * ae * e * inv_count : 0.0f;
                } else {
                    const float d = o[c] - log1pf(tc / ae);
                    s += fabsf(d);
                    gv = d > 0.0f ? inv_count : (d < 0.0f ? -inv_count : 0.0f);
                }
            }
            g[c] = __float2bfloat16_rn(gv);
        }
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if ((int)threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, red[0]);
}

__global__ void k_adam(float* __restrict__ w, float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       size_t n, float lr, float b1, float b2, float eps, float bc1, float bc2) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
        g[i] = 0.0f;
    }
}

__global__ void k_cast_flip(const float* __restrict__ w32, bf16* __restrict__ w16, bf16* __restrict__ wt16, int cout,
                            int cin) {
    const size_t total = (size_t)cout * 9 * cin;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int ci = (int)(i % cin);
        const int tap = (int)((i / cin) % 9);
        const int co = (int)(i / ((size_t)cin * 9));
        const bf16 b = __float2bfloat16_rn(w32[i]);
        w16[i] = b;
        if (wt16) wt16[((size_t)ci * 9 + (8 - tap)) * cout + co] = b;
    }
}

unsigned grid_for(size_t n, unsigned block) {
    size_t g = (n + block - 1) / block;
    if (g > 152u * 32u) g = 152u * 32u;
    return (unsigned)(g ? g : 1);
}

template <int BK, int BN>
cudaError_t launch_conv(const ConvArgs& a, cudaStream_t st) {
    const int P = a.n * a.h * a.w;
    dim3 grid((P + 127) / 128, (a.cout + BN - 1) / BN);
    k_conv3x3<BK, BN><<<grid, 256, 0, st>>>(a);
    return cudaGetLastError();
}

template <int BM, int BN>
cudaError_t launch_wgrad(WgradArgs a, cudaStream_t st) {
    const int P = a.n * a.h * a.w;
    const int cin = a.c1 + a.c2;
    const int tiles = ((a.cout + BM - 1) / BM) * 9 * (cin / BN);
    // about four CTAs per SM, splits of at least 512 pixels
    int splits = (152 * 4 + tiles - 1) / tiles;
    const int max_splits = (P + 511) / 512;
    if (splits > max_splits) splits = max_splits;
    if (splits < 1) splits = 1;
    int pps = (P + splits - 1) / splits;
    pps = (pps + 31) / 32 * 32;
    a.pix_per_split = pps;
    splits = (P + pps - 1) / pps;
    dim3 grid((a.cout + BM - 1) / BM, 9 * (cin / BN), splits);
    k_conv3x3_wgrad<BM, BN><<<grid, 128, 0, st>>>(a);
    return cudaGetLastError();
}


// Weight gradient with all nine taps per CTA: the K loop walks 4 x 8-pixel
// blocks of the image; per block the CTA stages the 32 pixels' output
// gradients (A, [pixel][co]) once and one 6 x 10 halo of the input (B,
// [halo pixel][ci]) once, and each tap's B operand is that halo seen through
// per-lane ldmatrix row addresses (pixel (r, c) of the block -> halo row
// (r + dy + 1) * 10 + (c + dx + 1)).  Warps are (BM / 16) x (BN / 16), each
// owning a 16 (co) x 16 (ci) tile of all nine taps; partial sums over a CTA's
// range of blocks are added to dw with fp32 atomics.  Needs h % 4 == 0 and
// w % 8 == 0.
template <int BM, int BN>
__global__ void __launch_bounds__(32 * (BM / 16) * (BN / 16)) k_conv3x3_wgrad9(const WgradArgs a) {
    constexpr int STAGES = 3, CPA = BM / 8, CPB = BN / 8, WN = BN / 16;
    constexpr int NTHREADS = 32 * (BM / 16) * WN;
    constexpr int A_ROWS = 32, B_ROWS = 60;
    constexpr int NT = 2;  // two 8-wide n tiles per warp
    __shared__ __align__(128) bf16 sA[STAGES][A_ROWS * BM];
    __shared__ __align__(128) bf16 sB[STAGES][B_ROWS * BN];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = warp / WN, wn = warp % WN;
    const int cin = a.c1 + a.c2;
    const int co0 = blockIdx.x * BM, ci0 = blockIdx.y * BN;
    const int bx_n = a.w >> 3, by_n = a.h >> 2, per_img = bx_n * by_n;
    const int nblk = a.n * per_img;
    const int b0 = blockIdx.z * a.pix_per_split, b1 = min(nblk, b0 + a.pix_per_split);  // in blocks here
    if (b0 >= b1) return;
    const int nk = b1 - b0;

    auto load = [&](int stage, int kb) {
        const int blk = b0 + kb;
        const int img = blk / per_img, rem = blk - img * per_img;
        const int y0 = (rem / bx_n) * 4, x0 = (rem % bx_n) * 8;
        for (int idx = tid; idx < A_ROWS * CPA; idx += NTHREADS) {
            const int row = idx / CPA, ch = idx % CPA;
            const int y = y0 + (row >> 3), x = x0 + (row & 7), co = co0 + ch * 8;
            const bool ok = co < a.cout;
            const bf16* src = ok ? a.dz + ((size_t)(img * a.h + y) * a.w + x) * a.cout + co : a.dz;
            cp_async16(smem_u32(&sA[stage][row * BM + ((ch ^ swz<CPA>(row)) << 3)]), src, ok);
        }
        for (int idx = tid; idx < B_ROWS * CPB; idx += NTHREADS) {
            const int row = idx / CPB, ch = idx % CPB;
            const int yy = y0 - 1 + row / 10, xx = x0 - 1 + row % 10;
            const bool ok = yy >= 0 && yy < a.h && xx >= 0 && xx < a.w;
            const bf16* src = ok ? in_addr(a.src1, a.src2, a.c1, a.c2, a.up1, a.h, a.w, img, yy, xx, ci0 + ch * 8)
                                 : a.dz;
            cp_async16(smem_u32(&sB[stage][row * BN + ((ch ^ swz<CPB>(row)) << 3)]), src, ok);
        }
    };

    float acc[9][NT][4];
#pragma unroll
    for (int t = 0; t < 9; ++t)
#pragma unroll
        for (int j = 0; j < NT; ++j)
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[t][j][k] = 0.0f;

#pragma unroll
    for (int s = 0; s < STAGES - 1; ++s) {
        if (s < nk) load(s, s);
        cp_commit();
    }
    const int i4 = lane >> 3;
    // fused bias gradient (CTAs of the first ci tile): thread -> one output
    // channel column of the staged dz block and a quarter... of its 32 rows
    const bool bias = a.db && blockIdx.y == 0;
    constexpr int BIAS_PARTS = NTHREADS / BM;  // threads per column
    const int bcol = tid % BM, bpart = tid / BM;
    float bsum = 0.0f;
    for (int kb = 0; kb < nk; ++kb) {
        cp_wait<STAGES - 2>();
        __syncthreads();
        if (kb + STAGES - 1 < nk) load((kb + STAGES - 1) % STAGES, kb + STAGES - 1);
        cp_commit();
        const bf16* tA = sA[kb % STAGES];
        const bf16* tB = sB[kb % STAGES];
        if (bias)
            for (int row = bpart; row < A_ROWS; row += BIAS_PARTS)
                bsum += __bfloat162float(tA[row * BM + (((bcol >> 3) ^ swz<CPA>(row)) << 3) + (bcol & 7)]);
#pragma unroll
        for (int kk = 0; kk < 32; kk += 16) {
            // A: 16 pixels x 16 co (transposed load of the [pixel][co] tile)
            uint32_t af[4];
            {
                const int krow = kk + (lane & 7) + ((i4 >> 1) << 3);
                const int ch = (wm * 16 + ((i4 & 1) << 3)) >> 3;
                ldsm_x4_t(smem_u32(tA + krow * BM + ((ch ^ swz<CPA>(krow)) << 3)), af[0], af[1], af[2], af[3]);
            }
            // this lane's pixel of the k16 chunk: block row and column
            const int q = kk + (lane & 7) + ((i4 & 1) << 3);
            const int qr = q >> 3, qc = q & 7;
            const int chb = (wn * 16 + ((i4 >> 1) << 3)) >> 3;
#pragma unroll
            for (int t = 0; t < 9; ++t) {
                const int hrow = (qr + t / 3) * 10 + (qc + t % 3);
                uint32_t bfr[NT][2];
                ldsm_x4_t(smem_u32(tB + hrow * BN + ((chb ^ swz<CPB>(hrow)) << 3)), bfr[0][0], bfr[0][1], bfr[1][0],
                          bfr[1][1]);
#pragma unroll
                for (int nt = 0; nt < NT; ++nt) mma_bf16(acc[t][nt], af, bfr[nt]);
            }
        }
    }
    cp_wait<0>();
    if (bias) {  // the column's partial sums, one atomic per output channel
        __shared__ float bred[NTHREADS];
        bred[tid] = bsum;
        __syncthreads();
        if (bpart == 0 && co0 + bcol < a.cout) {
            float s = 0.0f;
            for (int k = 0; k < BIAS_PARTS; ++k) s += bred[k * BM + bcol];
            atomicAdd(a.db + co0 + bcol, s);
        }
    }

#pragma unroll
    for (int t = 0; t < 9; ++t)
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
            const int ci = ci0 + wn * 16 + nt * 8 + 2 * (lane & 3);
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
                const int co = co0 + wm * 16 + (lane >> 2) + 8 * hh;
                if (co >= a.cout) continue;
                float* d = a.dw + ((size_t)co * 9 + t) * cin + ci;
                atomicAdd(d, acc[t][nt][2 * hh]);
                atomicAdd(d + 1, acc[t][nt][2 * hh + 1]);
            }
        }
}

template <int BM, int BN>
cudaError_t launch_wgrad9(WgradArgs a, cudaStream_t st) {
    const int cin = a.c1 + a.c2;
    const int nblk = a.n * (a.h / 4) * (a.w / 8);
    const int tiles = ((a.cout + BM - 1) / BM) * (cin / BN);
    // about two CTAs per SM: long K ranges keep the atomics few
    int splits = (152 * 2 + tiles - 1) / tiles;
    if (splits > nblk) splits = nblk;
    if (splits < 1) splits = 1;
    const int bps = (nblk + splits - 1) / splits;
    a.pix_per_split = bps;  // blocks per split
    splits = (nblk + bps - 1) / bps;
    dim3 grid((a.cout + BM - 1) / BM, cin / BN, splits);
    k_conv3x3_wgrad9<BM, BN><<<grid, 32 * (BM / 16) * (BN / 16), 0, st>>>(a);
    return cudaGetLastError();
}
}  // namespace

cudaError_t conv3x3(const ConvArgs& a, cudaStream_t st) {
    const int cin = a.c1 + a.c2;
    if (a.n <= 0 || a.h <= 0 || a.w <= 0 || cin % 16 || a.c1 % 16 || a.c2 % 16 || a.cout % 16 ||
        (a.up1 && ((a.h | a.w) & 1)) || (!a.out && !a.out_f32))
        return cudaErrorInvalidValue;
    const bool k32 = (cin % 32 == 0) && (a.c1 % 32 == 0) && (a.c2 % 32 == 0);
    const int bn = (a.cout % 128 == 0) ? 128 : (a.cout % 64 == 0) ? 64 : (a.cout % 32 == 0) ? 32 : 16;
    if (k32) {
        switch (bn) {
            case 128: return launch_conv<32, 128>(a, st);
            case 64: return launch_conv<32, 64>(a, st);
            case 32: return launch_conv<32, 32>(a, st);
            default: return launch_conv<32, 16>(a, st);
        }
    }
    switch (bn) {
        case 128: return launch_conv<16, 128>(a, st);
        case 64: return launch_conv<16, 64>(a, st);
        case 32: return launch_conv<16, 32>(a, st);
        default: return launch_conv<16, 16>(a, st);
    }
}

// VR_DN_WGRAD=per_tap forces the one-tap-per-CTA kernel (for tests and measurements)
static bool wgrad_per_tap() {
    static const bool v = [] {
        const char* e = std::getenv("VR_DN_WGRAD");
        return e && std::strcmp(e, "per_tap") == 0;
    }();
    return v;
}

cudaError_t conv3x3_wgrad(const WgradArgs& a, cudaStream_t st) {
    const int cin = a.c1 + a.c2;
    if (a.n <= 0 || a.h <= 0 || a.w <= 0 || cin % 16 || a.c1 % 8 || a.c2 % 8 || a.cout % 16 ||
        (a.up1 && ((a.h | a.w) & 1)))
        return cudaErrorInvalidValue;
    const bool bn32 = cin % 32 == 0;
    if (a.h % 4 == 0 && a.w % 8 == 0 && !wgrad_per_tap()) {  // the bias gradient rides along
        if (a.cout >= 64) return bn32 ? launch_wgrad9<64, 32>(a, st) : launch_wgrad9<64, 16>(a, st);
        return bn32 ? launch_wgrad9<32, 32>(a, st) : launch_wgrad9<32, 16>(a, st);
    }
    WgradArgs b = a;
    b.db = nullptr;
    const cudaError_t e = (a.cout >= 64) ? (bn32 ? launch_wgrad<64, 32>(b, st) : launch_wgrad<64, 16>(b, st))
                                         : (bn32 ? launch_wgrad<32, 32>(b, st) : launch_wgrad<32, 16>(b, st));
    if (e != cudaSuccess || !a.db) return e;
    return bias_grad(a.dz, a.n * a.h * a.w, a.cout, a.db, st);
}

cudaError_t bias_grad(const bf16* dz, int p, int c, float* db, cudaStream_t st) {
    if (c <= 0 || c > 256 || (256 % c) != 0 || c % 8 || (reinterpret_cast<uintptr_t>(dz) & 15))
        return cudaErrorInvalidValue;
    // about eight blocks per SM, each a multiple of the pixels one step covers
    const int slots = 256 / (c / 8);
    const int target = (p + 152 * 8 - 1) / (152 * 8);
    const int rows = std::max(slots, (target + slots - 1) / slots * slots);
    k_bias_grad<<<(p + rows - 1) / rows, 256, 0, st>>>(dz, p, c, rows, db);
    return cudaGetLastError();
}

cudaError_t avgpool2(const bf16* in, bf16* out, int n, int h, int w, int c, cudaStream_t st) {
    if ((h | w) & 1 || c % 8) return cudaErrorInvalidValue;
    const size_t total = (size_t)n * (h / 2) * (w / 2) * (c / 8);
    k_avgpool2<<<grid_for(total, 256), 256, 0, st>>>(in, out, n, h, w, c);
    return cudaGetLastError();
}

cudaError_t upsample2(const bf16* in, bf16* out, int n, int h, int w, int c, cudaStream_t st) {
    if ((h | w) & 1 || c % 8) return cudaErrorInvalidValue;
    const size_t total = (size_t)n * h * w * (c / 8);
    k_upsample2<<<grid_for(total, 256), 256, 0, st>>>(reinterpret_cast<const uint4*>(in), reinterpret_cast<uint4*>(out),
                                                      n, h, w, c / 8);
    return cudaGetLastError();
}

cudaError_t skip_bwd(const bf16* dcat, int ccat, int coff, const bf16* dpool, const bf16* act, bf16* dz, int n,
                     int h, int w, int c, cudaStream_t st) {
    if ((h | w) & 1 || c % 8 || coff % 8 || ccat % 8) return cudaErrorInvalidValue;
    const size_t total = (size_t)n * h * w * (c / 8);
    k_skip_bwd<<<grid_for(total, 256), 256, 0, st>>>(dcat, ccat, coff, dpool, act, dz, n, h, w, c);
    return cudaGetLastError();
}

cudaError_t up_bwd(const bf16* dcat, int ccat, const bf16* act, bf16* dz, int n, int hc, int wc, int c1,
                   cudaStream_t st) {
    if (c1 % 8 || ccat % 8) return cudaErrorInvalidValue;
    const size_t total = (size_t)n * hc * wc * (c1 / 8);
    k_up_bwd<<<grid_for(total, 256), 256, 0, st>>>(dcat, ccat, act, dz, n, hc, wc, c1);
    return cudaGetLastError();
}

cudaError_t preprocess(const float4* rad, const float4* alb, const float4* nrm, float scale, const float* scales,
                       int n, int img_h, int img_w, int h, int w, bf16* x0, cudaStream_t st) {
    const size_t total = (size_t)n * h * w;
    k_preprocess<<<grid_for(total, 256), 256, 0, st>>>(rad, alb, nrm, scale, scales, n, img_h, img_w, h, w, x0);
    return cudaGetLastError();
}

cudaError_t postprocess(const float* out, int cout, const float4* alb, float scale, const float* scales, int n,
                        int img_h, int img_w, int h, int w, float4* rgba, cudaStream_t st) {
    const size_t total = (size_t)n * img_h * img_w;
    k_postprocess<<<grid_for(total, 256), 256, 0, st>>>(out, cout, alb, scale, scales, n, img_h, img_w, h, w, rgba);
    return cudaGetLastError();
}

cudaError_t loss(const float* out, int cout, const float4* target, const float4* alb, float scale_target,
                 float scale_alb, int n, int h, int w, float inv_count, int kind, bf16* grad, float* loss_sum,
                 cudaStream_t st) {
    const size_t total = (size_t)n * h * w;
    k_loss<<<grid_for(total, 256), 256, 0, st>>>(out, cout, target, alb, scale_target, scale_alb, total, inv_count,
                                                  kind, grad, loss_sum);
    return cudaGetLastError();
}

cudaError_t adam(float* w, float* g, float* m, float* v, size_t n, float lr, float b1, float b2, float eps, float bc1,
                 float bc2, cudaStream_t st) {
    k_adam<<<grid_for(n, 256), 256, 0, st>>>(w, g, m, v, n, lr, b1, b2, eps, bc1, bc2);
    return cudaGetLastError();
}

cudaError_t cast_flip(const float* w32, bf16* w16, bf16* wt16, int cout, int cin, cudaStream_t st) {
    const size_t total = (size_t)cout * 9 * cin;
    k_cast_flip<<<grid_for(total, 256), 256, 0, st>>>(w32, w16, wt16, cout, cin);
    return cudaGetLastError();
}

}  // namespace dn
