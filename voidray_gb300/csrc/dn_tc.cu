// dn_tc.cu — Blackwell-native 3x3 convolution of the denoiser: tcgen05.mma
// with the accumulator in tensor memory (TMEM), operands staged in shared
// memory by TMA (cp.async.bulk.tensor, no multicast), an mbarrier pipeline
// between one producer thread, one MMA-issuing thread and a 4-warp epilogue.
//
// Implicit GEMM per CTA: M = 128 output pixels (an 8 x 16 block of one
// image), N = up to 256 output channels (Cout split into equal tiles of a
// multiple of 16 over blockIdx.y), K = 9 taps x Cin in chunks of BK
// channels.  For tap (dy, dx) and channel chunk c0 the A tile is one 4-D TMA
// box (BK channels x 16 columns x 8 rows x 1 image) of the NHWC activation at
// (c0, x0 + dx, y0 + dy, n); out-of-image coordinates read zeros, which is
// the convolution's zero padding.  The B tile is the (N x BK) slice of the
// [Cout][9 * Cin] weight matrix.  Both land K-major and swizzled (BK = 64:
// 128-byte, 32: 64-byte, 16: 32-byte rows), the layout tcgen05 reads through
// its shared-memory descriptors.  The epilogue reads the fp32 accumulator
// with tcgen05.ld (warp w owns TMEM lanes 32w..32w+31, i.e. pixels), adds
// the bias, applies ReLU and/or a ReLU-backward mask and stores bf16 (or
// fp32) NHWC rows.  With flipped weights the same kernel is the backward-data
// convolution.
//
// Every mbarrier wait is bounded: a wait that runs out sets an error bit in
// the caller's status word and the CTA still drains and frees its TMEM.
//
// k_conv3x3_halo runs shapes of up to 128 output channels per CTA (the tile
// kernel above the wider ones; conv3x3_tc chooses).  Its tile is 16 rows x 8 columns of
// output pixels (M = 128, one 8-pixel row segment per 8-row core matrix).
// Per K chunk it loads one 18 x 10 halo of the input (BK/8 TMA boxes of
// 8 channels x 10 x 18) into the no-swizzle canonical K-major layout
// [channel group][halo pixel][8 channels]: the nine taps are then nine
// descriptor start addresses into the same buffer (start + (dy * 10 + dx) *
// 16 B; leading byte offset = one channel group, stride byte offset = one
// halo row), so each input pixel is staged 1.4 times instead of 9 times.
// When the CTA's weight slice fits it is loaded once and stays resident; the
// CTAs are persistent over tiles, and the accumulator is double-buffered in
// TMEM so that the epilogue of one tile overlaps the MMAs of the next.  Warp
// roles: warp 0 TMA producer, warp 1 MMA issuer, warps 2-5 epilogue.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>

#include "dn_kernels.h"

namespace dn {
namespace {

constexpr int TC_THREADS = 128;
constexpr int TC_STAGES = 4;
constexpr uint32_t WAIT_LIMIT = 1u << 24;  // iterations of a bounded mbarrier wait

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// true when the phase with this parity has completed; gives up after WAIT_LIMIT polls
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    const uint32_t a = smem_addr(bar);
    for (uint32_t it = 0; it < WAIT_LIMIT; ++it) {
        uint32_t done = 0;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2,
                                            int c3) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];\n" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];\n" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(smem_addr(bar))
        : "memory");
}

// Shared-memory matrix descriptor of a K-major, swizzled operand whose rows
// are `row_bytes` (= the swizzle span) long: start address, leading byte
// offset 16 (unused for swizzled K-major), stride byte offset = 8 rows,
// descriptor version 1, swizzle mode.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t row_bytes) {
    const uint64_t swz = row_bytes == 128 ? 2ull : row_bytes == 64 ? 4ull : 6ull;
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)(16u >> 4) << 16;
    d |= (uint64_t)((8u * row_bytes) >> 4) << 32;
    d |= 1ull << 46;
    d |= swz << 61;
    return d;
}

// Descriptor of a K-major operand in the no-swizzle canonical layout: core
// matrices of 8 rows x 16 B stored contiguously; `lbo` = byte distance of
// core matrices adjacent in K, `sbo` = of core matrices adjacent in M/N.
__device__ __forceinline__ uint64_t smem_desc_noswz(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo & 0x3FFFFu) >> 4) << 16;
    d |= (uint64_t)((sbo & 0x3FFFFu) >> 4) << 32;
    d |= 1ull << 46;
    return d;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                     smem_addr(bar))
                 : "memory");
}

// Instruction descriptor, kind::f16: fp32 accumulator, bf16 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t instr_desc(uint32_t m, uint32_t n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

struct TcArgs {
    const float* bias;
    const bf16* mask;  // zero the output where mask <= 0 (ReLU backward), [P][cout], or null
    bf16* out;
    float* out_f32;
    uint32_t* status;
    int n, h, w;
    int c1, cin, cout;
    int ntile;        // output channels per CTA (16..256; cout is a multiple)
    int bk;           // channels per K chunk (16, 32, 64)
    int relu;
    int tiles_x, tiles_y;
};

__global__ void __launch_bounds__(TC_THREADS, 1)
    k_conv3x3_tc(const __grid_constant__ CUtensorMap map_a1, const __grid_constant__ CUtensorMap map_a2,
                 const __grid_constant__ CUtensorMap map_b, const TcArgs a) {
    extern __shared__ __align__(1024) uint8_t dsmem[];
    __shared__ uint64_t full_bar[TC_STAGES], empty_bar[TC_STAGES], done_bar;
    __shared__ uint32_t tmem_base;
    // 1024-byte aligned stage buffers (the 128-byte swizzle atom is 8 x 128 B)
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(dsmem) + 1023) & ~uintptr_t(1023));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int N = a.ntile;              // MMA N: this CTA's output channels
    const int n0 = blockIdx.y * N;      // first output channel of this CTA
    const uint32_t a_bytes = 128u * a.bk * 2u, b_bytes = (uint32_t)N * a.bk * 2u;
    const uint32_t stage_bytes = a_bytes + b_bytes;
    const uint32_t tmem_cols = N <= 32 ? 32u : N <= 64 ? 64u : N <= 128 ? 128u : 256u;

    int tile = blockIdx.x;
    const int tx = tile % a.tiles_x;
    tile /= a.tiles_x;
    const int ty = tile % a.tiles_y;
    const int img = tile / a.tiles_y;
    const int x0 = tx * 16, y0 = ty * 8;

    if (threadIdx.x == 0) {
        for (int s = 0; s < TC_STAGES; ++s) {
            mbar_init(&full_bar[s], 1);
            mbar_init(&empty_bar[s], 1);
        }
        mbar_init(&done_bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_addr(&tmem_base)),
                     "r"(tmem_cols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = tmem_base;

    const int kc = a.cin / a.bk;
    const int nk = 9 * kc;
    bool ok = true;

    if (warp == 0 && lane == 0) {
        // producer: TMA loads of the A (activation box) and B (weight slice) tiles
        for (int kt = 0; kt < nk; ++kt) {
            const int s = kt % TC_STAGES;
            if (kt >= TC_STAGES && !mbar_wait(&empty_bar[s], ((kt / TC_STAGES) & 1) ^ 1)) {
                ok = false;
                break;
            }
            const int tap = kt / kc, c0 = (kt % kc) * a.bk;
            const int dy = tap / 3 - 1, dx = tap % 3 - 1;
            uint8_t* sa = smem + (size_t)s * stage_bytes;
            uint8_t* sb = sa + a_bytes;
            mbar_expect_tx(&full_bar[s], stage_bytes);
            if (c0 < a.c1) tma_load_4d(sa, &map_a1, &full_bar[s], c0, x0 + dx, y0 + dy, img);
            else tma_load_4d(sa, &map_a2, &full_bar[s], c0 - a.c1, x0 + dx, y0 + dy, img);
            tma_load_2d(sb, &map_b, &full_bar[s], tap * a.cin + c0, n0);
        }
    } else if (warp == 1 && lane == 0) {
        // MMA issuer: BK/16 tcgen05.mma per stage, accumulating in TMEM
        const uint32_t idesc = instr_desc(128, (uint32_t)N);
        const uint32_t row_bytes = (uint32_t)a.bk * 2u;
        for (int kt = 0; kt < nk; ++kt) {
            const int s = kt % TC_STAGES;
            if (!mbar_wait(&full_bar[s], (kt / TC_STAGES) & 1)) {
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t sa = smem_addr(smem + (size_t)s * stage_bytes);
            const uint32_t sb = sa + a_bytes;
            for (int kk = 0; kk < a.bk / 16; ++kk) {
                const uint64_t da = smem_desc(sa + kk * 32, row_bytes);
                const uint64_t db = smem_desc(sb + kk * 32, row_bytes);
                const uint32_t acc = (kt > 0 || kk > 0) ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(da), "l"(db), "r"(idesc), "r"(acc));
            }
            // frees the stage once these MMAs have read it
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             smem_addr(&empty_bar[s]))
                         : "memory");
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                         smem_addr(&done_bar))
                     : "memory");
    }
    if (!ok && a.status) atomicOr(a.status, 1u);
    __syncwarp();

    // epilogue: all four warps wait for the accumulator
    const bool acc_ready = mbar_wait(&done_bar, 0);
    if (!acc_ready && lane == 0 && a.status) atomicOr(a.status, 2u);
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const int m = warp * 32 + lane;  // TMEM lane = pixel of the 8 x 16 block
    const int y = y0 + (m >> 4), x = x0 + (m & 15);
    const bool in_img = y < a.h && x < a.w;
    const size_t pix = ((size_t)img * a.h + y) * a.w + x;
    for (int c0 = 0; c0 < N; c0 += 16) {
        uint32_t r[16];
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
            "[%16];\n"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
        if (!in_img || !acc_ready) continue;
        float v[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            v[j] = __uint_as_float(r[j]) + (a.bias ? a.bias[n0 + c0 + j] : 0.0f);
            if (a.relu) v[j] = fmaxf(v[j], 0.0f);
        }
        const size_t o0 = pix * (size_t)a.cout + n0 + c0;
        if (a.mask) {
            union {
                uint4 u[2];
                bf16 h[16];
            } mk;
            const uint4* mp = reinterpret_cast<const uint4*>(a.mask + o0);
            mk.u[0] = mp[0];
            mk.u[1] = mp[1];
#pragma unroll
            for (int j = 0; j < 16; ++j)
                if (!(__bfloat162float(mk.h[j]) > 0.0f)) v[j] = 0.0f;
        }
        if (a.out_f32) {
            float4* o = reinterpret_cast<float4*>(a.out_f32 + o0);
#pragma unroll
            for (int j = 0; j < 4; ++j) o[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
        } else {
            union {
                uint4 u[2];
                bf16 h[16];
            } pk;
#pragma unroll
            for (int j = 0; j < 16; ++j) pk.h[j] = __float2bfloat16_rn(v[j]);
            uint4* o = reinterpret_cast<uint4*>(a.out + o0);
            o[0] = pk.u[0];
            o[1] = pk.u[1];
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(tmem_cols));
    }
}


// ---------------------------------------------------------- halo variant --
constexpr int HALO_THREADS = 192;
constexpr int HALO_MAX_STAGES = 4;
constexpr int HALO_W = 10, HALO_H = 18, HALO_PIX = HALO_W * HALO_H;  // 16 x 8 outputs + 1-pixel border
constexpr uint32_t HALO_BOX_BYTES = HALO_PIX * 16u;                   // one 8-channel group: 2880 B
// distance between channel groups: a TMA tensor copy writes to a 128-byte
// aligned shared-memory address, so each group starts on a 128-byte boundary
constexpr uint32_t HALO_GROUP_BYTES = (HALO_BOX_BYTES + 127u) & ~127u;  // 2944 B
static_assert(HALO_GROUP_BYTES % 128u == 0, "TMA destinations are 128-byte aligned");

struct HaloArgs {
    const float* bias;
    const bf16* mask;
    bf16* out;
    float* out_f32;
    uint32_t* status;
    int n, h, w;
    int c1, cin, cout;
    int ntile, bk, stages, resident;
    int relu;
    int tiles_x, tiles_y, ntiles;
    uint32_t a_stage;  // bytes per A stage (bk / 8 channel groups of a halo, rounded to 1024)
    uint32_t b_box;    // bytes per weight box (ntile x bk, rounded to 1024)
    uint32_t b_off;    // offset of the weight region
};

// bias, ReLU, ReLU-backward mask and the bf16 / fp32 store of 16 accumulator
// columns of one pixel
__device__ __forceinline__ void store16(const HaloArgs& a, const uint32_t* r, size_t pix, int ch) {
    float v[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        v[j] = __uint_as_float(r[j]) + (a.bias ? a.bias[ch + j] : 0.0f);
        if (a.relu) v[j] = fmaxf(v[j], 0.0f);
    }
    const size_t o0 = pix * (size_t)a.cout + ch;
    if (a.mask) {
        union {
            uint4 u[2];
            bf16 h[16];
        } mk;
        const uint4* mp = reinterpret_cast<const uint4*>(a.mask + o0);
        mk.u[0] = mp[0];
        mk.u[1] = mp[1];
#pragma unroll
        for (int j = 0; j < 16; ++j)
            if (!(__bfloat162float(mk.h[j]) > 0.0f)) v[j] = 0.0f;
    }
    if (a.out_f32) {
        float4* o = reinterpret_cast<float4*>(a.out_f32 + o0);
#pragma unroll
        for (int j = 0; j < 4; ++j) o[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
    } else {
        union {
            uint4 u[2];
            bf16 h[16];
        } pk;
#pragma unroll
        for (int j = 0; j < 16; ++j) pk.h[j] = __float2bfloat16_rn(v[j]);
        uint4* o = reinterpret_cast<uint4*>(a.out + o0);
        o[0] = pk.u[0];
        o[1] = pk.u[1];
    }
}

__device__ __forceinline__ void halo_tile(const HaloArgs& a, int t, int& img, int& y0, int& x0) {
    x0 = (t % a.tiles_x) * 8;
    t /= a.tiles_x;
    y0 = (t % a.tiles_y) * 16;
    img = t / a.tiles_y;
}

__global__ void __launch_bounds__(HALO_THREADS, 1)
    k_conv3x3_halo(const __grid_constant__ CUtensorMap map_a1, const __grid_constant__ CUtensorMap map_a2,
                   const __grid_constant__ CUtensorMap map_b, const HaloArgs a) {
    extern __shared__ __align__(1024) uint8_t dsmem[];
    __shared__ uint64_t full_bar[HALO_MAX_STAGES], empty_bar[HALO_MAX_STAGES];
    __shared__ uint64_t acc_full[2], acc_empty[2], w_bar, mma_done;
    __shared__ uint32_t tmem_base;
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(dsmem) + 1023) & ~uintptr_t(1023));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int N = a.ntile;
    const int n0 = blockIdx.y * N;
    const int S = a.stages;
    const int KG = a.cin / a.bk;  // K chunks per tile
    const uint32_t ncols = N <= 32 ? 32u : N <= 64 ? 64u : N <= 128 ? 128u : 256u;
    const uint32_t tmem_cols = 2u * ncols;  // two accumulators
    const uint32_t wbox_bytes = (uint32_t)N * a.bk * 2u;

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(&full_bar[s], 1);
            mbar_init(&empty_bar[s], 1);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(&acc_full[i], 1);
            mbar_init(&acc_empty[i], 4);
        }
        mbar_init(&w_bar, 1);
        mbar_init(&mma_done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_addr(&tmem_base)),
                     "r"(tmem_cols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = tmem_base;
    bool ok = true;

    if (warp == 0 && lane == 0) {
        // ------------------------------------------------ TMA producer
        if (a.resident) {
            mbar_expect_tx(&w_bar, (uint32_t)KG * 9u * wbox_bytes);
            for (int kg = 0; kg < KG; ++kg)
                for (int tap = 0; tap < 9; ++tap)
                    tma_load_2d(smem + a.b_off + (size_t)(kg * 9 + tap) * a.b_box, &map_b, &w_bar,
                                tap * a.cin + kg * a.bk, n0);
        }
        const uint32_t a_tx = (uint32_t)(a.bk / 8) * HALO_BOX_BYTES;
        const uint32_t tx = a_tx + (a.resident ? 0u : 9u * wbox_bytes);
        uint32_t it = 0;
        for (int t = blockIdx.x; t < a.ntiles && ok; t += gridDim.x) {
            int img, y0, x0;
            halo_tile(a, t, img, y0, x0);
            for (int kg = 0; kg < KG; ++kg, ++it) {
                const int s = (int)(it % (uint32_t)S);
                if (it >= (uint32_t)S && !mbar_wait(&empty_bar[s], ((it / S) & 1) ^ 1)) {
                    ok = false;
                    break;
                }
                uint8_t* sa = smem + (size_t)s * a.a_stage;
                mbar_expect_tx(&full_bar[s], tx);
                const int c0 = kg * a.bk;
                for (int g = 0; g < a.bk / 8; ++g) {
                    const int cc = c0 + 8 * g;
                    if (cc < a.c1) tma_load_4d(sa + g * HALO_GROUP_BYTES, &map_a1, &full_bar[s], cc, x0 - 1, y0 - 1, img);
                    else tma_load_4d(sa + g * HALO_GROUP_BYTES, &map_a2, &full_bar[s], cc - a.c1, x0 - 1, y0 - 1, img);
                }
                if (!a.resident)
                    for (int tap = 0; tap < 9; ++tap)
                        tma_load_2d(smem + a.b_off + (size_t)(s * 9 + tap) * a.b_box, &map_b, &full_bar[s],
                                    tap * a.cin + c0, n0);
            }
        }
        // no copy may still be in flight when the CTA exits: wait for the last
        // phase of every stage this thread filled (bounded)
        const uint32_t first = it > (uint32_t)S ? it - S : 0u;
        for (uint32_t j = first; j < it; ++j)
            if (!mbar_wait(&full_bar[j % S], (j / S) & 1)) ok = false;
        if (a.resident && !mbar_wait(&w_bar, 0)) ok = false;
    } else if (warp == 1 && lane == 0) {
        // ------------------------------------------------ MMA issuer
        const uint32_t idesc = instr_desc(128, (uint32_t)N);
        const uint32_t row_bytes = (uint32_t)a.bk * 2u;
        if (a.resident && !mbar_wait(&w_bar, 0)) ok = false;
        uint32_t it = 0;
        int local = 0;
        for (int t = blockIdx.x; t < a.ntiles && ok; t += gridDim.x, ++local) {
            const int acc = local & 1;
            if (local >= 2 && !mbar_wait(&acc_empty[acc], ((local >> 1) & 1) ^ 1)) {
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t d_tmem = tmem + (uint32_t)acc * ncols;
            for (int kg = 0; kg < KG; ++kg, ++it) {
                const int s = (int)(it % (uint32_t)S);
                if (!mbar_wait(&full_bar[s], (it / S) & 1)) {
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const uint32_t sa = smem_addr(smem + (size_t)s * a.a_stage);
                for (int tap = 0; tap < 9; ++tap) {
                    const int dy = tap / 3, dx = tap % 3;
                    const uint32_t sb =
                        smem_addr(smem + a.b_off + (size_t)((a.resident ? kg : s) * 9 + tap) * a.b_box);
                    for (int kk = 0; kk < a.bk / 16; ++kk) {
                        const uint64_t da = smem_desc_noswz(sa + (uint32_t)(dy * HALO_W + dx) * 16u +
                                                                (uint32_t)kk * 2u * HALO_GROUP_BYTES,
                                                            HALO_GROUP_BYTES, HALO_W * 16u);
                        const uint64_t db = smem_desc(sb + kk * 32, row_bytes);
                        const uint32_t accum = (kg > 0 || tap > 0 || kk > 0) ? 1u : 0u;
                        asm volatile(
                            "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
                            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
                            "l"(da), "l"(db), "r"(idesc), "r"(accum));
                    }
                }
                mma_commit(&empty_bar[s]);  // frees the stage once these MMAs have read it
            }
            if (!ok) break;
            mma_commit(&acc_full[acc]);
        }
        mma_commit(&mma_done);  // arrives when every MMA above has completed
    } else if (warp >= 2) {
        // ------------------------------------------------ epilogue (warps 2-5)
        const int q = warp & 3;  // TMEM lane quadrant this warp may read
        const int m = q * 32 + lane;
        int local = 0;
        for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x, ++local) {
            const int acc = local & 1;
            if (!mbar_wait(&acc_full[acc], (local >> 1) & 1)) {
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            int img, y0, x0;
            halo_tile(a, t, img, y0, x0);
            const int y = y0 + (m >> 3), x = x0 + (m & 7);
            const bool in_img = y < a.h && x < a.w;
            const size_t pix = ((size_t)img * a.h + y) * a.w + x;
            for (int c0 = 0; c0 < N; c0 += 16) {
                uint32_t r[16];
                const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)acc * ncols + (uint32_t)c0;
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                    "[%16];\n"
                    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                      "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                      "=r"(r[15])
                    : "r"(taddr));
                asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
                if (in_img) store16(a, r, pix, n0 + c0);
            }
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(&acc_empty[acc]);
        }
    }
    if (!ok && a.status) atomicOr(a.status, 1u);
    __syncwarp();
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        // every MMA has completed before the accumulator is freed (bounded wait)
        const bool drained = mbar_wait(&mma_done, 0);
        if (!drained && lane == 0 && a.status) atomicOr(a.status, 2u);
        __syncwarp();
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(tmem_cols));
    }
}

// ------------------------------------------------------------- host side --
using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
    static EncodeTiled fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(p);
        else
            cudaGetLastError();
    }
    return fn;
}

CUtensorMapSwizzle swizzle_for(int bk) {
    return bk == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : bk == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B;
}

// NHWC activation (c channels) as a 4-D map with boxes of bk x 16 x 8 x 1
bool encode_act(CUtensorMap* m, const bf16* p, int n, int h, int w, int c, int bk) {
    const cuuint64_t dims[4] = {(cuuint64_t)c, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)n};
    const cuuint64_t strides[3] = {(cuuint64_t)c * 2, (cuuint64_t)c * w * 2, (cuuint64_t)c * w * h * 2};
    const cuuint32_t box[4] = {(cuuint32_t)bk, 16, 8, 1};
    const cuuint32_t es[4] = {1, 1, 1, 1};
    return encode_fn()(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<bf16*>(p), dims, strides, box, es,
                       CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_for(bk), CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                       CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// NHWC activation as a 4-D map with halo boxes of 8 channels x 10 x 18 x 1,
// unswizzled: a box lands as [18][10][8 channels], one core-matrix row per pixel
bool encode_act_halo(CUtensorMap* m, const bf16* p, int n, int h, int w, int c) {
    const cuuint64_t dims[4] = {(cuuint64_t)c, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)n};
    const cuuint64_t strides[3] = {(cuuint64_t)c * 2, (cuuint64_t)c * w * 2, (cuuint64_t)c * w * h * 2};
    const cuuint32_t box[4] = {8, (cuuint32_t)HALO_W, (cuuint32_t)HALO_H, 1};
    const cuuint32_t es[4] = {1, 1, 1, 1};
    return encode_fn()(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<bf16*>(p), dims, strides, box, es,
                       CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                       CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// weights [cout][9 * cin] as a 2-D map with boxes of bk x ntile
bool encode_wgt(CUtensorMap* m, const bf16* p, int cout, int cin, int bk, int ntile) {
    const cuuint64_t dims[2] = {(cuuint64_t)9 * cin, (cuuint64_t)cout};
    const cuuint64_t strides[1] = {(cuuint64_t)9 * cin * 2};
    const cuuint32_t box[2] = {(cuuint32_t)bk, (cuuint32_t)ntile};
    const cuuint32_t es[2] = {1, 1};
    return encode_fn()(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<bf16*>(p), dims, strides, box, es,
                       CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_for(bk), CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                       CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace

// output channels per CTA: all of them up to 256, else the largest multiple
// of 16 up to 256 that divides cout
int ntile_for(int cout) {
    if (cout <= 256) return cout;
    for (int t = 256; t >= 16; t -= 16)
        if (cout % t == 0) return t;
    return 0;
}

bool conv3x3_tc_supported(const ConvArgs& a) {
    const int cin = a.c1 + a.c2;
    if (a.up1 || !encode_fn()) return false;
    if (a.cout < 16 || a.cout % 16 || !ntile_for(a.cout)) return false;
    if (a.mask && !aligned16(a.mask)) return false;
    if (cin % 16 || a.c1 % 16 || a.c2 % 16) return false;
    if (!aligned16(a.src1) || (a.c2 && !aligned16(a.src2)) || !aligned16(a.weight)) return false;
    return true;
}

namespace {

constexpr size_t HALO_RESIDENT_MAX = 128 * 1024;

// Dynamic shared memory a halo plan may use.  Up to 64 output channels per
// CTA a 110 KB plan (two CTAs per SM) beat the 200 KB one (one CTA per SM)
// by 20-27% per layer at 1080p; with 128 the larger chunks of the 200 KB plan
// won by 5-10%.  VR_DN_HALO_SMEM_KB overrides both, for measurements.
size_t halo_smem_budget(int ntile) {
    static const long forced = [] {
        const char* e = std::getenv("VR_DN_HALO_SMEM_KB");
        const long kb = e ? std::strtol(e, nullptr, 10) : 0;
        return (kb >= 32 && kb <= 200) ? kb : 0L;
    }();
    if (forced) return (size_t)forced * 1024;
    return (size_t)(ntile <= 64 ? 110 : 200) * 1024;
}

size_t round1k(size_t x) { return (x + 1023) & ~size_t(1023); }

struct HaloPlan {
    int bk = 0, stages = 0, resident = 0;
    size_t a_stage = 0, b_box = 0, b_off = 0, smem = 0;
};

// chunk size, stage count and weight residency within the shared-memory budget:
// resident weights when they fit in 128 KB with at least two A stages beside
// them, else streamed weights with the largest chunk that leaves two stages
HaloPlan plan_halo(int c1, int c2, int ntile) {
    const int cin = c1 + c2;
    const size_t budget = halo_smem_budget(ntile);
    HaloPlan p;
    for (int bk = 64; bk >= 16; bk >>= 1) {
        if (c1 % bk || c2 % bk) continue;
        const size_t a_stage = round1k((size_t)(bk / 8) * HALO_GROUP_BYTES);
        const size_t b_box = round1k((size_t)ntile * bk * 2);
        const size_t w = (size_t)(cin / bk) * 9 * b_box;
        if (w <= HALO_RESIDENT_MAX && w + 2 * a_stage <= budget) {
            p.bk = bk;
            p.resident = 1;
            p.stages = (int)std::min<size_t>(HALO_MAX_STAGES, (budget - w) / a_stage);
            p.a_stage = a_stage;
            p.b_box = b_box;
            p.b_off = (size_t)p.stages * a_stage;
            p.smem = p.b_off + w + 1024;
            return p;
        }
    }
    for (int bk = 64; bk >= 16; bk >>= 1) {
        if (c1 % bk || c2 % bk) continue;
        const size_t a_stage = round1k((size_t)(bk / 8) * HALO_GROUP_BYTES);
        const size_t b_box = round1k((size_t)ntile * bk * 2);
        const size_t stage = a_stage + 9 * b_box;
        if (2 * stage > budget) continue;
        p.bk = bk;
        p.resident = 0;
        p.stages = (int)std::min<size_t>(HALO_MAX_STAGES, budget / stage);
        p.a_stage = a_stage;
        p.b_box = b_box;
        p.b_off = (size_t)p.stages * a_stage;
        p.smem = p.b_off + (size_t)p.stages * 9 * b_box + 1024;
        return p;
    }
    return p;
}

// Variant per shape, from per-layer launch lists of the 1080p forward pass on
// GB300: with several CTAs per SM the halo kernel is 1.4-2.3x faster than the
// tile kernel up to 128 output channels per CTA; at 256 the streamed weights
// dominate and the tile kernel is faster.  VR_DN_TC_VARIANT=tile / halo forces
// one variant.
bool use_tile_variant(int ntile) {
    static const int forced = [] {
        const char* e = std::getenv("VR_DN_TC_VARIANT");
        if (e && std::strcmp(e, "tile") == 0) return 1;
        if (e && std::strcmp(e, "halo") == 0) return 2;
        return 0;
    }();
    if (forced) return forced == 1;
    return ntile > 128;
}

cudaError_t conv3x3_halo(const ConvArgs& a, uint32_t* status, cudaStream_t st) {
    const int cin = a.c1 + a.c2;
    const int ntile = ntile_for(a.cout);
    const HaloPlan pl = plan_halo(a.c1, a.c2, ntile);
    if (!pl.bk) return cudaErrorNotSupported;  // no plan within the budget: the caller runs the tile kernel
    CUtensorMap ma1, ma2, mb;
    std::memset(&ma2, 0, sizeof ma2);
    if (!encode_act_halo(&ma1, a.src1, a.n, a.h, a.w, a.c1)) return cudaErrorInvalidValue;
    if (a.c2 && !encode_act_halo(&ma2, a.src2, a.n, a.h, a.w, a.c2)) return cudaErrorInvalidValue;
    if (!a.c2) ma2 = ma1;
    if (!encode_wgt(&mb, a.weight, a.cout, cin, pl.bk, ntile)) return cudaErrorInvalidValue;
    HaloArgs t{};
    t.bias = a.bias;
    t.mask = a.mask;
    t.out = a.out;
    t.out_f32 = a.out_f32;
    t.status = status;
    t.n = a.n;
    t.h = a.h;
    t.w = a.w;
    t.c1 = a.c1;
    t.cin = cin;
    t.cout = a.cout;
    t.ntile = ntile;
    t.bk = pl.bk;
    t.stages = pl.stages;
    t.resident = pl.resident;
    t.relu = a.relu;
    t.tiles_x = (a.w + 7) / 8;
    t.tiles_y = (a.h + 15) / 16;
    t.ntiles = t.tiles_x * t.tiles_y * a.n;
    t.a_stage = (uint32_t)pl.a_stage;
    t.b_box = (uint32_t)pl.b_box;
    t.b_off = (uint32_t)pl.b_off;
    static size_t configured = 0;
    if (pl.smem > configured) {
        cudaError_t e = cudaFuncSetAttribute(k_conv3x3_halo, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem);
        if (e != cudaSuccess) return e;
        // the whole unified L1 / shared array as shared memory, so that several
        // CTAs of the smaller plans share an SM (their pipelines are latency-bound)
        e = cudaFuncSetAttribute(k_conv3x3_halo, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 cudaSharedmemCarveoutMaxShared);
        if (e != cudaSuccess) return e;
        configured = pl.smem;
    }
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 1;
    }
    // resident CTAs per SM, from the kernel's registers and static shared memory
    // and the SM's shared memory (the maximum carveout is requested above);
    // any grid is correct (CTAs stride over the tiles), this only sizes it
    static int regs = -1, static_smem = 0, sm_smem = 0, reserved = 0;
    if (regs < 0) {
        cudaFuncAttributes fa{};
        int dev = 0;
        cudaGetDevice(&dev);
        regs = cudaFuncGetAttributes(&fa, k_conv3x3_halo) == cudaSuccess ? fa.numRegs : 0;
        static_smem = (int)fa.sharedSizeBytes;
        if (cudaDeviceGetAttribute(&sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess)
            sm_smem = 0;
        if (cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev) != cudaSuccess)
            reserved = 0;
        cudaGetLastError();
    }
    int per_sm = 1;
    if (regs > 0 && sm_smem > 0) {
        const int by_smem = sm_smem / (int)(pl.smem + (size_t)static_smem + (size_t)reserved);
        const int regs_per_warp = ((regs + 7) / 8) * 8 * 32;
        const int by_regs = 65536 / (regs_per_warp * (HALO_THREADS / 32));
        per_sm = std::max(1, std::min({by_smem, by_regs, 2048 / HALO_THREADS}));
    }
    const int ncols = ntile <= 32 ? 32 : ntile <= 64 ? 64 : ntile <= 128 ? 128 : 256;
    per_sm = std::min(per_sm, 512 / (2 * ncols));  // the accumulators of co-resident CTAs fit in TMEM
    const int ny = a.cout / ntile;
    const int gx = std::max(1, std::min(t.ntiles, (sms * per_sm + ny - 1) / ny));
    k_conv3x3_halo<<<dim3((unsigned)gx, (unsigned)ny), HALO_THREADS, pl.smem, st>>>(ma1, ma2, mb, t);
    return cudaGetLastError();
}

}  // namespace

cudaError_t conv3x3_tc(const ConvArgs& a, uint32_t* status, cudaStream_t st) {
    if (!conv3x3_tc_supported(a)) return cudaErrorInvalidValue;
    if (!use_tile_variant(ntile_for(a.cout))) {
        const cudaError_t e = conv3x3_halo(a, status, st);
        if (e != cudaErrorNotSupported) return e;
    }
    const int cin = a.c1 + a.c2;
    // largest chunk that divides both sources (a chunk never straddles them)
    int bk = 64;
    while (bk > 16 && ((a.c1 % bk) || (a.c2 % bk))) bk >>= 1;
    CUtensorMap ma1, ma2, mb;
    std::memset(&ma2, 0, sizeof ma2);
    if (!encode_act(&ma1, a.src1, a.n, a.h, a.w, a.c1, bk)) return cudaErrorInvalidValue;
    if (a.c2 && !encode_act(&ma2, a.src2, a.n, a.h, a.w, a.c2, bk)) return cudaErrorInvalidValue;
    if (!a.c2) ma2 = ma1;
    const int ntile = ntile_for(a.cout);
    if (!encode_wgt(&mb, a.weight, a.cout, cin, bk, ntile)) return cudaErrorInvalidValue;
    TcArgs t{};
    t.bias = a.bias;
    t.mask = a.mask;
    t.ntile = ntile;
    t.out = a.out;
    t.out_f32 = a.out_f32;
    t.status = status;
    t.n = a.n;
    t.h = a.h;
    t.w = a.w;
    t.c1 = a.c1;
    t.cin = cin;
    t.cout = a.cout;
    t.bk = bk;
    t.relu = a.relu;
    t.tiles_x = (a.w + 15) / 16;
    t.tiles_y = (a.h + 7) / 8;
    const size_t stage = (size_t)128 * bk * 2 + (size_t)ntile * bk * 2;
    const size_t smem = TC_STAGES * stage + 1024;
    static size_t configured = 0;
    if (smem > configured) {
        cudaError_t e = cudaFuncSetAttribute(k_conv3x3_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        e = cudaFuncSetAttribute(k_conv3x3_tc, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 cudaSharedmemCarveoutMaxShared);
        if (e != cudaSuccess) return e;
        configured = smem;
    }
    const dim3 grid((unsigned)(t.tiles_x * t.tiles_y * a.n), (unsigned)(a.cout / ntile));
    k_conv3x3_tc<<<grid, TC_THREADS, smem, st>>>(ma1, ma2, mb, t);
    return cudaGetLastError();
}

}  // namespace dn
