// vr_serve.cu — error statistics of a serving pass: one launch computes, for
// every job of the pass and every 16 x 16 pixel tile, the half-buffer
// variance term of the plain estimate and the five moments of the denoised
// blend prediction, in fp64, reduced in a fixed order.
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/voidray_gpu.h"
#include "vr_host.h"

namespace {

constexpr int TILE = VR_STATS_TILE;
constexpr int THREADS = TILE * TILE;
constexpr double EPS_REL = 1e-2;

struct StatsJob {
    const float4* a;
    const float4* b;
    const float4* da;
    const float4* db;
    double na, nb;
    uint32_t w, h, tiles_x, tiles;
    uint64_t out_off;
    uint32_t first_block;  // prefix over jobs of their tile counts
};

struct StatsTable {
    StatsJob job[VR_STATS_MAX_JOBS];
    uint32_t count;
};

__device__ __forceinline__ double block_sum(double v, double* red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < THREADS / 32; ++i) s += red[i];
    return s;  // valid in thread 0
}

__global__ void __launch_bounds__(THREADS) k_serve_stats(const __grid_constant__ StatsTable t, double* out) {
    __shared__ double red[THREADS / 32];
    // the job of this block: last job whose first block is <= blockIdx.x
    uint32_t j = 0;
    for (uint32_t i = 1; i < t.count; ++i)
        if (t.job[i].first_block <= blockIdx.x) j = i;
    const StatsJob& J = t.job[j];
    const uint32_t tile = blockIdx.x - J.first_block;
    const uint32_t tx = tile % J.tiles_x, ty = tile / J.tiles_x;
    const uint32_t x = tx * TILE + (threadIdx.x % TILE), y = ty * TILE + (threadIdx.x / TILE);
    const bool in = x < J.w && y < J.h;
    const double n = J.na + J.nb, wv = J.na * J.nb / (n * n);
    double v[6] = {0, 0, 0, 0, 0, 0};
    if (in) {
        const size_t p = (size_t)y * J.w + x;
        const float4 A = J.a[p], B = J.b[p];
        const double As[3] = {A.x, A.y, A.z}, Bs[3] = {B.x, B.y, B.z};
        float4 DA = make_float4(0, 0, 0, 0), DB = DA;
        if (J.da) {
            DA = J.da[p];
            DB = J.db[p];
        }
        const double Da[3] = {DA.x, DA.y, DA.z}, Db[3] = {DB.x, DB.y, DB.z};
        for (int c = 0; c < 3; ++c) {
            const double a = As[c] / J.na, b = Bs[c] / J.nb;
            const double m = (As[c] + Bs[c]) / n;
            const double d = m * m + EPS_REL;
            const double ab = a - b;
            v[0] += ab * ab * wv / d;
            if (J.da) {
                const double dd = Da[c] - Db[c];
                v[1] += ab * ab / d;
                v[2] += (Da[c] - b) * (Da[c] - b) / d;
                v[3] += (Db[c] - a) * (Db[c] - a) / d;
                v[4] += dd * dd / d;
                v[5] += dd * ab / d;
            }
        }
    }
    const uint32_t vx = min(J.w - tx * TILE, (uint32_t)TILE), vy = min(J.h - ty * TILE, (uint32_t)TILE);
    const double cnt = 3.0 * vx * vy;
    const int nk = J.da ? 6 : 1;
    for (int k = 0; k < nk; ++k) {
        const double s = block_sum(v[k], red);
        if (threadIdx.x == 0) out[J.out_off + (uint64_t)k * J.tiles + tile] = k == 0 ? s : s / cnt;
    }
}

// out[i] = a[i] + b[i] over the float4 elements of `pairs` buffer pairs
// (the full sums of a job's radiance, albedo and normal halves).
struct SumPairs {
    const float4* a[3];
    const float4* b[3];
    float4* out[3];
};
__global__ void k_serve_sum(const SumPairs sp, uint32_t pairs, uint64_t n) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint32_t k = 0; k < pairs; ++k)
        for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
            const float4 x = sp.a[k][i], y = sp.b[k][i];
            sp.out[k][i] = make_float4(x.x + y.x, x.y + y.y, x.z + y.z, x.w + y.w);
        }
}

// rgb[p] = alpha D[p] + (1 - alpha) (A[p] + B[p]) / n, alpha the weight of
// p's TILE x TILE tile (0 everywhere without a denoised image).
__global__ void k_serve_blend(const float4* __restrict__ a, const float4* __restrict__ b, float inv_n,
                              const float4* __restrict__ d, const float* __restrict__ alpha, uint32_t w, uint32_t h,
                              float* __restrict__ rgb) {
    const uint64_t np = (uint64_t)w * h, stride = (uint64_t)gridDim.x * blockDim.x;
    const uint32_t tiles_x = (w + TILE - 1) / TILE;
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < np; p += stride) {
        const float4 x = a[p], y = b[p];
        float r = (x.x + y.x) * inv_n, g = (x.y + y.y) * inv_n, bl = (x.z + y.z) * inv_n;
        if (d) {
            const uint32_t px = (uint32_t)(p % w), py = (uint32_t)(p / w);
            const float al = alpha[(py / TILE) * tiles_x + px / TILE];
            if (al != 0.0f) {
                const float4 dv = d[p];
                r = al * dv.x + (1.0f - al) * r;
                g = al * dv.y + (1.0f - al) * g;
                bl = al * dv.z + (1.0f - al) * bl;
            }
        }
        rgb[3 * p] = r;
        rgb[3 * p + 1] = g;
        rgb[3 * p + 2] = bl;
    }
}

unsigned serve_grid(uint64_t n) {
    const uint64_t g = (n + 255) / 256;
    return (unsigned)(g < 4096 ? (g ? g : 1) : 4096);
}

bool misaligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) != 0; }

}  // namespace

vr_status vr_serve_sum_device(const float* const* a, const float* const* b, float* const* out, uint32_t pairs,
                              uint64_t pixels, void* stream) {
    if (!a || !b || !out || pairs == 0 || pairs > 3) return vr::set_error(VR_ERR_INVALID, "serve sum: bad arguments");
    if (pixels == 0) return VR_OK;
    if (!vr::device_usable()) return vr::set_error(VR_ERR_NO_DEVICE, "no CUDA device");
    SumPairs sp{};
    for (uint32_t k = 0; k < pairs; ++k) {
        if (!a[k] || !b[k] || !out[k] || misaligned16(a[k]) || misaligned16(b[k]) || misaligned16(out[k]))
            return vr::set_error(VR_ERR_INVALID, "serve sum: buffers must be set and 16-byte aligned");
        sp.a[k] = reinterpret_cast<const float4*>(a[k]);
        sp.b[k] = reinterpret_cast<const float4*>(b[k]);
        sp.out[k] = reinterpret_cast<float4*>(out[k]);
    }
    k_serve_sum<<<serve_grid(pixels), 256, 0, static_cast<cudaStream_t>(stream)>>>(sp, pairs, pixels);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return vr::set_error(VR_ERR_CUDA, std::string("serve sum: ") + cudaGetErrorString(e));
    return VR_OK;
}

vr_status vr_serve_blend_device(const float* sum_a, const float* sum_b, uint32_t samples, const float* denoised,
                                const float* alpha_tiles, uint32_t width, uint32_t height, float* rgb, void* stream) {
    if (!sum_a || !sum_b || !rgb || !width || !height || !samples || (!denoised) != (!alpha_tiles))
        return vr::set_error(VR_ERR_INVALID, "serve blend: bad arguments");
    if (misaligned16(sum_a) || misaligned16(sum_b) || (denoised && misaligned16(denoised)))
        return vr::set_error(VR_ERR_INVALID, "serve blend: RGBA buffers must be 16-byte aligned");
    if (!vr::device_usable()) return vr::set_error(VR_ERR_NO_DEVICE, "no CUDA device");
    k_serve_blend<<<serve_grid((uint64_t)width * height), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        reinterpret_cast<const float4*>(sum_a), reinterpret_cast<const float4*>(sum_b), 1.0f / (float)samples,
        reinterpret_cast<const float4*>(denoised), alpha_tiles, width, height, rgb);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return vr::set_error(VR_ERR_CUDA, std::string("serve blend: ") + cudaGetErrorString(e));
    return VR_OK;
}

vr_status vr_serve_stats_device(const vr_stats_job* jobs, uint32_t count, double* out, void* stream) {
    if (!jobs || !out) return vr::set_error(VR_ERR_INVALID, "null argument");
    if (count == 0) return VR_OK;
    if (count > VR_STATS_MAX_JOBS) return vr::set_error(VR_ERR_INVALID, "too many jobs for one stats call");
    if (!vr::device_usable()) return vr::set_error(VR_ERR_NO_DEVICE, "no CUDA device");
    StatsTable t{};
    t.count = count;
    uint32_t blocks = 0;
    for (uint32_t i = 0; i < count; ++i) {
        const vr_stats_job& s = jobs[i];
        if (!s.sum_a || !s.sum_b || !s.width || !s.height || !s.n_a || !s.n_b || (!s.den_a) != (!s.den_b))
            return vr::set_error(VR_ERR_INVALID, "stats job " + std::to_string(i) + ": bad buffers or counts");
        for (const void* q : {(const void*)s.sum_a, (const void*)s.sum_b, (const void*)s.den_a, (const void*)s.den_b})
            if (reinterpret_cast<uintptr_t>(q) & 15u)
                return vr::set_error(VR_ERR_INVALID, "stats job " + std::to_string(i) + ": buffers must be 16-byte aligned");
        StatsJob& J = t.job[i];
        J.a = reinterpret_cast<const float4*>(s.sum_a);
        J.b = reinterpret_cast<const float4*>(s.sum_b);
        J.da = reinterpret_cast<const float4*>(s.den_a);
        J.db = reinterpret_cast<const float4*>(s.den_b);
        J.na = s.n_a;
        J.nb = s.n_b;
        J.w = s.width;
        J.h = s.height;
        J.tiles_x = (s.width + TILE - 1) / TILE;
        J.tiles = J.tiles_x * ((s.height + TILE - 1) / TILE);
        J.out_off = s.tile_offset;
        J.first_block = blocks;
        if ((uint64_t)blocks + J.tiles > 0x7fffffffu) return vr::set_error(VR_ERR_INVALID, "too many tiles");
        blocks += J.tiles;
    }
    k_serve_stats<<<blocks, THREADS, 0, static_cast<cudaStream_t>(stream)>>>(t, out);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return vr::set_error(VR_ERR_CUDA, std::string("serve stats: ") + cudaGetErrorString(e));
    return VR_OK;
}
