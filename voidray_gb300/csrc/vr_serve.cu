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

}  // namespace

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
