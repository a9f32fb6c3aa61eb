// dn_unet.cu — the denoiser network on the BF16 kernels: layer table,
// parameters and Adam state, activation workspace, inference, backward pass
// and training step; C ABI of include/voidray_denoise.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/voidray_denoise.h"
#include "dn_kernels.h"
#include "vr_host.h"

namespace {

using dn::bf16;

// Activation tensors of the U-Net: channels and pyramid level (resolution >> level).
enum Act { X0, A0A, S0, P0, A1A, S1, P1, A2A, S2, P2, BA, BT, D2A, U2, D1A, U1, D0A, U0, NACT };
struct ActDef {
    int c, lvl;
};
constexpr ActDef ACTS[NACT] = {{16, 0},  {32, 0},  {32, 0},  {32, 1},  {64, 1},  {64, 1},
                               {64, 2},  {128, 2}, {128, 2}, {128, 3}, {256, 3}, {256, 3},
                               {128, 2}, {128, 2}, {64, 1},  {64, 1},  {32, 0},  {32, 0}};
constexpr int OUT = -1;  // the fp32 network output
constexpr int OUT_C = 16;

struct LayerDef {
    int in1, in2, up1, out, cout, relu;
};
constexpr int NL = 15;
constexpr LayerDef LAYERS[NL] = {
    {X0, -1, 0, A0A, 32, 1},  {A0A, -1, 0, S0, 32, 1},  {P0, -1, 0, A1A, 64, 1},   {A1A, -1, 0, S1, 64, 1},
    {P1, -1, 0, A2A, 128, 1}, {A2A, -1, 0, S2, 128, 1}, {P2, -1, 0, BA, 256, 1},   {BA, -1, 0, BT, 256, 1},
    {BT, S2, 1, D2A, 128, 1}, {D2A, -1, 0, U2, 128, 1}, {U2, S1, 1, D1A, 64, 1},   {D1A, -1, 0, U1, 64, 1},
    {U1, S0, 1, D0A, 32, 1},  {D0A, -1, 0, U0, 32, 1},  {U0, -1, 0, OUT, OUT_C, 0}};
// pooling after layers 1, 3, 5: S0 -> P0, S1 -> P1, S2 -> P2
// the concatenating layer that consumes each skip tensor
int skip_consumer(int act) { return act == S0 ? 12 : act == S1 ? 10 : 8; }

int cin_of(const LayerDef& L) { return ACTS[L.in1].c + (L.in2 >= 0 ? ACTS[L.in2].c : 0); }
int level_of(const LayerDef& L) { return L.in2 >= 0 ? ACTS[L.in2].lvl : ACTS[L.in1].lvl; }

struct Offsets {
    size_t w[NL], b[NL], total;
};
Offsets offsets() {
    Offsets o{};
    size_t at = 0;
    for (int l = 0; l < NL; ++l) {
        o.w[l] = at;
        at += (size_t)LAYERS[l].cout * 9 * cin_of(LAYERS[l]);
        o.b[l] = at;
        at += LAYERS[l].cout;
    }
    o.total = at;
    return o;
}

double flops_per_pixel() {
    double f = 0;
    for (int l = 0; l < NL; ++l)
        f += 2.0 * 9.0 * cin_of(LAYERS[l]) * LAYERS[l].cout / double(1 << (2 * level_of(LAYERS[l])));
    return f;
}

#define DN_CK(expr)                                                                                          \
    do {                                                                                                     \
        cudaError_t e_ = (expr);                                                                             \
        if (e_ != cudaSuccess)                                                                               \
            return vr::set_error(e_ == cudaErrorMemoryAllocation ? VR_ERR_OOM : VR_ERR_CUDA,                 \
                                 std::string(#expr) + ": " + cudaGetErrorString(e_));                        \
    } while (0)

// deterministic host normal variates: splitmix64 + Box-Muller
struct HostRng {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
    double normal() {
        const double u1 = uniform(), u2 = uniform();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
};

}  // namespace

struct vr_denoiser {
    int device = 0;
    Offsets off{};
    float* w32 = nullptr;  // master weights
    float* g32 = nullptr;  // gradients (accumulated by the backward kernels)
    float* m = nullptr;
    float* v = nullptr;
    bf16* w16 = nullptr;   // bf16 weights [cout][9][cin]
    bf16* wt16 = nullptr;  // bf16 flipped weights [cin][9][cout] (backward-data)
    float* loss = nullptr; // device scalar
    uint64_t steps = 0;
    // workspace for (n, h, w)
    int wn = 0, wh = 0, ww = 0;  // dimensions of the current call
    size_t cap_px = 0;           // pixels the workspace holds (reused by any call that fits)
    std::vector<void*> ws;
    uint64_t ws_bytes = 0;
    bf16* act[NACT] = {};
    float* out = nullptr;
    bf16* gout = nullptr;
    bf16* dz[2] = {};
    bf16* dpool = nullptr;
    bf16* dcat[NL] = {};  // input gradients of the concatenating layers (8, 10, 12)
    bool train_ws = false;
    int loss_kind = dn::LOSS_L1_LOG;
    int backend = VR_DN_BACKEND_MMA_SYNC;  // forward convolutions
    bf16* up_tmp = nullptr;                // materialised 2x upsample (tcgen05 forward)
    uint32_t* status = nullptr;            // device: bounded-wait timeouts of the tcgen05 kernel
    float* scales_dev = nullptr;           // per-image input scales of batched inference
    uint32_t scales_cap = 0;
};

namespace {

void free_ws(vr_denoiser* d) {
    for (void* p : d->ws) cudaFree(p);
    d->ws.clear();
    d->ws_bytes = 0;
    std::memset(d->act, 0, sizeof d->act);
    std::memset(d->dcat, 0, sizeof d->dcat);
    d->out = nullptr;
    d->gout = nullptr;
    d->dz[0] = d->dz[1] = nullptr;
    d->dpool = nullptr;
    d->up_tmp = nullptr;
    d->wn = d->wh = d->ww = 0;
    d->cap_px = 0;
    d->train_ws = false;
}

template <class T>
vr_status ws_alloc(vr_denoiser* d, T** out, size_t count) {
    void* p = nullptr;
    const size_t b = std::max<size_t>(count * sizeof(T), 256);
    DN_CK(cudaMalloc(&p, b));
    d->ws.push_back(p);
    d->ws_bytes += b;
    *out = static_cast<T*>(p);
    return VR_OK;
}

// activations for an n x h x w batch (h, w multiples of 8); gradients too
// when train.  Every buffer scales with the pixel count, so a workspace
// allocated for P pixels serves any later call of at most P pixels without
// reallocating (a reallocation frees memory, which synchronises the device).
// The workspace belongs to the handle: calls on one handle from different
// streams must be ordered by the caller.
vr_status ensure_ws(vr_denoiser* d, int n, int h, int w, bool train) {
    const size_t need = (size_t)n * h * w;
    if (need <= d->cap_px && (d->train_ws || !train)) {
        d->wn = n;
        d->wh = h;
        d->ww = w;
        return VR_OK;
    }
    const bool was_train = d->train_ws;
    const size_t P = std::max(need, d->cap_px);
    free_ws(d);
    train = train || was_train;
    vr_status r;
    for (int a = 0; a < NACT; ++a)
        if ((r = ws_alloc(d, &d->act[a], (P >> (2 * ACTS[a].lvl)) * ACTS[a].c)) != VR_OK) return free_ws(d), r;
    if ((r = ws_alloc(d, &d->out, P * OUT_C)) != VR_OK) return free_ws(d), r;
    {
        size_t upmax = 0;  // full-resolution copy of the upsampled input of layers 8, 10, 12
        for (int l = 0; l < NL; ++l)
            if (LAYERS[l].up1) upmax = std::max(upmax, (P >> (2 * level_of(LAYERS[l]))) * ACTS[LAYERS[l].in1].c);
        if ((r = ws_alloc(d, &d->up_tmp, upmax)) != VR_OK) return free_ws(d), r;
    }
    if (train) {
        size_t dzmax = 0, dpmax = 0;
        for (int l = 0; l < NL; ++l) {
            const size_t pl = P >> (2 * level_of(LAYERS[l]));
            dzmax = std::max(dzmax, pl * LAYERS[l].cout);
            if (LAYERS[l].in1 == P0 || LAYERS[l].in1 == P1 || LAYERS[l].in1 == P2)
                dpmax = std::max(dpmax, (P >> (2 * ACTS[LAYERS[l].in1].lvl)) * ACTS[LAYERS[l].in1].c);
            if (LAYERS[l].in2 >= 0 && (r = ws_alloc(d, &d->dcat[l], pl * cin_of(LAYERS[l]))) != VR_OK)
                return free_ws(d), r;
        }
        if ((r = ws_alloc(d, &d->gout, P * OUT_C)) != VR_OK) return free_ws(d), r;
        if ((r = ws_alloc(d, &d->dz[0], dzmax)) != VR_OK) return free_ws(d), r;
        if ((r = ws_alloc(d, &d->dz[1], dzmax)) != VR_OK) return free_ws(d), r;
        if ((r = ws_alloc(d, &d->dpool, dpmax)) != VR_OK) return free_ws(d), r;
    }
    d->wn = n;
    d->wh = h;
    d->ww = w;
    d->cap_px = P;
    d->train_ws = train;
    return VR_OK;
}

vr_status refresh_bf16(vr_denoiser* d, cudaStream_t st) {
    for (int l = 0; l < NL; ++l)
        DN_CK(dn::cast_flip(d->w32 + d->off.w[l], d->w16 + d->off.w[l], d->wt16 + d->off.w[l], LAYERS[l].cout,
                            cin_of(LAYERS[l]), st));
    return VR_OK;
}

vr_status forward(vr_denoiser* d, cudaStream_t st) {
    const int n = d->wn, h = d->wh, w = d->ww;
    for (int l = 0; l < NL; ++l) {
        const LayerDef& L = LAYERS[l];
        const int lv = level_of(L);
        dn::ConvArgs a{};
        a.src1 = d->act[L.in1];
        a.src2 = L.in2 >= 0 ? d->act[L.in2] : nullptr;
        a.weight = d->w16 + d->off.w[l];
        a.bias = d->w32 + d->off.b[l];
        a.out = L.out >= 0 ? d->act[L.out] : nullptr;
        a.out_f32 = L.out >= 0 ? nullptr : d->out;
        a.n = n;
        a.h = h >> lv;
        a.w = w >> lv;
        a.c1 = ACTS[L.in1].c;
        a.c2 = L.in2 >= 0 ? ACTS[L.in2].c : 0;
        a.cout = L.cout;
        a.up1 = L.up1;
        a.relu = L.relu;
        if (d->backend == VR_DN_BACKEND_TCGEN05) {
            if (a.up1) {  // the TMA boxes read plain NHWC tiles: materialise the upsample
                DN_CK(dn::upsample2(a.src1, d->up_tmp, n, a.h, a.w, a.c1, st));
                a.src1 = d->up_tmp;
                a.up1 = 0;
            }
            if (dn::conv3x3_tc_supported(a)) {
                DN_CK(dn::conv3x3_tc(a, d->status, st));
            } else {
                DN_CK(dn::conv3x3(a, st));
            }
        } else {
            DN_CK(dn::conv3x3(a, st));
        }
        if (l == 1 || l == 3 || l == 5) {
            const int s = L.out, p = s + 1;  // S0 -> P0, S1 -> P1, S2 -> P2
            DN_CK(dn::avgpool2(d->act[s], d->act[p], n, h >> lv, w >> lv, ACTS[s].c, st));
        }
    }
    return VR_OK;
}

// backward from d->gout; accumulates into d->g32
vr_status backward(vr_denoiser* d, cudaStream_t st) {
    const int n = d->wn, h = d->wh, w = d->ww;
    const bf16* cur = d->gout;
    int flip = 0;
    for (int l = NL - 1; l >= 0; --l) {
        const LayerDef& L = LAYERS[l];
        const int lv = level_of(L), hl = h >> lv, wl = w >> lv;
        const int c1 = ACTS[L.in1].c, c2 = L.in2 >= 0 ? ACTS[L.in2].c : 0, cin = c1 + c2;
        dn::WgradArgs g{};
        g.dz = cur;
        g.src1 = d->act[L.in1];
        g.src2 = L.in2 >= 0 ? d->act[L.in2] : nullptr;
        g.dw = d->g32 + d->off.w[l];
        g.n = n;
        g.h = hl;
        g.w = wl;
        g.c1 = c1;
        g.c2 = c2;
        g.cout = L.cout;
        g.up1 = L.up1;
        g.db = d->g32 + d->off.b[l];  // the bias gradient, fused into the weight gradient's pass over dz
        DN_CK(dn::conv3x3_wgrad(g, st));
        if (l == 0) break;
        // input gradient: conv of dz with the flipped weights
        dn::ConvArgs a{};
        a.src1 = cur;
        a.weight = d->wt16 + d->off.w[l];
        a.n = n;
        a.h = hl;
        a.w = wl;
        a.c1 = L.cout;
        a.cout = cin;
        bf16* next = d->dz[flip];
        // backward-data on tcgen05 when the forward runs there
        auto conv = [&](const dn::ConvArgs& c) -> cudaError_t {
            if (d->backend == VR_DN_BACKEND_TCGEN05 && dn::conv3x3_tc_supported(c))
                return dn::conv3x3_tc(c, d->status, st);
            return dn::conv3x3(c, st);
        };
        if (L.in2 >= 0) {
            a.out = d->dcat[l];
            DN_CK(conv(a));
            const int lc = ACTS[L.in1].lvl;
            DN_CK(dn::up_bwd(d->dcat[l], cin, d->act[L.in1], next, n, h >> lc, w >> lc, c1, st));
        } else if (L.in1 == P0 || L.in1 == P1 || L.in1 == P2) {
            a.out = d->dpool;
            DN_CK(conv(a));
            const int s = L.in1 - 1;  // the pooled skip tensor
            const int k = skip_consumer(s);
            const int ls = ACTS[s].lvl;
            DN_CK(dn::skip_bwd(d->dcat[k], cin_of(LAYERS[k]), ACTS[LAYERS[k].in1].c, d->dpool, d->act[s], next, n,
                               h >> ls, w >> ls, ACTS[s].c, st));
        } else {
            a.mask = d->act[L.in1];
            a.out = next;
            DN_CK(conv(a));
        }
        cur = next;
        flip ^= 1;
    }
    return VR_OK;
}

vr_status check_dims(uint32_t batch, uint32_t width, uint32_t height) {
    if (!batch || !width || !height || (width & 7) || (height & 7))
        return vr::set_error(VR_ERR_INVALID, "batch, width and height must be positive, width and height multiples of 8");
    if ((uint64_t)batch * width * height > (1ull << 28))
        return vr::set_error(VR_ERR_INVALID, "batch too large (more than 2^28 pixels)");
    return VR_OK;
}

vr_status loss_and_grads(vr_denoiser* d, const float* rgba, const float* albedo, const float* normal,
                         const float* target, float scale_in, float scale_target, uint32_t batch, uint32_t width,
                         uint32_t height, cudaStream_t st) {
    vr_status r;
    if (!rgba || !albedo || !normal || !target) return vr::set_error(VR_ERR_INVALID, "null buffer");
    if ((r = check_dims(batch, width, height)) != VR_OK) return r;
    if ((r = ensure_ws(d, (int)batch, (int)height, (int)width, true)) != VR_OK) return r;
    const int n = (int)batch, h = (int)height, w = (int)width;
    DN_CK(dn::preprocess(reinterpret_cast<const float4*>(rgba), reinterpret_cast<const float4*>(albedo),
                         reinterpret_cast<const float4*>(normal), scale_in, nullptr, n, h, w, h, w, d->act[X0], st));
    if ((r = forward(d, st)) != VR_OK) return r;
    DN_CK(cudaMemsetAsync(d->loss, 0, sizeof(float), st));
    const float inv = 1.0f / (3.0f * (float)n * h * w);
    DN_CK(dn::loss(d->out, OUT_C, reinterpret_cast<const float4*>(target), reinterpret_cast<const float4*>(albedo),
                   scale_target, scale_in, n, h, w, inv, d->loss_kind, d->gout, d->loss, st));
    return backward(d, st);
}

vr_status read_loss(vr_denoiser* d, uint32_t batch, uint32_t width, uint32_t height, float* loss_host,
                    cudaStream_t st) {
    if (!loss_host) return VR_OK;
    float s = 0;
    DN_CK(cudaMemcpyAsync(&s, d->loss, sizeof s, cudaMemcpyDeviceToHost, st));
    DN_CK(cudaStreamSynchronize(st));
    *loss_host = s / (3.0f * (float)batch * width * height);  // mean over pixels and colour channels
    return VR_OK;
}

}  // namespace

extern "C" {

vr_status vr_denoiser_layer_get(uint32_t index, vr_denoiser_layer* out) {
    if (!out || index >= (uint32_t)NL) return vr::set_error(VR_ERR_INVALID, "bad layer index");
    const Offsets o = offsets();
    const LayerDef& L = LAYERS[index];
    out->c1 = ACTS[L.in1].c;
    out->c2 = L.in2 >= 0 ? ACTS[L.in2].c : 0;
    out->up1 = L.up1;
    out->cout = L.cout;
    out->relu = L.relu;
    out->level = level_of(L);
    out->w_offset = o.w[index];
    out->b_offset = o.b[index];
    return VR_OK;
}

vr_status vr_denoiser_create(uint64_t seed, vr_denoiser** out) {
    if (!out) return vr::set_error(VR_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (!vr::device_usable()) return vr::set_error(VR_ERR_NO_DEVICE, "no CUDA device");
    vr_denoiser* d = new vr_denoiser();
    d->off = offsets();
    cudaGetDevice(&d->device);
    const size_t np = d->off.total;
    auto fail_free = [&](vr_status s) {
        vr_denoiser_destroy(d);
        return s;
    };
#define DN_ALLOC(ptr, count)                                                                               \
    do {                                                                                                   \
        cudaError_t e_ = cudaMalloc(&(ptr), (count) * sizeof(*(ptr)));                                     \
        if (e_ != cudaSuccess) return fail_free(vr::set_error(VR_ERR_OOM, cudaGetErrorString(e_)));        \
    } while (0)
    DN_ALLOC(d->w32, np);
    DN_ALLOC(d->g32, np);
    DN_ALLOC(d->m, np);
    DN_ALLOC(d->v, np);
    DN_ALLOC(d->w16, np);
    DN_ALLOC(d->wt16, np);
    DN_ALLOC(d->loss, 1);
    DN_ALLOC(d->status, 1);
#undef DN_ALLOC
    if (cudaMemset(d->status, 0, sizeof(uint32_t)) != cudaSuccess)
        return fail_free(vr::set_error(VR_ERR_CUDA, "status init"));
    // He-normal init; the zero-padded input channels of layer 0 and output
    // channels >= 3 of the last layer stay zero
    std::vector<float> host(np, 0.0f);
    HostRng rng{seed};
    for (int l = 0; l < NL; ++l) {
        const LayerDef& L = LAYERS[l];
        const int cin = cin_of(L);
        const int cin_real = (l == 0) ? 9 : cin;
        const int cout_real = (l == NL - 1) ? 3 : L.cout;
        const double sd = std::sqrt((L.relu ? 2.0 : 1.0) / (9.0 * cin_real));
        for (int co = 0; co < cout_real; ++co)
            for (int t = 0; t < 9; ++t)
                for (int ci = 0; ci < cin_real; ++ci)
                    host[d->off.w[l] + ((size_t)co * 9 + t) * cin + ci] = (float)(sd * rng.normal());
    }
    vr_status r = vr_denoiser_set_params(d, host.data(), np);
    if (r != VR_OK) return fail_free(r);
    *out = d;
    return VR_OK;
}

vr_status vr_denoiser_destroy(vr_denoiser* d) {
    if (!d) return VR_OK;
    cudaDeviceSynchronize();
    free_ws(d);
    for (void* p : {(void*)d->w32, (void*)d->g32, (void*)d->m, (void*)d->v, (void*)d->w16, (void*)d->wt16,
                    (void*)d->loss, (void*)d->status, (void*)d->scales_dev})
        if (p) cudaFree(p);
    delete d;
    return VR_OK;
}

vr_status vr_denoiser_info_get(const vr_denoiser* d, vr_denoiser_info* info) {
    if (!info) return vr::set_error(VR_ERR_INVALID, "info is NULL");
    std::memset(info, 0, sizeof *info);
    info->param_count = offsets().total;
    info->num_layers = NL;
    info->input_channels = 9;
    info->flops_per_pixel = flops_per_pixel();
    if (d) {
        info->steps = d->steps;
        info->workspace_bytes = d->ws_bytes;
    }
    return VR_OK;
}

vr_status vr_denoiser_set_loss(vr_denoiser* d, int32_t kind) {
    if (!d) return vr::set_error(VR_ERR_INVALID, "null denoiser");
    if (kind != VR_DN_LOSS_L1_LOG && kind != VR_DN_LOSS_RELMSE) return vr::set_error(VR_ERR_INVALID, "bad loss kind");
    d->loss_kind = kind == VR_DN_LOSS_RELMSE ? dn::LOSS_RELMSE : dn::LOSS_L1_LOG;
    return VR_OK;
}

vr_status vr_denoiser_set_backend(vr_denoiser* d, int32_t backend) {
    if (!d) return vr::set_error(VR_ERR_INVALID, "null denoiser");
    if (backend != VR_DN_BACKEND_MMA_SYNC && backend != VR_DN_BACKEND_TCGEN05)
        return vr::set_error(VR_ERR_INVALID, "bad backend");
    d->backend = backend;
    return VR_OK;
}

vr_status vr_denoiser_status(vr_denoiser* d, uint32_t* flags) {
    if (!d || !flags) return vr::set_error(VR_ERR_INVALID, "null argument");
    DN_CK(cudaDeviceSynchronize());
    DN_CK(cudaMemcpy(flags, d->status, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    DN_CK(cudaMemset(d->status, 0, sizeof(uint32_t)));
    if (*flags) return vr::set_error(VR_ERR_TIMEOUT, "a tcgen05 convolution gave up a bounded wait");
    return VR_OK;
}

vr_status vr_denoiser_get_params(vr_denoiser* d, float* host, uint64_t count) {
    if (!d || !host) return vr::set_error(VR_ERR_INVALID, "null argument");
    if (count != d->off.total) return vr::set_error(VR_ERR_INVALID, "count must equal param_count");
    DN_CK(cudaDeviceSynchronize());
    DN_CK(cudaMemcpy(host, d->w32, count * sizeof(float), cudaMemcpyDeviceToHost));
    return VR_OK;
}

vr_status vr_denoiser_set_params(vr_denoiser* d, const float* host, uint64_t count) {
    if (!d || !host) return vr::set_error(VR_ERR_INVALID, "null argument");
    if (count != d->off.total) return vr::set_error(VR_ERR_INVALID, "count must equal param_count");
    DN_CK(cudaDeviceSynchronize());
    DN_CK(cudaMemcpy(d->w32, host, count * sizeof(float), cudaMemcpyHostToDevice));
    DN_CK(cudaMemset(d->g32, 0, count * sizeof(float)));
    DN_CK(cudaMemset(d->m, 0, count * sizeof(float)));
    DN_CK(cudaMemset(d->v, 0, count * sizeof(float)));
    d->steps = 0;
    vr_status r = refresh_bf16(d, nullptr);
    if (r != VR_OK) return r;
    DN_CK(cudaDeviceSynchronize());
    return VR_OK;
}

namespace {
vr_status denoise_impl(vr_denoiser* d, const float* rgba, const float* albedo, const float* normal, float scale,
                       const float* scales_host, float* out_rgba, uint32_t batch, uint32_t width, uint32_t height,
                       void* stream) {
    if (!d || !rgba || !albedo || !normal || !out_rgba) return vr::set_error(VR_ERR_INVALID, "null argument");
    if (!batch || !width || !height || (uint64_t)batch * width * height > (1ull << 28))
        return vr::set_error(VR_ERR_INVALID, "bad image size");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int h = (int)((height + 7) & ~7u), w = (int)((width + 7) & ~7u), n = (int)batch;
    vr_status r;
    if ((size_t)n * h * w > d->cap_px) DN_CK(cudaStreamSynchronize(st));
    if ((r = ensure_ws(d, n, h, w, false)) != VR_OK) return r;
    const float* scales = nullptr;
    if (scales_host) {
        if (d->scales_cap < batch) {
            DN_CK(cudaStreamSynchronize(st));
            if (d->scales_dev) cudaFree(d->scales_dev);
            d->scales_dev = nullptr;
            d->scales_cap = 0;
            DN_CK(cudaMalloc(&d->scales_dev, batch * sizeof(float)));
            d->scales_cap = batch;
        }
        // pageable source: staged before the call returns, ordered on the stream
        DN_CK(cudaMemcpyAsync(d->scales_dev, scales_host, batch * sizeof(float), cudaMemcpyHostToDevice, st));
        scales = d->scales_dev;
    }
    DN_CK(dn::preprocess(reinterpret_cast<const float4*>(rgba), reinterpret_cast<const float4*>(albedo),
                         reinterpret_cast<const float4*>(normal), scale, scales, n, (int)height, (int)width, h, w,
                         d->act[X0], st));
    if ((r = forward(d, st)) != VR_OK) return r;
    DN_CK(dn::postprocess(d->out, OUT_C, reinterpret_cast<const float4*>(albedo), scale, scales, n, (int)height,
                          (int)width, h, w, reinterpret_cast<float4*>(out_rgba), st));
    return VR_OK;
}
}  // namespace

vr_status vr_denoise_device(vr_denoiser* d, const float* rgba, const float* albedo, const float* normal, float scale,
                            float* out_rgba, uint32_t width, uint32_t height, void* stream) {
    return denoise_impl(d, rgba, albedo, normal, scale, nullptr, out_rgba, 1, width, height, stream);
}

vr_status vr_denoise_batch_device(vr_denoiser* d, const float* rgba, const float* albedo, const float* normal,
                                  const float* scales, float* out_rgba, uint32_t batch, uint32_t width,
                                  uint32_t height, void* stream) {
    if (!scales) return vr::set_error(VR_ERR_INVALID, "scales is NULL");
    return denoise_impl(d, rgba, albedo, normal, 1.0f, scales, out_rgba, batch, width, height, stream);
}

vr_status vr_denoiser_gradients_device(vr_denoiser* d, const float* rgba, const float* albedo, const float* normal,
                                       const float* target, float scale_in, float scale_target, uint32_t batch,
                                       uint32_t width, uint32_t height, float* loss_host, float* grads_host,
                                       void* stream) {
    if (!d) return vr::set_error(VR_ERR_INVALID, "null denoiser");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    DN_CK(cudaStreamSynchronize(st));
    DN_CK(cudaMemsetAsync(d->g32, 0, d->off.total * sizeof(float), st));
    vr_status r = loss_and_grads(d, rgba, albedo, normal, target, scale_in, scale_target, batch, width, height, st);
    if (r != VR_OK) return r;
    if ((r = read_loss(d, batch, width, height, loss_host, st)) != VR_OK) return r;
    if (grads_host) {
        DN_CK(cudaMemcpyAsync(grads_host, d->g32, d->off.total * sizeof(float), cudaMemcpyDeviceToHost, st));
        DN_CK(cudaStreamSynchronize(st));
    }
    DN_CK(cudaMemsetAsync(d->g32, 0, d->off.total * sizeof(float), st));
    return VR_OK;
}

vr_status vr_denoiser_train_step_device(vr_denoiser* d, const float* rgba, const float* albedo, const float* normal,
                                        const float* target, float scale_in, float scale_target, uint32_t batch,
                                        uint32_t width, uint32_t height, float lr, float* loss_host, void* stream) {
    if (!d) return vr::set_error(VR_ERR_INVALID, "null denoiser");
    if (!(lr >= 0.0f) || !std::isfinite(lr)) return vr::set_error(VR_ERR_INVALID, "bad learning rate");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if ((size_t)batch * width * height > d->cap_px || !d->train_ws) DN_CK(cudaStreamSynchronize(st));
    vr_status r = loss_and_grads(d, rgba, albedo, normal, target, scale_in, scale_target, batch, width, height, st);
    if (r != VR_OK) return r;
    if ((r = read_loss(d, batch, width, height, loss_host, st)) != VR_OK) return r;
    d->steps += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float bc1 = (float)(1.0 - std::pow(0.9, (double)d->steps));
    const float bc2 = (float)(1.0 - std::pow(0.999, (double)d->steps));
    DN_CK(dn::adam(d->w32, d->g32, d->m, d->v, d->off.total, lr, b1, b2, 1e-8f, bc1, bc2, st));
    return refresh_bf16(d, st);
}

vr_status vr_dn_conv3x3_device(const uint16_t* src1, uint32_t c1, int32_t up1, const uint16_t* src2, uint32_t c2,
                               const uint16_t* weight, const float* bias, const uint16_t* mask, uint16_t* out_bf16,
                               float* out_f32, uint32_t cout, uint32_t n, uint32_t h, uint32_t w, int32_t relu,
                               void* stream) {
    if (!src1 || !weight || (!out_bf16 == !out_f32) || (c2 && !src2))
        return vr::set_error(VR_ERR_INVALID, "src1, weight and exactly one output are required");
    dn::ConvArgs a{};
    a.src1 = reinterpret_cast<const bf16*>(src1);
    a.src2 = reinterpret_cast<const bf16*>(src2);
    a.weight = reinterpret_cast<const bf16*>(weight);
    a.bias = bias;
    a.mask = reinterpret_cast<const bf16*>(mask);
    a.out = reinterpret_cast<bf16*>(out_bf16);
    a.out_f32 = out_f32;
    a.n = (int)n;
    a.h = (int)h;
    a.w = (int)w;
    a.c1 = (int)c1;
    a.c2 = (int)c2;
    a.cout = (int)cout;
    a.up1 = up1 ? 1 : 0;
    a.relu = relu ? 1 : 0;
    const cudaError_t e = dn::conv3x3(a, static_cast<cudaStream_t>(stream));
    if (e == cudaErrorInvalidValue)
        return vr::set_error(VR_ERR_INVALID, "channel counts must be multiples of 16, h and w even when up1");
    DN_CK(e);
    return VR_OK;
}

vr_status vr_dn_conv3x3_tc_device(const uint16_t* src1, uint32_t c1, const uint16_t* src2, uint32_t c2,
                                  const uint16_t* weight, const float* bias, const uint16_t* mask,
                                  uint16_t* out_bf16, float* out_f32, uint32_t cout, uint32_t n, uint32_t h,
                                  uint32_t w, int32_t relu, uint32_t* status_device, void* stream) {
    if (!src1 || !weight || (!out_bf16 == !out_f32) || (c2 && !src2))
        return vr::set_error(VR_ERR_INVALID, "src1, weight and exactly one output are required");
    dn::ConvArgs a{};
    a.src1 = reinterpret_cast<const bf16*>(src1);
    a.src2 = reinterpret_cast<const bf16*>(src2);
    a.weight = reinterpret_cast<const bf16*>(weight);
    a.bias = bias;
    a.mask = reinterpret_cast<const bf16*>(mask);
    a.out = reinterpret_cast<bf16*>(out_bf16);
    a.out_f32 = out_f32;
    a.n = (int)n;
    a.h = (int)h;
    a.w = (int)w;
    a.c1 = (int)c1;
    a.c2 = (int)c2;
    a.cout = (int)cout;
    a.relu = relu ? 1 : 0;
    if (!dn::conv3x3_tc_supported(a))
        return vr::set_error(VR_ERR_UNSUPPORTED, "tcgen05 convolution: channels multiples of 16, 16-byte aligned");
    DN_CK(dn::conv3x3_tc(a, status_device, static_cast<cudaStream_t>(stream)));
    return VR_OK;
}

vr_status vr_dn_conv3x3_wgrad_device(const uint16_t* dz, const uint16_t* src1, uint32_t c1, int32_t up1,
                                     const uint16_t* src2, uint32_t c2, float* dw, uint32_t cout, uint32_t n,
                                     uint32_t h, uint32_t w, void* stream) {
    if (!dz || !src1 || !dw || (c2 && !src2)) return vr::set_error(VR_ERR_INVALID, "null argument");
    dn::WgradArgs a{};
    a.dz = reinterpret_cast<const bf16*>(dz);
    a.src1 = reinterpret_cast<const bf16*>(src1);
    a.src2 = reinterpret_cast<const bf16*>(src2);
    a.dw = dw;
    a.n = (int)n;
    a.h = (int)h;
    a.w = (int)w;
    a.c1 = (int)c1;
    a.c2 = (int)c2;
    a.cout = (int)cout;
    a.up1 = up1 ? 1 : 0;
    const cudaError_t e = dn::conv3x3_wgrad(a, static_cast<cudaStream_t>(stream));
    if (e == cudaErrorInvalidValue)
        return vr::set_error(VR_ERR_INVALID, "channel counts must be multiples of 16, h and w even when up1");
    DN_CK(e);
    return VR_OK;
}

}  // extern "C"
