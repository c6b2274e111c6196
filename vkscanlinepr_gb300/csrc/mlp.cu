// mlp.cu — learned buffer sizing: path features, labels, and a small MLP
// trained and run by hand-written kernels.
//
// The reference sizes its intersection and fragment buffers by reading the
// count pass back to the host every frame (scanline_rasterizer.cpp:337-369,
// :578-584).  Here a 6-64-64-2 GELU network predicts, per path, log(1 + the
// number of intersection records) and log(1 + the number of draw records)
// from cheap features of its control points, so a frame can be sized when
// its scenes are uploaded and then enqueued without that read-back.  The
// prediction changes allocation only; an overflow is detected on the device
// and the frame reruns with exact sizing.
//
// Weights are BF16 (an FP32 master copy is kept for Adam); every product is
// accumulated in FP32.  Layout of the packed parameter vector:
//   W1[64][6] b1[64] W2[64][64] b2[64] W3[2][64] b3[2]
// Inputs and targets are standardised with a fixed normaliser
//   norm = x_mean[6] x_inv_std[6] y_mean[2] y_std[2]
// so the network works in standard units; predictions are returned in
// log(1 + count) units.
#include <cuda_bf16.h>

#include "common.cuh"
#include "kernels.h"

namespace sr {

namespace {
constexpr int kIn = kMlpIn, kH = kMlpHidden, kOut = kMlpOut;
constexpr int oW1 = 0, oB1 = oW1 + kH * kIn, oW2 = oB1 + kH, oB2 = oW2 + kH * kH, oW3 = oB2 + kH,
              oB3 = oW3 + kOut * kH, kParams = oB3 + kOut;
static_assert(kParams == kMlpParams, "parameter layout");
constexpr int nXm = 0, nXs = kIn, nYm = 2 * kIn, nYs = 2 * kIn + kOut;
static_assert(nYs + kOut == kMlpNorm, "normaliser layout");
constexpr int kSamples = 64;   // samples per training block (one per thread)
constexpr int kPad = kH + 1;   // shared-memory row stride: row q starts in bank q

SR_DEV float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
// d/dx [x Phi(x)] = Phi(x) + x phi(x)
SR_DEV float gelu_grad(float x) {
    const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
    const float pdf = 0.39894228040143268f * expf(-0.5f * x * x);
    return fmaf(x, pdf, cdf);
}

SR_DEV bool is_bias(int i) { return (i >= oB1 && i < oW2) || (i >= oB2 && i < oW3) || i >= oB3; }

// Parameters as the forward pass uses them: weights rounded to BF16, biases FP32.
SR_DEV void load_params(const __nv_bfloat16* __restrict__ wb, const float* __restrict__ master, float* s) {
    for (int i = threadIdx.x; i < kParams; i += blockDim.x) s[i] = is_bias(i) ? master[i] : __bfloat162float(wb[i]);
}
}  // namespace

// ------------------------------------------------------------ features ---
// Per path, from its transformed control points: segment count, bounding
// box clipped to one pixel around its canvas, control-polygon length, sum of
// absolute turning angles between successive control-polygon edges, and the
// fraction of cubic segments.  Lengths are in cells; counts, lengths and the
// turn sum enter as log(1 + x).
__global__ void k_path_features(const GeomArgs g, const uint32_t* __restrict__ path_first_curve, uint32_t n_paths,
                                float* __restrict__ feats) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n_paths) return;
    const SceneInfo& si = scene_of_path(g.st, p);
    const float W = (float)si.W, H = (float)si.H;
    const uint32_t c0 = path_first_curve[p], c1 = path_first_curve[p + 1];
    float xmin = 3.0e38f, ymin = 3.0e38f, xmax = -3.0e38f, ymax = -3.0e38f;
    float len = 0.0f, turn = 0.0f;
    uint32_t cubics = 0;
    float pex = 0.0f, pey = 0.0f;   // previous non-degenerate edge
    bool have_edge = false;
    for (uint32_t c = c0; c < c1; ++c) {
        const uint32_t type = g.curve_type[c];
        const uint32_t np = type & 7u;
        const float2* cp = g.tpos + g.curve_pos[c];
        cubics += type == 4u ? 1u : 0u;
        float2 a = cp[0];
        xmin = fminf(xmin, a.x); xmax = fmaxf(xmax, a.x);
        ymin = fminf(ymin, a.y); ymax = fmaxf(ymax, a.y);
        for (uint32_t k = 1; k < np; ++k) {
            const float2 b = cp[k];
            xmin = fminf(xmin, b.x); xmax = fmaxf(xmax, b.x);
            ymin = fminf(ymin, b.y); ymax = fmaxf(ymax, b.y);
            const float ex = b.x - a.x, ey = b.y - a.y;
            const float el = sqrtf(ex * ex + ey * ey);
            if (el > 0.0f) {
                len += el;
                if (have_edge) turn += fabsf(atan2f(pex * ey - pey * ex, pex * ex + pey * ey));
                pex = ex;
                pey = ey;
                have_edge = true;
            }
            a = b;
        }
    }
    const uint32_t segs = c1 - c0;
    float bw = 0.0f, bh = 0.0f;
    if (segs) {
        bw = fmaxf(fminf(xmax, W + 1.0f) - fmaxf(xmin, -1.0f), 0.0f);
        bh = fmaxf(fminf(ymax, H + 1.0f) - fmaxf(ymin, -1.0f), 0.0f);
    }
    const float invF = inv_F(g.F);
    float* f = feats + (size_t)p * kIn;
    f[0] = log1pf((float)segs);
    f[1] = log1pf(bw * invF);
    f[2] = log1pf(bh * invF);
    f[3] = log1pf(fminf(len, 1.0e30f) * invF);
    f[4] = log1pf(turn * 0.15915494309189535f);   // in turns
    f[5] = segs ? (float)cubics / (float)segs : 0.0f;
}

// Per path: log(1 + records) from the count pass and log(1 + draw records)
// from the emit's per-path counters.
__global__ void k_path_labels(const uint32_t* __restrict__ path_first_curve, uint32_t n_paths,
                              const int32_t* __restrict__ count, const uint32_t* __restrict__ path_draw,
                              float* __restrict__ labels) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n_paths) return;
    int64_t n = 0;
    for (uint32_t c = path_first_curve[p]; c < path_first_curve[p + 1]; ++c) n += count[c];
    labels[(size_t)p * kOut + 0] = log1pf((float)n);
    labels[(size_t)p * kOut + 1] = log1pf((float)path_draw[p]);
}

// ------------------------------------------------------------ inference --
// One path per thread; parameters staged once per block in shared memory.
__global__ void __launch_bounds__(128) k_mlp_predict(const __nv_bfloat16* __restrict__ wb,
                                                     const float* __restrict__ master,
                                                     const float* __restrict__ norm, const float* __restrict__ x,
                                                     uint32_t n, float* __restrict__ y) {
    __shared__ float s[kParams];
    __shared__ float nm[kMlpNorm];
    load_params(wb, master, s);
    if (threadIdx.x < kMlpNorm) nm[threadIdx.x] = norm[threadIdx.x];
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float in[kIn];
#pragma unroll
        for (int k = 0; k < kIn; ++k) in[k] = (x[(size_t)i * kIn + k] - nm[nXm + k]) * nm[nXs + k];
        float h1[kH];
#pragma unroll
        for (int j = 0; j < kH; ++j) {
            float a = s[oB1 + j];
#pragma unroll
            for (int k = 0; k < kIn; ++k) a = fmaf(s[oW1 + j * kIn + k], in[k], a);
            h1[j] = gelu(a);
        }
        float o0 = s[oB3], o1 = s[oB3 + 1];
        for (int j = 0; j < kH; ++j) {
            float a = s[oB2 + j];
#pragma unroll
            for (int k = 0; k < kH; ++k) a = fmaf(s[oW2 + j * kH + k], h1[k], a);
            const float h2 = gelu(a);
            o0 = fmaf(s[oW3 + j], h2, o0);
            o1 = fmaf(s[oW3 + kH + j], h2, o1);
        }
        y[(size_t)i * kOut] = fmaf(o0, nm[nYs], nm[nYm]);
        y[(size_t)i * kOut + 1] = fmaf(o1, nm[nYs + 1], nm[nYm + 1]);
    }
}

// ------------------------------------------------------------- training --
// Forward and backward of the mean squared error (in standard units) over
// one minibatch: rows idx[0..n) of (x, t), or rows 0..n when idx is NULL.
// Each block takes 64 samples, one per thread, keeps their activations in
// shared memory, then reduces its parameter gradients over the samples and
// adds them into grad.  loss_sum receives the sum of squared errors.
__global__ void __launch_bounds__(kSamples) k_mlp_grad(const __nv_bfloat16* __restrict__ wb,
                                                       const float* __restrict__ master,
                                                       const float* __restrict__ norm, const float* __restrict__ x,
                                                       const float* __restrict__ t, const uint32_t* __restrict__ idx,
                                                       uint32_t n, float scale, float* __restrict__ grad,
                                                       float* __restrict__ loss_sum) {
    extern __shared__ float sm[];
    float* s = sm;                          // parameters [kParams]
    float* a1 = s + kParams;                // layer-1 pre-activations [kSamples][kPad]
    float* h1 = a1 + kSamples * kPad;       // layer-1 outputs
    float* a2 = h1 + kSamples * kPad;       // layer-2 pre-activations
    float* h2 = a2 + kSamples * kPad;       // layer-2 outputs
    float* d2 = h2 + kSamples * kPad;       // dL/da2
    float* d1 = d2 + kSamples * kPad;       // dL/da1
    float* xin = d1 + kSamples * kPad;      // standardised inputs [kSamples][kIn]
    float* dy = xin + kSamples * kIn;       // dL/dy [kSamples][kOut]
    float* nm = dy + kSamples * kOut;       // normaliser [kMlpNorm]
    load_params(wb, master, s);
    const int tid = threadIdx.x;
    if (tid < kMlpNorm) nm[tid] = norm[tid];
    const uint32_t sidx = blockIdx.x * kSamples + tid;
    const bool live = sidx < n;
    const uint32_t row = live ? (idx ? idx[sidx] : sidx) : 0u;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kIn; ++k)
        xin[tid * kIn + k] = live ? (x[(size_t)row * kIn + k] - nm[nXm + k]) * nm[nXs + k] : 0.0f;
    for (int j = 0; j < kH; ++j) {
        float a = s[oB1 + j];
#pragma unroll
        for (int k = 0; k < kIn; ++k) a = fmaf(s[oW1 + j * kIn + k], xin[tid * kIn + k], a);
        a1[tid * kPad + j] = a;
        h1[tid * kPad + j] = gelu(a);
    }
    float y0 = s[oB3], y1 = s[oB3 + 1];
    for (int j = 0; j < kH; ++j) {
        float a = s[oB2 + j];
        for (int k = 0; k < kH; ++k) a = fmaf(s[oW2 + j * kH + k], h1[tid * kPad + k], a);
        a2[tid * kPad + j] = a;
        const float hv = gelu(a);
        h2[tid * kPad + j] = hv;
        y0 = fmaf(s[oW3 + j], hv, y0);
        y1 = fmaf(s[oW3 + kH + j], hv, y1);
    }
    float e0 = 0.0f, e1 = 0.0f;
    if (live) {
        e0 = y0 - (t[(size_t)row * kOut] - nm[nYm]) / nm[nYs];
        e1 = y1 - (t[(size_t)row * kOut + 1] - nm[nYm + 1]) / nm[nYs + 1];
        atomicAdd(loss_sum, e0 * e0 + e1 * e1);
    }
    // d(mean squared error)/dy with scale = 1 / (samples * outputs)
    const float g0 = 2.0f * scale * e0, g1 = 2.0f * scale * e1;
    dy[tid * kOut] = g0;
    dy[tid * kOut + 1] = g1;
    for (int j = 0; j < kH; ++j)
        d2[tid * kPad + j] = (s[oW3 + j] * g0 + s[oW3 + kH + j] * g1) * gelu_grad(a2[tid * kPad + j]);
    for (int k = 0; k < kH; ++k) {
        float a = 0.0f;
        for (int j = 0; j < kH; ++j) a = fmaf(s[oW2 + j * kH + k], d2[tid * kPad + j], a);
        d1[tid * kPad + k] = a * gelu_grad(a1[tid * kPad + k]);
    }
    __syncthreads();
    // parameter gradients: sums over the block's samples
    for (int e = tid; e < kParams; e += kSamples) {
        float acc = 0.0f;
        if (e < oB1) {                       // W1[j][k]
            const int j = e / kIn, k = e % kIn;
            for (int q = 0; q < kSamples; ++q) acc = fmaf(d1[q * kPad + j], xin[q * kIn + k], acc);
        } else if (e < oW2) {                // b1
            const int j = e - oB1;
            for (int q = 0; q < kSamples; ++q) acc += d1[q * kPad + j];
        } else if (e < oB2) {                // W2[j][k]
            const int j = (e - oW2) / kH, k = (e - oW2) % kH;
            for (int q = 0; q < kSamples; ++q) acc = fmaf(d2[q * kPad + j], h1[q * kPad + k], acc);
        } else if (e < oW3) {                // b2
            const int j = e - oB2;
            for (int q = 0; q < kSamples; ++q) acc += d2[q * kPad + j];
        } else if (e < oB3) {                // W3[o][j]
            const int o = (e - oW3) / kH, j = (e - oW3) % kH;
            for (int q = 0; q < kSamples; ++q) acc = fmaf(dy[q * kOut + o], h2[q * kPad + j], acc);
        } else {                             // b3
            const int o = e - oB3;
            for (int q = 0; q < kSamples; ++q) acc += dy[q * kOut + o];
        }
        atomicAdd(&grad[e], acc);
    }
}

// Adam on the FP32 master copy (bias-corrected moments); refreshes the BF16
// weights and clears the gradient for the next step.
__global__ void k_adam(float* __restrict__ master, __nv_bfloat16* __restrict__ wb, float* __restrict__ grad,
                       float* __restrict__ m, float* __restrict__ v, float lr, float b1, float b2, float eps,
                       float bc1, float bc2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParams) return;
    const float g = grad[i];
    const float mi = b1 * m[i] + (1.0f - b1) * g;
    const float vi = b2 * v[i] + (1.0f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float w = master[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    master[i] = w;
    wb[i] = __float2bfloat16_rn(w);
    grad[i] = 0.0f;
}

__global__ void k_to_bf16(const float* __restrict__ master, __nv_bfloat16* __restrict__ wb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kParams) wb[i] = __float2bfloat16_rn(master[i]);
}

// Shuffle keys for one epoch: a splitmix64 hash of (seed, i).
__global__ void k_perm_keys(uint32_t* __restrict__ keys, uint32_t n, uint64_t seed) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(i + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    keys[i] = (uint32_t)((z ^ (z >> 31)) >> 32);
}

// ------------------------------------------------------------ allotment --
// ceil(exp(y + margin) - 1): a count from a prediction in log(1 + count) units.
SR_DEV uint32_t allot_of(float y, float margin) {
    const float a = ceilf(expm1f(fminf(y + margin, 21.0f)));   // exp(21) < 2^31
    return a > 0.0f ? (uint32_t)a : 0u;
}

// Per path: the allotment (path margins, judged path by path) and the
// path's share of the frame capacity (frame margins), summed per scene and
// over the batch.  tot = frame records, frame draws, allotted records,
// allotted draws; scene_tot[S][2] = frame records, frame draws.
__global__ void k_allot(const float* __restrict__ y, uint32_t n_paths, const uint32_t* __restrict__ path_scene,
                        float4 margins, uint32_t* __restrict__ allot, unsigned long long* __restrict__ scene_tot,
                        unsigned long long* __restrict__ tot) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    unsigned long long v[4] = {0, 0, 0, 0};
    if (p < n_paths) {
        const float yr = y[(size_t)p * kOut], yd = y[(size_t)p * kOut + 1];
        const uint32_t ar = allot_of(yr, margins.x), ad = allot_of(yd, margins.y);
        const uint32_t fr = allot_of(yr, margins.z), fd = allot_of(yd, margins.w);
        allot[2 * (size_t)p] = ar;
        allot[2 * (size_t)p + 1] = ad;
        const uint32_t s = path_scene[p];
        atomicAdd(&scene_tot[2 * (size_t)s], (unsigned long long)fr);
        atomicAdd(&scene_tot[2 * (size_t)s + 1], (unsigned long long)fd);
        v[0] = fr;
        v[1] = fd;
        v[2] = ar;
        v[3] = ad;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
#pragma unroll
        for (int o = 16; o; o >>= 1) v[k] += __shfl_xor_sync(0xFFFFFFFFu, v[k], o);
    }
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < 4; ++k) atomicAdd(&tot[k], v[k]);
    }
}

// Per path: the exact counts against the allotment.  out[0] paths whose
// records exceed their allotment, out[1] likewise for draw records, out[2]
// and out[3] the exact totals.
__global__ void k_judge(const uint32_t* __restrict__ path_first_curve, uint32_t n_paths,
                        const int32_t* __restrict__ count, const uint32_t* __restrict__ path_draw,
                        const uint32_t* __restrict__ allot, unsigned long long* __restrict__ out) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long over_r = 0, over_d = 0, nr = 0, nd = 0;
    if (p < n_paths) {
        for (uint32_t c = path_first_curve[p]; c < path_first_curve[p + 1]; ++c) nr += (uint32_t)count[c];
        nd = path_draw[p];
        over_r = nr > allot[2 * (size_t)p] ? 1u : 0u;
        over_d = nd > allot[2 * (size_t)p + 1] ? 1u : 0u;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        over_r += __shfl_xor_sync(0xFFFFFFFFu, over_r, o);
        over_d += __shfl_xor_sync(0xFFFFFFFFu, over_d, o);
        nr += __shfl_xor_sync(0xFFFFFFFFu, nr, o);
        nd += __shfl_xor_sync(0xFFFFFFFFu, nd, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&out[0], over_r);
        atomicAdd(&out[1], over_d);
        atomicAdd(&out[2], nr);
        atomicAdd(&out[3], nd);
    }
}

// ------------------------------------------------------------- launches --
size_t mlp_grad_smem() {
    return sizeof(float) * (kParams + 6 * kSamples * kPad + kSamples * kIn + kSamples * kOut + kMlpNorm);
}

void launch_path_features(const GeomArgs& g, const uint32_t* path_first_curve, uint32_t n_paths, float* feats,
                          cudaStream_t st) {
    if (!n_paths) return;
    count_launches(1);
    k_path_features<<<(n_paths + 127) / 128, 128, 0, st>>>(g, path_first_curve, n_paths, feats);
}

void launch_path_labels(const uint32_t* path_first_curve, uint32_t n_paths, const int32_t* count,
                        const uint32_t* path_draw, float* labels, cudaStream_t st) {
    if (!n_paths) return;
    count_launches(1);
    k_path_labels<<<(n_paths + 127) / 128, 128, 0, st>>>(path_first_curve, n_paths, count, path_draw, labels);
}

void launch_mlp_predict(const void* wb, const float* master, const float* norm, const float* x, uint32_t n, float* y,
                        int sm_count, cudaStream_t st) {
    if (!n) return;
    count_launches(1);
    unsigned blocks = (n + 127) / 128;
    const unsigned cap = 8u * (unsigned)(sm_count > 0 ? sm_count : 148);
    if (blocks > cap) blocks = cap;
    k_mlp_predict<<<blocks, 128, 0, st>>>(static_cast<const __nv_bfloat16*>(wb), master, norm, x, n, y);
}

cudaError_t launch_mlp_grad(const void* wb, const float* master, const float* norm, const float* x, const float* t,
                            const uint32_t* idx, uint32_t n, float* grad, float* loss_sum, cudaStream_t st) {
    if (!n) return cudaSuccess;
    const size_t smem = mlp_grad_smem();
    cudaError_t e = cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    count_launches(1);
    k_mlp_grad<<<(n + kSamples - 1) / kSamples, kSamples, smem, st>>>(
        static_cast<const __nv_bfloat16*>(wb), master, norm, x, t, idx, n, 1.0f / ((float)n * (float)kOut), grad,
        loss_sum);
    return cudaGetLastError();
}

void launch_adam(float* master, void* wb, float* grad, float* m, float* v, float lr, float b1, float b2, float eps,
                 float bc1, float bc2, cudaStream_t st) {
    count_launches(1);
    k_adam<<<(kParams + 255) / 256, 256, 0, st>>>(master, static_cast<__nv_bfloat16*>(wb), grad, m, v, lr, b1, b2,
                                                  eps, bc1, bc2);
}

void launch_to_bf16(const float* master, void* wb, cudaStream_t st) {
    count_launches(1);
    k_to_bf16<<<(kParams + 255) / 256, 256, 0, st>>>(master, static_cast<__nv_bfloat16*>(wb));
}

void launch_perm_keys(uint32_t* keys, uint32_t n, uint64_t seed, cudaStream_t st) {
    if (!n) return;
    count_launches(1);
    k_perm_keys<<<(n + 255) / 256, 256, 0, st>>>(keys, n, seed);
}

void launch_allot(const float* y, uint32_t n_paths, const uint32_t* path_scene, const float margins[4],
                  uint32_t* allot, unsigned long long* scene_tot, unsigned long long* tot, cudaStream_t st) {
    if (!n_paths) return;
    count_launches(1);
    const float4 m = make_float4(margins[0], margins[1], margins[2], margins[3]);
    k_allot<<<(n_paths + 255) / 256, 256, 0, st>>>(y, n_paths, path_scene, m, allot, scene_tot, tot);
}

void launch_judge(const uint32_t* path_first_curve, uint32_t n_paths, const int32_t* count, const uint32_t* path_draw,
                  const uint32_t* allot, unsigned long long* out, cudaStream_t st) {
    if (!n_paths) return;
    count_launches(1);
    k_judge<<<(n_paths + 255) / 256, 256, 0, st>>>(path_first_curve, n_paths, count, path_draw, allot, out);
}

}  // namespace sr
