// Temporal resolve (DirectX/Shaders/TemporalResolve.hlsl:97-249): resolves the per-frame Halton
// camera jitter of a running render into a stable image.  Per pixel: a 3x3 YCoCg neighbourhood of
// the current frame gives a variance box (gamma 1, intersected with the min/max and widened to
// contain the current colour); history is resampled at the motion-reprojected position with a
// Catmull-Rom bicubic, clipped toward the current colour into the box, rejected across depth
// changes (|motion.z| >= 5 % of view depth), off screen, on reset or when not finite, and blended
// with a feedback weight that grows with on-screen speed.
//
// One thread per pixel, 32x8 blocks: each block reads a (32+2)x(8+2) neighbourhood of the
// accumulation and a 4x4 history footprint per pixel, all through L1/L2; the pass is bound by HBM
// streaming of accumulation (16 B), history (16 B), motion (16 B), depth (4 B) and the 16 B write.
#include "agb_kernels.h"
#include "agb_temporal.cuh"

namespace agb
{
namespace
{

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

__device__ v3 catmullRomHistory(const float4* history, int W, int H, v2 pos)
{
    v2 sp   = v2{ pos.x - 0.5f, pos.y - 0.5f };
    v2 base = v2{ floorf(sp.x), floorf(sp.y) };
    v2 f    = v2{ sp.x - base.x, sp.y - base.y };
    v2 f2   = v2{ f.x * f.x, f.y * f.y };
    v2 f3   = v2{ f2.x * f.x, f2.y * f.y };
    float wx[4], wy[4];
    wx[0] = -0.5f * f3.x + f2.x - 0.5f * f.x;
    wx[1] = 1.5f * f3.x - 2.5f * f2.x + 1.0f;
    wx[2] = -1.5f * f3.x + 2.0f * f2.x + 0.5f * f.x;
    wx[3] = 0.5f * f3.x - 0.5f * f2.x;
    wy[0] = -0.5f * f3.y + f2.y - 0.5f * f.y;
    wy[1] = 1.5f * f3.y - 2.5f * f2.y + 1.0f;
    wy[2] = -1.5f * f3.y + 2.0f * f2.y + 0.5f * f.y;
    wy[3] = 0.5f * f3.y - 0.5f * f2.y;
    int bx = int(base.x), by = int(base.y);
    v3 r   = splat(0.f);
#pragma unroll
    for (int j = 0; j < 4; j++)
    {
        int ty = clampi(by + j - 1, 0, H - 1);
#pragma unroll
        for (int i = 0; i < 4; i++)
        {
            int tx   = clampi(bx + i - 1, 0, W - 1);
            float4 h = __ldg(history + size_t(ty) * W + tx);
            r        = r + v3{ h.x, h.y, h.z } * (wx[i] * wy[j]);
        }
    }
    return v3{ fmaxf(r.x, 0.f), fmaxf(r.y, 0.f), fmaxf(r.z, 0.f) };
}

__device__ v3 clipToBox(v3 history, v3 current, v3 boxMin, v3 boxMax)
{
    v3 dir = history - current;
    v3 mag = abs3(dir);
    float t[3];
    float d[3] = { dir.x, dir.y, dir.z }, m[3] = { mag.x, mag.y, mag.z };
    float c[3] = { current.x, current.y, current.z };
    float lo[3] = { boxMin.x, boxMin.y, boxMin.z }, hi[3] = { boxMax.x, boxMax.y, boxMax.z };
#pragma unroll
    for (int k = 0; k < 3; k++)
    {
        float limit = d[k] > 0.f ? hi[k] - c[k] : c[k] - lo[k];
        float mm    = m[k] > 1e-6f ? m[k] : 1e-6f;
        t[k]        = m[k] > 1e-6f ? limit / mm : 1.f;
    }
    float mn    = t[0] < t[1] ? t[0] : t[1];
    mn          = mn < t[2] ? mn : t[2];
    float scale = mn < 0.f ? 0.f : (mn > 1.f ? 1.f : mn);
    return current + dir * scale;
}

__global__ void __launch_bounds__(256) k_temporal_resolve(const float4* accum, const float4* history,
    const float4* motion, const float* depthView, int W, int H, TemporalSettings s, float4* out)
{
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H)
        return;
    float4 cur4 = __ldg(accum + size_t(y) * W + x);
    v3 current  = v3{ cur4.x, cur4.y, cur4.z };
    v3 currentY = rgbToYCoCg(current);
    v3 m1 = splat(0.f), m2 = splat(0.f);
    v3 nmin = splat(1e30f), nmax = splat(-1e30f);
#pragma unroll
    for (int j = -1; j <= 1; j++)
#pragma unroll
        for (int i = -1; i <= 1; i++)
        {
            v3 nb;
            if (i == 0 && j == 0)
                nb = currentY;
            else
            {
                float4 q = __ldg(accum + size_t(clampi(y + j, 0, H - 1)) * W + clampi(x + i, 0, W - 1));
                nb       = rgbToYCoCg(v3{ q.x, q.y, q.z });
            }
            m1   = m1 + nb;
            m2   = m2 + nb * nb;
            nmin = v3{ nmin.x < nb.x ? nmin.x : nb.x, nmin.y < nb.y ? nmin.y : nb.y,
                nmin.z < nb.z ? nmin.z : nb.z };
            nmax = v3{ nmax.x > nb.x ? nmax.x : nb.x, nmax.y > nb.y ? nmax.y : nb.y,
                nmax.z > nb.z ? nmax.z : nb.z };
        }
    const float gamma = 1.0f;
    v3 mean  = m1 / 9.0f;
    v3 var   = m2 / 9.0f - mean * mean;
    v3 sigma = v3{ sqrtf(fmaxf(var.x, 0.f)), sqrtf(fmaxf(var.y, 0.f)), sqrtf(fmaxf(var.z, 0.f)) };
    float lo[3] = { mean.x - gamma * sigma.x, mean.y - gamma * sigma.y, mean.z - gamma * sigma.z };
    float hi[3] = { mean.x + gamma * sigma.x, mean.y + gamma * sigma.y, mean.z + gamma * sigma.z };
    float nlo[3] = { nmin.x, nmin.y, nmin.z }, nhi[3] = { nmax.x, nmax.y, nmax.z };
    float cy[3]  = { currentY.x, currentY.y, currentY.z };
#pragma unroll
    for (int k = 0; k < 3; k++)
    {
        lo[k] = lo[k] > nlo[k] ? lo[k] : nlo[k];
        hi[k] = hi[k] < nhi[k] ? hi[k] : nhi[k];
        lo[k] = lo[k] < cy[k] ? lo[k] : cy[k];
        hi[k] = hi[k] > cy[k] ? hi[k] : cy[k];
    }
    float4 mv  = __ldg(motion + size_t(y) * W + x);
    v2 prevPos = v2{ float(x) + 0.5f + mv.x, float(y) + 0.5f + mv.y };
    bool valid = s.isReset == 0;
    valid      = valid && prevPos.x >= 0.f && prevPos.y >= 0.f && prevPos.x < float(W) &&
        prevPos.y < float(H);
    float vz   = fabsf(__ldg(depthView + size_t(y) * W + x));
    valid      = valid && (fabsf(mv.z) < 0.05f * (vz > 1e-4f ? vz : 1e-4f));
    v3 hist    = catmullRomHistory(history, W, H, prevPos);
    v3 histY   = clipToBox(rgbToYCoCg(hist), currentY, v3{ lo[0], lo[1], lo[2] },
        v3{ hi[0], hi[1], hi[2] });
    hist       = yCoCgToRgb(histY);
    bool bad   = isnan(hist.x) || isnan(hist.y) || isnan(hist.z) || isinf(hist.x) ||
        isinf(hist.y) || isinf(hist.z);
    valid      = valid && !bad;
    float speed = sqrtf(mv.x * mv.x + mv.y * mv.y);
    float ref   = s.speedReference > 1e-4f ? s.speedReference : 1e-4f;
    float q     = speed / ref;
    q           = q < 0.f ? 0.f : (q > 1.f ? 1.f : q);
    float alpha = s.blendAlphaMin + q * (s.blendAlphaMax - s.blendAlphaMin);
    alpha       = valid ? (alpha < 0.f ? 0.f : (alpha > 1.f ? 1.f : alpha)) : 1.f;
    v3 res      = hist + (current - hist) * alpha;
    out[size_t(y) * W + x] = make_float4(res.x, res.y, res.z, cur4.w);
}

} // namespace

cudaError_t launchTemporalResolve(const float4* accum, const float4* history, const float4* motion,
    const float* depthView, int W, int H, const TemporalSettings& s, float4* out, cudaStream_t st)
{
    dim3 block(32, 8);
    dim3 grid((W + 31) / 32, (H + 7) / 8);
    k_temporal_resolve<<<grid, block, 0, st>>>(accum, history, motion, depthView, W, H, s, out);
    return cudaGetLastError();
}

} // namespace agb
