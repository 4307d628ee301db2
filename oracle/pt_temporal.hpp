// Oracle (test infrastructure, never linked into the product): denoising AOV helpers, the Halton
// camera jitter and the temporal resolve, restated from
//   Shaders/GlobalPipelineState.slang:122-172   computeScreenMotion, computeViewZ,
//                                               computeMotionVector, computeSkyMotionVector
//   DirectX/PTRenderer.cpp:81-95,159-174        halton, getTemporalJitter
//   DirectX/Shaders/Colors.hlsli:42-56          RGBtoYCoCg, YCoCgtoRGB
//   DirectX/Shaders/TemporalResolve.hlsl:97-249 Catmull-Rom history, variance clip, feedback
// Matrices are the reference's FrameData matrices as bytes (glm column-major): element (row r,
// column c) of the shader's float4x4 is m[4 * c + r].
#pragma once

#include <cmath>
#include <cstdint>

#include "pt_math.hpp"

namespace orc
{

template <class T>
struct Temporal
{
    using v2 = V2<T>;
    using v3 = V3<T>;

    // mul(M, v) of the shader (row r = sum over c of M[r][c] v[c], left to right).
    static void mul4(const float* m, const T v[4], T out[4])
    {
        for (int r = 0; r < 4; r++)
            out[r] = T(m[r]) * v[0] + T(m[4 + r]) * v[1] + T(m[8 + r]) * v[2] + T(m[12 + r]) * v[3];
    }

    // GlobalPipelineState.slang:124-141
    static v2 screenMotion(const float* viewProj, const float* viewProjPrev, const T w[4], T width,
        T height)
    {
        T cur[4], prev[4];
        mul4(viewProj, w, cur);
        mul4(viewProjPrev, w, prev);
        T cw = std::fabs(cur[3]), pw = std::fabs(prev[3]);
        cw   = cw > T(1e-6f) ? cw : T(1e-6f);
        pw   = pw > T(1e-6f) ? pw : T(1e-6f);
        v2 cn(cur[0] / cw, cur[1] / cw);
        v2 pn(prev[0] / pw, prev[1] / pw);
        v2 cs((cn.x * T(0.5f) + T(0.5f)) * width, (-cn.y * T(0.5f) + T(0.5f)) * height);
        v2 ps((pn.x * T(0.5f) + T(0.5f)) * width, (-pn.y * T(0.5f) + T(0.5f)) * height);
        return v2(ps.x - cs.x, ps.y - cs.y);
    }

    // GlobalPipelineState.slang:144-150: rows of the transposed inverse view are right / up /
    // back / eye.
    static T viewZ(const float* invView, const v3& w)
    {
        v3 forward = -v3(T(invView[2]), T(invView[6]), T(invView[10]));
        v3 eye{ T(invView[3]), T(invView[7]), T(invView[11]) };
        return -dot(w - eye, forward);
    }

    // GlobalPipelineState.slang:155-163
    static void motionVector(const float* viewProj, const float* viewProjPrev,
        const float* invViewPrev, const v3& w, T currentViewZ, T width, T height, T out[4])
    {
        T prevViewZ = viewZ(invViewPrev, w);
        T w4[4]     = { w.x, w.y, w.z, T(1) };
        v2 m        = screenMotion(viewProj, viewProjPrev, w4, width, height);
        out[0]      = m.x;
        out[1]      = m.y;
        out[2]      = currentViewZ - prevViewZ;
        out[3]      = T(0);
    }

    // GlobalPipelineState.slang:166-172
    static void skyMotionVector(const float* viewProj, const float* viewProjPrev, const v3& d,
        T width, T height, T out[4])
    {
        T w4[4] = { d.x, d.y, d.z, T(0) };
        v2 m    = screenMotion(viewProj, viewProjPrev, w4, width, height);
        out[0]  = m.x;
        out[1]  = m.y;
        out[2]  = T(0);
        out[3]  = T(0);
    }

    static v3 toYCoCg(const v3& c)
    {
        return v3(T(0.25f) * c.x + T(0.5f) * c.y + T(0.25f) * c.z, T(0.5f) * c.x - T(0.5f) * c.z,
            -T(0.25f) * c.x + T(0.5f) * c.y - T(0.25f) * c.z);
    }
    static v3 fromYCoCg(const v3& c)
    {
        T t = c.x - c.z;
        return v3(t + c.y, c.x + c.z, t - c.y);
    }

    struct Settings
    {
        uint32_t isReset;
        float blendAlphaMin, blendAlphaMax, speedReference;
    };

    // TemporalResolve.hlsl:104-143
    static v3 sampleHistoryCatmullRom(const float* history, int W, int H, v2 pos)
    {
        v2 sp(pos.x - T(0.5f), pos.y - T(0.5f));
        v2 base(std::floor(sp.x), std::floor(sp.y));
        v2 f(sp.x - base.x, sp.y - base.y);
        v2 f2(f.x * f.x, f.y * f.y);
        v2 f3(f2.x * f.x, f2.y * f.y);
        T wx[4], wy[4];
        for (int a = 0; a < 2; a++)
        {
            T F = a == 0 ? f.x : f.y, F2 = a == 0 ? f2.x : f2.y, F3 = a == 0 ? f3.x : f3.y;
            T* w = a == 0 ? wx : wy;
            w[0] = -T(0.5f) * F3 + F2 - T(0.5f) * F;
            w[1] = T(1.5f) * F3 - T(2.5f) * F2 + T(1.0f);
            w[2] = -T(1.5f) * F3 + T(2.0f) * F2 + T(0.5f) * F;
            w[3] = T(0.5f) * F3 - T(0.5f) * F2;
        }
        v3 result(T(0));
        int bx = int(base.x), by = int(base.y);
        for (int j = 0; j < 4; j++)
            for (int i = 0; i < 4; i++)
            {
                int tx = bx + i - 1, ty = by + j - 1;
                tx     = tx < 0 ? 0 : (tx > W - 1 ? W - 1 : tx);
                ty     = ty < 0 ? 0 : (ty > H - 1 ? H - 1 : ty);
                const float* h = history + 4 * (size_t(ty) * size_t(W) + size_t(tx));
                v3 hv{ T(h[0]), T(h[1]), T(h[2]) };
                result += hv * (wx[i] * wy[j]);
            }
        return max3(result, T(0));
    }

    // TemporalResolve.hlsl:150-166
    static v3 clipToBox(const v3& history, const v3& current, const v3& boxMin, const v3& boxMax)
    {
        v3 direction = history - current;
        v3 magnitude = abs3(direction);
        v3 t;
        for (int k = 0; k < 3; k++)
        {
            T limit = direction[k] > T(0) ? boxMax[k] - current[k] : current[k] - boxMin[k];
            T mag   = magnitude[k] > T(1e-6f) ? magnitude[k] : T(1e-6f);
            t[k]    = magnitude[k] > T(1e-6f) ? limit / mag : T(1);
        }
        T m     = t.x < t.y ? t.x : t.y;
        m       = m < t.z ? m : t.z;
        T scale = saturate(m);
        return current + direction * scale;
    }

    // TemporalResolve.hlsl:171-248 for one pixel.  accum / history: RGBA, motion: 4 per pixel,
    // depthView: 1 per pixel.  Writes RGBA to out.
    static void resolvePixel(const float* accum, const float* history, const float* motion,
        const float* depthView, int W, int H, const Settings& s, int x, int y, T out[4])
    {
        const float* cp = accum + 4 * (size_t(y) * size_t(W) + size_t(x));
        v3 current{ T(cp[0]), T(cp[1]), T(cp[2]) };
        v3 currentY = toYCoCg(current);
        v3 m1(T(0)), m2(T(0));
        v3 nmin(T(1e30f)), nmax(T(-1e30f));
        for (int j = -1; j <= 1; j++)
            for (int i = -1; i <= 1; i++)
            {
                int nx = x + i, ny = y + j;
                nx     = nx < 0 ? 0 : (nx > W - 1 ? W - 1 : nx);
                ny     = ny < 0 ? 0 : (ny > H - 1 ? H - 1 : ny);
                v3 nb;
                if (i == 0 && j == 0)
                    nb = currentY;
                else
                {
                    const float* q = accum + 4 * (size_t(ny) * size_t(W) + size_t(nx));
                    nb             = toYCoCg(v3(T(q[0]), T(q[1]), T(q[2])));
                }
                m1 += nb;
                m2 += nb * nb;
                for (int k = 0; k < 3; k++)
                {
                    nmin[k] = nmin[k] < nb[k] ? nmin[k] : nb[k];
                    nmax[k] = nmax[k] > nb[k] ? nmax[k] : nb[k];
                }
            }
        const T gamma = T(1.0f);
        v3 mean       = m1 / T(9.0f);
        v3 var        = m2 / T(9.0f) - mean * mean;
        v3 sigma      = sqrt3(max3(var, T(0)));
        v3 boxMin, boxMax;
        for (int k = 0; k < 3; k++)
        {
            T lo      = mean[k] - gamma * sigma[k];
            T hi      = mean[k] + gamma * sigma[k];
            boxMin[k] = lo > nmin[k] ? lo : nmin[k];
            boxMax[k] = hi < nmax[k] ? hi : nmax[k];
            boxMin[k] = boxMin[k] < currentY[k] ? boxMin[k] : currentY[k];
            boxMax[k] = boxMax[k] > currentY[k] ? boxMax[k] : currentY[k];
        }
        const float* mv = motion + 4 * (size_t(y) * size_t(W) + size_t(x));
        v2 prevPos(T(float(x)) + T(0.5f) + T(mv[0]), T(float(y)) + T(0.5f) + T(mv[1]));
        bool valid = s.isReset == 0;
        valid      = valid && prevPos.x >= T(0) && prevPos.y >= T(0) && prevPos.x < T(float(W)) &&
            prevPos.y < T(float(H));
        T vz       = std::fabs(T(depthView[size_t(y) * size_t(W) + size_t(x)]));
        T vzf      = vz > T(1e-4f) ? vz : T(1e-4f);
        valid      = valid && (std::fabs(T(mv[2])) < T(0.05f) * vzf);
        v3 hist    = sampleHistoryCatmullRom(history, W, H, prevPos);
        v3 histY   = clipToBox(toYCoCg(hist), currentY, boxMin, boxMax);
        hist       = fromYCoCg(histY);
        bool bad   = std::isnan(hist.x) || std::isnan(hist.y) || std::isnan(hist.z) ||
            std::isinf(hist.x) || std::isinf(hist.y) || std::isinf(hist.z);
        valid      = valid && !bad;
        T speed    = std::sqrt(T(mv[0]) * T(mv[0]) + T(mv[1]) * T(mv[1]));
        T ref      = T(s.speedReference) > T(1e-4f) ? T(s.speedReference) : T(1e-4f);
        T alpha    = lerp(T(s.blendAlphaMin), T(s.blendAlphaMax), saturate(speed / ref));
        alpha      = valid ? saturate(alpha) : T(1);
        v3 res     = lerp(hist, current, alpha);
        out[0]     = res.x;
        out[1]     = res.y;
        out[2]     = res.z;
        out[3]     = T(cp[3]);
    }
};

// PTRenderer.cpp:81-95
inline float halton(uint32_t index, uint32_t base)
{
    float result = 0.0f;
    float scale  = 1.0f / static_cast<float>(base);
    while (index > 0)
    {
        result += scale * static_cast<float>(index % base);
        index /= base;
        scale /= static_cast<float>(base);
    }
    return result;
}

// PTRenderer.cpp:168-174
inline void temporalJitter(uint32_t frameIndex, uint32_t phaseCount, float out[2])
{
    uint32_t index = (phaseCount > 0u ? frameIndex % phaseCount : frameIndex) + 1u;
    out[0]         = halton(index, 2) - 0.5f;
    out[1]         = halton(index, 3) - 0.5f;
}

} // namespace orc
