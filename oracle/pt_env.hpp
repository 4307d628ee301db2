// Oracle (test infrastructure, never linked into the product): environment lighting and texture
// sampling restated from
//   Shaders/Environment.slang:35-186  (lat-long mapping, evaluate, alias-map sampling)
//   AliasMap.cpp:31-166               (luminance x solid angle, Walker alias table, integral)
//   Shaders/DefaultMaterial.slang:97-127 (UV transform, normal map)
// Texture2D.SampleLevel is restated for repeat addressing with nearest or bilinear filtering.
#pragma once

#include <vector>

#include "pt_bsdf.hpp"
#include "pt_scene.hpp"

namespace orc
{

template <class T>
struct Env
{
    using v2 = V2<T>;
    using v3 = V3<T>;
    static constexpr T PI = Consts<T>::PI;

    // Repeat-addressed texel fetch.
    static v3 texel(const Image& img, int64_t x, int64_t y)
    {
        int64_t w = img.width, h = img.height;
        x         = ((x % w) + w) % w;
        y         = ((y % h) + h) % h;
        const float* p = img.rgba + 4 * (size_t(y) * size_t(w) + size_t(x));
        return v3(T(p[0]), T(p[1]), T(p[2]));
    }
    static T texelAlpha(const Image& img, int64_t x, int64_t y)
    {
        int64_t w = img.width, h = img.height;
        x         = ((x % w) + w) % w;
        y         = ((y % h) + h) % h;
        return T(img.rgba[4 * (size_t(y) * size_t(w) + size_t(x)) + 3]);
    }
    // SampleLevel(uv, 0) with repeat addressing.  Texel centres sit at (i + 0.5) / size.
    static void sample(const Image& img, v2 uv, v3& rgb, T& alpha)
    {
        T fw = T(img.width), fh = T(img.height);
        if (!img.linear)
        {
            int64_t x = int64_t(std::floor(uv.x * fw));
            int64_t y = int64_t(std::floor(uv.y * fh));
            rgb       = texel(img, x, y);
            alpha     = texelAlpha(img, x, y);
            return;
        }
        T x     = uv.x * fw - T(0.5f);
        T y     = uv.y * fh - T(0.5f);
        T x0f   = std::floor(x);
        T y0f   = std::floor(y);
        T fx    = x - x0f;
        T fy    = y - y0f;
        int64_t x0 = int64_t(x0f), y0 = int64_t(y0f);
        v3 a    = lerp(texel(img, x0, y0), texel(img, x0 + 1, y0), fx);
        v3 b    = lerp(texel(img, x0, y0 + 1), texel(img, x0 + 1, y0 + 1), fx);
        rgb     = lerp(a, b, fy);
        T aa    = lerp(texelAlpha(img, x0, y0), texelAlpha(img, x0 + 1, y0), fx);
        T ab    = lerp(texelAlpha(img, x0, y0 + 1), texelAlpha(img, x0 + 1, y0 + 1), fx);
        alpha   = lerp(aa, ab, fy);
    }

    // Environment.slang:35-42
    static v2 directionToLatLongUV(const v3& d)
    {
        v2 uv;
        uv.x = ((tatan2(d.x, -d.z) * T(1)) / PI) * T(0.5f) + T(0.5f);
        uv.y = ((-tasin(d.y)) * T(1)) / PI + T(0.5f);
        return uv;
    }
    // Environment.slang:46-59
    static v3 latLongUVToDirection(v2 uv)
    {
        T phi   = (uv.x + T(0.25f)) * T(2) * PI;
        T theta = uv.y * PI;
        return v3(tcos(phi) * tsin(theta), tcos(theta), tsin(phi) * tsin(theta));
    }
    static v3 mulDir(const float* m, const v3& d)
    {
        return v3(T(m[0]) * d.x + T(m[1]) * d.y + T(m[2]) * d.z + T(m[3]) * T(0),
            T(m[4]) * d.x + T(m[5]) * d.y + T(m[6]) * d.z + T(m[7]) * T(0),
            T(m[8]) * d.x + T(m[9]) * d.y + T(m[10]) * d.z + T(m[11]) * T(0));
    }
    // Environment.slang:62-79 (screen-space UV uses the pixel index, as the reference does)
    static v2 computeEnvironmentUV(
        const float* transform, bool useScreen, v3 direction, v2 pixel, v2 screenSize)
    {
        if (useScreen)
            return v2(pixel.x / screenSize.x, pixel.y / screenSize.y);
        direction = normalize(mulDir(transform, direction));
        return directionToLatLongUV(direction);
    }

    struct Scene
    {
        const EnvData* data       = nullptr;
        const Image* lightImage   = nullptr; // required when data->hasLightTex
        const Image* background   = nullptr; // required when data->hasBackgroundTex
        const AliasEntry* alias   = nullptr; // width*height entries when data->hasLightTex
    };

    // Environment.slang:98-133
    static v3 evaluate(const Scene& env, const v3& direction, bool asBackground, v2 pixel,
        v2 screenSize)
    {
        const EnvData& c = *env.data;
        if (asBackground)
        {
            v2 uv = computeEnvironmentUV(
                c.backgroundTransform, c.backgroundUseScreen != 0, direction, pixel, screenSize);
            if (c.hasBackgroundTex)
            {
                v3 rgb;
                T a;
                sample(*env.background, uv, rgb, a);
                return rgb;
            }
            return lerp(v3::from(c.backgroundTop), v3::from(c.backgroundBottom), uv.y);
        }
        v2 uv = computeEnvironmentUV(c.lightTransform, false, direction, pixel, screenSize);
        if (c.hasLightTex)
        {
            v3 rgb;
            T a;
            sample(*env.lightImage, uv, rgb, a);
            return rgb;
        }
        return lerp(v3::from(c.lightTop), v3::from(c.lightBottom), uv.y);
    }

    // Environment.slang:137-186
    static v3 sampleEnvironment(const Scene& env, v2 random, v3& L, T& pdf)
    {
        const EnvData& c = *env.data;
        if (c.hasLightTex)
        {
            uint32_t width = env.lightImage->width, height = env.lightImage->height;
            uint32_t count = width * height;
            // uint(count * random[0]) in FP32 regardless of T: the index is a discrete choice.
            float prod      = float(count) * float(random[0]);
            uint32_t index  = uint32_t(prod);
            index           = index < count - 1 ? index : count - 1;
            AliasEntry e    = env.alias[index];
            if (T(e.prob) < random[1])
            {
                index = e.alias;
                e     = env.alias[index];
            }
            pdf        = T(e.pdf);
            uint32_t x = index % width, y = index / width;
            L = latLongUVToDirection(
                v2((T(x) + T(0.5f)) / T(width), (T(y) + T(0.5f)) / T(height)));
            L = normalize(mulDir(c.lightTransformInv, L));
            return texel(*env.lightImage, x, y);
        }
        L         = BSDF<T>::sampleUniformDirection(random, pdf);
        L         = normalize(mulDir(c.lightTransformInv, L));
        v2 uv     = directionToLatLongUV(L);
        return lerp(v3::from(c.lightTop), v3::from(c.lightBottom), uv.y);
    }
};

// AliasMap::build (AliasMap.cpp:71-166) restated in scalar type T.  pixels are RGB (3 floats per
// texel), row-major from the top row.  With T = float this is the reference's own FP32 arithmetic.
template <class T>
inline void buildAliasMap(const float* rgb, uint32_t width, uint32_t height,
    std::vector<AliasEntry>& out, T& luminanceIntegral)
{
    const uint32_t n = width * height;
    std::vector<T> lum(n), lumArea(n);
    luminanceIntegral = T(0);
    // Solid angles follow the reference's float arithmetic (static_cast<float> of the increments).
    const T PI      = Consts<T>::PI;
    T lonIncrement  = T(float(2.0 * 3.14159265358979323846 / width));
    T latIncrement  = T(float(3.14159265358979323846 / height));
    T latAngle      = T(float(3.14159265358979323846 / 2.0));
    (void)PI;
    size_t k        = 0;
    for (uint32_t y = 0; y < height; y++)
    {
        T solidAngle = (std::sin(latAngle) - std::sin(latAngle - latIncrement)) * lonIncrement;
        latAngle -= latIncrement;
        for (uint32_t x = 0; x < width; x++, k++)
        {
            const float* p = rgb + 3 * k;
            T l = T(p[0]) * T(0.2125f) + T(p[1]) * T(0.7154f) + T(p[2]) * T(0.0721f);
            lum[k]     = l;
            lumArea[k] = solidAngle * l;
            luminanceIntegral += lumArea[k];
        }
    }
    out.assign(n, AliasEntry{ 0, 0.f, 0.f, 0.f });
    std::vector<T> prob(n);
    std::vector<uint32_t> indexMap(n);
    T average    = luminanceIntegral / T(n);
    uint32_t sml = 0, lrg = n;
    for (uint32_t i = 0; i < n; i++)
    {
        prob[i]      = lumArea[i] / average;
        out[i].pdf   = float(lum[i] / luminanceIntegral);
        uint32_t idx = prob[i] < T(1) ? sml++ : --lrg;
        indexMap[idx] = i;
        out[i].alias  = i;
    }
    for (sml = 0; sml < lrg && lrg < n; sml++)
    {
        uint32_t s = indexMap[sml];
        uint32_t l = indexMap[lrg];
        out[s].alias = l;
        prob[l] -= T(1) - prob[s];
        lrg += prob[l] < T(1) ? 1 : 0;
    }
    for (uint32_t i = 0; i < n; i++)
        out[i].prob = float(prob[i]);
}

} // namespace orc
