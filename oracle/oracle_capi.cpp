// Oracle (test infrastructure, never linked into the product): C ABI over the CPU restatement of
// Aurora's path tracer, for the parity tests and for the CPU baseline that bench.py reports.
// Layouts of every struct passed in are those of pt_scene.hpp (byte-compatible with the product's
// include/agb.h).  precision selects the FP32 (32) or FP64 (64) instantiation.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <thread>
#include <vector>

#include "pt_path.hpp"

using namespace orc;

#define ORC_API extern "C" __attribute__((visibility("default")))

namespace
{

template <class T>
ShadingData<T> frameFrom(const float* sh)
{
    // 12 floats per shading frame: normal, tangent, bitangent, unused
    ShadingData<T> s;
    s.normal    = V3<T>::from(sh + 0);
    s.tangent   = V3<T>::from(sh + 3);
    s.bitangent = V3<T>::from(sh + 6);
    return s;
}

template <class T>
Material<T> materialFrom(const MaterialBlock& b)
{
    Scene sc;
    sc.materials = &b;
    sc.materialCount = 1;
    PathTracer<T> pt;
    pt.scene = &sc;
    ShadingData<T> sh;
    V3<T> mn;
    bool gen;
    return pt.evaluateDefaultMaterial(0, sh, mn, gen);
}

template <class T>
void bsdfBatch(int op, const MaterialBlock* mats, const int32_t* matIndex, const float* frames,
    const float* V, const float* L, const float* rnd, int64_t n, float* outValue, float* outDir,
    float* outPdf, int32_t* outLobe)
{
    for (int64_t i = 0; i < n; i++)
    {
        Material<T> m     = materialFrom<T>(mats[matIndex[i]]);
        ShadingData<T> sh = frameFrom<T>(frames + 12 * i);
        V3<T> v           = V3<T>::from(V + 3 * i);
        V3<T> res(0);
        if (op == 0)
        {
            res = BSDF<T>::evaluateMaterial(m, sh, v, V3<T>::from(L + 3 * i));
        }
        else if (op == 1)
        {
            V3<T> lw;
            T pdf;
            int lobe;
            res = BSDF<T>::sampleMaterial(m, sh, v, V2<T>(T(rnd[2 * i]), T(rnd[2 * i + 1])), lw,
                pdf, lobe);
            outDir[3 * i] = float(lw.x);
            outDir[3 * i + 1] = float(lw.y);
            outDir[3 * i + 2] = float(lw.z);
            outPdf[i]  = float(pdf);
            outLobe[i] = lobe;
        }
        else
        {
            T pdf;
            int lobe;
            res = BSDF<T>::evaluateMaterialAndPDF(m, sh, v, V3<T>::from(L + 3 * i),
                V2<T>(T(rnd[2 * i]), T(rnd[2 * i + 1])), pdf, lobe);
            outPdf[i]  = float(pdf);
            outLobe[i] = lobe;
        }
        outValue[3 * i]     = float(res.x);
        outValue[3 * i + 1] = float(res.y);
        outValue[3 * i + 2] = float(res.z);
    }
}

template <class T>
void renderT(const PathTracer<T>& pt, uint32_t w, uint32_t h, uint32_t sampleStart,
    uint32_t sampleCount, int threads, float* accumMean, double* accumSum, float* lastSample,
    uint64_t* stats, const uint32_t* rect)
{
    uint32_t x0 = 0, y0 = 0, x1 = w, y1 = h;
    if (rect)
    {
        x0 = rect[0];
        y0 = rect[1];
        x1 = rect[2];
        y1 = rect[3];
    }
    const uint32_t tile = 16;
    uint32_t tilesX = (x1 - x0 + tile - 1) / tile, tilesY = (y1 - y0 + tile - 1) / tile;
    std::atomic<uint32_t> next(0);
    std::atomic<uint64_t> rays(0), shadows(0);
    auto worker = [&]() {
        const PathTracer<T>& local = pt;
        typename PathTracer<T>::Stats& st = PathTracer<T>::stats();
        st = typename PathTracer<T>::Stats();
        for (;;)
        {
            uint32_t t = next.fetch_add(1);
            if (t >= tilesX * tilesY)
                break;
            uint32_t tx = x0 + (t % tilesX) * tile, ty = y0 + (t / tilesX) * tile;
            for (uint32_t y = ty; y < std::min(ty + tile, y1); y++)
                for (uint32_t x = tx; x < std::min(tx + tile, x1); x++)
                {
                    size_t p = size_t(y) * w + x;
                    for (uint32_t si = sampleStart; si < sampleStart + sampleCount; si++)
                    {
                        T r[4];
                        local.tracePath(x, y, si, r);
                        float rf[4] = { float(r[0]), float(r[1]), float(r[2]), float(r[3]) };
                        if (accumMean)
                            accumulateRunningMean(accumMean + 4 * p, rf, si);
                        if (accumSum)
                            for (int k = 0; k < 4; k++)
                                accumSum[4 * p + k] += double(r[k]);
                        if (lastSample)
                            for (int k = 0; k < 4; k++)
                                lastSample[4 * p + k] = rf[k];
                    }
                }
        }
        rays += st.raysTraced;
        shadows += st.shadowRaysTraced;
    };
    int nt = threads > 0 ? threads : 1;
    std::vector<std::thread> pool;
    for (int i = 1; i < nt; i++)
        pool.emplace_back(worker);
    worker();
    for (auto& th : pool)
        th.join();
    if (stats)
    {
        stats[0] = rays.load();
        stats[1] = shadows.load();
    }
}

} // namespace

// Version / layout probe for the tests.
ORC_API int orc_layout(int which)
{
    switch (which)
    {
    case 0:
        return int(sizeof(MaterialBlock));
    case 1:
        return int(sizeof(FrameData));
    case 2:
        return int(sizeof(EnvData));
    case 3:
        return int(sizeof(Mesh));
    case 4:
        return int(sizeof(Instance));
    case 5:
        return int(sizeof(Image));
    case 6:
        return int(sizeof(Scene));
    case 7:
        return int(sizeof(Layer));
    case 8:
        return int(sizeof(GroundPlaneData));
    default:
        return -1;
    }
}

// PCG2D stream: writes n pairs drawn from the generator seeded for (sample, pixel).
ORC_API void orc_random_stream(uint32_t sampleIndex, uint32_t screenWidth, uint32_t px,
    uint32_t py, int n, float* out)
{
    Rng r = pcg2DInit(sampleIndex, screenWidth, px, py);
    for (int i = 0; i < n; i++)
    {
        V2<float> v = random2Df(r);
        out[2 * i]     = v.x;
        out[2 * i + 1] = v.y;
    }
}

// MaterialX's noise functions (the graph interpreter's NOISE operation): kind 0 Perlin 2D of
// (x, y), 1 Perlin 3D, 2 cell 2D, 3 cell 3D; xyz: 3 floats per point; out: n values.
ORC_API void orc_mx_noise(int precision, int kind, const float* xyz, int64_t n, double* out)
{
    for (int64_t i = 0; i < n; i++)
    {
        const float* p = xyz + 3 * i;
        if (precision == 64)
        {
            using N = MxNoise<double>;
            out[i] = kind == 0 ? N::perlin2(p[0], p[1]) : kind == 1 ? N::perlin3(p[0], p[1], p[2])
                : kind == 2    ? N::cell2(p[0], p[1])
                               : N::cell3(p[0], p[1], p[2]);
        }
        else
        {
            using N = MxNoise<float>;
            out[i] = kind == 0 ? N::perlin2(p[0], p[1]) : kind == 1 ? N::perlin3(p[0], p[1], p[2])
                : kind == 2    ? N::cell2(p[0], p[1])
                               : N::cell3(p[0], p[1], p[2]);
        }
    }
}

// op: 0 evaluateMaterial, 1 sampleMaterial, 2 evaluateMaterialAndPDF.  frames: 12 floats each.
ORC_API void orc_bsdf_batch(int op, int precision, const MaterialBlock* mats,
    const int32_t* matIndex, const float* frames, const float* V, const float* L, const float* rnd,
    int64_t n, float* outValue, float* outDir, float* outPdf, int32_t* outLobe)
{
    if (precision == 64)
        bsdfBatch<double>(op, mats, matIndex, frames, V, L, rnd, n, outValue, outDir, outPdf, outLobe);
    else
        bsdfBatch<float>(op, mats, matIndex, frames, V, L, rnd, n, outValue, outDir, outPdf, outLobe);
}

// AliasMap::build restated; precision 32 reproduces the reference's FP32 arithmetic.
ORC_API void orc_alias_build(int precision, const float* rgb, uint32_t width, uint32_t height,
    AliasEntry* out, double* integral)
{
    std::vector<AliasEntry> v;
    if (precision == 64)
    {
        double I;
        buildAliasMap<double>(rgb, width, height, v, I);
        *integral = I;
    }
    else
    {
        float I;
        buildAliasMap<float>(rgb, width, height, v, I);
        *integral = I;
    }
    std::copy(v.begin(), v.end(), out);
}

// Environment sampling / evaluation batches (Environment.slang:98-186).
ORC_API void orc_env_sample(int precision, const EnvData* env, const Image* light,
    const AliasEntry* alias, const float* rnd, int64_t n, float* outRadiance, float* outDir,
    float* outPdf)
{
    for (int64_t i = 0; i < n; i++)
    {
        if (precision == 64)
        {
            Env<double>::Scene s{ env, light, nullptr, alias };
            V3<double> L;
            double pdf;
            V3<double> r = Env<double>::sampleEnvironment(s, V2<double>(rnd[2 * i], rnd[2 * i + 1]), L, pdf);
            for (int k = 0; k < 3; k++)
            {
                outRadiance[3 * i + k] = float(r[k]);
                outDir[3 * i + k]      = float(L[k]);
            }
            outPdf[i] = float(pdf);
        }
        else
        {
            Env<float>::Scene s{ env, light, nullptr, alias };
            V3<float> L;
            float pdf;
            V3<float> r = Env<float>::sampleEnvironment(s, V2<float>(rnd[2 * i], rnd[2 * i + 1]), L, pdf);
            for (int k = 0; k < 3; k++)
            {
                outRadiance[3 * i + k] = r[k];
                outDir[3 * i + k]      = L[k];
            }
            outPdf[i] = pdf;
        }
    }
}

ORC_API void orc_env_evaluate(const EnvData* env, const Image* light, const Image* background,
    const float* dirs, const int32_t* asBackground, int64_t n, float* out)
{
    Env<float>::Scene s{ env, light, background, nullptr };
    for (int64_t i = 0; i < n; i++)
    {
        V3<float> r = Env<float>::evaluate(s, V3<float>::from(dirs + 3 * i), asBackground[i] != 0,
            V2<float>(0.f, 0.f), V2<float>(1.f, 1.f));
        out[3 * i]     = r.x;
        out[3 * i + 1] = r.y;
        out[3 * i + 2] = r.z;
    }
}

// Closest-hit (anyHit = 0) or occlusion (anyHit = 1) casts.  rays: 8 floats each
// (origin, tmin, direction, tmax).  hits: t, u, v as floats and inst, prim as int32.
ORC_API void orc_intersect(int precision, const Scene* s, const float* rays, int64_t n,
    int anyHit, int brute, float* outTUV, int32_t* outInstPrim)
{
    auto run = [&](auto tag) {
        using T = decltype(tag);
        Caster<T> c;
        c.bruteForce = brute != 0;
        c.build(s->meshes, s->meshCount, s->instances, s->instanceCount);
        for (int64_t i = 0; i < n; i++)
        {
            const float* r = rays + 8 * i;
            V3<T> o = V3<T>::from(r), d = V3<T>::from(r + 4);
            Hit h;
            bool hit = c.cast(o, d, T(r[3]), T(r[7]), h, anyHit != 0);
            outTUV[3 * i]         = hit ? h.t : -1.f;
            outTUV[3 * i + 1]     = h.u;
            outTUV[3 * i + 2]     = h.v;
            outInstPrim[2 * i]     = hit ? h.inst : -1;
            outInstPrim[2 * i + 1] = hit ? h.prim : -1;
        }
    };
    if (precision == 64)
        run(double());
    else
        run(float());
}

// A path tracer with its BVHs built, reusable across renders.
struct OrcTracer
{
    int precision;
    PathTracer<float> f32;
    PathTracer<double> f64;
};

ORC_API void* orc_tracer_create(int precision, const Scene* s, const FrameData* f, uint32_t w,
    uint32_t h, int brute)
{
    OrcTracer* t  = new OrcTracer();
    t->precision = precision;
    if (precision == 64)
        t->f64.init(s, f, w, h, brute != 0);
    else
        t->f32.init(s, f, w, h, brute != 0);
    return t;
}

ORC_API void orc_tracer_destroy(void* t) { delete static_cast<OrcTracer*>(t); }

ORC_API void orc_tracer_set_seed_offset(void* handle, uint32_t seedOffset)
{
    OrcTracer* t = static_cast<OrcTracer*>(handle);
    t->f32.seedOffset = t->f64.seedOffset = seedOffset;
}

// The scene's ground plane (null: none), restated in GroundPlane.slang's order by the tracer.
ORC_API void orc_tracer_set_ground_plane(void* handle, const GroundPlaneData* g)
{
    OrcTracer* t = static_cast<OrcTracer*>(handle);
    t->f32.setGroundPlane(g);
    t->f64.setGroundPlane(g);
}

// Denoising AOV targets (width*height: depth 1 float, normal / albedo / motion 4 floats per
// pixel) written by later renders for their last sample when the frame enables the AOVs; null
// pointers turn them off.
ORC_API void orc_tracer_set_aov(void* handle, float* depth, float* normal, float* albedo,
    float* motion)
{
    OrcTracer* t = static_cast<OrcTracer*>(handle);
    bool on      = depth && normal && albedo && motion;
    t->f32.aovDepth = t->f64.aovDepth = on ? depth : nullptr;
    t->f32.aovNormal = t->f64.aovNormal = on ? normal : nullptr;
    t->f32.aovAlbedo = t->f64.aovAlbedo = on ? albedo : nullptr;
    t->f32.aovMotion = t->f64.aovMotion = on ? motion : nullptr;
}

// TemporalResolve.hlsl over a whole image.  settings: isReset (as float bits of a uint), alpha
// min, alpha max, speed reference.
ORC_API void orc_temporal_resolve(int precision, const float* accum, const float* history,
    const float* motion, const float* depthView, int w, int h, uint32_t isReset, float alphaMin,
    float alphaMax, float speedReference, float* out)
{
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++)
        {
            float* o = out + 4 * (size_t(y) * size_t(w) + size_t(x));
            if (precision == 64)
            {
                Temporal<double>::Settings st{ isReset, alphaMin, alphaMax, speedReference };
                double r[4];
                Temporal<double>::resolvePixel(accum, history, motion, depthView, w, h, st, x, y, r);
                for (int k = 0; k < 4; k++)
                    o[k] = float(r[k]);
            }
            else
            {
                Temporal<float>::Settings st{ isReset, alphaMin, alphaMax, speedReference };
                float r[4];
                Temporal<float>::resolvePixel(accum, history, motion, depthView, w, h, st, x, y, r);
                for (int k = 0; k < 4; k++)
                    o[k] = r[k];
            }
        }
}

// PTRenderer.cpp:168-174
ORC_API void orc_temporal_jitter(uint32_t frameIndex, uint32_t phaseCount, float* out)
{
    temporalJitter(frameIndex, phaseCount, out);
}

// Renders sampleCount samples starting at sampleStart.  Any of accumMean (running mean, FP32 as
// the reference's accumulation pass), accumSum (FP64 sum of samples) and lastSample may be null.
// rect (x0, y0, x1, y1) restricts the pixels, or is null.  stats[0..1] = camera-path segments and
// shadow rays traced.  Returns the wall seconds of the rendering loop (BVH build excluded).
ORC_API double orc_tracer_render(void* handle, const FrameData* f, uint32_t sampleStart,
    uint32_t sampleCount, int threads, float* accumMean, double* accumSum, float* lastSample,
    uint64_t* stats, const uint32_t* rect)
{
    OrcTracer* t = static_cast<OrcTracer*>(handle);
    auto t0      = std::chrono::steady_clock::now();
    int64_t aovSample = sampleCount > 0 ? int64_t(sampleStart) + int64_t(sampleCount) - 1 : -1;
    t->f64.aovSample = t->f32.aovSample = aovSample;
    if (t->precision == 64)
    {
        if (f)
            t->f64.frame = f;
        renderT<double>(t->f64, t->f64.screenW, t->f64.screenH, sampleStart, sampleCount, threads,
            accumMean, accumSum, lastSample, stats, rect);
    }
    else
    {
        if (f)
            t->f32.frame = f;
        renderT<float>(t->f32, t->f32.screenW, t->f32.screenH, sampleStart, sampleCount, threads,
            accumMean, accumSum, lastSample, stats, rect);
    }
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

ORC_API double orc_render(int precision, const Scene* s, const FrameData* f, uint32_t w,
    uint32_t h, uint32_t sampleStart, uint32_t sampleCount, int threads, int brute,
    float* accumMean, double* accumSum, float* lastSample, uint64_t* stats, const uint32_t* rect)
{
    void* t   = orc_tracer_create(precision, s, f, w, h, brute);
    double dt = orc_tracer_render(t, f, sampleStart, sampleCount, threads, accumMean, accumSum,
        lastSample, stats, rect);
    orc_tracer_destroy(t);
    return dt;
}

ORC_API void orc_post_process(const float* accum, int64_t pixels, const float* brightness,
    int toneMap, int gamma, float* out)
{
    for (int64_t i = 0; i < pixels; i++)
        postProcess(accum + 4 * i, brightness, toneMap != 0, gamma != 0, out + 4 * i);
}

// The single-precision transcendentals the FP32 instantiation uses (agb_fmath.h), for the
// accuracy test against double-precision libm.  which: 0 sin, 1 cos, 2 exp2, 3 log2, 4 pow(x, y),
// 5 atan2(x, y), 6 asin.
ORC_API void orc_fmath(int which, const float* x, const float* y, int64_t n, float* out)
{
    for (int64_t i = 0; i < n; i++)
    {
        switch (which)
        {
        case 0:
            out[i] = agb_fm::sin(x[i]);
            break;
        case 1:
            out[i] = agb_fm::cos(x[i]);
            break;
        case 2:
            out[i] = agb_fm::exp2(x[i]);
            break;
        case 3:
            out[i] = agb_fm::log2(x[i]);
            break;
        case 4:
            out[i] = agb_fm::pow(x[i], y[i]);
            break;
        case 5:
            out[i] = agb_fm::atan2(x[i], y[i]);
            break;
        default:
            out[i] = agb_fm::asin(x[i]);
            break;
        }
    }
}
