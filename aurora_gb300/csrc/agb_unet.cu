// The learned denoiser: a 4-level U-Net (32 / 64 / 128 / 256 channels, two 3x3 convolutions per
// level, 2x2 average pooling down, nearest 2x upsampling up with skip concatenation, ReLU) over 16
// input feature channels, trained with an L1 loss and Adam.  Every convolution - forward, data
// gradient and weight gradient - runs on the tcgen05 tensor cores (agb_denoise.cu) with BF16
// operands and FP32 accumulation; activations are stored in BF16, gradients between layers are
// accumulated in FP32, the master weights and Adam moments are FP32.
//
// Prediction: log1p(radiance) = log1p(noisy input) + network output (channels 0-2), i.e. the network
// learns a residual correction in log space.
//
// Features (agb_denoiser_features): 0-2 log1p(noisy RGB), 3-5 base colour, 6-7 octahedral guide
// normal, 8 view depth / sky depth clamped to [0, 1], 9 log1p(sample luminance variance), 10-15
// zero.
#include <algorithm>
#include <cmath>
#include <cuda_bf16.h>
#include <vector>

#include "agb_kernels.h"

namespace agb
{
namespace
{

__device__ __forceinline__ float bf(uint16_t b) { return __uint_as_float(uint32_t(b) << 16); }
__device__ __forceinline__ uint16_t tobf(float v) { return __bfloat16_as_ushort(__float2bfloat16_rn(v)); }

inline unsigned gridFor(long n, int block = 256)
{
    long g = (n + block - 1) / block;
    return unsigned(std::min<long>(std::max<long>(g, 1), 1L << 20));
}

#ifndef AGB_PREACT_BLOCKS_PER_SM
#define AGB_PREACT_BLOCKS_PER_SM 4
#endif
// The gradient of one layer's pre-activation and of its bias, from the gradient of its output:
//   dPre[p][c] = bf16((g[p][c] + 0.25 * gp[p / 2x2][c]) * (y[p][c] > 0)),  db[c] += sum_p dPre[p][c]
// gp (the gradient of the 2x2 average pool of y, H/2 x W/2) and y (ReLU) are optional; the bias
// gradient sums the BF16-rounded values the weight gradient uses.  Thread i handles channels
// 8 (i % G8) .. + 7 of pixel i / G8; the grid stride is a multiple of 256 and so of G8 (C / 8 divides
// 256), so a thread keeps its channel group and the block reduces per channel in shared memory.
__global__ void __launch_bounds__(256) k_preact_grad(const float4* g, const float4* gp, const uint4* y, uint4* dpre,
    float* db, int B, int H, int W, int C)
{
    __shared__ float part[256][8];
    const int G8   = C / 8;
    const long n8  = long(B) * H * W * G8;
    const int t    = threadIdx.x;
    float acc[8]   = {};
    for (long i = blockIdx.x * 256L + t; i < n8; i += long(gridDim.x) * 256)
    {
        const float4 g0 = g[2 * i], g1 = g[2 * i + 1];
        float v[8]      = { g0.x, g0.y, g0.z, g0.w, g1.x, g1.y, g1.z, g1.w };
        if (gp)
        {
            const long pix = i / G8;
            const int x    = int(pix % W);
            const long r   = pix / W;
            const int yy   = int(r % H);
            const long b   = r / H;
            const long q   = ((b * (H / 2) + yy / 2) * (W / 2) + x / 2) * G8 + (i - pix * G8);
            const float4 p0 = gp[2 * q], p1 = gp[2 * q + 1];
            const float pv[8] = { p0.x, p0.y, p0.z, p0.w, p1.x, p1.y, p1.z, p1.w };
#pragma unroll
            for (int k = 0; k < 8; k++)
                v[k] += 0.25f * pv[k];
        }
        if (y)
        {
            const uint4 yv      = y[i];
            const uint32_t w[4] = { yv.x, yv.y, yv.z, yv.w };
#pragma unroll
            for (int k = 0; k < 4; k++)
            {
                if (!(__uint_as_float(w[k] << 16) > 0.f))
                    v[2 * k] = 0.f;
                if (!(__uint_as_float(w[k] & 0xFFFF0000u) > 0.f))
                    v[2 * k + 1] = 0.f;
            }
        }
        uint32_t o[4];
#pragma unroll
        for (int k = 0; k < 4; k++)
        {
            o[k] = uint32_t(tobf(v[2 * k])) | (uint32_t(tobf(v[2 * k + 1])) << 16);
            acc[2 * k] += __uint_as_float(o[k] << 16);
            acc[2 * k + 1] += __uint_as_float(o[k] & 0xFFFF0000u);
        }
        dpre[i] = make_uint4(o[0], o[1], o[2], o[3]);
    }
#pragma unroll
    for (int k = 0; k < 8; k++)
        part[t][k] = acc[k];
    __syncthreads();
    for (int c = t; c < C; c += 256)
    {
        float sum = 0.f;
        for (int u = c / 8; u < 256; u += G8)
            sum += part[u][c % 8];
        atomicAdd(db + c, sum);
    }
}

// L1 loss on log1p(radiance): prediction = out32[p][c] + log1p input (feature channel c), target
// RGBA FP32.  g (P x 16) = d loss / d out32; loss += sum |pred - log1p(target)| * scale.
__global__ void k_l1_loss(const float* out32, const uint16_t* x, const float* target, float* g, float* loss,
    long P, float scale)
{
    float acc = 0.f;
    for (long p = blockIdx.x * long(blockDim.x) + threadIdx.x; p < P; p += long(gridDim.x) * blockDim.x)
    {
#pragma unroll
        for (int c = 0; c < 16; c++)
        {
            float gv = 0.f;
            if (c < 3)
            {
                float pred = out32[p * 16 + c] + bf(x[p * 16 + c]);
                float t    = log1pf(fmaxf(target[p * 4 + c], 0.f));
                float d    = pred - t;
                acc += fabsf(d);
                gv = d > 0.f ? scale : (d < 0.f ? -scale : 0.f);
            }
            g[p * 16 + c] = gv;
        }
    }
    for (int o = 16; o > 0; o >>= 1)
        acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0)
        atomicAdd(loss, acc * scale);
}

__global__ void k_adam(float* w, const float* g, float* m, float* v, long n, float lr, float b1, float b2,
    float eps, float c1, float c2)
{
    for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x)
    {
        float gi = g[i];
        float mi = b1 * m[i] + (1.f - b1) * gi;
        float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i]     = mi;
        v[i]     = vi;
        w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

__device__ __forceinline__ float2 octEncode(float3 n)
{
    float s = fabsf(n.x) + fabsf(n.y) + fabsf(n.z);
    if (!(s > 0.f))
        return make_float2(0.f, 0.f);
    float x = n.x / s, y = n.y / s;
    if (n.z < 0.f)
    {
        float ox = (1.f - fabsf(y)) * (x >= 0.f ? 1.f : -1.f);
        float oy = (1.f - fabsf(x)) * (y >= 0.f ? 1.f : -1.f);
        x = ox;
        y = oy;
    }
    return make_float2(x, y);
}

__global__ void k_features(const float4* mean, const float2* moments, float samples, const float4* albedo,
    const float4* normal, const float* depth, float skyZ, long P, uint16_t* out)
{
    for (long p = blockIdx.x * long(blockDim.x) + threadIdx.x; p < P; p += long(gridDim.x) * blockDim.x)
    {
        float f[16];
        float4 m = mean[p];
        f[0] = log1pf(fmaxf(m.x, 0.f));
        f[1] = log1pf(fmaxf(m.y, 0.f));
        f[2] = log1pf(fmaxf(m.z, 0.f));
        float4 a = albedo[p];
        f[3] = fminf(fmaxf(a.x, 0.f), 1.f);
        f[4] = fminf(fmaxf(a.y, 0.f), 1.f);
        f[5] = fminf(fmaxf(a.z, 0.f), 1.f);
        float4 nn = normal[p];
        float2 o  = octEncode(make_float3(nn.x, nn.y, nn.z));
        f[6] = o.x;
        f[7] = o.y;
        float d = skyZ != 0.f ? depth[p] / skyZ : 0.f;
        f[8] = fminf(fmaxf(d, 0.f), 1.f);
        float var = 0.f;
        if (moments && samples > 1.f)
        {
            float2 mm = moments[p];
            float mu  = mm.x / samples;
            var       = fmaxf(mm.y / samples - mu * mu, 0.f);
        }
        f[9] = log1pf(var);
#pragma unroll
        for (int c = 10; c < 16; c++)
            f[c] = 0.f;
        uint32_t w[8];
#pragma unroll
        for (int j = 0; j < 8; j++)
            w[j] = uint32_t(tobf(f[2 * j])) | (uint32_t(tobf(f[2 * j + 1])) << 16);
        uint4* dst = reinterpret_cast<uint4*>(out + p * 16);
        dst[0]     = make_uint4(w[0], w[1], w[2], w[3]);
        dst[1]     = make_uint4(w[4], w[5], w[6], w[7]);
    }
}

// Deterministic normal deviates (splitmix64 + Box-Muller), identical on every host.
struct Normal
{
    uint64_t s;
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z          = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z          = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double operator()()
    {
        double u1 = (double(next() >> 11) + 0.5) / 9007199254740992.0;
        double u2 = (double(next() >> 11) + 0.5) / 9007199254740992.0;
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
};

} // namespace

// ------------------------------------------------------------------------------- network graph
enum Act
{
    A_X, A_E0A, A_S0, A_P0, A_E1A, A_S1, A_P1, A_E2A, A_S2, A_P2, A_BA, A_BB, A_D2A, A_D2, A_D1A, A_D1,
    A_D0A, A_D0, A_COUNT
};
static const int kActLevel[A_COUNT] = { 0, 0, 0, 1, 1, 1, 2, 2, 2, 3, 3, 3, 2, 2, 1, 1, 0, 0 };
static const int kActChannels[A_COUNT] = { 16, 32, 32, 32, 64, 64, 64, 128, 128, 128, 256, 256, 128, 128,
    64, 64, 32, 32 };

struct LayerDef
{
    int in0, in1, out; // activations (in1 = -1: none; out = -1: the FP32 output)
    int up0, relu, level;
};
static const LayerDef kLayerDefs[UnetDenoiser::kLayers] = {
    { A_X, -1, A_E0A, 0, 1, 0 }, { A_E0A, -1, A_S0, 0, 1, 0 },
    { A_P0, -1, A_E1A, 0, 1, 1 }, { A_E1A, -1, A_S1, 0, 1, 1 },
    { A_P1, -1, A_E2A, 0, 1, 2 }, { A_E2A, -1, A_S2, 0, 1, 2 },
    { A_P2, -1, A_BA, 0, 1, 3 }, { A_BA, -1, A_BB, 0, 1, 3 },
    { A_BB, A_S2, A_D2A, 1, 1, 2 }, { A_D2A, -1, A_D2, 0, 1, 2 },
    { A_D2, A_S1, A_D1A, 1, 1, 1 }, { A_D1A, -1, A_D1, 0, 1, 1 },
    { A_D1, A_S0, A_D0A, 1, 1, 0 }, { A_D0A, -1, A_D0, 0, 1, 0 },
    { A_D0, -1, -1, 0, 0, 0 },
};

static int layerCin(int i) { return kActChannels[kLayerDefs[i].in0] + (kLayerDefs[i].in1 >= 0 ? kActChannels[kLayerDefs[i].in1] : 0); }
static int layerCout(int i) { return kLayerDefs[i].out >= 0 ? kActChannels[kLayerDefs[i].out] : 16; }

UnetDenoiser::~UnetDenoiser() { release(); }

void UnetDenoiser::dropGraphs()
{
    for (Graph& g : graphs_)
        cudaGraphExecDestroy(g.exec);
    graphs_.clear();
    pending_ = Graph{};
}

void UnetDenoiser::release()
{
    dropGraphs();
    if (flagHost_)
        cudaFreeHost(flagHost_);
    flagHost_ = nullptr;
    for (void* p : allocs_)
        cudaFree(p);
    allocs_.clear();
    for (void* p : shapeAllocs_)
        cudaFree(p);
    shapeAllocs_.clear();
    B_ = H_ = W_ = 0;
}

cudaError_t UnetDenoiser::alloc(void** p, size_t bytes, std::vector<void*>& list)
{
    cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaSuccess)
    {
        list.push_back(*p);
        e = cudaMemsetAsync(*p, 0, bytes, stream_);
    }
    return e;
}

size_t UnetDenoiser::paramCount()
{
    size_t n = 0;
    for (int i = 0; i < kLayers; i++)
        n += size_t(9) * layerCin(i) * layerCout(i) + layerCout(i);
    return n;
}

cudaError_t UnetDenoiser::init(uint64_t seed, cudaStream_t st, int smCount)
{
    stream_  = st;
    smCount_ = smCount;
    nParams_ = paramCount();
    cudaError_t e;
    if ((e = alloc(reinterpret_cast<void**>(&params_), nParams_ * 4, allocs_)) != cudaSuccess ||
        (e = alloc(reinterpret_cast<void**>(&grads_), nParams_ * 4, allocs_)) != cudaSuccess ||
        (e = alloc(reinterpret_cast<void**>(&adamM_), nParams_ * 4, allocs_)) != cudaSuccess ||
        (e = alloc(reinterpret_cast<void**>(&adamV_), nParams_ * 4, allocs_)) != cudaSuccess ||
        (e = alloc(reinterpret_cast<void**>(&loss_), 4, allocs_)) != cudaSuccess)
        return e;
    size_t off = 0, packOff = 0;
    for (int i = 0; i < kLayers; i++)
    {
        wOff_[i] = off;
        off += size_t(9) * layerCin(i) * layerCout(i);
        bOff_[i] = off;
        off += size_t(layerCout(i));
        packOff_[i] = packOff;
        packOff += size_t(9) * layerCin(i) * layerCout(i);
    }
    if ((e = alloc(reinterpret_cast<void**>(&pack_), packOff * 2, allocs_)) != cudaSuccess ||
        (e = alloc(reinterpret_cast<void**>(&packFlip_), packOff * 2, allocs_)) != cudaSuccess)
        return e;
    // He-normal weights (fan-in 9 x the real input channels; the first layer has 10), zero biases;
    // the output layer starts small so the initial prediction is close to the noisy input.
    std::vector<float> h(nParams_, 0.f);
    Normal rng{ seed };
    for (int i = 0; i < kLayers; i++)
    {
        int cin = layerCin(i), cout = layerCout(i);
        int fan = 9 * (i == 0 ? 10 : cin);
        double sd = std::sqrt(2.0 / fan) * (i == kLayers - 1 ? 0.1 : 1.0);
        for (size_t k = 0; k < size_t(9) * cin * cout; k++)
            h[wOff_[i] + k] = float(sd * rng());
    }
    if ((e = cudaMemcpyAsync(params_, h.data(), nParams_ * 4, cudaMemcpyHostToDevice, stream_)) != cudaSuccess)
        return e;
    step_ = 0;
    return repack();
}

cudaError_t UnetDenoiser::repack()
{
    // Every layer packed both ways (forward and data-gradient layouts) in one launch.
    PackJob jobs[kLayers];
    for (int i = 0; i < kLayers; i++)
        jobs[i] = PackJob{ params_ + wOff_[i], pack_ + packOff_[i], packFlip_ + packOff_[i], layerCin(i), layerCout(i) };
    return launchPackConvWeightsMany(jobs, kLayers, stream_);
}

cudaError_t UnetDenoiser::ensureShape(int B, int H, int W, bool training)
{
    if (B == B_ && H == H_ && W == W_ && (!training || grad_[A_E0A]))
        return cudaSuccess;
    dropGraphs(); // they name the buffers freed here
    for (void* p : shapeAllocs_)
        cudaFree(p);
    shapeAllocs_.clear();
    for (int a = 0; a < A_COUNT; a++)
    {
        act_[a]  = nullptr;
        grad_[a] = nullptr;
    }
    out32_ = gOut_ = nullptr;
    dpre_  = nullptr;
    B_ = H_ = W_ = 0;
    cudaError_t e;
    size_t maxDpre = 0;
    for (int a = 1; a < A_COUNT; a++)
    {
        size_t n = pixels(B, H, W, kActLevel[a]) * kActChannels[a];
        if ((e = alloc(reinterpret_cast<void**>(&act_[a]), n * 2, shapeAllocs_)) != cudaSuccess)
            return e;
        if (training && (e = alloc(reinterpret_cast<void**>(&grad_[a]), n * 4, shapeAllocs_)) != cudaSuccess)
            return e;
    }
    size_t p0 = pixels(B, H, W, 0);
    if ((e = alloc(reinterpret_cast<void**>(&out32_), p0 * 16 * 4, shapeAllocs_)) != cudaSuccess)
        return e;
    if (training)
    {
        for (int i = 0; i < kLayers; i++)
        {
            size_t pl = pixels(B, H, W, kLayerDefs[i].level);
            maxDpre   = std::max(maxDpre, pl * layerCout(i));
        }
        if ((e = alloc(reinterpret_cast<void**>(&gOut_), p0 * 16 * 4, shapeAllocs_)) != cudaSuccess ||
            (e = alloc(reinterpret_cast<void**>(&dpre_), maxDpre * 2, shapeAllocs_)) != cudaSuccess)
            return e;
    }
    B_ = B;
    H_ = H;
    W_ = W;
    return cudaSuccess;
}

size_t UnetDenoiser::pixels(int B, int H, int W, int level) { return size_t(B) * (H >> level) * (W >> level); }

ConvLaunch UnetDenoiser::layerLaunch(int i, const uint16_t* x) const
{
    const LayerDef& L = kLayerDefs[i];
    ConvLaunch c{};
    c.in0   = L.in0 == A_X ? x : act_[L.in0];
    c.in1   = L.in1 >= 0 ? act_[L.in1] : nullptr;
    c.wpack = pack_ + packOff_[i];
    c.bias  = params_ + bOff_[i];
    c.out   = L.out >= 0 ? act_[L.out] : nullptr;
    c.out32 = L.out >= 0 ? nullptr : out32_;
    c.B     = B_;
    c.H     = H_ >> L.level;
    c.W     = W_ >> L.level;
    c.C0    = kActChannels[L.in0];
    c.C1    = L.in1 >= 0 ? kActChannels[L.in1] : 0;
    c.Cout  = layerCout(i);
    c.up0   = L.up0;
    c.relu  = L.relu;
    return c;
}

cudaError_t UnetDenoiser::forward(const uint16_t* x, int B, int H, int W, bool training, float* rgba)
{
    cudaError_t e = ensureShape(B, H, W, training);
    if (e != cudaSuccess)
        return e;
    input_ = x;
    for (int i = 0; i < kLayers; i++)
    {
        ConvLaunch c = layerLaunch(i, x);
        // The encoder's 2x2 average pools run in the epilogue of the convolution whose output they
        // downsample (S0 -> P0, S1 -> P1, S2 -> P2).
        if (i == 1 || i == 3 || i == 5)
            c.pool = act_[kLayerDefs[i].out + 1];
        // Inference: the output layer's epilogue writes the radiance (expm1 of the prediction)
        // instead of the FP32 prediction.
        if (i == kLayers - 1 && rgba && !training)
        {
            c.out32         = nullptr;
            c.radiance      = rgba;
            c.radianceInput = x;
        }
        if ((e = launchConv3x3(c, stream_)) != cudaSuccess)
            return e;
    }
    return cudaSuccess;
}

bool UnetDenoiser::inferTimedOut()
{
    if (!flagHost_ || *flagHost_ == 0)
        return false;
    int flag = 0;
    takeTcError(&flag);
    *flagHost_ = 0;
    return true;
}

cudaError_t UnetDenoiser::infer(const uint16_t* x, int B, int H, int W, float* rgba)
{
    cudaError_t e = ensureShape(B, H, W, false);
    if (e != cudaSuccess)
        return e;
    if (!flagHost_)
    {
        if ((e = cudaMallocHost(reinterpret_cast<void**>(&flagHost_), sizeof(int))) != cudaSuccess)
            return e;
        *flagHost_ = 0;
    }
    int* flagDev = nullptr;
    if ((e = tcErrorFlag(&flagDev)) != cudaSuccess)
        return e;
    e = inferLaunch(x, B, H, W, rgba);
    if (e != cudaSuccess)
        return e;
    return cudaMemcpyAsync(flagHost_, flagDev, sizeof(int), cudaMemcpyDeviceToHost, stream_);
}

cudaError_t UnetDenoiser::inferLaunch(const uint16_t* x, int B, int H, int W, float* rgba)
{
    cudaError_t e;
    for (size_t i = 0; i < graphs_.size(); i++)
    {
        Graph g = graphs_[i];
        if (g.x == x && g.rgba == rgba && g.B == B && g.H == H && g.W == W)
        {
            graphs_.erase(graphs_.begin() + long(i));
            graphs_.push_back(g);
            input_ = x;
            return cudaGraphLaunch(g.exec, stream_);
        }
    }
    // The first call with these buffers runs directly (it also loads and configures the kernels);
    // the second captures.  Capture on this thread only: other threads keep using their streams.
    if (!(pending_.x == x && pending_.rgba == rgba && pending_.B == B && pending_.H == H && pending_.W == W))
    {
        pending_ = Graph{ x, rgba, B, H, W, nullptr };
        return forward(x, B, H, W, false, rgba);
    }
    if ((e = cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
        return e;
    cudaError_t fe = forward(x, B, H, W, false, rgba);
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(stream_, &graph);
    if (fe != cudaSuccess || e != cudaSuccess)
    {
        if (graph)
            cudaGraphDestroy(graph);
        return fe != cudaSuccess ? fe : e;
    }
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess)
        return e;
    if (graphs_.size() >= 8)
    {
        cudaGraphExecDestroy(graphs_.front().exec);
        graphs_.erase(graphs_.begin());
    }
    graphs_.push_back(Graph{ x, rgba, B, H, W, exec });
    return cudaGraphLaunch(exec, stream_);
}

cudaError_t UnetDenoiser::backward(const float* target)
{
    cudaError_t e;
    if ((e = cudaMemsetAsync(grads_, 0, nParams_ * 4, stream_)) != cudaSuccess ||
        (e = cudaMemsetAsync(loss_, 0, 4, stream_)) != cudaSuccess)
        return e;
    for (int a = 1; a < A_COUNT; a++)
        if ((e = cudaMemsetAsync(grad_[a], 0, pixels(B_, H_, W_, kActLevel[a]) * kActChannels[a] * 4, stream_)) !=
            cudaSuccess)
            return e;
    long P0 = long(pixels(B_, H_, W_, 0));
    k_l1_loss<<<gridFor(P0), 256, 0, stream_>>>(out32_, input_, target, gOut_, loss_, P0, 1.f / float(P0 * 3));
    for (int i = kLayers - 1; i >= 0; i--)
    {
        const LayerDef& L = kLayerDefs[i];
        const int cin = layerCin(i), cout = layerCout(i);
        const long Pl = long(pixels(B_, H_, W_, L.level));
        const float* gy = L.out >= 0 ? grad_[L.out] : gOut_;
        // The 2x2 pools of layers 1, 3 and 5 (S -> P): their gradient reaches S here, at half
        // resolution, beside the gradient from the skip connection.
        const bool pooled = i == 1 || i == 3 || i == 5;
        const long n8     = Pl * cout / 8;
        k_preact_grad<<<unsigned(std::min<long>((n8 + 255) / 256, long(AGB_PREACT_BLOCKS_PER_SM) * smCount_)), 256, 0,
            stream_>>>(
            reinterpret_cast<const float4*>(gy), pooled ? reinterpret_cast<const float4*>(grad_[L.out + 1]) : nullptr,
            L.relu ? reinterpret_cast<const uint4*>(act_[L.out]) : nullptr, reinterpret_cast<uint4*>(dpre_),
            grads_ + bOff_[i], B_, H_ >> L.level, W_ >> L.level, cout);
        ConvLaunch c = layerLaunch(i, input_);
        if ((e = launchConvWgrad(c, dpre_, grads_ + wOff_[i], smCount_, stream_)) != cudaSuccess)
            return e;
        if (i > 0)
        {
            // dX = the convolution of dPre with the flipped weights, added straight into the
            // gradients of the layer's inputs (the upsampled one summed over 2x2 blocks).
            ConvLaunch d{};
            d.in0    = dpre_;
            d.wpack  = packFlip_ + packOff_[i];
            d.B      = B_;
            d.H      = c.H;
            d.W      = c.W;
            d.C0     = cout;
            d.Cout   = cin;
            d.grad0  = grad_[L.in0];
            d.grad1  = L.in1 >= 0 ? grad_[L.in1] : nullptr;
            d.gradC0 = c.C0;
            d.gradUp = L.up0;
            if ((e = launchConv3x3(d, stream_)) != cudaSuccess)
                return e;
        }
    }
    return cudaGetLastError();
}

cudaError_t UnetDenoiser::adam(float lr)
{
    step_++;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    float c1 = 1.f - float(std::pow(double(b1), double(step_)));
    float c2 = 1.f - float(std::pow(double(b2), double(step_)));
    k_adam<<<gridFor(long(nParams_)), 256, 0, stream_>>>(params_, grads_, adamM_, adamV_, long(nParams_), lr, b1, b2,
        eps, c1, c2);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    return repack();
}

cudaError_t UnetDenoiser::setParams(const float* host)
{
    cudaError_t e = cudaMemcpyAsync(params_, host, nParams_ * 4, cudaMemcpyHostToDevice, stream_);
    if (e != cudaSuccess)
        return e;
    return repack();
}

double UnetDenoiser::flopsPerPixel(bool training)
{
    double f = 0;
    for (int i = 0; i < kLayers; i++)
        f += 2.0 * 9 * layerCin(i) * layerCout(i) / double(1 << (2 * kLayerDefs[i].level));
    return training ? 3.0 * f : f;
}

cudaError_t launchDenoiseFeatures(const float4* mean, const float2* moments, float samples, const float4* albedo,
    const float4* normal, const float* depth, float skyZ, long P, uint16_t* out, cudaStream_t st)
{
    k_features<<<gridFor(P), 256, 0, st>>>(mean, moments, samples, albedo, normal, depth, skyZ, P, out);
    return cudaGetLastError();
}

} // namespace agb
