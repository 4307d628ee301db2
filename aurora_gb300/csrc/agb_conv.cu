// The denoiser's 3x3 convolution on the tcgen05 tensor cores: a persistent, warp-specialised
// implicit GEMM fed by TMA tensor copies.
//
// Work unit (tile): R consecutive output rows x 256 consecutive output pixels x N output channels
// of one image.  The 256 pixels are split by parity into two MMA tiles of 128 rows: even pixels
// x = 2j and odd pixels x = 2j + 1, j in [j0, j0 + 128).  Every input that a tap of such a tile
// reads is then a run of 128 consecutive entries of a 130-entry "halo row" at offset 0, 1 or 2:
//   - a full-resolution input row is staged as its even-pixel row E and its odd-pixel row O
//     (pairs j0 - 1 .. j0 + 128); taps dx = -1, 0, +1 read O+0, E+1, O+1 for even outputs and
//     E+1, O+1, E+2 for odd outputs;
//   - a nearest-2x-upsampled input (the decoder's in0) is staged at its own half resolution
//     (pixels j0 - 1 .. j0 + 128 of row (y + dy) >> 1), and the same taps read it at offsets
//     0, 1, 1 (even) and 1, 1, 2 (odd): the upsample costs nothing and is never materialised.
// A staged row is K-major without swizzle: for one 16-channel group, channels 0-7 of entry i at
// byte 16 i, channels 8-15 at kHalfBytes + 16 i, so one TMA box (8 channels x 130 entries) lands
// exactly there and an MMA A descriptor at +16 bytes per entry of offset addresses any run.
//
// Roles (320 threads, one CTA per SM, static round-robin over tiles):
//   warp 0   TMA producer: per 16-channel group, (R + 2) x 2 halo rows (E, O) x 2 channel halves
//            (or the fewer half-resolution rows of an upsampled input) by cp.async.bulk.tensor
//            with zero fill outside the image, and the group's 9 weight slices (N x 16 each) by
//            one 1D bulk copy, into a ring of `stages` shared-memory stages (full / empty
//            mbarriers);
//   warp 1   MMA issuer: per stage 2 R x 9 tcgen05.mma (M = 128, N, K = 16) into the tile's
//            accumulators in TMEM, double-buffered (2 x 256 columns) so that the epilogue of one
//            tile overlaps the MMAs of the next;
//   warps 2-9 epilogue: tcgen05.ld of the accumulators, + bias, optional ReLU, BF16 (and / or FP32)
//            NHWC stores, and optionally the 2x2 average pool of the BF16 outputs (the encoder's
//            downsampling, exactly as a separate pool over the stored values would compute it).
// Every wait is bounded; a wait that runs out sets an error flag and the roles wind down, waiting
// (bounded) for their own copies and MMAs in flight before the TMEM is released.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <mutex>

#include "agb_kernels.h"
#include "agb_tc.cuh"

namespace agb
{

// Set by a conv kernel whose bounded wait ran out; read and cleared with takeConvError.
__device__ int g_convError;

namespace
{

constexpr int kHaloEntries      = 130;               // 128 MMA rows + offsets 0..2
constexpr uint32_t kBoxBytes    = kHaloEntries * 16; // one TMA box: 8 channels x 130 entries
constexpr uint32_t kHalfBytes   = 2176;              // kBoxBytes rounded up to 128 (TMA alignment)
constexpr uint32_t kRowBytes    = 2 * kHalfBytes;    // one staged row: both channel halves
constexpr int kThreads          = 320; // producer, MMA issuer, 8 epilogue warps
constexpr uint32_t kAccStride   = 256;               // TMEM columns per accumulator buffer
constexpr int kMaxStages        = 4;
constexpr size_t kSmemBudget    = 220 * 1024;

struct ConvTmaArgs
{
    const uint16_t* wpack; // per (channel tile, group): 9 slices (dy, dx) of N x 16, B layout
    const float* bias;     // [Cout] or null
    uint16_t* out;         // [B][H][W][Cout] or null
    float* out32;          // [B][H][W][Cout] or null
    uint16_t* pool;        // [B][H/2][W/2][Cout] or null (2x2 average of the BF16 outputs)
    int B, H, W, Cout, up0, relu;
    int N, nTiles, R, G, G0, stages;
    int tilesX, rowBlocks, numTiles;
    uint32_t stageBytes, aBytes;
};

struct Tile
{
    int nt, j0, y0, b;
};

__device__ __forceinline__ Tile decodeTile(const ConvTmaArgs& a, int t)
{
    Tile q;
    q.nt = t % a.nTiles;
    t /= a.nTiles;
    q.j0 = (t % a.tilesX) * 128;
    t /= a.tilesX;
    q.y0 = (t % a.rowBlocks) * a.R;
    q.b  = t / a.rowBlocks;
    return q;
}

// Staged half-resolution rows of an upsampled input for output rows y0 .. y0 + R - 1: rows
// (y0 - 1) >> 1 .. (y0 + R) >> 1 (arithmetic shifts: row -1 is outside the image, read as zero).
__device__ __forceinline__ int upRowBase(int y0) { return (y0 - 1) >> 1; }
__device__ __forceinline__ int upRowCount(int y0, int R) { return ((y0 + R) >> 1) - upRowBase(y0) + 1; }

__device__ __forceinline__ bool leaderWait(uint64_t* bar, uint32_t parity, int lane)
{
    int got = 0;
    if (lane == 0)
        got = tc::mbarWait(bar, parity) ? 1 : 0;
    return __shfl_sync(0xffffffffu, got, 0) != 0;
}

__device__ __forceinline__ float bfv(uint16_t b) { return __uint_as_float(uint32_t(b) << 16); }
__device__ __forceinline__ uint16_t tobf(float v) { return __bfloat16_as_ushort(__float2bfloat16_rn(v)); }

__global__ void __launch_bounds__(kThreads, 1) k_conv3x3_tma(const __grid_constant__ CUtensorMap tm0,
    const __grid_constant__ CUtensorMap tm1, const ConvTmaArgs a)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t full[kMaxStages], empty[kMaxStages], accFull[2], accEmpty[2], drain;
    __shared__ uint32_t tmemBase;
    const int tid  = threadIdx.x;
    const int warp = tid >> 5;
    const int lane = tid & 31;
    const int S    = a.stages;
    const int N    = a.N;
    const int R    = a.R;

    if (warp == 1)
        tc::tmemAlloc(&tmemBase, 2 * kAccStride);
    if (tid == 0)
    {
        for (int s = 0; s < S; s++)
        {
            tc::mbarInit(&full[s], 1);
            tc::mbarInit(&empty[s], 1);
        }
        for (int i = 0; i < 2; i++)
        {
            tc::mbarInit(&accFull[i], 1);
            tc::mbarInit(&accEmpty[i], 8);
        }
        tc::mbarInit(&drain, 1);
        tc::fenceMbarInit();
    }
    tc::fenceBeforeSync();
    __syncthreads();
    tc::fenceAfterSync();
    const uint32_t tmem = tmemBase;
    bool ok             = true;

    if (warp == 0)
    {
        // ---------------------------------------------------------------- TMA producer
        if (lane == 0)
        {
            uint32_t it = 0;
            uint32_t lastParity[kMaxStages];
            bool issued[kMaxStages];
            for (int s = 0; s < S; s++)
                issued[s] = false;
            const uint32_t wBytes = 9u * uint32_t(N) * 32u;
            for (int t = blockIdx.x; t < a.numTiles && ok; t += gridDim.x)
            {
                const Tile q = decodeTile(a, t);
                for (int g = 0; g < a.G; g++, it++)
                {
                    const int s        = int(it % uint32_t(S));
                    const uint32_t ph  = (it / uint32_t(S)) & 1u;
                    if (!tc::mbarWait(&empty[s], ph ^ 1u))
                    {
                        ok = false;
                        break;
                    }
                    uint8_t* A      = smem + size_t(s) * a.stageBytes;
                    uint8_t* Bw     = A + a.aBytes;
                    const bool in0  = g < a.G0;
                    const bool up   = in0 && a.up0;
                    const int c     = (in0 ? g : g - a.G0) * 16;
                    const void* map = in0 ? static_cast<const void*>(&tm0) : static_cast<const void*>(&tm1);
                    const int rows  = up ? upRowCount(q.y0, R) : (R + 2) * 2;
                    tc::mbarExpectTx(&full[s], wBytes + uint32_t(rows) * 2u * kBoxBytes);
                    tc::bulkLoad(Bw, a.wpack + (size_t(q.nt) * a.G + g) * 9 * size_t(N) * 16, wBytes, &full[s]);
                    if (up)
                    {
                        const int h0 = upRowBase(q.y0);
                        for (int i = 0; i < rows; i++)
                            for (int h = 0; h < 2; h++)
                                tc::tensorLoad4(A + i * kRowBytes + h * kHalfBytes, map, c + 8 * h, q.j0 - 1, h0 + i,
                                    q.b, &full[s]);
                    }
                    else
                    {
                        for (int i = 0; i < R + 2; i++)
                            for (int p = 0; p < 2; p++)
                                for (int h = 0; h < 2; h++)
                                    tc::tensorLoad5(A + (i * 2 + p) * kRowBytes + h * kHalfBytes, map, c + 8 * h, p,
                                        q.j0 - 1, q.y0 - 1 + i, q.b, &full[s]);
                    }
                    issued[s]     = true;
                    lastParity[s] = ph;
                }
            }
            // Copies still in flight (a consumer that gave up never waited for them) land before
            // the CTA exits.
            for (int s = 0; s < S; s++)
                if (issued[s] && !tc::mbarWait(&full[s], lastParity[s]))
                    ok = false;
        }
        __syncwarp();
    }
    else if (warp == 1)
    {
        // ---------------------------------------------------------------- MMA issuer
        if (lane == 0)
        {
            const uint32_t idesc = tc::idescBf16(128, uint32_t(N));
            uint32_t it = 0;
            int k       = 0;
            for (int t = blockIdx.x; t < a.numTiles && ok; t += gridDim.x, k++)
            {
                const Tile q       = decodeTile(a, t);
                const int buf      = k & 1;
                const uint32_t aph = uint32_t(k >> 1) & 1u;
                if (!tc::mbarWait(&accEmpty[buf], aph ^ 1u))
                {
                    ok = false;
                    break;
                }
                tc::fenceAfterSync();
                const uint32_t dBase = tmem + uint32_t(buf) * kAccStride;
                for (int g = 0; g < a.G; g++, it++)
                {
                    const int s       = int(it % uint32_t(S));
                    const uint32_t ph = (it / uint32_t(S)) & 1u;
                    if (!tc::mbarWait(&full[s], ph))
                    {
                        ok = false;
                        break;
                    }
                    tc::fenceAfterSync();
                    const uint32_t aAddr = tc::smemAddr(smem + size_t(s) * a.stageBytes);
                    const uint32_t bAddr = aAddr + a.aBytes;
                    const bool up        = g < a.G0 && a.up0;
                    const int h0         = upRowBase(q.y0);
                    for (int r = 0; r < R; r++)
                        for (int par = 0; par < 2; par++)
                        {
                            const uint32_t d = dBase + uint32_t((r * 2 + par) * N);
                            for (int dy = 0; dy < 3; dy++)
                                for (int dx = 0; dx < 3; dx++)
                                {
                                    // Entry offset of the run: 0, 1, 1 (even outputs), 1, 1, 2 (odd).
                                    const uint32_t shift = par == 0 ? (dx == 0 ? 0u : 1u) : (dx == 2 ? 2u : 1u);
                                    uint32_t row;
                                    if (up)
                                        row = uint32_t(((q.y0 + r + dy - 1) >> 1) - h0);
                                    else
                                    {
                                        // E for the centre tap of even outputs and the side taps of
                                        // odd outputs, O otherwise.
                                        const int odd = par == 0 ? (dx == 1 ? 0 : 1) : (dx == 1 ? 1 : 0);
                                        row           = uint32_t((r + dy) * 2 + odd);
                                    }
                                    const uint64_t ad =
                                        tc::smemDesc(aAddr + row * kRowBytes + shift * 16u, kHalfBytes, 128);
                                    const uint64_t bd = tc::smemDesc(bAddr + uint32_t((dy * 3 + dx) * N) * 32u,
                                        tc::kSliceLbo, tc::kSliceSbo);
                                    tc::mma(d, ad, bd, idesc, (g | dy | dx) != 0 ? 1u : 0u);
                                }
                        }
                    tc::commit(&empty[s]);
                }
                if (!ok)
                    break;
                tc::commit(&accFull[buf]);
            }
            // Every MMA issued by this thread has completed before the TMEM is released.
            tc::commit(&drain);
            if (!tc::mbarWait(&drain, 0))
                ok = false;
        }
        __syncwarp();
    }
    else
    {
        // ---------------------------------------------------------------- epilogue (warps 2-9)
        // Two warps per TMEM lane quadrant; the tile's work items (a row, or a row pair when
        // pooling, x a 16-channel chunk) alternate between them.
        const int quad     = warp & 3; // TMEM lanes 32 quad .. 32 quad + 31
        const int half     = (warp - 2) >> 2;
        const int m        = quad * 32 + lane;
        const int W2       = a.W >> 1;
        const int step     = a.pool ? 2 : 1;
        const int chunks   = N / 16;
        const int items    = (R / step) * chunks;
        int k              = 0;
        for (int t = blockIdx.x; t < a.numTiles; t += gridDim.x, k++)
        {
            const Tile q       = decodeTile(a, t);
            const int buf      = k & 1;
            const uint32_t aph = uint32_t(k >> 1) & 1u;
            if (!leaderWait(&accFull[buf], aph, lane))
            {
                ok = false;
                break;
            }
            tc::fenceAfterSync();
            const int j          = q.j0 + m;
            const bool colOk     = j < W2;
            const int cb         = q.nt * N;
            const uint32_t tBase = tmem + (uint32_t(quad * 32) << 16) + uint32_t(buf) * kAccStride;
            for (int item = half; item < items; item += 2)
            {
                const int r  = (item / chunks) * step;
                const int c0 = (item % chunks) * 16;
                // All accumulators of the item (2 or 4) in flight before one wait.
                uint32_t v[4][16];
                tc::tmemLoad16(tBase + uint32_t((r * 2 + 0) * N + c0), v[0]);
                tc::tmemLoad16(tBase + uint32_t((r * 2 + 1) * N + c0), v[1]);
                if (step == 2)
                {
                    tc::tmemLoad16(tBase + uint32_t((r * 2 + 2) * N + c0), v[2]);
                    tc::tmemLoad16(tBase + uint32_t((r * 2 + 3) * N + c0), v[3]);
                }
                tc::tmemWaitLoad();
                float bv[16];
#pragma unroll
                for (int i = 0; i < 16; i++)
                    bv[i] = a.bias ? __ldg(a.bias + cb + c0 + i) : 0.f;
                float psum[16];
#pragma unroll
                for (int acc = 0; acc < 4; acc++)
                {
                    if (acc >= 2 * step)
                        break;
                    const int par = acc & 1;
                    const int y   = q.y0 + r + (acc >> 1);
                    float f[16];
                    uint16_t h[16];
#pragma unroll
                    for (int i = 0; i < 16; i++)
                    {
                        f[i] = __uint_as_float(v[acc][i]) + bv[i];
                        if (a.relu)
                            f[i] = fmaxf(f[i], 0.f);
                        h[i] = tobf(f[i]);
                    }
                    const bool st   = colOk && y < a.H;
                    const size_t px = (size_t(q.b) * a.H + y) * a.W + 2 * j + par;
                    if (st && a.out)
                    {
                        uint32_t w[8];
#pragma unroll
                        for (int i = 0; i < 8; i++)
                            w[i] = uint32_t(h[2 * i]) | (uint32_t(h[2 * i + 1]) << 16);
                        uint4* o = reinterpret_cast<uint4*>(a.out + px * a.Cout + cb + c0);
                        o[0]     = make_uint4(w[0], w[1], w[2], w[3]);
                        o[1]     = make_uint4(w[4], w[5], w[6], w[7]);
                    }
                    if (st && a.out32)
                    {
                        float4* o = reinterpret_cast<float4*>(a.out32 + px * a.Cout + cb + c0);
#pragma unroll
                        for (int i = 0; i < 4; i++)
                            o[i] = make_float4(f[4 * i], f[4 * i + 1], f[4 * i + 2], f[4 * i + 3]);
                    }
                    // ((x00 + x01) + x10) + x11 over the stored BF16 values.
#pragma unroll
                    for (int i = 0; i < 16; i++)
                        psum[i] = acc == 0 ? bfv(h[i]) : psum[i] + bfv(h[i]);
                }
                if (step == 2 && colOk && q.y0 + r + 1 < a.H)
                {
                    uint32_t w[8];
#pragma unroll
                    for (int i = 0; i < 8; i++)
                        w[i] = uint32_t(tobf(psum[2 * i] * 0.25f)) | (uint32_t(tobf(psum[2 * i + 1] * 0.25f)) << 16);
                    const size_t pp = (size_t(q.b) * (a.H >> 1) + ((q.y0 + r) >> 1)) * W2 + j;
                    uint4* o        = reinterpret_cast<uint4*>(a.pool + pp * a.Cout + cb + c0);
                    o[0]            = make_uint4(w[0], w[1], w[2], w[3]);
                    o[1]            = make_uint4(w[4], w[5], w[6], w[7]);
                }
            }
            tc::fenceBeforeSync();
            __syncwarp();
            if (lane == 0)
                tc::mbarArrive(&accEmpty[buf]);
        }
    }
    tc::fenceBeforeSync();
    __syncthreads();
    tc::fenceAfterSync();
    if (warp == 1)
        tc::tmemDealloc(tmem, 2 * kAccStride);
    if (!ok)
        atomicExch(&g_convError, 1);
}

// ----------------------------------------------------------------------------- host side

PFN_cuTensorMapEncodeTiled_v12000 encodeTiled()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// Even / odd view of a full-resolution NHWC BF16 tensor: (C, parity, W / 2, H, B), box 8 x 1 x 130.
cudaError_t mapPairs(CUtensorMap* m, const uint16_t* base, int B, int H, int W, int C)
{
    auto enc = encodeTiled();
    if (!enc)
        return cudaErrorNotSupported;
    cuuint64_t dims[5]    = { cuuint64_t(C), 2, cuuint64_t(W / 2), cuuint64_t(H), cuuint64_t(B) };
    cuuint64_t strides[4] = { cuuint64_t(C) * 2, cuuint64_t(C) * 4, cuuint64_t(W) * C * 2, cuuint64_t(H) * W * C * 2 };
    cuuint32_t box[5]     = { 8, 1, kHaloEntries, 1, 1 };
    cuuint32_t es[5]      = { 1, 1, 1, 1, 1 };
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<uint16_t*>(base), dims, strides, box, es,
        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// Plain view of a half-resolution NHWC BF16 tensor: (C, W0, H0, B), box 8 x 130.
cudaError_t mapRows(CUtensorMap* m, const uint16_t* base, int B, int H0, int W0, int C)
{
    auto enc = encodeTiled();
    if (!enc)
        return cudaErrorNotSupported;
    cuuint64_t dims[4]    = { cuuint64_t(C), cuuint64_t(W0), cuuint64_t(H0), cuuint64_t(B) };
    cuuint64_t strides[3] = { cuuint64_t(C) * 2, cuuint64_t(W0) * C * 2, cuuint64_t(H0) * W0 * C * 2 };
    cuuint32_t box[4]     = { 8, kHaloEntries, 1, 1 };
    cuuint32_t es[4]      = { 1, 1, 1, 1 };
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<uint16_t*>(base), dims, strides, box, es,
        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

int smCountOf(int dev)
{
    static int counts[64] = {};
    if (dev < 0 || dev >= 64)
        return 148;
    if (counts[dev] == 0)
    {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
            n = 148;
        counts[dev] = n;
    }
    return counts[dev];
}

} // namespace

// Output channels per tile: 64, 32 or 16, the widest that divides cout.  Narrow tiles keep two or
// more output rows per tile (the halo rows are shared between them, the 2x2 pool needs both rows
// of a pair) and move fewer weight bytes per MMA than 128-channel tiles would.
int convTileChannels(int cout) { return cout % 64 == 0 ? 64 : cout % 32 == 0 ? 32 : 16; }

// Output rows per tile: as many as the 256 accumulator columns of one TMEM buffer hold (2 x N each),
// at most 4.
int convTileRows(int n) { return std::min(4, std::max(1, 256 / (2 * n))); }

cudaError_t launchConv3x3(const ConvLaunch& c, cudaStream_t st)
{
    if (c.W % 2 || (c.up0 && c.H % 2) || (c.pool && c.H % 2))
        return cudaErrorInvalidValue;
    ConvTmaArgs a{};
    a.wpack = c.wpack;
    a.bias  = c.bias;
    a.out   = c.out;
    a.out32 = c.out32;
    a.pool  = c.pool;
    a.B = c.B, a.H = c.H, a.W = c.W, a.Cout = c.Cout, a.up0 = c.up0, a.relu = c.relu;
    a.N      = convTileChannels(c.Cout);
    a.nTiles = c.Cout / a.N;
    a.R      = convTileRows(a.N);
    if (c.pool && a.R < 2)
        return cudaErrorInvalidValue;
    a.G         = (c.C0 + c.C1) / 16;
    a.G0        = c.C0 / 16;
    a.tilesX    = (c.W / 2 + 127) / 128;
    a.rowBlocks = (c.H + a.R - 1) / a.R;
    long tiles  = long(c.B) * a.rowBlocks * a.tilesX * a.nTiles;
    if (tiles >= (1L << 31))
        return cudaErrorInvalidValue;
    a.numTiles   = int(tiles);
    a.aBytes     = uint32_t(a.R + 2) * 2 * kRowBytes;
    a.stageBytes = (a.aBytes + 9u * uint32_t(a.N) * 32u + 127u) & ~127u;
    a.stages     = int(std::min<size_t>(kMaxStages, kSmemBudget / a.stageBytes));
    if (a.stages < 2)
        return cudaErrorInvalidValue;
    CUtensorMap m0, m1;
    cudaError_t e = c.up0 ? mapRows(&m0, c.in0, c.B, c.H / 2, c.W / 2, c.C0) : mapPairs(&m0, c.in0, c.B, c.H, c.W, c.C0);
    if (e != cudaSuccess)
        return e;
    if (c.C1 > 0)
    {
        if ((e = mapPairs(&m1, c.in1, c.B, c.H, c.W, c.C1)) != cudaSuccess)
            return e;
    }
    else
        m1 = m0;
    // At least half of the SM's shared memory, so that one CTA (with all 512 TMEM columns) runs
    // per SM.
    const size_t smem = std::max<size_t>(size_t(a.stages) * a.stageBytes, 120 * 1024);
    if ((e = cudaFuncSetAttribute(k_conv3x3_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem))) !=
        cudaSuccess)
        return e;
    int dev = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess)
        return e;
    const int grid = int(std::min<long>(tiles, smCountOf(dev)));
    k_conv3x3_tma<<<grid, kThreads, smem, st>>>(m0, m1, a);
    return cudaGetLastError();
}

// Packs FP32 weights w[tap][ci][co] (9 x Cin x Cout) into the conv kernel's B layout (BF16): per
// channel tile and 16-channel input group, the 9 slices in (dy, dx) order, each N x 16 in the
// K-major core-matrix layout.  flip: pack the data-gradient weights instead, w'[tap'][co][ci] =
// w[8 - tap'][ci][co], so that the convolution over dY computes dX (its Cin is then the layer's
// Cout and vice versa).
__global__ void k_pack_conv_weights(const float* w, int Cin, int Cout, int flip, int nt, uint16_t* out)
{
    const int kCin = flip ? Cout : Cin, kCout = flip ? Cin : Cout;
    const long total = 9L * kCin * kCout;
    for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < total; i += long(gridDim.x) * blockDim.x)
    {
        const int n   = int(i % kCout); // kernel output channel
        const long kk = i / kCout;      // tap * kCin + c
        const int tap = int(kk / kCin), c = int(kk % kCin);
        const float v = flip ? w[(size_t(8 - tap) * Cin + n) * Cout + c] : w[(size_t(tap) * Cin + c) * Cout + n];
        const int G = kCin / 16, tile = n / nt, nn = n % nt;
        const size_t slice = (size_t(tile) * G + c / 16) * 9 + tap;
        const size_t off   = slice * nt * 16 + tc::sliceOffset(uint32_t(nn), uint32_t(c % 16)) / 2;
        out[off]           = __bfloat16_as_ushort(__float2bfloat16_rn(v));
    }
}

cudaError_t launchPackConvWeights(const float* w, int Cin, int Cout, int flip, uint16_t* out, cudaStream_t st)
{
    k_pack_conv_weights<<<256, 256, 0, st>>>(w, Cin, Cout, flip, convTileChannels(flip ? Cin : Cout), out);
    return cudaGetLastError();
}

cudaError_t takeConvError(int* flag)
{
    int zero      = 0;
    cudaError_t e = cudaMemcpyFromSymbol(flag, g_convError, sizeof(int));
    if (e != cudaSuccess)
        return e;
    return cudaMemcpyToSymbol(g_convError, &zero, sizeof(int));
}

} // namespace agb
