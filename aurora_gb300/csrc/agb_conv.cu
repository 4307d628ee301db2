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
// A staged row is one TMA box (16 channels x 130 entries, 32 bytes per entry) in the K-major
// 32-byte-swizzled layout: the 16-byte halves of entry i sit at 32 i and 32 i + 16, exchanged when
// bit 7 of the address is set.  Both the TMA write and the MMA read apply the swizzle to the shared
// memory address itself, so an A descriptor started 32 bytes per entry of offset later addresses
// the run: every staged byte is a whole 32-byte sector of the source (one request per entry).
//
// Roles (320 threads, one CTA per SM, static round-robin over tiles):
//   warp 0   TMA producer: per 16-channel group, (R + 2) x 2 halo rows (E, O) (or the fewer
//            half-resolution rows of an upsampled input) by cp.async.bulk.tensor
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

namespace
{

constexpr int kHaloEntries      = 130;               // 128 MMA rows + offsets 0..2
constexpr uint32_t kEntryBytes  = 32;                // 16 channels of one entry
constexpr uint32_t kBoxBytes    = kHaloEntries * kEntryBytes; // one TMA box: 16 channels x 130 entries
constexpr uint32_t kRowBytes    = 4352;              // kBoxBytes rounded up to 256 (the swizzle atom)
constexpr int kThreads          = 320; // producer, MMA issuer, 8 epilogue warps
constexpr uint32_t kAccStride   = 256;               // TMEM columns per accumulator buffer
constexpr int kMaxStages        = 4;
constexpr size_t kSmemBudget    = 226 * 1024; // of the 227 KB a CTA may have, static shared memory aside

struct ConvTmaArgs
{
    const uint16_t* wpack; // per (channel tile, group): 9 slices (dy, dx) of N x 16, B layout
    const float* bias;     // [Cout] or null
    uint16_t* out;         // [B][H][W][Cout] or null
    float* out32;          // [B][H][W][Cout] or null
    uint16_t* pool;        // [B][H/2][W/2][Cout] or null (2x2 average of the BF16 outputs)
    float4* rad;           // [B][H][W] RGBA radiance or null (the denoiser's output layer)
    const uint16_t* radIn; // [B][H][W][16] features (log1p noisy radiance in channels 0-2)
    int* error;            // set to 1 when a bounded wait runs out
    float* g0;             // data-gradient split (see ConvLaunch)
    float* g1;
    int gC0, gUp;
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

// Waits until the grid this one programmatically depends on has completed and its memory is
// visible (returns at once when the launch had no programmatic dependency), then lets the next
// grid in the stream begin its own prologue.
__device__ __forceinline__ void gridDependencyWait()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// One 32-byte store (the address 32-byte aligned): a whole sector per lane.
__device__ __forceinline__ void st256(void* p, const uint32_t (&w)[8])
{
    asm volatile("st.global.v8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "r"(w[0]), "r"(w[1]), "r"(w[2]),
        "r"(w[3]), "r"(w[4]), "r"(w[5]), "r"(w[6]), "r"(w[7])
                 : "memory");
}

__device__ __forceinline__ float bfv(uint16_t b) { return __uint_as_float(uint32_t(b) << 16); }

// Output rows per tile for N output channels: as many as one TMEM buffer of 256 columns holds
// (2 R N), at most 4 (six rows for 16 channels measured slower: 77 against 66 us for the output
// layer at 1920x1080).
__host__ __device__ constexpr int tileRows(int n) { return n >= 64 ? 2 : 4; }

// The MMAs of one pipeline stage (one 16-channel input group), fully unrolled.  Halo row i (input
// row y0 - 1 + i) feeds output rows r = i - 2 .. i (those inside the tile) through the vertical taps
// dy = i - r; their accumulators are adjacent in TMEM and the weight slices of the three dy are
// stacked (dy = 2, 1, 0), so one MMA per (halo row, parity, dx) covers every output row the halo
// row feeds: N, 2N or 3N accumulator columns at once.  In the first group of a tile an
// accumulator starts its sum (accumulate = 0) with the dx = 0 MMA of halo row r, split off as an
// MMA of its own.
template <int N, bool UP>
__device__ __forceinline__ void issueStage(uint32_t aAddr, uint32_t bAddr, uint32_t dBase, bool first)
{
    constexpr int R = tileRows(N);
    // K-major, 32-byte swizzle: entries of 32 bytes (16 channels), 8-entry atoms 256 bytes apart.
    const uint64_t aDesc0 = tc::smemDescSw32(aAddr, 256);
    const uint64_t bDesc0 = tc::smemDesc(bAddr, tc::kSliceLbo, tc::kSliceSbo);
#pragma unroll
    for (int i = 0; i < R + 2; i++)
    {
        const int rLo   = i - 2 > 0 ? i - 2 : 0;
        const int rHi   = i < R - 1 ? i : R - 1;
        const int count = rHi - rLo + 1;
#pragma unroll
        for (int par = 0; par < 2; par++)
#pragma unroll
            for (int dx = 0; dx < 3; dx++)
            {
                // Entry offset of the run: 0, 1, 1 (even outputs), 1, 1, 2 (odd outputs).
                const uint32_t shift = par == 0 ? (dx == 0 ? 0u : 1u) : (dx == 2 ? 2u : 1u);
                uint32_t row;
                if (UP)
                    row = uint32_t(((i - 1) >> 1) + 1); // half-resolution row of input row y0 - 1 + i
                else
                {
                    // E for the centre tap of even outputs and the side taps of odd outputs.
                    const int odd = par == 0 ? (dx == 1 ? 0 : 1) : (dx == 1 ? 1 : 0);
                    row           = uint32_t(i * 2 + odd);
                }
                const uint64_t ad = aDesc0 + ((row * kRowBytes + shift * kEntryBytes) >> 4);
                const uint64_t bd =
                    bDesc0 + ((uint32_t(dx) * 3u * N * 32u + uint32_t(2 - (i - rLo)) * N * 32u) >> 4);
                const uint32_t d = dBase + uint32_t((par * R + rLo) * N);
                if (first && dx == 0 && i <= R - 1)
                {
                    if (count > 1)
                        tc::mma(d, ad, bd, tc::idescBf16(128, uint32_t((count - 1) * N)), 1u);
                    tc::mma(d + uint32_t((count - 1) * N), ad, bd + ((uint32_t(count - 1) * N * 32u) >> 4),
                        tc::idescBf16(128, uint32_t(N)), 0u);
                }
                else
                    tc::mma(d, ad, bd, tc::idescBf16(128, uint32_t(count * N)), 1u);
            }
    }
}

template <int N, bool SPLIT>
__global__ void __launch_bounds__(kThreads, 1) k_conv3x3_tma(const __grid_constant__ CUtensorMap tm0,
    const __grid_constant__ CUtensorMap tm1, const ConvTmaArgs a)
{
    constexpr int R = tileRows(N);
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t full[kMaxStages], empty[kMaxStages], accFull[2], accEmpty[2], drain;
    __shared__ uint32_t tmemBase;
    const int tid  = threadIdx.x;
    const int warp = tid >> 5;
    const int lane = tid & 31;
    const int S    = a.stages;

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
    // Programmatic dependent launch: the prologue above may overlap the previous kernel's tail;
    // everything below reads or writes memory that kernel may still touch.
    gridDependencyWait();

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
                    tc::mbarExpectTx(&full[s], wBytes + uint32_t(rows) * kBoxBytes);
                    tc::bulkLoad(Bw, a.wpack + (size_t(q.nt) * a.G + g) * 9 * size_t(N) * 16, wBytes, &full[s]);
                    if (up)
                    {
                        const int h0 = upRowBase(q.y0);
                        for (int i = 0; i < rows; i++)
                            tc::tensorLoad4(A + i * kRowBytes, map, c, q.j0 - 1, h0 + i, q.b, &full[s]);
                    }
                    else
                    {
                        for (int i = 0; i < R + 2; i++)
                            for (int p = 0; p < 2; p++)
                                tc::tensorLoad5(A + (i * 2 + p) * kRowBytes, map, c, p,
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
            uint32_t it = 0;
            int k       = 0;
            for (int t = blockIdx.x; t < a.numTiles && ok; t += gridDim.x, k++)
            {
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
                    if (g < a.G0 && a.up0)
                        issueStage<N, true>(aAddr, bAddr, dBase, g == 0);
                    else
                        issueStage<N, false>(aAddr, bAddr, dBase, g == 0);
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
        // The data-gradient split is its own instantiation: the forward epilogue keeps its registers.
        constexpr bool split = SPLIT;
        // An item is a row pair x 16 channels: its four accumulators are loaded before one wait,
        // and a pool or an upsample gradient finds its 2x2 blocks in them (R is even).
        constexpr int step = 2;
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
                // Accumulator (row r, parity p) at columns (p R + r) N.
                tc::tmemLoad16(tBase + uint32_t(r * N + c0), v[0]);
                tc::tmemLoad16(tBase + uint32_t((R + r) * N + c0), v[1]);
                tc::tmemLoad16(tBase + uint32_t((r + 1) * N + c0), v[2]);
                tc::tmemLoad16(tBase + uint32_t((R + r + 1) * N + c0), v[3]);
                tc::tmemWaitLoad();
                float bv[16];
                if (a.bias)
                {
                    const float4* bp = reinterpret_cast<const float4*>(a.bias + cb + c0);
#pragma unroll
                    for (int i = 0; i < 4; i++)
                    {
                        const float4 t4 = __ldg(bp + i);
                        bv[4 * i]       = t4.x;
                        bv[4 * i + 1]   = t4.y;
                        bv[4 * i + 2]   = t4.z;
                        bv[4 * i + 3]   = t4.w;
                    }
                }
                else
                {
#pragma unroll
                    for (int i = 0; i < 16; i++)
                        bv[i] = 0.f;
                }
                float psum[16], gsum[16];
                const int cch   = cb + c0; // output channel of the chunk
                const bool toG0 = split && cch < a.gC0;
#pragma unroll
                for (int acc = 0; acc < 4; acc++)
                {
                    if (acc >= 2 * step)
                        break;
                    const int par = acc & 1;
                    const int y   = q.y0 + r + (acc >> 1);
                    float f[16];
#pragma unroll
                    for (int i = 0; i < 16; i++)
                    {
                        f[i] = __uint_as_float(v[acc][i]) + bv[i];
                        if (a.relu)
                            f[i] = fmaxf(f[i], 0.f);
                    }
                    // BF16 pairs, round to nearest even (low half = the even channel).
                    uint32_t w[8];
#pragma unroll
                    for (int i = 0; i < 8; i++)
                    {
                        const __nv_bfloat162 h2 = __floats2bfloat162_rn(f[2 * i], f[2 * i + 1]);
                        w[i]                    = *reinterpret_cast<const uint32_t*>(&h2);
                    }
                    const bool st   = colOk && y < a.H;
                    const size_t px = (size_t(q.b) * a.H + y) * a.W + 2 * j + par;
                    if (st && a.out)
                        st256(a.out + px * a.Cout + cb + c0, w);
                    if (st && a.out32)
                    {
                        uint32_t w0[8], w1[8];
#pragma unroll
                        for (int i = 0; i < 8; i++)
                        {
                            w0[i] = __float_as_uint(f[i]);
                            w1[i] = __float_as_uint(f[8 + i]);
                        }
                        st256(a.out32 + px * a.Cout + cb + c0, w0);
                        st256(a.out32 + px * a.Cout + cb + c0 + 8, w1);
                    }
                    if (st && a.rad && c0 == 0)
                    {
                        const uint16_t* xin = a.radIn + px * 16;
                        a.rad[px] = make_float4(fmaxf(expm1f(f[0] + bfv(__ldg(xin + 0))), 0.f),
                            fmaxf(expm1f(f[1] + bfv(__ldg(xin + 1))), 0.f), fmaxf(expm1f(f[2] + bfv(__ldg(xin + 2))), 0.f),
                            1.f);
                    }
                    if (split)
                    {
                        if (toG0 && a.gUp)
                        {
                            // 2x2 block sum ((x00 + x01) + x10) + x11, added below.
#pragma unroll
                            for (int i = 0; i < 16; i++)
                                gsum[i] = acc == 0 ? f[i] : gsum[i] + f[i];
                        }
                        else if (st)
                        {
                            float* g   = toG0 ? a.g0 + px * a.gC0 + cch : a.g1 + px * (a.Cout - a.gC0) + (cch - a.gC0);
                            float4* g4 = reinterpret_cast<float4*>(g);
#pragma unroll
                            for (int i = 0; i < 4; i++)
                            {
                                float4 o = g4[i];
                                o.x += f[4 * i];
                                o.y += f[4 * i + 1];
                                o.z += f[4 * i + 2];
                                o.w += f[4 * i + 3];
                                g4[i] = o;
                            }
                        }
                    }
                    if (a.pool)
                    {
                        // ((x00 + x01) + x10) + x11 over the stored BF16 values.
#pragma unroll
                        for (int i = 0; i < 8; i++)
                        {
                            const float lo = __uint_as_float(w[i] << 16), hi = __uint_as_float(w[i] & 0xFFFF0000u);
                            psum[2 * i]     = acc == 0 ? lo : psum[2 * i] + lo;
                            psum[2 * i + 1] = acc == 0 ? hi : psum[2 * i + 1] + hi;
                        }
                    }
                }
                if (split && toG0 && a.gUp && colOk && q.y0 + r + 1 < a.H)
                {
                    const size_t pp = (size_t(q.b) * (a.H >> 1) + ((q.y0 + r) >> 1)) * W2 + j;
                    float4* g4      = reinterpret_cast<float4*>(a.g0 + pp * a.gC0 + cch);
#pragma unroll
                    for (int i = 0; i < 4; i++)
                    {
                        float4 o = g4[i];
                        o.x += gsum[4 * i];
                        o.y += gsum[4 * i + 1];
                        o.z += gsum[4 * i + 2];
                        o.w += gsum[4 * i + 3];
                        g4[i] = o;
                    }
                }
                if (a.pool && colOk && q.y0 + r + 1 < a.H)
                {
                    uint32_t w[8];
#pragma unroll
                    for (int i = 0; i < 8; i++)
                    {
                        const __nv_bfloat162 h2 = __floats2bfloat162_rn(psum[2 * i] * 0.25f, psum[2 * i + 1] * 0.25f);
                        w[i]                    = *reinterpret_cast<const uint32_t*>(&h2);
                    }
                    const size_t pp = (size_t(q.b) * (a.H >> 1) + ((q.y0 + r) >> 1)) * W2 + j;
                    st256(a.pool + pp * a.Cout + cb + c0, w);
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
        atomicExch(a.error, 1);
}

// ----------------------------------------------------------------------------- weight gradient
// dW[tap][ci][co] += sum over pixels p of X[p + d(tap)][ci] dY[p][co], X = concat(up?(in0), in1):
// a tcgen05 GEMM with M = input channels, N = output channels and K = pixels, both operands
// MN-major (NHWC keeps a pixel's channels contiguous).  A unit of K is 128 output pixels of one
// row (64 pairs), split by parity as in the forward pass: dY is staged as its even and odd rows
// (64 entries each), X as the even and odd halo rows of 66 entries, so that the horizontal taps
// are K offsets of 0, 1 or 2 entries into the same staged rows (an upsampled source is staged at
// half resolution, the same row in both slots).  The vertical taps: when 3 x Cin <= 128 the M
// rows are (dy, ci) - the three halo rows' channel groups are stacked at a uniform stride, so one
// MMA covers all nine taps' rows for its horizontal tap - otherwise a work item takes one dy and
// 128 input channels.  Accumulators: the three horizontal taps x N columns in TMEM, summed over
// the item's units, then added to dW with vector reductions (red.global.add.v4.f32).
constexpr uint32_t kWgEntriesA = 66;   // 64 pairs + offsets 0..2
constexpr uint32_t kWgEntriesB = 64;
constexpr uint32_t kWgSlotA    = 2304; // 66 x 32 bytes rounded up to the 256-byte swizzle atom
constexpr uint32_t kWgSlotB    = 2048; // 64 x 32 bytes
constexpr int kWgThreads       = 192;  // producer, MMA issuer, 4 epilogue warps
constexpr int kWgMaxStages     = 6;

struct WgradTmaArgs
{
    float* dw;
    int B, H, W, Cin, Cout, C0, up0;
    int T;               // vertical taps per item: 3 (M = (dy, ci)) or 1 (M = ci)
    int Gci;             // 16-channel groups of X per tap in an item
    int ciTiles, coTiles, N, splits;
    int unitsX, numUnits, unitsPerItem, numItems;
    uint32_t stageBytes, aBytes;
    int stages;
    int* error;
};

template <int N>
__global__ void __launch_bounds__(kWgThreads, 1) k_conv_wgrad_tma(const __grid_constant__ CUtensorMap tm0,
    const __grid_constant__ CUtensorMap tm1, const __grid_constant__ CUtensorMap tmDy, const WgradTmaArgs a)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t full[kWgMaxStages], empty[kWgMaxStages], accFull;
    __shared__ uint32_t tmemBase;
    const int tid  = threadIdx.x;
    const int warp = tid >> 5;
    const int lane = tid & 31;
    const int S    = a.stages;
    // Item: (dy or all three, ci tile, co tile, unit range).
    int item      = blockIdx.x;
    const int sp  = item % a.splits;
    item /= a.splits;
    const int coT = item % a.coTiles;
    item /= a.coTiles;
    const int ciT  = item % a.ciTiles;
    const int dyIt = item / a.ciTiles; // the item's dy when T == 1
    const int u0   = sp * a.unitsPerItem;
    const int u1   = min(a.numUnits, u0 + a.unitsPerItem);

    if (warp == 1)
        tc::tmemAlloc(&tmemBase, 512);
    if (tid == 0)
    {
        for (int s = 0; s < S; s++)
        {
            tc::mbarInit(&full[s], 1);
            tc::mbarInit(&empty[s], 1);
        }
        tc::mbarInit(&accFull, 1);
        tc::fenceMbarInit();
    }
    tc::fenceBeforeSync();
    __syncthreads();
    tc::fenceAfterSync();
    const uint32_t tmem = tmemBase;
    bool ok             = true;
    // Programmatic dependent launch: the prologue above may overlap the previous kernel's tail;
    // everything below reads or writes memory that kernel may still touch.
    gridDependencyWait();

    if (warp == 0)
    {
        if (lane == 0)
        {
            uint32_t lastParity[kWgMaxStages];
            bool issued[kWgMaxStages];
            for (int s = 0; s < S; s++)
                issued[s] = false;
            const uint32_t bytesA = uint32_t(a.T * a.Gci) * 2u * kWgEntriesA * 32u;
            const uint32_t bytesB = uint32_t(N / 16) * 2u * kWgEntriesB * 32u;
            uint32_t it = 0;
            for (int u = u0; u < u1; u++, it++)
            {
                const int s       = int(it % uint32_t(S));
                const uint32_t ph = (it / uint32_t(S)) & 1u;
                if (!tc::mbarWait(&empty[s], ph ^ 1u))
                {
                    ok = false;
                    break;
                }
                const int xs = u % a.unitsX;
                const int r  = u / a.unitsX;
                const int y  = r % a.H;
                const int b  = r / a.H;
                const int j0 = xs * 64;
                uint8_t* A   = smem + size_t(s) * a.stageBytes;
                uint8_t* Bm  = A + a.aBytes;
                tc::mbarExpectTx(&full[s], bytesA + bytesB);
                // X: slot (parity p, tap row t, group g) at ((p * 8) + t * Gci + g) * kWgSlotA.
                for (int t = 0; t < a.T; t++)
                {
                    const int dy = a.T == 3 ? t : dyIt;
                    const int yi = y + dy - 1;
                    for (int g = 0; g < a.Gci; g++)
                    {
                        const int c = (a.T == 3 ? 0 : ciT * 128) + g * 16;
                        for (int p = 0; p < 2; p++)
                        {
                            uint8_t* dst = A + (p * 8 + t * a.Gci + g) * kWgSlotA;
                            if (c < a.C0 && a.up0)
                                tc::tensorLoad4(dst, &tm0, c, j0 - 1, yi >> 1, b, &full[s]);
                            else if (c < a.C0)
                                tc::tensorLoad5(dst, &tm0, c, p, j0 - 1, yi, b, &full[s]);
                            else
                                tc::tensorLoad5(dst, &tm1, c - a.C0, p, j0 - 1, yi, b, &full[s]);
                        }
                    }
                }
                // dY: slot (parity p, group g) at (p * N / 16 + g) * kWgSlotB.
                for (int g = 0; g < N / 16; g++)
                    for (int p = 0; p < 2; p++)
                        tc::tensorLoad5(Bm + (p * (N / 16) + g) * kWgSlotB, &tmDy, coT * N + g * 16, p, j0, y, b,
                            &full[s]);
                issued[s]     = true;
                lastParity[s] = ph;
            }
            for (int s = 0; s < S; s++)
                if (issued[s] && !tc::mbarWait(&full[s], lastParity[s]))
                    ok = false;
        }
        __syncwarp();
    }
    else if (warp == 1)
    {
        if (lane == 0)
        {
            // MN-major A and B (bits 15, 16), M = 128, N.
            const uint32_t idesc = tc::idescBf16(128, N) | (1u << 15) | (1u << 16);
            uint32_t it          = 0;
            bool first           = true;
            for (int u = u0; u < u1; u++, it++)
            {
                const int s       = int(it % uint32_t(S));
                const uint32_t ph = (it / uint32_t(S)) & 1u;
                if (!tc::mbarWait(&full[s], ph))
                {
                    ok = false;
                    break;
                }
                tc::fenceAfterSync();
                const uint32_t aAddr  = tc::smemAddr(smem + size_t(s) * a.stageBytes);
                const uint32_t bAddr  = aAddr + a.aBytes;
                // MN-major, 32-byte swizzle: 16-channel atoms a slot apart (leading byte offset), 8-entry
                // atoms 256 bytes apart (stride byte offset).
                const uint64_t aDesc0 = tc::smemDesc(aAddr, kWgSlotA, 256) | (uint64_t(6) << 61);
                const uint64_t bDesc0 = tc::smemDesc(bAddr, kWgSlotB, 256) | (uint64_t(6) << 61);
#pragma unroll
                for (int par = 0; par < 2; par++)
#pragma unroll
                    for (int dx = 0; dx < 3; dx++)
                    {
                        const uint32_t shift = par == 0 ? (dx == 0 ? 0u : 1u) : (dx == 2 ? 2u : 1u);
                        const uint32_t odd   = par == 0 ? (dx == 1 ? 0u : 1u) : (dx == 1 ? 1u : 0u);
                        const uint64_t ad    = aDesc0 + ((odd * 8u * kWgSlotA + shift * 32u) >> 4);
                        const uint64_t bd    = bDesc0 + ((uint32_t(par) * (N / 16) * kWgSlotB) >> 4);
#pragma unroll
                        for (int ks = 0; ks < 4; ks++)
                            tc::mma(tmem + uint32_t(dx * N), ad + ((uint32_t(ks) * 16u * 32u) >> 4),
                                bd + ((uint32_t(ks) * 16u * 32u) >> 4), idesc,
                                (first && par == 0 && ks == 0) ? 0u : 1u);
                    }
                first = false;
                tc::commit(&empty[s]);
            }
            tc::commit(&accFull);
            if (!tc::mbarWait(&accFull, 0))
                ok = false;
        }
        __syncwarp();
    }
    else
    {
        // Epilogue (warps 2-5): TMEM lane m = the M row of this thread.
        const int quad = warp & 3;
        const int m    = quad * 32 + lane;
        if (!leaderWait(&accFull, 0, lane))
            ok = false;
        else if (u1 > u0)
        {
            tc::fenceAfterSync();
            const int rowsPerTap = a.Gci * 16;
            const int t          = m / rowsPerTap;
            const int dy         = a.T == 3 ? t : dyIt;
            const int ci         = (a.T == 3 ? 0 : ciT * 128) + m % rowsPerTap;
            const bool valid     = t < a.T && ci < a.Cin;
            for (int dx = 0; dx < 3; dx++)
                for (int c0 = 0; c0 < N; c0 += 16)
                {
                    uint32_t v[16];
                    tc::tmemLoad16(tmem + (uint32_t(quad * 32) << 16) + uint32_t(dx * N + c0), v);
                    tc::tmemWaitLoad();
                    if (valid)
                    {
                        float* dst = a.dw + (size_t(dy * 3 + dx) * a.Cin + ci) * a.Cout + coT * N + c0;
#pragma unroll
                        for (int q = 0; q < 4; q++)
                            asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(dst + 4 * q),
                                "f"(__uint_as_float(v[4 * q])), "f"(__uint_as_float(v[4 * q + 1])),
                                "f"(__uint_as_float(v[4 * q + 2])), "f"(__uint_as_float(v[4 * q + 3]))
                                         : "memory");
                    }
                }
        }
    }
    tc::fenceBeforeSync();
    __syncthreads();
    tc::fenceAfterSync();
    if (warp == 1)
        tc::tmemDealloc(tmem, 512);
    if (!ok)
        atomicExch(a.error, 1);
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

// Even / odd view of a full-resolution NHWC BF16 tensor: (C, parity, W / 2, H, B), box 16 x 1 x
// entries, 32-byte swizzle.
cudaError_t mapPairs(CUtensorMap* m, const uint16_t* base, int B, int H, int W, int C, int entries = kHaloEntries)
{
    auto enc = encodeTiled();
    if (!enc)
        return cudaErrorNotSupported;
    cuuint64_t dims[5]    = { cuuint64_t(C), 2, cuuint64_t(W / 2), cuuint64_t(H), cuuint64_t(B) };
    cuuint64_t strides[4] = { cuuint64_t(C) * 2, cuuint64_t(C) * 4, cuuint64_t(W) * C * 2, cuuint64_t(H) * W * C * 2 };
    cuuint32_t box[5]     = { 16, 1, cuuint32_t(entries), 1, 1 };
    cuuint32_t es[5]      = { 1, 1, 1, 1, 1 };
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<uint16_t*>(base), dims, strides, box, es,
        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_32B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// Plain view of a half-resolution NHWC BF16 tensor: (C, W0, H0, B), box 16 x entries, 32-byte
// swizzle.
cudaError_t mapRows(CUtensorMap* m, const uint16_t* base, int B, int H0, int W0, int C, int entries = kHaloEntries)
{
    auto enc = encodeTiled();
    if (!enc)
        return cudaErrorNotSupported;
    cuuint64_t dims[4]    = { cuuint64_t(C), cuuint64_t(W0), cuuint64_t(H0), cuuint64_t(B) };
    cuuint64_t strides[3] = { cuuint64_t(C) * 2, cuuint64_t(W0) * C * 2, cuuint64_t(H0) * W0 * C * 2 };
    cuuint32_t box[4]     = { 16, cuuint32_t(entries), 1, 1 };
    cuuint32_t es[4]      = { 1, 1, 1, 1 };
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<uint16_t*>(base), dims, strides, box, es,
        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_32B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// Launch with programmatic stream serialisation: the kernel may start while the previous kernel
// in the stream finishes (its prologue overlaps that kernel's last wave).
template <typename... Args, typename... Params>
cudaError_t launchOverlapped(void (*kern)(Params...), unsigned grid, unsigned block, size_t smem, cudaStream_t st,
    Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim            = dim3(grid);
    cfg.blockDim           = dim3(block);
    cfg.dynamicSmemBytes   = smem;
    cfg.stream             = st;
    cudaLaunchAttribute attr[1];
    attr[0].id                                         = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs                                          = attr;
    cfg.numAttrs                                       = 1;
    return cudaLaunchKernelEx(&cfg, kern, args...);
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
__host__ __device__ int convTileChannels(int cout) { return cout % 64 == 0 ? 64 : cout % 32 == 0 ? 32 : 16; }

cudaError_t launchConv3x3(const ConvLaunch& c, cudaStream_t st)
{
    if (c.W % 2 || (c.up0 && c.H % 2) || (c.pool && c.H % 2))
        return cudaErrorInvalidValue;
    // Outputs are written in 32-byte pieces, the bias read in 16-byte ones.
    if (((reinterpret_cast<uintptr_t>(c.out) | reinterpret_cast<uintptr_t>(c.out32) | reinterpret_cast<uintptr_t>(c.pool)) &
            31u) ||
        (reinterpret_cast<uintptr_t>(c.bias) & 15u))
        return cudaErrorInvalidValue;
    ConvTmaArgs a{};
    a.wpack = c.wpack;
    a.bias  = c.bias;
    a.out   = c.out;
    a.out32 = c.out32;
    a.pool  = c.pool;
    a.rad   = reinterpret_cast<float4*>(c.radiance);
    a.radIn = c.radianceInput;
    a.g0    = c.grad0;
    a.g1    = c.grad1;
    a.gC0   = c.gradC0;
    a.gUp   = c.gradUp;
    if ((c.grad0 || c.grad1) && (c.gradC0 % 16 || (c.gradUp && c.H % 2) ||
                                    ((reinterpret_cast<uintptr_t>(c.grad0) | reinterpret_cast<uintptr_t>(c.grad1)) & 15u)))
        return cudaErrorInvalidValue;
    a.B = c.B, a.H = c.H, a.W = c.W, a.Cout = c.Cout, a.up0 = c.up0, a.relu = c.relu;
    a.N      = convTileChannels(c.Cout);
    a.nTiles = c.Cout / a.N;
    a.R      = tileRows(a.N);
    a.G         = (c.C0 + c.C1) / 16;
    a.G0        = c.C0 / 16;
    a.tilesX    = (c.W / 2 + 127) / 128;
    a.rowBlocks = (c.H + a.R - 1) / a.R;
    long tiles  = long(c.B) * a.rowBlocks * a.tilesX * a.nTiles;
    if (tiles >= (1L << 31))
        return cudaErrorInvalidValue;
    a.numTiles   = int(tiles);
    a.aBytes     = uint32_t(a.R + 2) * 2 * kRowBytes;
    a.stageBytes = (a.aBytes + 9u * uint32_t(a.N) * 32u + 1023u) & ~1023u;
    a.stages     = int(std::min<size_t>(kMaxStages, kSmemBudget / a.stageBytes));
    if (a.stages < 2)
        return cudaErrorInvalidValue;
    cudaError_t e0 = tcErrorFlag(&a.error);
    if (e0 != cudaSuccess)
        return e0;
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
    const bool split = c.grad0 || c.grad1;
    auto kern        = split ? (a.N == 64 ? k_conv3x3_tma<64, true> : a.N == 32 ? k_conv3x3_tma<32, true> : k_conv3x3_tma<16, true>)
                             : (a.N == 64 ? k_conv3x3_tma<64, false> : a.N == 32 ? k_conv3x3_tma<32, false> : k_conv3x3_tma<16, false>);
    if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem))) != cudaSuccess)
        return e;
    int dev = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess)
        return e;
    const int grid = int(std::min<long>(tiles, smCountOf(dev)));
    return launchOverlapped(kern, unsigned(grid), kThreads, smem, st, m0, m1, a);
}

cudaError_t launchConvWgrad(const ConvLaunch& c, const uint16_t* dy, float* dw, int smCount, cudaStream_t st)
{
    if (c.W % 2 || (c.up0 && c.H % 2) || (reinterpret_cast<uintptr_t>(dw) & 15u))
        return cudaErrorInvalidValue;
    WgradTmaArgs a{};
    a.dw = dw;
    a.B = c.B, a.H = c.H, a.W = c.W, a.Cin = c.C0 + c.C1, a.Cout = c.Cout, a.C0 = c.C0, a.up0 = c.up0;
    a.T       = 3 * a.Cin <= 128 ? 3 : 1;
    a.Gci     = a.T == 3 ? a.Cin / 16 : std::min(8, a.Cin / 16);
    a.ciTiles = a.T == 3 ? 1 : (a.Cin + 127) / 128;
    a.N       = c.Cout <= 128 ? c.Cout : (c.Cout % 128 == 0 ? 128 : 64);
    if (c.Cout % a.N || (a.N != 16 && a.N != 32 && a.N != 48 && a.N != 64 && a.N != 96 && a.N != 128))
        return cudaErrorInvalidValue;
    a.coTiles  = c.Cout / a.N;
    a.unitsX   = (c.W / 2 + 63) / 64;
    a.numUnits = c.B * c.H * a.unitsX;
    const int fixedItems = (a.T == 3 ? 1 : 3) * a.ciTiles * a.coTiles;
    const int sms        = smCount > 0 ? smCount : 148;
    a.splits       = std::max(1, std::min(a.numUnits, (2 * sms + fixedItems - 1) / fixedItems));
    a.unitsPerItem = (a.numUnits + a.splits - 1) / a.splits;
    a.splits       = (a.numUnits + a.unitsPerItem - 1) / a.unitsPerItem;
    a.numItems     = fixedItems * a.splits;
    a.aBytes       = 2u * 8u * kWgSlotA; // all eight M atoms of both parities (unloaded ones unused)
    a.stageBytes   = (a.aBytes + 2u * uint32_t(a.N / 16) * kWgSlotB + 1023u) & ~1023u;
    a.stages       = int(std::min<size_t>(kWgMaxStages, kSmemBudget / a.stageBytes));
    cudaError_t e  = tcErrorFlag(&a.error);
    if (e != cudaSuccess)
        return e;
    CUtensorMap m0, m1, md;
    e = c.up0 ? mapRows(&m0, c.in0, c.B, c.H / 2, c.W / 2, c.C0, kWgEntriesA)
              : mapPairs(&m0, c.in0, c.B, c.H, c.W, c.C0, kWgEntriesA);
    if (e != cudaSuccess)
        return e;
    if (c.C1 > 0)
    {
        if ((e = mapPairs(&m1, c.in1, c.B, c.H, c.W, c.C1, kWgEntriesA)) != cudaSuccess)
            return e;
    }
    else
        m1 = m0;
    if ((e = mapPairs(&md, dy, c.B, c.H, c.W, c.Cout, kWgEntriesB)) != cudaSuccess)
        return e;
    const size_t smem = std::max<size_t>(size_t(a.stages) * a.stageBytes, 120 * 1024);
    auto kern = a.N == 128 ? k_conv_wgrad_tma<128> : a.N == 96 ? k_conv_wgrad_tma<96> : a.N == 64 ? k_conv_wgrad_tma<64>
        : a.N == 48 ? k_conv_wgrad_tma<48> : a.N == 32 ? k_conv_wgrad_tma<32> : k_conv_wgrad_tma<16>;
    if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem))) != cudaSuccess)
        return e;
    return launchOverlapped(kern, unsigned(a.numItems), kWgThreads, smem, st, m0, m1, md, a);
}

// Packs FP32 weights w[tap][ci][co] (9 x Cin x Cout) into the conv kernel's B layout (BF16): per
// channel tile and 16-channel input group, for dx = 0, 1, 2 a stack of the three vertical taps'
// slices (dy = 2, 1, 0; N x 16 each) in the K-major core-matrix layout, so that any run of them is
// one B operand.  flip: pack the data-gradient weights instead, w'[tap'][co][ci] =
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
        const int dy = tap / 3, dx = tap % 3;
        const size_t stack = (size_t(tile) * G + c / 16) * 3 + dx;
        const uint32_t row = uint32_t((2 - dy) * nt + nn);
        const size_t off   = stack * 3 * nt * 16 + tc::sliceOffset(row, uint32_t(c % 16)) / 2;
        out[off]           = __bfloat16_as_ushort(__float2bfloat16_rn(v));
    }
}

struct PackJobs
{
    PackJob job[kMaxPackJobs];
    long first[kMaxPackJobs + 1]; // element offsets of the jobs
    int count;
};

// Position of element (tap, c, n) of a kCin x kCout layer in the packed B layout (tiles of nt).
__device__ __forceinline__ size_t packedOffset(int kCin, int nt, int tap, int c, int n)
{
    const int G = kCin / 16, tile = n / nt, nn = n % nt;
    const int dy = tap / 3, dx = tap % 3;
    const size_t stack = (size_t(tile) * G + c / 16) * 3 + dx;
    const uint32_t row = uint32_t((2 - dy) * nt + nn);
    return stack * 3 * nt * 16 + tc::sliceOffset(row, uint32_t(c % 16)) / 2;
}

__global__ void k_pack_conv_weights_many(const PackJobs jobs)
{
    const long total = jobs.first[jobs.count];
    for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < total; i += long(gridDim.x) * blockDim.x)
    {
        int k = 0;
        while (i >= jobs.first[k + 1])
            k++;
        const PackJob& J = jobs.job[k];
        const long e     = i - jobs.first[k]; // (tap, ci, co) in w's order
        const int co     = int(e % J.cout);
        const long kk    = e / J.cout;
        const int tap = int(kk / J.cin), ci = int(kk % J.cin);
        const uint16_t v = __bfloat16_as_ushort(__float2bfloat16_rn(J.w[e]));
        if (J.out)
            J.out[packedOffset(J.cin, convTileChannels(J.cout), tap, ci, co)] = v;
        if (J.outFlip)
            J.outFlip[packedOffset(J.cout, convTileChannels(J.cin), 8 - tap, co, ci)] = v;
    }
}

cudaError_t launchPackConvWeightsMany(const PackJob* jobs, int count, cudaStream_t st)
{
    if (count < 0 || count > kMaxPackJobs)
        return cudaErrorInvalidValue;
    PackJobs p{};
    p.count    = count;
    p.first[0] = 0;
    for (int k = 0; k < count; k++)
    {
        p.job[k]       = jobs[k];
        p.first[k + 1] = p.first[k] + 9L * jobs[k].cin * jobs[k].cout;
    }
    const long total = p.first[count];
    if (total == 0)
        return cudaSuccess;
    const unsigned grid = unsigned(std::min<long>((total + 255) / 256, 4096));
    k_pack_conv_weights_many<<<grid, 256, 0, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launchPackConvWeights(const float* w, int Cin, int Cout, int flip, uint16_t* out, cudaStream_t st)
{
    k_pack_conv_weights<<<256, 256, 0, st>>>(w, Cin, Cout, flip, convTileChannels(flip ? Cin : Cout), out);
    return cudaGetLastError();
}


} // namespace agb
