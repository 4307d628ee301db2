// Ray casting on the device: two-level BVH2 traversal (TLAS over instances, BLAS per mesh) with
// the traversal stack in shared memory, 128-bit node and triangle fetches, and the watertight
// ray/triangle test of Woop, Benthin and Wald (JCGT 2(1), 2013).
//
// This replaces the driver's hardware traversal behind TraceRay (Shaders/RayTrace.slang:185-270):
//   closest hit:  RAY_FLAG_FORCE_OPAQUE, tmin <= t < tmax, barycentrics (u, v) = weights of
//                 vertices 1 and 2 (Shaders/Geometry.slang:108-118);
//   shadow rays:  RAY_FLAG_ACCEPT_FIRST_HIT_AND_END_SEARCH | FORCE_OPAQUE, any hit ends the search.
//
// The triangle test uses explicit round-to-nearest intrinsics so that no multiply-add is
// contracted: the edge functions of two triangles sharing an edge are then computed from the same
// operands in the same order, which is what makes the test watertight.  Box tests are widened by
// a few ulp so they never reject a hit the triangle test accepts.
#pragma once

#include <type_traits>
#include <utility>

#include "agb_scene.cuh"

namespace agb
{

#ifndef AGB_STACK_ENTRIES
#define AGB_STACK_ENTRIES 48
#endif
constexpr int kStackSize = AGB_STACK_ENTRIES; // entries per thread; the BVH builder keeps TLAS + BLAS depth below
#ifndef AGB_SMEM_STACK
#define AGB_SMEM_STACK 24
#endif
// The first kSmemStack entries live in shared memory, the rest in local memory: a smaller shared
// stack leaves more of the SM's combined L1 / shared storage to the L1 cache.
constexpr int kSmemStack = AGB_SMEM_STACK < AGB_STACK_ENTRIES ? AGB_SMEM_STACK : AGB_STACK_ENTRIES;
// Depth budgets: a BLAS is built at most kBlasMaxDepth deep, which leaves at least kTlasMaxDepth
// levels of the stack to the TLAS beside one instance-exit marker and a spare entry; the TLAS
// builder takes whatever the deepest BLAS of the scene leaves (agb_instances_set).
constexpr int kTlasMaxDepth = 12;
constexpr int kBlasMaxDepth = kStackSize - kTlasMaxDepth - 2;

struct TraceCounters
{
    unsigned long long nodes;
    unsigned long long tris;
};

struct RayHit
{
    float t, u, v;
    int32_t inst, prim;
};

AGB_D float sel3(v3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

// Per-ray constants of the watertight test.
struct WtRay
{
    v3 o;
    int kx, ky, kz;
    float Sx, Sy, Sz;
};
AGB_D WtRay wtSetup(v3 o, v3 d)
{
    WtRay r;
    r.o      = o;
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    r.kz     = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    r.kx     = r.kz + 1 == 3 ? 0 : r.kz + 1;
    r.ky     = r.kx + 1 == 3 ? 0 : r.kx + 1;
    float dz = sel3(d, r.kz);
    if (dz < 0.f)
    {
        int t = r.kx;
        r.kx  = r.ky;
        r.ky  = t;
    }
    r.Sx = __fdiv_rn(sel3(d, r.kx), dz);
    r.Sy = __fdiv_rn(sel3(d, r.ky), dz);
    r.Sz = __fdiv_rn(1.f, dz);
    return r;
}

// Watertight test; accepts tmin <= t < tmax.
AGB_D bool wtIntersect(const WtRay& r, float4 a4, float4 b4, float4 c4, float tmin, float tmax,
    bool inclusive, float& t, float& u, float& v)
{
    v3 A = v3{ __fsub_rn(a4.x, r.o.x), __fsub_rn(a4.y, r.o.y), __fsub_rn(a4.z, r.o.z) };
    v3 B = v3{ __fsub_rn(b4.x, r.o.x), __fsub_rn(b4.y, r.o.y), __fsub_rn(b4.z, r.o.z) };
    v3 C = v3{ __fsub_rn(c4.x, r.o.x), __fsub_rn(c4.y, r.o.y), __fsub_rn(c4.z, r.o.z) };
    float Akz = sel3(A, r.kz), Bkz = sel3(B, r.kz), Ckz = sel3(C, r.kz);
    float Ax = __fsub_rn(sel3(A, r.kx), __fmul_rn(r.Sx, Akz));
    float Ay = __fsub_rn(sel3(A, r.ky), __fmul_rn(r.Sy, Akz));
    float Bx = __fsub_rn(sel3(B, r.kx), __fmul_rn(r.Sx, Bkz));
    float By = __fsub_rn(sel3(B, r.ky), __fmul_rn(r.Sy, Bkz));
    float Cx = __fsub_rn(sel3(C, r.kx), __fmul_rn(r.Sx, Ckz));
    float Cy = __fsub_rn(sel3(C, r.ky), __fmul_rn(r.Sy, Ckz));
    float U  = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
    float V  = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
    float W  = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
    if (U == 0.f || V == 0.f || W == 0.f)
    {
        // Edge functions that round to zero are re-evaluated in double (paper, section 3.4).
        U = float(__dsub_rn(__dmul_rn(double(Cx), double(By)), __dmul_rn(double(Cy), double(Bx))));
        V = float(__dsub_rn(__dmul_rn(double(Ax), double(Cy)), __dmul_rn(double(Ay), double(Cx))));
        W = float(__dsub_rn(__dmul_rn(double(Bx), double(Ay)), __dmul_rn(double(By), double(Ax))));
    }
    if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f))
        return false;
    float det = __fadd_rn(__fadd_rn(U, V), W);
    if (det == 0.f)
        return false;
    float Az = __fmul_rn(r.Sz, Akz), Bz = __fmul_rn(r.Sz, Bkz), Cz = __fmul_rn(r.Sz, Ckz);
    float Tn  = __fadd_rn(__fadd_rn(__fmul_rn(U, Az), __fmul_rn(V, Bz)), __fmul_rn(W, Cz));
    float rcp = __fdiv_rn(1.f, det);
    float tt  = __fmul_rn(Tn, rcp);
    if (!(tt >= tmin && (tt < tmax || (inclusive && tt == tmax))))
        return false;
    t = tt;
    u = __fmul_rn(V, rcp);
    v = __fmul_rn(W, rcp);
    return true;
}

// Affine transform of a ray into object space, unrounded-contraction-free so that host and device
// agree: ((m0 x + m1 y) + m2 z) + m3.
AGB_D v3 xfPointRn(const float* m, v3 p)
{
    return v3{ __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[0], p.x), __fmul_rn(m[1], p.y)),
                             __fmul_rn(m[2], p.z)), m[3]),
        __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[4], p.x), __fmul_rn(m[5], p.y)),
                      __fmul_rn(m[6], p.z)), m[7]),
        __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[8], p.x), __fmul_rn(m[9], p.y)),
                      __fmul_rn(m[10], p.z)), m[11]) };
}
AGB_D v3 xfVectorRn(const float* m, v3 v)
{
    return v3{ __fadd_rn(__fadd_rn(__fmul_rn(m[0], v.x), __fmul_rn(m[1], v.y)), __fmul_rn(m[2], v.z)),
        __fadd_rn(__fadd_rn(__fmul_rn(m[4], v.x), __fmul_rn(m[5], v.y)), __fmul_rn(m[6], v.z)),
        __fadd_rn(__fadd_rn(__fmul_rn(m[8], v.x), __fmul_rn(m[9], v.y)), __fmul_rn(m[10], v.z)) };
}

struct SlabRay
{
    v3 inv;  // 1 / direction (tiny components clamped)
    v3 oinv; // origin * inv
};
// Reciprocal with about 1 ulp error (PTX rcp.approx); the slab test only culls, and its boxes are
// widened by about 8 ulp, so it does not need a correctly rounded reciprocal.
AGB_D float rcpApprox(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
AGB_D SlabRay slabSetup(v3 o, v3 d)
{
    const float eps = 1e-20f;
    float dx = fabsf(d.x) > eps ? d.x : copysignf(eps, d.x);
    float dy = fabsf(d.y) > eps ? d.y : copysignf(eps, d.y);
    float dz = fabsf(d.z) > eps ? d.z : copysignf(eps, d.z);
    SlabRay s;
    s.inv  = v3{ rcpApprox(dx), rcpApprox(dy), rcpApprox(dz) };
    s.oinv = v3{ o.x * s.inv.x, o.y * s.inv.y, o.z * s.inv.z };
    return s;
}
// Three-operand minimum / maximum (one instruction each on sm_100 and later).
AGB_D float fmax3f(float a, float b, float c)
{
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
AGB_D float fmin3f(float a, float b, float c)
{
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
// Two child boxes of a node against [tmin, tmax] (tmin >= 0); returns entry distances.
AGB_D void slab2(const SlabRay& s, float4 c0xy, float4 c1xy, float4 cz, float tmin, float tmax,
    bool& h0, bool& h1, float& t0, float& t1)
{
    // Box planes at lo/hi per axis, entry/exit distances with one FMA each.
    float a0 = fmaf(c0xy.x, s.inv.x, -s.oinv.x), b0 = fmaf(c0xy.y, s.inv.x, -s.oinv.x);
    float a1 = fmaf(c0xy.z, s.inv.y, -s.oinv.y), b1 = fmaf(c0xy.w, s.inv.y, -s.oinv.y);
    float a2 = fmaf(cz.x, s.inv.z, -s.oinv.z), b2 = fmaf(cz.y, s.inv.z, -s.oinv.z);
    float n0 = fmax3f(fminf(a0, b0), fminf(a1, b1), fmaxf(fminf(a2, b2), tmin));
    float f0 = fmin3f(fmaxf(a0, b0), fmaxf(a1, b1), fminf(fmaxf(a2, b2), tmax));
    float c0 = fmaf(c1xy.x, s.inv.x, -s.oinv.x), d0 = fmaf(c1xy.y, s.inv.x, -s.oinv.x);
    float c1 = fmaf(c1xy.z, s.inv.y, -s.oinv.y), d1 = fmaf(c1xy.w, s.inv.y, -s.oinv.y);
    float c2 = fmaf(cz.z, s.inv.z, -s.oinv.z), d2 = fmaf(cz.w, s.inv.z, -s.oinv.z);
    float n1 = fmax3f(fminf(c0, d0), fminf(c1, d1), fmaxf(fminf(c2, d2), tmin));
    float f1 = fmin3f(fmaxf(c0, d0), fmaxf(c1, d1), fminf(fmaxf(c2, d2), tmax));
    // Conservative widening (about 16 ulp relative plus an absolute floor).  The entry distance
    // is at least tmin >= 0, so widening the exit distance alone covers both ends: a box whose
    // exit lies behind the origin (f < 0) is not hit.
    const float kWiden2 = 1.0000020f;
    h0 = n0 <= fmaf(f0, kWiden2, 1e-30f);
    h1 = n1 <= fmaf(f1, kWiden2, 1e-30f);
    t0 = n0;
    t1 = n1;
}

// ------------------------------------------------------------------ persistent traversal
// Each warp loops over a shared work counter: lanes whose ray has finished take the next ray
// indices (one atomic per warp per refill), so no lane idles while a slower ray in its warp is
// still traversing (Aila & Laine, "Understanding the Efficiency of Ray Traversal on GPUs",
// HPG 2009: persistent threads, while-while traversal with postponed leaves).
//
// Every outer iteration has three phases with uniform work inside each, so the lanes of a warp run
// the same instructions together:
//   node phase      lanes step through internal nodes (TLAS or BLAS).  A lane that reaches a BLAS
//                   leaf parks it (in `leaf`, then `leaf2`) and keeps traversing speculatively
//                   until it holds kParkLeaves leaves and reaches another; a lane that reaches an
//                   instance boundary waits.  The phase ends once every lane holds a parked leaf,
//                   waits at a boundary or has finished.
//   leaf phase      lanes test the triangles of their parked leaves, one triangle per iteration.
//   boundary phase  lanes at a TLAS leaf enter its instance (object-space ray, watertight and slab
//                   setup); lanes at kExitInstance return to the world-space ray and the TLAS.
// Entering an instance pushes kExitInstance on the shared-memory stack; popping it restores the
// world-space ray and the TLAS.  A parked leaf belongs to the instance the lane is in, so a lane
// with a parked leaf stops at an instance boundary until the leaf has been tested.
//
// Closest hit keeps the smallest (t, instance, triangle): a triangle at exactly the current t
// replaces the hit only with a smaller (instance, triangle) key, so the result does not depend on
// traversal order (edges shared by two triangles give equal t).

constexpr int32_t kExitInstance = int32_t(0x80000000);
// No leaf ref equals kExitInstance or kDone: leaves hold at most 4 triangles (low 3 bits <= 3) and
// meshes at most 2^28 triangles.
constexpr int32_t kDone = int32_t(0x80000001);

// Leaf refs are the negative values above kDone (the two most negative values are the markers).
AGB_D bool isLeafRef(int32_t ref) { return uint32_t(ref) - uint32_t(kDone + 1) < 0x7fffffffu - 1u; }

#ifndef AGB_TRACE_PARK
#define AGB_TRACE_PARK 1
#endif
#ifndef AGB_NODE_EXIT
#define AGB_NODE_EXIT 8
#endif
#ifndef AGB_NODE_LOAD256
#define AGB_NODE_LOAD256 1
#endif
// One 32-byte read-only load (two float4) per lane: a node is two of them instead of four 16-byte
// loads, which halves the L1 wavefronts of the divergent node fetches.  p must be 32-byte aligned.
AGB_D void ldg256(const float4* p, float4& a, float4& b)
{
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}
#ifndef AGB_SHADOW_PARK
#define AGB_SHADOW_PARK 2
#endif
#ifndef AGB_SHADOW_NODE_EXIT
#define AGB_SHADOW_NODE_EXIT AGB_NODE_EXIT
#endif
// Leaves a lane may park before it stops in the node phase (1 or 2): closest-hit and any-hit rays.
constexpr int kParkLeavesClosest = AGB_TRACE_PARK;
constexpr int kParkLeavesAny     = AGB_SHADOW_PARK;
// The node phase also ends once fewer than this many lanes are still searching for their first
// leaf while some lane holds a parked leaf (0: only when none is searching).
constexpr int kNodeExitLanesClosest = AGB_NODE_EXIT;
constexpr int kNodeExitLanesAny     = AGB_SHADOW_NODE_EXIT;

// A Writer whose kRestart is true is called as write(scene, ray, hit?, hit, tmin) and returns
// false to trace the same ray again from the tmin it sets (transparent shadows walk the hits
// along the ray this way); other writers are called as write(ray, hit?, hit) and end the ray.
template <class W, class = void>
struct WriterRestarts
{
    static constexpr bool value = false;
};
template <class W>
struct WriterRestarts<W, std::void_t<decltype(W::kRestart)>>
{
    static constexpr bool value = W::kRestart;
};

// The TLAS root a ray starts from: the scene's, or the loader's own per-ray root (batched waves,
// where rays of several scenes share a queue).
template <class L, class = void>
struct LoaderHasRoot : std::false_type
{
};
template <class L>
struct LoaderHasRoot<L, decltype(void(std::declval<const L&>().root(0u)))> : std::true_type
{
};
template <class Loader>
AGB_D int32_t rayRoot(const Loader& load, const DevScene& s, uint32_t i)
{
    if constexpr (LoaderHasRoot<Loader>::value)
        return load.root(i);
    else
        return s.instanceCount > 0 ? s.tlasRoot : kDone;
}

template <bool kAnyHit, bool kCount, class Loader, class Writer>
AGB_D void persistentTrace(const DevScene& s, uint32_t n, uint32_t* work, const Loader& load,
    const Writer& write, int32_t* stack, int stride, TraceCounters& cnt, bool& overflow)
{
    constexpr int kParkLeaves    = kAnyHit ? kParkLeavesAny : kParkLeavesClosest;
    constexpr int kNodeExitLanes = kAnyHit ? kNodeExitLanesAny : kNodeExitLanesClosest;
    static_assert(kParkLeaves == 1 || kParkLeaves == 2, "one or two parked leaves");
    const unsigned FULL = 0xffffffffu;
    const int lane      = threadIdx.x & 31;
    bool active = false, exhausted = false;
    uint32_t rayIdx = 0;
    v3 o = splat(0.f), d = splat(0.f);
    float tmin = 0.f, tmax = 0.f, tmaxRay = 0.f;
    SlabRay sr;
    WtRay wr;
    int32_t ref = kDone, leaf = 0, leaf2 = 0;
    int sp       = 0;
    int32_t inst = -1;
    const float4* nodes = nullptr;
    const float4* tris  = nullptr;
    RayHit hit;
    bool found = false;
    int32_t spill[kStackSize > kSmemStack ? kStackSize - kSmemStack : 1];
    auto pop = [&]() -> int32_t {
        if (sp == 0)
            return kDone;
        sp--;
        if (kStackSize == kSmemStack || sp < kSmemStack)
            return stack[sp * stride];
        return spill[sp - kSmemStack];
    };
    auto push = [&](int32_t v) {
        if (kStackSize == kSmemStack || sp < kSmemStack)
            stack[sp * stride] = v;
        else
            spill[sp - kSmemStack] = v;
        sp++;
    };
    for (;;)
    {
        // Refill lanes whose ray is done.
        bool need         = !active && !exhausted;
        unsigned needMask = __ballot_sync(FULL, need);
        if (needMask)
        {
            int leader    = __ffs(needMask) - 1;
            uint32_t base = 0;
            if (lane == leader)
                base = atomicAdd(work, uint32_t(__popc(needMask)));
            base = __shfl_sync(FULL, base, leader);
            if (need)
            {
                rayIdx = base + uint32_t(__popc(needMask & ((1u << lane) - 1u)));
                if (rayIdx < n)
                {
                    load(rayIdx, o, d, tmin, tmax);
                    tmaxRay  = tmax;
                    sr       = slabSetup(o, d);
                    ref      = rayRoot(load, s, rayIdx);
                    leaf     = 0;
                    leaf2    = 0;
                    sp       = 0;
                    inst     = -1;
                    nodes    = reinterpret_cast<const float4*>(s.tlas);
                    found    = false;
                    hit.inst = hit.prim = -1;
                    hit.t = hit.u = hit.v = 0.f;
                    active   = true;
                }
                else
                    exhausted = true;
            }
        }
        if (__all_sync(FULL, exhausted))
            break;

        // Node phase: internal nodes only.  A lane stops at a BLAS leaf once it holds kParkLeaves
        // parked leaves (until then it parks the leaf and goes on speculatively), at an instance
        // boundary (TLAS leaf or kExitInstance) or at the end of its ray.
        for (;;)
        {
            if (active && inst >= 0 && isLeafRef(ref))
            {
                if (leaf == 0)
                {
                    leaf = ref;
                    ref  = pop();
                }
                else if (kParkLeaves > 1 && leaf2 == 0)
                {
                    leaf2 = ref;
                    ref   = pop();
                }
            }
            bool nodeWork      = active && ref >= 0;
            unsigned searching = __ballot_sync(FULL, nodeWork && leaf == 0);
            if (searching == 0)
                break;
            if (kNodeExitLanes > 0 && __popc(searching) < kNodeExitLanes && __any_sync(FULL, leaf != 0))
                break;
            if (!nodeWork)
                continue;
            const float4* np = nodes + 4 * size_t(ref);
            float4 c0xy, c1xy, cz;
            int4 refs;
#if AGB_NODE_LOAD256
            ldg256(np, c0xy, c1xy);
            {
                float4 r4;
                ldg256(np + 2, cz, r4);
                refs = make_int4(__float_as_int(r4.x), __float_as_int(r4.y), __float_as_int(r4.z),
                    __float_as_int(r4.w));
            }
#else
            c0xy = __ldg(np), c1xy = __ldg(np + 1), cz = __ldg(np + 2);
            refs = __ldg(reinterpret_cast<const int4*>(np + 3));
#endif
            if (kCount)
                cnt.nodes++;
            bool h0, h1;
            float t0, t1;
            slab2(sr, c0xy, c1xy, cz, tmin, tmax, h0, h1, t0, t1);
            if (h0 && h1)
            {
                if (sp >= kStackSize - 1)
                {
                    overflow = true;
                    ref = kDone, leaf = leaf2 = 0, sp = 0;
                    continue;
                }
                push(t0 <= t1 ? refs.y : refs.x);
                ref = t0 <= t1 ? refs.x : refs.y;
            }
            else if (h0 || h1)
                ref = h0 ? refs.x : refs.y;
            else
                ref = pop();
        }

        // Leaf phase: one triangle per lane per iteration over the lanes' parked leaves, so lanes
        // whose leaves hold different triangle counts do not wait for one another leaf by leaf.
        uint32_t cur = 0, end = 0;
        if (leaf != 0)
        {
            uint32_t code = uint32_t(~leaf);
            cur           = code >> 3;
            end           = cur + (code & 7u) + 1u;
            leaf          = 0;
        }
        while (__any_sync(FULL, cur < end))
        {
            if (cur >= end)
                continue;
            const float4* tp = tris + 3 * size_t(cur);
            float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
            if (kCount)
                cnt.tris++;
            cur++;
            if (cur == end && leaf2 != 0)
            {
                uint32_t code = uint32_t(~leaf2);
                cur           = code >> 3;
                end           = cur + (code & 7u) + 1u;
                leaf2         = 0;
            }
            float t, u, v;
            if (wtIntersect(wr, a, b, c, tmin, tmax, !kAnyHit && found, t, u, v))
            {
                int32_t prim = __float_as_int(a.w);
                if (!found || t < tmax || inst < hit.inst || (inst == hit.inst && prim < hit.prim))
                {
                    found    = true;
                    tmax     = t;
                    hit.t    = t;
                    hit.u    = u;
                    hit.v    = v;
                    hit.inst = inst;
                    hit.prim = prim;
                }
                if (kAnyHit)
                {
                    ref = kDone, sp = 0;
                    cur = end = 0;
                    leaf2     = 0;
                }
            }
        }

        // Instance boundaries, taken together by the lanes that reached one.
        if (active && ref == kExitInstance)
        {
            inst  = -1;
            nodes = reinterpret_cast<const float4*>(s.tlas);
            sr    = slabSetup(o, d);
            ref   = pop();
        }
        else if (active && inst < 0 && isLeafRef(ref))
        {
            // TLAS leaf: one instance (the TLAS is built with single-instance leaves).
            if (sp >= kStackSize - 1)
            {
                overflow = true;
                ref = kDone, sp = 0;
            }
            else
            {
                uint32_t first = uint32_t(~ref) >> 3;
                int32_t ii     = __ldg(s.tlasOrder + first);
                const DevInstance& in = s.instances[ii];
                const DevMesh& m      = s.meshes[in.mesh];
                push(kExitInstance);
                v3 oo = xfPointRn(in.w2o, o);
                v3 od = xfVectorRn(in.w2o, d);
                wr    = wtSetup(oo, od);
                sr    = slabSetup(oo, od);
                inst  = ii;
                nodes = reinterpret_cast<const float4*>(m.nodes);
                tris  = m.tris;
                ref   = m.root;
            }
        }
        if (active && ref == kDone)
        {
            if constexpr (WriterRestarts<Writer>::value)
            {
                if (write(s, rayIdx, found, hit, tmin))
                    active = false;
                else
                {
                    // Trace the ray again beyond the hit (the writer moved tmin past it).
                    ref      = rayRoot(load, s, rayIdx);
                    sp       = 0;
                    inst     = -1;
                    nodes    = reinterpret_cast<const float4*>(s.tlas);
                    sr       = slabSetup(o, d);
                    tmax     = tmaxRay;
                    found    = false;
                    hit.inst = hit.prim = -1;
                }
            }
            else
            {
                write(rayIdx, found, hit);
                active = false;
            }
        }
    }
}

} // namespace agb
