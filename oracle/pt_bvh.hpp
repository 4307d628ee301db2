// Oracle (test infrastructure, never linked into the product): CPU ray casting for the restated
// path tracer.  The reference delegates BVH build, traversal and intersection to the GPU driver
// (HGI/HGIGeometry.cpp:127-160, HGI/HGIScene.cpp:377-420, Shaders/RayTrace.slang:202-209,266), so
// there is no reference source to follow; the oracle uses
//   * watertight ray/triangle intersection (Woop, Benthin, Wald, JCGT 2(1), 2013) with the paper's
//     double-precision re-evaluation of edge functions that come out exactly zero, barycentrics
//     reported as (u, v) = weights of vertices 1 and 2 (Shaders/Geometry.slang:108-118);
//   * a binned-SAH BVH2 per mesh and one over the instances, or brute force (checker of checkers);
//   * closest hit accepts tmin <= t < tmax and keeps the smallest (t, instance, triangle); shadow
//     rays accept any hit (RAY_FLAG_ACCEPT_FIRST_HIT).
// Rays are intersected in object space: origin and direction go through the instance's
// world-to-object transform without renormalisation, so t is shared by all instances.
#pragma once

#include <algorithm>
#include <vector>

#include "pt_math.hpp"
#include "pt_scene.hpp"

namespace orc
{

struct Hit
{
    float t       = 0;
    float u       = 0; // weight of vertex 1
    float v       = 0; // weight of vertex 2
    int32_t inst  = -1;
    int32_t prim  = -1;
};

// Double-precision inverse of a 3x4 affine transform, rounded to float.  The product computes the
// same inverse with the same cofactor formula.
inline void invertAffine(const float* m, float* out)
{
    double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g = m[8], h = m[9], i = m[10];
    double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
    double det = a * A + b * B + c * C;
    double inv[9] = { A / det, -(b * i - c * h) / det, (b * f - c * e) / det, B / det,
        (a * i - c * g) / det, -(a * f - c * d) / det, C / det, -(a * h - b * g) / det,
        (a * e - b * d) / det };
    double tx = m[3], ty = m[7], tz = m[11];
    for (int r = 0; r < 3; r++)
    {
        out[4 * r + 0] = float(inv[3 * r + 0]);
        out[4 * r + 1] = float(inv[3 * r + 1]);
        out[4 * r + 2] = float(inv[3 * r + 2]);
        out[4 * r + 3] = float(-(inv[3 * r + 0] * tx + inv[3 * r + 1] * ty + inv[3 * r + 2] * tz));
    }
}

// Per-ray constants of the watertight test (Woop et al. section 3).
template <class T>
struct WatertightRay
{
    V3<T> org, dir;
    int kx, ky, kz;
    T Sx, Sy, Sz;
    void setup(const V3<T>& o, const V3<T>& d)
    {
        org = o;
        dir = d;
        T ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
        kz   = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
        kx   = kz + 1 == 3 ? 0 : kz + 1;
        ky   = kx + 1 == 3 ? 0 : kx + 1;
        if (d[kz] < T(0))
            std::swap(kx, ky);
        Sx = d[kx] / d[kz];
        Sy = d[ky] / d[kz];
        Sz = T(1) / d[kz];
    }
    // Returns true and writes t/u/v when tmin <= t < tmax (t <= tmax when inclusive).
    bool intersect(const V3<T>& p0, const V3<T>& p1, const V3<T>& p2, T tmin, T tmax, bool inclusive,
        T& tOut, T& uOut, T& vOut) const
    {
        V3<T> A = p0 - org, B = p1 - org, C = p2 - org;
        T Ax = A[kx] - Sx * A[kz], Ay = A[ky] - Sy * A[kz];
        T Bx = B[kx] - Sx * B[kz], By = B[ky] - Sy * B[kz];
        T Cx = C[kx] - Sx * C[kz], Cy = C[ky] - Sy * C[kz];
        T U  = Cx * By - Cy * Bx;
        T V  = Ax * Cy - Ay * Cx;
        T W  = Bx * Ay - By * Ax;
        if (U == T(0) || V == T(0) || W == T(0))
        {
            U = T(double(Cx) * double(By) - double(Cy) * double(Bx));
            V = T(double(Ax) * double(Cy) - double(Ay) * double(Cx));
            W = T(double(Bx) * double(Ay) - double(By) * double(Ax));
        }
        if ((U < T(0) || V < T(0) || W < T(0)) && (U > T(0) || V > T(0) || W > T(0)))
            return false;
        T det = U + V + W;
        if (det == T(0))
            return false;
        T Az = Sz * A[kz], Bz = Sz * B[kz], Cz = Sz * C[kz];
        T Tn  = U * Az + V * Bz + W * Cz;
        T rcp = T(1) / det;
        T t   = Tn * rcp;
        if (!(t >= tmin && (t < tmax || (inclusive && t == tmax))))
            return false;
        tOut = t;
        uOut = V * rcp;
        vOut = W * rcp;
        return true;
    }
};

struct AABB
{
    float lo[3] = { 1e30f, 1e30f, 1e30f };
    float hi[3] = { -1e30f, -1e30f, -1e30f };
    void grow(const float* p)
    {
        for (int k = 0; k < 3; k++)
        {
            lo[k] = std::min(lo[k], p[k]);
            hi[k] = std::max(hi[k], p[k]);
        }
    }
    void grow(const AABB& b)
    {
        for (int k = 0; k < 3; k++)
        {
            lo[k] = std::min(lo[k], b.lo[k]);
            hi[k] = std::max(hi[k], b.hi[k]);
        }
    }
    float area() const
    {
        float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        if (dx < 0 || dy < 0 || dz < 0)
            return 0.f;
        return 2.f * (dx * dy + dy * dz + dz * dx);
    }
};

// Binned-SAH BVH2 over a set of boxes (triangles of a mesh, or instances).
struct BVH2
{
    struct Node
    {
        AABB box;
        int32_t left = -1; // interior: child index; leaf: -1
        int32_t first = 0, count = 0;
    };
    std::vector<Node> nodes;
    std::vector<uint32_t> order; // primitive indices in leaf order

    void build(const std::vector<AABB>& boxes)
    {
        nodes.clear();
        order.resize(boxes.size());
        for (size_t i = 0; i < boxes.size(); i++)
            order[i] = uint32_t(i);
        if (boxes.empty())
            return;
        std::vector<float> cen(boxes.size() * 3);
        for (size_t i = 0; i < boxes.size(); i++)
            for (int k = 0; k < 3; k++)
                cen[3 * i + k] = 0.5f * (boxes[i].lo[k] + boxes[i].hi[k]);
        nodes.reserve(boxes.size() * 2);
        nodes.push_back(Node());
        nodes[0].first = 0;
        nodes[0].count = int32_t(boxes.size());
        std::vector<int32_t> stack = { 0 };
        const int kBins = 16;
        while (!stack.empty())
        {
            int32_t ni = stack.back();
            stack.pop_back();
            Node node = nodes[ni];
            AABB box, cbox;
            for (int32_t i = node.first; i < node.first + node.count; i++)
            {
                box.grow(boxes[order[i]]);
                cbox.grow(&cen[3 * order[i]]);
            }
            nodes[ni].box = box;
            if (node.count <= 4)
                continue;
            float bestCost = 1e30f;
            int bestAxis = -1, bestSplit = -1;
            for (int axis = 0; axis < 3; axis++)
            {
                float ext = cbox.hi[axis] - cbox.lo[axis];
                if (ext <= 0.f)
                    continue;
                AABB bb[kBins];
                int bc[kBins] = { 0 };
                for (int32_t i = node.first; i < node.first + node.count; i++)
                {
                    int b = int(kBins * (cen[3 * order[i] + axis] - cbox.lo[axis]) / ext);
                    b     = std::min(std::max(b, 0), kBins - 1);
                    bc[b]++;
                    bb[b].grow(boxes[order[i]]);
                }
                float rightArea[kBins];
                int rightCount[kBins];
                AABB acc;
                int cnt = 0;
                for (int b = kBins - 1; b > 0; b--)
                {
                    acc.grow(bb[b]);
                    cnt += bc[b];
                    rightArea[b]  = acc.area();
                    rightCount[b] = cnt;
                }
                acc = AABB();
                cnt = 0;
                for (int b = 0; b < kBins - 1; b++)
                {
                    acc.grow(bb[b]);
                    cnt += bc[b];
                    if (cnt == 0 || rightCount[b + 1] == 0)
                        continue;
                    float cost = acc.area() * cnt + rightArea[b + 1] * rightCount[b + 1];
                    if (cost < bestCost)
                    {
                        bestCost  = cost;
                        bestAxis  = axis;
                        bestSplit = b;
                    }
                }
            }
            int32_t mid;
            if (bestAxis >= 0 && (bestCost < box.area() * node.count || node.count > 8))
            {
                float ext = cbox.hi[bestAxis] - cbox.lo[bestAxis];
                auto it   = std::partition(order.begin() + node.first,
                    order.begin() + node.first + node.count, [&](uint32_t p) {
                        int b = int(kBins * (cen[3 * p + bestAxis] - cbox.lo[bestAxis]) / ext);
                        b     = std::min(std::max(b, 0), kBins - 1);
                        return b <= bestSplit;
                    });
                mid = int32_t(it - order.begin());
                if (mid == node.first || mid == node.first + node.count)
                    mid = node.first + node.count / 2;
            }
            else if (bestAxis < 0 && node.count > 8)
                mid = node.first + node.count / 2; // coincident centroids: split in half
            else
                continue; // leaf
            int32_t l = int32_t(nodes.size());
            nodes.push_back(Node());
            nodes.push_back(Node());
            nodes[l].first     = node.first;
            nodes[l].count     = mid - node.first;
            nodes[l + 1].first = mid;
            nodes[l + 1].count = node.first + node.count - mid;
            nodes[ni].left     = l;
            stack.push_back(l);
            stack.push_back(l + 1);
        }
    }
};

// Slab test in scalar type T.
template <class T>
inline bool slab(const AABB& b, const V3<T>& o, const V3<T>& invd, T tmin, T tmax, T& tEnter)
{
    T t0 = tmin, t1 = tmax;
    for (int k = 0; k < 3; k++)
    {
        T a = (T(b.lo[k]) - o[k]) * invd[k];
        T c = (T(b.hi[k]) - o[k]) * invd[k];
        if (a > c)
            std::swap(a, c);
        // Widen slightly so rounding in the box test never rejects a hit the exact triangle test
        // accepts.
        a = a - std::fabs(a) * T(1e-6) - T(1e-30);
        c = c + std::fabs(c) * T(1e-6) + T(1e-30);
        t0 = a > t0 ? a : t0;
        t1 = c < t1 ? c : t1;
        if (t0 > t1)
            return false;
    }
    tEnter = t0;
    return true;
}

// Scene-level ray caster over instanced meshes.
template <class T>
struct Caster
{
    const Mesh* meshes          = nullptr;
    const Instance* instances   = nullptr;
    int32_t instanceCount       = 0;
    std::vector<BVH2> blas;
    BVH2 tlas;
    std::vector<float> worldToObject; // 12 per instance
    bool bruteForce = false;

    void build(const Mesh* m, int32_t meshCount, const Instance* inst, int32_t instCount)
    {
        meshes        = m;
        instances     = inst;
        instanceCount = instCount;
        blas.resize(meshCount);
        std::vector<AABB> meshBox(meshCount);
        for (int32_t mi = 0; mi < meshCount; mi++)
        {
            std::vector<AABB> boxes(m[mi].triangleCount);
            for (uint32_t t = 0; t < m[mi].triangleCount; t++)
                for (int k = 0; k < 3; k++)
                {
                    const float* p = m[mi].positions + 3 * size_t(m[mi].indices[3 * size_t(t) + k]);
                    boxes[t].grow(p);
                    meshBox[mi].grow(p);
                }
            blas[mi].build(boxes);
        }
        worldToObject.resize(size_t(instCount) * 12);
        std::vector<AABB> iboxes(instCount);
        for (int32_t i = 0; i < instCount; i++)
        {
            invertAffine(inst[i].objectToWorld, &worldToObject[12 * size_t(i)]);
            const AABB& mb = meshBox[inst[i].mesh];
            for (int c = 0; c < 8; c++)
            {
                float p[3] = { (c & 1) ? mb.hi[0] : mb.lo[0], (c & 2) ? mb.hi[1] : mb.lo[1],
                    (c & 4) ? mb.hi[2] : mb.lo[2] };
                const float* M = inst[i].objectToWorld;
                float w[3];
                for (int r = 0; r < 3; r++)
                    w[r] = M[4 * r] * p[0] + M[4 * r + 1] * p[1] + M[4 * r + 2] * p[2] + M[4 * r + 3];
                iboxes[i].grow(w);
            }
            // Pad for rounding in the transform.
            for (int k = 0; k < 3; k++)
            {
                float pad = 1e-5f * (std::fabs(iboxes[i].lo[k]) + std::fabs(iboxes[i].hi[k]) + 1.f);
                iboxes[i].lo[k] -= pad;
                iboxes[i].hi[k] += pad;
            }
        }
        tlas.build(iboxes);
    }

    // Object-space ray for instance i (float transform applied in T).
    void objectRay(int32_t i, const V3<T>& o, const V3<T>& d, V3<T>& oo, V3<T>& od) const
    {
        Xform<T> x;
        for (int k = 0; k < 12; k++)
            x.m[k] = T(worldToObject[12 * size_t(i) + k]);
        oo = x.point(o);
        od = x.vector(d);
    }

    V3<T> vertex(const Mesh& m, uint32_t tri, int k) const
    {
        return V3<T>::from(m.positions + 3 * size_t(m.indices[3 * size_t(tri) + k]));
    }

    // Traverses one mesh's BLAS; updates best (closest) or returns true at the first hit (anyHit).
    bool traverseMesh(int32_t inst, const V3<T>& o, const V3<T>& d, T tmin, T& tmax, Hit& best,
        bool anyHit) const
    {
        const Instance& in = instances[inst];
        const Mesh& m      = meshes[in.mesh];
        const BVH2& bv     = blas[in.mesh];
        WatertightRay<T> wr;
        wr.setup(o, d);
        bool found = false;
        // Closest hit keeps the smallest (t, instance, triangle), so the result does not depend on
        // the order triangles are tested in (a hit on an edge shared by two triangles has equal t).
        auto testTri = [&](uint32_t tri) -> bool {
            T t, u, v;
            bool have = best.inst >= 0;
            if (wr.intersect(vertex(m, tri, 0), vertex(m, tri, 1), vertex(m, tri, 2), tmin, tmax,
                    !anyHit && have, t, u, v))
            {
                if (have && !anyHit && !(t < tmax) &&
                    !(inst < best.inst || (inst == best.inst && int32_t(tri) < best.prim)))
                    return false;
                tmax      = t;
                best.t    = float(t);
                best.u    = float(u);
                best.v    = float(v);
                best.inst = inst;
                best.prim = int32_t(tri);
                found     = true;
                return true;
            }
            return false;
        };
        if (bruteForce || bv.nodes.empty())
        {
            for (uint32_t tri = 0; tri < m.triangleCount; tri++)
                if (testTri(tri) && anyHit)
                    return true;
            return found;
        }
        V3<T> invd{T(1) / d.x, T(1) / d.y, T(1) / d.z};
        int32_t stack[128];
        int sp = 0;
        stack[sp++] = 0;
        while (sp)
        {
            const BVH2::Node& n = bv.nodes[stack[--sp]];
            T te;
            if (!slab(n.box, o, invd, tmin, tmax, te))
                continue;
            if (n.left < 0)
            {
                for (int32_t k = n.first; k < n.first + n.count; k++)
                    if (testTri(bv.order[k]) && anyHit)
                        return true;
                continue;
            }
            stack[sp++] = n.left + 1;
            stack[sp++] = n.left;
        }
        return found;
    }

    // Closest hit over the scene: world-space ray, tmin <= t < tmax.
    bool closest(const V3<T>& o, const V3<T>& d, T tmin, T tmax, Hit& hit) const
    {
        return cast(o, d, tmin, tmax, hit, false);
    }
    bool occluded(const V3<T>& o, const V3<T>& d, T tmin, T tmax) const
    {
        Hit h;
        return cast(o, d, tmin, tmax, h, true);
    }
    bool cast(const V3<T>& o, const V3<T>& d, T tmin, T tmax, Hit& hit, bool anyHit) const
    {
        bool found = false;
        hit        = Hit();
        auto visit = [&](int32_t i) -> bool {
            V3<T> oo, od;
            objectRay(i, o, d, oo, od);
            if (traverseMesh(i, oo, od, tmin, tmax, hit, anyHit))
            {
                found = true;
                if (anyHit)
                    return true;
            }
            return false;
        };
        if (bruteForce || tlas.nodes.empty())
        {
            for (int32_t i = 0; i < instanceCount; i++)
                if (visit(i))
                    return true;
            return found;
        }
        V3<T> invd{T(1) / d.x, T(1) / d.y, T(1) / d.z};
        int32_t stack[128];
        int sp = 0;
        stack[sp++] = 0;
        while (sp)
        {
            const BVH2::Node& n = tlas.nodes[stack[--sp]];
            T te;
            if (!slab(n.box, o, invd, tmin, tmax, te))
                continue;
            if (n.left < 0)
            {
                for (int32_t k = n.first; k < n.first + n.count; k++)
                    if (visit(int32_t(tlas.order[k])))
                        return true;
                continue;
            }
            stack[sp++] = n.left + 1;
            stack[sp++] = n.left;
        }
        return found;
    }
};

} // namespace orc
