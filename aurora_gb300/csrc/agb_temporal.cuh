// Denoising / temporal-resolve AOV arithmetic shared by the shading kernel and the temporal resolve
// (Shaders/GlobalPipelineState.slang:122-172, DirectX/Shaders/Colors.hlsli:42-56).
// Matrices are FrameData matrices as bytes (glm column-major): element (row r, column c) of the
// shader's float4x4 is m[4 * c + r].
#pragma once

#include "agb_math.cuh"

namespace agb
{

// mul(M, v): row r = sum over c of M[r][c] v[c], left to right.
AGB_HD void mul4(const float* m, const float v[4], float out[4])
{
    for (int r = 0; r < 4; r++)
        out[r] = m[r] * v[0] + m[4 + r] * v[1] + m[8 + r] * v[2] + m[12 + r] * v[3];
}

// Previous-minus-current pixel position of a homogeneous world point (w = 1) or direction (w = 0).
AGB_HD v2 screenMotion(const float* viewProj, const float* viewProjPrev, const float w[4],
    float width, float height)
{
    float cur[4], prev[4];
    mul4(viewProj, w, cur);
    mul4(viewProjPrev, w, prev);
    float cw = fabsf(cur[3]), pw = fabsf(prev[3]);
    cw       = cw > 1e-6f ? cw : 1e-6f;
    pw       = pw > 1e-6f ? pw : 1e-6f;
    v2 cn    = v2{ cur[0] / cw, cur[1] / cw };
    v2 pn    = v2{ prev[0] / pw, prev[1] / pw };
    v2 cs    = v2{ (cn.x * 0.5f + 0.5f) * width, (-cn.y * 0.5f + 0.5f) * height };
    v2 ps    = v2{ (pn.x * 0.5f + 0.5f) * width, (-pn.y * 0.5f + 0.5f) * height };
    return v2{ ps.x - cs.x, ps.y - cs.y };
}

// View-space depth (negative in front of the camera).  Rows of the transposed inverse view are
// right / up / back / eye.
AGB_HD float viewDepth(const float* invView, v3 w)
{
    v3 forward = -v3{ invView[2], invView[6], invView[10] };
    v3 eye     = v3{ invView[3], invView[7], invView[11] };
    return -dot(w - eye, forward);
}

// 2.5D motion: screen delta (previous - current), then current view Z - previous view Z.
AGB_HD float4 surfaceMotion(const float* viewProj, const float* viewProjPrev,
    const float* invViewPrev, v3 w, float currentViewZ, float width, float height)
{
    float prevViewZ = viewDepth(invViewPrev, w);
    float w4[4]     = { w.x, w.y, w.z, 1.f };
    v2 m            = screenMotion(viewProj, viewProjPrev, w4, width, height);
    return make_float4(m.x, m.y, currentViewZ - prevViewZ, 0.f);
}

AGB_HD float4 skyMotion(const float* viewProj, const float* viewProjPrev, v3 d, float width,
    float height)
{
    float w4[4] = { d.x, d.y, d.z, 0.f };
    v2 m        = screenMotion(viewProj, viewProjPrev, w4, width, height);
    return make_float4(m.x, m.y, 0.f, 0.f);
}

AGB_HD v3 rgbToYCoCg(v3 c)
{
    return v3{ 0.25f * c.x + 0.5f * c.y + 0.25f * c.z, 0.5f * c.x - 0.5f * c.z,
        -0.25f * c.x + 0.5f * c.y - 0.25f * c.z };
}
AGB_HD v3 yCoCgToRgb(v3 c)
{
    float t = c.x - c.z;
    return v3{ t + c.y, c.x + c.z, t - c.y };
}

} // namespace agb
