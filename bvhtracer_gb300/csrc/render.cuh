// Pieces of the tiled render shared by the single-BLAS render (kernels_trace.cu) and the scene
// render (kernels_scene.cu): the camera ray of a pixel (Camera::get_ray_eye / get_ray_world,
// camera.rs:994-1010), the accumulators (renderer.rs:134-334) and the pixel shaders
// (renderer.rs:116-222), all in the reference's f32 operation order with Rust's saturating casts.
#pragma once

#include <cuda_runtime.h>

#include <cfloat>
#include <cstdint>

#include "bvhgpu.h"
#include "common.cuh"

namespace bvhgpu {

__device__ __forceinline__ float3 xf_point(const float* m, float3 p) {
    return make_float3(fadd(fadd(fadd(fmul(m[0], p.x), fmul(m[4], p.y)), fmul(m[8], p.z)), fmul(m[12], 1.0f)),
                       fadd(fadd(fadd(fmul(m[1], p.x), fmul(m[5], p.y)), fmul(m[9], p.z)), fmul(m[13], 1.0f)),
                       fadd(fadd(fadd(fmul(m[2], p.x), fmul(m[6], p.y)), fmul(m[10], p.z)), fmul(m[14], 1.0f)));
}
__device__ __forceinline__ float3 xf_vector(const float* m, float3 p) {
    return make_float3(fadd(fadd(fadd(fmul(m[0], p.x), fmul(m[4], p.y)), fmul(m[8], p.z)), fmul(m[12], 0.0f)),
                       fadd(fadd(fadd(fmul(m[1], p.x), fmul(m[5], p.y)), fmul(m[9], p.z)), fmul(m[13], 0.0f)),
                       fadd(fadd(fadd(fmul(m[2], p.x), fmul(m[6], p.y)), fmul(m[10], p.z)), fmul(m[14], 0.0f)));
}
__device__ __forceinline__ float3 normalize3(float3 v) {
    float m = __fsqrt_rn(dot3(v.x, v.y, v.z, v.x, v.y, v.z));
    return make_float3(__fdiv_rn(v.x, m), __fdiv_rn(v.y, m), __fdiv_rn(v.z, m));
}

struct RenderParams {
    float cam[9 + 16];
    float acc[16];
    float sh[8];
    int width, height, acc_kind, shader_kind;
    const float* tex_coords;  // BVHGPU_ACC_TEXTURE: 6 floats per triangle (per-corner u, v)
    const uint8_t* texels;    //   RGB8, row-major
    uint32_t tex_w, tex_h;
};

__device__ __forceinline__ unsigned long long f32_as_usize(float x) {  // Rust `as usize`: saturating
    if (!(x > 0.0f)) return 0ull;
    if (x >= 18446744073709551616.0f) return 0xFFFFFFFFFFFFFFFFull;
    return (unsigned long long)x;
}
__device__ __forceinline__ uint8_t f32_as_u8(float x) {  // Rust `as u8`: saturating, NaN -> 0
    if (!(x > 0.0f)) return 0;
    if (x >= 255.0f) return 255;
    return (uint8_t)x;
}
__device__ __forceinline__ int32_t f32_as_i32(float x) {  // Rust `as i32`: saturating, NaN -> 0
    if (x != x) return 0;
    if (x >= 2147483648.0f) return INT32_MAX;
    if (x <= -2147483648.0f) return INT32_MIN;
    return (int32_t)x;
}

// The world-space ray through pixel (x, y)'s top-left corner, u = x / w, v = y / h
// (renderer.rs:358-361): Camera::get_ray_eye (camera.rs:994-1002) then get_ray_world (:1004-1010).
__device__ __forceinline__ void camera_ray(const RenderParams& P, int x, int y, float3& o, float3& d) {
    const float* C = P.cam;
    const float u = __fdiv_rn((float)x, (float)P.width);
    const float v = __fdiv_rn((float)y, (float)P.height);
    const float3 tl = make_float3(C[0], C[1], C[2]), tr = make_float3(C[3], C[4], C[5]),
                 bl = make_float3(C[6], C[7], C[8]);
    const float3 org = make_float3(0.0f, 0.0f, 0.0f);
    float3 p = make_float3(fadd(org.x, tl.x), fadd(org.y, tl.y), fadd(org.z, tl.z));
    p = make_float3(fadd(p.x, fmul(fsub(tr.x, tl.x), u)), fadd(p.y, fmul(fsub(tr.y, tl.y), u)),
                    fadd(p.z, fmul(fsub(tr.z, tl.z), u)));
    p = make_float3(fadd(p.x, fmul(fsub(bl.x, tl.x), v)), fadd(p.y, fmul(fsub(bl.y, tl.y), v)),
                    fadd(p.z, fmul(fsub(bl.z, tl.z), v)));
    const float3 dir = normalize3(make_float3(fsub(p.x, org.x), fsub(p.y, org.y), fsub(p.z, org.z)));
    o = xf_point(C + 9, org);
    d = xf_vector(C + 9, dir);
}

// The accumulator's radiance for a closest hit (hit, t, u, v, primitive hp).  normals / normal_xf
// (the normal accumulator) and tex_coords / texels (the texture accumulator) are the looked-up
// model's data and object transform.
__device__ __forceinline__ float3 accumulate(const RenderParams& P, bool hit, float t, float hu, float hv,
                                             uint32_t hp, const float* normals, const float* normal_xf,
                                             const float* tex_coords, const uint8_t* texels, uint32_t tex_w,
                                             uint32_t tex_h) {
    float3 rad = make_float3(0.0f, 0.0f, 0.0f);
    switch (P.acc_kind) {
        case BVHGPU_ACC_INTERSECTION:  // renderer.rs:145-153
            rad = hit ? make_float3(P.acc[0], P.acc[1], P.acc[2]) : make_float3(P.acc[3], P.acc[4], P.acc[5]);
            break;
        case BVHGPU_ACC_DEPTH: {  // renderer.rs:184-193
            float tt = hit ? t : FLT_MAX;
            rad = make_float3(tt, tt, tt);
            break;
        }
        case BVHGPU_ACC_UV:  // renderer.rs:233-244
            if (hit) rad = make_float3(hu, hv, fsub(1.0f, fadd(hu, hv)));
            break;
        case BVHGPU_ACC_NORMAL:  // renderer.rs:256-285
            if (hit) {
                const float* nn = normals + 9ull * hp;
                float w0 = fsub(fsub(1.0f, hu), hv);
                float3 nm;
                nm.x = fadd(fadd(fmul(nn[0], w0), fmul(nn[3], hu)), fmul(nn[6], hv));
                nm.y = fadd(fadd(fmul(nn[1], w0), fmul(nn[4], hu)), fmul(nn[7], hv));
                nm.z = fadd(fadd(fmul(nn[2], w0), fmul(nn[5], hu)), fmul(nn[8], hv));
                float3 nz = normalize3(xf_vector(normal_xf, nm));
                rad = make_float3(fmul(fadd(nz.x, 1.0f), 0.5f), fmul(fadd(nz.y, 1.0f), 0.5f),
                                  fmul(fadd(nz.z, 1.0f), 0.5f));
            }
            break;
        case BVHGPU_ACC_TEXTURE:  // TextureMaterialAccumulator, renderer.rs:289-334
            if (hit) {
                const float* tc = tex_coords + 6ull * hp;
                const float w0 = fsub(fsub(1.0f, hu), hv);
                const float uvx = fadd(fadd(fmul(tc[0], w0), fmul(tc[2], hu)), fmul(tc[4], hv));
                const float uvy = fadd(fadd(fmul(tc[1], w0), fmul(tc[3], hu)), fmul(tc[5], hv));
                // TextureMaterial::evaluate (materials/material.rs:44-52)
                const unsigned long long iu = f32_as_usize(fmul(uvx, __uint2float_rn(tex_w))) % tex_w;
                const unsigned long long iv = f32_as_usize(fmul(uvy, __uint2float_rn(tex_h))) % tex_h;
                const uint8_t* px = texels + 3ull * (iv * tex_w + iu);
                const float sc = 0.00390625f;  // 1 / 256, exact
                rad = make_float3(fmul(__uint2float_rn(px[0]), sc), fmul(__uint2float_rn(px[1]), sc),
                                  fmul(__uint2float_rn(px[2]), sc));
            }
            break;
        default:
            break;
    }
    return rad;
}

// The pixel shader's colour for a radiance value.
__device__ __forceinline__ uchar4 shade(const RenderParams& P, float3 rad) {
    uchar4 c;
    switch (P.shader_kind) {
        case BVHGPU_SHADER_INTERSECTION: {  // renderer.rs:166-173
            bool nz = !(rad.x == 0.0f && rad.y == 0.0f && rad.z == 0.0f);
            const float* s = nz ? P.sh : P.sh + 4;
            c = make_uchar4((uint8_t)s[0], (uint8_t)s[1], (uint8_t)s[2], (uint8_t)s[3]);
            break;
        }
        case BVHGPU_SHADER_DEPTH: {  // renderer.rs:207-221 (u32 arithmetic wraps)
            if (rad.x < FLT_MAX) {
                uint32_t col = 255u - (uint32_t)f32_as_i32(fmul(fsub(rad.x, P.sh[1]), P.sh[0]));
                uint32_t cc = col * 0x010101u;
                c = make_uchar4((uint8_t)((cc & 0x00FF0000u) >> 16), (uint8_t)((cc & 0x0000FF00u) >> 8),
                                (uint8_t)(cc & 0xFFu), 255);
            } else {
                c = make_uchar4(0, 0, 0, 255);
            }
            break;
        }
        default:  // RadianceToRgbShader (renderer.rs:124-131)
            c = make_uchar4(f32_as_u8(fmul(255.0f, rad.x)), f32_as_u8(fmul(255.0f, rad.y)),
                            f32_as_u8(fmul(255.0f, rad.z)), 255);
            break;
    }
    return c;
}

// Host side: the camera, accumulator and shader parameters of a render launch.
inline RenderParams make_render_params(const bvhgpu_camera& cam, int w, int h, int acc, const float* acc_params,
                                       int shader, const float* shader_params) {
    RenderParams P;
    for (int k = 0; k < 3; ++k) {
        P.cam[k] = cam.top_left[k];
        P.cam[3 + k] = cam.top_right[k];
        P.cam[6 + k] = cam.bottom_left[k];
    }
    for (int k = 0; k < 16; ++k) P.cam[9 + k] = cam.view_inv[k];
    for (int k = 0; k < 16; ++k) P.acc[k] = 0.0f;
    for (int k = 0; k < 8; ++k) P.sh[k] = 0.0f;
    if (acc == BVHGPU_ACC_INTERSECTION && acc_params)
        for (int k = 0; k < 6; ++k) P.acc[k] = acc_params[k];
    if (acc == BVHGPU_ACC_NORMAL && acc_params)
        for (int k = 0; k < 16; ++k) P.acc[k] = acc_params[k];
    if (shader == BVHGPU_SHADER_INTERSECTION && shader_params)
        for (int k = 0; k < 8; ++k) P.sh[k] = shader_params[k];
    if (shader == BVHGPU_SHADER_DEPTH && shader_params)
        for (int k = 0; k < 2; ++k) P.sh[k] = shader_params[k];
    P.width = w;
    P.height = h;
    P.acc_kind = acc;
    P.shader_kind = shader;
    P.tex_coords = nullptr;
    P.texels = nullptr;
    P.tex_w = P.tex_h = 0;
    return P;
}

}  // namespace bvhgpu
