// sgi_scene.cu - GPU ray casting of the GI stage's inputs for box scenes:
// the G-buffer (formats of pbr_geometry_pass.fs:95-141), the CSM depth
// (RenderCSMDepth_, StratusRendererBackend.cpp:1081-1158: depth clamp and a
// slope-scaled polygon offset of factor 2) and the VPL distance cubes
// (shadowVpl.fs:26-34: saturate(distance / farPlane) per texel).
//
// Compiled with -fmad=false like the shading kernels, so a CPU ray caster
// that evaluates the same expressions produces the same bytes.
#include <cuda_runtime.h>
#include <stdint.h>

#include "sgi_internal.h"
#include "sgi_math.cuh"

namespace sgi {

constexpr int kMaxSceneBoxes = 256;

// Slab test: entry t (may be negative) and entry axis; false on a miss.
SGI_D bool ray_box(const float* o, const float* d, const sgi_box& b, float& tnear, int& axis) {
    tnear = -__int_as_float(0x7f800000);
    float tfar = __int_as_float(0x7f800000);
    axis = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if (d[k] == 0.0f) {
            if (o[k] < b.min[k] || o[k] > b.max[k]) return false;
            continue;
        }
        float t1 = (b.min[k] - o[k]) / d[k];
        float t2 = (b.max[k] - o[k]) / d[k];
        float lo = t1 < t2 ? t1 : t2, hi = t1 < t2 ? t2 : t1;
        if (lo > tnear) { tnear = lo; axis = k; }
        if (hi < tfar) tfar = hi;
    }
    return tnear <= tfar;
}

SGI_D uint32_t enc_unorm8(float v) {
    v = gclamp(v, 0.0f, 1.0f);
    return (uint32_t)(v * 255.0f + 0.5f);
}

__device__ void load_boxes(sgi_box* sb, const sgi_box* boxes, int nb) {
    const int tid = threadIdx.y * blockDim.x + threadIdx.x, nt = blockDim.x * blockDim.y;
    const float4* src = reinterpret_cast<const float4*>(boxes);
    float4* dst = reinterpret_cast<float4*>(sb);
    for (int k = tid; k < nb * 4; k += nt) dst[k] = __ldg(src + k);
    __syncthreads();
}

__global__ void scene_gbuffer_kernel(const sgi_box* __restrict__ boxes, int nb, sgi_scene_camera cam, int W, int H,
                                     sgi_gbuffer out) {
    __shared__ sgi_box sb[kMaxSceneBoxes];
    load_boxes(sb, boxes, nb);
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const size_t i = (size_t)y * W + x;
    float* depth = const_cast<float*>(out.depth);
    uint32_t* normal = const_cast<uint32_t*>(out.normal);
    uint32_t* albedo = const_cast<uint32_t*>(out.albedo);
    uint16_t* refl = const_cast<uint16_t*>(out.base_reflectivity);
    uint32_t* rma = const_cast<uint32_t*>(out.roughness_metallic_ambient);
    uint32_t* velocity = const_cast<uint32_t*>(out.velocity);
    float* id = const_cast<float*>(out.id);
    uint16_t* ssao = const_cast<uint16_t*>(out.ssao);
    const float nx = ((float(x) + 0.5f) / float(W)) * 2.0f - 1.0f;
    const float ny = ((float(y) + 0.5f) / float(H)) * 2.0f - 1.0f;
    V4 a = mat4_mul(cam.inv_proj_view, nx, ny, -1.0f, 1.0f);
    V4 b = mat4_mul(cam.inv_proj_view, nx, ny, 1.0f, 1.0f);
    float o[3] = {a.x / a.w, a.y / a.w, a.z / a.w};
    float e[3] = {b.x / b.w, b.y / b.w, b.z / b.w};
    float d[3] = {e[0] - o[0], e[1] - o[1], e[2] - o[2]};
    float best = __int_as_float(0x7f800000);
    int bi = -1, bax = 0;
    for (int k = 0; k < nb; ++k) {
        float tn; int ax;
        if (!ray_box(o, d, sb[k], tn, ax)) continue;
        if (tn > 0.0f && tn < best) { best = tn; bi = k; bax = ax; }
    }
    if (bi < 0) {
        depth[i] = 1.0f; normal[i] = 0x00ff8080u; albedo[i] = 0; refl[i] = 0; rma[i] = 0;
        velocity[i] = 0; id[i] = 0.0f; ssao[i] = f2h(1.0f);
        return;
    }
    const sgi_box& bx = sb[bi];
    float p[3] = {o[0] + d[0] * best, o[1] + d[1] * best, o[2] + d[2] * best};
    float n[3] = {0.0f, 0.0f, 0.0f};
    n[bax] = d[bax] > 0.0f ? -1.0f : 1.0f;
    V4 c = mat4_mul(cam.proj_view, p[0], p[1], p[2], 1.0f);
    V4 pc = mat4_mul(cam.prev_proj_view, p[0], p[1], p[2], 1.0f);
    depth[i] = (c.z / c.w) * 0.5f + 0.5f;
    const float cu = (c.x / c.w) * 0.5f + 0.5f, cv = (c.y / c.w) * 0.5f + 0.5f;
    const float pu = (pc.x / pc.w) * 0.5f + 0.5f, pv = (pc.y / pc.w) * 0.5f + 0.5f;
    velocity[i] = (uint32_t)f2h(cu - pu) | ((uint32_t)f2h(cv - pv) << 16);
    normal[i] = enc_unorm8(n[0] * 0.5f + 0.5f) | (enc_unorm8(n[1] * 0.5f + 0.5f) << 8) |
                (enc_unorm8(n[2] * 0.5f + 0.5f) << 16) | 0xff000000u;
    albedo[i] = enc_unorm8(bx.albedo[0]) | (enc_unorm8(bx.albedo[1]) << 8) | (enc_unorm8(bx.albedo[2]) << 16) |
                (enc_unorm8(bx.albedo[3]) << 24);
    refl[i] = (uint16_t)enc_unorm8(bx.reflectance);
    rma[i] = enc_unorm8(bx.roughness) | (enc_unorm8(bx.metallic) << 8) | 0xff000000u;
    id[i] = bx.id;
    const float h = p[1] < 0.0f ? 0.0f : p[1];
    ssao[i] = f2h(0.2f + 0.8f * (h / (h + 0.5f)));
}

struct CsmGen {
    float pv[16];
    float inv[16];
    int R;
    float* out;
};

__global__ void scene_csm_kernel(const sgi_box* __restrict__ boxes, int nb, CsmGen g) {
    __shared__ sgi_box sb[kMaxSceneBoxes];
    load_boxes(sb, boxes, nb);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int R = g.R;
    if (i >= R || j >= R) return;
    const float nx = ((float(i) + 0.5f) / float(R)) * 2.0f - 1.0f;
    const float ny = ((float(j) + 0.5f) / float(R)) * 2.0f - 1.0f;
    V4 a = mat4_mul(g.inv, nx, ny, -1.0f, 1.0f);
    V4 b = mat4_mul(g.inv, nx, ny, 1.0f, 1.0f);
    float o[3] = {a.x / a.w, a.y / a.w, a.z / a.w};
    float e[3] = {b.x / b.w, b.y / b.w, b.z / b.w};
    float d[3] = {e[0] - o[0], e[1] - o[1], e[2] - o[2]};
    float best = __int_as_float(0x7f800000);
    int bi = -1, bax = 0;
    for (int k = 0; k < nb; ++k) {
        float tn; int ax;
        if (!ray_box(o, d, sb[k], tn, ax)) continue;
        if (tn < best) { best = tn; bi = k; bax = ax; }
    }
    float outv = 1.0f;
    if (bi >= 0) {
        float p[3] = {o[0] + d[0] * best, o[1] + d[1] * best, o[2] + d[2] * best};
        V4 cc = mat4_mul(g.pv, p[0], p[1], p[2], 1.0f);
        const float z = (cc.z / cc.w) * 0.5f + 0.5f;
        const float ncx = g.inv[0 * 4 + bax], ncy = g.inv[1 * 4 + bax], ncz = g.inv[2 * 4 + bax];
        const float anz = gabs(ncz);
        float slope = gmax(gabs(ncx), gabs(ncy)) / (anz * float(R));
        if (!(slope < 1.0f)) slope = 1.0f;
        outv = gclamp(z + 2.0f * slope, 0.0f, 1.0f);
    }
    g.out[(size_t)j * R + i] = outv;
}

SGI_D void cube_dir(int face, float sc, float tc, float* d) {
    switch (face) {
        case 0: d[0] = 1.0f; d[1] = -tc; d[2] = -sc; break;
        case 1: d[0] = -1.0f; d[1] = -tc; d[2] = sc; break;
        case 2: d[0] = sc; d[1] = 1.0f; d[2] = tc; break;
        case 3: d[0] = sc; d[1] = -1.0f; d[2] = -tc; break;
        case 4: d[0] = sc; d[1] = -tc; d[2] = 1.0f; break;
        default: d[0] = -sc; d[1] = -tc; d[2] = -1.0f; break;
    }
}

// grid: (ceil(n/16), ceil(n/16), count*6), block 16x16
__global__ void scene_cube_kernel(const sgi_box* __restrict__ boxes, int nb, const sgi_vpl* __restrict__ vpls,
                                  const sgi_atlas_entry* __restrict__ entries, sgi_cube_atlas at) {
    __shared__ sgi_box sb[kMaxSceneBoxes];
    load_boxes(sb, boxes, nb);
    const int n = at.face_size;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int v = blockIdx.z / 6, f = blockIdx.z % 6;
    if (i >= n || j >= n) return;
    const sgi_vpl& vp = vpls[v];
    const sgi_atlas_entry e = entries[v];
    if (e.index < 0 || e.index >= at.num_atlases || e.layer < 0 || e.layer >= at.layers_per_atlas) return;
    const float sc = ((float(i) + 0.5f) / float(n)) * 2.0f - 1.0f;
    const float tc = ((float(j) + 0.5f) / float(n)) * 2.0f - 1.0f;
    float d[3];
    cube_dir(f, sc, tc, d);
    float o[3] = {vp.position[0], vp.position[1], vp.position[2]};
    float best = __int_as_float(0x7f800000);
    for (int k = 0; k < nb; ++k) {
        float tn; int ax;
        if (!ray_box(o, d, sb[k], tn, ax)) continue;
        if (tn > 0.0f && tn < best) best = tn;
    }
    float val = 1.0f;
    if (best < __int_as_float(0x7f800000)) {
        const float len = sqrtf((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]);
        val = saturate((best * len) / vp.far_plane);
    }
    const size_t off = (((size_t)e.layer * 6 + f) * n + j) * n + i;
    void* base = const_cast<void*>(at.atlas[e.index]);
    if (at.format == SGI_CUBE_F32) ((float*)base)[off] = val;
    else if (at.format == SGI_CUBE_F16) ((uint16_t*)base)[off] = f2h(val);
    else ((uint16_t*)base)[off] = (uint16_t)(val * 65535.0f + 0.5f);
}

// Diffuse colour cubes: RGB8 albedo of the first box hit (A = 255), 0 on a miss.
__global__ void scene_diffuse_kernel(const sgi_box* __restrict__ boxes, int nb, const sgi_vpl* __restrict__ vpls,
                                     const sgi_atlas_entry* __restrict__ entries, sgi_diffuse_atlas at) {
    __shared__ sgi_box sb[kMaxSceneBoxes];
    load_boxes(sb, boxes, nb);
    const int n = at.face_size;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int v = blockIdx.z / 6, f = blockIdx.z % 6;
    if (i >= n || j >= n) return;
    const sgi_vpl& vp = vpls[v];
    const sgi_atlas_entry e = entries[v];
    if (e.index < 0 || e.index >= at.num_atlases || e.layer < 0 || e.layer >= at.layers_per_atlas) return;
    const float sc = ((float(i) + 0.5f) / float(n)) * 2.0f - 1.0f;
    const float tc = ((float(j) + 0.5f) / float(n)) * 2.0f - 1.0f;
    float d[3];
    cube_dir(f, sc, tc, d);
    float o[3] = {vp.position[0], vp.position[1], vp.position[2]};
    float best = __int_as_float(0x7f800000);
    int bi = -1;
    for (int k = 0; k < nb; ++k) {
        float tn; int ax;
        if (!ray_box(o, d, sb[k], tn, ax)) continue;
        if (tn > 0.0f && tn < best) { best = tn; bi = k; }
    }
    uint32_t t = 0;
    if (bi >= 0)
        t = enc_unorm8(sb[bi].albedo[0]) | (enc_unorm8(sb[bi].albedo[1]) << 8) | (enc_unorm8(sb[bi].albedo[2]) << 16) |
            0xff000000u;
    const size_t off = (((size_t)e.layer * 6 + f) * n + j) * n + i;
    ((uint32_t*)const_cast<void*>(at.atlas[e.index]))[off] = t;
}

cudaError_t launch_scene_gbuffer(const sgi_box* boxes, int32_t nb, const sgi_scene_camera& cam, int32_t W,
                                 int32_t H, const sgi_gbuffer& out, cudaStream_t s) {
    if (nb > kMaxSceneBoxes) return cudaErrorInvalidValue;
    dim3 block(16, 16), grid((W + 15) / 16, (H + 15) / 16);
    scene_gbuffer_kernel<<<grid, block, 0, s>>>(boxes, nb, cam, W, H, out);
    return cudaGetLastError();
}

cudaError_t launch_scene_csm(const sgi_box* boxes, int32_t nb, const sgi_csm& csm, const float (*inv)[16],
                             cudaStream_t s) {
    if (nb > kMaxSceneBoxes) return cudaErrorInvalidValue;
    const int R = csm.resolution;
    for (int c = 0; c < csm.num_cascades; ++c) {
        CsmGen g;
        for (int k = 0; k < 16; ++k) { g.pv[k] = csm.cascade_proj_view[c][k]; g.inv[k] = inv[c][k]; }
        g.R = R;
        g.out = const_cast<float*>(csm.depth) + (size_t)c * R * R;
        dim3 block(16, 16), grid((R + 15) / 16, (R + 15) / 16);
        scene_csm_kernel<<<grid, block, 0, s>>>(boxes, nb, g);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_scene_cubes(const sgi_box* boxes, int32_t nb, const sgi_vpl* vpls, const sgi_atlas_entry* entries,
                               int32_t count, const sgi_cube_atlas& atlas, cudaStream_t s) {
    if (nb > kMaxSceneBoxes) return cudaErrorInvalidValue;
    const int n = atlas.face_size;
    // blockIdx.z is limited to 65535: launch in slices of 10000 VPLs (60000 faces)
    for (int first = 0; first < count; first += 10000) {
        const int c = count - first < 10000 ? count - first : 10000;
        dim3 block(16, 16), grid((n + 15) / 16, (n + 15) / 16, c * 6);
        scene_cube_kernel<<<grid, block, 0, s>>>(boxes, nb, vpls + first, entries + first, atlas);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_scene_diffuse(const sgi_box* boxes, int32_t nb, const sgi_vpl* vpls,
                                 const sgi_atlas_entry* entries, int32_t count, const sgi_diffuse_atlas& atlas,
                                 cudaStream_t s) {
    if (nb > kMaxSceneBoxes || atlas.face_size < 1) return cudaErrorInvalidValue;
    const int n = atlas.face_size;
    for (int first = 0; first < count; first += 10000) {
        const int c = count - first < 10000 ? count - first : 10000;
        dim3 block(16, 16), grid((n + 15) / 16, (n + 15) / 16, c * 6);
        scene_diffuse_kernel<<<grid, block, 0, s>>>(boxes, nb, vpls + first, entries + first, atlas);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace sgi
