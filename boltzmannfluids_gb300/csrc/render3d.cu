// render3d.cu -- headless volume ray-marcher over the solver's fields: the
// images that LBM::render3d_density / _velocity / _boundries / _forces /
// _temperature (BoltzmannFluids/Source/LBM/LBM.cpp:1207-1376) draw with the
// fragment shaders GLSL/Renderer3D/*_volumetric.frag, computed by a CUDA
// kernel into an RGBA float image instead of a GL framebuffer.
//
// Per pixel (one thread): the ray from the camera position through the
// pixel centre (unprojected with the inverse of projection * view) is
// clipped to the unit cube [-0.5, 0.5]^3 (the model matrix is the identity,
// LBM.cpp:1219) and marched from the entry point in steps of 1/sample_count
// while the marched length is below the chord length, sampling the field at
// texture coordinate position + 0.5 with trilinear filtering (texel centres
// at (i + 1/2)/n, clamped to the edge).  Per mode, as the shaders accumulate:
//   density      T *= exp(-8 a h); colour += T (0.5, 0.8, 1) h;  out (colour/(1-T), 1-T)
//   velocity     v += 32 |s(p).rgb - s(p + 0.01).rgb| h;          out (v, v.x)
//   boundries    hit |= boundary id > 0;                           out (1, 1, 1, hit)
//   forces       v += 256 |F| h, then 1 - exp(-v);                 out (v, v.x)
//   temperature  v += T h;                                         out (1, 0, 0, v)
// (a = density, h = step length; the velocity and force shaders write a vec3
// into the alpha channel, whose first component GLSL keeps.)  Pixels whose
// ray misses the cube stay (0, 0, 0, 0).  exp is the Cody-Waite / Taylor
// exp_f32 of the step kernels, so the image is reproducible on the CPU.
#include <cuda_runtime.h>

#include <cmath>
#include <string>

#include "../../include/bf_lbm.h"
#include "lbm_kernels.cuh"

namespace {

struct RenderParams {
    const float4* vel_den;
    const float4* force_temp;
    const uint8_t* bnd;
    int nx, ny, nz;
    int width, height, samples, mode;
    float inv_pv[16];  // inverse of projection * view, column-major
    float cam[3];      // camera position (inverse view applied to the origin)
    float4* out;
};

__device__ __forceinline__ void unproject(const float* m, float x, float y, float z, float out[3]) {
    float r[4];
#pragma unroll
    for (int row = 0; row < 4; row++)
        r[row] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[row], x), __fmul_rn(m[4 + row], y)), __fmul_rn(m[8 + row], z)),
                           m[12 + row]);
    out[0] = __fdiv_rn(r[0], r[3]);
    out[1] = __fdiv_rn(r[1], r[3]);
    out[2] = __fdiv_rn(r[2], r[3]);
}

// trilinear sample of component c of a float4 field (or of the boundary ids
// as R8 normalised values when f4 is null) at texture coordinate u in [0,1]^3
__device__ float sample(const RenderParams& p, const float4* f4, int c, float ux, float uy, float uz) {
    const float gx = __fsub_rn(__fmul_rn(ux, (float)p.nx), 0.5f);
    const float gy = __fsub_rn(__fmul_rn(uy, (float)p.ny), 0.5f);
    const float gz = __fsub_rn(__fmul_rn(uz, (float)p.nz), 0.5f);
    const float fx = floorf(gx), fy = floorf(gy), fz = floorf(gz);
    const float tx = __fsub_rn(gx, fx), ty = __fsub_rn(gy, fy), tz = __fsub_rn(gz, fz);
    const int x0 = (int)fx, y0 = (int)fy, z0 = (int)fz;
    auto at = [&](int x, int y, int z) -> float {
        x = min(max(x, 0), p.nx - 1);
        y = min(max(y, 0), p.ny - 1);
        z = min(max(z, 0), p.nz - 1);
        const size_t n = (size_t)x + (size_t)p.nx * ((size_t)y + (size_t)p.ny * (size_t)z);
        if (!f4) return __fdiv_rn((float)p.bnd[n], 255.0f);
        const float4 v = f4[n];
        return c == 0 ? v.x : (c == 1 ? v.y : (c == 2 ? v.z : v.w));
    };
    auto lerp = [](float a, float b, float t) { return __fadd_rn(a, __fmul_rn(__fsub_rn(b, a), t)); };
    const float c00 = lerp(at(x0, y0, z0), at(x0 + 1, y0, z0), tx);
    const float c10 = lerp(at(x0, y0 + 1, z0), at(x0 + 1, y0 + 1, z0), tx);
    const float c01 = lerp(at(x0, y0, z0 + 1), at(x0 + 1, y0, z0 + 1), tx);
    const float c11 = lerp(at(x0, y0 + 1, z0 + 1), at(x0 + 1, y0 + 1, z0 + 1), tx);
    return lerp(lerp(c00, c10, ty), lerp(c01, c11, ty), tz);
}

__global__ void render_kernel(const RenderParams p) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= p.width || j >= p.height) return;
    float4* o = p.out + (size_t)j * p.width + i;
    *o = make_float4(0.f, 0.f, 0.f, 0.f);
    // ray through the pixel centre (NDC, y up, row 0 at the bottom)
    const float ndx = __fsub_rn(__fdiv_rn((float)(2 * i + 1), (float)p.width), 1.0f);
    const float ndy = __fsub_rn(__fdiv_rn((float)(2 * j + 1), (float)p.height), 1.0f);
    float far_pt[3];
    unproject(p.inv_pv, ndx, ndy, 1.0f, far_pt);
    float d[3] = {__fsub_rn(far_pt[0], p.cam[0]), __fsub_rn(far_pt[1], p.cam[1]), __fsub_rn(far_pt[2], p.cam[2])};
    const float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(d[0], d[0]), __fmul_rn(d[1], d[1])), __fmul_rn(d[2], d[2])));
    if (!(len > 0.0f)) return;
    for (int k = 0; k < 3; k++) d[k] = __fdiv_rn(d[k], len);
    // slab intersection with [-0.5, 0.5]^3 (ray_intersect_aabb of the shaders)
    float tmin = -INFINITY, tmax = INFINITY;
    for (int k = 0; k < 3; k++) {
        const float inv = __fdiv_rn(1.0f, d[k]);
        const float t0 = __fmul_rn(__fsub_rn(-0.5f, p.cam[k]), inv);
        const float t1 = __fmul_rn(__fsub_rn(0.5f, p.cam[k]), inv);
        tmin = fmaxf(tmin, fminf(t0, t1));
        tmax = fminf(tmax, fmaxf(t0, t1));
    }
    const float to_box = fmaxf(0.0f, tmin);
    const float in_box = fmaxf(0.0f, __fsub_rn(tmax, to_box));
    if (!(in_box > 0.0f)) return;  // the cube's back faces cover no fragment here
    float pos[3];
    for (int k = 0; k < 3; k++) pos[k] = __fadd_rn(p.cam[k], __fmul_rn(to_box, d[k]));
    const float h = __fdiv_rn(1.0f, (float)p.samples);
    float depth = 0.0f;
    float acc[3] = {0.f, 0.f, 0.f};
    float trans = 1.0f;
    bool hit = false;
    while (depth < in_box) {
        const float u = __fadd_rn(pos[0], 0.5f), v = __fadd_rn(pos[1], 0.5f), w = __fadd_rn(pos[2], 0.5f);
        switch (p.mode) {
        case BF_RENDER_DENSITY: {
            const float a = sample(p, p.vel_den, 3, u, v, w);
            trans = __fmul_rn(trans, bf::exp_f32(__fmul_rn(__fmul_rn(-a, 8.0f), h)));
            const float light[3] = {0.5f, 0.8f, 1.0f};
            for (int k = 0; k < 3; k++) acc[k] = __fadd_rn(acc[k], __fmul_rn(__fmul_rn(trans, light[k]), h));
            break;
        }
        case BF_RENDER_VELOCITY:
            for (int k = 0; k < 3; k++) {
                const float s0 = sample(p, p.vel_den, k, u, v, w);
                const float s1 = sample(p, p.vel_den, k, __fadd_rn(0.01f, u), __fadd_rn(0.01f, v), __fadd_rn(0.01f, w));
                acc[k] = __fadd_rn(acc[k], __fmul_rn(__fmul_rn(fabsf(__fsub_rn(s0, s1)), 32.0f), h));
            }
            break;
        case BF_RENDER_BOUNDRIES:
            hit = hit || sample(p, nullptr, 0, u, v, w) > 0.0f;
            break;
        case BF_RENDER_FORCES:
            for (int k = 0; k < 3; k++)
                acc[k] = __fadd_rn(acc[k], __fmul_rn(__fmul_rn(fabsf(sample(p, p.force_temp, k, u, v, w)), 256.0f), h));
            break;
        default:  // temperature
            acc[0] = __fadd_rn(acc[0], __fmul_rn(sample(p, p.force_temp, 3, u, v, w), h));
            break;
        }
        depth = __fadd_rn(depth, h);
        for (int k = 0; k < 3; k++) pos[k] = __fadd_rn(pos[k], __fmul_rn(d[k], h));
    }
    switch (p.mode) {
    case BF_RENDER_DENSITY: {
        const float a = __fsub_rn(1.0f, trans);
        *o = make_float4(__fdiv_rn(acc[0], a), __fdiv_rn(acc[1], a), __fdiv_rn(acc[2], a), a);
        break;
    }
    case BF_RENDER_VELOCITY: *o = make_float4(acc[0], acc[1], acc[2], acc[0]); break;
    case BF_RENDER_BOUNDRIES: *o = make_float4(1.f, 1.f, 1.f, hit ? 1.f : 0.f); break;
    case BF_RENDER_FORCES: {
        float r[3];
        for (int k = 0; k < 3; k++) r[k] = __fsub_rn(1.0f, bf::exp_f32(-acc[k]));
        *o = make_float4(r[0], r[1], r[2], r[0]);
        break;
    }
    default: *o = make_float4(1.f, 0.f, 0.f, acc[0]); break;
    }
}

// column-major 4x4 inverse (cofactors, double precision)
bool invert4(const double* m, double* inv) {
    double a[16];
    a[0] = m[5] * m[10] * m[15] - m[5] * m[11] * m[14] - m[9] * m[6] * m[15] + m[9] * m[7] * m[14] + m[13] * m[6] * m[11] - m[13] * m[7] * m[10];
    a[4] = -m[4] * m[10] * m[15] + m[4] * m[11] * m[14] + m[8] * m[6] * m[15] - m[8] * m[7] * m[14] - m[12] * m[6] * m[11] + m[12] * m[7] * m[10];
    a[8] = m[4] * m[9] * m[15] - m[4] * m[11] * m[13] - m[8] * m[5] * m[15] + m[8] * m[7] * m[13] + m[12] * m[5] * m[11] - m[12] * m[7] * m[9];
    a[12] = -m[4] * m[9] * m[14] + m[4] * m[10] * m[13] + m[8] * m[5] * m[14] - m[8] * m[6] * m[13] - m[12] * m[5] * m[10] + m[12] * m[6] * m[9];
    a[1] = -m[1] * m[10] * m[15] + m[1] * m[11] * m[14] + m[9] * m[2] * m[15] - m[9] * m[3] * m[14] - m[13] * m[2] * m[11] + m[13] * m[3] * m[10];
    a[5] = m[0] * m[10] * m[15] - m[0] * m[11] * m[14] - m[8] * m[2] * m[15] + m[8] * m[3] * m[14] + m[12] * m[2] * m[11] - m[12] * m[3] * m[10];
    a[9] = -m[0] * m[9] * m[15] + m[0] * m[11] * m[13] + m[8] * m[1] * m[15] - m[8] * m[3] * m[13] - m[12] * m[1] * m[11] + m[12] * m[3] * m[9];
    a[13] = m[0] * m[9] * m[14] - m[0] * m[10] * m[13] - m[8] * m[1] * m[14] + m[8] * m[2] * m[13] + m[12] * m[1] * m[10] - m[12] * m[2] * m[9];
    a[2] = m[1] * m[6] * m[15] - m[1] * m[7] * m[14] - m[5] * m[2] * m[15] + m[5] * m[3] * m[14] + m[13] * m[2] * m[7] - m[13] * m[3] * m[6];
    a[6] = -m[0] * m[6] * m[15] + m[0] * m[7] * m[14] + m[4] * m[2] * m[15] - m[4] * m[3] * m[14] - m[12] * m[2] * m[7] + m[12] * m[3] * m[6];
    a[10] = m[0] * m[5] * m[15] - m[0] * m[7] * m[13] - m[4] * m[1] * m[15] + m[4] * m[3] * m[13] + m[12] * m[1] * m[7] - m[12] * m[3] * m[5];
    a[14] = -m[0] * m[5] * m[14] + m[0] * m[6] * m[13] + m[4] * m[1] * m[14] - m[4] * m[2] * m[13] - m[12] * m[1] * m[6] + m[12] * m[2] * m[5];
    a[3] = -m[1] * m[6] * m[11] + m[1] * m[7] * m[10] + m[5] * m[2] * m[11] - m[5] * m[3] * m[10] - m[9] * m[2] * m[7] + m[9] * m[3] * m[6];
    a[7] = m[0] * m[6] * m[11] - m[0] * m[7] * m[10] - m[4] * m[2] * m[11] + m[4] * m[3] * m[10] + m[8] * m[2] * m[7] - m[8] * m[3] * m[6];
    a[11] = -m[0] * m[5] * m[11] + m[0] * m[7] * m[9] + m[4] * m[1] * m[11] - m[4] * m[3] * m[9] - m[8] * m[1] * m[7] + m[8] * m[3] * m[5];
    a[15] = m[0] * m[5] * m[10] - m[0] * m[6] * m[9] - m[4] * m[1] * m[10] + m[4] * m[2] * m[9] + m[8] * m[1] * m[6] - m[8] * m[2] * m[5];
    const double det = m[0] * a[0] + m[1] * a[4] + m[2] * a[8] + m[3] * a[12];
    if (det == 0.0 || !std::isfinite(det)) return false;
    for (int k = 0; k < 16; k++) inv[k] = a[k] / det;
    return true;
}

int render_fail(int code, const std::string& msg) {
    bf::record_error(msg);
    return code;
}

}  // namespace

extern "C" int bf_render3d(bf_solver* s, int32_t mode, const float view[16], const float projection[16],
                           int32_t width, int32_t height, int32_t sample_count, float* rgba_device, void* stream) {
    if (!s || !view || !projection || !rgba_device) return render_fail(BF_ERR_INVALID_ARGUMENT, "bf_render3d: NULL argument");
    if (mode < BF_RENDER_DENSITY || mode > BF_RENDER_TEMPERATURE) return render_fail(BF_ERR_INVALID_ARGUMENT, "bf_render3d: unknown mode");
    if (width < 1 || height < 1 || sample_count < 1) return render_fail(BF_ERR_INVALID_ARGUMENT, "bf_render3d: bad image size or sample count");
    // the fields of the last saved step, complete on the solver's stream
    int r = bf_synchronize(s, 0);
    if (r != BF_OK) return r;
    bf_field vd{}, ft{}, bd{};
    if ((r = bf_get_field(s, BF_FIELD_VELOCITY_DENSITY, &vd)) != BF_OK) return r;
    if ((r = bf_get_field(s, BF_FIELD_FORCE_TEMPERATURE, &ft)) != BF_OK) return r;
    if ((r = bf_get_field(s, BF_FIELD_BOUNDARY, &bd)) != BF_OK) return r;
    RenderParams p{};
    p.vel_den = static_cast<const float4*>(vd.device_ptr);
    p.force_temp = static_cast<const float4*>(ft.device_ptr);
    p.bnd = static_cast<const uint8_t*>(bd.device_ptr);
    p.nx = vd.resolution[0]; p.ny = vd.resolution[1]; p.nz = vd.resolution[2];
    p.width = width; p.height = height; p.samples = sample_count; p.mode = mode;
    // inverse(projection * view) and the camera position inverse(view) * (0,0,0,1)
    double pv[16], inv[16], vinv[16], vd64[16];
    for (int c = 0; c < 4; c++)
        for (int row = 0; row < 4; row++) {
            double acc = 0;
            for (int k = 0; k < 4; k++) acc += (double)projection[k * 4 + row] * (double)view[c * 4 + k];
            pv[c * 4 + row] = acc;
        }
    for (int k = 0; k < 16; k++) vd64[k] = view[k];
    if (!invert4(pv, inv) || !invert4(vd64, vinv)) return render_fail(BF_ERR_INVALID_ARGUMENT, "bf_render3d: singular camera matrices");
    for (int k = 0; k < 16; k++) p.inv_pv[k] = (float)inv[k];
    for (int k = 0; k < 3; k++) p.cam[k] = (float)(vinv[12 + k] / vinv[15]);
    p.out = reinterpret_cast<float4*>(rgba_device);
    const dim3 block(16, 16);
    const dim3 grid((unsigned)((width + 15) / 16), (unsigned)((height + 15) / 16));
    render_kernel<<<grid, block, 0, static_cast<cudaStream_t>(stream)>>>(p);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return render_fail(BF_ERR_CUDA, std::string("bf_render3d: ") + cudaGetErrorString(e));
    return BF_OK;
}
