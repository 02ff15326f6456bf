// Smoke and flame volume ray march of Photon's viewer (the VOL_FS fragment
// shader, src/render/renderer.cpp:119-283, over the volume uploadVolume packs,
// src/app/viewer.cpp:941-949) as a CUDA kernel writing an RGB image into a
// device buffer: no window, no GL. One thread per pixel; the volume is one
// float4 per cell (soot density, aerosol density, T, heat release), sampled
// trilinearly with clamp-to-edge addressing as the shader's GL_LINEAR 3D
// texture is. The scene behind the volume is a constant background colour
// with an optional depth buffer (the opaque pass's colour and depth
// textures). All arithmetic is FP32, as in the shader.
#pragma once
#include "phx_dev.cuh"

namespace phx {

struct V3 { float x, y, z; };
__host__ __device__ __forceinline__ V3 v3(float a, float b, float c) { return {a, b, c}; }
__host__ __device__ __forceinline__ V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__host__ __device__ __forceinline__ V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__host__ __device__ __forceinline__ V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__host__ __device__ __forceinline__ V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }

// GLSL built-ins (GLSL 3.30 definitions)
__device__ __forceinline__ float vFract(float x) { return x - floorf(x); }
__device__ __forceinline__ float vClamp(float x, float a, float b) { return fminf(fmaxf(x, a), b); }
__device__ __forceinline__ float vMix(float a, float b, float t) { return a * (1.0f - t) + b * t; }
__device__ __forceinline__ V3 vMix(V3 a, V3 b, float t) { return a * (1.0f - t) + b * t; }
__device__ __forceinline__ float vSmooth(float e0, float e1, float x) {
    float t = vClamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}
__device__ __forceinline__ float vDot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

__device__ __forceinline__ V3 vHeatmap(float t) {
    t = vClamp(t, 0.0f, 1.0f);
    const V3 c0 = v3(0.10f, 0.15f, 0.55f), c1 = v3(0.10f, 0.65f, 0.85f), c2 = v3(0.95f, 0.90f, 0.20f),
             c3 = v3(0.95f, 0.35f, 0.05f), c4 = v3(0.85f, 0.05f, 0.05f);
    if (t < 0.25f) return vMix(c0, c1, t / 0.25f);
    if (t < 0.5f) return vMix(c1, c2, (t - 0.25f) / 0.25f);
    if (t < 0.75f) return vMix(c2, c3, (t - 0.5f) / 0.25f);
    return vMix(c3, c4, (t - 0.75f) / 0.25f);
}
__device__ __forceinline__ V3 vGlow(float T) {
    float t = vClamp((T - 700.0f) / 1000.0f, 0.0f, 1.0f);
    return v3(1.0f, 0.22f + 0.6f * t, 0.04f + 0.45f * t * t) * t * t;
}
__device__ __forceinline__ float vHash2(float px, float py) {
    return vFract(sinf(px * 12.9898f + py * 78.233f) * 43758.5453f);
}
__device__ __forceinline__ float vHash3(V3 p) {
    p = v3(vFract(p.x * 0.3183099f + 0.1f), vFract(p.y * 0.3183099f + 0.1f), vFract(p.z * 0.3183099f + 0.1f));
    p = p * 17.0f;
    return vFract(p.x * p.y * p.z * (p.x + p.y + p.z));
}
inline __device__ float vNoise(V3 x) {
    V3 i = v3(floorf(x.x), floorf(x.y), floorf(x.z));
    V3 f = v3(vFract(x.x), vFract(x.y), vFract(x.z));
    f = v3(f.x * f.x * (3.0f - 2.0f * f.x), f.y * f.y * (3.0f - 2.0f * f.y), f.z * f.z * (3.0f - 2.0f * f.z));
    return vMix(vMix(vMix(vHash3(i), vHash3(i + v3(1, 0, 0)), f.x), vMix(vHash3(i + v3(0, 1, 0)), vHash3(i + v3(1, 1, 0)), f.x), f.y),
                vMix(vMix(vHash3(i + v3(0, 0, 1)), vHash3(i + v3(1, 0, 1)), f.x), vMix(vHash3(i + v3(0, 1, 1)), vHash3(i + v3(1, 1, 1)), f.x), f.y),
                f.z);
}
__device__ __forceinline__ float vFlameNoise(V3 p, float time) {
    V3 q = p * v3(5.0f, 5.0f, 2.6f) - v3(0.0f, 0.0f, time * 3.2f);
    return 0.55f * vNoise(q) + 0.30f * vNoise(q * 2.1f + v3(0.0f, 0.0f, -time * 2.0f)) + 0.15f * vNoise(q * 4.3f);
}
__device__ __forceinline__ float vSmokeNoise(V3 p, float time) {
    V3 q = p * 1.6f - v3(0.0f, 0.0f, time * 0.35f);
    q = q + (v3(vNoise(q + v3(5.2f, 1.3f, 0.0f)), vNoise(q + v3(1.7f, 9.2f, 3.1f)), vNoise(q + v3(8.3f, 2.8f, 4.7f))) * 0.6f -
             v3(0.3f, 0.3f, 0.3f));
    float n = 0.5f * vNoise(q) + 0.3f * vNoise(q * 2.03f + v3(1.7f, 1.7f, 1.7f)) + 0.2f * vNoise(q * 4.1f + v3(3.3f, 3.3f, 3.3f));
    return vSmooth(0.2f, 0.8f, n);
}
__device__ __forceinline__ V3 vFlameColor(float k) {
    return vMix(vMix(v3(0.9f, 0.18f, 0.02f), v3(1.0f, 0.5f, 0.08f), vSmooth(0.0f, 0.4f, k)), v3(1.0f, 0.9f, 0.55f),
                vSmooth(0.45f, 1.0f, k));
}

struct VolGrid {
    const float4* vol;
    int nx, ny, nz;
    V3 bmin, bmax;
};
// texture(uVol, (p - boxMin) / (boxMax - boxMin)) with GL_LINEAR, CLAMP_TO_EDGE
inline __device__ float4 vSample(const VolGrid& G, V3 p) {
    const V3 u = v3((p.x - G.bmin.x) / (G.bmax.x - G.bmin.x), (p.y - G.bmin.y) / (G.bmax.y - G.bmin.y),
                    (p.z - G.bmin.z) / (G.bmax.z - G.bmin.z));
    float x = u.x * G.nx - 0.5f, y = u.y * G.ny - 0.5f, z = u.z * G.nz - 0.5f;
    float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    float ax = x - fx, ay = y - fy, az = z - fz;
    int i0 = (int)fmaxf(fminf(fx, (float)(G.nx - 1)), 0.0f), i1 = (int)fmaxf(fminf(fx + 1.0f, (float)(G.nx - 1)), 0.0f);
    int j0 = (int)fmaxf(fminf(fy, (float)(G.ny - 1)), 0.0f), j1 = (int)fmaxf(fminf(fy + 1.0f, (float)(G.ny - 1)), 0.0f);
    int k0 = (int)fmaxf(fminf(fz, (float)(G.nz - 1)), 0.0f), k1 = (int)fmaxf(fminf(fz + 1.0f, (float)(G.nz - 1)), 0.0f);
    auto at = [&](int i, int j, int k) { return __ldg(G.vol + i + (size_t)G.nx * (j + (size_t)G.ny * k)); };
    auto lerp4 = [](float4 a, float4 b, float t) {
        return make_float4(a.x * (1.0f - t) + b.x * t, a.y * (1.0f - t) + b.y * t, a.z * (1.0f - t) + b.z * t,
                           a.w * (1.0f - t) + b.w * t);
    };
    float4 c00 = lerp4(at(i0, j0, k0), at(i1, j0, k0), ax), c10 = lerp4(at(i0, j1, k0), at(i1, j1, k0), ax);
    float4 c01 = lerp4(at(i0, j0, k1), at(i1, j0, k1), ax), c11 = lerp4(at(i0, j1, k1), at(i1, j1, k1), ax);
    return lerp4(lerp4(c00, c10, ay), lerp4(c01, c11, ay), az);
}

// uploadVolume (src/app/viewer.cpp:941-949): soot and aerosol density, T, heat release
template <class R>
__global__ void k_vol_pack(const Scn<R>* __restrict__ S, int s, float4* __restrict__ vol) {
    const Scn<R>& g = S[s];
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.N) return;
    if (g.blocked[c]) { vol[c] = make_float4(0, 0, 0, 0); return; }
    const float T = (float)tAbs(g.sc[0][c]);
    const float rho = (float)g.Pb[c] / (287.0f * T);
    vol[c] = make_float4((float)g.sc[3][c] * rho, (float)g.sc[4][c] * rho, T, (float)g.hrr[c]);
}

// the fragment shader's main(), one thread per pixel; rgb rows from the bottom
// (GL window order). R is the engine's precision; the render is FP32 in both.
template <class R>
__global__ void __launch_bounds__(128) k_vol_render(VolGrid G, phx_vol_params P, const float* __restrict__ depth,
                                                    float* __restrict__ rgb) {
    const int px = blockIdx.x * 16 + (threadIdx.x & 15), py = blockIdx.y * 8 + (threadIdx.x >> 4);
    if (px >= P.width || py >= P.height) return;
    const float uvx = (px + 0.5f) / P.width, uvy = (py + 0.5f) / P.height;
    const float* M = P.inv_vp;
    auto worldAt = [&](float d) {
        const float a = uvx * 2.0f - 1.0f, b = uvy * 2.0f - 1.0f, c = d * 2.0f - 1.0f;
        const float X = M[0] * a + M[4] * b + M[8] * c + M[12], Y = M[1] * a + M[5] * b + M[9] * c + M[13];
        const float Z = M[2] * a + M[6] * b + M[10] * c + M[14], W = M[3] * a + M[7] * b + M[11] * c + M[15];
        return v3(X / W, Y / W, Z / W);
    };
    const V3 base = v3(P.background[0], P.background[1], P.background[2]);
    const float d = depth ? depth[(size_t)py * P.width + px] : 1.0f;
    const V3 ro = v3(P.eye[0], P.eye[1], P.eye[2]);
    V3 rd = worldAt(1.0f) - ro;
    rd = rd * (1.0f / sqrtf(vDot(rd, rd)));
    const float tScene = d < 1.0f ? sqrtf(vDot(worldAt(d) - ro, worldAt(d) - ro)) : 1e9f;
    const V3 bmax = v3(G.bmax.x, G.bmax.y, fminf(G.bmax.z, P.clip_z));
    const V3 inv = v3(1.0f / rd.x, 1.0f / rd.y, 1.0f / rd.z);
    const V3 ta = (G.bmin - ro) * inv, tb = (bmax - ro) * inv;
    const V3 tmn = v3(fminf(ta.x, tb.x), fminf(ta.y, tb.y), fminf(ta.z, tb.z));
    const V3 tmx = v3(fmaxf(ta.x, tb.x), fmaxf(ta.y, tb.y), fmaxf(ta.z, tb.z));
    const float t0 = fmaxf(fmaxf(fmaxf(tmn.x, tmn.y), tmn.z), 0.0f);
    const float t1 = fminf(fminf(tmx.x, tmx.y), tmx.z);
    const float tEnd = fminf(t1, tScene);
    V3 col = v3(0, 0, 0);
    float tr = 1.0f;
    const float tS = (P.slice_z - ro.z) / rd.z;
    const bool sliceHit = P.slice == 1 && tS > t0 && tS < tEnd && P.slice_z < bmax.z;
    const V3 sun = v3(P.sun_dir[0], P.sun_dir[1], P.sun_dir[2]);
    auto slice = [&]() {
        float4 sv = vSample(G, ro + rd * tS);
        if (sv.z > 150.0f) {
            float tn = (sv.z - P.t_min) / (P.t_max - P.t_min);
            float sa = vMix(0.12f, 0.88f, vSmooth(0.0f, 0.2f, tn));
            col = col + vHeatmap(tn) * (tr * sa);
            tr *= 1.0f - sa;
        }
    };
    bool sliceDone = !sliceHit;
    if (t0 < tEnd) {
        const float ds = P.step;
        const float jit = vHash2(px + 0.5f, py + 0.5f);
        const int n = (int)fminf(600.0f, (tEnd - t0) / ds + 1.0f);
        for (int i = 0; i < n; ++i) {
            const float t = t0 + ((float)i + jit) * ds;
            if (t > tEnd) break;
            if (!sliceDone && t >= tS) { slice(); sliceDone = true; }
            if (P.smoke == 0 && P.fire == 0) continue;
            const V3 p = ro + rd * t;
            const float4 v = vSample(G, p);
            const float soot = fmaxf(v.x, 0.0f), aero = fmaxf(v.y, 0.0f);
            const float sigma0 = (8700.0f * soot + 3000.0f * aero) * P.smoke_scale;
            float sigma = sigma0;
            float a = 0.0f;
            const float lightFrac = aero / (soot * 3.0f + aero + 1e-12f);
            V3 scat = v3(0, 0, 0);
            if (P.smoke == 1 && sigma0 > 0.02f) {
                const float bill = vSmokeNoise(p, P.time);
                sigma = sigma0 * vMix(0.25f, 1.75f, bill);
                a = 1.0f - expf(-sigma * ds);
                float od = 0.0f;
                for (int sh = 1; sh <= 4; ++sh) {
                    const float4 sv2 = vSample(G, p + sun * (0.35f * (float)sh));
                    od += (8700.0f * fmaxf(sv2.x, 0.0f) + 3000.0f * fmaxf(sv2.y, 0.0f)) * P.smoke_scale * 0.35f;
                }
                const float sunT = expf(-od);
                const float gg = 0.35f, ct = vDot(rd, sun);
                const float hg = (1.0f - gg * gg) / powf(1.0f + gg * gg - 2.0f * gg * ct, 1.5f) * 0.25f;
                const V3 albedo = vMix(v3(0.10f, 0.095f, 0.09f), v3(0.86f, 0.84f, 0.78f), lightFrac);
                const float amb = 0.45f + 0.25f * vClamp((p.z - G.bmin.z) * 0.15f, 0.0f, 1.0f);
                scat = albedo * (amb * vMix(0.55f, 1.0f, sunT) + 1.6f * hg * sunT);
                scat = scat * vMix(0.85f, 1.1f, bill);
            }
            if (P.fire == 1) {
                const float alb = vMix(0.45f, 0.95f, lightFrac);
                float fl = 0.0f;
                for (int li = 0; li < P.n_lights; ++li) {
                    const V3 dl = v3(P.lights[li][0], P.lights[li][1], P.lights[li][2]) - p;
                    fl += P.lights[li][3] / (0.6f + vDot(dl, dl));
                }
                scat = scat + v3(1.0f, 0.45f, 0.15f) * fl * alb * 0.9f;
            }
            V3 emit = v3(0, 0, 0);
            if (P.fire == 1) {
                const float q = v.w / 1.0e6f;
                const float hot = vSmooth(1000.0f, 1600.0f, v.z);
                const float drive = vClamp(q * 0.9f, 0.0f, 3.0f) + hot * 0.9f;
                if (drive > 0.01f) {
                    const float nn = vFlameNoise(p, P.time);
                    const float shape = vSmooth(0.62f - 0.25f * vClamp(drive, 0.0f, 1.5f), 0.85f, nn + 0.15f * fminf(drive, 1.5f));
                    const float k = vClamp(0.25f * drive + 0.6f * nn * shape, 0.0f, 1.0f);
                    emit = vFlameColor(k) * shape * drive * 6.0f;
                }
                emit = emit + vGlow(v.z) * vClamp(sigma * 0.6f, 0.0f, 1.0f) * 4.0f;
            }
            col = col + (scat * a + emit * ds) * tr;
            tr *= 1.0f - a;
            if (tr < 0.004f) break;
        }
        if (!sliceDone) slice();
    }
    float* o = rgb + 3 * ((size_t)py * P.width + px);
    o[0] = base.x * tr + (1.0f - expf(-col.x * 1.1f));
    o[1] = base.y * tr + (1.0f - expf(-col.y * 1.1f));
    o[2] = base.z * tr + (1.0f - expf(-col.z * 1.1f));
}

}  // namespace phx
