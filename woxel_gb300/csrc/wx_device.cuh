// wx_device.cuh — device-side HDDA march and shading for sm_103a.
//
// Restates src/shaders/raycast.comp.wgsl:60-519 over the device node pools
// (one u32 slot word per child slot; see wx_common.h). Every FP32 operation
// keeps the shader's order; the translation unit is compiled with
// -fmad=false (no contraction) and IEEE division/square root, so each ray
// performs the same operation sequence as the CPU restatement and the
// results are bit-identical. Choices WGSL leaves open are pinned:
// normalize(v) = v / sqrt((x*x + y*y) + z*z); min/max return the non-NaN
// operand and the first operand on ties; f32->i32 saturates (NaN -> 0);
// unorm8 = NaN/x<=0 -> 0, x>=1 -> 255, else floor(x*255 + 0.5).
#pragma once

#include <cstdint>

#include "woxel_gb300.h"

namespace wxd {

constexpr uint32_t kChild = 0x80000000u;
constexpr uint32_t kMaxSteps = 1000u;  // HDDA_MAX_RAY_STEPS, raycast.comp.wgsl:82

struct DevGrid {
    const int4 *o5;         // N5 origins (x, y, z, 0), DFS order
    const uint32_t *slot5;  // n5 * 32768
    const uint32_t *slot4;  // n4 * 4096
    const uint32_t *slot3;  // n3 * 512
    uint32_t n5;
};

struct Uniform {  // the 256-byte ComputeState, read from kernel parameter space
    wx_state_uniform s;
};

__device__ __forceinline__ float pmin(float a, float b) { return (b < a || a != a) ? b : a; }
__device__ __forceinline__ float pmax(float a, float b) { return (b > a || a != a) ? b : a; }
__device__ __forceinline__ float sign11(float x) { return x < 0.0f ? -1.0f : 1.0f; }

struct F3 {
    float x, y, z;
};
__device__ __forceinline__ F3 f3(float x, float y, float z) { return F3{x, y, z}; }
__device__ __forceinline__ F3 operator+(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ F3 operator-(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ F3 operator*(F3 a, F3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ F3 operator*(float s, F3 a) { return f3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ F3 operator*(F3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ F3 operator-(F3 a) { return f3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float dot3(F3 a, F3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ F3 normalize3(F3 a) {
    const float l = __fsqrt_rn(dot3(a, a));
    return f3(__fdiv_rn(a.x, l), __fdiv_rn(a.y, l), __fdiv_rn(a.z, l));
}
__device__ __forceinline__ F3 splat(float s) { return f3(s, s, s); }
__device__ __forceinline__ F3 mix3(F3 a, F3 b, float t) {
    const float omt = 1.0f - t;
    return f3(a.x * omt + b.x * t, a.y * omt + b.y * t, a.z * omt + b.z * t);
}
__device__ __forceinline__ int f2i(float x) { return __float2int_rz(x); }  // saturating, NaN -> 0
__device__ __forceinline__ uint32_t unorm8(float x) {
    if (!(x > 0.0f)) return 0u;
    if (x >= 1.0f) return 255u;
    const float y = x * 255.0f;
    return (uint32_t)floorf(y + 0.5f);
}

struct March {
    F3 p;
    uint32_t state;  // 0 hit, 1 out of bounds, 2 step cap
    uint32_t np;     // cached parents (level)
    uint32_t node;   // pool index of the deepest cached node
    uint32_t i;      // loop iteration at return
    uint32_t mask;   // bit0 x, bit1 y, bit2 z
};

// hdda_ray (raycast.comp.wgsl:84-126) with the cached descent of
// get_vdb_leaf_from_{leaf,nothing,node5,node4,node3} (:360-494).
__device__ __forceinline__ March hdda(const DevGrid &g, F3 src, F3 dir) {
    float px = src.x, py = src.y, pz = src.z;
    const float sx = sign11(dir.x), sy = sign11(dir.y), sz = sign11(dir.z);
    const float ax = pmax(0.0f, sx), ay = pmax(0.0f, sy), az = pmax(0.0f, sz);
    const float ix = __frcp_rn(dir.x), iy = __frcp_rn(dir.y), iz = __frcp_rn(dir.z);
    uint32_t np = 0, i5 = 0, i4 = 0, i3 = 0, mask = 0;
    int o5x = 0, o5y = 0, o5z = 0, o4x = 0, o4y = 0, o4z = 0, o3x = 0, o3y = 0, o3z = 0;
    March out;
    for (uint32_t i = 0; i < kMaxSteps; i++) {
        const int x = f2i(floorf(px)), y = f2i(floorf(py)), z = f2i(floorf(pz));
        // get_vdb_leaf_from_leaf: deepest cached node whose origin contains pos.
        int lvl;
        if (np == 3 && (x & ~7) == o3x && (y & ~7) == o3y && (z & ~7) == o3z) lvl = 3;
        else if (np >= 2 && (x & ~127) == o4x && (y & ~127) == o4y && (z & ~127) == o4z) lvl = 4;
        else if (np >= 1 && (x & ~4095) == o5x && (y & ~4095) == o5y && (z & ~4095) == o5z) lvl = 5;
        else lvl = 0;
        uint32_t dist = 1;
        if (lvl == 0) {  // get_vdb_leaf_from_nothing: scan the N5 origins
            const int kx = x & ~4095, ky = y & ~4095, kz = z & ~4095;
            np = 0;
            for (uint32_t k = 0; k < g.n5; k++) {
                const int4 o = __ldg(&g.o5[k]);
                if (o.x == kx && o.y == ky && o.z == kz) {
                    i5 = k;
                    o5x = kx; o5y = ky; o5z = kz;
                    lvl = 5;
                    break;
                }
            }
        }
        if (lvl == 5) {
            const uint32_t off = ((((uint32_t)x & 4095u) >> 7) << 10) | ((((uint32_t)y & 4095u) >> 7) << 5) |
                                 (((uint32_t)z & 4095u) >> 7);
            const uint32_t w = __ldg(&g.slot5[(size_t)i5 * 32768u + off]);
            np = 1;
            if (w & kChild) {
                i4 = w & ~kChild;
                o4x = x & ~127; o4y = y & ~127; o4z = z & ~127;
                lvl = 4;
            } else {
                dist = w;
            }
        }
        if (lvl == 4) {
            const uint32_t off = ((((uint32_t)x & 127u) >> 3) << 8) | ((((uint32_t)y & 127u) >> 3) << 4) |
                                 (((uint32_t)z & 127u) >> 3);
            const uint32_t w = __ldg(&g.slot4[(size_t)i4 * 4096u + off]);
            np = 2;
            if (w & kChild) {
                i3 = w & ~kChild;
                o3x = x & ~7; o3y = y & ~7; o3z = z & ~7;
                lvl = 3;
            } else {
                dist = w;
            }
        }
        if (lvl == 3) {
            const uint32_t off = (((uint32_t)x & 7u) << 6) | (((uint32_t)y & 7u) << 3) | ((uint32_t)z & 7u);
            dist = __ldg(&g.slot3[(size_t)i3 * 512u + off]);
            np = 3;
        }
        if (dist == 0u) {
            out.state = 0;
            out.i = i;
            goto done;
        }
        if (4096.0f < fabsf(px) || 4096.0f < fabsf(py) || 4096.0f < fabsf(pz)) {
            out.state = 1;
            out.i = i;
            goto done;
        }
        {
            float size = __uint2float_rn(dist);
            size = size * (np == 3 ? 1.0f : np == 2 ? 8.0f : np == 1 ? 128.0f : 4096.0f);
            const float tx = ix * (size * ax - (px - size * floorf(__fdiv_rn(px, size))));
            const float ty = iy * (size * ay - (py - size * floorf(__fdiv_rn(py, size))));
            const float tz = iz * (size * az - (pz - size * floorf(__fdiv_rn(pz, size))));
            const float t = pmin(pmin(tx, ty), tz);
            px = px + t * dir.x;
            py = py + t * dir.y;
            pz = pz + t * dir.z;
            const bool mx = (tx <= ty) && (tx <= tz);
            const bool my = (ty <= tz) && (ty <= tx);
            const bool mz = (tz <= tx) && (tz <= ty);
            mask = (mx ? 1u : 0u) | (my ? 2u : 0u) | (mz ? 4u : 0u);
            px = px + (4e-4f * sx) * (mx ? 1.0f : 0.0f);
            py = py + (4e-4f * sy) * (my ? 1.0f : 0.0f);
            pz = pz + (4e-4f * sz) * (mz ? 1.0f : 0.0f);
        }
    }
    out.state = 2;
    out.i = kMaxSteps;
done:
    out.p = f3(px, py, pz);
    out.np = np;
    out.node = np == 3 ? i3 : np == 2 ? i4 : np == 1 ? i5 : 0xFFFFFFFFu;
    out.mask = mask;
    return out;
}

__device__ __forceinline__ F3 maskf(uint32_t m) {
    return f3((m & 1u) ? 1.0f : 0.0f, (m & 2u) ? 1.0f : 0.0f, (m & 4u) ? 1.0f : 0.0f);
}
__device__ __forceinline__ F3 step3(F3 d) { return f3(sign11(d.x), sign11(d.y), sign11(d.z)); }

constexpr float kKd = 0.7f, kKa = 0.3f, kReflect = 0.9f, kWall = 0.1f;  // :145-150

__device__ __forceinline__ F3 wall_colour(F3 N) {  // :300-305 / :333-338
    const F3 Np = f3(pmax(0.0f, N.x), pmax(0.0f, N.y), pmax(0.0f, N.z));
    const F3 Nn = -f3(pmin(0.0f, N.x), pmin(0.0f, N.y), pmin(0.0f, N.z));
    F3 r = f3(kWall, 0.0f, 0.0f) * Np.x;
    r = r + f3(0.0f, kWall, 0.0f) * Np.y;
    r = r + f3(0.0f, 0.0f, kWall) * Np.z;
    r = r + f3(kWall, kWall, 0.0f) * Nn.x;
    r = r + f3(0.0f, kWall, kWall) * Nn.y;
    r = r + f3(kWall, 0.0f, kWall) * Nn.z;
    return r;
}

struct ShadowRec {
    uint32_t traced, state, steps;
};

// Lit material colour shared by mode 4 and reflect_ray2/1 (:199-208, :280-290, :317-325).
__device__ __forceinline__ F3 lit_colour(const DevGrid &g, const wx_state_uniform &s, const March &h,
                                         F3 step, F3 N) {
    const F3 sun = f3(s.sun_dir[0], s.sun_dir[1], s.sun_dir[2]);
    const F3 sc = f3(s.sun_color[0], s.sun_color[1], s.sun_color[2]);
    float I = (s.sun_color[3] * kKd) * dot3(-sun, N);
    I = pmax(0.0f, I);
    const F3 base = f3(0.4f, 0.2f, 0.2f);
    if (I != 0.0f) {
        const F3 src = h.p - (4e-2f * step) * maskf(h.mask);
        if (hdda(g, src, -sun).state == 0u) return base + (I * sc) * 0.05f;
    }
    return base + I * sc;
}

__device__ F3 reflect_ray1(const DevGrid &g, const wx_state_uniform &s, F3 src, F3 dir) {  // :311-342
    const March h = hdda(g, src, dir);
    const F3 step = step3(dir);
    if (h.state == 0u) return lit_colour(g, s, h, step, normalize3((-step) * maskf(h.mask)));
    if (h.state == 1u) return wall_colour(normalize3((-step) * maskf(h.mask)));
    return dir;
}

__device__ F3 reflect_ray2(const DevGrid &g, const wx_state_uniform &s, F3 src, F3 dir) {  // :267-309
    const March h = hdda(g, src, dir);
    const F3 step = step3(dir);
    if (h.state == 0u) {
        const F3 m = maskf(h.mask);
        const F3 N = normalize3((-step) * m);
        const F3 rdir = normalize3(dir - (2.0f * N) * dot3(dir, N));
        const F3 rsrc = h.p - (4e-2f * step) * m;
        const F3 rcol = reflect_ray1(g, s, rsrc, rdir);
        const F3 mcol = lit_colour(g, s, h, step, N);
        return mix3(mcol, rcol, kReflect);
    }
    if (h.state == 1u) return wall_colour(normalize3((-step) * maskf(h.mask)));
    return dir;
}

__device__ __forceinline__ bool grid_line(float f, float m) { return fmodf(f, m) == 0.0f; }

// ray_trace (:152-265) for the primary ray; also returns its march and shadow record.
__device__ __forceinline__ F3 ray_trace(const DevGrid &g, const wx_state_uniform &s, F3 eye, F3 dir,
                                        March &hit, ShadowRec &sh) {
    hit = hdda(g, eye, dir);
    const F3 step = step3(dir);
    const uint32_t mode = s.render_mode[0];
    sh.traced = 0;
    if (hit.state == 0u) {
        F3 grid = splat(0.0f);
        const float fx = floorf(hit.p.x), fy = floorf(hit.p.y), fz = floorf(hit.p.z);
        if (s.show_345[2] == 1u && (grid_line(fx, 4096.0f) || grid_line(fy, 4096.0f) || grid_line(fz, 4096.0f)))
            grid = f3(-0.3f, -0.3f, 1.0f);
        else if (s.show_345[1] == 1u &&
                 (grid_line(fx, 128.0f) || grid_line(fy, 128.0f) || grid_line(fz, 128.0f)))
            grid = f3(0.6f, -0.2f, -0.2f);
        else if (s.show_345[0] == 1u && (grid_line(fx, 8.0f) || grid_line(fy, 8.0f) || grid_line(fz, 8.0f)))
            grid = f3(-0.1f, 0.5f, 0.3f);
        const F3 m = maskf(hit.mask);
        if (mode == 1u) return (grid + splat(0.1f)) + m * splat(0.4f);
        if (mode == 2u) {
            const float t = __fdiv_rn(__uint2float_rn(hit.i), 200.0f);
            return grid + mix3(f3(0.72f, 1.0f, 0.99f), f3(1.0f, 0.0f, 0.0f), t);
        }
        if (mode == 3u) {
            const F3 sun = f3(s.sun_dir[0], s.sun_dir[1], s.sun_dir[2]);
            const F3 sc = f3(s.sun_color[0], s.sun_color[1], s.sun_color[2]);
            const F3 N = normalize3((-step) * m);
            const float LN = pmax(0.0f, s.sun_color[3] * dot3(-sun, N));
            const F3 I_d = ((kKd * sc) * f3(0.4f, 0.2f, 0.2f)) * LN;
            const F3 I_a = (kKa * f3(0.4f, 0.4f, 0.3f)) * f3(0.4f, 0.2f, 0.2f);
            if (LN != 0.0f) {
                const March shd = hdda(g, hit.p - (4e-2f * step) * m, -sun);
                sh.traced = 1;
                sh.state = shd.state;
                sh.steps = shd.i;
                if (shd.state == 0u) return I_a;
            }
            return I_a + I_d;
        }
        if (mode == 4u) {
            const F3 N = normalize3((-step) * m);
            const F3 mcol = lit_colour(g, s, hit, step, N);
            const F3 rdir = normalize3(dir - (2.0f * N) * dot3(dir, N));
            const F3 rsrc = hit.p - (4e-2f * step) * m;
            const F3 rcol = reflect_ray2(g, s, rsrc, rdir);
            return mix3(mcol, rcol, kReflect);
        }
        const F3 a = m * f3(0.2f, 0.2f, 0.3f);  // mode 0 and default
        return grid + splat((a.x + a.y) + a.z);
    }
    if (hit.state == 1u) {
        const F3 m = maskf(hit.mask);
        if (mode == 2u) {
            const float t = __fdiv_rn(__uint2float_rn(hit.i), 200.0f);
            const F3 a = m * f3(0.04f, 0.08f, 0.12f);
            return mix3(f3(0.72f, 1.0f, 0.99f), f3(1.0f, 0.0f, 0.0f), t) + splat((a.x + a.y) + a.z);
        }
        if (mode == 4u) {
            const F3 N = normalize3((-step) * m);
            const F3 Np = f3(pmax(0.0f, N.x), pmax(0.0f, N.y), pmax(0.0f, N.z));
            const F3 Nn = -f3(pmin(0.0f, N.x), pmin(0.0f, N.y), pmin(0.0f, N.z));
            const float ty = __fdiv_rn(hit.p.y, 4096.0f);
            const float w1 = kWall * 0.1f;
            F3 r = mix3(f3(kWall, 0.0f, 0.0f), f3(w1, 0.0f, 0.0f), ty) * Np.x;
            r = r + f3(0.0f, kWall, 0.0f) * Np.y;
            r = r + mix3(f3(0.0f, 0.0f, kWall), f3(0.0f, 0.0f, w1), ty) * Np.z;
            r = r + mix3(f3(kWall, kWall, 0.0f), f3(w1, w1, 0.0f), ty) * Nn.x;
            r = r + f3(0.0f, kWall, kWall) * Nn.y;
            r = r + mix3(f3(kWall, 0.0f, kWall), f3(w1, 0.0f, w1), ty) * Nn.z;
            return r;
        }
        const F3 a = m * f3(0.01f, 0.02f, 0.03f);
        return splat(0.0f) + splat((a.x + a.y) + a.z);
    }
    return dir;
}

// cp_main (raycast.comp.wgsl:60-68) for pixel (gx, gy): colour and hit record.
__device__ __forceinline__ void shade_pixel(const DevGrid &g, const wx_state_uniform &s, uint32_t gx,
                                            uint32_t gy, uint32_t &rgba, wx_hit &rec) {
    const float px = __uint2float_rn(gx) + 0.001f, py = __uint2float_rn(gy) + 0.001f;
    const F3 r = f3((px * s.u[0] + py * s.mv[0]) + s.wp[0], (px * s.u[1] + py * s.mv[1]) + s.wp[1],
                    (px * s.u[2] + py * s.mv[2]) + s.wp[2]);
    const F3 dir = normalize3(r);
    const F3 eye = f3(s.eye[0], s.eye[1], s.eye[2]);
    March hit;
    ShadowRec sh;
    const F3 c = ray_trace(g, s, eye, dir, hit, sh);
    rgba = unorm8(c.x) | (unorm8(c.y) << 8) | (unorm8(c.z) << 16) | (255u << 24);
    rec.p[0] = hit.p.x;
    rec.p[1] = hit.p.y;
    rec.p[2] = hit.p.z;
    rec.t = dot3(hit.p - eye, dir);
    rec.node = hit.node;
    rec.info = hit.state | (hit.np << 2) | (hit.mask << 4) | (hit.i << 8);
    rec.shadow = sh.traced ? (1u | (sh.state << 1) | (sh.steps << 8)) : 0u;
    rec.reserved = 0u;
}

}  // namespace wxd
