// wx_device.cuh — device-side HDDA march and shading for sm_103a.
//
// Restates src/shaders/raycast.comp.wgsl:60-519 over the device node pools
// (one u32 slot word per child slot; see wx_common.h). Every FP32 operation of
// the shader keeps its order; the translation unit is compiled with
// -fmad=false (no contraction), and division / square root are IEEE, so each
// ray performs the same operation sequence as the CPU restatement and the
// results are bit-identical. Choices WGSL leaves open are pinned:
// normalize(v) = v / sqrt((x*x + y*y) + z*z); min/max return the non-NaN
// operand and the first operand on ties; f32->i32 saturates (NaN -> 0);
// unorm8 = NaN/x<=0 -> 0, x>=1 -> 255, else floor(x*255 + 0.5).
#pragma once

#include <cstdint>

#include "woxel_gb300.h"
#include "wx_kernels.h"

namespace wxd {

constexpr uint32_t kChild = 0x80000000u;
constexpr uint32_t kMaxSteps = 1000u;  // HDDA_MAX_RAY_STEPS, raycast.comp.wgsl:82

// root: header, N5 origins in DFS order and the dense root-key table;
// slot5/slot4: n5*32768 and n4*4096 slot words; leaf: n3*512 voxel bytes
// (0 hit, 1..254 distance, 255 = exact distance in ovf).
using DevGrid = wxk::DevGrid;

// RN(1 / d) for 1 <= d < kRcp (entry 0 unused): filled once per device from
// host IEEE division (wxk::init_device_tables). Defined here: kernels.cu is
// the only translation unit that includes this header.
constexpr uint32_t kRcp = 4096;
__device__ float g_rcp[kRcp];

// Bounds-checked builds (WX_BOUNDS_CHECK): wx_in_range(i, n) is i < n; an index
// out of range is counted in g_bounds_violations (read by wx_bounds_violations)
// and the caller skips the access. Other builds compile the checks away.
#ifdef WX_BOUNDS_CHECK
__device__ unsigned long long g_bounds_violations;
__device__ __forceinline__ bool wx_in_range(uint64_t i, uint64_t n) {
    if (i < n) return true;
    atomicAdd(&g_bounds_violations, 1ull);
    return false;
}
#else
__device__ __forceinline__ constexpr bool wx_in_range(uint64_t, uint64_t) { return true; }
#endif

__device__ __forceinline__ float pmin(float a, float b) { return (b < a || a != a) ? b : a; }
__device__ __forceinline__ float pmax(float a, float b) { return (b > a || a != a) ? b : a; }
__device__ __forceinline__ float sign11(float x) { return x < 0.0f ? -1.0f : 1.0f; }

// RN(p / size) for the three coordinates of one step. size = dist * 2^sk, so
// y = RN(1/dist) * 2^-sk equals RN(1/size) exactly (a power-of-two scaling).
// With q0 = RN(p*y), the residual e = p - q0*size is exact in one FMA and
// RN(q0 + e*y) is the correctly rounded quotient (Markstein, IBM J. Res. Dev.
// 34(1), 1990). The identity is invariant under power-of-two scaling while
// every intermediate stays a normal number, so the exhaustive GPU check over
// every divisor d < 4096 and every significand of [1,2) and [-2,-1)
// (wx_check_division) covers every exponent. The result is bit-identical to
// __fdiv_rn except that a zero quotient may come out +0 for p = -0; the march
// cannot observe that sign (mod = p - size*floor(q) enters only
// size*step01 - mod, where +0 and -0 give the same value). Other cases
// (dist >= 4096, or a coordinate with |p| < 2^-64, where q0 could underflow)
// take __fdiv_rn.
__device__ __forceinline__ float rcp_size(uint32_t dist, uint32_t rbits, bool *fast) {
    *fast = dist < kRcp;
    const float r = __ldg(&g_rcp[*fast ? dist : 1u]);
    return r * __uint_as_float(rbits);  // rbits = 2^-sk, sk <= 12
}
__device__ __forceinline__ float div_fast(float p, float size, float y) {
    const float q0 = p * y;
    const float e = __fmaf_rn(-q0, size, p);
    return __fmaf_rn(e, y, q0);
}

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

// State of one hdda_ray (raycast.comp.wgsl:84-126) between iterations. The
// cached parent chain of get_vdb_leaf_from_leaf (:360-396) is kept as the
// pool indices of the cached N5/N4/N3 plus the voxel of the previous lookup:
// that voxel lies inside every cached node (levels 1..np), so "pos is in the
// cached node of side S" is ((x ^ lx) | (y ^ ly) | (z ^ lz)) & ~(S - 1) == 0.
// Per-ray constant: idir = 1/dir. step01 = max(0, sign11(dir)) (:86-88) is
// 0 where dir < 0 and 1 elsewhere (NaN included); it is derived from dir in each
// step rather than kept (fewer live registers). The nudge 4e-4 * step of :122 is
// (step01 - 0.5) * RN(8e-4), exactly +-RN(8e-4) / 2 because RN commutes with
// scaling by two.
struct Ray {
    float px, py, pz;
    float dx, dy, dz;
    float ix, iy, iz;
    int lx, ly, lz;
    uint32_t np, i5, i4, i3;
    uint32_t i;
    bool mx, my, mz;   // mask of the last step
};

__device__ __forceinline__ void ray_init(Ray &r, F3 src, F3 dir) {
    r.px = src.x; r.py = src.y; r.pz = src.z;
    r.dx = dir.x; r.dy = dir.y; r.dz = dir.z;
    r.ix = __frcp_rn(dir.x); r.iy = __frcp_rn(dir.y); r.iz = __frcp_rn(dir.z);
    r.lx = r.ly = r.lz = 0;
    r.np = 0; r.i5 = r.i4 = r.i3 = 0;
    r.mx = r.my = r.mz = false;
    r.i = 0;
}

__device__ __forceinline__ uint32_t ray_mask(const Ray &r) {
    return (uint32_t)r.mx | ((uint32_t)r.my << 1) | ((uint32_t)r.mz << 2);
}

// A ray takes the careful step (ray_step<true>) when
// * 1/dir can be infinite (a direction component of magnitude below 2^-126,
//   zero, or NaN): only then can idir * (size*step01 - mod) be inf * 0 = NaN;
//   otherwise every tMax is a number and min/argmin need no NaN handling;
// * a source coordinate is -0: only then can a position coordinate be -0
//   (an RN sum is -0 only when both addends are -0), and only for -0 does
//   p + (4e-4 * step) * 0 differ from p (it gives +0 when step > 0), so
//   elsewhere the nudge of an unmasked axis is the identity.
__device__ __forceinline__ bool ray_needs_careful_step(F3 src, F3 dir) {
    const bool neg0 = (__float_as_uint(src.x) == 0x80000000u) | (__float_as_uint(src.y) == 0x80000000u) |
                      (__float_as_uint(src.z) == 0x80000000u);
    // Each comparison is false for NaN (fminf would drop a NaN component).
    return neg0 || !(fabsf(dir.x) >= 0x1p-126f && fabsf(dir.y) >= 0x1p-126f && fabsf(dir.z) >= 0x1p-126f);
}

// Exact distance of a leaf voxel whose byte is 255 (distance >= 255): binary
// search of the grid's sorted overflow table, which holds every such voxel.
// Inlined: as a call, the registers live across it spilled around the march
// (measured: 132 -> 108 bytes of spill stores in k_pixel, +0.4% on 1080p frames).
__device__ __forceinline__ uint32_t leaf_overflow(const DevGrid &g, uint32_t key) {
    uint32_t lo = 0, hi = g.n_ovf;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&g.ovf[mid].x) < key) lo = mid + 1;
        else hi = mid;
    }
    return lo < g.n_ovf ? __ldg(&g.ovf[lo].y) : 255u;
}

constexpr uint32_t kNoNode = 0xFFFFFFFFu;

// Index of the N5 whose origin is (x, y, z) & ~4095, or kNoNode: the dense
// table of root keys (the first matching origin of the shader's scan), or the
// scan itself when the key box was too large for a table.
__device__ __forceinline__ uint32_t root_find(const DevGrid &g, int x, int y, int z) {
    const int4 h0 = __ldg(g.root), h1 = __ldg(g.root + 1);
    if (h1.w) {
        const uint32_t ux = (uint32_t)((x >> 12) - h0.x), uy = (uint32_t)((y >> 12) - h0.y),
                       uz = (uint32_t)((z >> 12) - h0.z);
        if (ux < (uint32_t)h0.w && uy < (uint32_t)h1.x && uz < (uint32_t)h1.y) {
            const uint32_t *tab = reinterpret_cast<const uint32_t *>(g.root + 2 + g.n5);
            const uint32_t e = __ldg(tab + (uz * (uint32_t)h1.x + uy) * (uint32_t)h0.w + ux);
            if (e) return e - 1u;
        }
        return kNoNode;
    }
    const int kx = x & ~4095, ky = y & ~4095, kz = z & ~4095;
    for (uint32_t k = 0; k < g.n5; k++) {
        const int4 o = __ldg(g.root + 2 + k);
        if (o.x == kx && o.y == ky && o.z == kz) return k;
    }
    return kNoNode;
}

// One loop iteration of hdda_ray. Returns 0xFF while the march continues,
// otherwise the final state (0 hit, 1 out of bounds, 2 step cap); on return
// r.i is the iteration count the shader reports. kCareful selects the
// NaN-aware min/argmin and the literal nudge (see ray_needs_careful_step);
// both variants give identical results on the rays the fast one is used for.
template <bool kCareful, bool kFmaStep01 = true>
__device__ __forceinline__ uint32_t ray_step(const DevGrid &g, Ray &r) {
    if (r.i >= kMaxSteps) return 2u;
    // vec3<i32>(floor(p)): one saturating round-down conversion (NaN -> 0).
    const int x = __float2int_rd(r.px), y = __float2int_rd(r.py), z = __float2int_rd(r.pz);
    const uint32_t d = (uint32_t)((x ^ r.lx) | (y ^ r.ly) | (z ^ r.lz));
    r.lx = x; r.ly = y; r.lz = z;
    int lvl;
    if (r.np == 3 && d < 8u) lvl = 3;
    else if (r.np >= 2 && d < 128u) lvl = 4;
    else if (r.np >= 1 && d < 4096u) lvl = 5;
    else lvl = 0;
    uint32_t dist = 1;
    if (lvl == 0) {  // get_vdb_leaf_from_nothing (:398-413): the N5 whose origin is floor(p) & ~4095
        const uint32_t k = root_find(g, x, y, z);
        if (k != kNoNode) {
            r.i5 = k;
            lvl = 5;
        }
    }
    if (lvl == 5) {  // get_vdb_leaf_from_node5 (:415-444)
        if (!wx_in_range(r.i5, g.n5)) return 1u;
        const uint32_t off = ((((uint32_t)x >> 7) & 31u) << 10) | ((((uint32_t)y >> 7) & 31u) << 5) |
                             (((uint32_t)z >> 7) & 31u);
        const uint32_t w = __ldg(g.slot5 + ((r.i5 << 15) | off));
        if (w & kChild) {
            r.i4 = w & ~kChild;
            lvl = 4;
        } else {
            dist = w;
        }
    }
    if (lvl == 4) {  // get_vdb_leaf_from_node4 (:446-475)
        if (!wx_in_range(r.i4, g.n4)) return 1u;
        const uint32_t off = ((((uint32_t)x >> 3) & 15u) << 8) | ((((uint32_t)y >> 3) & 15u) << 4) |
                             (((uint32_t)z >> 3) & 15u);
        const uint32_t w = __ldg(g.slot4 + ((r.i4 << 12) | off));
        if (w & kChild) {
            r.i3 = w & ~kChild;
            lvl = 3;
        } else {
            dist = w;
        }
    }
    if (lvl == 3) {  // get_vdb_leaf_from_node3 (:477-494)
        if (!wx_in_range(r.i3, g.n3)) return 1u;
        const uint32_t key = (r.i3 << 9) | (((uint32_t)x & 7u) << 6) | (((uint32_t)y & 7u) << 3) | ((uint32_t)z & 7u);
        dist = __ldg(g.leaf + key);
        if (dist == 255u) dist = leaf_overflow(g, key);
    }
    // The levels reached set the cached parents once, after the lookup: the
    // level that resolved the voxel is 5, 4 or 3 (one, two or three cached
    // parents), or 0 after a root miss (none). The size scale of the resolving
    // level (:105-112) is 2^sk with sk = 12, 7, 3, 0 for 0..3 cached parents;
    // sbits and rbits are 2^sk and 2^-sk as float bits. (Setting np and the
    // scale inside each level block instead kept them live through the blocks:
    // 3.34 against 3.54 Grays/s on the 16 x 1080p spheres frames.)
    r.np = lvl ? 6u - (uint32_t)lvl : 0u;
    const uint32_t sk = (0x0003070Cu >> (8u * r.np)) & 0xFFu;
    const uint32_t sbits = (127u + sk) << 23, rbits = (127u - sk) << 23;
    if (dist == 0u) return 0u;
    const float apx = fabsf(r.px), apy = fabsf(r.py), apz = fabsf(r.pz);
    // any(4096 < |p|); a NaN coordinate compares false, and fmaxf skips NaN.
    // Not needed when this step found an N5 (r.np >= 1) of a grid whose N5s
    // all lie in [-4096, 4096)^3: then floor(p) is in that box, so |p| <= 4096.
    // (The fast step makes no NaN coordinate; an infinite one floors outside
    // every N5, so its step has r.np == 0 and is tested.)
    if ((kCareful || r.np == 0u || !g.inside) && 4096.0f < fmaxf(fmaxf(apx, apy), apz)) return 1u;
    // size = f32(dist) * scale[by num_parents] (:105-112); log2 scale by np = 12, 7, 3, 0.
    const float size = __uint2float_rn(dist) * __uint_as_float(sbits);
    bool fast;
    const float ys = rcp_size(dist, rbits, &fast);
    // tMax = idir * (size * step01 - (p - size * floor(p / size)))  (:78-80, :114)
    // step01 = max(0, sign11(dir)): 0 where dir < 0, else 1. The fast step only
    // takes rays whose direction components are nonzero numbers, for which
    // copysign(0.5, d) + 0.5 gives the same 0 or 1 (on the FMA pipe).
    // kFmaStep01 = false keeps the compare-and-select form in the fast step too:
    // the persistent kernels spill more with the copysign form and run slower
    // with it (4.45 -> 4.32 Grays/s on the mixed batch), while k_pixel gains.
    constexpr bool kSel = kCareful || !kFmaStep01;
    const float ax = kSel ? (r.dx < 0.0f ? 0.0f : 1.0f) : __fadd_rn(copysignf(0.5f, r.dx), 0.5f);
    const float ay = kSel ? (r.dy < 0.0f ? 0.0f : 1.0f) : __fadd_rn(copysignf(0.5f, r.dy), 0.5f);
    const float az = kSel ? (r.dz < 0.0f ? 0.0f : 1.0f) : __fadd_rn(copysignf(0.5f, r.dz), 0.5f);
    float tx, ty, tz;
    // The fast quotient needs every coordinate of magnitude >= 2^-64 (a zero
    // coordinate also takes the IEEE path here; both give the same floor).
    if (fast && fminf(fminf(apx, apy), apz) >= 0x1p-64f) {
        // Here both products are exact, so each subtraction of a product is
        // one FMA with the same rounding: size * step01 is 0 or size, and
        // size * floor(p / size) = dist * f * 2^sk with |dist * f| <=
        // 4096 / 2^sk + dist < 2^24 (|p| <= 4096 past the bounds test or where
        // it was skipped).
        const float fx = floorf(div_fast(r.px, size, ys));
        const float fy = floorf(div_fast(r.py, size, ys));
        const float fz = floorf(div_fast(r.pz, size, ys));
        tx = r.ix * __fmaf_rn(size, ax, -__fmaf_rn(-size, fx, r.px));
        ty = r.iy * __fmaf_rn(size, ay, -__fmaf_rn(-size, fy, r.py));
        tz = r.iz * __fmaf_rn(size, az, -__fmaf_rn(-size, fz, r.pz));
    } else {
        tx = r.ix * (size * ax - (r.px - size * floorf(__fdiv_rn(r.px, size))));
        ty = r.iy * (size * ay - (r.py - size * floorf(__fdiv_rn(r.py, size))));
        tz = r.iz * (size * az - (r.pz - size * floorf(__fdiv_rn(r.pz, size))));
    }
    float t;
    bool mx, my, mz;
    if (kCareful) {
        t = pmin(pmin(tx, ty), tz);
        mx = (tx <= ty) && (tx <= tz);
        my = (ty <= tz) && (ty <= tx);
        mz = (tz <= tx) && (tz <= ty);
    } else {
        // Without NaN, min(min(tx, ty), tz) is one of the three values; on a tie
        // of +0 and -0 the shader keeps its first operand and fminf may return
        // the other zero, which changes nothing: p + (+-0) * d is p (p is never
        // -0 here, see ray_needs_careful_step). (a <= b && a <= c) is
        // a == min(a, b, c), +0 and -0 comparing equal.
        t = fminf(fminf(tx, ty), tz);
        mx = tx == t;
        my = ty == t;
        mz = tz == t;
    }
    r.px = r.px + t * r.dx;
    r.py = r.py + t * r.dy;
    r.pz = r.pz + t * r.dz;
    r.mx = mx;
    r.my = my;
    r.mz = mz;
    // p += (4e-4 * step) * f32(mask)  (:122); without a -0 coordinate the
    // unmasked axes are unchanged.
    // +-kNudge as ax * 2 kNudge - kNudge, exact for ax in {0, 1}.
    const float kNudge = 0.5f * 8e-4f;
    const float nx = __fmaf_rn(ax, 2.0f * kNudge, -kNudge), ny = __fmaf_rn(ay, 2.0f * kNudge, -kNudge),
                nz = __fmaf_rn(az, 2.0f * kNudge, -kNudge);
    if (kCareful) {
        r.px = r.px + nx * (mx ? 1.0f : 0.0f);
        r.py = r.py + ny * (my ? 1.0f : 0.0f);
        r.pz = r.pz + nz * (mz ? 1.0f : 0.0f);
    } else {
        r.px = mx ? r.px + nx : r.px;
        r.py = my ? r.py + ny : r.py;
        r.pz = mz ? r.pz + nz : r.pz;
    }
    r.i++;
    return 0xFFu;
}

__device__ __forceinline__ uint32_t ray_node(const Ray &r) {
    return r.np == 3 ? r.i3 : r.np == 2 ? r.i4 : r.np == 1 ? r.i5 : 0xFFFFFFFFu;
}

struct March {
    F3 p;
    uint32_t state;  // 0 hit, 1 out of bounds, 2 step cap
    uint32_t np;     // cached parents (level)
    uint32_t node;   // pool index of the deepest cached node
    uint32_t i;      // loop iteration at return
    uint32_t mask;   // bit0 x, bit1 y, bit2 z
};

// HDDAout of a ray that returned state st (raycast.comp.wgsl:128-142).
__device__ __forceinline__ March march_result(const Ray &r, uint32_t st) {
    March m;
    m.p = f3(r.px, r.py, r.pz);
    m.state = st;
    m.np = r.np;
    m.node = ray_node(r);
    m.i = r.i;
    m.mask = ray_mask(r);
    return m;
}

// hdda_ray (raycast.comp.wgsl:84-126) run to completion.
template <bool kFmaStep01 = true>
__device__ __forceinline__ March hdda(const DevGrid &g, F3 src, F3 dir) {
    Ray r;
    ray_init(r, src, dir);
    uint32_t st;
    if (ray_needs_careful_step(src, dir)) {
        while ((st = ray_step<true, kFmaStep01>(g, r)) == 0xFFu) {
        }
    } else {
        while ((st = ray_step<false, kFmaStep01>(g, r)) == 0xFFu) {
        }
    }
    return march_result(r, st);
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

// Lit material colour shared by mode 4 and reflect_ray2/1 (:199-208, :280-290, :317-325).
__device__ __forceinline__ F3 lit_colour(const DevGrid &g, const wx_state_uniform &s, const March &h, F3 step,
                                         F3 N) {
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

__device__ __noinline__ F3 reflect_ray1(const DevGrid &g, const wx_state_uniform &s, F3 src, F3 dir) {  // :311-342
    const March h = hdda(g, src, dir);
    const F3 step = step3(dir);
    if (h.state == 0u) return lit_colour(g, s, h, step, normalize3((-step) * maskf(h.mask)));
    if (h.state == 1u) return wall_colour(normalize3((-step) * maskf(h.mask)));
    return dir;
}

__device__ __noinline__ F3 reflect_ray2(const DevGrid &g, const wx_state_uniform &s, F3 src, F3 dir) {  // :267-309
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

// The `grid` tint of ray_trace (:157-166).
__device__ __forceinline__ F3 grid_tint(const wx_state_uniform &s, F3 p) {
    const float fx = floorf(p.x), fy = floorf(p.y), fz = floorf(p.z);
    if (s.show_345[2] == 1u && (grid_line(fx, 4096.0f) || grid_line(fy, 4096.0f) || grid_line(fz, 4096.0f)))
        return f3(-0.3f, -0.3f, 1.0f);
    if (s.show_345[1] == 1u && (grid_line(fx, 128.0f) || grid_line(fy, 128.0f) || grid_line(fz, 128.0f)))
        return f3(0.6f, -0.2f, -0.2f);
    if (s.show_345[0] == 1u && (grid_line(fx, 8.0f) || grid_line(fy, 8.0f) || grid_line(fz, 8.0f)))
        return f3(-0.1f, 0.5f, 0.3f);
    return splat(0.0f);
}

// I_a of mode 3 (:186), the colour of a shadowed lit pixel.
__device__ __forceinline__ F3 ambient_colour() { return (kKa * f3(0.4f, 0.4f, 0.3f)) * f3(0.4f, 0.2f, 0.2f); }

// Colour of a finished primary ray for modes 0-2 and the non-lit part of
// modes 0-3 (:156-194 for state 0, :231-262 for state 1, :264 otherwise).
// For mode 3 with a hit, *need_shadow tells the caller to trace the shadow
// ray (:188-193); the colour returned is then I_a + I_d (the unshadowed case)
// and *shadowed_colour receives I_a.
__device__ __forceinline__ F3 primary_colour(const wx_state_uniform &s, const March &hit, F3 dir, bool *need_shadow,
                                             F3 *shadowed_colour, F3 *shadow_src) {
    const F3 step = step3(dir);
    const uint32_t mode = s.render_mode[0];
    *need_shadow = false;
    if (hit.state == 0u) {
        const F3 m = maskf(hit.mask);
        const F3 grid = grid_tint(s, hit.p);
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
            const F3 I_a = ambient_colour();
            if (LN != 0.0f) {
                *need_shadow = true;
                *shadowed_colour = I_a;
                *shadow_src = hit.p - (4e-2f * step) * m;
            }
            return I_a + I_d;
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
        const F3 a = m * f3(0.01f, 0.02f, 0.03f);
        return splat(0.0f) + splat((a.x + a.y) + a.z);
    }
    return dir;
}

// Glossy mode (:195-224 for state 0, :246-257 for state 1), up to six rays.
__device__ __noinline__ F3 glossy_colour(const DevGrid &g, const wx_state_uniform &s, const March &hit, F3 dir) {
    const F3 step = step3(dir);
    const F3 m = maskf(hit.mask);
    const F3 N = normalize3((-step) * m);
    if (hit.state == 0u) {
        const F3 mcol = lit_colour(g, s, hit, step, N);
        const F3 rdir = normalize3(dir - (2.0f * N) * dot3(dir, N));
        const F3 rsrc = hit.p - (4e-2f * step) * m;
        const F3 rcol = reflect_ray2(g, s, rsrc, rdir);
        return mix3(mcol, rcol, kReflect);
    }
    if (hit.state == 1u) {
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
    return dir;
}

// cp_main's ray (raycast.comp.wgsl:62-63) for pixel (gx, gy).
__device__ __forceinline__ F3 primary_dir(const wx_state_uniform &s, uint32_t gx, uint32_t gy) {
    const float px = __uint2float_rn(gx) + 0.001f, py = __uint2float_rn(gy) + 0.001f;
    return normalize3(f3((px * s.u[0] + py * s.mv[0]) + s.wp[0], (px * s.u[1] + py * s.mv[1]) + s.wp[1],
                         (px * s.u[2] + py * s.mv[2]) + s.wp[2]));
}

__device__ __forceinline__ uint32_t pack_rgba(F3 c) {
    return unorm8(c.x) | (unorm8(c.y) << 8) | (unorm8(c.z) << 16) | (255u << 24);
}

__device__ __forceinline__ void store_hit(wx_hit *h, F3 p, float t, uint32_t node, uint32_t info, uint32_t shadow,
                                          uint32_t reserved = 0u) {
    uint4 *q = reinterpret_cast<uint4 *>(h);
    q[0] = make_uint4(__float_as_uint(p.x), __float_as_uint(p.y), __float_as_uint(p.z), __float_as_uint(t));
    q[1] = make_uint4(node, info, shadow, reserved);
}

// ---------------------------------------------------------------------------
// Zero-crossing hit mode (WX_MODE_SURFACE). An extension with no counterpart
// in the reference, specified by the oracle's surf_* functions, which this
// code follows operation for operation.
// ---------------------------------------------------------------------------
constexpr float kSurfH = 0.25f;   // sample spacing along the ray, voxels
constexpr uint32_t kSurfN = 64u;  // samples

// Level-set value of voxel (i, j, k): the leaf value, -band inside an active
// tile (slot word 0), +band anywhere else.
__device__ __forceinline__ float surf_phi(const DevGrid &g, int i, int j, int k) {
    const uint32_t n5 = root_find(g, i, j, k);
    if (n5 == kNoNode) return g.band;
    const uint32_t w5 = __ldg(g.slot5 + ((n5 << 15) | ((((uint32_t)i >> 7) & 31u) << 10) |
                                         ((((uint32_t)j >> 7) & 31u) << 5) | (((uint32_t)k >> 7) & 31u)));
    if (!(w5 & kChild)) return w5 == 0u ? -g.band : g.band;
    if (!wx_in_range(w5 & ~kChild, g.n4)) return g.band;
    const uint32_t w4 = __ldg(g.slot4 + (((w5 & ~kChild) << 12) | ((((uint32_t)i >> 3) & 15u) << 8) |
                                         ((((uint32_t)j >> 3) & 15u) << 4) | (((uint32_t)k >> 3) & 15u)));
    if (!(w4 & kChild)) return w4 == 0u ? -g.band : g.band;
    if (!wx_in_range(w4 & ~kChild, g.n3)) return g.band;
    return __ldg(g.values + (((w4 & ~kChild) << 9) | (((uint32_t)i & 7u) << 6) | (((uint32_t)j & 7u) << 3) |
                             ((uint32_t)k & 7u)));
}

__device__ __forceinline__ float lerpf(float a, float b, float t) { return a + t * (b - a); }

// Corner values of the cell of q (corner n = dx << 2 | dy << 1 | dz) and q's
// position inside it.
__device__ __forceinline__ void surf_cell(const DevGrid &g, F3 q, float c[8], float f[3]) {
    const float fx = floorf(q.x), fy = floorf(q.y), fz = floorf(q.z);
    const int i = __float2int_rd(q.x), j = __float2int_rd(q.y), k = __float2int_rd(q.z);
    f[0] = q.x - fx;
    f[1] = q.y - fy;
    f[2] = q.z - fz;
#pragma unroll
    for (int n = 0; n < 8; n++) c[n] = surf_phi(g, i + (n >> 2), j + ((n >> 1) & 1), k + (n & 1));
}

__device__ __forceinline__ float surf_interp(const float c[8], const float f[3]) {
    const float a00 = lerpf(c[0], c[4], f[0]), a10 = lerpf(c[2], c[6], f[0]);
    const float a01 = lerpf(c[1], c[5], f[0]), a11 = lerpf(c[3], c[7], f[0]);
    return lerpf(lerpf(a00, a10, f[1]), lerpf(a01, a11, f[1]), f[2]);
}

__device__ __forceinline__ F3 surf_gradient(const float c[8], const float f[3]) {
    const float gx = lerpf(lerpf(c[4] - c[0], c[6] - c[2], f[1]), lerpf(c[5] - c[1], c[7] - c[3], f[1]), f[2]);
    const float gy = lerpf(lerpf(c[2] - c[0], c[6] - c[4], f[0]), lerpf(c[3] - c[1], c[7] - c[5], f[0]), f[2]);
    const float gz = lerpf(lerpf(c[1] - c[0], c[5] - c[4], f[0]), lerpf(c[3] - c[2], c[7] - c[6], f[0]), f[1]);
    return f3(gx, gy, gz);
}

__device__ __forceinline__ float surf_sample(const DevGrid &g, F3 eye, F3 dir, float t) {
    float c[8], f[3];
    surf_cell(g, f3(eye.x + t * dir.x, eye.y + t * dir.y, eye.z + t * dir.z), c, f);
    return surf_interp(c, f);
}

// Search from t_hit - 1 (the HDDA hit's t); true with t*, the sample index and
// the normal when phi changes sign within kSurfN samples.
__device__ __noinline__ bool surf_search(const DevGrid &g, F3 eye, F3 dir, float t_hit, float *ts, uint32_t *ks,
                                         F3 *N) {
    if (!g.values) return false;
    float t0 = t_hit - 1.0f;
    if (!(t0 > 0.0f)) t0 = 0.0f;
    float prev = surf_sample(g, eye, dir, t0);
    bool found = false;
    if (prev <= 0.0f) {
        *ts = t0;
        *ks = 0;
        found = true;
    } else {
        for (uint32_t k = 1; k < kSurfN; k++) {
            const float tk = t0 + __uint2float_rn(k) * kSurfH;
            const float ph = surf_sample(g, eye, dir, tk);
            if (ph <= 0.0f) {
                const float tp = t0 + __uint2float_rn(k - 1u) * kSurfH;
                *ts = tp + kSurfH * __fdiv_rn(prev, prev - ph);
                *ks = k;
                found = true;
                break;
            }
            prev = ph;
        }
    }
    if (!found) return false;
    float c[8], f[3];
    surf_cell(g, f3(eye.x + *ts * dir.x, eye.y + *ts * dir.y, eye.z + *ts * dir.z), c, f);
    const F3 gr = surf_gradient(c, f);
    *N = dot3(gr, gr) == 0.0f ? -dir : normalize3(gr);
    return true;
}

// Mode 5 colour: mode 3's I_a + I_d with normal N, no shadow ray.
__device__ __forceinline__ F3 surface_colour(const wx_state_uniform &s, F3 N) {
    const F3 sun = f3(s.sun_dir[0], s.sun_dir[1], s.sun_dir[2]);
    const F3 sc = f3(s.sun_color[0], s.sun_color[1], s.sun_color[2]);
    const float LN = pmax(0.0f, s.sun_color[3] * dot3(-sun, N));
    const F3 I_d = ((kKd * sc) * f3(0.4f, 0.2f, 0.2f)) * LN;
    return ambient_colour() + I_d;
}

}  // namespace wxd
