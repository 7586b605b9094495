// scene.cpp — synthetic VDB345 grids (seeded), orbit cameras and the
// ComputeState uniform builder. Host code, no GPU.
//
// The reference ships no generator: its grids come from .vdb files. These are
// the seeded stand-ins for the benchmark workloads: f32 narrow-band level sets
// of one sphere / a union of spheres (value = signed distance in voxels, a
// voxel is active iff |d| < band), and a sparse noise-driven leaf field.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <unordered_map>

#include "wx_common.h"

namespace wx {

// splitmix64 (Steele, Lea, Flood 2014): the seeded stream behind every generator.
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }  // [0, 1)
};
static inline uint64_t mix64(uint64_t a, uint64_t b) {
    Rng r(a * 0xD6E8FEB86659FD93ull ^ (b + 0x632BE59BD9B4E019ull));
    return r.next();
}

static int hw_threads(int n) {
    if (n > 0) return n;
    unsigned h = std::thread::hardware_concurrency();
    return h ? (int)h : 4;
}

template <class F>
static void parallel_for(size_t n, int nthreads, F f) {
    nthreads = std::max(1, std::min<int>(nthreads, (int)std::max<size_t>(n, 1)));
    if (nthreads == 1) {
        for (size_t i = 0; i < n; i++) f(i);
        return;
    }
    std::vector<std::thread> th;
    std::atomic<size_t> next{0};
    for (int t = 0; t < nthreads; t++)
        th.emplace_back([&] {
            for (;;) {
                size_t i = next.fetch_add(1);
                if (i >= n) break;
                f(i);
            }
        });
    for (auto &x : th) x.join();
}

struct Sphere {
    double c[3], r;
};

// Active-voxel masks of one leaf: |min_s(|v - c_s| - r_s)| < band.
static bool sphere_leaf(const I3 &o, const Sphere *s, const uint32_t *ids, size_t nids, double band,
                        uint64_t m[8]) {
    bool any = false;
    for (int w = 0; w < 8; w++) m[w] = 0;
    for (uint32_t v = 0; v < 512; v++) {
        const double x = o[0] + (int)(v >> 6), y = o[1] + (int)((v >> 3) & 7), z = o[2] + (int)(v & 7);
        double d = INFINITY;
        for (size_t k = 0; k < nids; k++) {
            const Sphere &q = s[ids[k]];
            const double dx = x - q.c[0], dy = y - q.c[1], dz = z - q.c[2];
            d = std::min(d, std::sqrt(dx * dx + dy * dy + dz * dz) - q.r);
        }
        if (std::fabs(d) < band) {
            m[v >> 6] |= 1ull << (v & 63);
            any = true;
        }
    }
    return any;
}

struct LeafHash {
    size_t operator()(const I3 &k) const {
        return (size_t)mix64(((uint64_t)(uint32_t)k[0] << 32) | (uint32_t)k[1], (uint32_t)k[2]);
    }
};
using SphereBins = std::unordered_map<I3, std::vector<uint32_t>, LeafHash>;

// The spheres whose band can touch each leaf, by leaf origin.
static SphereBins bin_spheres(const std::vector<Sphere> &sph, double band) {
    SphereBins bins;
    for (uint32_t i = 0; i < sph.size(); i++) {
        int32_t lo[3], hi[3];
        for (int a = 0; a < 3; a++) {
            lo[a] = node_origin((int32_t)std::floor(sph[i].c[a] - sph[i].r - band), 3);
            hi[a] = node_origin((int32_t)std::ceil(sph[i].c[a] + sph[i].r + band), 3);
        }
        for (int32_t x = lo[0]; x <= hi[0]; x += 8)
            for (int32_t y = lo[1]; y <= hi[1]; y += 8)
                for (int32_t z = lo[2]; z <= hi[2]; z += 8) bins[I3{x, y, z}].push_back(i);
    }
    return bins;
}

static int spheres_to_topology(const std::vector<Sphere> &sph, double band, int nthreads,
                               wx_topology **out) {
    const SphereBins bins = bin_spheres(sph, band);
    std::vector<I3> keys;
    keys.reserve(bins.size());
    for (auto &kv : bins) keys.push_back(kv.first);
    std::vector<uint64_t> masks(keys.size() * 8);
    std::vector<uint8_t> keep(keys.size());
    parallel_for(keys.size(), hw_threads(nthreads), [&](size_t i) {
        const auto &ids = bins.at(keys[i]);
        keep[i] = sphere_leaf(keys[i], sph.data(), ids.data(), ids.size(), band, &masks[8 * i]);
    });
    std::vector<int32_t> org;
    std::vector<uint64_t> msk;
    for (size_t i = 0; i < keys.size(); i++) {
        if (!keep[i]) continue;
        org.insert(org.end(), keys[i].begin(), keys[i].end());
        msk.insert(msk.end(), &masks[8 * i], &masks[8 * i] + 8);
    }
    return wx_topology_from_leaves(org.data(), msk.data(), org.size() / 3, out);
}

// 3-octave value noise on the leaf lattice: corner values uniform in [0,1)
// from a hash of (seed, octave, corner), smoothstep-weighted trilinear
// interpolation, cell sizes n/8, n/16, n/32 leaves, amplitudes 1, 1/2, 1/4.
struct ValueNoise {
    int n;
    int cells[3];
    std::vector<float> corners[3];
    ValueNoise(int lattice, uint64_t seed) : n(lattice) {
        for (int k = 0; k < 3; k++) {
            cells[k] = 8 << k;
            const int c = cells[k] + 1;
            corners[k].resize((size_t)c * c * c);
            for (int x = 0; x < c; x++)
                for (int y = 0; y < c; y++)
                    for (int z = 0; z < c; z++) {
                        uint64_t h = mix64(seed ^ (0x1000193ull * (k + 1)),
                                           ((uint64_t)x << 42) | ((uint64_t)y << 21) | (uint64_t)z);
                        corners[k][((size_t)x * c + y) * c + z] = (float)((h >> 40) * 0x1.0p-24);
                    }
        }
    }
    float at(int lx, int ly, int lz) const {
        float sum = 0.0f, amp = 1.0f;
        for (int k = 0; k < 3; k++) {
            const int c = cells[k] + 1;
            const float scale = (float)cells[k] / (float)n;
            float u[3] = {(lx + 0.5f) * scale, (ly + 0.5f) * scale, (lz + 0.5f) * scale};
            int i0[3];
            float w[3];
            for (int a = 0; a < 3; a++) {
                i0[a] = std::min((int)std::floor(u[a]), cells[k] - 1);
                const float f = u[a] - (float)i0[a];
                w[a] = f * f * (3.0f - 2.0f * f);
            }
            const float *g = corners[k].data();
            auto G = [&](int dx, int dy, int dz) {
                return g[((size_t)(i0[0] + dx) * c + (i0[1] + dy)) * c + (i0[2] + dz)];
            };
            const float x00 = G(0, 0, 0) + w[0] * (G(1, 0, 0) - G(0, 0, 0));
            const float x10 = G(0, 1, 0) + w[0] * (G(1, 1, 0) - G(0, 1, 0));
            const float x01 = G(0, 0, 1) + w[0] * (G(1, 0, 1) - G(0, 0, 1));
            const float x11 = G(0, 1, 1) + w[0] * (G(1, 1, 1) - G(0, 1, 1));
            const float y0 = x00 + w[1] * (x10 - x00), y1 = x01 + w[1] * (x11 - x01);
            sum += amp * (y0 + w[2] * (y1 - y0));
            amp *= 0.5f;
        }
        return sum;
    }
};

}  // namespace wx

using namespace wx;

extern "C" {

const char *wx_version(void) { return "woxel_gb300 0.1.0 (sm_103a)"; }

void wx_sun_default(float dir[3], float color[3], float *intensity) {
    // SunSettings::default (egui_dev.rs:355-368): glam Vec3::normalize = v * (1 / |v|).
    const float v[3] = {1.0f, -1.0f, 0.5f};
    const float len = std::sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
    const float r = 1.0f / len;
    for (int i = 0; i < 3; i++) dir[i] = v[i] * r;
    color[0] = 255.0f / 255.0f;
    color[1] = 210.0f / 255.0f;
    color[2] = 160.0f / 255.0f;
    *intensity = 1.0f;
}

// ComputeState::build (compute_state.rs:87-131) for Camera::build_view_projection_matrix
// (camera.rs:31-35, cgmath 0.18 Matrix4::look_at_rh). cgmath normalises as
// v * (1 / |v|) and sums dot products left to right; the inverse is an
// adjugate/determinant expansion (cgmath's own Matrix4::invert is not in the
// reference tree, so the last bits of camera_to_world are not pinned to it).
int wx_state_build(const float eye[3], const float target[3], const float up[3], float aspect,
                   float fovy_deg, float width, uint32_t render_mode, const uint32_t show_345[3],
                   const float sun_dir[3], const float sun_color[3], float sun_intensity,
                   wx_state_uniform *o) {
    if (!eye || !target || !up || !sun_dir || !sun_color || !o || !(aspect > 0.0f)) {
        set_thread_error("wx_state_build: null pointer or non-positive aspect");
        return WX_ERR_INVALID;
    }
    memset(o, 0, sizeof(*o));
    auto norm = [](float v[3]) {
        const float m = std::sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
        const float s = 1.0f / m;
        for (int i = 0; i < 3; i++) v[i] = v[i] * s;
    };
    auto cross = [](const float a[3], const float b[3], float r[3]) {
        r[0] = a[1] * b[2] - a[2] * b[1];
        r[1] = a[2] * b[0] - a[0] * b[2];
        r[2] = a[0] * b[1] - a[1] * b[0];
    };
    auto dot = [](const float a[3], const float b[3]) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; };
    float f[3] = {target[0] - eye[0], target[1] - eye[1], target[2] - eye[2]};
    norm(f);
    float s[3], u[3];
    cross(f, up, s);
    norm(s);
    cross(s, f, u);
    const float view[16] = {s[0], u[0], -f[0], 0.0f, s[1], u[1], -f[1], 0.0f,
                            s[2], u[2], -f[2], 0.0f, -dot(eye, s), -dot(eye, u), dot(eye, f), 1.0f};
    // Inverse by cofactors; m is column-major (m[c*4 + r]).
    auto det3 = [](float a, float b, float c, float d, float e, float f_, float g, float h, float i) {
        return a * (e * i - f_ * h) - b * (d * i - f_ * g) + c * (d * h - e * g);
    };
    float cof[16];
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) {
            float m9[9];
            int k = 0;
            for (int rr = 0; rr < 4; rr++) {
                if (rr == r) continue;
                for (int cc = 0; cc < 4; cc++)
                    if (cc != c) m9[k++] = view[cc * 4 + rr];
            }
            const float d = det3(m9[0], m9[1], m9[2], m9[3], m9[4], m9[5], m9[6], m9[7], m9[8]);
            cof[c * 4 + r] = ((r + c) & 1) ? -d : d;
        }
    const float det = view[0] * cof[0] + view[4] * cof[4] + view[8] * cof[8] + view[12] * cof[12];
    if (det == 0.0f) {
        set_thread_error("wx_state_build: camera matrix is not invertible");
        return WX_ERR_INVALID;
    }
    const float inv = 1.0f / det;
    float c2w[16];
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) c2w[c * 4 + r] = cof[r * 4 + c] * inv;
    memcpy(o->view_projection, view, sizeof view);
    memcpy(o->camera_to_world, c2w, sizeof c2w);
    for (int i = 0; i < 3; i++) o->eye[i] = eye[i];
    const float height = width / aspect;
    const float fovy_rad = fovy_deg * (3.14159265358979323846f / 180.0f);
    const float tan_half = std::tan(fovy_rad * 0.5f);
    const float a = -width / 2.0f, b = height / 2.0f;
    for (int i = 0; i < 4; i++) {
        const float uu = c2w[i], vv = c2w[4 + i], ww = c2w[8 + i];
        o->u[i] = uu;
        o->mv[i] = -vv;
        o->wp[i] = (a * uu + b * vv) - (ww * b) / tan_half;
    }
    o->render_mode[0] = render_mode;
    for (int i = 0; i < 3; i++) {
        o->show_345[i] = show_345 ? show_345[i] : 0u;
        o->sun_dir[i] = sun_dir[i];
        o->sun_color[i] = sun_color[i];
    }
    o->sun_color[3] = sun_intensity;
    return WX_OK;
}

int wx_gen_sphere(float cx, float cy, float cz, float radius, float band, wx_topology **out) {
    return wx::guard("wx_gen_sphere", [&]() -> int {
        if (!out || !(radius >= 0.0f) || !(band > 0.0f)) {
            set_thread_error("wx_gen_sphere: bad radius/band");
            return WX_ERR_INVALID;
        }
        std::vector<Sphere> s{{{cx, cy, cz}, radius}};
        return spheres_to_topology(s, band, 0, out);
    });
}

static std::vector<Sphere> sphere_list(uint32_t count, float rmin, float rmax, float lo, float hi, uint64_t seed) {
    Rng rng(seed);
    std::vector<Sphere> s(count);
    for (auto &q : s) {  // draw order per sphere: cx, cy, cz, r
        for (int a = 0; a < 3; a++) q.c[a] = lo + (hi - lo) * rng.uniform();
        q.r = rmin + (rmax - rmin) * rng.uniform();
    }
    return s;
}

int wx_gen_spheres(uint32_t count, float rmin, float rmax, float lo, float hi, float band,
                   uint64_t seed, wx_topology **out) {
    if (!out || !(rmin >= 0.0f) || !(rmax >= rmin) || !(hi > lo) || !(band > 0.0f)) {
        set_thread_error("wx_gen_spheres: bad parameters");
        return WX_ERR_INVALID;
    }
    return spheres_to_topology(sphere_list(count, rmin, rmax, lo, hi, seed), band, 0, out);
}

// Level-set values of the sphere generators for every voxel of every leaf of
// t, in DFS leaf order and voxel order x << 6 | y << 3 | z: the signed distance
// min_s(|v - c_s| - r_s) (the quantity whose |.| < band made the voxel active),
// clamped to [-band, band] as a narrow-band level set stores it.
static int spheres_values(const wx_topology *t, const std::vector<Sphere> &sph, double band, float *out) {
    SphereBins bins;
    try {
        bins = bin_spheres(sph, band);
    } catch (...) {
        set_thread_error("sphere values: host allocation failed");
        return WX_ERR_OOM;
    }
    parallel_for(t->o3.size(), hw_threads(0), [&](size_t i) {
        const I3 &o = t->o3[i];
        const auto it = bins.find(o);
        for (uint32_t v = 0; v < 512; v++) {
            double d = INFINITY;
            if (it != bins.end()) {
                const double x = o[0] + (int)(v >> 6), y = o[1] + (int)((v >> 3) & 7), z = o[2] + (int)(v & 7);
                for (uint32_t id : it->second) {
                    const Sphere &q = sph[id];
                    const double dx = x - q.c[0], dy = y - q.c[1], dz = z - q.c[2];
                    d = std::min(d, std::sqrt(dx * dx + dy * dy + dz * dz) - q.r);
                }
            }
            out[i * 512 + v] = (float)std::min(band, std::max(-band, d));
        }
    });
    return WX_OK;
}

int wx_gen_sphere_values(const wx_topology *t, float cx, float cy, float cz, float radius, float band,
                         float *values) {
    return wx::guard("wx_gen_sphere_values", [&]() -> int {
        if (!t || !values || !(radius >= 0.0f) || !(band > 0.0f)) {
            set_thread_error("wx_gen_sphere_values: bad arguments");
            return WX_ERR_INVALID;
        }
        std::vector<Sphere> s{{{cx, cy, cz}, radius}};
        return spheres_values(t, s, band, values);
    });
}

int wx_gen_spheres_values(const wx_topology *t, uint32_t count, float rmin, float rmax, float lo, float hi,
                          float band, uint64_t seed, float *values) {
    if (!t || !values || !(rmin >= 0.0f) || !(rmax >= rmin) || !(hi > lo) || !(band > 0.0f)) {
        set_thread_error("wx_gen_spheres_values: bad arguments");
        return WX_ERR_INVALID;
    }
    return spheres_values(t, sphere_list(count, rmin, rmax, lo, hi, seed), band, values);
}

int wx_gen_noise_leaves(int32_t lo, uint32_t extent, double occupancy, double p_voxel,
                        uint64_t seed, int nthreads, wx_topology **out) {
    if (!out || extent < 64 || (extent & 7) || !(occupancy > 0.0 && occupancy < 1.0) ||
        !(p_voxel >= 0.0 && p_voxel <= 1.0) || node_origin(lo, 3) != lo) {
        set_thread_error("wx_gen_noise_leaves: bad parameters");
        return WX_ERR_INVALID;
    }
    const int n = (int)(extent / 8);
    const size_t total = (size_t)n * n * n;
    ValueNoise noise(n, seed);
    std::vector<float> val;
    try {
        val.resize(total);
    } catch (...) {
        set_thread_error("wx_gen_noise_leaves: host allocation failed");
        return WX_ERR_OOM;
    }
    const int nt = hw_threads(nthreads);
    parallel_for((size_t)n, nt, [&](size_t x) {
        for (int y = 0; y < n; y++)
            for (int z = 0; z < n; z++) val[((size_t)x * n + y) * n + z] = noise.at((int)x, y, z);
    });
    // Threshold = the value with exactly round(occupancy * total) leaves above it.
    const size_t keep = (size_t)std::llround(occupancy * (double)total);
    float thr;
    {
        std::vector<float> tmp(val);
        const size_t kth = total - keep - (keep < total ? 1 : 0);
        std::nth_element(tmp.begin(), tmp.begin() + kth, tmp.end());
        thr = tmp[kth];
    }
    std::vector<int32_t> org;
    std::vector<uint64_t> msk;
    org.reserve(keep * 3);
    msk.reserve(keep * 8);
    for (size_t i = 0; i < total; i++) {
        if (!(val[i] > thr)) continue;
        const int x = (int)(i / ((size_t)n * n)), y = (int)((i / n) % n), z = (int)(i % n);
        org.push_back(lo + 8 * x);
        org.push_back(lo + 8 * y);
        org.push_back(lo + 8 * z);
        uint64_t m[8];
        for (int w = 0; w < 8; w++) {
            const uint64_t h = mix64(seed ^ 0xA5A5A5A5DEADBEEFull, (uint64_t)i * 8 + w);
            if (p_voxel == 0.5) {
                m[w] = h;
            } else {
                Rng r(h);
                uint64_t b = 0;
                for (int k = 0; k < 64; k++)
                    if (r.uniform() < p_voxel) b |= 1ull << k;
                m[w] = b;
            }
        }
        msk.insert(msk.end(), m, m + 8);
    }
    return wx_topology_from_leaves(org.data(), msk.data(), org.size() / 3, out);
}

int wx_orbit_eyes(uint32_t count, float radius, uint64_t seed, float *eyes) {
    if (!eyes || !(radius > 0.0f)) return WX_ERR_INVALID;
    Rng rng(seed);
    for (uint32_t i = 0; i < count; i++) {
        double y;
        do {
            y = 2.0 * rng.uniform() - 1.0;
        } while (std::fabs(y) > 0.9);
        const double phi = 2.0 * M_PI * rng.uniform();
        const double r = std::sqrt(1.0 - y * y);
        eyes[3 * i + 0] = (float)(radius * r * std::cos(phi));
        eyes[3 * i + 1] = (float)(radius * y);
        eyes[3 * i + 2] = (float)(radius * r * std::sin(phi));
    }
    return WX_OK;
}

}  // extern "C"
