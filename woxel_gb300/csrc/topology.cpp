// topology.cpp — VDB345 node structure, the per-level SDF sweep, and the
// reference-layout (masks/origins/atlas) export. Host code, no GPU.
//
// The SDF follows VDB345::compute_sdf (src/vdb/vdb345.rs:290-670). That
// routine walks the whole tree in DFS order twice (forward with the 13
// "earlier" neighbours, backward with the 13 "later" ones) and updates every
// tile slot to min(own, neighbour + 1), where a neighbour that is a child node
// or an active leaf voxel — or that get_voxel resolves to anything but a tile
// of the same level, including a missing node — counts as distance 0. Three
// facts make it cheaper to restate than to transcribe:
//   * the three levels never read each other's values (an N4 tile only looks
//     at N4-level slots, vdb345.rs:430-435; N5 at N5, :390-395; N3 at N3,
//     :470-476), so each level is an independent sweep;
//   * "solid" neighbours can be stored as distance 0, because min(d, 0 + 1)
//     reproduces the reference's "set to 1" (all tile distances are >= 1);
//   * while one node is being swept, no other node changes, so its 26
//     neighbours can be copied into a halo once, at the start of that node.
// Node order, slot order and in-place (Gauss-Seidel) updates are kept, so the
// result is bit-identical to the reference's, scan-order quirks included.

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <memory>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <thread>

#include "wx_common.h"

namespace wx {

static thread_local std::string g_thread_error;
void set_thread_error(const std::string &msg) { g_thread_error = msg; }

// Open-addressing map from node origin to DFS index.
class OriginIndex {
  public:
    explicit OriginIndex(const std::vector<I3> &keys) {
        size_t cap = 16;
        while (cap < keys.size() * 2 + 1) cap <<= 1;
        mask_ = cap - 1;
        keys_.assign(cap, I3{0, 0, 0});
        vals_.assign(cap, UINT32_MAX);
        for (size_t i = 0; i < keys.size(); i++) {
            size_t h = hash(keys[i]) & mask_;
            while (vals_[h] != UINT32_MAX) h = (h + 1) & mask_;
            keys_[h] = keys[i];
            vals_[h] = (uint32_t)i;
        }
    }
    uint32_t find(int64_t x, int64_t y, int64_t z) const {
        if (x < INT32_MIN || x > INT32_MAX || y < INT32_MIN || y > INT32_MAX || z < INT32_MIN ||
            z > INT32_MAX)
            return UINT32_MAX;
        I3 k{(int32_t)x, (int32_t)y, (int32_t)z};
        size_t h = hash(k) & mask_;
        while (vals_[h] != UINT32_MAX) {
            if (keys_[h] == k) return vals_[h];
            h = (h + 1) & mask_;
        }
        return UINT32_MAX;
    }

  private:
    static size_t hash(const I3 &k) {
        uint64_t h = (uint64_t)(uint32_t)k[0] * 0x9E3779B97F4A7C15ull;
        h ^= (uint64_t)(uint32_t)k[1] * 0xC2B2AE3D27D4EB4Full + (h >> 29);
        h ^= (uint64_t)(uint32_t)k[2] * 0x165667B19E3779F9ull + (h >> 31);
        return (size_t)(h ^ (h >> 33));
    }
    size_t mask_;
    std::vector<I3> keys_;
    std::vector<uint32_t> vals_;
};

// One level of compute_sdf. Containers (nodes of this level) are given in DFS
// order with their origins in voxels and extent 2^span_log2; cells hold 0 for
// solid slots and kSdfInf for tiles on entry, final distances on exit.
//
// The reference sweeps the containers one after the other (forward in DFS
// order, then backward). A container's sweep reads only itself and its 26
// neighbours, so the sequential order only matters between neighbours: in
// the forward pass a container must see its lower-index neighbours finished
// and its higher-index neighbours untouched (mirrored backward). With nthreads
// > 1 the sweeps run as a wavefront over that dependency DAG: a container
// becomes ready when all its earlier neighbours are done, so every container
// reads exactly the values the sequential order gives it.
template <int L>
static void chamfer_level(const std::vector<I3> &org, int span_log2, uint32_t *dist, int nthreads) {
    constexpr int D = 1 << L, P = D + 2, N = D * D * D;
    const size_t nc = org.size();
    if (nc == 0) return;
    OriginIndex index(org);
    const int64_t span = (int64_t)1 << span_log2;
    std::vector<uint32_t> nb(nc * 27);
    for (size_t c = 0; c < nc; c++)
        for (int k = 0; k < 27; k++) {
            const int dx = k / 9 - 1, dy = (k / 3) % 3 - 1, dz = k % 3 - 1;
            nb[c * 27 + k] = (k == 13) ? (uint32_t)c
                                       : index.find(org[c][0] + dx * span, org[c][1] + dy * span,
                                                    org[c][2] + dz * span);
        }
    auto bidx = [](int x, int y, int z) { return ((x + 1) * P + (y + 1)) * P + (z + 1); };

    auto fill = [&](size_t c, uint32_t *buf) {
        for (int k = 0; k < 27; k++) {
            const int d[3] = {k / 9 - 1, (k / 3) % 3 - 1, k % 3 - 1};
            int lo[3], hi[3], src[3];
            for (int a = 0; a < 3; a++) {
                if (d[a] < 0) { lo[a] = -1; hi[a] = 0; src[a] = D - 1; }      // halo cell -1 <- cell D-1
                else if (d[a] == 0) { lo[a] = 0; hi[a] = D; src[a] = 0; }
                else { lo[a] = D; hi[a] = D + 1; src[a] = 0; }                 // halo cell D <- cell 0
            }
            const uint32_t n = nb[c * 27 + k];
            const uint32_t *nd = (n == UINT32_MAX) ? nullptr : dist + (size_t)n * N;
            for (int x = lo[0]; x < hi[0]; x++)
                for (int y = lo[1]; y < hi[1]; y++)
                    for (int z = lo[2]; z < hi[2]; z++) {
                        uint32_t v = 0;
                        if (nd) {
                            const int sx = x - lo[0] + src[0], sy = y - lo[1] + src[1],
                                      sz = z - lo[2] + src[2];
                            v = nd[(sx << (2 * L)) | (sy << L) | sz];
                        }
                        buf[bidx(x, y, z)] = v;
                    }
        }
    };
    auto store = [&](size_t c, const uint32_t *buf) {
        uint32_t *dc = dist + c * N;
        for (int x = 0; x < D; x++)
            for (int y = 0; y < D; y++)
                for (int z = 0; z < D; z++) dc[(x << (2 * L)) | (y << L) | z] = buf[bidx(x, y, z)];
    };
    // Neighbour offsets in the halo buffer, vdb345.rs:327-343.
    int fo[13], bo[13], k = 0;
    for (int dy = -1; dy <= 1; dy++)
        for (int dz = -1; dz <= 1; dz++) {
            fo[k] = -P * P + dy * P + dz;
            bo[k] = P * P + dy * P + dz;
            k++;
        }
    for (int dz = -1; dz <= 1; dz++) {
        fo[k] = -P + dz;
        bo[k] = P + dz;
        k++;
    }
    fo[k] = -1;
    bo[k] = 1;

    auto sweep = [&](uint32_t *buf, bool backward) {
        const int *off = backward ? bo : fo;
        for (int s = 0; s < N; s++) {
            const int cell = backward ? N - 1 - s : s;
            const int x = cell >> (2 * L), y = (cell >> L) & (D - 1), z = cell & (D - 1);
            uint32_t *self = &buf[bidx(x, y, z)];
            if (*self == 0) continue;  // child node / active voxel: not a tile
            uint32_t m = self[off[0]];
            for (int j = 1; j < 13; j++) m = std::min(m, self[off[j]]);
            if (m + 1u < *self) *self = m + 1u;
        }
    };
    auto process = [&](size_t c, uint32_t *buf, bool backward) {
        fill(c, buf);
        sweep(buf, backward);
        store(c, buf);
    };

    if (nthreads <= 1 || nc < 256) {
        std::vector<uint32_t> buf((size_t)P * P * P);
        for (size_t c = 0; c < nc; c++) process(c, buf.data(), false);
        for (size_t c = nc; c-- > 0;) process(c, buf.data(), true);
        return;
    }
    std::unique_ptr<std::atomic<uint32_t>[]> indeg(new std::atomic<uint32_t>[nc]);
    for (int pass = 0; pass < 2; pass++) {
        const bool backward = pass == 1;
        // A neighbour comes before c in this pass's order when its index is smaller
        // (forward) or larger (backward).
        auto before = [&](uint32_t n, size_t c) { return backward ? n > c : n < c; };
        std::vector<uint32_t> ready;
        for (size_t c = 0; c < nc; c++) {
            uint32_t deg = 0;
            for (int j = 0; j < 27; j++) {
                const uint32_t n = nb[c * 27 + j];
                if (j != 13 && n != UINT32_MAX && before(n, c)) deg++;
            }
            indeg[c].store(deg, std::memory_order_relaxed);
            if (deg == 0) ready.push_back((uint32_t)c);
        }
        std::mutex mu;
        std::condition_variable cv;
        size_t done = 0;
        auto worker = [&] {
            std::vector<uint32_t> buf((size_t)P * P * P);
            std::unique_lock<std::mutex> lk(mu);
            for (;;) {
                cv.wait(lk, [&] { return !ready.empty() || done == nc; });
                if (ready.empty()) return;
                const uint32_t c = ready.back();
                ready.pop_back();
                lk.unlock();
                process(c, buf.data(), backward);
                uint32_t woke[26];
                int nw = 0;
                for (int j = 0; j < 27; j++) {
                    const uint32_t n = nb[(size_t)c * 27 + j];
                    if (j == 13 || n == UINT32_MAX || before(n, c)) continue;
                    if (indeg[n].fetch_sub(1, std::memory_order_acq_rel) == 1) woke[nw++] = n;
                }
                lk.lock();
                for (int w = 0; w < nw; w++) ready.push_back(woke[w]);
                done++;
                if (nw > 1 || done == nc) cv.notify_all();
                else if (nw == 1) cv.notify_one();
            }
        };
        std::vector<std::thread> th;
        for (int t = 1; t < nthreads; t++) th.emplace_back(worker);
        worker();
        for (auto &t : th) t.join();
    }
}

}  // namespace wx

using namespace wx;

void wx_topology::derive() {
    o4.clear();
    o3.clear();
    first4.assign(o5.size(), 0);
    first3.clear();
    for (size_t i = 0; i < o5.size(); i++) {
        first4[i] = (uint32_t)o4.size();
        for (uint32_t s5 = 0; s5 < kN5Slots; s5++) {
            if (!test_bit(&kid5[i * kN5Words], s5)) continue;
            uint32_t c5[3];
            offset_child(s5, kN5Log2, c5);
            I3 g4{o5[i][0] + (int32_t)c5[0] * 128, o5[i][1] + (int32_t)c5[1] * 128,
                  o5[i][2] + (int32_t)c5[2] * 128};
            o4.push_back(g4);
        }
    }
    // first3 / o3 need the N4 masks, which must hold one entry per N4.
    first3.assign(o4.size(), 0);
    for (size_t j = 0; j < o4.size(); j++) {
        first3[j] = (uint32_t)o3.size();
        if ((j + 1) * kN4Words > kid4.size()) break;
        for (uint32_t s4 = 0; s4 < kN4Slots; s4++) {
            if (!test_bit(&kid4[j * kN4Words], s4)) continue;
            uint32_t c4[3];
            offset_child(s4, kN4Log2, c4);
            o3.push_back(I3{o4[j][0] + (int32_t)c4[0] * 8, o4[j][1] + (int32_t)c4[1] * 8,
                            o4[j][2] + (int32_t)c4[2] * 8});
        }
    }
}

extern "C" {

const char *wx_thread_last_error(void) { return g_thread_error.c_str(); }

int wx_topology_from_masks(const uint32_t *kids5, const uint32_t *vals5, uint64_t n5,
                           const uint32_t *kids4, const uint32_t *vals4, uint64_t n4,
                           const uint32_t *vals3, uint64_t n3, const int32_t *origins,
                           uint32_t origin_stride, wx_topology **out) {
    return wx::guard("wx_topology_from_masks", [&]() -> int {
        if (!out || (n5 && (!kids5 || !vals5 || !origins)) || (n4 && (!kids4 || !vals4)) ||
            (n3 && !vals3) || origin_stride < 3) {
            set_thread_error("wx_topology_from_masks: null pointer or origin_stride < 3");
            return WX_ERR_INVALID;
        }
        auto *t = new (std::nothrow) wx_topology();
        if (!t) return WX_ERR_OOM;
        auto w2u = [](const uint32_t *w, size_t nwords64, std::vector<uint64_t> &dst) {
            dst.resize(nwords64);
            for (size_t i = 0; i < nwords64; i++) dst[i] = (uint64_t)w[2 * i] | ((uint64_t)w[2 * i + 1] << 32);
        };
        t->o5.resize(n5);
        for (uint64_t i = 0; i < n5; i++) {
            for (int a = 0; a < 3; a++) t->o5[i][a] = origins[i * origin_stride + a];
            for (int a = 0; a < 3; a++)
                if (node_origin(t->o5[i][a], kN5Total) != t->o5[i][a]) {
                    delete t;
                    set_thread_error("wx_topology_from_masks: origin not 4096-aligned");
                    return WX_ERR_INVALID;
                }
            if (i && !(t->o5[i - 1] < t->o5[i])) {
                delete t;
                set_thread_error("wx_topology_from_masks: origins not strictly ascending");
                return WX_ERR_INVALID;
            }
        }
        w2u(kids5, n5 * kN5Words, t->kid5);
        w2u(vals5, n5 * kN5Words, t->val5);
        w2u(kids4, n4 * kN4Words, t->kid4);
        w2u(vals4, n4 * kN4Words, t->val4);
        w2u(vals3, n3 * kN3Words, t->val3);
        t->derive();
        if (t->o4.size() != n4 || t->o3.size() != n3) {
            char msg[160];
            snprintf(msg, sizeof msg,
                     "wx_topology_from_masks: child masks name %zu N4 / %zu N3 nodes, view has %llu / %llu",
                     t->o4.size(), t->o3.size(), (unsigned long long)n4, (unsigned long long)n3);
            delete t;
            set_thread_error(msg);
            return WX_ERR_INVALID;
        }
        *out = t;
        return WX_OK;
    });
}

int wx_topology_from_leaves(const int32_t *origins, const uint64_t *masks, uint64_t n,
                            wx_topology **out) {
    return wx::guard("wx_topology_from_leaves", [&]() -> int {
        if (!out || (n && (!origins || !masks))) {
            set_thread_error("wx_topology_from_leaves: null pointer");
            return WX_ERR_INVALID;
        }
        struct Leaf {
            I3 o;
            uint64_t m[8];
        };
        std::vector<Leaf> leaves(n);
        for (uint64_t i = 0; i < n; i++) {
            for (int a = 0; a < 3; a++) {
                leaves[i].o[a] = origins[3 * i + a];
                if (node_origin(leaves[i].o[a], kN3Total) != leaves[i].o[a]) {
                    set_thread_error("wx_topology_from_leaves: leaf origin not 8-aligned");
                    return WX_ERR_INVALID;
                }
            }
            memcpy(leaves[i].m, masks + 8 * i, 64);
        }
        // DFS order: N5 key (lexicographic), then N5 slot offset, then N4 slot offset.
        auto key = [](const I3 &o) {
            struct K {
                I3 k5;
                uint32_t s5, s4;
            } k;
            for (int a = 0; a < 3; a++) k.k5[a] = node_origin(o[a], kN5Total);
            k.s5 = slot_offset(o[0], o[1], o[2], kN5Log2, kN5Total);
            k.s4 = slot_offset(o[0], o[1], o[2], kN4Log2, kN4Total);
            return k;
        };
        std::sort(leaves.begin(), leaves.end(), [&](const Leaf &a, const Leaf &b) {
            auto ka = key(a.o), kb = key(b.o);
            if (ka.k5 != kb.k5) return ka.k5 < kb.k5;
            if (ka.s5 != kb.s5) return ka.s5 < kb.s5;
            return ka.s4 < kb.s4;
        });
        auto *t = new (std::nothrow) wx_topology();
        if (!t) return WX_ERR_OOM;
        size_t i = 0;
        while (i < leaves.size()) {
            auto k = key(leaves[i].o);
            if (t->o5.empty() || t->o5.back() != k.k5) {
                t->o5.push_back(k.k5);
                t->kid5.resize(t->kid5.size() + kN5Words, 0);
                t->val5.resize(t->val5.size() + kN5Words, 0);
            }
            uint64_t *k5 = &t->kid5[(t->o5.size() - 1) * kN5Words];
            if (!test_bit(k5, k.s5)) {
                k5[k.s5 >> 6] |= 1ull << (k.s5 & 63);
                t->kid4.resize(t->kid4.size() + kN4Words, 0);
                t->val4.resize(t->val4.size() + kN4Words, 0);
            }
            uint64_t *k4 = &t->kid4[t->kid4.size() - kN4Words];
            uint64_t m[8] = {0};
            size_t j = i;
            while (j < leaves.size() && leaves[j].o == leaves[i].o) {  // merge duplicates
                for (int w = 0; w < 8; w++) m[w] |= leaves[j].m[w];
                j++;
            }
            k4[k.s4 >> 6] |= 1ull << (k.s4 & 63);
            t->val3.insert(t->val3.end(), m, m + 8);
            i = j;
        }
        t->derive();
        *out = t;
        return WX_OK;
    });
}

int wx_topology_from_voxels(const int32_t *ijk, uint64_t n, wx_topology **out) {
    return wx::guard("wx_topology_from_voxels", [&]() -> int {
        if (!out || (n && !ijk)) {
            set_thread_error("wx_topology_from_voxels: null pointer");
            return WX_ERR_INVALID;
        }
        std::vector<std::pair<I3, uint32_t>> v(n);
        for (uint64_t i = 0; i < n; i++) {
            I3 o{node_origin(ijk[3 * i], 3), node_origin(ijk[3 * i + 1], 3), node_origin(ijk[3 * i + 2], 3)};
            v[i] = {o, slot_offset(ijk[3 * i], ijk[3 * i + 1], ijk[3 * i + 2], kN3Log2, kN3Total)};
        }
        std::sort(v.begin(), v.end());
        std::vector<int32_t> org;
        std::vector<uint64_t> masks;
        for (size_t i = 0; i < v.size(); i++) {
            if (i == 0 || v[i].first != v[i - 1].first) {
                org.insert(org.end(), v[i].first.begin(), v[i].first.end());
                masks.resize(masks.size() + 8, 0);
            }
            masks[masks.size() - 8 + (v[i].second >> 6)] |= 1ull << (v[i].second & 63);
        }
        return wx_topology_from_leaves(org.data(), masks.data(), org.size() / 3, out);
    });
}

void wx_topology_free(wx_topology *topo) { delete topo; }

int wx_topology_counts(const wx_topology *t, uint64_t counts[3]) {
    if (!t || !counts) return WX_ERR_INVALID;
    counts[0] = t->n5();
    counts[1] = t->n4();
    counts[2] = t->n3();
    return WX_OK;
}

uint64_t wx_topology_active_voxels(const wx_topology *t) {
    if (!t) return 0;
    uint64_t s = 0;
    for (uint64_t w : t->val3) s += (uint64_t)__builtin_popcountll(w);
    return s;
}

int wx_topology_masks(const wx_topology *t, uint32_t *kids5, uint32_t *vals5, uint32_t *kids4,
                      uint32_t *vals4, uint32_t *vals3, int32_t *origins) {
    return wx::guard("wx_topology_masks", [&]() -> int {
        if (!t) return WX_ERR_INVALID;
        auto u2w = [](const std::vector<uint64_t> &src, uint32_t *dst) {  // arr32_from_arr64
            if (!dst) return;
            for (size_t i = 0; i < src.size(); i++) {
                dst[2 * i] = (uint32_t)src[i];
                dst[2 * i + 1] = (uint32_t)(src[i] >> 32);
            }
        };
        u2w(t->kid5, kids5);
        u2w(t->val5, vals5);
        u2w(t->kid4, kids4);
        u2w(t->val4, vals4);
        u2w(t->val3, vals3);
        if (origins)
            for (size_t i = 0; i < t->o5.size(); i++) {
                for (int a = 0; a < 3; a++) origins[4 * i + a] = t->o5[i][a];
                origins[4 * i + 3] = 0;
            }
        return WX_OK;
    });
}

int wx_topology_sdf(wx_topology *t, int nthreads) {
    if (!t) return WX_ERR_INVALID;
    if (t->has_sdf) return WX_OK;
    try {
        t->d5.resize(t->n5() * kN5Slots);
        t->d4.resize(t->n4() * kN4Slots);
        t->slot3.resize(t->n3() * kN3Slots);
    } catch (...) {
        set_thread_error("wx_topology_sdf: host allocation failed");
        return WX_ERR_OOM;
    }
    auto init = [](const std::vector<uint64_t> &solid, uint32_t slots, std::vector<uint32_t> &d) {
        for (size_t c = 0; c < d.size() / slots; c++)
            for (uint32_t s = 0; s < slots; s++)
                d[c * slots + s] = test_bit(&solid[c * (slots / 64)], s) ? 0u : kSdfInf;
    };
    // The three levels are independent sweeps; the small N5/N4 levels run on
    // one helper thread while the leaf level uses the remaining workers.
    if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
    std::thread upper([&] {
        init(t->kid5, kN5Slots, t->d5);
        chamfer_level<5>(t->o5, kN5Total, t->d5.data(), 1);
        init(t->kid4, kN4Slots, t->d4);
        chamfer_level<4>(t->o4, kN4Total, t->d4.data(), std::max(1, nthreads / 4));
    });
    init(t->val3, kN3Slots, t->slot3);
    chamfer_level<3>(t->o3, kN3Total, t->slot3.data(), std::max(1, nthreads - 1));
    upper.join();
    t->has_sdf = true;
    return WX_OK;
}

static uint64_t cube_side(uint64_t n) {  // closest_power_of_3 (vdb345.rs:684-690)
    uint64_t i = 0;
    while (i * i * i < n) i++;
    return i;
}

int wx_topology_atlas(const wx_topology *t, uint32_t side[3], uint32_t *a5, uint32_t *a4,
                      uint32_t *a3, uint32_t value_texel) {
    if (!t || !side) return WX_ERR_INVALID;
    const uint64_t d5 = cube_side(t->n5()), d4 = cube_side(t->n4()), d3 = cube_side(t->n3());
    side[0] = (uint32_t)(32 * d5);
    side[1] = (uint32_t)(16 * d4);
    side[2] = (uint32_t)(8 * d3);
    if (!a5 || !a4 || !a3) return WX_OK;
    if (!t->has_sdf) {
        set_thread_error("wx_topology_atlas: run wx_topology_sdf first");
        return WX_ERR_INVALID;
    }
    const uint64_t S5 = side[0], S4 = side[1], S3 = side[2];
    memset(a5, 0, S5 * S5 * S5 * 4);
    memset(a4, 0, S4 * S4 * S4 * 4);
    memset(a3, 0, S3 * S3 * S3 * 4);
    auto at = [](uint64_t S, uint64_t x, uint64_t y, uint64_t z) { return (z * S + y) * S + x; };
    uint64_t i4 = 0, i3 = 0;
    for (uint64_t i5 = 0; i5 < t->n5(); i5++) {
        const uint64_t O5[3] = {(i5 % d5) * 32, ((i5 / d5) % d5) * 32, (i5 / (d5 * d5)) * 32};
        for (uint32_t s5 = 0; s5 < kN5Slots; s5++) {
            uint32_t c[3];
            offset_child(s5, kN5Log2, c);
            const uint64_t P5 = at(S5, O5[0] + c[0], O5[1] + c[1], O5[2] + c[2]);
            if (!test_bit(&t->kid5[i5 * kN5Words], s5)) {
                a5[P5] = t->d5[i5 * kN5Slots + s5];
                continue;
            }
            const uint64_t O4[3] = {(i4 % d4) * 16, ((i4 / d4) % d4) * 16, (i4 / (d4 * d4)) * 16};
            for (uint32_t s4 = 0; s4 < kN4Slots; s4++) {
                offset_child(s4, kN4Log2, c);
                const uint64_t P4 = at(S4, O4[0] + c[0], O4[1] + c[1], O4[2] + c[2]);
                if (!test_bit(&t->kid4[i4 * kN4Words], s4)) {
                    a4[P4] = t->d4[i4 * kN4Slots + s4];
                    continue;
                }
                const uint64_t O3[3] = {(i3 % d3) * 8, ((i3 / d3) % d3) * 8, (i3 / (d3 * d3)) * 8};
                for (uint32_t s3 = 0; s3 < kN3Slots; s3++) {
                    offset_child(s3, kN3Log2, c);
                    a3[at(S3, O3[0] + c[0], O3[1] + c[1], O3[2] + c[2])] =
                        test_bit(&t->val3[i3 * kN3Words], s3) ? value_texel : t->slot3[i3 * kN3Slots + s3];
                }
                a4[P4] = (uint32_t)i3++;
            }
            a5[P5] = (uint32_t)i4++;
        }
    }
    return WX_OK;
}

}  // extern "C"
