// wx_common.h — host-side internals shared by the woxel_gb300 translation units.
#pragma once

#include <array>
#include <cstdint>
#include <new>
#include <string>
#include <vector>

#include "woxel_gb300.h"

namespace wx {

// Node geometry of VDB345 (src/vdb/vdb345.rs:8-12, data_structure.rs:17-36):
// N5 = 32^3 children of N4 (4096 voxels a side), N4 = 16^3 children of N3
// (128 voxels), N3 = 8^3 voxels.
constexpr int kN5Log2 = 5, kN4Log2 = 4, kN3Log2 = 3;
constexpr int kN5Total = 12, kN4Total = 7, kN3Total = 3;
constexpr uint32_t kN5Slots = 32768, kN4Slots = 4096, kN3Slots = 512;
constexpr uint32_t kN5Words = 512, kN4Words = 64, kN3Words = 8;  // u64 mask words

// Device slot words (one u32 per child slot at every level):
//   N5/N4: bit 31 set -> child pool index in bits 0..30; otherwise the skip
//          distance (0 means the slot is an active tile: a hit).
//   N3:    skip distance of an inactive voxel; 0 for an active voxel (a hit).
constexpr uint32_t kChildFlag = 0x80000000u;
constexpr uint32_t kSdfInf = 0xFFFFFFFEu;  // u32::MAX - 1, the reference's initial tile value

using I3 = std::array<int32_t, 3>;

inline int32_t node_origin(int32_t c, int total_log2) {
    return (int32_t)((uint32_t)c & ~((1u << total_log2) - 1u));
}
// global_to_offset (data_structure.rs:58-70)
inline uint32_t slot_offset(int32_t x, int32_t y, int32_t z, int log2d, int total_log2) {
    const int ct = total_log2 - log2d;
    const uint32_t m = (1u << total_log2) - 1u;
    return ((((uint32_t)x & m) >> ct) << (2 * log2d)) | ((((uint32_t)y & m) >> ct) << log2d) |
           (((uint32_t)z & m) >> ct);
}
// offset_to_child (data_structure.rs:80-87)
inline void offset_child(uint32_t off, int log2d, uint32_t c[3]) {
    const uint32_t dm = (1u << log2d) - 1u;
    c[0] = off >> (2 * log2d);
    c[1] = (off >> log2d) & dm;
    c[2] = off & dm;
}
inline bool test_bit(const uint64_t *w, uint32_t i) { return (w[i >> 6] >> (i & 63)) & 1u; }

void set_thread_error(const std::string &msg);

// Runs an entry point's body so that no C++ exception crosses the C ABI: a failed
// host allocation is WX_ERR_OOM, anything else WX_ERR_INVALID (the message is kept
// when it can still be stored).
template <class F>
int guard(const char *who, F &&f) noexcept {
    try {
        return f();
    } catch (const std::bad_alloc &) {
        try {
            set_thread_error(std::string(who) + ": host allocation failed");
        } catch (...) {
        }
        return WX_ERR_OOM;
    } catch (...) {
        try {
            set_thread_error(std::string(who) + ": unexpected error");
        } catch (...) {
        }
        return WX_ERR_INVALID;
    }
}

}  // namespace wx

// The node structure of one grid in DFS order (sorted N5 keys, then child
// offsets ascending), i.e. the order masks()/origins()/atlas() use.
struct wx_topology {
    std::vector<wx::I3> o5;                 // N5 origins (root keys), sorted
    std::vector<uint64_t> kid5, val5;       // n5 * 512
    std::vector<uint64_t> kid4, val4;       // n4 * 64
    std::vector<uint64_t> val3;             // n3 * 8
    std::vector<wx::I3> o4, o3;             // derived origins, DFS order
    std::vector<uint32_t> first4;           // per N5: index of its first N4 child
    std::vector<uint32_t> first3;           // per N4: index of its first N3 child
    bool has_sdf = false;
    std::vector<uint32_t> d5, d4;           // per-slot distance (0 on child slots)
    std::vector<uint32_t> slot3;            // per-voxel distance (0 on active voxels) == device N3 pool

    uint64_t n5() const { return o5.size(); }
    uint64_t n4() const { return o4.size(); }
    uint64_t n3() const { return o3.size(); }
    void derive();  // fills o4, o3, first4, first3 from masks; validates counts
};
