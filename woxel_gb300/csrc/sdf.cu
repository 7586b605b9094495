// sdf.cu — compute_sdf and the slot packing on the GPU (wx_grid_build_gpu).
//
// Same result, word for word, as the host sweep in topology.cpp, which
// restates VDB345::compute_sdf (src/vdb/vdb345.rs:290-670) as three
// independent per-level chamfer sweeps. A sweep visits the containers (nodes of
// one level) in DFS order, forward and then backward; each tile slot becomes
// min(own, neighbour + 1) over its 13 "earlier" (forward) or "later"
// (backward) neighbours in slot order, updated in place; child slots, active
// leaf voxels and missing neighbours read as 0.
//
// Parallel form with identical values:
//   * inside a container, slot (x, y, z) only reads slots whose index
//     (x << 2L | y << L | z) is smaller (forward) — all of which lie on lower
//     planes 4x + 2y + z — so one CTA sweeps plane by plane, the cells of a
//     plane in parallel;
//   * across containers, a container reads its neighbours' final values when
//     they come earlier in DFS order and their untouched values when they come
//     later; so a container becomes ready when its earlier neighbours are done.
//     A persistent kernel hands out tickets in order and a container is
//     appended to the ready queue by the last of its earlier neighbours to
//     finish. Every waiting CTA holds a ticket whose queue slot is filled by
//     CTAs that are already running, so the wait always ends; it is bounded
//     nonetheless and sets an error flag when the bound is hit.
// The containers' neighbour tables come from the tree itself: a neighbour's
// origin is looked up through the root-key table and the child-index tables.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "wx_kernels.h"

namespace {

constexpr uint32_t kNone = 0xFFFFFFFFu;   // no node / empty queue slot
constexpr uint32_t kInf = 0xFFFFFFFEu;    // initial tile distance (u32::MAX - 1)
constexpr uint32_t kChild = 0x80000000u;

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// ---------------------------------------------------------------------------
// Structure: child-index tables, derived origins, initial distances.
// ---------------------------------------------------------------------------

// cidx[node * S + s] = DFS index of the child in slot s (first[node] + rank of
// the child bit among the node's child bits), or kNone. pre[node * W + w] is
// the number of child bits in words 0..w-1 of the node (host prefix).
__global__ void k_child_table(const uint64_t *__restrict__ kid, const uint32_t *__restrict__ pre,
                              const uint32_t *__restrict__ first, uint64_t nslots, int slots_log2,
                              uint32_t *__restrict__ cidx) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nslots) return;
    const uint64_t node = i >> slots_log2;
    const uint64_t w = i >> 6;
    const uint64_t word = kid[w];
    const uint32_t bit = (uint32_t)(i & 63);
    if (!((word >> bit) & 1u)) {
        cidx[i] = kNone;
        return;
    }
    const uint32_t below = __popcll(word & ((1ull << bit) - 1ull));
    cidx[i] = first[node] + pre[w] + below;
}

// Origins of the children: org_child[cidx] = org_parent + coords(s) * child_span.
__global__ void k_child_origins(const uint32_t *__restrict__ cidx, const int4 *__restrict__ org, uint64_t nslots,
                                int log2d, int child_span_log2, int4 *__restrict__ org_child) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nslots) return;
    const uint32_t c = cidx[i];
    if (c == kNone) return;
    const uint64_t node = i >> (3 * log2d);
    const uint32_t s = (uint32_t)(i & ((1u << (3 * log2d)) - 1u)), dm = (1u << log2d) - 1u;
    const int4 o = org[node];
    org_child[c] = make_int4(o.x + (int)((s >> (2 * log2d)) << child_span_log2),
                             o.y + (int)(((s >> log2d) & dm) << child_span_log2),
                             o.z + (int)((s & dm) << child_span_log2), 0);
}

// d[i] = 0 where the solid mask bit is set (child slots for N5/N4, active voxels
// for N3), else the initial tile distance.
__global__ void k_sdf_init(const uint64_t *__restrict__ solid, uint64_t ncells, uint32_t *__restrict__ d) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ncells) return;
    d[i] = ((solid[i >> 6] >> (i & 63)) & 1u) ? 0u : kInf;
}

// ---------------------------------------------------------------------------
// Neighbour tables.
// ---------------------------------------------------------------------------

// N5 index of the node whose origin is exactly (x, y, z), or kNone. Origins are
// multiples of 4096 (checked on the host), so the root table applies.
__device__ __forceinline__ uint32_t find_n5(const wxk::SdfTree &t, int64_t x, int64_t y, int64_t z) {
    if (x < INT32_MIN || x > INT32_MAX || y < INT32_MIN || y > INT32_MAX || z < INT32_MIN || z > INT32_MAX)
        return kNone;
    const int xi = (int)x, yi = (int)y, zi = (int)z;
    if ((xi & 4095) || (yi & 4095) || (zi & 4095)) return kNone;
    const int4 h0 = t.root[0], h1 = t.root[1];
    if (h1.w) {
        const uint32_t ux = (uint32_t)((xi >> 12) - h0.x), uy = (uint32_t)((yi >> 12) - h0.y),
                       uz = (uint32_t)((zi >> 12) - h0.z);
        if (ux >= (uint32_t)h0.w || uy >= (uint32_t)h1.x || uz >= (uint32_t)h1.y) return kNone;
        const uint32_t *tab = reinterpret_cast<const uint32_t *>(t.root + 2 + t.n5);
        const uint32_t e = tab[(uz * (uint32_t)h1.x + uy) * (uint32_t)h0.w + ux];
        return e ? e - 1u : kNone;
    }
    for (uint32_t k = 0; k < t.n5; k++) {
        const int4 o = t.root[2 + k];
        if (o.x == xi && o.y == yi && o.z == zi) return k;
    }
    return kNone;
}

// nb[c * 27 + k] = index of the container at origin + (dx, dy, dz) * span,
// k = (dx+1)*9 + (dy+1)*3 + (dz+1); k = 13 is c itself.
template <int L>
__global__ void k_sdf_neighbours(const int4 *__restrict__ org, uint32_t nc, wxk::SdfTree t, uint32_t *__restrict__ nb) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint64_t)nc * 27) return;
    const uint32_t c = (uint32_t)(i / 27), k = (uint32_t)(i % 27);
    if (k == 13) {
        nb[i] = c;
        return;
    }
    constexpr int span_log2 = L == 5 ? 12 : L == 4 ? 7 : 3;
    const int4 o = org[c];
    const int64_t x = (int64_t)o.x + ((int)(k / 9) - 1) * (int64_t(1) << span_log2);
    const int64_t y = (int64_t)o.y + ((int)((k / 3) % 3) - 1) * (int64_t(1) << span_log2);
    const int64_t z = (int64_t)o.z + ((int)(k % 3) - 1) * (int64_t(1) << span_log2);
    uint32_t n = find_n5(t, x & ~int64_t(4095), y & ~int64_t(4095), z & ~int64_t(4095));
    if (L <= 4 && n != kNone) {
        const uint32_t s5 = ((uint32_t)((x >> 7) & 31) << 10) | ((uint32_t)((y >> 7) & 31) << 5) | (uint32_t)((z >> 7) & 31);
        n = t.c5[((size_t)n << 15) | s5];
    }
    if (L == 3 && n != kNone) {
        const uint32_t s4 = ((uint32_t)((x >> 3) & 15) << 8) | ((uint32_t)((y >> 3) & 15) << 4) | (uint32_t)((z >> 3) & 15);
        n = t.c4[((size_t)n << 12) | s4];
    }
    nb[i] = n;
}

// In-degree of each container for one pass (its earlier neighbours); the ones
// with none start the ready queue.
__global__ void k_sdf_indeg(const uint32_t *__restrict__ nb, uint32_t nc, int backward, uint32_t *__restrict__ indeg,
                            uint32_t *__restrict__ queue, uint32_t *__restrict__ ctr) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) return;
    uint32_t deg = 0;
    for (int k = 0; k < 27; k++) {
        const uint32_t n = nb[(size_t)c * 27 + k];
        if (k != 13 && n != kNone && (backward ? n > c : n < c)) deg++;
    }
    indeg[c] = deg;
    if (deg == 0) queue[atomicAdd(&ctr[1], 1u)] = c;  // at most nc pushes
}

// ---------------------------------------------------------------------------
// The sweep: one CTA per container at a time, D*D threads (one per (x, y)
// column), the container plus a one-cell halo in shared memory.
// ctr[0] next ticket, ctr[1] queue length, ctr[2] error flag.
// ---------------------------------------------------------------------------
template <int L>
__global__ void __launch_bounds__((1 << L) * (1 << L)) k_sdf_sweep(uint32_t *d, const uint32_t *__restrict__ nb,
                                                                   uint32_t nc, int backward, uint32_t *indeg,
                                                                   uint32_t *queue, uint32_t *ctr,
                                                                   uint32_t spin_limit) {
    constexpr int D = 1 << L, P = D + 2, N = D * D * D, T = D * D, TMAX = 7 * (D - 1);
    extern __shared__ uint32_t buf[];  // P^3
    __shared__ uint32_t s_node;
    const int tid = threadIdx.x, cx = tid / D, cy = tid % D;
    // Offsets of the 13 earlier (forward) neighbours in the halo buffer,
    // vdb345.rs:327-343; the backward ones are their negatives.
    int off[13];
    {
        int k = 0;
        for (int dy = -1; dy <= 1; dy++)
            for (int dz = -1; dz <= 1; dz++) off[k++] = -P * P + dy * P + dz;
        for (int dz = -1; dz <= 1; dz++) off[k++] = -P + dz;
        off[k] = -1;
        if (backward)
            for (int j = 0; j < 13; j++) off[j] = -off[j];
    }
    for (;;) {
        if (tid == 0) {
            uint32_t node = kNone;
            const uint32_t ticket = atomicAdd(&ctr[0], 1u);
            if (ticket < nc) {
                for (uint32_t spin = 0;; spin++) {
                    node = ld_acquire(&queue[ticket]);
                    if (node != kNone) break;
                    if (ld_acquire(&ctr[2]) != 0u) break;
                    if (spin >= spin_limit) {  // give up: set the error flag, every CTA then returns
                        atomicExch(&ctr[2], 1u);
                        break;
                    }
                    __nanosleep(256);
                }
            }
            s_node = node;
            __threadfence();
        }
        __syncthreads();
        const uint32_t node = s_node;
        if (node == kNone) return;
        // Halo fill: buffer cell (bx, by, bz) holds container cell (bx-1, by-1, bz-1),
        // taken from the neighbour that contains it; a missing neighbour reads 0.
        for (int i = tid; i < P * P * P; i += T) {
            const int x = i / (P * P) - 1, y = (i / P) % P - 1, z = i % P - 1;
            const int dx = x < 0 ? -1 : (x >= D ? 1 : 0), dy = y < 0 ? -1 : (y >= D ? 1 : 0),
                      dz = z < 0 ? -1 : (z >= D ? 1 : 0);
            const int sx = x - dx * D, sy = y - dy * D, sz = z - dz * D;
            const uint32_t n = nb[(size_t)node * 27 + (dx + 1) * 9 + (dy + 1) * 3 + (dz + 1)];
            buf[i] = n == kNone ? 0u : __ldcg(d + (size_t)n * N + ((sx << (2 * L)) | (sy << L) | sz));
        }
        __syncthreads();
        for (int s = 0; s <= TMAX; s++) {
            const int t = backward ? TMAX - s : s;
            const int z = t - 4 * cx - 2 * cy;
            if (z >= 0 && z < D) {
                const int b = ((cx + 1) * P + (cy + 1)) * P + (z + 1);
                const uint32_t self = buf[b];
                if (self != 0u) {
                    uint32_t m = buf[b + off[0]];
#pragma unroll
                    for (int j = 1; j < 13; j++) m = min(m, buf[b + off[j]]);
                    if (m + 1u < self) buf[b] = m + 1u;
                }
            }
            __syncthreads();
        }
        for (int c = tid; c < N; c += T) {
            const int x = c >> (2 * L), y = (c >> L) & (D - 1), z = c & (D - 1);
            __stcg(d + (size_t)node * N + c, buf[((x + 1) * P + (y + 1)) * P + (z + 1)]);
        }
        __threadfence();
        __syncthreads();
        if (tid == 0) {
            for (int k = 0; k < 27; k++) {
                const uint32_t n = nb[(size_t)node * 27 + k];
                if (k == 13 || n == kNone || (backward ? n > node : n < node)) continue;
                if (atomicSub(&indeg[n], 1u) == 1u) {
                    const uint32_t pos = atomicAdd(&ctr[1], 1u);
                    if (pos < nc) atomicExch(&queue[pos], n);
                    else atomicExch(&ctr[2], 1u);  // more pushes than containers: cannot happen
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Packing.
// ---------------------------------------------------------------------------

// Slot words of N5/N4: active tile -> 0, child -> flag | index, else the
// distance (must be < 2^31; err[0] is set otherwise).
__global__ void k_pack_internal(const uint64_t *__restrict__ kid, const uint64_t *__restrict__ val,
                                const uint32_t *__restrict__ cidx, const uint32_t *__restrict__ d, uint64_t nslots,
                                uint32_t *__restrict__ slot, uint32_t *__restrict__ err) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nslots) return;
    const bool k = (kid[i >> 6] >> (i & 63)) & 1u, v = (val[i >> 6] >> (i & 63)) & 1u;
    uint32_t w;
    if (v) w = 0u;
    else if (k) w = kChild | cidx[i];
    else {
        w = d[i];
        if (w >= kChild) atomicExch(err, 1u);
    }
    slot[i] = w;
}

// Leaf bytes: the distance when below 255, else 255 and an overflow entry
// (cell index, distance); entries beyond cap are only counted, and leaf ==
// nullptr only counts.
__global__ void k_pack_leaves(const uint32_t *__restrict__ d, uint64_t ncells, uint8_t *__restrict__ leaf,
                              uint2 *__restrict__ ovf, uint32_t cap, uint32_t *__restrict__ n_ovf) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ncells) return;
    const uint32_t v = d[i];
    if (leaf) leaf[i] = (uint8_t)(v < 255u ? v : 255u);
    if (v >= 255u) {
        const uint32_t p = atomicAdd(n_ovf, 1u);
        if (p < cap) ovf[p] = make_uint2((uint32_t)i, v);
    }
}

template <class K>
int resident_blocks(K kernel, int threads, size_t smem) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, smem) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return n > 0 ? n : 1;
}

unsigned grid_for(uint64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

}  // namespace

namespace wxk {

cudaError_t sdf_child_table(const uint64_t *kid, const uint32_t *pre, const uint32_t *first, uint64_t nodes,
                            int slots_log2, uint32_t *cidx, cudaStream_t st) {
    const uint64_t n = nodes << slots_log2;
    if (n) k_child_table<<<grid_for(n, 256), 256, 0, st>>>(kid, pre, first, n, slots_log2, cidx);
    return cudaGetLastError();
}

cudaError_t sdf_child_origins(const uint32_t *cidx, const int4 *org, uint64_t nodes, int log2d, int child_span_log2,
                              int4 *org_child, cudaStream_t st) {
    const uint64_t n = nodes << (3 * log2d);
    if (n) k_child_origins<<<grid_for(n, 256), 256, 0, st>>>(cidx, org, n, log2d, child_span_log2, org_child);
    return cudaGetLastError();
}

cudaError_t sdf_init(const uint64_t *solid, uint64_t ncells, uint32_t *d, cudaStream_t st) {
    if (ncells) k_sdf_init<<<grid_for(ncells, 256), 256, 0, st>>>(solid, ncells, d);
    return cudaGetLastError();
}

cudaError_t sdf_neighbours(int level, const int4 *org, uint32_t nc, const SdfTree &t, uint32_t *nb, cudaStream_t st) {
    const uint64_t n = (uint64_t)nc * 27;
    if (!n) return cudaSuccess;
    if (level == 5) k_sdf_neighbours<5><<<grid_for(n, 256), 256, 0, st>>>(org, nc, t, nb);
    else if (level == 4) k_sdf_neighbours<4><<<grid_for(n, 256), 256, 0, st>>>(org, nc, t, nb);
    else k_sdf_neighbours<3><<<grid_for(n, 256), 256, 0, st>>>(org, nc, t, nb);
    return cudaGetLastError();
}

template <int L>
static cudaError_t sweep_level(uint32_t *d, const uint32_t *nb, uint32_t nc, uint32_t *indeg, uint32_t *queue,
                               uint32_t *ctr, int num_sms, uint32_t spin_limit, cudaStream_t st) {
    constexpr int D = 1 << L, P = D + 2, T = D * D;
    const size_t smem = (size_t)P * P * P * 4;
    cudaError_t e = cudaFuncSetAttribute(k_sdf_sweep<L>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int per_sm = resident_blocks(k_sdf_sweep<L>, T, smem);
    const uint64_t blocks = std::min<uint64_t>((uint64_t)per_sm * num_sms, nc);
    for (int pass = 0; pass < 2; pass++) {
        if ((e = cudaMemsetAsync(queue, 0xFF, (size_t)nc * 4, st)) != cudaSuccess) return e;
        if ((e = cudaMemsetAsync(ctr, 0, 2 * sizeof(uint32_t), st)) != cudaSuccess) return e;  // keeps ctr[2]
        k_sdf_indeg<<<grid_for(nc, 256), 256, 0, st>>>(nb, nc, pass, indeg, queue, ctr);
        k_sdf_sweep<L><<<(unsigned)blocks, T, smem, st>>>(d, nb, nc, pass, indeg, queue, ctr, spin_limit);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t sdf_sweep(int level, uint32_t *d, const uint32_t *nb, uint32_t nc, uint32_t *indeg, uint32_t *queue,
                      uint32_t *ctr, int num_sms, uint32_t spin_limit, cudaStream_t st) {
    if (!nc) return cudaSuccess;
    if (level == 5) return sweep_level<5>(d, nb, nc, indeg, queue, ctr, num_sms, spin_limit, st);
    if (level == 4) return sweep_level<4>(d, nb, nc, indeg, queue, ctr, num_sms, spin_limit, st);
    return sweep_level<3>(d, nb, nc, indeg, queue, ctr, num_sms, spin_limit, st);
}

cudaError_t sdf_pack_internal(const uint64_t *kid, const uint64_t *val, const uint32_t *cidx, const uint32_t *d,
                              uint64_t nslots, uint32_t *slot, uint32_t *err, cudaStream_t st) {
    if (nslots) k_pack_internal<<<grid_for(nslots, 256), 256, 0, st>>>(kid, val, cidx, d, nslots, slot, err);
    return cudaGetLastError();
}

cudaError_t sdf_pack_leaves(const uint32_t *d, uint64_t ncells, uint8_t *leaf, uint2 *ovf, uint32_t cap,
                            uint32_t *n_ovf, cudaStream_t st) {
    if (ncells) k_pack_leaves<<<grid_for(ncells, 256), 256, 0, st>>>(d, ncells, leaf, ovf, cap, n_ovf);
    return cudaGetLastError();
}

}  // namespace wxk
