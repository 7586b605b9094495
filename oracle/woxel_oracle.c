/*
 * woxel_oracle.c — CPU oracle for woxel's primary-ray pass (see woxel_oracle.h).
 *
 * TEST INFRASTRUCTURE ONLY: what the CUDA path is checked against, never part of it.
 * Build with -O2 -ffp-contract=off (no FMA contraction, IEEE '/' and sqrt).
 *
 * Every function cites the reference file:line it restates. The structure of
 * the loops follows the reference literally (including get_voxel lookups in
 * compute_sdf and the textureLoad-on-atlas lookups of the shader) so that the
 * product's re-designed data layout and SDF sweep are checked against an
 * independent statement of the same algorithm.
 */
#include "woxel_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* Pinned scalar semantics (documented in woxel_oracle.h).                   */
/* ------------------------------------------------------------------------ */
static inline float pmin(float a, float b) {
    if (a != a) return b;
    if (b != b) return a;
    return (b < a) ? b : a;
}
static inline float pmax(float a, float b) {
    if (a != a) return b;
    if (b != b) return a;
    return (b > a) ? b : a;
}
static inline int32_t f2i_sat(float x) {
    if (x != x) return 0;
    if (x >= 2147483648.0f) return INT32_MAX;
    if (x <= -2147483648.0f) return INT32_MIN;
    return (int32_t)x;
}
static inline uint8_t unorm8(float x) {
    if (!(x > 0.0f)) return 0;
    if (x >= 1.0f) return 255;
    float y = x * 255.0f;
    y = y + 0.5f;
    return (uint8_t)floorf(y);
}

typedef struct { float x, y, z; } v3;
static inline v3 V3(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline v3 vadd(v3 a, v3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vmul(v3 a, v3 b) { return V3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline v3 vscale(float s, v3 a) { return V3(s * a.x, s * a.y, s * a.z); }
static inline v3 vscale_r(v3 a, float s) { return V3(a.x * s, a.y * s, a.z * s); }
static inline v3 vneg(v3 a) { return V3(-a.x, -a.y, -a.z); }
static inline float vdot(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline v3 vnormalize(v3 a) {
    float l = sqrtf(vdot(a, a));
    return V3(a.x / l, a.y / l, a.z / l);
}
static inline v3 vsplat(float s) { return V3(s, s, s); }
static inline v3 vmix(v3 a, v3 b, float t) {
    float omt = 1.0f - t;
    return V3(a.x * omt + b.x * t, a.y * omt + b.y * t, a.z * omt + b.z * t);
}

/* ------------------------------------------------------------------------ */
/* Coordinate maths — data_structure.rs:43-91                                */
/* ------------------------------------------------------------------------ */
static inline int32_t g2n(int32_t c, int t) {  /* (c >> t) << t, arithmetic */
    return (int32_t)((uint32_t)c & ~((1u << t) - 1u));
}
void orc_global_to_node(const int32_t g[3], int total_log2, int32_t out[3]) {
    for (int i = 0; i < 3; i++) out[i] = g2n(g[i], total_log2);
}
uint64_t orc_global_to_offset(const int32_t g[3], int log2d, int total_log2) {
    int ct = total_log2 - log2d;
    uint32_t m = (1u << total_log2) - 1u;
    uint32_t x = ((uint32_t)g[0] & m) >> ct, y = ((uint32_t)g[1] & m) >> ct,
             z = ((uint32_t)g[2] & m) >> ct;
    return ((uint64_t)x << (2 * log2d)) | ((uint64_t)y << log2d) | z;
}
void orc_offset_to_child(uint64_t offset, int log2d, uint32_t out[3]) {
    uint32_t o = (uint32_t)offset, dm = (1u << log2d) - 1u;
    out[0] = o >> (2 * log2d);
    out[1] = (o >> log2d) & dm;
    out[2] = o & dm;
}
uint64_t orc_child_to_offset(const uint32_t c[3], int log2d) {
    return ((uint64_t)c[0] << (2 * log2d)) | ((uint64_t)c[1] << log2d) | c[2];
}

/* ------------------------------------------------------------------------ */
/* VDB345 tree — data_structure.rs:95-247, vdb345.rs:8-12                    */
/* ------------------------------------------------------------------------ */
typedef struct {
    uint64_t val[8];
    uint8_t is_value[512];
    uint32_t value[512];
    uint64_t tile[512]; /* LeafData::Tile(usize) */
} ON3;
typedef struct {
    uint64_t kid[64], val[64];
    int32_t child[4096]; /* index into tree->n3, -1 = InternalData::Tile */
    uint32_t tile[4096];
} ON4;
typedef struct {
    uint64_t kid[512], val[512];
    int32_t child[32768]; /* index into tree->n4, -1 = Tile */
    uint32_t tile[32768];
} ON5;
typedef struct {
    int32_t key[3];
    int32_t n5;
} RootEntry;

struct orc_tree {
    RootEntry *roots; /* kept sorted by key: the reference sorts the HashMap keys */
    size_t nroots, caproots;
    ON5 **n5; size_t n5c, n5cap;
    ON4 **n4; size_t n4c, n4cap;
    ON3 **n3; size_t n3c, n3cap;
};

static int keycmp(const int32_t a[3], const int32_t b[3]) {
    for (int i = 0; i < 3; i++) {
        if (a[i] < b[i]) return -1;
        if (a[i] > b[i]) return 1;
    }
    return 0;
}
static long root_find(const orc_tree *t, const int32_t key[3], size_t *ins) {
    size_t lo = 0, hi = t->nroots;
    while (lo < hi) {
        size_t mid = (lo + hi) / 2;
        int c = keycmp(t->roots[mid].key, key);
        if (c == 0) return (long)mid;
        if (c < 0) lo = mid + 1; else hi = mid;
    }
    if (ins) *ins = lo;
    return -1;
}
#define GROW(arr, cnt, cap)                                                   \
    do {                                                                      \
        if ((cnt) == (cap)) {                                                 \
            (cap) = (cap) ? 2 * (cap) : 16;                                   \
            (arr) = realloc((arr), (cap) * sizeof(*(arr)));                   \
        }                                                                     \
    } while (0)

static int32_t new_n5(orc_tree *t) {
    GROW(t->n5, t->n5c, t->n5cap);
    ON5 *n = calloc(1, sizeof(ON5));
    for (int i = 0; i < 32768; i++) n->child[i] = -1;
    t->n5[t->n5c] = n;
    return (int32_t)t->n5c++;
}
static int32_t new_n4(orc_tree *t) {
    GROW(t->n4, t->n4c, t->n4cap);
    ON4 *n = calloc(1, sizeof(ON4));
    for (int i = 0; i < 4096; i++) n->child[i] = -1;
    t->n4[t->n4c] = n;
    return (int32_t)t->n4c++;
}
static int32_t new_n3(orc_tree *t) {
    GROW(t->n3, t->n3c, t->n3cap);
    ON3 *n = calloc(1, sizeof(ON3));
    t->n3[t->n3c] = n;
    return (int32_t)t->n3c++;
}
static int32_t root_insert(orc_tree *t, const int32_t key[3]) {
    size_t ins = 0;
    long f = root_find(t, key, &ins);
    if (f >= 0) return t->roots[f].n5;
    GROW(t->roots, t->nroots, t->caproots);
    memmove(&t->roots[ins + 1], &t->roots[ins], (t->nroots - ins) * sizeof(RootEntry));
    memcpy(t->roots[ins].key, key, sizeof(int32_t) * 3);
    t->roots[ins].n5 = new_n5(t);
    t->nroots++;
    return t->roots[ins].n5;
}

orc_tree *orc_tree_new(void) { return calloc(1, sizeof(orc_tree)); }
void orc_tree_free(orc_tree *t) {
    if (!t) return;
    for (size_t i = 0; i < t->n5c; i++) free(t->n5[i]);
    for (size_t i = 0; i < t->n4c; i++) free(t->n4[i]);
    for (size_t i = 0; i < t->n3c; i++) free(t->n3[i]);
    free(t->n5); free(t->n4); free(t->n3); free(t->roots);
    free(t);
}

/* set_voxel — vdb345.rs:26-66 */
void orc_set_voxel(orc_tree *t, const int32_t p[3], uint32_t value) {
    int32_t key[3];
    orc_global_to_node(p, 12, key);
    uint64_t b4 = orc_global_to_offset(p, 5, 12);
    uint64_t b3 = orc_global_to_offset(p, 4, 7);
    uint64_t b0 = orc_global_to_offset(p, 3, 3);
    int32_t i5 = root_insert(t, key);
    ON5 *n5 = t->n5[i5];
    if (n5->child[b4] < 0) {
        int32_t c = new_n4(t);
        n5 = t->n5[i5];
        n5->child[b4] = c;
    }
    n5->kid[b4 >> 6] |= 1ull << (b4 & 63);
    ON4 *n4 = t->n4[n5->child[b4]];
    if (n4->child[b3] < 0) {
        int32_t c = new_n3(t);
        n4->child[b3] = c;
    }
    n4->kid[b3 >> 6] |= 1ull << (b3 & 63);
    ON3 *n3 = t->n3[n4->child[b3]];
    n3->val[b0 >> 6] |= 1ull << (b0 & 63);
    n3->is_value[b0] = 1;
    n3->value[b0] = value;
}

/* get_voxel — vdb345.rs:69-106. Kinds: 0 Offs, 1 Leaf, 2 Innr, 3 Root, 4 Bkgr. */
int orc_get_voxel(const orc_tree *t, const int32_t p[3], uint64_t *value, int *level) {
    int32_t key[3];
    orc_global_to_node(p, 12, key);
    long r = root_find(t, key, NULL);
    *level = 0;
    *value = 0;
    if (r < 0) return 4;
    const ON5 *n5 = t->n5[t->roots[r].n5];
    uint64_t b4 = orc_global_to_offset(p, 5, 12);
    if (n5->child[b4] < 0) { *value = n5->tile[b4]; *level = 5; return 2; }
    const ON4 *n4 = t->n4[n5->child[b4]];
    uint64_t b3 = orc_global_to_offset(p, 4, 7);
    if (n4->child[b3] < 0) { *value = n4->tile[b3]; *level = 4; return 2; }
    const ON3 *n3 = t->n3[n4->child[b3]];
    uint64_t b0 = orc_global_to_offset(p, 3, 3);
    if (n3->is_value[b0]) { *value = n3->value[b0]; return 1; }
    *value = n3->tile[b0];
    return 0;
}

static void words_to_u64(const uint32_t *w, uint64_t *out, int n64) {
    for (int i = 0; i < n64; i++) out[i] = (uint64_t)w[2 * i] | ((uint64_t)w[2 * i + 1] << 32);
}
static void u64_to_words(const uint64_t *in, uint32_t *w, int n64) { /* arr32_from_arr64 vdb345.rs:673-682 */
    for (int i = 0; i < n64; i++) {
        w[2 * i] = (uint32_t)in[i];
        w[2 * i + 1] = (uint32_t)(in[i] >> 32);
    }
}

/* Rebuild the tree that masks()/origins() (vdb345.rs:108-161) were taken from.
 * DFS order: N5 in sorted-key order, N4 in visit order, N3 in visit order. */
orc_tree *orc_tree_from_masks(const uint32_t *kids5, const uint32_t *vals5, uint64_t n5c,
                              const uint32_t *kids4, const uint32_t *vals4, uint64_t n4c,
                              const uint32_t *vals3, uint64_t n3c, const int32_t *origins) {
    orc_tree *t = orc_tree_new();
    uint64_t c4 = 0, c3 = 0;
    for (uint64_t i = 0; i < n5c; i++) {
        int32_t key[3] = {origins[4 * i], origins[4 * i + 1], origins[4 * i + 2]};
        if (root_find(t, key, NULL) >= 0) goto fail;
        int32_t i5 = root_insert(t, key);
        ON5 *n5 = t->n5[i5];
        words_to_u64(kids5 + 1024 * i, n5->kid, 512);
        words_to_u64(vals5 + 1024 * i, n5->val, 512);
        for (int o5 = 0; o5 < 32768; o5++) {
            if (!((n5->kid[o5 >> 6] >> (o5 & 63)) & 1)) continue;
            if (c4 >= n4c) goto fail;
            int32_t i4 = new_n4(t);
            n5 = t->n5[i5];
            n5->child[o5] = i4;
            ON4 *n4 = t->n4[i4];
            words_to_u64(kids4 + 128 * c4, n4->kid, 64);
            words_to_u64(vals4 + 128 * c4, n4->val, 64);
            c4++;
            for (int o4 = 0; o4 < 4096; o4++) {
                if (!((n4->kid[o4 >> 6] >> (o4 & 63)) & 1)) continue;
                if (c3 >= n3c) goto fail;
                int32_t i3 = new_n3(t);
                n4 = t->n4[i4];
                n4->child[o4] = i3;
                ON3 *n3 = t->n3[i3];
                words_to_u64(vals3 + 16 * c3, n3->val, 8);
                for (int o3 = 0; o3 < 512; o3++)
                    if ((n3->val[o3 >> 6] >> (o3 & 63)) & 1) { n3->is_value[o3] = 1; n3->value[o3] = 1; }
                c3++;
            }
        }
    }
    if (c4 != n4c || c3 != n3c) goto fail;
    return t;
fail:
    orc_tree_free(t);
    return NULL;
}

/* count_nodes — vdb345.rs:266-287 */
void orc_count_nodes(const orc_tree *t, uint64_t out[3]) {
    out[0] = out[1] = out[2] = 0;
    for (size_t r = 0; r < t->nroots; r++) {
        const ON5 *n5 = t->n5[t->roots[r].n5];
        out[0]++;
        for (int o5 = 0; o5 < 32768; o5++) {
            if (n5->child[o5] < 0) continue;
            out[1]++;
            const ON4 *n4 = t->n4[n5->child[o5]];
            for (int o4 = 0; o4 < 4096; o4++)
                if (n4->child[o4] >= 0) out[2]++;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* compute_sdf — vdb345.rs:290-670, restated loop for loop.                  */
/* ------------------------------------------------------------------------ */
static int FN[13][3], BN[13][3];
static void build_neighbours(void) { /* vdb345.rs:327-343 */
    int k = 0;
    for (int dy = -1; dy <= 1; dy++)
        for (int dz = -1; dz <= 1; dz++) {
            FN[k][0] = -1; FN[k][1] = dy; FN[k][2] = dz;
            BN[k][0] = 1;  BN[k][1] = dy; BN[k][2] = dz;
            k++;
        }
    for (int dz = -1; dz <= 1; dz++) {
        FN[k][0] = 0; FN[k][1] = -1; FN[k][2] = dz;
        BN[k][0] = 0; BN[k][1] = 1;  BN[k][2] = dz;
        k++;
    }
    FN[k][0] = 0; FN[k][1] = 0; FN[k][2] = -1;
    BN[k][0] = 0; BN[k][1] = 0; BN[k][2] = 1;
}

static int same_node(const int32_t a[3], const int32_t b[3], int t) {
    return g2n(a[0], t) == g2n(b[0], t) && g2n(a[1], t) == g2n(b[1], t) && g2n(a[2], t) == g2n(b[2], t);
}

/* One slot update at the N5 level (vdb345.rs:368-395 / 508-535). */
static void sdf_n5_tile(orc_tree *t, ON5 *n5, int o5, const int32_t origin5[3], int (*NB)[3]) {
    uint32_t c5[3];
    orc_offset_to_child((uint64_t)o5, 5, c5);
    int32_t global[3];
    for (int i = 0; i < 3; i++) global[i] = origin5[i] + (int32_t)c5[i] * 128;
    uint32_t *tv = &n5->tile[o5];
    for (int k = 0; k < 13; k++) {
        int32_t nglobal[3];
        uint32_t nchild[3];
        for (int i = 0; i < 3; i++) {
            nglobal[i] = global[i] + NB[k][i] * 128;
            nchild[i] = (uint32_t)((int32_t)c5[i] + NB[k][i]);
        }
        if (same_node(nglobal, global, 12)) {
            uint64_t nid = orc_child_to_offset(nchild, 5);
            if (n5->child[nid] >= 0) { *tv = 1; break; }
            uint32_t v = n5->tile[nid];
            if (v + 1 < *tv) *tv = v + 1;
            continue;
        }
        uint64_t v; int lvl;
        int kind = orc_get_voxel(t, nglobal, &v, &lvl);
        if (kind == 2 && lvl == 5) { if ((uint32_t)v + 1 < *tv) *tv = (uint32_t)v + 1; }
        else *tv = 1;
    }
}
/* One slot update at the N4 level (vdb345.rs:405-435 / 545-575). */
static void sdf_n4_tile(orc_tree *t, ON4 *n4, int o4, const int32_t g5[3], int (*NB)[3]) {
    uint32_t c4[3];
    orc_offset_to_child((uint64_t)o4, 4, c4);
    int32_t global[3];
    for (int i = 0; i < 3; i++) global[i] = g5[i] + (int32_t)c4[i] * 8;
    uint32_t *tv = &n4->tile[o4];
    for (int k = 0; k < 13; k++) {
        int32_t nglobal[3];
        uint32_t nchild[3];
        for (int i = 0; i < 3; i++) {
            nglobal[i] = global[i] + NB[k][i] * 8;
            nchild[i] = (uint32_t)((int32_t)c4[i] + NB[k][i]);
        }
        if (same_node(nglobal, global, 7)) {
            uint64_t nid = orc_child_to_offset(nchild, 4);
            if (n4->child[nid] >= 0) { *tv = 1; break; }
            uint32_t v = n4->tile[nid];
            if (v + 1 < *tv) *tv = v + 1;
            continue;
        }
        uint64_t v; int lvl;
        int kind = orc_get_voxel(t, nglobal, &v, &lvl);
        if (kind == 2 && lvl == 4) { if ((uint32_t)v + 1 < *tv) *tv = (uint32_t)v + 1; }
        else *tv = 1;
    }
}
/* One voxel update at the N3 level (vdb345.rs:444-476 / 586-618). */
static void sdf_n3_voxel(orc_tree *t, ON3 *n3, int vi, const int32_t g4[3], int (*NB)[3]) {
    uint32_t c3[3];
    orc_offset_to_child((uint64_t)vi, 3, c3);
    int32_t global[3];
    for (int i = 0; i < 3; i++) global[i] = g4[i] + (int32_t)c3[i];
    uint64_t *tv = &n3->tile[vi];
    for (int k = 0; k < 13; k++) {
        int32_t nglobal[3];
        uint32_t nchild[3];
        for (int i = 0; i < 3; i++) {
            nglobal[i] = global[i] + NB[k][i];
            nchild[i] = (uint32_t)((int32_t)c3[i] + NB[k][i]);
        }
        if (same_node(nglobal, global, 3)) {
            uint64_t nid = orc_child_to_offset(nchild, 3);
            if (n3->is_value[nid]) { *tv = 1; break; }
            uint64_t v = n3->tile[nid];
            if (v + 1 < *tv) *tv = v + 1;
            continue;
        }
        uint64_t v; int lvl;
        int kind = orc_get_voxel(t, nglobal, &v, &lvl);
        if (kind == 0) { if (v + 1 < *tv) *tv = v + 1; }
        else *tv = 1;
    }
}

static void sdf_visit_n5(orc_tree *t, size_t r, int backward) {
    int (*NB)[3] = backward ? BN : FN;
    ON5 *n5 = t->n5[t->roots[r].n5];
    const int32_t *origin5 = t->roots[r].key;
    for (int s5 = 0; s5 < 32768; s5++) {
        int o5 = backward ? 32767 - s5 : s5;
        uint32_t c5[3];
        orc_offset_to_child((uint64_t)o5, 5, c5);
        int32_t g5[3];
        for (int i = 0; i < 3; i++) g5[i] = origin5[i] + (int32_t)c5[i] * 128;
        if (n5->child[o5] < 0) { sdf_n5_tile(t, n5, o5, origin5, NB); continue; }
        ON4 *n4 = t->n4[n5->child[o5]];
        for (int s4 = 0; s4 < 4096; s4++) {
            int o4 = backward ? 4095 - s4 : s4;
            uint32_t c4[3];
            orc_offset_to_child((uint64_t)o4, 4, c4);
            int32_t g4[3];
            for (int i = 0; i < 3; i++) g4[i] = g5[i] + (int32_t)c4[i] * 8;
            if (n4->child[o4] < 0) { sdf_n4_tile(t, n4, o4, g5, NB); continue; }
            ON3 *n3 = t->n3[n4->child[o4]];
            for (int s3 = 0; s3 < 512; s3++) {
                int vi = backward ? 511 - s3 : s3;
                if (n3->is_value[vi]) continue;
                sdf_n3_voxel(t, n3, vi, g4, NB);
            }
        }
    }
}

void orc_compute_sdf(orc_tree *t) {
    build_neighbours();
    /* Initialise every tile with MAX - 1 (vdb345.rs:292-325). */
    for (size_t r = 0; r < t->nroots; r++) {
        ON5 *n5 = t->n5[t->roots[r].n5];
        for (int o5 = 0; o5 < 32768; o5++) {
            if (n5->child[o5] < 0) { n5->tile[o5] = UINT32_MAX - 1; continue; }
            ON4 *n4 = t->n4[n5->child[o5]];
            for (int o4 = 0; o4 < 4096; o4++) {
                if (n4->child[o4] < 0) { n4->tile[o4] = UINT32_MAX - 1; continue; }
                ON3 *n3 = t->n3[n4->child[o4]];
                for (int o3 = 0; o3 < 512; o3++)
                    if (!n3->is_value[o3]) n3->tile[o3] = UINT64_MAX - 1;
            }
        }
    }
    for (size_t r = 0; r < t->nroots; r++) sdf_visit_n5(t, r, 0);       /* forward */
    for (size_t r = t->nroots; r-- > 0;) sdf_visit_n5(t, r, 1);         /* backward */
}

/* masks() / origins() — vdb345.rs:108-161 */
void orc_masks(const orc_tree *t, uint32_t *kids5, uint32_t *vals5, uint32_t *kids4,
               uint32_t *vals4, uint32_t *vals3, int32_t *origins) {
    size_t i5 = 0, i4 = 0, i3 = 0;
    for (size_t r = 0; r < t->nroots; r++) {
        const ON5 *n5 = t->n5[t->roots[r].n5];
        for (int o5 = 0; o5 < 32768; o5++) {
            if (n5->child[o5] < 0) continue;
            const ON4 *n4 = t->n4[n5->child[o5]];
            for (int o4 = 0; o4 < 4096; o4++) {
                if (n4->child[o4] < 0) continue;
                u64_to_words(t->n3[n4->child[o4]]->val, vals3 + 16 * i3, 8);
                i3++;
            }
            u64_to_words(n4->val, vals4 + 128 * i4, 64);
            u64_to_words(n4->kid, kids4 + 128 * i4, 64);
            i4++;
        }
        u64_to_words(n5->val, vals5 + 1024 * i5, 512);
        u64_to_words(n5->kid, kids5 + 1024 * i5, 512);
        for (int i = 0; i < 3; i++) origins[4 * i5 + i] = t->roots[r].key[i];
        origins[4 * i5 + 3] = 0;
        i5++;
    }
}

/* closest_power_of_3 — vdb345.rs:684-690 */
static uint64_t cpow3(uint64_t n) {
    uint64_t i = 0;
    while (i * i * i < n) i++;
    return i;
}

/* atlas() — vdb345.rs:163-264, stored in the texture layout the upload at
 * wgpu_context.rs:119-151 produces: texel (x,y,z) = cube[x][y][z] at (z*S + y)*S + x. */
void orc_atlas(const orc_tree *t, uint32_t side[3], uint32_t *a5, uint32_t *a4, uint32_t *a3) {
    uint64_t cnt[3];
    orc_count_nodes(t, cnt);
    uint64_t d5 = cpow3(cnt[0]), d4 = cpow3(cnt[1]), d3 = cpow3(cnt[2]);
    side[0] = (uint32_t)(32 * d5);
    side[1] = (uint32_t)(16 * d4);
    side[2] = (uint32_t)(8 * d3);
    if (!a5 || !a4 || !a3) return;
    uint64_t S5 = side[0], S4 = side[1], S3 = side[2];
    memset(a5, 0, S5 * S5 * S5 * 4);
    memset(a4, 0, S4 * S4 * S4 * 4);
    memset(a3, 0, S3 * S3 * S3 * 4);
#define AIDX(S, x, y, z) ((((uint64_t)(z)) * (S) + (uint64_t)(y)) * (S) + (uint64_t)(x))
    uint64_t i5 = 0, i4 = 0, i3 = 0;
    for (size_t r = 0; r < t->nroots; r++) {
        const ON5 *n5 = t->n5[t->roots[r].n5];
        uint64_t O5[3] = {(i5 % d5) * 32, ((i5 / d5) % d5) * 32, (i5 / (d5 * d5)) * 32};
        for (int o5 = 0; o5 < 32768; o5++) {
            uint32_t c5[3];
            orc_offset_to_child((uint64_t)o5, 5, c5);
            uint64_t P5 = AIDX(S5, O5[0] + c5[0], O5[1] + c5[1], O5[2] + c5[2]);
            if (n5->child[o5] < 0) { a5[P5] = n5->tile[o5]; continue; }
            const ON4 *n4 = t->n4[n5->child[o5]];
            uint64_t O4[3] = {(i4 % d4) * 16, ((i4 / d4) % d4) * 16, (i4 / (d4 * d4)) * 16};
            for (int o4 = 0; o4 < 4096; o4++) {
                uint32_t c4[3];
                orc_offset_to_child((uint64_t)o4, 4, c4);
                uint64_t P4 = AIDX(S4, O4[0] + c4[0], O4[1] + c4[1], O4[2] + c4[2]);
                if (n4->child[o4] < 0) { a4[P4] = n4->tile[o4]; continue; }
                const ON3 *n3 = t->n3[n4->child[o4]];
                uint64_t O3[3] = {(i3 % d3) * 8, ((i3 / d3) % d3) * 8, (i3 / (d3 * d3)) * 8};
                for (int o3 = 0; o3 < 512; o3++) {
                    uint32_t c3[3];
                    orc_offset_to_child((uint64_t)o3, 3, c3);
                    uint64_t P3 = AIDX(S3, O3[0] + c3[0], O3[1] + c3[1], O3[2] + c3[2]);
                    a3[P3] = n3->is_value[o3] ? n3->value[o3] : (uint32_t)n3->tile[o3];
                }
                a4[P4] = (uint32_t)i3;
                i3++;
            }
            a5[P5] = (uint32_t)i4;
            i4++;
        }
        i5++;
    }
#undef AIDX
}

/* ------------------------------------------------------------------------ */
/* Uniform — compute_state.rs:87-131 with camera.rs:31-35 (cgmath 0.18       */
/* look_at_rh; normalize(v) = v * (1 / |v|)). The 4x4 inverse is a cofactor  */
/* expansion; cgmath's own Matrix4::invert source is not in the reference    */
/* tree, so this builder is not bit-pinned to it.                            */
/* ------------------------------------------------------------------------ */
static v3 cg_normalize(v3 a) {
    float m = sqrtf((a.x * a.x + a.y * a.y) + a.z * a.z);
    float s = 1.0f / m;
    return V3(a.x * s, a.y * s, a.z * s);
}
static v3 cg_cross(v3 a, v3 b) {
    return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static float det3(float a, float b, float c, float d, float e, float f, float g, float h, float i) {
    return a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
}
static void invert4(const float m[16], float out[16]) {
    /* m is column-major: m[c*4 + r]. Inverse = adjugate / det. */
#define M(r, c) m[(c) * 4 + (r)]
    float cof[16];
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) {
            float s[9];
            int k = 0;
            for (int rr = 0; rr < 4; rr++) {
                if (rr == r) continue;
                for (int cc = 0; cc < 4; cc++) {
                    if (cc == c) continue;
                    s[k++] = M(rr, cc);
                }
            }
            float d = det3(s[0], s[1], s[2], s[3], s[4], s[5], s[6], s[7], s[8]);
            cof[c * 4 + r] = ((r + c) & 1) ? -d : d;
        }
    float det = M(0, 0) * cof[0 * 4 + 0] + M(0, 1) * cof[1 * 4 + 0] + M(0, 2) * cof[2 * 4 + 0] +
                M(0, 3) * cof[3 * 4 + 0];
    float inv = 1.0f / det;
    /* inverse(r, c) = cof(c, r) / det */
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) out[c * 4 + r] = cof[r * 4 + c] * inv;
#undef M
}

void orc_state_build(const float eye[3], const float target[3], const float up[3],
                     float aspect, float fovy_deg, float width, uint32_t render_mode,
                     const uint32_t show_345[3], const float sun_dir[3], const float sun_color[3],
                     float sun_intensity, orc_state *o) {
    memset(o, 0, sizeof(*o));
    v3 e = V3(eye[0], eye[1], eye[2]);
    v3 f = cg_normalize(vsub(V3(target[0], target[1], target[2]), e));
    v3 s = cg_normalize(cg_cross(f, V3(up[0], up[1], up[2])));
    v3 u = cg_cross(s, f);
    float view[16] = {s.x, u.x, -f.x, 0.0f, s.y, u.y, -f.y, 0.0f, s.z, u.z, -f.z, 0.0f,
                      -vdot(e, s), -vdot(e, u), vdot(e, f), 1.0f};
    float c2w[16];
    invert4(view, c2w);
    memcpy(o->view_projection, view, sizeof(view));
    memcpy(o->camera_to_world, c2w, sizeof(c2w));
    o->eye[0] = eye[0]; o->eye[1] = eye[1]; o->eye[2] = eye[2]; o->eye[3] = 0.0f;
    float height = width / aspect;
    float fovy_rad = fovy_deg * (3.14159265358979323846f / 180.0f);
    float tan_half = tanf(fovy_rad * 0.5f);
    float a = -width / 2.0f, b = height / 2.0f;
    for (int i = 0; i < 4; i++) {
        float uu = c2w[0 * 4 + i], vv = c2w[1 * 4 + i], ww = c2w[2 * 4 + i];
        float w_term = (ww * b) / tan_half;
        o->u[i] = uu;
        o->mv[i] = -vv;
        o->wp[i] = (a * uu + b * vv) - w_term;
    }
    o->render_mode[0] = render_mode;
    for (int i = 0; i < 3; i++) {
        o->show_345[i] = show_345 ? show_345[i] : 0;
        o->sun_dir[i] = sun_dir[i];
        o->sun_color[i] = sun_color[i];
    }
    o->sun_color[3] = sun_intensity;
}

/* ------------------------------------------------------------------------ */
/* The raycast shader — raycast.comp.wgsl:60-519                             */
/* ------------------------------------------------------------------------ */
typedef struct { int32_t o[3]; uint32_t idx; } Parent;            /* :344-347 */
typedef struct { uint32_t dist, np; Parent par[3]; } VdbLeaf;      /* :349-354 */
typedef struct {
    uint32_t state;
    VdbLeaf leaf;
    v3 p;
    int mask[3];
    uint32_t i;
    uint32_t bytes;
    uint32_t grazing;
} HDDAout;                                                         /* :128-142 */

static inline uint32_t tex_load(const orc_view *v, int lvl, uint32_t x, uint32_t y, uint32_t z) {
    const uint32_t *d = v->dims[lvl];
    return v->atlas[lvl][((uint64_t)z * d[1] + y) * d[0] + x];
}
static inline int bit(const uint32_t *words, uint32_t off) {
    return (words[off >> 5] & (1u << (off & 31u))) != 0;
}

static VdbLeaf from_node3(const orc_view *v, const int32_t pos[3], VdbLeaf leaf, uint32_t *bytes) { /* :477-494 */
    uint32_t l[3] = {(uint32_t)pos[0] & 7u, (uint32_t)pos[1] & 7u, (uint32_t)pos[2] & 7u};
    uint32_t off = (l[0] << 6) | (l[1] << 3) | l[2];
    uint32_t idx = leaf.par[2].idx;
    int in_val3 = bit(v->vals3 + 16ull * idx, off);
    uint32_t d = v->dims[2][0] >> 3;
    uint32_t ox = 8 * (idx % d), oy = 8 * ((idx / d) % d), oz = 8 * (idx / (d * d));
    uint32_t voxel = tex_load(v, 2, l[0] + ox, l[1] + oy, l[2] + oz);
    *bytes += 8;
    leaf.np = 3;
    leaf.dist = in_val3 ? 0u : voxel;
    return leaf;
}
static VdbLeaf from_node4(const orc_view *v, const int32_t pos[3], VdbLeaf leaf, uint32_t *bytes) { /* :446-475 */
    uint32_t c[3] = {((uint32_t)pos[0] & 127u) >> 3, ((uint32_t)pos[1] & 127u) >> 3,
                     ((uint32_t)pos[2] & 127u) >> 3};
    uint32_t off = (c[0] << 8) | (c[1] << 4) | c[2];
    uint32_t idx = leaf.par[1].idx;
    int in_kid4 = bit(v->kids4 + 128ull * idx, off);
    int in_val4 = bit(v->vals4 + 128ull * idx, off);
    uint32_t d = v->dims[1][0] >> 4;
    uint32_t ox = 16 * (idx % d), oy = 16 * ((idx / d) % d), oz = 16 * (idx / (d * d));
    uint32_t n3 = tex_load(v, 1, c[0] + ox, c[1] + oy, c[2] + oz);
    *bytes += 12;
    if (in_val4) { leaf.dist = 0; leaf.np = 2; return leaf; }
    if (!in_kid4) { leaf.dist = n3; leaf.np = 2; return leaf; }
    for (int i = 0; i < 3; i++) leaf.par[2].o[i] = g2n(pos[i], 3);
    leaf.par[2].idx = n3;
    leaf.np = 3;
    return from_node3(v, pos, leaf, bytes);
}
static VdbLeaf from_node5(const orc_view *v, const int32_t pos[3], VdbLeaf leaf, uint32_t *bytes) { /* :415-444 */
    uint32_t c[3] = {((uint32_t)pos[0] & 4095u) >> 7, ((uint32_t)pos[1] & 4095u) >> 7,
                     ((uint32_t)pos[2] & 4095u) >> 7};
    uint32_t off = (c[0] << 10) | (c[1] << 5) | c[2];
    uint32_t idx = leaf.par[0].idx;
    int in_kid5 = bit(v->kids5 + 1024ull * idx, off);
    int in_val5 = bit(v->vals5 + 1024ull * idx, off);
    uint32_t d = v->dims[0][1] >> 5; /* the reference reads .y here */
    uint32_t ox = 32 * (idx % d), oy = 32 * ((idx / d) % d), oz = 32 * (idx / (d * d));
    uint32_t n4 = tex_load(v, 0, c[0] + ox, c[1] + oy, c[2] + oz);
    *bytes += 12;
    if (in_val5) { leaf.dist = 0; leaf.np = 1; return leaf; }
    if (!in_kid5) { leaf.dist = n4; leaf.np = 1; return leaf; }
    for (int i = 0; i < 3; i++) leaf.par[1].o[i] = g2n(pos[i], 7);
    leaf.par[1].idx = n4;
    leaf.np = 2;
    return from_node4(v, pos, leaf, bytes);
}
static VdbLeaf from_nothing(const orc_view *v, const int32_t pos[3], VdbLeaf leaf, uint32_t *bytes) { /* :398-413 */
    int32_t g[3] = {g2n(pos[0], 12), g2n(pos[1], 12), g2n(pos[2], 12)};
    for (uint64_t i = 0; i < v->n5; i++) {
        *bytes += 16;
        const int32_t *o = v->origins + 4 * i;
        if (o[0] == g[0] && o[1] == g[1] && o[2] == g[2]) {
            for (int k = 0; k < 3; k++) leaf.par[0].o[k] = g[k];
            leaf.par[0].idx = (uint32_t)i;
            leaf.np = 1;
            return from_node5(v, pos, leaf, bytes);
        }
    }
    leaf.dist = 1;
    leaf.np = 0;
    return leaf;
}
static int origin_eq(const Parent *p, const int32_t pos[3], int t) {
    return p->o[0] == g2n(pos[0], t) && p->o[1] == g2n(pos[1], t) && p->o[2] == g2n(pos[2], t);
}
static VdbLeaf from_leaf(const orc_view *v, const int32_t pos[3], VdbLeaf leaf, uint32_t *bytes) { /* :360-396 */
    if (leaf.np == 3) {
        if (origin_eq(&leaf.par[2], pos, 3)) return from_node3(v, pos, leaf, bytes);
        if (origin_eq(&leaf.par[1], pos, 7)) return from_node4(v, pos, leaf, bytes);
        if (origin_eq(&leaf.par[0], pos, 12)) return from_node5(v, pos, leaf, bytes);
        return from_nothing(v, pos, leaf, bytes);
    }
    if (leaf.np == 2) {
        if (origin_eq(&leaf.par[1], pos, 7)) return from_node4(v, pos, leaf, bytes);
        if (origin_eq(&leaf.par[0], pos, 12)) return from_node5(v, pos, leaf, bytes);
        return from_nothing(v, pos, leaf, bytes);
    }
    if (leaf.np == 1) {
        if (origin_eq(&leaf.par[0], pos, 12)) return from_node5(v, pos, leaf, bytes);
        return from_nothing(v, pos, leaf, bytes);
    }
    return from_nothing(v, pos, leaf, bytes);
}

static inline float sign11f(float x) { return (x < 0.0f) ? -1.0f : 1.0f; } /* :70-76 */

static int near_tie(float a, float b) {
    if (a != a || b != b) return 0;
    float m = fabsf(a) > fabsf(b) ? fabsf(a) : fabsf(b);
    float ulp = nextafterf(m, INFINITY) - m;
    return fabsf(a - b) <= ulp;
}
static int near_boundary(float x) {
    if (x != x || isinf(x)) return 0;
    return floorf(nextafterf(x, INFINITY)) != floorf(x) || floorf(nextafterf(x, -INFINITY)) != floorf(x);
}

static HDDAout hdda_ray(const orc_view *v, v3 src, v3 dir) { /* :84-126 */
    static const float scale[4] = {1.0f, 8.0f, 128.0f, 4096.0f}; /* :83 */
    HDDAout out;
    memset(&out, 0, sizeof(out));
    v3 p = src;
    v3 step = V3(sign11f(dir.x), sign11f(dir.y), sign11f(dir.z));
    v3 step01 = V3(pmax(0.0f, step.x), pmax(0.0f, step.y), pmax(0.0f, step.z));
    v3 idir = V3(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
    int mask[3] = {0, 0, 0};
    VdbLeaf leaf;
    memset(&leaf, 0, sizeof(leaf));
    uint32_t bytes = 0, grazing = 0;
    for (uint32_t i = 0; i < 1000u; i++) {
        int32_t pos[3] = {f2i_sat(floorf(p.x)), f2i_sat(floorf(p.y)), f2i_sat(floorf(p.z))};
        leaf = from_leaf(v, pos, leaf, &bytes);
        if (leaf.dist == 0u) {
            out.state = 0; out.leaf = leaf; out.p = p; out.i = i;
            memcpy(out.mask, mask, sizeof(mask));
            out.bytes = bytes; out.grazing = grazing;
            return out;
        }
        if (4096.0f < fabsf(p.x) || 4096.0f < fabsf(p.y) || 4096.0f < fabsf(p.z)) {
            out.state = 1; out.leaf = leaf; out.p = p; out.i = i;
            memcpy(out.mask, mask, sizeof(mask));
            out.bytes = bytes; out.grazing = grazing;
            return out;
        }
        float size = (float)leaf.dist;
        switch (leaf.np) {
            case 3u: size *= scale[0]; break;
            case 2u: size *= scale[1]; break;
            case 1u: size *= scale[2]; break;
            case 0u: size *= scale[3]; break;
            default: size = scale[0]; break;
        }
        float pm[3] = {p.x, p.y, p.z}, st[3] = {step01.x, step01.y, step01.z},
              id[3] = {idir.x, idir.y, idir.z}, tm[3];
        for (int c = 0; c < 3; c++) {
            float q = floorf(pm[c] / size);
            float mod = pm[c] - size * q;
            float a = size * st[c];
            tm[c] = id[c] * (a - mod);
        }
        float t = pmin(pmin(tm[0], tm[1]), tm[2]);
        p = V3(p.x + t * dir.x, p.y + t * dir.y, p.z + t * dir.z);
        mask[0] = (tm[0] <= tm[1]) && (tm[0] <= tm[2]);
        mask[1] = (tm[1] <= tm[2]) && (tm[1] <= tm[0]);
        mask[2] = (tm[2] <= tm[0]) && (tm[2] <= tm[1]);
        v3 nudge = vmul(vscale(4e-4f, step), V3((float)mask[0], (float)mask[1], (float)mask[2]));
        p = vadd(p, nudge);
        /* Grazing: a rounded (non-zero) step whose winning tMax is within 1 ulp of
         * another, or that leaves a non-stepped coordinate within 1 ulp of a cell
         * boundary. Exact zero-length steps (p already on a boundary) are stable. */
        if (t != 0.0f && t == t) {
            int tie = 0;
            for (int a = 0; a < 3; a++)
                for (int b = a + 1; b < 3; b++)
                    if ((tm[a] == t || tm[b] == t) && near_tie(tm[a], tm[b])) tie = 1;
            if (tie || (!mask[0] && near_boundary(p.x)) || (!mask[1] && near_boundary(p.y)) ||
                (!mask[2] && near_boundary(p.z)))
                grazing = 1;
        }
    }
    out.state = 2; out.leaf = leaf; out.p = p; out.i = 1000u;
    memcpy(out.mask, mask, sizeof(mask));
    out.bytes = bytes; out.grazing = grazing;
    return out;
}

/* Material constants :145-150 */
#define K_D 0.7f
#define K_A 0.3f
#define REFLECTIVITY 0.9f
#define WALL_I 0.1f

static v3 maskf(const int m[3]) { return V3((float)m[0], (float)m[1], (float)m[2]); }

typedef struct {
    const orc_view *v;
    const orc_state *s;
    uint32_t shadow_traced, shadow_state, shadow_steps, shadow_bytes;
    uint32_t surf_found, surf_k;  /* mode 5: crossing found, sample index */
    float surf_t;
} Ctx;

static v3 sun3(const orc_state *s) { return V3(s->sun_dir[0], s->sun_dir[1], s->sun_dir[2]); }
static v3 suncol3(const orc_state *s) { return V3(s->sun_color[0], s->sun_color[1], s->sun_color[2]); }

static HDDAout shadow_ray(Ctx *c, v3 src) {
    HDDAout h = hdda_ray(c->v, src, vneg(sun3(c->s)));
    return h;
}

static v3 wall_colour(v3 N) { /* :300-305 / :333-338 */
    v3 Np = V3(pmax(0.0f, N.x), pmax(0.0f, N.y), pmax(0.0f, N.z));
    v3 Nn = vneg(V3(pmin(0.0f, N.x), pmin(0.0f, N.y), pmin(0.0f, N.z)));
    v3 r = vscale_r(V3(WALL_I, 0.0f, 0.0f), Np.x);
    r = vadd(r, vscale_r(V3(0.0f, WALL_I, 0.0f), Np.y));
    r = vadd(r, vscale_r(V3(0.0f, 0.0f, WALL_I), Np.z));
    r = vadd(r, vscale_r(V3(WALL_I, WALL_I, 0.0f), Nn.x));
    r = vadd(r, vscale_r(V3(0.0f, WALL_I, WALL_I), Nn.y));
    r = vadd(r, vscale_r(V3(WALL_I, 0.0f, WALL_I), Nn.z));
    return r;
}

static v3 lit_colour(Ctx *c, const HDDAout *hit, v3 step, v3 N, float *I_out) { /* shared by :280-290, :317-325 */
    const orc_state *s = c->s;
    float I = (s->sun_color[3] * K_D) * vdot(vneg(sun3(s)), N);
    I = pmax(0.0f, I);
    *I_out = I;
    v3 base = V3(0.4f, 0.2f, 0.2f);
    if (I != 0.0f) {
        v3 src = vsub(hit->p, vmul(vscale(4e-2f, step), maskf(hit->mask)));
        if (shadow_ray(c, src).state == 0u) return vadd(base, vscale_r(vscale(I, suncol3(s)), 0.05f));
    }
    return vadd(base, vscale(I, suncol3(s)));
}

static v3 reflect_ray1(Ctx *c, v3 src, v3 dir) { /* :311-342 */
    HDDAout hit = hdda_ray(c->v, src, dir);
    v3 step = V3(sign11f(dir.x), sign11f(dir.y), sign11f(dir.z));
    if (hit.state == 0u) {
        v3 N = vnormalize(vmul(vneg(step), maskf(hit.mask)));
        float I;
        return lit_colour(c, &hit, step, N, &I);
    }
    if (hit.state == 1u) return wall_colour(vnormalize(vmul(vneg(step), maskf(hit.mask))));
    return dir;
}

static v3 reflect_ray2(Ctx *c, v3 src, v3 dir) { /* :267-309 */
    HDDAout hit = hdda_ray(c->v, src, dir);
    v3 step = V3(sign11f(dir.x), sign11f(dir.y), sign11f(dir.z));
    if (hit.state == 0u) {
        v3 N = vnormalize(vmul(vneg(step), maskf(hit.mask)));
        v3 rdir = vnormalize(vsub(dir, vscale_r(vscale(2.0f, N), vdot(dir, N))));
        v3 rsrc = vsub(hit.p, vmul(vscale(4e-2f, step), maskf(hit.mask)));
        v3 rcol = reflect_ray1(c, rsrc, rdir);
        float I;
        v3 mcol = lit_colour(c, &hit, step, N, &I);
        return vmix(mcol, rcol, REFLECTIVITY);
    }
    if (hit.state == 1u) return wall_colour(vnormalize(vmul(vneg(step), maskf(hit.mask))));
    return dir;
}

/* ------------------------------------------------------------------------ */
/* Zero-crossing hit mode (render_mode 5). An extension with no counterpart in */
/* the reference (its hit is the first active voxel); the product kernel      */
/* follows this specification operation for operation:                        */
/*   phi(i,j,k): the leaf value of voxel (i,j,k); -band inside an active tile  */
/*     (value bit of an N5/N4 slot); +band anywhere else;                     */
/*   phi(q) for a point q: trilinear in the cell floor(q) .. floor(q) + 1;     */
/*   search: from t0 = max(0, t_hit - 1), where t_hit = dot(p_hit - eye, dir)  */
/*     of the primary HDDA hit, samples t_k = t0 + k * 0.25 for k < 64; the    */
/*     first k with phi(t_k) <= 0 ends it (k = 0: t* = t0; else the secant     */
/*     t* = t_{k-1} + 0.25 * (phi_{k-1} / (phi_{k-1} - phi_k)));              */
/*   normal: the gradient of the trilinear phi at eye + t* dir, normalised     */
/*     (-dir when it is zero); colour: mode 3's I_a + I_d with that normal and */
/*     no shadow ray; no crossing: mode 0's colour of the HDDA hit.            */
/* ------------------------------------------------------------------------ */
#define SURF_H 0.25f
#define SURF_N 64u

static float surf_phi(const orc_view *v, int32_t i, int32_t j, int32_t k) {
    const float band = v->band;
    const int32_t pos[3] = {i, j, k};
    const int32_t g[3] = {g2n(i, 12), g2n(j, 12), g2n(k, 12)};
    uint64_t n5 = UINT64_MAX;
    for (uint64_t a = 0; a < v->n5; a++) {
        const int32_t *o = v->origins + 4 * a;
        if (o[0] == g[0] && o[1] == g[1] && o[2] == g[2]) { n5 = a; break; }
    }
    if (n5 == UINT64_MAX) return band;
    uint32_t c5[3] = {((uint32_t)pos[0] & 4095u) >> 7, ((uint32_t)pos[1] & 4095u) >> 7, ((uint32_t)pos[2] & 4095u) >> 7};
    uint32_t off5 = (c5[0] << 10) | (c5[1] << 5) | c5[2];
    if (bit(v->vals5 + 1024ull * n5, off5)) return -band;
    if (!bit(v->kids5 + 1024ull * n5, off5)) return band;
    uint32_t d5 = v->dims[0][1] >> 5;
    uint32_t n4 = tex_load(v, 0, c5[0] + 32 * (uint32_t)(n5 % d5), c5[1] + 32 * (uint32_t)((n5 / d5) % d5),
                           c5[2] + 32 * (uint32_t)(n5 / (d5 * d5)));
    uint32_t c4[3] = {((uint32_t)pos[0] & 127u) >> 3, ((uint32_t)pos[1] & 127u) >> 3, ((uint32_t)pos[2] & 127u) >> 3};
    uint32_t off4 = (c4[0] << 8) | (c4[1] << 4) | c4[2];
    if (bit(v->vals4 + 128ull * n4, off4)) return -band;
    if (!bit(v->kids4 + 128ull * n4, off4)) return band;
    uint32_t d4 = v->dims[1][0] >> 4;
    uint32_t n3 = tex_load(v, 1, c4[0] + 16 * (n4 % d4), c4[1] + 16 * ((n4 / d4) % d4), c4[2] + 16 * (n4 / (d4 * d4)));
    uint32_t off3 = (((uint32_t)pos[0] & 7u) << 6) | (((uint32_t)pos[1] & 7u) << 3) | ((uint32_t)pos[2] & 7u);
    return v->values[512ull * n3 + off3];
}

static inline float lerpf(float a, float b, float t) { return a + t * (b - a); }

/* The 8 corner values of the cell of q and q's position inside it. */
static void surf_cell(const orc_view *v, v3 q, float c[8], float f[3]) {
    float fl[3] = {floorf(q.x), floorf(q.y), floorf(q.z)};
    int32_t i = f2i_sat(fl[0]), j = f2i_sat(fl[1]), k = f2i_sat(fl[2]);
    f[0] = q.x - fl[0]; f[1] = q.y - fl[1]; f[2] = q.z - fl[2];
    for (int n = 0; n < 8; n++)  /* corner n = (dx << 2) | (dy << 1) | dz */
        c[n] = surf_phi(v, i + (n >> 2), j + ((n >> 1) & 1), k + (n & 1));
}

static float surf_interp(const float c[8], const float f[3]) {
    float a00 = lerpf(c[0], c[4], f[0]), a10 = lerpf(c[2], c[6], f[0]);
    float a01 = lerpf(c[1], c[5], f[0]), a11 = lerpf(c[3], c[7], f[0]);
    return lerpf(lerpf(a00, a10, f[1]), lerpf(a01, a11, f[1]), f[2]);
}

static v3 surf_gradient(const float c[8], const float f[3]) {
    float gx = lerpf(lerpf(c[4] - c[0], c[6] - c[2], f[1]), lerpf(c[5] - c[1], c[7] - c[3], f[1]), f[2]);
    float gy = lerpf(lerpf(c[2] - c[0], c[6] - c[4], f[0]), lerpf(c[3] - c[1], c[7] - c[5], f[0]), f[2]);
    float gz = lerpf(lerpf(c[1] - c[0], c[5] - c[4], f[0]), lerpf(c[3] - c[2], c[7] - c[6], f[0]), f[1]);
    return V3(gx, gy, gz);
}

static float surf_sample(const orc_view *v, v3 eye, v3 dir, float t) {
    float c[8], f[3];
    surf_cell(v, V3(eye.x + t * dir.x, eye.y + t * dir.y, eye.z + t * dir.z), c, f);
    return surf_interp(c, f);
}

/* Returns 1 and t*, the sample index and the normal when a crossing is found. */
static int surf_search(const orc_view *v, v3 eye, v3 dir, float t_hit, float *ts, uint32_t *ks, v3 *N) {
    if (!v->values) return 0;
    float t0 = t_hit - 1.0f;
    if (!(t0 > 0.0f)) t0 = 0.0f;
    float prev = surf_sample(v, eye, dir, t0);
    int found = 0;
    if (prev <= 0.0f) {
        *ts = t0; *ks = 0; found = 1;
    } else {
        for (uint32_t k = 1; k < SURF_N; k++) {
            float tk = t0 + (float)k * SURF_H;
            float ph = surf_sample(v, eye, dir, tk);
            if (ph <= 0.0f) {
                float tp = t0 + (float)(k - 1) * SURF_H;
                *ts = tp + SURF_H * (prev / (prev - ph));
                *ks = k; found = 1;
                break;
            }
            prev = ph;
        }
    }
    if (!found) return 0;
    float c[8], f[3];
    surf_cell(v, V3(eye.x + *ts * dir.x, eye.y + *ts * dir.y, eye.z + *ts * dir.z), c, f);
    v3 g = surf_gradient(c, f);
    *N = vdot(g, g) == 0.0f ? vneg(dir) : vnormalize(g);
    return 1;
}

static v3 ray_trace(Ctx *c, v3 src, v3 dir, HDDAout *primary) { /* :152-265 */
    const orc_state *s = c->s;
    HDDAout hit = hdda_ray(c->v, src, dir);
    *primary = hit;
    v3 step = V3(sign11f(dir.x), sign11f(dir.y), sign11f(dir.z));
    uint32_t mode = s->render_mode[0];
    if (hit.state == 0u) {
        v3 grid = vsplat(0.0f);
        float fx = floorf(hit.p.x), fy = floorf(hit.p.y), fz = floorf(hit.p.z);
        if (s->show_345[2] == 1u &&
            (fmodf(fx, 4096.0f) == 0.0f || fmodf(fy, 4096.0f) == 0.0f || fmodf(fz, 4096.0f) == 0.0f))
            grid = V3(-0.3f, -0.3f, 1.0f);
        else if (s->show_345[1] == 1u &&
                 (fmodf(fx, 128.0f) == 0.0f || fmodf(fy, 128.0f) == 0.0f || fmodf(fz, 128.0f) == 0.0f))
            grid = V3(0.6f, -0.2f, -0.2f);
        else if (s->show_345[0] == 1u &&
                 (fmodf(fx, 8.0f) == 0.0f || fmodf(fy, 8.0f) == 0.0f || fmodf(fz, 8.0f) == 0.0f))
            grid = V3(-0.1f, 0.5f, 0.3f);
        v3 m = maskf(hit.mask);
        switch (mode) {
            case 0u: {
                v3 a = vmul(m, V3(0.2f, 0.2f, 0.3f));
                return vadd(grid, vsplat((a.x + a.y) + a.z));
            }
            case 1u:
                return vadd(vadd(grid, vsplat(0.1f)), vmul(m, vsplat(0.4f)));
            case 2u: {
                float t = (float)hit.i / 200.0f;
                return vadd(grid, vmix(V3(0.72f, 1.0f, 0.99f), V3(1.0f, 0.0f, 0.0f), t));
            }
            case 3u: {
                v3 N = vnormalize(vmul(vneg(step), m));
                float LN = pmax(0.0f, s->sun_color[3] * vdot(vneg(sun3(s)), N));
                v3 I_d = vscale_r(vmul(vscale(K_D, suncol3(s)), V3(0.4f, 0.2f, 0.2f)), LN);
                v3 I_a = vmul(vscale(K_A, V3(0.4f, 0.4f, 0.3f)), V3(0.4f, 0.2f, 0.2f));
                if (LN != 0.0f) {
                    v3 ssrc = vsub(hit.p, vmul(vscale(4e-2f, step), m));
                    HDDAout sh = shadow_ray(c, ssrc);
                    c->shadow_traced = 1;
                    c->shadow_state = sh.state;
                    c->shadow_steps = sh.i;
                    c->shadow_bytes = sh.bytes;
                    if (sh.state == 0u) return I_a;
                }
                return vadd(I_a, I_d);
            }
            case 4u: {
                v3 N = vnormalize(vmul(vneg(step), m));
                float I;
                v3 mcol = lit_colour(c, &hit, step, N, &I);
                v3 rdir = vnormalize(vsub(dir, vscale_r(vscale(2.0f, N), vdot(dir, N))));
                v3 rsrc = vsub(hit.p, vmul(vscale(4e-2f, step), m));
                v3 rcol = reflect_ray2(c, rsrc, rdir);
                return vmix(mcol, rcol, REFLECTIVITY);
            }
            case 5u: {
                float ts;
                uint32_t ks;
                v3 N;
                v3 d = vsub(hit.p, src);
                if (surf_search(c->v, src, dir, vdot(d, dir), &ts, &ks, &N)) {
                    c->surf_found = 1; c->surf_k = ks; c->surf_t = ts;
                    float LN = pmax(0.0f, s->sun_color[3] * vdot(vneg(sun3(s)), N));
                    v3 I_d = vscale_r(vmul(vscale(K_D, suncol3(s)), V3(0.4f, 0.2f, 0.2f)), LN);
                    v3 I_a = vmul(vscale(K_A, V3(0.4f, 0.4f, 0.3f)), V3(0.4f, 0.2f, 0.2f));
                    return vadd(I_a, I_d);
                }
                v3 a = vmul(m, V3(0.2f, 0.2f, 0.3f));
                return vsplat((a.x + a.y) + a.z);
            }
            default: {
                v3 a = vmul(m, V3(0.2f, 0.2f, 0.3f));
                return vadd(grid, vsplat((a.x + a.y) + a.z));
            }
        }
    }
    if (hit.state == 1u) {
        v3 m = maskf(hit.mask);
        switch (mode) {
            case 2u: {
                float t = (float)hit.i / 200.0f;
                v3 a = vmul(m, V3(0.04f, 0.08f, 0.12f));
                return vadd(vmix(V3(0.72f, 1.0f, 0.99f), V3(1.0f, 0.0f, 0.0f), t), vsplat((a.x + a.y) + a.z));
            }
            case 4u: {
                v3 N = vnormalize(vmul(vneg(step), m));
                v3 Np = V3(pmax(0.0f, N.x), pmax(0.0f, N.y), pmax(0.0f, N.z));
                v3 Nn = vneg(V3(pmin(0.0f, N.x), pmin(0.0f, N.y), pmin(0.0f, N.z)));
                float ty = hit.p.y / 4096.0f;
                v3 r = vscale_r(vmix(V3(WALL_I, 0.0f, 0.0f), V3(WALL_I * 0.1f, 0.0f, 0.0f), ty), Np.x);
                r = vadd(r, vscale_r(V3(0.0f, WALL_I, 0.0f), Np.y));
                r = vadd(r, vscale_r(vmix(V3(0.0f, 0.0f, WALL_I), V3(0.0f, 0.0f, WALL_I * 0.1f), ty), Np.z));
                r = vadd(r, vscale_r(vmix(V3(WALL_I, WALL_I, 0.0f), V3(WALL_I * 0.1f, WALL_I * 0.1f, 0.0f), ty), Nn.x));
                r = vadd(r, vscale_r(V3(0.0f, WALL_I, WALL_I), Nn.y));
                r = vadd(r, vscale_r(vmix(V3(WALL_I, 0.0f, WALL_I), V3(WALL_I * 0.1f, 0.0f, WALL_I * 0.1f), ty), Nn.z));
                return r;
            }
            default: { /* modes 0, 1, 3 and others */
                v3 a = vmul(m, V3(0.01f, 0.02f, 0.03f));
                return vadd(vsplat(0.0f), vsplat((a.x + a.y) + a.z));
            }
        }
    }
    return dir;
}

/* cp_main — raycast.comp.wgsl:60-68 for one pixel. */
static void shade_pixel(const orc_view *v, const orc_state *s, uint32_t gx, uint32_t gy,
                        uint32_t width, uint8_t *rgba, orc_hit *hits, orc_stats *stats) {
    float px = (float)gx + 0.001f, py = (float)gy + 0.001f;
    v3 r = V3((px * s->u[0] + py * s->mv[0]) + s->wp[0], (px * s->u[1] + py * s->mv[1]) + s->wp[1],
              (px * s->u[2] + py * s->mv[2]) + s->wp[2]);
    v3 dir = vnormalize(r);
    v3 eye = V3(s->eye[0], s->eye[1], s->eye[2]);
    Ctx c;
    memset(&c, 0, sizeof(c));
    c.v = v;
    c.s = s;
    HDDAout prim;
    v3 col = ray_trace(&c, eye, dir, &prim);
    uint64_t pix = (uint64_t)gy * width + gx;
    rgba[4 * pix + 0] = unorm8(col.x);
    rgba[4 * pix + 1] = unorm8(col.y);
    rgba[4 * pix + 2] = unorm8(col.z);
    rgba[4 * pix + 3] = unorm8(1.0f);
    if (hits) {
        orc_hit *h = &hits[pix];
        h->p[0] = prim.p.x; h->p[1] = prim.p.y; h->p[2] = prim.p.z;
        v3 d = vsub(prim.p, eye);
        h->t = vdot(d, dir);
        h->node = prim.leaf.np ? prim.leaf.par[prim.leaf.np - 1].idx : 0xFFFFFFFFu;
        h->info = prim.state | (prim.leaf.np << 2) | ((uint32_t)prim.mask[0] << 4) |
                  ((uint32_t)prim.mask[1] << 5) | ((uint32_t)prim.mask[2] << 6) | (prim.i << 8);
        h->shadow = c.shadow_traced ? (1u | (c.shadow_state << 1) | (c.shadow_steps << 8)) : 0u;
        h->reserved = 0;
        if (s->render_mode[0] == 5u) {  /* zero-crossing: found | sample index << 8, t* bits */
            h->shadow = c.surf_found ? (1u | (c.surf_k << 8)) : 0u;
            uint32_t tb;
            float tsv = c.surf_found ? c.surf_t : NAN;
            memcpy(&tb, &tsv, 4);
            h->reserved = c.surf_found ? tb : 0x7FC00000u;
        }
    }
    if (stats) {
        orc_stats *st = &stats[pix];
        st->steps = prim.i;
        st->bytes = prim.bytes;
        st->shadow_steps = c.shadow_traced ? c.shadow_steps : 0;
        st->shadow_bytes = c.shadow_traced ? c.shadow_bytes : 0;
        st->grazing = prim.grazing;
    }
}

typedef struct {
    const orc_view *v;
    const orc_state *s;
    uint32_t width, tiles_x;
    uint64_t tile_begin, tile_end;
    const uint64_t *list; /* optional: tile indices list[tile_begin..tile_end) */
    uint8_t *rgba;
    orc_hit *hits;
    orc_stats *stats;
    atomic_ullong next;
} Job;

static void *worker(void *arg) {
    Job *j = (Job *)arg;
    for (;;) {
        uint64_t k = atomic_fetch_add(&j->next, 1) + j->tile_begin;
        if (k >= j->tile_end) break;
        uint64_t tile = j->list ? j->list[k] : k;
        uint32_t tx = (uint32_t)(tile % j->tiles_x), ty = (uint32_t)(tile / j->tiles_x);
        for (uint32_t ly = 0; ly < 4; ly++)
            for (uint32_t lx = 0; lx < 8; lx++)
                shade_pixel(j->v, j->s, tx * 8 + lx, ty * 4 + ly, j->width, j->rgba, j->hits, j->stats);
    }
    return NULL;
}

static void run_job(Job *j, int nthreads) {
    if (nthreads <= 1) {
        worker(j);
        return;
    }
    pthread_t *th = malloc(sizeof(pthread_t) * (size_t)nthreads);
    for (int i = 0; i < nthreads; i++) pthread_create(&th[i], NULL, worker, j);
    for (int i = 0; i < nthreads; i++) pthread_join(th[i], NULL);
    free(th);
}

int orc_render_tiles(const orc_view *v, const orc_state *s, uint32_t width, uint32_t height,
                     uint64_t tile_begin, uint64_t tile_end, uint8_t *rgba, orc_hit *hits,
                     orc_stats *stats, int nthreads) {
    uint32_t tiles_x = width / 8, tiles_y = height / 4;
    uint64_t ntiles = (uint64_t)tiles_x * tiles_y;
    if (tile_end > ntiles) tile_end = ntiles;
    if (tile_begin >= tile_end) return 0;
    Job j;
    j.v = v; j.s = s; j.width = width; j.tiles_x = tiles_x;
    j.tile_begin = tile_begin; j.tile_end = tile_end; j.list = NULL;
    j.rgba = rgba; j.hits = hits; j.stats = stats;
    atomic_init(&j.next, 0);
    run_job(&j, nthreads);
    return 0;
}

int orc_render_tile_list(const orc_view *v, const orc_state *s, uint32_t width, uint32_t height,
                         const uint64_t *tiles, uint64_t ntiles, uint8_t *rgba, orc_hit *hits,
                         orc_stats *stats, int nthreads) {
    uint64_t total = (uint64_t)(width / 8) * (height / 4);
    for (uint64_t i = 0; i < ntiles; i++)
        if (tiles[i] >= total) return 1;
    Job j;
    j.v = v; j.s = s; j.width = width; j.tiles_x = width / 8;
    j.tile_begin = 0; j.tile_end = ntiles; j.list = tiles;
    j.rgba = rgba; j.hits = hits; j.stats = stats;
    atomic_init(&j.next, 0);
    run_job(&j, nthreads);
    return 0;
}

int orc_render(const orc_view *v, const orc_state *s, uint32_t width, uint32_t height,
               uint8_t *rgba, orc_hit *hits, orc_stats *stats, int nthreads) {
    return orc_render_tiles(v, s, width, height, 0, UINT64_MAX, rgba, hits, stats, nthreads);
}

/* ------------------------------------------------------------------------ */
/* Synthetic workloads. The reference reads its grids from .vdb files and has */
/* no generator; these are the benchmark's seeded stand-ins, stated here once */
/* more so that a CPU run (the reference arm of the benchmark, the parity     */
/* tests) can build its grid, cameras and uniforms without the product:       */
/*   splitmix64 (Steele, Lea & Flood 2014) as the seeded stream;              */
/*   narrow-band spheres: voxel ijk active iff |min_s(|ijk - c_s| - r_s)| <   */
/*     band, in double precision, set through set_voxel (vdb345.rs:26-66);    */
/*   3-octave value noise on the leaf lattice, thresholded to an occupancy;   */
/*   orbit eyes uniform on the sphere with |y| <= 0.9 radius.                 */
/* ------------------------------------------------------------------------ */
static uint64_t sm64_next(uint64_t *s) {
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double sm64_uniform(uint64_t *s) { return (double)(sm64_next(s) >> 11) * 0x1.0p-53; }
static uint64_t hash2(uint64_t a, uint64_t b) {
    uint64_t s = (a * 0xD6E8FEB86659FD93ull) ^ (b + 0x632BE59BD9B4E019ull);
    return sm64_next(&s);
}

/* Sun defaults of the reference app (egui_dev.rs:355-368): glam's
 * Vec3::normalize is v * (1 / sqrt((x*x + y*y) + z*z)). */
void orc_sun_default(float dir[3], float color[3], float *intensity) {
    const float v[3] = {1.0f, -1.0f, 0.5f};
    const float r = 1.0f / sqrtf((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
    for (int i = 0; i < 3; i++) dir[i] = v[i] * r;
    color[0] = 255.0f / 255.0f;
    color[1] = 210.0f / 255.0f;
    color[2] = 160.0f / 255.0f;
    *intensity = 1.0f;
}

void orc_sphere_list(uint32_t count, float rmin, float rmax, float lo, float hi, uint64_t seed,
                     double *out) {
    uint64_t s = seed;
    const float span = hi - lo, rspan = rmax - rmin; /* single-precision differences */
    for (uint32_t i = 0; i < count; i++) { /* per sphere: cx, cy, cz, then r */
        for (int a = 0; a < 3; a++) out[4 * i + a] = (double)lo + (double)span * sm64_uniform(&s);
        out[4 * i + 3] = (double)rmin + (double)rspan * sm64_uniform(&s);
    }
}

static double sphere_dist(const double *q, int32_t x, int32_t y, int32_t z) {
    const double dx = (double)x - q[0], dy = (double)y - q[1], dz = (double)z - q[2];
    return sqrt(dx * dx + dy * dy + dz * dz) - q[3];
}

/* Every voxel whose |signed distance to the union| is below band becomes active.
 * A voxel can only be active through a sphere whose shell (|d_s| < band) holds it,
 * so each sphere's bounding box is scanned for its own shell voxels, and for those
 * the union distance is taken over every sphere whose box (c +- (r + band)) covers
 * a 64-voxel cell around it. Returns 0, or 1 when an allocation fails. */
int orc_gen_spheres(orc_tree *t, const double *sph, uint32_t count, double band) {
    if (!count) return 0;
    enum { C = 64 };
    double blo[3] = {INFINITY, INFINITY, INFINITY}, bhi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = 0; i < count; i++)
        for (int a = 0; a < 3; a++) {
            blo[a] = fmin(blo[a], floor(sph[4 * i + a] - sph[4 * i + 3] - band));
            bhi[a] = fmax(bhi[a], ceil(sph[4 * i + a] + sph[4 * i + 3] + band));
        }
    int64_t c0[3], nc[3];
    for (int a = 0; a < 3; a++) {
        c0[a] = (int64_t)floor(blo[a] / C);
        nc[a] = (int64_t)floor(bhi[a] / C) - c0[a] + 1;
    }
    const size_t ncell = (size_t)(nc[0] * nc[1] * nc[2]);
    /* Cell lists in CSR form: start[c] .. start[c + 1] index ids. */
    size_t *start = calloc(ncell + 1, sizeof(size_t));
    if (!start) return 1;
    uint32_t *ids = NULL;
    for (int pass = 0; pass < 2; pass++) {
        if (pass == 1) {
            for (size_t c = 0; c < ncell; c++) start[c + 1] += start[c];
            ids = malloc(sizeof(uint32_t) * (start[ncell] ? start[ncell] : 1));
            if (!ids) { free(start); return 1; }
        }
        for (uint32_t i = 0; i < count; i++) {
            int64_t lc[3], hc[3];
            for (int a = 0; a < 3; a++) {
                lc[a] = (int64_t)floor(floor(sph[4 * i + a] - sph[4 * i + 3] - band) / C) - c0[a];
                hc[a] = (int64_t)floor(ceil(sph[4 * i + a] + sph[4 * i + 3] + band) / C) - c0[a];
            }
            for (int64_t x = lc[0]; x <= hc[0]; x++)
                for (int64_t y = lc[1]; y <= hc[1]; y++)
                    for (int64_t z = lc[2]; z <= hc[2]; z++) {
                        const size_t c = (size_t)((x * nc[1] + y) * nc[2] + z);
                        if (pass == 0) start[c + 1]++;
                        else ids[start[c]++] = i; /* advances start[c] to cell c's end */
                    }
        }
    }
    /* After the fill start[c] is the end of cell c's list, so cell c spans
     * [c ? start[c - 1] : 0, start[c]). */
    for (uint32_t i = 0; i < count; i++) {
        const double *q = sph + 4 * i;
        int32_t lv[3], hv[3];
        for (int a = 0; a < 3; a++) {
            lv[a] = (int32_t)floor(q[a] - q[3] - band);
            hv[a] = (int32_t)ceil(q[a] + q[3] + band);
        }
        for (int32_t x = lv[0]; x <= hv[0]; x++)
            for (int32_t y = lv[1]; y <= hv[1]; y++)
                for (int32_t z = lv[2]; z <= hv[2]; z++) {
                    if (!(fabs(sphere_dist(q, x, y, z)) < band)) continue;
                    const int64_t cx = (int64_t)floor((double)x / C) - c0[0];
                    const int64_t cy = (int64_t)floor((double)y / C) - c0[1];
                    const int64_t cz = (int64_t)floor((double)z / C) - c0[2];
                    const size_t c = (size_t)((cx * nc[1] + cy) * nc[2] + cz);
                    double d = INFINITY;
                    for (size_t k = c ? start[c - 1] : 0; k < start[c]; k++)
                        d = fmin(d, sphere_dist(sph + 4 * ids[k], x, y, z));
                    if (fabs(d) < band) {
                        const int32_t p[3] = {x, y, z};
                        orc_set_voxel(t, p, 1);
                    }
                }
    }
    free(ids);
    free(start);
    return 0;
}

/* Level-set values of a sphere union for every voxel of every leaf of t (DFS leaf order,
 * voxel x<<6 | y<<3 | z): the signed distance min_s(|ijk - c_s| - r_s) clamped to
 * [-band, band], as a narrow-band level set stores it. The minimum runs over the spheres
 * whose box c +- (r + band) meets the leaf; any other sphere is farther than band from
 * every voxel of the leaf, so it cannot change the clamped value. 0, or 1 (no memory). */
int orc_gen_spheres_values(const orc_tree *t, const double *sph, uint32_t count, double band, float *out) {
    uint32_t *ids = malloc(sizeof(uint32_t) * (count ? count : 1));
    if (!ids) return 1;
    size_t leaf = 0;
    for (size_t r = 0; r < t->nroots; r++) {
        const ON5 *n5 = t->n5[t->roots[r].n5];
        const int32_t *key = t->roots[r].key;
        for (int o5 = 0; o5 < 32768; o5++) {
            if (n5->child[o5] < 0) continue;
            const ON4 *n4 = t->n4[n5->child[o5]];
            uint32_t c5[3];
            orc_offset_to_child((uint64_t)o5, 5, c5);
            for (int o4 = 0; o4 < 4096; o4++) {
                if (n4->child[o4] < 0) continue;
                uint32_t c4[3];
                orc_offset_to_child((uint64_t)o4, 4, c4);
                int32_t org[3];
                for (int a = 0; a < 3; a++) org[a] = key[a] + (int32_t)c5[a] * 128 + (int32_t)c4[a] * 8;
                uint32_t nid = 0;
                for (uint32_t i = 0; i < count; i++) {
                    const double *q = sph + 4 * i;
                    int meets = 1;
                    for (int a = 0; a < 3 && meets; a++)
                        meets = floor(q[a] - q[3] - band) <= (double)(org[a] + 7) &&
                                ceil(q[a] + q[3] + band) >= (double)org[a];
                    if (meets) ids[nid++] = i;
                }
                for (int v = 0; v < 512; v++) {
                    const int32_t x = org[0] + (v >> 6), y = org[1] + ((v >> 3) & 7), z = org[2] + (v & 7);
                    double d = INFINITY;
                    for (uint32_t k = 0; k < nid; k++) d = fmin(d, sphere_dist(sph + 4 * ids[k], x, y, z));
                    out[leaf * 512 + (size_t)v] = (float)fmin(band, fmax(-band, d));
                }
                leaf++;
            }
        }
    }
    free(ids);
    return 0;
}

/* set_voxel(p, 1) for every set bit of a leaf's 512-bit mask (bit x<<6 | y<<3 | z):
 * the nodes on the way are created and marked as set_voxel (vdb345.rs:26-66) does for
 * the leaf's first voxel, then the leaf's value bits are or-ed in. */
void orc_set_leaf(orc_tree *t, const int32_t origin[3], const uint64_t mask[8]) {
    int first = -1;
    for (int w = 0; w < 8 && first < 0; w++)
        if (mask[w]) first = 64 * w + __builtin_ctzll(mask[w]);
    if (first < 0) return;
    const int32_t p[3] = {origin[0] + (first >> 6), origin[1] + ((first >> 3) & 7), origin[2] + (first & 7)};
    orc_set_voxel(t, p, 1);
    int32_t key[3];
    orc_global_to_node(p, 12, key);
    const ON5 *n5 = t->n5[t->roots[root_find(t, key, NULL)].n5];
    const ON4 *n4 = t->n4[n5->child[orc_global_to_offset(p, 5, 12)]];
    ON3 *n3 = t->n3[n4->child[orc_global_to_offset(p, 4, 7)]];
    for (int v = 0; v < 512; v++) {
        if (!((mask[v >> 6] >> (v & 63)) & 1)) continue;
        n3->val[v >> 6] |= 1ull << (v & 63);
        n3->is_value[v] = 1;
        n3->value[v] = 1;
    }
}

/* Value noise: octave k has 8 << k cells over the n-leaf lattice; corner values
 * are (hash >> 40) * 2^-24 in [0, 1); smoothstep weights; amplitudes 1, 1/2, 1/4.
 * All arithmetic single precision except the corner draw. */
static float noise_at(float *const corners[3], int n, int lx, int ly, int lz) {
    float sum = 0.0f, amp = 1.0f;
    for (int k = 0; k < 3; k++) {
        const int cells = 8 << k, c = cells + 1;
        const float scale = (float)cells / (float)n;
        const float u[3] = {((float)lx + 0.5f) * scale, ((float)ly + 0.5f) * scale, ((float)lz + 0.5f) * scale};
        int i0[3];
        float w[3];
        for (int a = 0; a < 3; a++) {
            int fl = (int)floorf(u[a]);
            i0[a] = fl < cells - 1 ? fl : cells - 1;
            const float f = u[a] - (float)i0[a];
            w[a] = f * f * (3.0f - 2.0f * f);
        }
#define G(dx, dy, dz) corners[k][((size_t)(i0[0] + (dx)) * c + (size_t)(i0[1] + (dy))) * c + (size_t)(i0[2] + (dz))]
        const float x00 = G(0, 0, 0) + w[0] * (G(1, 0, 0) - G(0, 0, 0));
        const float x10 = G(0, 1, 0) + w[0] * (G(1, 1, 0) - G(0, 1, 0));
        const float x01 = G(0, 0, 1) + w[0] * (G(1, 0, 1) - G(0, 0, 1));
        const float x11 = G(0, 1, 1) + w[0] * (G(1, 1, 1) - G(0, 1, 1));
#undef G
        const float y0 = x00 + w[1] * (x10 - x00), y1 = x01 + w[1] * (x11 - x01);
        sum += amp * (y0 + w[2] * (y1 - y0));
        amp *= 0.5f;
    }
    return sum;
}

/* Noise value of every lattice leaf, x-major; x-slabs spread over threads (each value
 * depends only on its own coordinates). */
typedef struct {
    float *const *corners;
    float *val;
    int n;
    atomic_int next;
} NoiseJob;
static void *noise_worker(void *arg) {
    NoiseJob *j = (NoiseJob *)arg;
    for (;;) {
        const int x = atomic_fetch_add(&j->next, 1);
        if (x >= j->n) break;
        for (int y = 0; y < j->n; y++)
            for (int z = 0; z < j->n; z++)
                j->val[((size_t)x * j->n + y) * j->n + z] = noise_at(j->corners, j->n, x, y, z);
    }
    return NULL;
}
static void noise_fill(float *const corners[3], int n, float *val) {
    NoiseJob j = {corners, val, n, 0};
    enum { T = 16 };
    pthread_t th[T];
    int started = 0;
    for (; started < T; started++)
        if (pthread_create(&th[started], NULL, noise_worker, &j) != 0) break;
    noise_worker(&j);
    for (int i = 0; i < started; i++) pthread_join(th[i], NULL);
}

/* k-th smallest of a[0..n) (0-based); reorders a. Hoare partition, middle pivot. */
static float select_kth(float *a, size_t n, size_t k) {
    size_t lo = 0, hi = n - 1;
    while (lo < hi) {
        const float piv = a[lo + (hi - lo) / 2];
        size_t i = lo, j = hi;
        while (i <= j) {
            while (a[i] < piv) i++;
            while (a[j] > piv) j--;
            if (i <= j) {
                float tmp = a[i]; a[i] = a[j]; a[j] = tmp;
                i++;
                if (j == 0) break;
                j--;
            }
        }
        if (k <= j) hi = j;
        else if (k >= i) lo = i;
        else return a[k];
    }
    return a[k];
}

/* Leaves of [lo, lo + extent)^3 whose noise value exceeds the value with exactly
 * round(occupancy * leaves) leaves above it; voxels of a kept leaf active with
 * probability p_voxel (p = 0.5: the raw hash bits). Only leaves whose origin lies in
 * [box_lo, box_hi) on every axis are set (the whole domain when box_lo >= box_hi).
 * Returns the number of leaves kept in the whole domain, or -1 on a bad argument or
 * a failed allocation. */
int64_t orc_gen_noise_leaves(orc_tree *t, int32_t lo, uint32_t extent, double occupancy, double p_voxel,
                             uint64_t seed, int32_t box_lo, int32_t box_hi) {
    if (extent < 64 || (extent & 7) || !(occupancy > 0.0 && occupancy < 1.0) || (lo & 7)) return -1;
    const int n = (int)(extent / 8);
    const size_t total = (size_t)n * n * n;
    float *corners[3] = {NULL, NULL, NULL};
    for (int k = 0; k < 3; k++) {
        const int c = (8 << k) + 1;
        corners[k] = malloc(sizeof(float) * (size_t)c * c * c);
        if (!corners[k]) goto oom;
        for (int x = 0; x < c; x++)
            for (int y = 0; y < c; y++)
                for (int z = 0; z < c; z++) {
                    uint64_t h = hash2(seed ^ (0x1000193ull * (uint64_t)(k + 1)),
                                       ((uint64_t)x << 42) | ((uint64_t)y << 21) | (uint64_t)z);
                    corners[k][((size_t)x * c + y) * c + z] = (float)((double)(h >> 40) * 0x1.0p-24);
                }
    }
    float *val = malloc(sizeof(float) * total), *tmp = malloc(sizeof(float) * total);
    if (!val || !tmp) { free(val); free(tmp); goto oom; }
    noise_fill(corners, n, val);
    const size_t keep = (size_t)llround(occupancy * (double)total);
    memcpy(tmp, val, sizeof(float) * total);
    const float thr = select_kth(tmp, total, total - keep - (keep < total ? 1 : 0));
    free(tmp);
    int64_t kept = 0;
    for (size_t i = 0; i < total; i++) {
        if (!(val[i] > thr)) continue;
        kept++;
        const int32_t o[3] = {lo + 8 * (int32_t)(i / ((size_t)n * n)), lo + 8 * (int32_t)((i / n) % n),
                              lo + 8 * (int32_t)(i % n)};
        if (box_lo < box_hi && (o[0] < box_lo || o[0] >= box_hi || o[1] < box_lo || o[1] >= box_hi ||
                                o[2] < box_lo || o[2] >= box_hi))
            continue;
        uint64_t m[8];
        for (int w = 0; w < 8; w++) {
            const uint64_t h = hash2(seed ^ 0xA5A5A5A5DEADBEEFull, (uint64_t)i * 8 + (uint64_t)w);
            if (p_voxel == 0.5) {
                m[w] = h;
            } else {
                uint64_t s = h, b = 0;
                for (int k = 0; k < 64; k++)
                    if (sm64_uniform(&s) < p_voxel) b |= 1ull << k;
                m[w] = b;
            }
        }
        orc_set_leaf(t, o, m);
    }
    free(val);
    for (int k = 0; k < 3; k++) free(corners[k]);
    return kept;
oom:
    for (int k = 0; k < 3; k++) free(corners[k]);
    return -1;
}

void orc_orbit_eyes(uint32_t count, float radius, uint64_t seed, float *eyes) {
    uint64_t s = seed;
    for (uint32_t i = 0; i < count; i++) {
        double y;
        do {
            y = 2.0 * sm64_uniform(&s) - 1.0;
        } while (fabs(y) > 0.9);
        const double phi = 2.0 * 3.14159265358979323846 * sm64_uniform(&s);
        const double r = sqrt(1.0 - y * y);
        eyes[3 * i + 0] = (float)(radius * r * cos(phi));
        eyes[3 * i + 1] = (float)(radius * y);
        eyes[3 * i + 2] = (float)(radius * r * sin(phi));
    }
}
