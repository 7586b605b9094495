// inflate.cpp — a DEFLATE decoder (RFC 1951) inside the zlib format (RFC 1950).
//
// Huffman codes are canonical (RFC 1951 section 3.2.2): a code is decoded bit by bit
// against the number of codes of each length, which needs no lookup tables beyond
// the per-length counts and the symbols in code order. Stored, fixed-Huffman and
// dynamic-Huffman blocks are supported; preset dictionaries are not (OpenVDB
// writes none).

#include "inflate.h"

#include <cstring>

namespace wx {
namespace {

constexpr int kMaxBits = 15;

struct Bits {
    const uint8_t *p;
    size_t n, pos = 0;
    uint32_t buf = 0;
    int cnt = 0;
    bool eof = false;
    uint32_t get(int k) {  // k <= 16 bits, least significant first
        while (cnt < k) {
            if (pos >= n) {
                eof = true;
                return 0;
            }
            buf |= (uint32_t)p[pos++] << cnt;
            cnt += 8;
        }
        const uint32_t v = buf & ((1u << k) - 1u);
        buf >>= k;
        cnt -= k;
        return v;
    }
    void align() {  // drop the bits left in the current byte
        buf = 0;
        cnt = 0;
    }
};

struct Huffman {
    uint16_t count[kMaxBits + 1];
    uint16_t symbol[288];
    // Builds the canonical code of n symbols with the given lengths (0 = unused).
    // Returns false for an over-subscribed set of lengths.
    bool build(const uint8_t *len, int n) {
        memset(count, 0, sizeof count);
        for (int s = 0; s < n; s++) count[len[s]]++;
        count[0] = 0;
        int left = 1;
        for (int l = 1; l <= kMaxBits; l++) {
            left = left * 2 - count[l];
            if (left < 0) return false;
        }
        uint16_t offs[kMaxBits + 2];
        offs[1] = 0;
        for (int l = 1; l <= kMaxBits; l++) offs[l + 1] = (uint16_t)(offs[l] + count[l]);
        for (int s = 0; s < n; s++)
            if (len[s]) symbol[offs[len[s]]++] = (uint16_t)s;
        return true;
    }
    int decode(Bits &b) const {  // -1 on a code that is not in the table or at the end of input
        int code = 0, first = 0, index = 0;
        for (int l = 1; l <= kMaxBits; l++) {
            code |= (int)b.get(1);
            if (b.eof) return -1;
            const int c = count[l];
            if (code - first < c) return symbol[index + (code - first)];
            index += c;
            first = (first + c) << 1;
            code <<= 1;
        }
        return -1;
    }
};

// Length symbols 257..285 and distance symbols 0..29: base value and extra bits.
constexpr uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                                   31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
constexpr uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
constexpr uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                    193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
constexpr uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
// Order in which the code-length code's lengths are stored (RFC 1951 section 3.2.7).
constexpr uint8_t kClOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

struct Out {
    uint8_t *d;
    size_t cap, n = 0;
    bool full() const { return n >= cap; }
};

// Decodes one Huffman-coded block. 0 = block done, 1 = output full, -1 = error.
int codes(Bits &b, Out &o, const Huffman &lit, const Huffman &dist, std::string *err) {
    for (;;) {
        const int s = lit.decode(b);
        if (s < 0) {
            *err = "zlib: invalid literal/length code";
            return -1;
        }
        if (s < 256) {
            if (o.full()) return 1;
            o.d[o.n++] = (uint8_t)s;
            continue;
        }
        if (s == 256) return 0;
        if (s > 285) {
            *err = "zlib: invalid length symbol";
            return -1;
        }
        const int li = s - 257;
        const size_t len = kLenBase[li] + b.get(kLenExtra[li]);
        const int ds = dist.decode(b);
        if (ds < 0 || ds > 29) {
            *err = "zlib: invalid distance code";
            return -1;
        }
        const size_t d = kDistBase[ds] + b.get(kDistExtra[ds]);
        if (b.eof) {
            *err = "zlib: truncated stream";
            return -1;
        }
        if (d > o.n) {
            *err = "zlib: distance beyond the output";
            return -1;
        }
        for (size_t k = 0; k < len; k++) {  // byte by byte: the copy may overlap itself
            if (o.full()) return 1;
            o.d[o.n] = o.d[o.n - d];
            o.n++;
        }
    }
}

uint32_t adler32(const uint8_t *p, size_t n) {
    uint32_t a = 1, b = 0;
    for (size_t i = 0; i < n; i++) {
        a = (a + p[i]) % 65521u;
        b = (b + a) % 65521u;
    }
    return (b << 16) | a;
}

}  // namespace

long long zlib_inflate(const uint8_t *src, size_t src_len, uint8_t *dst, size_t dst_len, std::string *err) {
    if (src_len < 2) {
        *err = "zlib: truncated header";
        return -1;
    }
    const uint32_t cmf = src[0], flg = src[1];
    if ((cmf & 15u) != 8u || (cmf >> 4) > 7u || ((cmf << 8) | flg) % 31u != 0u) {
        *err = "zlib: not a deflate stream";
        return -1;
    }
    if (flg & 0x20u) {
        *err = "zlib: preset dictionaries are not supported";
        return -1;
    }
    Bits b{src + 2, src_len - 2};
    Out o{dst, dst_len};
    static Huffman fixed_lit, fixed_dist;
    static const bool fixed_ok = [] {
        uint8_t l[288];
        for (int i = 0; i < 144; i++) l[i] = 8;
        for (int i = 144; i < 256; i++) l[i] = 9;
        for (int i = 256; i < 280; i++) l[i] = 7;
        for (int i = 280; i < 288; i++) l[i] = 8;
        uint8_t d[30];
        memset(d, 5, sizeof d);
        return fixed_lit.build(l, 288) && fixed_dist.build(d, 30);
    }();
    (void)fixed_ok;
    bool last = false;
    while (!last) {
        last = b.get(1) != 0;
        const uint32_t type = b.get(2);
        if (b.eof) {
            *err = "zlib: truncated stream";
            return -1;
        }
        if (type == 0) {  // stored
            b.align();
            if (b.pos + 4 > b.n) {
                *err = "zlib: truncated stored block";
                return -1;
            }
            const uint32_t len = b.p[b.pos] | (b.p[b.pos + 1] << 8), nlen = b.p[b.pos + 2] | (b.p[b.pos + 3] << 8);
            b.pos += 4;
            if ((len ^ 0xFFFFu) != nlen) {
                *err = "zlib: stored block length check failed";
                return -1;
            }
            if (b.pos + len > b.n) {
                *err = "zlib: truncated stored block";
                return -1;
            }
            const size_t take = len < o.cap - o.n ? len : o.cap - o.n;
            memcpy(o.d + o.n, b.p + b.pos, take);
            o.n += take;
            b.pos += len;
            if (o.full() && take < len) return (long long)o.n;
            continue;
        }
        int rc;
        if (type == 1) {
            rc = codes(b, o, fixed_lit, fixed_dist, err);
        } else if (type == 2) {
            const int hlit = (int)b.get(5) + 257, hdist = (int)b.get(5) + 1, hclen = (int)b.get(4) + 4;
            if (b.eof || hlit > 286 || hdist > 30) {
                *err = "zlib: bad dynamic block header";
                return -1;
            }
            uint8_t cl[19] = {0};
            for (int i = 0; i < hclen; i++) cl[kClOrder[i]] = (uint8_t)b.get(3);
            Huffman clh;
            if (b.eof || !clh.build(cl, 19)) {
                *err = "zlib: bad code-length code";
                return -1;
            }
            uint8_t lens[286 + 30];
            int k = 0;
            while (k < hlit + hdist) {
                const int s = clh.decode(b);
                if (s < 0) {
                    *err = "zlib: bad code lengths";
                    return -1;
                }
                if (s < 16) {
                    lens[k++] = (uint8_t)s;
                    continue;
                }
                uint8_t v = 0;
                int rep;
                if (s == 16) {
                    if (k == 0) {
                        *err = "zlib: repeat with no previous length";
                        return -1;
                    }
                    v = lens[k - 1];
                    rep = 3 + (int)b.get(2);
                } else if (s == 17) {
                    rep = 3 + (int)b.get(3);
                } else {
                    rep = 11 + (int)b.get(7);
                }
                if (b.eof || k + rep > hlit + hdist) {
                    *err = "zlib: code lengths overflow";
                    return -1;
                }
                while (rep--) lens[k++] = v;
            }
            if (lens[256] == 0) {
                *err = "zlib: no end-of-block code";
                return -1;
            }
            Huffman lit, dist;
            if (!lit.build(lens, hlit) || !dist.build(lens + hlit, hdist)) {
                *err = "zlib: bad literal/length or distance code";
                return -1;
            }
            rc = codes(b, o, lit, dist, err);
        } else {
            *err = "zlib: invalid block type";
            return -1;
        }
        if (rc < 0) return -1;
        if (rc == 1) return (long long)o.n;  // output full: the rest is not needed
    }
    b.align();
    if (b.pos + 4 > b.n) {
        *err = "zlib: truncated checksum";
        return -1;
    }
    const uint32_t want = ((uint32_t)b.p[b.pos] << 24) | ((uint32_t)b.p[b.pos + 1] << 16) |
                          ((uint32_t)b.p[b.pos + 2] << 8) | b.p[b.pos + 3];
    if (adler32(dst, o.n) != want) {
        *err = "zlib: Adler-32 mismatch";
        return -1;
    }
    return (long long)o.n;
}

}  // namespace wx
