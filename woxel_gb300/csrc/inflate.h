// inflate.h — zlib stream decoding (RFC 1950 wrapper around RFC 1951 DEFLATE data)
// for the zip-compressed buffers of OpenVDB files.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>

namespace wx {

// Decodes the zlib stream src[0, src_len) into dst, stopping once dst_len bytes have
// been produced (as a reader that takes exactly the bytes it needs) or at the end of
// the stream, whose Adler-32 is then checked. Returns the number of bytes produced,
// or -1 with *err set when the stream is malformed or truncated.
long long zlib_inflate(const uint8_t *src, size_t src_len, uint8_t *dst, size_t dst_len, std::string *err);

}  // namespace wx
