// zlib stream encoder for the PNG writer: RFC 1950 framing around an RFC 1951 deflate
// stream of LZ77 matches (hash chains over a 32 KB window, one step of lazy matching)
// in dynamic-Huffman blocks. The reference writes its images through libpng and zlib
// (src/bitmap.c:67-151); neither is on this image, so this is written from the RFCs.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

namespace illume {

std::vector<uint8_t> zlib_compress(const uint8_t* data, size_t n);

}  // namespace illume
