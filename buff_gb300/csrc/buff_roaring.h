// Roaring bitmaps in the portable serialized format (host), used for the
// outlier row sets of the RAPG byte_residue images.  See buff_roaring.cpp.
#pragma once

#include <stddef.h>
#include <stdint.h>

#include <vector>

namespace buffroaring {

// The set bits of `words` (BitVec<u32> layout, `n` bits) as a bitmap built by
// ascending adds followed by run optimization, serialized.
std::vector<uint8_t> serialize(const uint32_t *words, uint32_t n);
// The rows of a serialized bitmap, ascending; false when `b` is not a
// well-formed portable image.
bool parse(const uint8_t *b, size_t len, std::vector<uint32_t> &rows);

}  // namespace buffroaring
