// Snappy raw-format codec (host) used for the outlier bitmaps of buff-major
// columns.  See buff_snappy.cpp.
#pragma once

#include <stddef.h>
#include <stdint.h>

#include <vector>

namespace buffsnappy {

std::vector<uint8_t> compress(const uint8_t *in, size_t n);
bool uncompressed_length(const uint8_t *in, size_t n, size_t *len);
bool decompress(const uint8_t *in, size_t n, std::vector<uint8_t> &out);

}  // namespace buffsnappy
