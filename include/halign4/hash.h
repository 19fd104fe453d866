// hash.h - drop-in for HAlign-4's include/hash.h on the align-to-center path:
// the 64-bit hash word every seed record carries.  The byte-string hashes the
// reference declares next to it (getHash, getHash2bit) only feed the MinHash
// sketches of multi-reference selection and are not part of this surface.
#ifndef HALIGN4_HASH_H
#define HALIGN4_HASH_H

#include <cstdint>

using hash_t = std::uint64_t;

#endif  // HALIGN4_HASH_H
