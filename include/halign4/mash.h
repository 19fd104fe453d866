// mash.h - drop-in for HAlign-4's include/mash.h: the MinHash sketches of
// multi-reference selection, implemented over the GB300 C ABI
// (include/halign_gb300.h) by libhalign4_dropin.so.  sketchFromSequence runs
// on the GPU (hg_sketch_batch); jaccard, the distance / identity conversions
// and the sorted intersection count are arithmetic on the caller's sketches.
// The Bloom-filter helpers of the reference header (filterFromSketch and the
// filter form of jaccard) serve no step of the align-to-center path and are
// not part of this surface.
#ifndef HALIGN4_MASH_H
#define HALIGN4_MASH_H

#include <array>
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "hash.h"

namespace mash
{
    namespace detail
    {
        // 2-bit base codes: A/a 0, C/c 1, G/g 2, T/t and U/u 3, every other byte 4
        constexpr std::array<std::uint8_t, 256> make_nt4()
        {
            std::array<std::uint8_t, 256> t{};
            for (auto& v : t) v = 4;
            const char* up = "ACGT";
            const char* lo = "acgt";
            for (int i = 0; i < 4; ++i) {
                t[static_cast<unsigned char>(up[i])] = static_cast<std::uint8_t>(i);
                t[static_cast<unsigned char>(lo[i])] = static_cast<std::uint8_t>(i);
            }
            t[static_cast<unsigned char>('U')] = 3;
            t[static_cast<unsigned char>('u')] = 3;
            return t;
        }
    }  // namespace detail

    inline constexpr std::array<std::uint8_t, 256> nt4_table = detail::make_nt4();

    struct Sketch
    {
        std::size_t k = 0;
        bool noncanonical = true;
        std::vector<hash_t> hashes;  // ascending, distinct

        std::size_t size() const noexcept { return hashes.size(); }
        bool empty() const noexcept { return hashes.empty(); }
    };
    using Sketches = std::vector<Sketch>;

    // The sketch_size smallest distinct getHash2bit hashes (XXH3-64 of the 8
    // big-endian bytes of the 2-bit k-mer code, seeded) of the valid k-mers of
    // seq, ascending; empty for k = 0, k > 32, sketch_size = 0 or a sequence
    // shorter than k.  Throws std::invalid_argument above HG_SKETCH_MAX
    // hashes, std::runtime_error on a device error.
    Sketch sketchFromSequence(const std::string& seq,
                              std::size_t k,
                              std::size_t sketch_size,
                              bool noncanonical = true,
                              int seed = 0);

    // |a & b| / min(|a|, |b|) over the two sorted sketches; 1 when both are
    // empty, 0 when one is.  Throws std::invalid_argument when k differs.
    double jaccard(const Sketch& a, const Sketch& b);

    // -ln(2j / (1 + j)) / k (infinity for j <= 0, 0 for j >= 1)
    double mashDistanceFromJaccard(double j, std::size_t k);

    // (2j / (1 + j))^(1/k) clamped to [0, 1]
    double aniFromJaccard(double j, std::size_t k);

    // exp(-d) clamped to [0, 1] (0 for a non-finite d, 1 for d <= 0)
    double aniFromMashDistance(double d);

    std::size_t intersectionSizeSortedUnique(const std::vector<hash_t>& a,
                                             const std::vector<hash_t>& b) noexcept;

}  // namespace mash

#endif  // HALIGN4_MASH_H
