// seed.h - drop-in for HAlign-4's include/seed.h: the seed-hit interface,
// the packed 16-byte minimizer hit, extractMinimizer and collect_anchors,
// implemented over the GB300 C ABI (include/halign_gb300.h) by
// libhalign4_dropin.so.  Both functions run on the GPU
// (hg_extract_minimizer, hg_collect_anchors).
#ifndef HALIGN4_SEED_H
#define HALIGN4_SEED_H

#include <cstddef>
#include <cstdint>
#include <string>
#include <type_traits>
#include <vector>

#include "anchor.h"
#include "hash.h"

namespace seed
{
    enum class SeedKind : std::uint8_t
    {
        minimizer = 0,
        syncmer = 1,
        strobemer = 2,
    };

    inline constexpr const char* seedKindToString(SeedKind k) noexcept
    {
        return k == SeedKind::minimizer ? "minimizer"
             : k == SeedKind::syncmer   ? "syncmer"
             : k == SeedKind::strobemer ? "strobemer"
                                        : "unknown";
    }

    // CRTP base of positioned seed hits: the derived type provides hash(),
    // pos(), rid(), strand() and span().  Ordering is by hash, then rid,
    // pos, strand (the order collect_anchors groups reference hits in).
    template <typename Derived>
    struct SeedHitBase
    {
        constexpr hash_t hash() const noexcept { return self().hash(); }
        constexpr std::uint32_t pos() const noexcept { return self().pos(); }
        constexpr std::uint32_t rid() const noexcept { return self().rid(); }
        constexpr bool strand() const noexcept { return self().strand(); }
        constexpr std::uint32_t span() const noexcept { return self().span(); }

        friend constexpr bool operator<(const SeedHitBase& a, const SeedHitBase& b) noexcept
        {
            if (a.hash() != b.hash()) return a.hash() < b.hash();
            if (a.rid() != b.rid()) return a.rid() < b.rid();
            if (a.pos() != b.pos()) return a.pos() < b.pos();
            return a.strand() < b.strand();
        }

        friend constexpr bool operator==(const SeedHitBase& a, const SeedHitBase& b) noexcept
        {
            return a.hash() == b.hash() && a.rid() == b.rid() && a.pos() == b.pos() && a.strand() == b.strand() &&
                   a.span() == b.span();
        }

    private:
        constexpr const Derived& self() const noexcept { return static_cast<const Derived&>(*this); }
    };

    template <typename T>
    struct has_position : std::false_type {};

    template <typename T>
    struct has_position_auto : std::is_base_of<SeedHitBase<T>, T> {};

    template <typename T>
    inline constexpr bool has_position_v = has_position<T>::value || has_position_auto<T>::value;

    template <typename SeedT>
    inline constexpr hash_t hash_value(const SeedT& s) noexcept { return s.hash(); }

    template <typename HitT>
    inline constexpr std::uint32_t get_pos(const HitT& h) noexcept { return h.pos(); }
    template <typename HitT>
    inline constexpr std::uint32_t get_rid(const HitT& h) noexcept { return h.rid(); }
    template <typename HitT>
    inline constexpr bool get_strand(const HitT& h) noexcept { return h.strand(); }
    template <typename HitT>
    inline constexpr std::uint32_t get_span(const HitT& h) noexcept { return h.span(); }

    struct HashOnlyLess
    {
        template <typename M>
        constexpr bool operator()(const M& a, const M& b) const noexcept { return hash_value(a) < hash_value(b); }
    };

    struct HashOnlyEqual
    {
        template <typename M>
        constexpr bool operator()(const M& a, const M& b) const noexcept { return hash_value(a) == hash_value(b); }
    };

}  // namespace seed

namespace minimizer
{
    // 2-bit nucleotide codes: A/a 0, C/c 1, G/g 2, T/t and U/u 3 (RNA), any other
    // byte 4 (the k-mer breaks there).
    inline constexpr std::uint8_t nt4_table[256] = {
        4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4,  //   0- 15
        4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4,  //  16- 31
        4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4,  //  32- 47
        4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4,  //  48- 63
        4, 0, 4, 1, 4, 4, 4, 2, 4, 4, 4, 4, 4, 4, 4, 4,  //  64- 79
        4, 4, 4, 4, 3, 3, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4,  //  80- 95
        4, 0, 4, 1, 4, 4, 4, 2, 4, 4, 4, 4, 4, 4, 4, 4,  //  96-111
        4, 4, 4, 4, 3, 3, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4,  // 112-127
        4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4,  // 128-143
        4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4,  // 144-159
        4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4,  // 160-175
        4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4,  // 176-191
        4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4,  // 192-207
        4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4,  // 208-223
        4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4,  // 224-239
        4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4  // 240-255
    };

    // One minimizer hit in 16 bytes: x = hash56 << 8 | span,
    // y = strand << 63 | rid (31 bits) << 32 | pos.
    struct MinimizerHit : public seed::SeedHitBase<MinimizerHit>
    {
        hash_t x{0};
        hash_t y{0};

        constexpr MinimizerHit() = default;
        constexpr MinimizerHit(hash_t x_, hash_t y_) : x(x_), y(y_) {}

        static constexpr hash_t pack_x(hash_t hash56, std::uint8_t span) noexcept
        {
            return (hash56 << 8) | static_cast<hash_t>(span);
        }
        static constexpr std::uint8_t span_from_x(hash_t x) noexcept { return static_cast<std::uint8_t>(x & 0xff); }
        static constexpr hash_t hash_from_x(hash_t x) noexcept { return x >> 8; }

        static constexpr hash_t pack_y(std::uint32_t pos, std::uint32_t rid, bool strand) noexcept
        {
            return (static_cast<hash_t>((rid & 0x7fffffffu) | (strand ? 0x80000000u : 0u)) << 32) | pos;
        }
        static constexpr std::uint32_t pos_from_y(hash_t y) noexcept { return static_cast<std::uint32_t>(y); }
        static constexpr std::uint32_t rid_with_strand_from_y(hash_t y) noexcept
        {
            return static_cast<std::uint32_t>(y >> 32);
        }
        static constexpr std::uint32_t rid_from_y(hash_t y) noexcept { return rid_with_strand_from_y(y) & 0x7fffffffu; }
        static constexpr bool strand_from_y(hash_t y) noexcept { return (y >> 63) != 0; }

        constexpr MinimizerHit(hash_t hash56, std::uint32_t pos, std::uint32_t rid, bool strand,
                               std::uint8_t span) noexcept
            : x(pack_x(hash56, span)), y(pack_y(pos, rid, strand))
        {
        }

        constexpr hash_t hash() const noexcept { return hash_from_x(x); }
        constexpr std::uint32_t pos() const noexcept { return pos_from_y(y); }
        constexpr std::uint32_t rid() const noexcept { return rid_from_y(y); }
        constexpr bool strand() const noexcept { return strand_from_y(y); }
        constexpr std::uint32_t span() const noexcept { return span_from_x(x); }
    };

    static_assert(sizeof(MinimizerHit) == 16, "MinimizerHit is two 64-bit words");
    using MinimizerHits = std::vector<MinimizerHit>;

    // Minimizer hits of `seq` in scan order (k-mer size k <= 31, window w in
    // k-mers; non_canonical: forward k-mers only).  Runs on the GPU.
    MinimizerHits extractMinimizer(const std::string& seq, std::size_t k, std::size_t w, bool non_canonical);

    // Anchors of every query hit against the reference hits, after the -f/-U,
    // --q-occ-frac and -e filters, in query-hit order (unsorted).  Runs on the
    // GPU; the reference side is indexed once per distinct hit list and filter
    // setting and kept resident.
    anchor::Anchors collect_anchors(const MinimizerHits& ref_hits, const MinimizerHits& qry_hits,
                                    anchor::SeedFilterParams params = anchor::default_mm2_params());

}  // namespace minimizer

#endif  // HALIGN4_SEED_H
