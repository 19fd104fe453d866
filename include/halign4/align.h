// align.h - drop-in for HAlign-4's include/align.h on the align-to-center
// path: CIGAR algebra (namespace cigar), the DNA5 scoring tables, auto_band,
// globalAlignKSW2, extendAlignKSW2 and globalAlignMM2 (namespace align),
// implemented over the GB300 C ABI (include/halign_gb300.h) by
// libhalign4_dropin.so.
//
// The alignments and the row projections run on the GPU; the CIGAR encode /
// decode / merge helpers are host bookkeeping on the caller's vectors.  Not
// here: globalAlignWFA2 (WFA2-lib, not on this path) and the RefAligner
// class (the CLI driver around the path: file I/O, SAM round trips, the
// external MSA step), whose per-query work is hg_align_batch / hg_align_query.
#ifndef HALIGN4_ALIGN_H
#define HALIGN4_ALIGN_H

#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <algorithm>
#include <functional>
#include <string>
#include <vector>

#include "anchor.h"
#include "ksw2.h"
#include "seed.h"

namespace cigar
{
    using CigarUnit = uint32_t;              // len << 4 | op
    using Cigar_t = std::vector<CigarUnit>;

    // Op codes: 0 M, 1 I, 2 D, 3 N, 4 S, 5 H, 6 P, 7 =, 8 X.  Invalid ops and
    // lengths outside 1 .. 2^28-1 throw std::runtime_error, as the reference.
    CigarUnit cigarToInt(char operation, uint32_t len);
    void intToCigar(CigarUnit cigar, char& operation, uint32_t& len);

    bool hasInsertion(const Cigar_t& cigar);
    std::string cigarToString(const Cigar_t& cigar);
    Cigar_t stringToCigar(const std::string& cigar_str);

    // Query projected onto the reference (GPU): pad keeps insertions, del
    // removes them; D/N become '-'.  An empty CIGAR leaves the query as is.
    void padQueryToRefByCigar(std::string& query, const Cigar_t& cigar);
    void delQueryToRefByCigar(std::string& query, const Cigar_t& cigar);

    void appendCigar(Cigar_t& result, const Cigar_t& cigar_to_add);
    std::size_t getRefLength(const Cigar_t& cigar);
    std::size_t getQueryLength(const Cigar_t& cigar);
}  // namespace cigar

namespace align
{
    using SeedHit = minimizer::MinimizerHit;
    using SeedHits = std::vector<SeedHit>;
    static constexpr seed::SeedKind kSeedKind = seed::SeedKind::minimizer;

    // DNA5 codes for KSW2: A/a 0, C/c 1, G/g 2, T/t 3, every other byte 4
    // (U is 4 here, unlike nt4_table).
    static constexpr uint8_t ScoreChar2Idx[256] = {
        4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4,  //   0- 15
        4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4,  //  16- 31
        4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4,  //  32- 47
        4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4,  //  48- 63
        4, 0, 4, 1, 4, 4, 4, 2, 4, 4, 4, 4, 4, 4, 4, 4,  //  64- 79
        4, 4, 4, 4, 3, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4,  //  80- 95
        4, 0, 4, 1, 4, 4, 4, 2, 4, 4, 4, 4, 4, 4, 4, 4,  //  96-111
        4, 4, 4, 4, 3, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4,  // 112-127
        4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4,  // 128-143
        4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4,  // 144-159
        4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4,  // 160-175
        4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4,  // 176-191
        4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4,  // 192-207
        4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4,  // 208-223
        4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4,  // 224-239
        4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4, 4   // 240-255
    };

    // 5 x 5 DNA5 matrix: +5 match, -4 mismatch, 0 against N.
    static constexpr int8_t dna5_simd_mat[25] = {
         5, -4, -4, -4, 0,
        -4,  5, -4, -4, 0,
        -4, -4,  5, -4, 0,
        -4, -4, -4,  5, 0,
         0,  0,  0,  0, 0,
    };

    struct KSW2AlignConfig {
        const int8_t* mat = dna5_simd_mat;
        int alphabet_size = 5;
        int gap_open = 6;
        int gap_extend = 2;
        int end_bonus = 0;
        int zdrop = -1;
        int band_width = -1;
        int flag = KSW_EZ_GENERIC_SC | KSW_EZ_RIGHT;
    };

    // Band for KSW2: -1 (no band) when the lengths differ by more than half
    // the longer one, else margin + (int)(indel_rate * (qlen + tlen / 2)).
    inline int auto_band(int qlen, int tlen, double indel_rate = 0.1, int margin = 200)
    {
        if ((double)std::abs(qlen - tlen) / (double)std::max(qlen, tlen) > 0.5) return -1;
        return margin + static_cast<int>(indel_rate * (qlen + tlen / 2));
    }

    // Global alignment of query against ref (GPU): DNA5 codes, the default
    // matrix and gaps, auto_band(ref, query), KSW_EZ_GENERIC_SC | KSW_EZ_RIGHT.
    cigar::Cigar_t globalAlignKSW2(const std::string& ref, const std::string& query);
    // The same with the caller's matrix, gaps, z-drop, end bonus and flag; the
    // band is auto_band(ref, query) whatever cfg.band_width holds, as in the
    // reference.
    cigar::Cigar_t globalAlignKSW2(const std::string& ref, const std::string& query, align::KSW2AlignConfig cfg);

    // Extension alignment (GPU): z-drop, end bonus 50, match/mismatch scoring
    // with N as the wildcard (no KSW_EZ_GENERIC_SC), EXTZ_ONLY | RIGHT |
    // APPROX_DROP, auto_band.
    cigar::Cigar_t extendAlignKSW2(const std::string& ref, const std::string& query, int zdrop = 200);

    using AlignFunc = std::function<cigar::Cigar_t(const std::string&, const std::string&)>;

    // Anchor-guided global alignment (GPU): chain the anchors, align the gaps
    // between chained anchors with globalAlignKSW2, stitch the CIGAR; without
    // a chain, one globalAlignKSW2 of the whole pair.
    cigar::Cigar_t globalAlignMM2(const std::string& ref, const std::string& query, const anchor::Anchors& anchors);
}  // namespace align

#endif  // HALIGN4_ALIGN_H
