// consensus.h - drop-in for HAlign-4's include/consensus.h on the
// align-to-center path: the per-column SiteCount record, the character
// classes, the consensus pick and the consensus of an aligned FASTA,
// implemented over the GB300 C ABI (hg_count_rows) by libhalign4_dropin.so.
//
// SiteCount and ConsensusJson keep the reference's fields and order; the
// JSON writer produces the reference's file without the cereal library.
// TopKLongestSelector (the center-selection step before an external MSA) is
// not part of this surface.
#ifndef HALIGN4_CONSENSUS_H
#define HALIGN4_CONSENSUS_H

#include <array>
#include <cstddef>
#include <cstdint>
#include <filesystem>
#include <string>
#include <vector>

using FilePath = std::filesystem::path;

namespace consensus
{
    // Counts of one alignment column: A, C, G, T, U, N (any other byte) and
    // gaps ('-' or '.'), in this order (seven uint32 words).
    struct SiteCount
    {
        std::uint32_t a = 0;
        std::uint32_t c = 0;
        std::uint32_t g = 0;
        std::uint32_t t = 0;
        std::uint32_t u = 0;
        std::uint32_t n = 0;
        std::uint32_t dash = 0;
    };

    struct ConsensusJson
    {
        std::uint64_t num_seqs = 0;
        std::uint64_t aln_len = 0;
        std::vector<SiteCount> counts;
    };

    // Column class of a byte: 0 A/a, 1 C/c, 2 G/g, 3 T/t, 4 U/u, 6 '-' or '.',
    // 5 for every other byte.
    inline constexpr std::array<std::uint8_t, 256> k_base_map = []() {
        std::array<std::uint8_t, 256> m{};
        for (std::size_t i = 0; i < m.size(); ++i) {
            const char ch = static_cast<char>(i);
            m[i] = (ch == 'A' || ch == 'a') ? 0
                 : (ch == 'C' || ch == 'c') ? 1
                 : (ch == 'G' || ch == 'g') ? 2
                 : (ch == 'T' || ch == 't') ? 3
                 : (ch == 'U' || ch == 'u') ? 4
                 : (ch == '-' || ch == '.') ? 6
                                            : 5;
        }
        return m;
    }();

    inline std::uint8_t mapBase(char ch) { return k_base_map[(unsigned char)ch]; }

    // Majority base among A, C, G, T, U (ties: A > C > G > T > U; 'A' when
    // all five are zero); never N or a gap.
    char pickConsensusChar(const SiteCount& sc);

    // ">consensus" then the sequence in 80-column lines.
    void writeConsensusFasta(const FilePath& out_fasta, const std::string& seq);

    // The counts as the reference's JSON document.
    void writeCountsJson(const FilePath& out_json, const ConsensusJson& cj);

    // Counts every column of an aligned FASTA (GPU), writes the consensus
    // FASTA and the counts JSON and returns the consensus.  Records are read
    // in batches of batch_size as the reference reads them, including the
    // record it skips between two full batches; seq_limit > 0 stops after
    // that many records.  `thread` is accepted for the signature only.
    std::string generateConsensusSequence(const FilePath& aligned_fasta, const FilePath& out_fasta,
                                          const FilePath& out_json, std::uint64_t seq_limit, int thread,
                                          size_t batch_size = 4096);
}  // namespace consensus

#endif  // HALIGN4_CONSENSUS_H
