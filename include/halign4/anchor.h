// anchor.h - drop-in for HAlign-4's include/anchor.h (anchor records, seeding
// filter and chaining parameters, chainAnchors), implemented over the GB300
// C ABI (include/halign_gb300.h) by libhalign4_dropin.so.
//
// Declarations keep the reference's names, types, defaults and record layout
// so HAlign-4's call sites compile unchanged.  chainAnchors runs on the GPU
// (hg_chain_anchors); the occurrence-threshold helpers are the host-side
// index set-up of collect_anchors (hg_occ_threshold).
#ifndef HALIGN4_ANCHOR_H
#define HALIGN4_ANCHOR_H

#include <cstddef>
#include <cstdint>
#include <vector>

#include "hash.h"

namespace anchor
{
    // One seed match between a reference and a query position
    // (include/anchor.h:39-50): 32 bytes, the layout hg_anchor_t mirrors.
    struct Anchor
    {
        hash_t hash{};
        std::uint32_t rid_ref{};
        std::uint32_t pos_ref{};
        std::uint32_t rid_qry{};
        std::uint32_t pos_qry{};
        std::uint32_t span{};
        bool is_rev{};
    };

    using Anchors = std::vector<Anchor>;

    // [start, start + count) of one hash in the sorted reference hits.
    struct HashIndex {
        std::size_t start;
        std::size_t count;
    };

    // minimap2-style seeding filters with the reference's defaults
    // (-f, -U lower/upper, --q-occ-frac, -e).
    struct SeedFilterParams {
        double f_top_frac = 2e-4;
        std::size_t u_floor = 10;
        std::size_t u_ceil = 1000000;
        double q_occ_frac = 0.01;
        std::size_t sample_every_bp = 500;
    };

    static inline SeedFilterParams default_mm2_params() { return SeedFilterParams{}; }

    // Occurrence count of the floor(f_top_frac * #distinct)-th most frequent
    // hash (SIZE_MAX when nothing is skipped, 1 when f_top_frac >= 1).
    std::size_t compute_occ_cutoff_top_frac(const std::vector<std::size_t>& occs, double f_top_frac);

    // max(u_floor, min(u_ceil, compute_occ_cutoff_top_frac(occs, f_top_frac))).
    std::size_t compute_ref_occ_threshold(const std::vector<std::size_t>& occs, const SeedFilterParams& p);

    // Chaining parameters with the reference's defaults.
    struct ChainParams {
        std::int32_t max_dist_x = 5000;
        std::int32_t max_dist_y = 5000;
        std::int32_t bw = 500;
        std::int32_t max_skip = 25;
        std::int32_t max_iter = 5000;
        std::int32_t min_cnt = 3;
        std::int32_t min_score = 40;
        float gap_penalty = 0.01f;
        float skip_penalty = 0.01f;
    };

    inline ChainParams default_chain_params() { return ChainParams{}; }

    // Sorts `anchors` in place by (rid_ref, is_rev, pos_ref, pos_qry) and
    // returns the best chain's anchors in position order (empty when no chain
    // reaches min_score and min_cnt).  Runs on the GPU.
    Anchors chainAnchors(Anchors& anchors, const ChainParams& params = default_chain_params());

}  // namespace anchor

#endif  // HALIGN4_ANCHOR_H
