// test_dropin.cpp - HAlign-4's C++ call surface (include/halign4/*.h) on the
// GPU, through libhalign4_dropin.so, checked against the reference.
//
// Two sources of expected values:
//   * known answers of the reference's own unit tests (test/test_anchor.cpp,
//     test/test_align.cpp, test/test_consensus.cpp), restated here;
//   * tests/golden/dropin_cases.txt and the consensus files next to it,
//     written by tests/golden/make_golden.py from the unmodified reference
//     (extractMinimizer, collect_anchors, chainAnchors, ksw_extz2_sse with
//     generic and match/mismatch scoring, globalAlignKSW2, extendAlignKSW2,
//     globalAlignMM2, delQueryToRefByCigar, padQueryToRefByCigar,
//     cigarToString, generateConsensusSequence).
// All comparisons are exact (integer work).  Also prints the single-call
// latency of globalAlignKSW2 and ksw_extz2_sse.
//
// usage: test_dropin <golden dir> <scratch dir>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <vector>

#include "align.h"
#include "anchor.h"
#include "consensus.h"
#include "ksw2.h"
#include "mash.h"
#include "seed.h"

namespace {

int g_fail = 0, g_pass = 0;

void check(bool ok, const std::string& what)
{
    if (ok) {
        ++g_pass;
    } else {
        ++g_fail;
        if (g_fail <= 40) std::cerr << "FAIL: " << what << "\n";
    }
}

template <typename F>
bool throws(F&& f)
{
    try {
        f();
    } catch (const std::runtime_error&) {
        return true;
    }
    return false;
}

// ---- fixture parsing
template <typename T>
std::vector<T> read_list(std::istringstream& in)
{
    size_t n = 0;
    in >> n;
    std::vector<T> v(n);
    for (size_t i = 0; i < n; ++i) {
        long long x = 0;
        unsigned long long ux = 0;
        if constexpr (std::is_unsigned<T>::value) {
            in >> ux;
            v[i] = (T)ux;
        } else {
            in >> x;
            v[i] = (T)x;
        }
    }
    return v;
}

std::string read_seq(std::istringstream& in)
{
    std::string s;
    in >> s;
    return s == "-" ? std::string() : s;
}

anchor::Anchors read_anchors(std::istringstream& in)
{
    size_t n = 0;
    in >> n;
    anchor::Anchors a(n);
    for (auto& x : a) {
        unsigned long long h;
        unsigned rr, pr, rq, pq, sp, rv;
        in >> h >> rr >> pr >> rq >> pq >> sp >> rv;
        x.hash = h, x.rid_ref = rr, x.pos_ref = pr, x.rid_qry = rq, x.pos_qry = pq, x.span = sp, x.is_rev = rv != 0;
    }
    return a;
}

bool same(const anchor::Anchors& a, const anchor::Anchors& b)
{
    if (a.size() != b.size()) return false;
    for (size_t i = 0; i < a.size(); ++i)
        if (a[i].hash != b[i].hash || a[i].rid_ref != b[i].rid_ref || a[i].pos_ref != b[i].pos_ref ||
            a[i].rid_qry != b[i].rid_qry || a[i].pos_qry != b[i].pos_qry || a[i].span != b[i].span ||
            a[i].is_rev != b[i].is_rev)
            return false;
    return true;
}

minimizer::MinimizerHits hits(const std::vector<uint64_t>& x, const std::vector<uint64_t>& y)
{
    minimizer::MinimizerHits h;
    for (size_t i = 0; i < x.size(); ++i) h.emplace_back(x[i], y[i]);
    return h;
}

std::string slurp(const std::string& path)
{
    std::ifstream f(path, std::ios::binary);
    std::ostringstream s;
    s << f.rdbuf();
    return s.str();
}

const int8_t kMat[25] = {5, -4, -4, -4, 0, -4, 5, -4, -4, 0, -4, -4, 5, -4, 0, -4, -4, -4, 5, 0, 0, 0, 0, 0, 0};

// ---- known answers restated from the reference's unit tests
void known_answers()
{
    using anchor::Anchor;
    using minimizer::MinimizerHit;
    // collect_anchors (test/test_anchor.cpp:60-246)
    // the reference's tests switch the query-side filter off (q_occ_frac 0,
    // f_top_frac 0): with one query hit the default 1% limit drops every hash
    anchor::SeedFilterParams p0;
    p0.q_occ_frac = 0.0, p0.f_top_frac = 0.0;
    minimizer::MinimizerHits none, one_ref{MinimizerHit(0x123456, 100, 0, false, 20)};
    check(minimizer::collect_anchors(none, none).empty(), "collect_anchors empty input");
    check(minimizer::collect_anchors(none, one_ref).empty(), "collect_anchors empty reference");
    check(minimizer::collect_anchors(one_ref, none).empty(), "collect_anchors empty query");
    {
        auto a = minimizer::collect_anchors(one_ref, {MinimizerHit(0x123456, 50, 0, false, 20)}, p0);
        check(a.size() == 1 && a[0].hash == 0x123456 && a[0].pos_ref == 100 && a[0].pos_qry == 50 &&
                  a[0].span == 20 && !a[0].is_rev,
              "collect_anchors single perfect match");
        a = minimizer::collect_anchors(one_ref, {MinimizerHit(0x123456, 50, 0, true, 20)}, p0);
        check(a.size() == 1 && a[0].is_rev, "collect_anchors reverse match");
        a = minimizer::collect_anchors(one_ref, {MinimizerHit(0x654321, 50, 0, false, 20)}, p0);
        check(a.empty(), "collect_anchors no shared hash");
        minimizer::MinimizerHits r3{MinimizerHit(0xabc, 300, 0, false, 15), MinimizerHit(0xabc, 100, 0, false, 15),
                                    MinimizerHit(0xabc, 200, 0, false, 15)};
        anchor::SeedFilterParams p;
        p.q_occ_frac = 0, p.f_top_frac = 0;
        a = minimizer::collect_anchors(r3, {MinimizerHit(0xabc, 50, 0, false, 15)}, p);
        check(a.size() == 3 && a[0].pos_qry == 50 && a[0].pos_ref == 100 && a[1].pos_ref == 200 &&
                  a[2].pos_ref == 300,
              "collect_anchors one-to-many expansion in sorted reference order");
        minimizer::MinimizerHits qmany;  // 50 of 100 query hits share the one reference hash
        for (int i = 0; i < 50; ++i) qmany.emplace_back(MinimizerHit(0x888888, i, 0, false, 15));
        for (int i = 0; i < 50; ++i) qmany.emplace_back(MinimizerHit(0x999900 + i, i, 0, false, 15));
        anchor::SeedFilterParams q10;
        q10.q_occ_frac = 0.10, q10.f_top_frac = 0.0;
        a = minimizer::collect_anchors({MinimizerHit(0x888888, 100, 0, false, 15)}, qmany, q10);
        check(a.empty(), "collect_anchors q_occ_frac drops a hash frequent in the query");
        a = minimizer::collect_anchors({MinimizerHit(0x77, 100, 0, false, 30)}, {MinimizerHit(0x77, 50, 0, false, 20)},
                                        p0);
        check(a.size() == 1 && a[0].span == 20, "collect_anchors span = min(ref, qry)");
        a = minimizer::collect_anchors({MinimizerHit(0x77, 100, 2, false, 20)}, {MinimizerHit(0x77, 50, 3, false, 20)},
                                        p0);
        check(a.size() == 1 && a[0].rid_ref == 2 && a[0].rid_qry == 3, "collect_anchors rid passed through");
    }
    // chainAnchors (test/test_anchor.cpp:260-481)
    auto A = [](uint32_t rid, uint32_t pr, uint32_t pq, uint32_t span, bool rev) {
        Anchor a;
        a.rid_ref = rid, a.pos_ref = pr, a.pos_qry = pq, a.span = span, a.is_rev = rev;
        return a;
    };
    anchor::ChainParams loose;
    loose.min_cnt = 1, loose.min_score = 0;
    {
        anchor::Anchors v;
        check(anchor::chainAnchors(v, loose).empty(), "chainAnchors empty");
        v = {A(0, 100, 50, 20, false)};
        auto c = anchor::chainAnchors(v, loose);
        check(c.size() == 1 && c[0].span == 20, "chainAnchors single anchor");
        v = {A(0, 200, 150, 20, false), A(0, 100, 50, 20, false)};
        c = anchor::chainAnchors(v, loose);
        check(c.size() == 2 && c[0].pos_ref == 100 && c[1].pos_ref == 200 && c[0].pos_qry == 50 &&
                  c[1].pos_qry == 150,
              "chainAnchors two linkable anchors, position order");
        check(v[0].pos_ref == 100 && v[1].pos_ref == 200, "chainAnchors sorts its input in place");
        v = {A(1, 100, 50, 20, false), A(0, 100, 50, 20, false), A(0, 200, 150, 20, false), A(0, 300, 250, 20, false)};
        c = anchor::chainAnchors(v, loose);
        check(!c.empty() && c[0].rid_ref == 0 && c.size() >= 2, "chainAnchors best chain across reference ids");
        v = {A(0, 100, 50, 20, true), A(0, 100, 50, 20, false), A(0, 200, 150, 20, false), A(0, 300, 250, 20, false)};
        c = anchor::chainAnchors(v, loose);
        check(!c.empty() && !c[0].is_rev && c.size() >= 2, "chainAnchors best chain across strands");
        v = {A(0, 100, 50, 20, false), A(0, 10000, 9950, 20, false)};
        check(anchor::chainAnchors(v, loose).size() == 1, "chainAnchors too far apart");
        v = {A(0, 100, 100, 20, false), A(0, 1000, 200, 20, false)};
        check(anchor::chainAnchors(v, loose).size() == 1, "chainAnchors diagonal beyond bw");
        anchor::ChainParams cnt3;
        cnt3.min_cnt = 3, cnt3.min_score = 0;
        v = {A(0, 100, 50, 20, false), A(0, 200, 150, 20, false)};
        check(anchor::chainAnchors(v, cnt3).empty(), "chainAnchors min_cnt");
        anchor::ChainParams sc;
        sc.min_cnt = 1, sc.min_score = 1000;
        check(anchor::chainAnchors(v, sc).empty(), "chainAnchors min_score");
    }
    // globalAlignKSW2 and CIGAR helpers (test/test_align.cpp:234-490)
    {
        const auto c = align::globalAlignKSW2("ACGTACGTACGT", "ACGTACGTACGT");
        char op = 0;
        uint32_t len = 0;
        if (!c.empty()) cigar::intToCigar(c[0], op, len);
        check(c.size() == 1 && op == 'M' && len == 12, "globalAlignKSW2 exact match is 12M");
        check(cigar::hasInsertion(align::globalAlignKSW2("ACGTACGTACGTACGT", "ACGTACGTTTTACGTACGT")),
              "globalAlignKSW2 single insertion");
        check(!throws([] { align::globalAlignKSW2("", "ACGT"); }) && !throws([] { align::globalAlignKSW2("ACGT", ""); }),
              "globalAlignKSW2 empty sequences");
        cigar::Cigar_t orig{cigar::cigarToInt('M', 100), cigar::cigarToInt('I', 5), cigar::cigarToInt('M', 95),
                            cigar::cigarToInt('D', 3), cigar::cigarToInt('M', 50)};
        const std::string s = cigar::cigarToString(orig);
        check(s == "100M5I95M3D50M" && cigar::stringToCigar(s) == orig, "cigarToString / stringToCigar round trip");
        cigar::Cigar_t big{cigar::cigarToInt('M', 999999), cigar::cigarToInt('D', 123456)};
        check(cigar::cigarToString(big) == "999999M123456D" && cigar::stringToCigar("999999M123456D") == big,
              "large CIGAR round trip");
        check(cigar::cigarToString({}).empty() && cigar::stringToCigar("").empty(), "empty CIGAR");
        check(throws([] { cigar::stringToCigar("M10"); }) && throws([] { cigar::stringToCigar("10Q"); }) &&
                  throws([] { cigar::stringToCigar("10M5"); }) && throws([] { cigar::stringToCigar("0M"); }),
              "stringToCigar rejects malformed strings");
        const auto r = cigar::stringToCigar("10M5I3D");
        check(r.size() == 3 && r[1] == cigar::cigarToInt('I', 5), "stringToCigar parses 10M5I3D");
        cigar::Cigar_t acc{cigar::cigarToInt('M', 3)};
        cigar::appendCigar(acc, {cigar::cigarToInt('M', 4), cigar::cigarToInt('I', 2)});
        check(acc.size() == 2 && (acc[0] >> 4) == 7, "appendCigar merges equal ops");
        check(cigar::getRefLength(cigar::stringToCigar("5M2I3D")) == 8 &&
                  cigar::getQueryLength(cigar::stringToCigar("5M2I3D")) == 7,
              "getRefLength / getQueryLength");
        std::string q = "ACGTTACG";
        cigar::delQueryToRefByCigar(q, cigar::stringToCigar("4M1I2D3M"));
        check(q == "ACGT--ACG", "delQueryToRefByCigar");
        q = "ACGTTACG";
        cigar::padQueryToRefByCigar(q, cigar::stringToCigar("4M1I2D3M"));
        check(q == "ACGTT--ACG", "padQueryToRefByCigar");
        // globalAlignMM2 without anchors equals globalAlignKSW2's lengths
        const std::string ref = "ACGTACGTAGCTAGCTAGCTGATCGATCGTAGCTAGCTAGCTAGC", qry = "ACGTACGTAGCTAGCAGCTGATCGATCGTAGCTAGCTTAGCTAGC";
        const auto mm = align::globalAlignMM2(ref, qry, {});
        check(mm == align::globalAlignKSW2(ref, qry) && cigar::getRefLength(mm) == ref.size() &&
                  cigar::getQueryLength(mm) == qry.size(),
              "globalAlignMM2 without anchors = globalAlignKSW2");
    }
    // pickConsensusChar (test/test_consensus.cpp): majority, A>C>G>T>U ties, 'A' on all zero
    {
        consensus::SiteCount s;
        check(consensus::pickConsensusChar(s) == 'A', "pickConsensusChar all zero");
        s.c = 3, s.g = 3;
        check(consensus::pickConsensusChar(s) == 'C', "pickConsensusChar tie C > G");
        s.u = 9, s.n = 20, s.dash = 30;
        check(consensus::pickConsensusChar(s) == 'U', "pickConsensusChar ignores N and gaps");
        check(consensus::mapBase('u') == 4 && consensus::mapBase('.') == 6 && consensus::mapBase('X') == 5,
              "k_base_map classes");
    }
}

// ---- reference outputs from the golden fixture
void golden_cases(const std::string& path)
{
    std::ifstream f(path);
    if (!f) {
        check(false, "golden fixture missing: " + path);
        return;
    }
    std::string line;
    int n = 0;
    while (std::getline(f, line)) {
        std::istringstream in(line);
        std::string tag;
        in >> tag;
        ++n;
        const std::string id = tag + " case " + std::to_string(n);
        if (tag == "MZ") {
            int k, w, nc;
            size_t len;
            in >> k >> w >> nc >> len;
            const std::string s = read_seq(in);
            const auto x = read_list<uint64_t>(in), y = read_list<uint64_t>(in);
            const auto h = minimizer::extractMinimizer(s, k, w, nc != 0);
            bool ok = h.size() == x.size();
            for (size_t i = 0; ok && i < h.size(); ++i) ok = h[i].x == x[i] && h[i].y == y[i];
            check(ok, id + " extractMinimizer");
        } else if (tag == "CA") {
            anchor::SeedFilterParams p;
            in >> p.f_top_frac >> p.u_floor >> p.u_ceil >> p.q_occ_frac >> p.sample_every_bp;
            const auto rx = read_list<uint64_t>(in), ry = read_list<uint64_t>(in);
            const auto qx = read_list<uint64_t>(in), qy = read_list<uint64_t>(in);
            const auto want = read_anchors(in);
            check(same(minimizer::collect_anchors(hits(rx, ry), hits(qx, qy), p), want), id + " collect_anchors");
        } else if (tag == "CH") {
            anchor::ChainParams p;
            in >> p.max_dist_x >> p.max_dist_y >> p.bw >> p.max_skip >> p.max_iter >> p.min_cnt >> p.min_score >>
                p.gap_penalty >> p.skip_penalty;
            auto a = read_anchors(in);
            const auto srt = read_anchors(in), ch = read_anchors(in);
            const auto got = anchor::chainAnchors(a, p);
            check(same(a, srt), id + " chainAnchors sorted input");
            check(same(got, ch), id + " chainAnchors chain");
        } else if (tag == "MM") {
            const std::string ref = read_seq(in), qry = read_seq(in);
            const auto a = read_anchors(in);
            const auto want = read_list<uint32_t>(in);
            check(align::globalAlignMM2(ref, qry, a) == want, id + " globalAlignMM2");
        } else if (tag == "DQ" || tag == "PQ") {
            std::string q = read_seq(in);
            const auto c = read_list<uint32_t>(in);
            const std::string want = read_seq(in);
            if (tag == "DQ") cigar::delQueryToRefByCigar(q, c);
            else cigar::padQueryToRefByCigar(q, c);
            check(q == want, id + (tag == "DQ" ? " delQueryToRefByCigar" : " padQueryToRefByCigar"));
        } else if (tag == "KS") {
            int w, zdrop, eb, flag;
            in >> w >> zdrop >> eb >> flag;
            const auto q = read_list<uint8_t>(in), t = read_list<uint8_t>(in);
            const auto ez = read_list<int32_t>(in);
            const auto c = read_list<uint32_t>(in);
            ksw_extz_t r{};
            ksw_extz2_sse(nullptr, (int)q.size(), q.data(), (int)t.size(), t.data(), 5, kMat, 6, 2, w, zdrop, eb, flag,
                          &r);
            const int32_t got[10] = {(int32_t)r.max, (int32_t)r.zdropped, r.max_q, r.max_t, r.mqe,
                                     r.mqe_t,        r.mte,               r.mte_q, r.score, r.reach_end};
            bool ok = (int)c.size() == r.n_cigar && ez.size() == 10;
            for (int i = 0; ok && i < 10; ++i) ok = got[i] == ez[i];
            for (int i = 0; ok && i < r.n_cigar; ++i) ok = r.cigar[i] == c[i];
            check(ok, id + " ksw_extz2_sse flag " + std::to_string(flag));
            std::free(r.cigar);
        } else if (tag == "GK") {
            int flag;
            in >> flag;
            const std::string ref = read_seq(in), qry = read_seq(in);
            const auto want = read_list<uint32_t>(in);
            align::KSW2AlignConfig cfg;
            if (flag >= 0) cfg.flag = flag;
            const auto got = flag < 0 ? align::globalAlignKSW2(ref, qry) : align::globalAlignKSW2(ref, qry, cfg);
            check(got == want, id + " globalAlignKSW2");
        } else if (tag == "EX") {
            int zd;
            in >> zd;
            const std::string ref = read_seq(in), qry = read_seq(in);
            check(align::extendAlignKSW2(ref, qry, zd) == read_list<uint32_t>(in), id + " extendAlignKSW2");
        } else if (tag == "CS") {
            const auto c = read_list<uint32_t>(in);
            std::string want;
            in >> want;
            check(cigar::cigarToString(c) == want, id + " cigarToString");
        } else if (tag == "SK") {
            int k, sz, nc, sd;
            size_t len;
            in >> k >> sz >> nc >> sd >> len;
            const std::string s = read_seq(in);
            const auto want = read_list<uint64_t>(in);
            const mash::Sketch sk = mash::sketchFromSequence(s, (size_t)k, (size_t)sz, nc != 0, sd);
            check(sk.hashes == want && sk.k == (size_t)k, id + " mash::sketchFromSequence");
        } else if (tag == "JC") {
            mash::Sketch a, b;
            in >> a.k;
            b.k = a.k;
            a.hashes = read_list<uint64_t>(in);
            b.hashes = read_list<uint64_t>(in);
            double want;
            in >> want;
            check(mash::jaccard(a, b) == want, id + " mash::jaccard");
        }
    }
    check(n > 100, "golden fixture holds the expected cases");
}

void consensus_cases(const std::string& gdir, const std::string& tmp)
{
    for (const auto& [tag, limit, bs] : {std::tuple<std::string, int, int>{"b3", 0, 3}, {"l5", 5, 4096}}) {
        const std::string fa = tmp + "/cons_" + tag + ".fa", js = tmp + "/cons_" + tag + ".json";
        const std::string cons =
            consensus::generateConsensusSequence(gdir + "/dropin_aln.fa", fa, js, (uint64_t)limit, 4, (size_t)bs);
        check(slurp(fa) == slurp(gdir + "/dropin_cons_" + tag + ".fa"), "generateConsensusSequence FASTA " + tag);
        check(slurp(js) == slurp(gdir + "/dropin_cons_" + tag + ".json"), "generateConsensusSequence JSON " + tag);
        check(!cons.empty(), "generateConsensusSequence returns the consensus " + tag);
    }
}

void latency()
{
    std::string ref(200, 'A'), qry;
    unsigned s = 12345;
    for (auto& c : ref) c = "ACGT"[(s = s * 1103515245u + 12345u) >> 30];
    qry = ref.substr(0, 90) + "TT" + ref.substr(95);
    align::globalAlignKSW2(ref, qry);  // warm-up (workspace growth)
    const int reps = 200;
    auto t0 = std::chrono::steady_clock::now();
    for (int i = 0; i < reps; ++i) align::globalAlignKSW2(ref, qry);
    const double us = std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now() - t0).count() / reps;
    std::cout << "latency globalAlignKSW2 200 bp: " << us << " us/call\n";
    const auto h = minimizer::extractMinimizer(ref + ref + ref, 15, 10, true);
    t0 = std::chrono::steady_clock::now();
    for (int i = 0; i < reps; ++i) minimizer::extractMinimizer(ref + ref + ref, 15, 10, true);
    const double us2 = std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now() - t0).count() / reps;
    std::cout << "latency extractMinimizer 600 bp: " << us2 << " us/call (" << h.size() << " hits)\n";
}

}  // namespace

int main(int argc, char** argv)
{
    if (argc < 3) {
        std::cerr << "usage: test_dropin <golden dir> <scratch dir>\n";
        return 2;
    }
    const std::string gdir = argv[1], tmp = argv[2];
    try {
        known_answers();
        golden_cases(gdir + "/dropin_cases.txt");
        consensus_cases(gdir, tmp);
        latency();
    } catch (const std::exception& e) {
        std::cerr << "exception: " << e.what() << "\n";
        ++g_fail;
    }
    std::cout << "dropin checks passed " << g_pass << " failed " << g_fail << "\n";
    return g_fail ? 1 : 0;
}
