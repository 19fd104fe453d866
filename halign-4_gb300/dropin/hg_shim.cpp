// hg_shim.cpp - the C++ call surface of HAlign-4's seed.h, anchor.h,
// align.h, ksw2.h, consensus.h and mash.h (include/halign4/*.h) over the GB300 C ABI
// (include/halign_gb300.h).  Built into libhalign4_dropin.so, which links
// libhalign_gb300.so; HAlign-4 links this library in place of the reference
// sources of those functions (minimizer.cpp, anchor.cpp, align.cpp,
// cigar.cpp, ksw2_extz2_sse.c, consensus.cpp).
//
// Every alignment, seeding, chaining, projection and counting step runs on
// the GPU through the C ABI.  What stays on the host here: converting between
// the reference's records and the ABI's, CIGAR encode/decode/merge on the
// caller's vectors, reading the aligned FASTA for generateConsensusSequence
// and writing its output files, and the caches that keep one resident GPU
// index per distinct reference hit list or center.
//
// Errors: the reference throws std::runtime_error; so do these functions,
// with the C ABI's message (ksw_extz2_sse, a C function, leaves the reset
// result instead).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <limits>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "halign4/align.h"
#include "halign4/anchor.h"
#include "halign4/consensus.h"
#include "halign4/ksw2.h"
#include "halign4/mash.h"
#include "halign4/seed.h"
#include "halign_gb300.h"

static_assert(sizeof(anchor::Anchor) == sizeof(hg_anchor_t), "anchor::Anchor and hg_anchor_t are both 32 bytes");

namespace {

[[noreturn]] void raise(const std::string& where)
{
    throw std::runtime_error(where + ": " + hg_last_error());
}

// 64-bit fingerprint of a word sequence (splitmix64 finaliser per word).
uint64_t mix(uint64_t h, uint64_t v)
{
    v += 0x9e3779b97f4a7c15ULL + h;
    v = (v ^ (v >> 30)) * 0xbf58476d1ce4e5b9ULL;
    v = (v ^ (v >> 27)) * 0x94d049bb133111ebULL;
    return v ^ (v >> 31);
}

// Reference hit lists of collect_anchors, indexed once on the GPU and kept
// (the reference re-sorts and re-hashes them on every call).
struct HitsKey {
    uint64_t fp;
    size_t n;
    double f;
    size_t uf, uc;
    bool operator<(const HitsKey& o) const { return std::tie(fp, n, f, uf, uc) < std::tie(o.fp, o.n, o.f, o.uf, o.uc); }
};
std::mutex g_hits_mu;
std::map<HitsKey, hg_hits_t*> g_hits;

hg_hits_t* hits_for(const minimizer::MinimizerHits& ref, const anchor::SeedFilterParams& p)
{
    uint64_t fp = 0x243f6a8885a308d3ULL;
    for (const auto& h : ref) fp = mix(mix(fp, h.x), h.y);
    const HitsKey key{fp, ref.size(), p.f_top_frac, p.u_floor, p.u_ceil};
    std::lock_guard<std::mutex> lock(g_hits_mu);
    auto it = g_hits.find(key);
    if (it != g_hits.end()) return it->second;
    std::vector<uint64_t> x(ref.size()), y(ref.size());
    for (size_t i = 0; i < ref.size(); ++i) x[i] = ref[i].x, y[i] = ref[i].y;
    hg_params_t prm;
    hg_default_params(&prm);
    prm.f_top_frac = p.f_top_frac, prm.u_floor = p.u_floor, prm.u_ceil = p.u_ceil;
    hg_hits_t* h = nullptr;
    if (hg_hits_create(x.data(), y.data(), (int64_t)x.size(), &prm, &h) != HG_OK) raise("collect_anchors");
    g_hits.emplace(key, h);
    return h;
}

// Resident center indexes for the anchor-guided alignment of one center.
struct IndexKey {
    uint64_t fp;
    size_t n;
    uint32_t k;
    bool operator<(const IndexKey& o) const { return std::tie(fp, n, k) < std::tie(o.fp, o.n, o.k); }
};
std::mutex g_ix_mu;
std::map<IndexKey, hg_index_t*> g_ix;

hg_index_t* index_for(const std::string& ref, uint32_t k)
{
    uint64_t fp = 0x13198a2e03707344ULL;
    for (size_t i = 0; i < ref.size(); i += 8) {
        uint64_t w = 0;
        std::memcpy(&w, ref.data() + i, std::min<size_t>(8, ref.size() - i));
        fp = mix(fp, w);
    }
    const IndexKey key{fp, ref.size(), k};
    std::lock_guard<std::mutex> lock(g_ix_mu);
    auto it = g_ix.find(key);
    if (it != g_ix.end()) return it->second;
    hg_index_t* ix = nullptr;
    if (hg_index_create(ref.data(), (int64_t)ref.size(), (int)k, 10, nullptr, &ix) != HG_OK)
        raise("globalAlignMM2");
    g_ix.emplace(key, ix);
    return ix;
}

hg_params_t chain_params(const anchor::ChainParams& c)
{
    hg_params_t p;
    hg_default_params(&p);
    p.max_dist_x = c.max_dist_x, p.max_dist_y = c.max_dist_y, p.bw = c.bw, p.max_skip = c.max_skip;
    p.max_iter = c.max_iter, p.min_cnt = c.min_cnt, p.min_score = c.min_score;
    p.gap_penalty = c.gap_penalty, p.skip_penalty = c.skip_penalty;
    return p;
}

hg_anchor_t to_c(const anchor::Anchor& a)
{
    hg_anchor_t r;
    r.hash = a.hash, r.rid_ref = a.rid_ref, r.pos_ref = a.pos_ref, r.rid_qry = a.rid_qry, r.pos_qry = a.pos_qry;
    r.span = a.span, r.is_rev = a.is_rev ? 1u : 0u;
    return r;
}

anchor::Anchor from_c(const hg_anchor_t& a)
{
    anchor::Anchor r;
    r.hash = a.hash, r.rid_ref = a.rid_ref, r.pos_ref = a.pos_ref, r.rid_qry = a.rid_qry, r.pos_qry = a.pos_qry;
    r.span = a.span, r.is_rev = a.is_rev != 0;
    return r;
}

std::vector<uint8_t> dna5(const std::string& s)
{
    std::vector<uint8_t> v(s.size());
    for (size_t i = 0; i < s.size(); ++i) v[i] = align::ScoreChar2Idx[(uint8_t)s[i]];
    return v;
}

// One ksw_extz2 call on the GPU; ez fields into r[10], CIGAR into cig.
int64_t ksw_call(int qlen, const uint8_t* query, int tlen, const uint8_t* target, int m, const int8_t* mat, int q,
                 int e, int w, int zdrop, int end_bonus, int flag, int32_t* r, std::vector<uint32_t>& cig)
{
    cig.resize((size_t)qlen + tlen + 4);
    return hg_ksw_extz2(qlen, query, tlen, target, (int8_t)m, mat, (int8_t)q, (int8_t)e, w, zdrop, end_bonus, flag, r,
                        cig.data(), (int64_t)cig.size());
}

}  // namespace

// ------------------------------------------------------------------ seeds

namespace minimizer
{
MinimizerHits extractMinimizer(const std::string& seq, std::size_t k, std::size_t w, bool non_canonical)
{
    MinimizerHits out;
    if (seq.empty()) return out;
    std::vector<uint64_t> x(seq.size() + 1), y(seq.size() + 1);
    int64_t need = 0;
    const int64_t n = hg_extract_minimizer(seq.data(), (int64_t)seq.size(), (int)k, (int)w, non_canonical ? 1 : 0,
                                           x.data(), y.data(), (int64_t)x.size(), &need);
    if (n < 0) raise("extractMinimizer");
    out.reserve((size_t)n);
    for (int64_t i = 0; i < n; ++i) out.emplace_back(x[i], y[i]);
    return out;
}

anchor::Anchors collect_anchors(const MinimizerHits& ref_hits, const MinimizerHits& qry_hits,
                                anchor::SeedFilterParams params)
{
    anchor::Anchors out;
    if (ref_hits.empty() || qry_hits.empty()) return out;
    hg_hits_t* h = hits_for(ref_hits, params);
    std::vector<uint64_t> x(qry_hits.size()), y(qry_hits.size());
    for (size_t i = 0; i < qry_hits.size(); ++i) x[i] = qry_hits[i].x, y[i] = qry_hits[i].y;
    hg_params_t prm;
    hg_default_params(&prm);
    prm.q_occ_frac = params.q_occ_frac, prm.sample_every_bp = params.sample_every_bp;
    std::vector<hg_anchor_t> a(qry_hits.size() + 16);
    int64_t need = 0;
    int64_t n = hg_collect_anchors(h, x.data(), y.data(), (int64_t)x.size(), &prm, a.data(), (int64_t)a.size(), &need);
    if (n == -HG_ERR_CAPACITY) {
        a.resize((size_t)need);
        n = hg_collect_anchors(h, x.data(), y.data(), (int64_t)x.size(), &prm, a.data(), (int64_t)a.size(), &need);
    }
    if (n < 0) raise("collect_anchors");
    out.reserve((size_t)n);
    for (int64_t i = 0; i < n; ++i) out.push_back(from_c(a[i]));
    return out;
}
}  // namespace minimizer

// ------------------------------------------------------------------ anchors

namespace anchor
{
std::size_t compute_occ_cutoff_top_frac(const std::vector<std::size_t>& occs, double f_top_frac)
{
    std::vector<uint64_t> v(occs.begin(), occs.end());
    hg_params_t p;
    hg_default_params(&p);
    p.f_top_frac = f_top_frac;
    uint64_t cut = 0;
    hg_occ_threshold(v.data(), (int64_t)v.size(), &p, &cut);
    return (std::size_t)cut;
}

std::size_t compute_ref_occ_threshold(const std::vector<std::size_t>& occs, const SeedFilterParams& sp)
{
    std::vector<uint64_t> v(occs.begin(), occs.end());
    hg_params_t p;
    hg_default_params(&p);
    p.f_top_frac = sp.f_top_frac, p.u_floor = sp.u_floor, p.u_ceil = sp.u_ceil;
    return (std::size_t)hg_occ_threshold(v.data(), (int64_t)v.size(), &p, nullptr);
}

Anchors chainAnchors(Anchors& anchors, const ChainParams& params)
{
    Anchors out;
    if (anchors.empty()) return out;
    std::vector<hg_anchor_t> a(anchors.size());
    for (size_t i = 0; i < anchors.size(); ++i) a[i] = to_c(anchors[i]);
    const hg_params_t prm = chain_params(params);
    std::vector<int64_t> chain(anchors.size());
    const int64_t m =
        hg_chain_anchors(a.data(), (int64_t)a.size(), &prm, chain.data(), (int64_t)chain.size(), nullptr, nullptr);
    if (m < 0) raise("chainAnchors");
    for (size_t i = 0; i < anchors.size(); ++i) anchors[i] = from_c(a[i]);  // sorted in place, as the reference
    out.reserve((size_t)m);
    for (int64_t i = 0; i < m; ++i) out.push_back(anchors[(size_t)chain[i]]);
    return out;
}
}  // namespace anchor

// ------------------------------------------------------------------ KSW2

extern "C" void ksw_extz2_sse(void* km, int qlen, const uint8_t* query, int tlen, const uint8_t* target, int8_t m,
                              const int8_t* mat, int8_t q, int8_t e, int w, int zdrop, int end_bonus, int flag,
                              ksw_extz_t* ez)
{
    (void)km;
    ksw_reset_extz(ez);
    if (m <= 0 || qlen <= 0 || tlen <= 0) return;
    int32_t r[10];
    std::vector<uint32_t> cig;
    const int64_t n = ksw_call(qlen, query, tlen, target, m, mat, q, e, w, zdrop, end_bonus, flag, r, cig);
    if (n < 0) return;
    ez->max = (uint32_t)r[0] & 0x7fffffffu, ez->zdropped = r[1] ? 1u : 0u;
    ez->max_q = r[2], ez->max_t = r[3], ez->mqe = r[4], ez->mqe_t = r[5], ez->mte = r[6], ez->mte_q = r[7];
    ez->score = r[8], ez->reach_end = r[9];
    if (flag & KSW_EZ_SCORE_ONLY) return;
    // the reference grows ez->cigar by doubling from m_cigar (4 when 0) as it
    // pushes ops; the same capacity results here
    if (n > ez->m_cigar) {
        int mc = ez->m_cigar > 0 ? ez->m_cigar : 4;
        while (mc < n) mc <<= 1;
        void* p = std::realloc(ez->cigar, sizeof(uint32_t) * (size_t)mc);
        if (!p) return;
        ez->cigar = static_cast<uint32_t*>(p);
        ez->m_cigar = mc;
    }
    if (n) std::memcpy(ez->cigar, cig.data(), sizeof(uint32_t) * (size_t)n);
    ez->n_cigar = (int)n;
}

// ------------------------------------------------------------------ CIGAR algebra

namespace cigar
{
namespace {
uint32_t op_code(char c)
{
    switch (c) {
    case 'M': return 0;
    case 'I': return 1;
    case 'D': return 2;
    case 'N': return 3;
    case 'S': return 4;
    case 'H': return 5;
    case 'P': return 6;
    case '=': return 7;
    case 'X': return 8;
    default: throw std::runtime_error(std::string("Unknown CIGAR op char: ") + c);
    }
}

char op_char(uint32_t code)
{
    static const char kOps[] = "MIDNSHP=X";
    if (code > 8) throw std::runtime_error("Unknown CIGAR op code: " + std::to_string(code));
    return kOps[code];
}

constexpr uint32_t kMaxLen = (1u << 28) - 1u;

void project(std::string& query, const Cigar_t& cigar, int pad)
{
    if (cigar.empty()) return;
    for (CigarUnit c : cigar) op_char(c & 0xfu);  // unknown op codes throw, as intToCigar does
    uint64_t cols = 0;
    for (CigarUnit c : cigar) cols += c >> 4;
    std::string out((size_t)cols + query.size() + 1, '\0');
    const int64_t n =
        hg_project_row(query.data(), (int64_t)query.size(), cigar.data(), (int64_t)cigar.size(), pad, out.data(),
                       (int64_t)out.size());
    if (n < 0) raise(pad ? "padQueryToRefByCigar" : "delQueryToRefByCigar");
    out.resize((size_t)n);
    query.swap(out);
}
}  // namespace

CigarUnit cigarToInt(char operation, uint32_t len)
{
    if (len == 0 || len > kMaxLen) throw std::runtime_error("cigarToInt: invalid length=" + std::to_string(len));
    return (len << 4) | op_code(operation);
}

void intToCigar(CigarUnit cigar, char& operation, uint32_t& len)
{
    len = cigar >> 4;
    operation = op_char(cigar & 0xfu);
}

bool hasInsertion(const Cigar_t& cigar)
{
    for (CigarUnit c : cigar) {
        if (op_char(c & 0xfu) == 'I') return true;
    }
    return false;
}

std::string cigarToString(const Cigar_t& cigar)
{
    std::string s;
    s.reserve(cigar.size() * 4);
    for (CigarUnit c : cigar) {
        s += std::to_string(c >> 4);
        s += op_char(c & 0xfu);
    }
    return s;
}

Cigar_t stringToCigar(const std::string& str)
{
    Cigar_t out;
    uint64_t len = 0;
    bool digits = false;
    for (char ch : str) {
        if (ch >= '0' && ch <= '9') {
            len = len * 10 + (uint64_t)(ch - '0');
            if (len > kMaxLen) throw std::runtime_error("stringToCigar: length overflow in '" + str + "'");
            digits = true;
        } else {
            if (!digits) throw std::runtime_error("stringToCigar: op without length in '" + str + "'");
            out.push_back(cigarToInt(ch, (uint32_t)len));
            len = 0, digits = false;
        }
    }
    if (digits) throw std::runtime_error("stringToCigar: trailing number without op in '" + str + "'");
    return out;
}

void padQueryToRefByCigar(std::string& query, const Cigar_t& cigar) { project(query, cigar, 1); }

void delQueryToRefByCigar(std::string& query, const Cigar_t& cigar) { project(query, cigar, 0); }

void appendCigar(Cigar_t& result, const Cigar_t& add)
{
    for (CigarUnit c : add) {
        const uint32_t len = c >> 4;
        const char op = op_char(c & 0xfu);
        if (len == 0) continue;
        if (!result.empty() && op_char(result.back() & 0xfu) == op) {
            const uint64_t merged = (uint64_t)(result.back() >> 4) + len;
            if (merged > kMaxLen) throw std::runtime_error("appendCigar: merged length overflow");
            result.back() = cigarToInt(op, (uint32_t)merged);
        } else {
            result.push_back(c);
        }
    }
}

std::size_t getRefLength(const Cigar_t& cigar)
{
    std::size_t n = 0;
    for (CigarUnit c : cigar) {
        const char op = op_char(c & 0xfu);
        if (op == 'M' || op == 'D' || op == 'N' || op == '=' || op == 'X') n += c >> 4;
    }
    return n;
}

std::size_t getQueryLength(const Cigar_t& cigar)
{
    std::size_t n = 0;
    for (CigarUnit c : cigar) {
        const char op = op_char(c & 0xfu);
        if (op == 'M' || op == 'I' || op == 'S' || op == '=' || op == 'X') n += c >> 4;
    }
    return n;
}
}  // namespace cigar

// ------------------------------------------------------------------ alignment

namespace align
{
cigar::Cigar_t globalAlignKSW2(const std::string& ref, const std::string& query)
{
    return globalAlignKSW2(ref, query, KSW2AlignConfig{});
}

cigar::Cigar_t globalAlignKSW2(const std::string& ref, const std::string& query, KSW2AlignConfig cfg)
{
    cigar::Cigar_t out;
    if (ref.empty() || query.empty()) {
        if (ref.empty() && !query.empty()) out.push_back(cigar::cigarToInt('I', (uint32_t)query.size()));
        else if (query.empty() && !ref.empty()) out.push_back(cigar::cigarToInt('D', (uint32_t)ref.size()));
        return out;
    }
    const std::vector<uint8_t> r = dna5(ref), q = dna5(query);
    const int w = auto_band((int)ref.size(), (int)query.size());
    int32_t ez[10];
    std::vector<uint32_t> cig;
    const int64_t n = ksw_call((int)q.size(), q.data(), (int)r.size(), r.data(), cfg.alphabet_size, cfg.mat,
                               cfg.gap_open, cfg.gap_extend, w, cfg.zdrop, cfg.end_bonus, cfg.flag, ez, cig);
    if (n < 0) raise("globalAlignKSW2");
    out.assign(cig.begin(), cig.begin() + n);
    return out;
}

cigar::Cigar_t extendAlignKSW2(const std::string& ref, const std::string& query, int zdrop)
{
    std::vector<uint32_t> cig(ref.size() + query.size() + 4);
    const int64_t n = hg_extend_align_ksw2(ref.data(), (int64_t)ref.size(), query.data(), (int64_t)query.size(),
                                           zdrop, cig.data(), (int64_t)cig.size());
    if (n < 0) raise("extendAlignKSW2");
    return cigar::Cigar_t(cig.begin(), cig.begin() + n);
}

cigar::Cigar_t globalAlignMM2(const std::string& ref, const std::string& query, const anchor::Anchors& anchors)
{
    // The align-to-center shape - one reference sequence on the forward
    // strand, one span, a reference of A/C/G/T/U letters, which is what
    // RefAligner's collect_anchors produces - runs the whole anchor-guided
    // alignment on the device against a resident center index.
    bool center_shape = !anchors.empty() && anchors.front().span >= 1 && anchors.front().span <= 31 &&
                        !ref.empty() && ref.size() <= 0x7fffffffu && query.size() <= 0x7fffffffu;
    for (const auto& a : anchors)
        if (a.is_rev || a.rid_ref != anchors.front().rid_ref || a.span != anchors.front().span) center_shape = false;
    for (unsigned char c : ref)
        if (!(c == 'A' || c == 'C' || c == 'G' || c == 'T' || c == 'U' || c == 'a' || c == 'c' || c == 'g' ||
              c == 't' || c == 'u'))
            center_shape = false;
    if (center_shape) {
        hg_index_t* ix = index_for(ref, anchors.front().span);
        std::vector<uint32_t> ar(anchors.size()), aq(anchors.size());
        for (size_t i = 0; i < anchors.size(); ++i) ar[i] = anchors[i].pos_ref, aq[i] = anchors[i].pos_qry;
        std::vector<uint32_t> cig(ref.size() + query.size() + 8);
        uint32_t st = 0;
        const int64_t n = hg_global_align_mm2(ix, query.data(), (int64_t)query.size(), ar.data(), aq.data(),
                                              (int64_t)ar.size(), cig.data(), (int64_t)cig.size(), &st);
        if (n < 0) raise("globalAlignMM2");
        return cigar::Cigar_t(cig.begin(), cig.begin() + n);
    }
    // Any other anchor set: chainAnchors on the device, then each gap segment
    // through globalAlignKSW2 on the device, stitched as the reference does
    // (src/align/align.cpp:189-305).
    KSW2AlignConfig cfg, first_cfg;
    first_cfg.flag = KSW_EZ_GENERIC_SC;
    const std::size_t ref_len = ref.size(), qry_len = query.size();
    anchor::Anchors sorted = anchors;
    anchor::Anchors chain = anchor::chainAnchors(sorted, anchor::default_chain_params());
    if (chain.empty()) return globalAlignKSW2(ref, query);
    std::sort(chain.begin(), chain.end(), [](const anchor::Anchor& a, const anchor::Anchor& b) {
        return a.pos_qry != b.pos_qry ? a.pos_qry < b.pos_qry : a.pos_ref < b.pos_ref;
    });
    cigar::Cigar_t result;
    std::size_t ref_pos = 0, qry_pos = 0;
    auto segment = [&](std::size_t rs, std::size_t re, std::size_t qs, std::size_t qe, const KSW2AlignConfig& c) {
        rs = std::min(rs, ref_len), re = std::min(re, ref_len), qs = std::min(qs, qry_len), qe = std::min(qe, qry_len);
        if (re < rs) re = rs;
        if (qe < qs) qe = qs;
        const cigar::Cigar_t sc = globalAlignKSW2(ref.substr(rs, re - rs), query.substr(qs, qe - qs), c);
        const std::size_t cr = cigar::getRefLength(sc), cq = cigar::getQueryLength(sc);
        if (cr != re - rs || cq != qe - qs) {
            cigar::Cigar_t forced;
            if (qe > qs) forced.push_back(cigar::cigarToInt('I', (uint32_t)(qe - qs)));
            if (re > rs) forced.push_back(cigar::cigarToInt('D', (uint32_t)(re - rs)));
            cigar::appendCigar(result, forced);
            ref_pos = re, qry_pos = qe;
            return;
        }
        cigar::appendCigar(result, sc);
        ref_pos = rs + cr, qry_pos = qs + cq;
    };
    segment(ref_pos, chain.front().pos_ref, qry_pos, chain.front().pos_qry, first_cfg);
    for (std::size_t i = 0; i < chain.size(); ++i) {
        const auto& a = chain[i];
        segment(ref_pos, (std::size_t)a.pos_ref + a.span, qry_pos, (std::size_t)a.pos_qry + a.span, cfg);
        if (i + 1 < chain.size()) segment(ref_pos, chain[i + 1].pos_ref, qry_pos, chain[i + 1].pos_qry, cfg);
    }
    segment(ref_pos, ref_len, qry_pos, qry_len, cfg);
    if (cigar::getRefLength(result) != ref_len || cigar::getQueryLength(result) != qry_len)
        return globalAlignKSW2(ref, query);
    return result;
}
}  // namespace align

// ------------------------------------------------------------------ consensus

namespace consensus
{
char pickConsensusChar(const SiteCount& sc)
{
    uint32_t best = sc.a;
    char ch = 'A';
    if (sc.c > best) best = sc.c, ch = 'C';
    if (sc.g > best) best = sc.g, ch = 'G';
    if (sc.t > best) best = sc.t, ch = 'T';
    if (sc.u > best) best = sc.u, ch = 'U';
    return ch;
}

namespace {
void ensure_parent(const FilePath& p)
{
    if (p.has_parent_path()) std::filesystem::create_directories(p.parent_path());
}

// FASTA/FASTQ records as the reference's kseq-based reader returns them: the
// sequence lines of a record joined, a trailing '\r' dropped, lines before
// the first header skipped.
class FastaReader {
public:
    explicit FastaReader(const FilePath& p) : in_(p, std::ios::binary)
    {
        if (!in_) throw std::runtime_error("failed to open " + p.string());
    }
    bool next(std::string& seq)
    {
        std::string line;
        if (!have_header_) {
            while (std::getline(in_, line))
                if (!line.empty() && (line[0] == '>' || line[0] == '@')) {
                    have_header_ = true;
                    break;
                }
            if (!have_header_) return false;
        }
        seq.clear();
        have_header_ = false;
        bool fastq = false;
        while (std::getline(in_, line)) {
            if (!line.empty() && (line[0] == '>' || line[0] == '@')) {
                have_header_ = true;
                break;
            }
            if (!line.empty() && line[0] == '+') {
                fastq = true;
                break;
            }
            if (line.empty()) continue;
            seq += line;
            if (seq.size() > 1 && seq.back() == '\r') seq.pop_back();
        }
        if (fastq) {  // quality lines until they cover the sequence
            std::size_t q = 0;
            while (q < seq.size() && std::getline(in_, line)) q += line.size();
        }
        return true;
    }

private:
    std::ifstream in_;
    bool have_header_ = false;
};
}  // namespace

void writeConsensusFasta(const FilePath& out_fasta, const std::string& seq)
{
    ensure_parent(out_fasta);
    std::ofstream o(out_fasta, std::ios::binary);
    if (!o) throw std::runtime_error("failed to open fasta output: " + out_fasta.string());
    o << ">consensus\n";
    for (std::size_t i = 0; i < seq.size(); i += 80) {
        o.write(seq.data() + i, (std::streamsize)std::min<std::size_t>(80, seq.size() - i));
        o.put('\n');
    }
}

void writeCountsJson(const FilePath& out_json, const ConsensusJson& cj)
{
    // The document the reference's JSON archive writes: an outer object with
    // one "consensus" member, four-space indentation, one counter per line.
    ensure_parent(out_json);
    std::ofstream o(out_json, std::ios::binary);
    if (!o) throw std::runtime_error("failed to open json output: " + out_json.string());
    o << "{\n    \"consensus\": {\n";
    o << "        \"num_seqs\": " << cj.num_seqs << ",\n";
    o << "        \"aln_len\": " << cj.aln_len << ",\n";
    o << "        \"counts\": [";
    static const char* kNames[7] = {"A", "C", "G", "T", "U", "N", "-"};
    for (std::size_t i = 0; i < cj.counts.size(); ++i) {
        const SiteCount& s = cj.counts[i];
        const uint32_t v[7] = {s.a, s.c, s.g, s.t, s.u, s.n, s.dash};
        o << (i ? ",\n" : "\n") << "            {\n";
        for (int k = 0; k < 7; ++k)
            o << "                \"" << kNames[k] << "\": " << v[k] << (k < 6 ? ",\n" : "\n");
        o << "            }";
    }
    o << (cj.counts.empty() ? "]\n" : "\n        ]\n");
    o << "    }\n}";
}

std::string generateConsensusSequence(const FilePath& aligned_fasta, const FilePath& out_fasta,
                                      const FilePath& out_json, std::uint64_t seq_limit, int thread,
                                      size_t batch_size)
{
    (void)thread;
    if (!std::filesystem::is_regular_file(aligned_fasta))
        throw std::runtime_error("aligned_fasta is not a regular file: " + aligned_fasta.string());
    FastaReader reader(aligned_fasta);
    std::string rec;
    if (!reader.next(rec)) throw std::runtime_error("aligned fasta is empty: " + aligned_fasta.string());
    const std::size_t L = rec.size();
    if (L == 0) throw std::runtime_error("first sequence length is 0: " + aligned_fasta.string());
    ConsensusJson cj;
    cj.aln_len = L;
    std::vector<uint32_t> counts(7 * L, 0);
    std::uint64_t num = 0;
    std::string batch;  // rows back to back, L bytes each
    std::size_t rows = 0;
    batch.reserve(std::min<std::size_t>(batch_size, 4096) * L);
    batch += rec, ++rows, ++num;
    while (seq_limit == 0 || num < seq_limit) {
        while (rows < batch_size && (seq_limit == 0 || num < seq_limit)) {
            if (!reader.next(rec)) break;
            if (rec.size() != L) throw std::runtime_error("alignment length mismatch when reading");
            batch += rec, ++rows, ++num;
        }
        if (rows) {
            if (hg_count_rows(batch.data(), (int64_t)rows, (int64_t)L, (int64_t)L, counts.data(), 1) != HG_OK)
                raise("generateConsensusSequence");
            batch.clear(), rows = 0;
        }
        // the reference reads one more record here and drops it when the
        // file continues (src/consensus/consensus.cpp:680)
        if (!reader.next(rec)) break;
    }
    if (num == 0) throw std::runtime_error("no sequences processed");
    cj.num_seqs = num;
    cj.counts.resize(L);
    std::string cons(L, 'N');
    for (std::size_t i = 0; i < L; ++i) {
        SiteCount& s = cj.counts[i];
        const uint32_t* c = &counts[7 * i];
        s.a = c[0], s.c = c[1], s.g = c[2], s.t = c[3], s.u = c[4], s.n = c[5], s.dash = c[6];
        cons[i] = pickConsensusChar(s);
    }
    writeConsensusFasta(out_fasta, cons);
    writeCountsJson(out_json, cj);
    return cons;
}
}  // namespace consensus

// ------------------------------------------------------------------ MinHash

namespace mash
{
Sketch sketchFromSequence(const std::string& seq, std::size_t k, std::size_t sketch_size, bool noncanonical, int seed)
{
    Sketch sk;
    sk.k = k;
    sk.noncanonical = noncanonical;
    if (k == 0 || sketch_size == 0 || seq.size() < k || k > 32) return sk;
    if (sketch_size > (std::size_t)HG_SKETCH_MAX)
        throw std::invalid_argument("mash::sketchFromSequence: sketch_size above HG_SKETCH_MAX");
    const int64_t off[2] = {0, (int64_t)seq.size()};
    int64_t pb = 0, ne = 0;
    if (hg_pack(seq.data(), off, 1, nullptr, 0, nullptr, nullptr, 0, nullptr, &pb, &ne) != HG_OK)
        raise("sketchFromSequence");
    std::vector<uint8_t> packed((size_t)std::max<int64_t>(pb, 16));
    std::vector<int32_t> exc((size_t)std::max<int64_t>(ne, 1) * 3);
    int64_t poff = 0, eoff[2] = {0, 0};
    if (hg_pack(seq.data(), off, 1, packed.data(), (int64_t)packed.size(), &poff, exc.data(), ne, eoff, nullptr,
                nullptr) != HG_OK)
        raise("sketchFromSequence");
    const int32_t qlen = (int32_t)seq.size();
    std::vector<uint64_t> h(sketch_size);
    int32_t cnt = 0;
    if (hg_sketch_batch(packed.data(), &poff, &qlen, exc.data(), eoff, 1, (int)k, (int)sketch_size,
                        noncanonical ? 1 : 0, seed, h.data(), (int64_t)sketch_size, &cnt) != HG_OK)
        raise("sketchFromSequence");
    sk.hashes.assign(h.begin(), h.begin() + cnt);
    return sk;
}

std::size_t intersectionSizeSortedUnique(const std::vector<hash_t>& a, const std::vector<hash_t>& b) noexcept
{
    std::size_t i = 0, j = 0, n = 0;
    while (i < a.size() && j < b.size()) {
        if (a[i] < b[j]) ++i;
        else if (b[j] < a[i]) ++j;
        else ++n, ++i, ++j;
    }
    return n;
}

double jaccard(const Sketch& a, const Sketch& b)
{
    if (a.k != b.k) throw std::invalid_argument("mash::jaccard: mismatched k");
    if (a.hashes.empty() && b.hashes.empty()) return 1.0;
    if (a.hashes.empty() || b.hashes.empty()) return 0.0;
    const std::size_t inter = intersectionSizeSortedUnique(a.hashes, b.hashes);
    return (double)inter / (double)std::min(a.hashes.size(), b.hashes.size());
}

double mashDistanceFromJaccard(double j, std::size_t k)
{
    if (k == 0) throw std::invalid_argument("mash::mashDistanceFromJaccard: k must be > 0");
    if (!(j > 0.0)) return std::numeric_limits<double>::infinity();
    if (j >= 1.0) return 0.0;
    const double x = (2.0 * j) / (1.0 + j);
    if (!(x > 0.0)) return std::numeric_limits<double>::infinity();
    return -std::log(x) / (double)k;
}

double aniFromJaccard(double j, std::size_t k)
{
    if (k == 0) throw std::invalid_argument("mash::aniFromJaccard: k must be > 0");
    if (!(j > 0.0)) return 0.0;
    if (j >= 1.0) return 1.0;
    const double x = (2.0 * j) / (1.0 + j);
    if (!(x > 0.0)) return 0.0;
    return std::min(1.0, std::max(0.0, std::pow(x, 1.0 / (double)k)));
}

double aniFromMashDistance(double d)
{
    if (!std::isfinite(d)) return 0.0;
    if (d <= 0.0) return 1.0;
    return std::min(1.0, std::max(0.0, std::exp(-d)));
}
}  // namespace mash
